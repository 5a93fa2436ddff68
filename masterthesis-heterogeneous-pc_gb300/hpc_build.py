"""Build of libheterogpc.so, the heterogpc CLI and the oracle libraries.

Everything is compiled in-tree with nvcc / g++ directly (no cmake), one
translation unit per process, for sm_103a only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["citest_l17s.cu", "citest_l17.cu", "citest_l13.cu", "citest_l9.cu", "citest.cu", "ctx.cu", "correlation.cu", "graph.cu", "gram_tc.cu",
              "noalloc.cu", "tune.cu", "compat.cu", "serve.cu", "gram_emu.cu"]
HOST_SOURCES = ["semgen.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".hpp", ".h"))]
    return hs


def _compile_cu(src, verbose_ptxas=False):
    out = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _newer(out, [src] + _headers()):
        return out
    cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "--expt-relaxed-constexpr", "-c", src, "-o", out]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    _run(cmd)
    return out


def _compile_host(src, extra=()):
    out = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _newer(out, [src] + _headers()):
        return out
    _run(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I",
          os.path.join(CUDA_HOME, "include"), *extra, "-c", src, "-o", out])
    return out


def build_library(jobs=8):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile_cu, os.path.join(CSRC, f)) for f in CU_SOURCES]
        futs += [ex.submit(_compile_host, os.path.join(HOST, f)) for f in HOST_SOURCES]
        objs = [f.result() for f in futs]
    so = os.path.join(LIB, "libheterogpc.so")
    if not _newer(so, objs):
        _run([NVCC, "-shared", *ARCH, "-o", so, *objs, "-cudart", "shared", "-lpthread"])
    build_cli(so)
    return so


CLI_SOURCES = ["main.cpp", "skeleton.cpp", "csv.cpp", "npy.cpp"]


def build_cli(so):
    """The heterogpc command line, linked against libheterogpc.so (rpath to lib/)."""
    objs = [_compile_host(os.path.join(HOST, f), extra=("-I", HOST)) for f in CLI_SOURCES]
    exe = os.path.join(LIB, "heterogpc")
    if not _newer(exe, objs + [so]):
        _run(["g++", "-o", exe, *objs, "-L", LIB, "-lheterogpc", "-Wl,-rpath,$ORIGIN", "-lpthread"])
    return exe


def build_oracle():
    """oracle/liboracle.so: the CPU restatement, plus the seeded SEM generator (host code,
    so that CPU-only legs can make the workloads' data without loading the product)."""
    so = os.path.join(ORACLE, "liboracle.so")
    src = os.path.join(ORACLE, "oracle.cpp")
    sem = os.path.join(HOST, "semgen.cpp")
    deps = [src, sem, os.path.join(ORACLE, "pinv_sym.hpp"), os.path.join(INCLUDE, "heterogpc.h")]
    if not _newer(so, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-I", INCLUDE, src, sem,
              "-o", so, "-lpthread"])
    return so


# where the reference tree is mounted in the build container (REF_ROOT overrides it)
REFERENCE_MOUNT = "/root/reference"


def build_reference_pin():
    """oracle/_ref/libref_cpu.so from the reference sources, only where they exist."""
    ref = os.environ.get("REF_ROOT", REFERENCE_MOUNT)
    if not os.path.isdir(os.path.join(ref, "src")):
        return None
    out = os.path.join(ORACLE, "_ref", "libref_cpu.so")
    if os.path.exists(out):
        return out
    _run(["bash", os.path.join(ORACLE, "build_ref.sh"), ref])
    return out


def build_all(jobs=8):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f_lib = ex.submit(build_library, jobs)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference_pin)
        return {"lib": f_lib.result(), "oracle": f_orc.result(), "ref": f_ref.result()}


if __name__ == "__main__":
    print(build_all())
