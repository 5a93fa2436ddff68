"""Generate the golden skeleton fixtures in tests/golden/golden.json.

Expected edge sets come from the reference's own CPU test code (src/executor/testing/
cpuRowTests.cpp, cpuUtil.cpp, cpuWorkstealingTests.cpp, cpuExecutor.cpp and
src/executor/independence/cpuInd.cpp), compiled from the reference tree by
oracle/build_ref.sh against restated Armadillo/Boost headers, run single-threaded.
Inputs are seeded linear-Gaussian SEM data from the library's generator (bit-identical
on every host; the fixture stores a SHA-256 of the data and of the FP64 correlation
matrix so a host that disagrees is caught) or small matrices stored inline.

Run from the repository root, naming the reference tree's root (its data/cooling_house.csv
is one of the cases):
    python tests/golden/make_golden.py <reference tree root>
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "masterthesis-heterogeneous-pc_gb300"))

import heterogpc as hg  # noqa: E402
from oracle import oracle as orc  # noqa: E402


# name, generator params, alpha, max_level
GEN_CASES = [
    ("c1_er50_seed1_a001", dict(p=50, n=1000, graph=hg.GRAPH_ER, degree=2.0, seed=1), 0.01, 12),
    ("c1_er50_seed2_a001", dict(p=50, n=1000, graph=hg.GRAPH_ER, degree=2.0, seed=2), 0.01, 12),
    ("c1_er50_seed3_a005", dict(p=50, n=1000, graph=hg.GRAPH_ER, degree=2.0, seed=3), 0.05, 12),
    ("er40_deg4_n300_a005", dict(p=40, n=300, graph=hg.GRAPH_ER, degree=4.0, seed=4), 0.05, 12),
    ("er80_deg3_n500_a001", dict(p=80, n=500, graph=hg.GRAPH_ER, degree=3.0, seed=5), 0.01, 12),
    ("pa60_n500_a005", dict(p=60, n=500, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=6), 0.05, 12),
    ("pa100_n2000_a001", dict(p=100, n=2000, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=7), 0.01, 12),
    ("er60_n200_maxlevel2", dict(p=60, n=200, graph=hg.GRAPH_ER, degree=5.0, seed=8), 0.05, 2),
    ("er30_n100_maxlevel0", dict(p=30, n=100, graph=hg.GRAPH_ER, degree=3.0, seed=9), 0.05, 0),
]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gen(params):
    kw = dict(degree=2.0, pa_parents=2, w_lo=0.1, w_hi=1.0)
    kw.update(params)
    return hg.sem_generate(kw["p"], kw["n"], kw["graph"], kw["degree"], kw["pa_parents"], kw["w_lo"], kw["w_hi"],
                           kw["seed"])


def expected(Cm, n, alpha, max_level):
    adj, sep, _ = orc.ref_run(Cm, n, alpha, max_level, threads=1)
    p = Cm.shape[0]
    edges = [[int(i), int(j)] for i in range(p) for j in range(i + 1, p) if adj[i, j]]
    mc = sep.shape[2]
    seps = []
    for i in range(p):
        for j in range(i + 1, p):
            if not adj[i, j]:
                row = sep[i, j]
                if row[0] == -2:
                    seps.append([i, j, 0, []])
                else:
                    ids = [int(v) for v in row if v >= 0]
                    seps.append([i, j, len(ids), ids])
    return edges, seps, mc


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference tree root>")
    ref_data = os.path.join(sys.argv[1], "data", "cooling_house.csv")
    if not orc.ref_available():
        sys.exit("oracle/_ref/libref_cpu.so missing: build it with oracle/build_ref.sh first")
    cases = []
    for name, params, alpha, ml in GEN_CASES:
        X = gen(params)
        Cm = orc.correlation(X)
        edges, seps, mc = expected(Cm, params["n"], alpha, ml)
        cases.append(dict(name=name, source="sem", params=params, alpha=alpha, max_level=ml, n_obs=params["n"],
                          data_sha256=sha(X), cor_sha256=sha(Cm), edges=edges, n_edges=len(edges),
                          ref_sepsets=seps))
    # edge cases on small SEM data: a variable with missing samples, a constant
    # variable (NaN correlations) and a duplicated variable (singular submatrices)
    base = dict(p=24, n=400, graph=hg.GRAPH_ER, degree=3.0, seed=21)
    X = gen(base)
    Xn = X.copy()
    Xn[3, ::7] = np.nan
    Xc = X.copy()
    Xc[5, :] = 1.25
    Xd = X.copy()
    Xd[7, :] = Xd[2, :]
    for name, Xe in (("nan_samples_var3", Xn), ("constant_var5", Xc), ("duplicate_var7_of_2", Xd)):
        Cm = orc.correlation(Xe)
        Cm = np.where(np.isnan(Cm), np.nan, Cm)  # one NaN bit pattern, as the JSON round trip gives
        edges, seps, mc = expected(Cm, base["n"], 0.05, 4)
        cases.append(dict(name=name, source="matrix", alpha=0.05, max_level=4, n_obs=base["n"],
                          cor=[[None if np.isnan(v) else float(v) for v in row] for row in Cm],
                          cor_sha256=sha(Cm), edges=edges, n_edges=len(edges), ref_sepsets=seps))
    if os.path.exists(ref_data):
        D = np.loadtxt(ref_data, delimiter=",").T.copy()
        Cm = orc.correlation(D)
        for alpha in (0.01, 0.05):
            edges, seps, mc = expected(Cm, D.shape[1], alpha, 4)
            cases.append(dict(name="cooling_house_a%g" % alpha, source="matrix", alpha=alpha, max_level=4,
                              n_obs=int(D.shape[1]), cor=Cm.tolist(), cor_sha256=sha(Cm), edges=edges,
                              n_edges=len(edges), ref_sepsets=seps))
    out = dict(generator="tests/golden/make_golden.py", expected_from="reference CPU sources (oracle/_ref)",
               cases=cases)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote %s: %d cases" % (path, len(cases)))
    for c in cases:
        print("  %-26s edges %d" % (c["name"], c["n_edges"]))


if __name__ == "__main__":
    main()
