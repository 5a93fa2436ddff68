"""Generate tests/golden/c4_golden.json: the oracle's skeleton of every instance of the
512-instance batched workload (p ~ U[20, 800], n ~ U[200, 8000], ER degree ~ U[1, 5],
weights +-[0.1, 1.0], alpha 0.01 / 0.05 alternating, FP32 data, levels until no edge
has enough neighbours).

Each instance's FP32 observations come from the library's seeded generator (host code,
bit-identical on every host); the oracle (oracle/oracle.cpp, the FP64 restatement of
the reference CPU path, itself pinned to the reference's own CPU sources) computes
the FP64 correlation and the skeleton. The fixture keeps per instance: the SHA-256 of
the data, the number of edges after every level, the SHA-256 of the final adjacency
(upper triangle, bit-packed), the number of separation-set records and the oracle's
single-thread seconds (the CPU legs of bench.py order instances by it). The GPU test
(tests/test_gpu_c4_parity.py) recomputes the same hashes from the device results.

The oracle's cost per instance ranges from milliseconds to minutes (levels up to 21
on the p ~ 800 instances), so the instances run in parallel, one per host core, most
expensive first; finished instances are appended to a progress file next to the
fixture so that an interrupted run resumes.

Run from the repository root:   python tests/golden/make_c4_golden.py [--jobs N]
"""
import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _d in (ROOT, os.path.join(ROOT, "masterthesis-heterogeneous-pc_gb300")):
    if _d not in sys.path:
        sys.path.insert(0, _d)

OUT = os.path.join(HERE, "c4_golden.json")
PROGRESS = os.path.join(HERE, "c4_golden.progress.jsonl")


def adjacency_sha(adj):
    """SHA-256 of the upper triangle (i < j, row by row) of a p x p 0/1 matrix, bit-packed."""
    p = adj.shape[0]
    iu = np.triu_indices(p, 1)
    return hashlib.sha256(np.packbits(np.asarray(adj)[iu] != 0).tobytes()).hexdigest()


def data_sha(X):
    return hashlib.sha256(np.ascontiguousarray(X).tobytes()).hexdigest()


def _one(b):
    import heterogpc as hg
    from oracle import oracle as orc

    import bench
    wl = bench.WORKLOADS["c4"]
    X = bench.c4_instance_data(wl, b)
    ps, ns, degs, alphas = bench.c4_instances(wl)
    Cm = orc.correlation(X.astype(np.float64))
    t0 = time.perf_counter()
    res = orc.run(Cm, int(ns[b]), float(alphas[b]), wl["max_level"], threads=1)
    dt = time.perf_counter() - t0
    return dict(b=int(b), p=int(ps[b]), n=int(ns[b]), alpha=float(alphas[b]), degree=float(degs[b]),
                data_sha256=data_sha(X), adj_sha256=adjacency_sha(res.adj), edges=res.edges(),
                edges_per_level=[int(l["edges_after"]) for l in res.levels],
                tests_per_level=[int(l["executed_tests"]) for l in res.levels],
                records=len(res.records), oracle_s=dt)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    ap.add_argument("--count", type=int, default=512)
    args = ap.parse_args()
    import hpc_build
    hpc_build.build_library()
    hpc_build.build_oracle()
    import bench
    wl = bench.WORKLOADS["c4"]
    ps, ns, degs, alphas = bench.c4_instances(wl)
    done = {}
    if os.path.exists(PROGRESS):
        with open(PROGRESS) as f:
            for line in f:
                if line.strip():
                    r = json.loads(line)
                    done[r["b"]] = r
    todo = [b for b in range(args.count) if b not in done]
    # most expensive first (p^2 x degree x log n as the estimate): the long ones start at once
    todo.sort(key=lambda b: -(float(ps[b]) ** 2 * float(degs[b]) * np.log(float(ns[b]))))
    print("%d instances done, %d to run on %d processes" % (len(done), len(todo), args.jobs), flush=True)
    ctx = mp.get_context("spawn")
    with ctx.Pool(args.jobs) as pool, open(PROGRESS, "a") as prog:
        for r in pool.imap_unordered(_one, todo):
            done[r["b"]] = r
            prog.write(json.dumps(r) + "\n")
            prog.flush()
            print("instance %3d p=%3d n=%4d: %5d edges, %2d levels, %.1f s (%d/%d)"
                  % (r["b"], r["p"], r["n"], r["edges"], len(r["edges_per_level"]), r["oracle_s"], len(done),
                     args.count), flush=True)
    rows = [done[b] for b in range(args.count)]
    out = dict(generator="tests/golden/make_c4_golden.py", expected_from="oracle (oracle/oracle.cpp, FP64)",
               workload=dict(wl, p=list(wl["p"]), n=list(wl["n"]), degree=list(wl["degree"]),
                             alphas=list(wl["alphas"])),
               instances=[dict({k: r[k] for k in ("b", "p", "n", "alpha", "data_sha256", "adj_sha256", "edges",
                                                  "edges_per_level", "records")}, oracle_s=round(r["oracle_s"], 3))
                          for r in rows],
               oracle_seconds_total=sum(r["oracle_s"] for r in rows))
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote %s (%d instances, %.0f oracle seconds)" % (OUT, len(rows), out["oracle_seconds_total"]))


if __name__ == "__main__":
    main()
