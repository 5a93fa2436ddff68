"""Generate tests/golden/c5_golden.json: the oracle's skeletons of a set of served
requests spanning the served workload's range (p up to 5000, n up to 20000, ER degree 3
and preferential attachment with 2 parents per node -- hub-heavy --, weights
+-[0.1, 1.0], alpha 0.01, FP32 data, levels 0-4: the served workload's cap -- on the
hub-heavy graphs the number of tests grows as C(d - 1, l) on the hubs' rows, so that
"until exhausted" is out of reach for the CPU and the GPU alike).

The data come from the library's seeded generator (host code, bit-identical on every
host); the oracle (oracle/oracle.cpp) computes the FP64 correlation and the skeleton on
all host cores. The fixture keeps per request the SHA-256 of the data and of the final
adjacency's upper triangle (bit-packed) and the edges after every level; the GPU test
(tests/test_gpu_serve.py) serves the same requests and compares.

Run from the repository root:   python tests/golden/make_c5_golden.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _d in (ROOT, os.path.join(ROOT, "masterthesis-heterogeneous-pc_gb300")):
    if _d not in sys.path:
        sys.path.insert(0, _d)

OUT = os.path.join(HERE, "c5_golden.json")
ALPHA = 0.01
MAX_LEVEL = 4
# (p, n, graph): the corners and the middle of p in [30, 5000] x n in [500, 20000]
REQUESTS = [(5000, 20000, 0), (5000, 2000, 1), (3000, 20000, 1), (4000, 8000, 1), (1500, 15000, 1),
            (800, 500, 0), (30, 500, 1), (200, 20000, 0), (2500, 1000, 0), (5000, 5000, 1), (60, 12000, 1),
            (1000, 3000, 0)]


def request_data(q):
    import heterogpc as hg
    p, n, graph = REQUESTS[q]
    return hg.sem_generate(p, n, graph, 3.0, 2, 0.1, 1.0, 777000 + q, dtype=np.float32)


def main():
    import hpc_build
    hpc_build.build_library()
    hpc_build.build_oracle()
    from oracle import oracle as orc

    sys.path.insert(0, HERE)
    from make_c4_golden import adjacency_sha, data_sha
    rows = []
    for q, (p, n, graph) in enumerate(REQUESTS):
        X = request_data(q)
        t0 = time.perf_counter()
        Cm = orc.correlation(X.astype(np.float64))
        t1 = time.perf_counter()
        res = orc.run(Cm, n, ALPHA, MAX_LEVEL)
        t2 = time.perf_counter()
        rows.append(dict(q=q, p=p, n=n, graph="PA" if graph else "ER", data_sha256=data_sha(X),
                         adj_sha256=adjacency_sha(res.adj), edges=res.edges(),
                         edges_per_level=[int(l["edges_after"]) for l in res.levels]))
        print("request %2d p=%4d n=%5d %s: %6d edges, %2d levels (correlation %.1f s, skeleton %.1f s)"
              % (q, p, n, rows[-1]["graph"], res.edges(), len(res.levels), t1 - t0, t2 - t1), flush=True)
    with open(OUT, "w") as f:
        json.dump(dict(generator="tests/golden/make_c5_golden.py", expected_from="oracle (oracle/oracle.cpp, FP64)",
                       alpha=ALPHA, max_level=MAX_LEVEL, requests=rows), f, separators=(",", ":"))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
