"""The measurement helpers of bench.py that its parity and sampling claims rest on: the
bitmask unpacking and adjacency hash that compare every instance with the committed
oracle results, the cost-balanced slices of the CPU samples, and the batch's seeded
shapes. CPU only."""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _pack(adj):
    """p x ceil(p/32) uint32 words, bit j % 32 of word j / 32 (the library's layout)."""
    p = adj.shape[0]
    W = (p + 31) // 32
    words = np.zeros((p, W), np.uint32)
    for i in range(p):
        for j in np.nonzero(adj[i])[0]:
            words[i, j // 32] |= np.uint32(1) << np.uint32(j % 32)
    return words.reshape(-1)


def _random_graph(p, seed):
    rng = np.random.default_rng(seed)
    a = np.triu(rng.random((p, p)) < 0.2, 1)
    return (a | a.T).astype(np.uint8)


def test_bits_to_matrix_inverts_the_library_layout():
    for p in (1, 31, 32, 33, 70, 129):
        adj = _random_graph(p, p)
        assert np.array_equal(bench.bits_to_matrix(_pack(adj), p), adj), p


def test_adjacency_hash_is_the_packed_upper_triangle():
    p = 45
    adj = _random_graph(p, 3)
    iu = np.triu_indices(p, 1)
    want = hashlib.sha256(np.packbits(adj[iu] != 0).tobytes()).hexdigest()
    assert bench.c4_adj_sha(adj) == want
    flipped = adj.copy()
    flipped[4, 17] ^= 1
    flipped[17, 4] ^= 1
    assert bench.c4_adj_sha(flipped) != want
    # the lower triangle does not enter the hash
    lower = adj.copy()
    lower[20, 2] ^= 1
    assert bench.c4_adj_sha(lower) == want


def test_slices_partition_the_batch_with_balanced_cost():
    rng = np.random.default_rng(7)
    count = 512
    costs = list(rng.pareto(1.5, count) + 0.01)
    for k in (1, 2, 6, 20):
        sl = bench.c4_slices(count, costs, k)
        assert len(sl) == k
        flat = sorted(b for s in sl for b in s)
        assert flat == list(range(count)), k
        tot = [sum(costs[b] for b in s) for s in sl]
        # back-and-forth dealing: no slice differs from another by more than the largest cost
        assert max(tot) - min(tot) <= max(costs) + 1e-9, k
    assert bench.c4_slices(5, None, 2) == [[0, 3, 4], [1, 2]]


def test_batch_shapes_are_seeded_and_in_range():
    wl = bench.WORKLOADS["c4"]
    a = bench.c4_instances(wl)
    b = bench.c4_instances(wl)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    ps, ns, degs, alphas = a
    assert len(ps) == wl["count"] == 512
    assert ps.min() >= wl["p"][0] and ps.max() <= wl["p"][1]
    assert ns.min() >= wl["n"][0] and ns.max() <= wl["n"][1]
    assert degs.min() >= wl["degree"][0] and degs.max() <= wl["degree"][1]
    assert set(alphas[:2]) == set(wl["alphas"])
    # a prefix of the batch is the same instances
    ps8 = bench.c4_instances(wl, 8)[0]
    assert np.array_equal(ps8, ps[:8])
