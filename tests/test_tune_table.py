"""The tile-policy table of the autotuner on the host (no GPU): keys fall into
bit-length buckets of (p, level, degree), entries round-trip through the text file,
and bad policies, keys and files are rejected with HPC_ERR_INVALID_ARG."""
import pytest

import heterogpc as hg


@pytest.fixture(autouse=True)
def _clean_table():
    hg.tune_clear()
    yield
    hg.tune_clear()


def test_defaults_without_entries():
    pol, found = hg.tune_lookup(2000, 1, 237)
    assert not found and pol == {"tile_cap": 64, "tiles_per_lane": 4, "edge_lanes": 32, "l1_prefetch": 0}


def test_buckets_and_erase():
    hg.tune_set(2000, 2, 100, 256, 8, 1)
    # same buckets: p in [1024, 2047], degree in [64, 127]
    assert hg.tune_lookup(1024, 2, 64) == ({"tile_cap": 256, "tiles_per_lane": 8, "edge_lanes": 1, "l1_prefetch": 0},
                                           True)
    assert hg.tune_lookup(2047, 2, 127)[1]
    # other buckets or levels
    assert not hg.tune_lookup(2048, 2, 100)[1]
    assert not hg.tune_lookup(2000, 2, 128)[1]
    assert not hg.tune_lookup(2000, 3, 100)[1]
    hg.tune_set(2000, 2, 100, None)
    assert not hg.tune_lookup(2000, 2, 100)[1]


def test_file_round_trip(tmp_path):
    hg.tune_set(15000, 1, 13000, 1024, 2, 32, 1)
    hg.tune_set(300, 7, 20, 16, 16, 1)
    path = str(tmp_path / "t.txt")
    hg.tune_save(path)
    hg.tune_clear()
    assert not hg.tune_lookup(300, 7, 20)[1]
    hg.tune_load(path)
    assert hg.tune_lookup(15000, 1, 13000) == ({"tile_cap": 1024, "tiles_per_lane": 2, "edge_lanes": 32, "l1_prefetch": 1},
                                               True)
    assert hg.tune_lookup(300, 7, 20) == ({"tile_cap": 16, "tiles_per_lane": 16, "edge_lanes": 1, "l1_prefetch": 0}, True)


@pytest.mark.parametrize("args", [(2000, 1, 10, 0, 4, 32), (2000, 1, 10, 65537, 4, 32), (2000, 1, 10, 64, 0, 32),
                                  (2000, 1, 10, 64, 65, 32), (2000, 1, 10, 64, 4, 8), (1, 1, 10, 64, 4, 32),
                                  (2000, 0, 10, 64, 4, 32), (2000, hg.HPC_MAX_LEVEL + 1, 10, 64, 4, 32),
                                  (2000, 1, -1, 64, 4, 32), (2000, 1, 10, 64, 4, 32, 2)])
def test_rejects_bad_policies_and_keys(args):
    with pytest.raises(hg.HpcError) as e:
        hg.tune_set(*args)
    assert e.value.status == 1


@pytest.mark.parametrize("text", ["not a policy file\n", "heterogpc-tile-policy 2 32 33 18\n1 0 3 64 4 32 0\n",
                                  "heterogpc-tile-policy 2 32 33 18\n1 2 3 64 4 32\n",
                                  "heterogpc-tile-policy 1 32 33 18\n", "heterogpc-tile-policy 2 32 33 18\n1 2 3 0 4 32 0\n"])
def test_rejects_bad_files(tmp_path, text):
    path = tmp_path / "bad.txt"
    path.write_text(text)
    with pytest.raises(hg.HpcError):
        hg.tune_load(str(path))
    with pytest.raises(hg.HpcError):
        hg.tune_load(str(tmp_path / "missing.txt"))
