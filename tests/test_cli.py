"""The heterogpc command line: flags, messages and exit codes of src/main.cpp, and
(on a GPU) the skeleton it prints against the oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

import heterogpc as hg
from helpers import gen
from oracle import oracle as orc

EXE = os.path.join(os.path.dirname(hg.LIB_PATH), "heterogpc")


def run(*args, cwd=None):
    return subprocess.run([EXE, *args], capture_output=True, text=True, cwd=cwd, timeout=600)


def test_help_lists_reference_flags():
    r = run("--help")
    assert r.returncode == 0
    for flag in ("--input-file", "--alpha", "--observations", "--row-mult", "--row-mult2", "--row-mult3",
                 "--max-level", "--corr", "--gpus", "--thread-count", "--csv-export", "--gpu-only", "--cpu-only",
                 "--power9-ats", "--workstealing", "--print-sepsets", "--verbose"):
        assert flag in r.stdout, flag
    assert "(=0.05)" in r.stdout and "(=4)" in r.stdout


def test_parse_errors_exit_1():
    assert run("--bogus").returncode == 1
    assert run("-a", "x").returncode == 1
    assert run("--alpha").returncode == 1


def test_corr_needs_observations(tmp_path):
    r = run("--corr", "-i", str(tmp_path / "c.csv"))
    assert r.returncode == 255 and "Observation count needed" in r.stdout


def test_non_csv_and_missing_file(tmp_path):
    r = run("-i", str(tmp_path / "data.txt"))
    assert r.returncode == 255 and "Has to be .csv format." in r.stdout
    r = run("-i", str(tmp_path / "missing.csv"))
    assert r.returncode == 1 and "Could not find file" in r.stdout


def write_csv(path, M, header=None):
    with open(path, "w") as f:
        if header:
            f.write(",".join(header) + "\n")
        for row in M:
            f.write(",".join(repr(float(v)) for v in row) + "\n")


def parse_output(out):
    edges = int(re.search(r"Total number of edges: (\d+)", out).group(1))
    seps = {}
    for m in re.finditer(r"Separation from (\d+) to (\d+)( via ([\d ]+))?\n", out):
        ids = tuple(int(x) for x in m.group(4).split()) if m.group(4) else ()
        seps[(int(m.group(1)), int(m.group(2)))] = ids
    return edges, seps


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-tc"])
def test_observations_csv_skeleton(tmp_path, precision):
    X = gen(dict(p=30, n=500, graph=hg.GRAPH_ER, degree=3.0, seed=17))
    path = tmp_path / "obs.csv"
    write_csv(path, X.T, header=["v%d" % i for i in range(30)])  # rows = observations
    Cm = orc.correlation(X)
    want = orc.run(Cm, 500, 0.05, 4)
    csv_out = tmp_path / "m.csv"
    r = run("-i", str(path), "-a", "0.05", "-m", "4", "-v", "-p", "--csv-export", str(csv_out), "--precision", precision)
    assert r.returncode == 0, r.stderr
    edges, seps = parse_output(r.stdout)
    assert edges == want.edges()
    removed = {(i, j) for i in range(30) for j in range(i + 1, 30) if not want.adj[i, j]}
    assert set(seps) == removed
    for (i, j), ids in seps.items():
        assert orc.verify_sepset(Cm, 500, 0.05, i, j, ids)
    cols = open(csv_out).read().strip().split(",")
    assert len(cols) == 3 + 4 * 5 + 1 and int(cols[2]) == want.edges()


@pytest.mark.gpu
def test_correlation_csv_skeleton(tmp_path):
    X = gen(dict(p=40, n=800, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=18))
    Cm = orc.correlation(X)
    path = tmp_path / "cor.csv"
    write_csv(path, Cm)
    want = orc.run(Cm, 800, 0.01, 3)
    r = run("--corr", "-o", "800", "-i", str(path), "-a", "0.01", "-m", "3", "-v", "-w", "--cpu-only")
    assert r.returncode == 0, r.stderr
    edges, _ = parse_output(r.stdout)
    assert edges == want.edges()
    assert "no effect" in r.stderr


@pytest.mark.gpu
def test_autotune_and_tune_file(tmp_path):
    """--autotune times the tile-policy candidates on the input and writes the table to
    --tune-file; a later run loads it. Both print the oracle's skeleton."""
    X = gen(dict(p=120, n=1500, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=19))
    Cm = orc.correlation(X)
    path = tmp_path / "cor.csv"
    write_csv(path, Cm)
    want = orc.run(Cm, 1500, 0.05, 3)
    table = tmp_path / "policy.txt"
    r = run("--corr", "-o", "1500", "-i", str(path), "-a", "0.05", "-m", "3", "-v", "--autotune", "--tune-file",
            str(table))
    assert r.returncode == 0, r.stderr
    assert parse_output(r.stdout)[0] == want.edges()
    assert "tile-policy entries" in r.stderr
    lines = open(table).read().splitlines()
    assert lines[0].startswith("heterogpc-tile-policy") and len(lines) > 1
    r = run("--corr", "-o", "1500", "-i", str(path), "-a", "0.05", "-m", "3", "-v", "--tune-file", str(table))
    assert r.returncode == 0, r.stderr
    assert parse_output(r.stdout)[0] == want.edges()


def test_bad_tune_file_is_an_error(tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("nonsense\n")
    X = gen(dict(p=10, n=100, graph=hg.GRAPH_ER, degree=2.0, seed=20))
    path = tmp_path / "cor.csv"
    write_csv(path, orc.correlation(X))
    r = run("--corr", "-o", "100", "-i", str(path), "--tune-file", str(bad))
    assert r.returncode == 2 and "not a tile-policy file" in r.stderr
