"""CPU tests of the host side of libcm: generators, METIS IO, partition
output, edge cut, and that the C-ABI library loads and exports every symbol
include/cm.h declares (no device calls)."""
import os
import re
import subprocess

import numpy as np
import pytest

import cumetis_gb300 as cm
from conftest import ROOT


def test_generators_match_configured_sizes():
    g = cm.gen_tri_grid(69, 69)
    assert (g.nvtxs, g.nedges) == (4761, 28016)
    g.validate()
    g = cm.gen_grid2d(725, 725)
    assert (g.nvtxs, g.nedges) == (525625, 2099600)
    g = cm.gen_grid3d(4, 5, 6)
    assert g.nvtxs == 120 and g.nedges == 2 * (3 * 5 * 6 + 4 * 4 * 6 + 4 * 5 * 5)
    g.validate()


def test_rmat_properties():
    g = cm.gen_rmat(12, 16, seed=7)
    g.validate()
    assert g.nvtxs == 4096
    assert g.adjwgt.min() >= 1 and g.adjwgt.max() <= 100
    # deterministic for a seed, different across seeds
    h = cm.gen_rmat(12, 16, seed=7)
    assert np.array_equal(g.adjncy, h.adjncy) and np.array_equal(g.adjwgt, h.adjwgt)
    assert not np.array_equal(g.adjncy, cm.gen_rmat(12, 16, seed=8).adjncy[: len(g.adjncy)])
    # skew: vertex 0 is the largest hub
    deg = np.diff(g.xadj)
    assert deg[0] == deg.max()


def test_rgg_mean_degree():
    g = cm.gen_rgg(20000, 8.0, seed=1)
    g.validate()
    assert 7.0 < g.nedges / g.nvtxs < 8.5


def test_rows_sorted():
    for g in (cm.gen_tri_grid(10, 12), cm.gen_rmat(10, seed=2), cm.gen_rgg(2000, 8.0, seed=2)):
        for v in range(g.nvtxs):
            r = g.adjncy[g.xadj[v]:g.xadj[v + 1]]
            assert np.all(np.diff(r) > 0)


def test_metis_roundtrip(tmp_path):
    for g in (cm.gen_tri_grid(7, 9), cm.gen_rmat(8, seed=1)):
        g.vwgt = (1 + np.arange(g.nvtxs) % 3).astype(np.int32)
        p = str(tmp_path / "g.graph")
        g.write(p)
        h = cm.read_graph(p)
        for a in ("xadj", "adjncy", "adjwgt", "vwgt"):
            assert np.array_equal(getattr(g, a), getattr(h, a)), a


def test_metis_reader_formats(tmp_path):
    p = tmp_path / "a.graph"
    p.write_text("% comment\n3 2\n2\n1 3\n% inner comment\n2\n")
    g = cm.read_graph(str(p))
    assert list(g.xadj) == [0, 1, 3, 4] and list(g.adjncy) == [1, 0, 2, 1]
    p.write_text("3 2 11\n5 2 7\n1 2 7 3 9\n4 2 9\n")
    g = cm.read_graph(str(p))
    assert list(g.vwgt) == [5, 1, 4] and list(g.adjwgt) == [7, 7, 9, 9]


@pytest.mark.parametrize("text", [
    "",                              # premature end
    "3\n",                           # no edge count
    "0 0\n",                         # non-positive sizes
    "2 1 112\n2\n1\n",               # unknown format
    "2 1\n3\n1\n",                   # edge out of bounds
    "2 1\n2\n",                      # premature end while reading vertices
    "2 1 1\n2\n1 1\n",               # missing edge weight
    "2 1 1\n2 0\n1 0\n",             # non-positive edge weight
    "2 1 10\n-1 2\n1 1\n",           # negative vertex weight
    "2 1\n2 2\n1\n",                 # more edges than declared
    "3 2\n2\n1\n\n",                 # fewer edges than declared
])
def test_metis_reader_errors(tmp_path, text):
    p = tmp_path / "bad.graph"
    p.write_text(text)
    with pytest.raises(cm.CMError) as e:
        cm.read_graph(str(p))
    assert e.value.code in (cm.CM_ERR_IO, cm.CM_ERR_UNSUPPORTED)


def test_missing_file():
    with pytest.raises(cm.CMError) as e:
        cm.read_graph("/nonexistent/x.graph")
    assert e.value.code == cm.CM_ERR_IO


def test_partition_file_and_cut(tmp_path):
    g = cm.gen_grid2d(4, 4)
    part = (np.arange(16) // 8).astype(np.int32)  # top / bottom halves
    assert g.edge_cut(part) == 4
    assert abs(g.imbalance(2, part) - 1.0) < 1e-9
    gp = str(tmp_path / "x.graph")
    cm.write_partition(gp, 2, part)
    lines = open(gp + ".part.2").read().split()
    assert [int(x) for x in lines] == list(part)


def test_threshold_rule():
    assert cm.coarsen_threshold(4761, 8) == 240
    assert cm.coarsen_threshold(525625, 64) == 4380
    assert cm.coarsen_threshold(4194304, 256) == 26214
    assert cm.maxvwgt_rule(4761, 240) == 29


def _declared_functions():
    text = open(os.path.join(ROOT, "include", "cm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+((?:cm|cuMetis)_[A-Za-z0-9_]+)\s*\(", text,
                       flags=re.M)
    return sorted(set(names))


def test_abi_exports_every_declared_symbol():
    lib = cm.lib()  # loads libcm.so (no device call)
    names = _declared_functions()
    assert len(names) >= 20
    assert "cuMetis_PartGraph" in names and "cm_part_graph" in names
    out = subprocess.run(["nm", "-D", "--defined-only", cm.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_no_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cm.CMError) as e:
        cm.Context(0)
    assert e.value.code == cm.CM_ERR_UNSUPPORTED


def test_cli_usage_without_arguments():
    exe = os.path.join(os.path.dirname(cm.LIB_PATH), "cuMetis")
    if not os.path.exists(exe):
        cm.lib()
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_engine_without_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cm.CMError) as e:
        cm.Engine(0, workers=2)
    assert e.value.code == cm.CM_ERR_UNSUPPORTED


MTX_CASES = {
    "symmetric": ("%%MatrixMarket matrix coordinate real symmetric\n% c\n5 5 6\n1 1 1\n2 1 1\n3 2 1\n5 3 1\n4 4 2\n5 1 3\n",
                  {(0, 1), (1, 2), (2, 4), (0, 4)}),
    "general": ("%%MatrixMarket matrix coordinate pattern general\n4 4 5\n1 2\n2 1\n3 4\n1 1\n4 2\n",
                {(0, 1), (2, 3), (1, 3)}),
    "skew": ("%%MatrixMarket matrix coordinate integer skew-symmetric\n3 3 2\n2 1 -4\n3 1 7\n", {(0, 1), (0, 2)}),
}


@pytest.mark.parametrize("name", sorted(MTX_CASES))
def test_mtx_reader(tmp_path, name):
    text, und = MTX_CASES[name]
    p = tmp_path / (name + ".mtx")
    p.write_text(text)
    g = cm.read_mtx(str(p))
    n = int(text.split("\n")[1 if not text.split("\n")[1].startswith("%") else 2].split()[0])
    pairs = sorted({(a, b) for a, b in und} | {(b, a) for a, b in und})
    xadj = np.zeros(n + 1, np.int64)
    for a, _ in pairs:
        xadj[a + 1] += 1
    np.testing.assert_array_equal(g.xadj, np.cumsum(xadj))
    np.testing.assert_array_equal(g.adjncy, [b for _, b in pairs])
    assert (g.adjwgt == 1).all() and (g.vwgt == 1).all()


@pytest.mark.parametrize("text", ["%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
                                  "%%MatrixMarket matrix coordinate real general\n3 4 1\n1 2 1\n",
                                  "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 2 1\n",
                                  "not a header\n3 3 0\n"])
def test_mtx_reader_errors(tmp_path, text):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(cm.CMError) as e:
        cm.read_mtx(str(p))
    assert e.value.code == cm.CM_ERR_IO


def test_cli_convert(tmp_path):
    p = tmp_path / "m.mtx"
    p.write_text(MTX_CASES["symmetric"][0])
    exe = os.path.join(os.path.dirname(cm.LIB_PATH), "cuMetis")
    r = subprocess.run([exe, "convert", str(p)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    g = cm.read_graph(str(tmp_path / "m.graph"))
    h = cm.read_mtx(str(p))
    np.testing.assert_array_equal(g.xadj, h.xadj)
    np.testing.assert_array_equal(g.adjncy, h.adjncy)
