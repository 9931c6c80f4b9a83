"""Host-side graph generators and the served-BFS checksum (no GPU calls)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def gcq_host():
    import gcq_gb300
    from gcq_gb300 import build
    build.build()
    return gcq_gb300


def _check_csr(off, idx):
    V = len(off) - 1
    assert off[0] == 0 and off[-1] == len(idx)
    assert (np.diff(off) >= 0).all()
    assert ((idx >= 0) & (idx < V)).all()
    src = np.repeat(np.arange(V), np.diff(off))
    assert (src != idx).all(), "self loop"
    for v in range(0, V, max(1, V // 200)):
        row = idx[off[v]:off[v + 1]]
        assert (np.diff(row) > 0).all(), "unsorted or duplicate neighbours"
    fwd = set(zip(src.tolist(), idx.tolist()))
    assert all((b, a) in fwd for a, b in list(fwd)[:20000]), "not undirected"


def test_rmat_shape_and_determinism(gcq_host):
    off, idx = gcq_host.graph_rmat(10, 16, seed=7)
    assert len(off) == 1025
    _check_csr(off, idx)
    off2, idx2 = gcq_host.graph_rmat(10, 16, seed=7)
    assert np.array_equal(off, off2) and np.array_equal(idx, idx2)
    off3, idx3 = gcq_host.graph_rmat(10, 16, seed=8)
    assert not (np.array_equal(off, off3) and np.array_equal(idx, idx3))
    deg = np.diff(off)
    assert deg.max() > 8 * max(1.0, deg.mean())   # skewed degrees


def test_grid_shape(gcq_host):
    off, idx = gcq_host.graph_grid(40, 50, 1.0, 0.0, 0)
    _check_csr(off, idx)
    assert len(idx) == 2 * (40 * 49 + 39 * 50)    # every 4-neighbour edge, both directions
    off, idx = gcq_host.graph_grid(40, 50, 0.6, 0.01, 2)
    _check_csr(off, idx)


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15))
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def test_levels_checksum_restatement(oracle_lib):
    rng = np.random.default_rng(1)
    lv = rng.integers(-1, 50, size=5000).astype(np.int32)
    v = np.arange(len(lv), dtype=np.uint64)
    l = np.where(lv < 0, np.uint64(0xFFFFFFFF), lv.astype(np.uint64))
    with np.errstate(over="ignore"):
        want = int(np.sum(_splitmix64((v << np.uint64(32)) | l), dtype=np.uint64))
    assert oracle_lib.levels_checksum(lv) == want


def test_bfs_summary(oracle_lib):
    # path 0-1-2, isolated 3
    off = np.array([0, 1, 3, 4, 4], np.int32)
    idx = np.array([1, 0, 2, 1], np.int32)
    cs, reached, ecc = oracle_lib.bfs_summary(off, idx, 0)
    assert (reached, ecc) == (3, 2)
    assert cs == oracle_lib.levels_checksum(np.array([0, 1, 2, -1], np.int32))


def _csr_from_edges(V, pairs):
    """csr_from_edges after sort + unique (bfs_bench.cpp:186-200, 222-223), in numpy."""
    e = sorted(set(pairs))
    off = np.zeros(V + 1, np.int64)
    for u, _ in e:
        off[u + 1] += 1
    return np.cumsum(off).astype(np.int32), np.array([v for _, v in e], np.int32)


def test_load_mtx(gcq_host, tmp_path):
    p = tmp_path / "g.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% comment\n"
                 "6 5 7\n1 2\n2 3\n3 3\n% inline comment\n4 2\n2 1\n7 1\n5 6\n")
    off, idx = gcq_host.graph_load(str(p))
    # 3-3 self loop dropped, 7-1 out of range (rows = 6), 5-6: column 6 > cols = 5 dropped,
    # 2-1 duplicates 1-2; V = max(6, 5)
    pairs = []
    for u, v in [(0, 1), (1, 2), (3, 1), (1, 0)]:
        pairs += [(u, v), (v, u)]
    want = _csr_from_edges(6, pairs)
    assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])


def test_load_snap(gcq_host, tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("# Directed graph\n# FromNodeId ToNodeId\n1 2\n2 3\n3 1\n4 4\n5 3\n2 3\n")
    off, idx = gcq_host.graph_load(str(p))
    # smallest id is 1: shifted down; V = 5; 4-4 dropped
    pairs = []
    for u, v in [(0, 1), (1, 2), (2, 0), (4, 2), (1, 2)]:
        pairs += [(u, v), (v, u)]
    want = _csr_from_edges(5, pairs)
    assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
    p0 = tmp_path / "g0.txt"
    p0.write_text("0 1\n1 2\n")
    off, idx = gcq_host.graph_load(str(p0))
    assert len(off) == 4 and list(idx) == [1, 0, 2, 1]


def test_load_rejects(gcq_host, tmp_path):
    import gcq_gb300
    bad = tmp_path / "bad.mtx"
    bad.write_text("not a matrix market file\n1 2\n")
    with pytest.raises(gcq_gb300.GcqError):
        gcq_host.graph_load(str(bad))
    with pytest.raises(gcq_gb300.GcqError):
        gcq_host.graph_load(str(tmp_path / "missing.mtx"))


@pytest.mark.parametrize("which", ["grid", "rmat"])
def test_oracle_bfs_against_scipy(gcq_host, oracle_lib, which):
    """The serial BFS that pins every GPU traversal, against an independent
    implementation (scipy's unweighted shortest paths) on generated graphs."""
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    if which == "grid":
        off, idx = gcq_host.graph_grid(60, 70, 0.6, 0.01, 3)
    else:
        off, idx = gcq_host.graph_rmat(11, 8, 0.57, 0.19, 0.19, seed=4)
    V = len(off) - 1
    A = sp.csr_matrix((np.ones(len(idx)), idx, off), shape=(V, V))
    for src in (0, V // 3, V - 1):
        want = csgraph.shortest_path(A, method="D", unweighted=True, indices=src)
        want = np.where(np.isinf(want), -1, want).astype(np.int32)
        got, ecc = oracle_lib.bfs(off, idx, src)
        assert np.array_equal(got, want), (which, src)
        assert ecc == want.max()
