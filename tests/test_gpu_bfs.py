"""BFS parity: depths from the GPU traversal (every queue, level-synchronous and
persistent) must equal the serial BFS of the oracle bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = ["gwfq", "glfq", "wfq", "sfq"]
SEED = 2   # vertex 0 lies in the giant component of both benchmark graphs with seed 2


@pytest.fixture(scope="module")
def graph_b(gcq):
    return gcq.graph_grid(212, 212, 0.6, 0.01, SEED)


def _serial(oracle_lib, off, idx, src=0):
    lv = np.empty(len(off) - 1, np.int32)
    oracle_lib.lib().oracle_bfs(len(off) - 1, off.ctypes.data, idx.ctypes.data, src, lv.ctypes.data)
    return lv


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("threads", [512, 8192])
def test_bfs_graph_b_plain(gcq, oracle_lib, graph_b, kind, threads):
    off, idx = graph_b
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs(kind, off, idx, threads=threads) as b:
        for rep in range(2):
            r, lv = b.run(src=0, block=256)
            assert np.array_equal(lv, want)
            assert r["reached"] == int((want >= 0).sum())
            assert r["levels"] == int(want.max()) + 1
            assert r["drops"] == 0


@pytest.mark.parametrize("kind", ["gwfq", "glfq", "sfq"])
def test_bfs_graph_b_persistent(gcq, oracle_lib, graph_b, kind):
    off, idx = graph_b
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs(kind, off, idx, threads=8192) as b:
        r, lv = b.run(src=0, block=256, persistent=True)
        assert np.array_equal(lv, want)
        assert r["reached"] == int((want >= 0).sum())


@pytest.mark.parametrize("kind", KINDS)
def test_bfs_full_grid_and_other_sources(gcq, oracle_lib, kind):
    # the reference's build_grid (every 4-neighbour edge), several sources
    off, idx = gcq.graph_grid(64, 96, 1.0, 0.0, 0)
    with gcq.Bfs(kind, off, idx, threads=1024) as b:
        for src in [0, 17, 64 * 96 - 1, 3000]:
            r, lv = b.run(src=src, block=128)
            assert np.array_equal(lv, _serial(oracle_lib, off, idx, src))


def test_bfs_hub_and_warp_paths(gcq, oracle_lib):
    """A star with a 5000-neighbour hub (hub kernel) and 100-neighbour vertices
    (warp-cooperative path) next to low-degree chains (inline path)."""
    rng = np.random.default_rng(3)
    V = 20000
    edges = set()
    for w in range(1, 5001):
        edges.add((0, w))
    for h in range(5001, 5101):          # medium-degree vertices
        for w in rng.choice(np.arange(5101, V), 100, replace=False):
            edges.add((h, int(w)))
        edges.add((int(rng.integers(1, 5001)), h))
    for v in range(5101, V - 1):
        edges.add((v, v + 1))
    und = sorted({(a, b) for a, b in edges} | {(b, a) for a, b in edges})
    src = np.array([a for a, b in und], np.int32)
    dst = np.array([b for a, b in und], np.int32)
    off = np.zeros(V + 1, np.int32)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    idx = dst[np.argsort(src, kind="stable")].astype(np.int32)
    want = _serial(oracle_lib, off, idx)
    for kind in ["gwfq", "glfq"]:
        with gcq.Bfs(kind, off, idx, threads=2048) as b:
            for persistent in (False, True):
                r, lv = b.run(src=0, block=256, persistent=persistent)
                assert np.array_equal(lv, want), (kind, persistent)


def test_bfs_graph_a_gwfq(gcq, oracle_lib):
    # the 4096 x 4096 benchmark graph, once per form, depths bit-exact
    off, idx = gcq.graph_grid(4096, 4096, 0.6, 0.01, SEED)
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs("gwfq", off, idx, threads=8192) as b:
        for persistent in (False, True):
            r, lv = b.run(src=0, block=256, persistent=persistent)
            assert np.array_equal(lv, want)
            assert r["levels"] == int(want.max()) + 1


# ------------------------------------------------------- asynchronous (persistent=2)
@pytest.mark.parametrize("kind", ["gwfq", "glfq"])
def test_bfs_async_graph_b_and_grid(gcq, oracle_lib, graph_b, kind):
    """The label-correcting form gives the same depths, whatever the order."""
    off, idx = graph_b
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs(kind, off, idx, threads=16384) as b:
        for rep in range(3):
            r, lv = b.run(src=0, block=256, persistent=2)
            assert np.array_equal(lv, want)
            assert r["reached"] == int((want >= 0).sum())
            assert r["levels"] == int(want.max()) + 1
    off, idx = gcq.graph_grid(64, 96, 1.0, 0.0, 0)
    with gcq.Bfs(kind, off, idx, threads=2048) as b:
        for src in [0, 17, 64 * 96 - 1]:
            r, lv = b.run(src=src, block=256, persistent=2)
            assert np.array_equal(lv, _serial(oracle_lib, off, idx, src))


def test_bfs_async_hubs_and_rmat(gcq, oracle_lib):
    off, idx = gcq.graph_rmat(14, 16, seed=9)      # skewed degrees: warp-wide expansion
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs("gwfq", off, idx, threads=65536) as b:
        r, lv = b.run(src=0, block=256, persistent=2)
        assert np.array_equal(lv, want)
        assert r["edges_scanned"] >= int(np.diff(off)[want >= 0].sum())   # every reached vertex expanded


def test_bfs_async_graph_a(gcq, oracle_lib):
    off, idx = gcq.graph_grid(4096, 4096, 0.6, 0.01, SEED)
    want = _serial(oracle_lib, off, idx)
    with gcq.Bfs("gwfq", off, idx, threads=65536) as b:
        r, lv = b.run(src=0, block=256, persistent=2)
        assert np.array_equal(lv, want)
        assert r["levels"] == int(want.max()) + 1


@pytest.mark.parametrize("kind", ["sfq", "wfq"])
def test_bfs_async_unsupported(gcq, graph_b, kind):
    off, idx = graph_b
    with gcq.Bfs(kind, off, idx, threads=512) as b:
        with pytest.raises(gcq.GcqError) as e:
            b.run(src=0, block=256, persistent=2)
        assert e.value.status == gcq.EUNSUPPORTED
