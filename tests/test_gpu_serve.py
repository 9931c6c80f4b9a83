"""Served BFS parity: every request answered by the persistent server must carry
the checksum, reached count and eccentricity of the oracle's serial BFS from the
same source, whatever the arrival schedule, slot reuse or graph mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 2
LIMITS = dict(timeout_s=5.0, run_limit_s=20.0)   # every run returns within ~20 s


def _star_chain(n_hub=5000, n_mid=100):
    """A hub of n_hub leaves, vertices of degree ~100 and a long chain: exercises
    the warp-wide path, the inline path and a deep traversal."""
    edges = []
    v = 1
    for _ in range(n_hub):
        edges.append((0, v)); v += 1
    mids = []
    for m in range(3):
        c = v; v += 1
        mids.append(c)
        edges.append((0, c))
        for _ in range(n_mid):
            edges.append((c, v)); v += 1
    prev = mids[-1]
    for _ in range(3000):
        edges.append((prev, v)); prev = v; v += 1
    V = v + 5   # a few isolated vertices
    return _csr(V, edges)


def _csr(V, edges):
    e = np.array(edges, dtype=np.int64)
    src = np.concatenate([e[:, 0], e[:, 1]])
    dst = np.concatenate([e[:, 1], e[:, 0]])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.int32), dst.astype(np.int32)


@pytest.fixture(scope="module")
def graphs(gcq):
    return [
        gcq.graph_grid(212, 212, 0.6, 0.01, SEED),   # the small benchmark grid
        gcq.graph_rmat(12, 16, seed=5),
        gcq.graph_rmat(14, 8, seed=6),
        gcq.graph_grid(64, 96, 1.0, 0.0, 0),          # full grid
        _star_chain(),
    ]


@pytest.fixture(scope="module")
def expected(oracle_lib, graphs):
    cache = {}

    def get(g, src):
        key = (g, int(src))
        if key not in cache:
            off, idx = graphs[g]
            cache[key] = oracle_lib.bfs_summary(off, idx, int(src))
        return cache[key]
    return get


def _check(res, reqs, expected):
    for i in range(len(reqs)):
        want = expected(int(reqs[i]["graph"]), int(reqs[i]["src"]))
        got = (int(res[i]["checksum"]), int(res[i]["reached"]), int(res[i]["max_level"]))
        assert got == want, (i, reqs[i], got, want)
        assert res[i]["admit_ns"] >= reqs[i]["arrival_ns"]
        assert res[i]["admit_ns"] <= res[i]["done_ns"] <= res[i]["finish_ns"]


def test_serve_closed_batch(gcq, graphs, expected):
    V = [len(o) - 1 for o, _ in graphs]
    reqs = gcq.serve_requests(300, len(graphs), V, rate_per_s=0, seed=11)
    reqs["src"][:5] = 0
    with gcq.Server(graphs, budget_bytes=1 << 30, threads=32768, **LIMITS) as s:
        res, st = s.run(reqs)
        _check(res, reqs, expected)
        assert st["completed"] == len(reqs)
        assert st["error_word"] == 0
        assert st["items"] >= int(res["reached"].sum())   # every reached vertex expanded at least once


def test_serve_poisson_and_reuse(gcq, graphs, expected):
    """Open-loop arrivals; a tiny budget forces few slots per graph, so level arrays
    are swept and reused many times; a second run reuses the server."""
    V = [len(o) - 1 for o, _ in graphs]
    per_graph = max(V) * 4 * 2          # two slots of the largest graph
    with gcq.Server(graphs, budget_bytes=per_graph * len(graphs), max_slots=2, threads=16384, **LIMITS) as s:
        assert s.info()["slots"] <= 2 * len(graphs)
        for seed, rate in [(21, 2e4), (22, 0)]:
            reqs = gcq.serve_requests(200, len(graphs), V, rate_per_s=rate, seed=seed)
            res, st = s.run(reqs)
            _check(res, reqs, expected)
            if rate:
                assert reqs["arrival_ns"][-1] > 0


def test_serve_default_threads(gcq, graphs, expected):
    """Every resident thread, one graph, the same source many times."""
    reqs = np.zeros(64, dtype=gcq.SERVE_REQ_DTYPE)
    reqs["graph"] = 0                               # the server holds graphs[1] only
    reqs["src"] = np.arange(64) * 37 % (len(graphs[1][0]) - 1)
    with gcq.Server(graphs[1:2], **LIMITS) as s:
        res, st = s.run(reqs)
    for i in range(len(reqs)):
        assert (int(res[i]["checksum"]), int(res[i]["reached"]), int(res[i]["max_level"])) == \
            expected(1, int(reqs[i]["src"]))


def test_serve_rejects(gcq, graphs):
    V = [len(o) - 1 for o, _ in graphs]
    with gcq.Server(graphs[:2], budget_bytes=1 << 28, threads=4096, **LIMITS) as s:
        bad = gcq.serve_requests(4, 2, V[:2], seed=1)
        bad["graph"][1] = 7
        with pytest.raises(gcq.GcqError) as e:
            s.run(bad)
        assert e.value.status == gcq.EINVAL
        bad = gcq.serve_requests(4, 2, V[:2], rate_per_s=1e3, seed=1)
        bad["arrival_ns"][2] = 0                    # not sorted by arrival
        with pytest.raises(gcq.GcqError) as e:
            s.run(bad)
        assert e.value.status == gcq.EINVAL
        bad = gcq.serve_requests(4, 2, V[:2], seed=1)
        bad["src"][0] = V[bad["graph"][0]]          # source out of range
        with pytest.raises(gcq.GcqError) as e:
            s.run(bad)
        assert e.value.status == gcq.EINVAL
        ok = gcq.serve_requests(8, 2, V[:2], seed=3)   # still serves after rejections
        res, _ = s.run(ok)
        assert (res["finish_ns"] > 0).all()
    with pytest.raises(gcq.GcqError) as e:
        gcq.Server(graphs[:1], budget_bytes=16)       # not one level array fits
    assert e.value.status == gcq.ECAPACITY


# ---------------------------------------------------------------- ray tiles
def _bounce_image(oracle_lib, scene, w, h, bounces=4, seed=1):
    img = np.zeros((h, w, 3), np.float32)
    n = oracle_lib.lib().oracle_rt_bounce_render(scene, w, h, bounces, seed, 16, img.ctypes.data)
    return img, n


def _check_tiles(gcq, res, reqs, ngraphs, images, tile_px=32):
    for i in range(len(reqs)):
        tgt = int(reqs[i]["graph"])
        if tgt < ngraphs:
            continue
        want = gcq.tile_checksum(images[tgt - ngraphs], int(reqs[i]["src"]), tile_px)
        assert int(res[i]["checksum"]) == want, (i, reqs[i])
        assert res[i]["reached"] >= (tile_px * tile_px) and res[i]["max_level"] >= 1
        assert res[i]["admit_ns"] <= res[i]["done_ns"] <= res[i]["finish_ns"]


def test_serve_tiles_full_image(gcq, oracle_lib):
    """Every 32x32 tile of both 1024x1024 scenes as a request, no graphs: the served
    images equal the serial renders bit for bit, each tile's checksum matches, and
    the tiles' ray counts add up to the render's."""
    images = [_bounce_image(oracle_lib, s, 1024, 1024) for s in (0, 1)]
    reqs = np.zeros(2048, dtype=gcq.SERVE_REQ_DTYPE)
    reqs["graph"] = np.repeat([0, 1], 1024)
    reqs["src"] = np.tile(np.arange(1024), 2)
    with gcq.Server([], rt_scenes=2, threads=65536, **LIMITS) as s:
        res, st = s.run(reqs)
        for sc in (0, 1):
            assert np.array_equal(s.image(sc).view(np.uint32), images[sc][0].view(np.uint32)), sc
            assert int(res["reached"][reqs["graph"] == sc].sum()) == images[sc][1]
        _check_tiles(gcq, res, reqs, 0, [im for im, _ in images])
        assert st["rays"] == images[0][1] + images[1][1]
        assert st["completed"] == len(reqs) and st["error_word"] == 0


def test_serve_mixed_poisson(gcq, oracle_lib, graphs, expected):
    """Traversals and tiles of both scenes interleaved, open-loop arrivals, few tile
    slots (reused many times) and a second run on the same server."""
    images = [_bounce_image(oracle_lib, s, 256, 192, bounces=5, seed=3)[0] for s in (0, 1)]
    ng = len(graphs)
    V = [len(o) - 1 for o, _ in graphs]
    with gcq.Server(graphs, budget_bytes=1 << 30, threads=32768, rt_scenes=2, rt_size=(256, 192),
                    rt_max_bounces=5, rt_seed=3, rt_slots=8, **LIMITS) as s:
        assert s.rt_tiles == 48
        for seed, rate in [(31, 3e4), (32, 0)]:
            rng = np.random.default_rng(seed)
            reqs = gcq.serve_requests(400, ng + 2, V + [48, 48], rate_per_s=rate, seed=seed)
            tiles = reqs["graph"] >= ng
            reqs["src"][tiles] = rng.integers(0, 48, size=int(tiles.sum()))
            res, st = s.run(reqs)
            bfs = ~tiles
            _check(res[bfs], reqs[bfs], expected)
            _check_tiles(gcq, res, reqs, ng, images)
            assert st["completed"] == len(reqs)


def test_serve_tiles_reject(gcq, graphs):
    with gcq.Server(graphs[:1], budget_bytes=1 << 28, threads=4096, rt_scenes=1, **LIMITS) as s:
        bad = np.zeros(2, dtype=gcq.SERVE_REQ_DTYPE)
        bad["graph"] = [1, 1]
        bad["src"] = [0, 1024]                       # tile index out of range
        with pytest.raises(gcq.GcqError) as e:
            s.run(bad)
        assert e.value.status == gcq.EINVAL
        bad["graph"][1] = 2                          # scene 1 is not served
        bad["src"][1] = 0
        with pytest.raises(gcq.GcqError) as e:
            s.run(bad)
        assert e.value.status == gcq.EINVAL
        with pytest.raises(gcq.GcqError) as e:
            s.image(1)
        assert e.value.status == gcq.EINVAL
