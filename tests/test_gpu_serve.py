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
