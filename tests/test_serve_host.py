"""Host-side logic of the served engine's Python layer, without a GPU."""


def test_serve_autotune_picks_fastest(monkeypatch):
    """Selection logic of serve_autotune with a stand-in server (no GPU): the
    candidate with the highest request rate wins; failing candidates are skipped."""
    import numpy as np
    import gcq_gb300 as gcq   # host-side helpers only: no library load

    ms = {(32768, 28): 4.0, (32768, 29): 2.0, (65536, 28): None, (65536, 29): 1.0}

    class FakeServer:
        def __init__(self, graphs, threads=0, work_log2=0, **kw):
            self.k = (threads, work_log2)
            if ms[self.k] is None:
                raise gcq.GcqError(gcq.ECAPACITY, "fake")

        def run(self, reqs):
            return None, {"kernel_ms": ms[self.k]}

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    monkeypatch.setattr(gcq, "Server", FakeServer)
    reqs = np.zeros(10, dtype=gcq.SERVE_REQ_DTYPE)
    cands = [dict(threads=t, work_log2=w) for t in (32768, 65536) for w in (28, 29)]
    best, table = gcq.serve_autotune([], reqs, candidates=cands)
    assert best == dict(threads=65536, work_log2=29)
    assert [r for _, r in table] == [2500.0, 5000.0, None, 10000.0]
