"""The FIFO linearizability checker (oracle/lincheck.cpp) pinned against the
reference's shipped histories and against project-written negatives."""
import json
import os
import random

import numpy as np
import pytest

from make_golden import mutations, _load

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = ["history_gwfq_m0_t32_o8.jsonl", "history_glfq_m0_t64_o16.jsonl"]


@pytest.mark.parametrize("name", FIXTURES)
def test_reference_histories_linearizable(oracle_lib, name):
    # correctness/histories/*.jsonl: the reference documents both as linearizable
    recs = oracle_lib.load_jsonl(os.path.join(GOLDEN, name))
    manifest = json.load(open(os.path.join(GOLDEN, "manifest.json")))[name]
    assert len(recs) == manifest["records"]
    assert int(((recs["op"] == 0) & (recs["ret"] == 1)).sum()) == manifest["ok_enq"]
    assert oracle_lib.check(recs) == "Linearizable (FIFO)"
    assert oracle_lib.search(recs) == "Linearizable (FIFO)"
    assert not oracle_lib.patterns(recs)["violations"]


@pytest.mark.parametrize("name", FIXTURES)
def test_mutated_histories_rejected(oracle_lib, name):
    seen = []
    for mname, m in mutations(_load(os.path.join(GOLDEN, name))):
        assert oracle_lib.check(oracle_lib.records_from_dicts(m)) == "Not linearizable (FIFO)", mname
        seen.append(mname)
    assert set(seen) == {"swapped_deq", "duplicate_deq", "phantom_value", "empty_while_nonempty"}


def test_cli_matches_reference_contract(oracle_lib, tmp_path):
    import subprocess
    from oracle import build
    cli = os.path.join(build.OUT, "lincheck")
    r = subprocess.run([cli, os.path.join(GOLDEN, FIXTURES[0])], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "Linearizable (FIFO)"
    bad = list(mutations(_load(os.path.join(GOLDEN, FIXTURES[0]))))[0][1]
    p = tmp_path / "bad.jsonl"
    p.write_text("".join(json.dumps(x) + "\n" for x in bad))
    r = subprocess.run([cli, str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.strip() == "Not linearizable (FIFO)"


def _random_history(rng, n_ops, n_procs, vals):
    """Random interval history: each process runs ops back to back with random gaps."""
    recs, t = [], 1
    events = []
    for p in range(n_procs):
        t = rng.randint(1, 4)
        for _ in range(n_ops // n_procs):
            call = t
            end = call + rng.randint(1, 6)
            t = end + rng.randint(1, 3)
            op = rng.choice([0, 1, 1, 2]) if vals else 0
            if op == 0:
                arg = rng.choice(vals)
                ret = rng.choice([1, 1, 1, 0])
            elif op == 1:
                arg, ret = 0, rng.choice([0] + vals)
            else:
                arg, ret = 0, 0
            events.append(dict(proc=p, op=op, arg=arg, ret=ret, call=call * 10 + p, end=end * 10 + p))
    return events


def test_search_agrees_with_brute_force(oracle_lib):
    """Exact search vs exhaustive enumeration on 600 random small histories."""
    rng = random.Random(1234)
    agree = {True: 0, False: 0}
    for it in range(600):
        vals = [rng.randint(1, 4) for _ in range(3)]
        h = _random_history(rng, rng.choice([4, 6]), rng.choice([2, 3]), vals)
        if not h:
            continue
        a = oracle_lib.records_from_dicts(h)
        want = oracle_lib.brute_force(a)
        got = oracle_lib.search(a, timeout_s=5.0)
        assert got == ("Linearizable (FIFO)" if want else "Not linearizable (FIFO)"), (h, want, got)
        agree[want] += 1
    # both verdicts must have been exercised
    assert agree[True] > 50 and agree[False] > 50, agree


def test_patterns_are_sound(oracle_lib):
    """Every history the pattern scan rejects is rejected by brute force too."""
    rng = random.Random(99)
    flagged = 0
    for it in range(400):
        # distinct values so the pattern procedure applies
        n = rng.choice([4, 6])
        h = _random_history(rng, n, rng.choice([2, 3]), list(range(1, 9)))
        seen, ok = set(), True
        for r in h:
            if r["op"] == 0:
                if r["arg"] in seen:
                    ok = False
                seen.add(r["arg"])
        if not ok:
            continue
        a = oracle_lib.records_from_dicts(h)
        if oracle_lib.patterns(a)["violations"]:
            flagged += 1
            assert not oracle_lib.brute_force(a), h
    assert flagged > 20


def test_empty_overlapping_values_linearizable(oracle_lib):
    """An "empty" overlapping the dequeue of one value and the enqueue of the next
    can be placed between them: linearizable, and the checker must say so."""
    h = [
        dict(proc=0, op=0, arg=1, ret=1, call=1, end=2),     # enq(1)
        dict(proc=1, op=0, arg=2, ret=1, call=3, end=10),    # enq(2) overlaps everything below
        dict(proc=0, op=1, arg=0, ret=1, call=4, end=8),     # deq -> 1
        dict(proc=2, op=1, arg=0, ret=0, call=5, end=12),    # "empty"
        dict(proc=0, op=1, arg=0, ret=2, call=13, end=14),   # deq -> 2
    ]
    a = oracle_lib.records_from_dicts(h)
    assert oracle_lib.brute_force(a)
    assert oracle_lib.check(a) == "Linearizable (FIFO)"
    assert oracle_lib.search(a) == "Linearizable (FIFO)"


def test_empty_covered_by_chain_rejected(oracle_lib):
    """No single value spans the "empty", but value 1 is queued until deq(1) is
    called at 8 and value 2 from the end of its enqueue at 7: every instant of the
    empty dequeue has a value queued."""
    h = [
        dict(proc=0, op=0, arg=1, ret=1, call=1, end=2),
        dict(proc=1, op=0, arg=2, ret=1, call=6, end=7),
        dict(proc=2, op=1, arg=0, ret=0, call=5, end=12),    # "empty"
        dict(proc=0, op=1, arg=0, ret=1, call=8, end=9),
        dict(proc=0, op=1, arg=0, ret=2, call=13, end=14),
    ]
    a = oracle_lib.records_from_dicts(h)
    assert not oracle_lib.brute_force(a)
    assert oracle_lib.patterns(a)["empty"] == 1
    assert oracle_lib.check(a) == "Not linearizable (FIFO)"
    assert oracle_lib.search(a) == "Not linearizable (FIFO)"


def test_patterns_complete_without_empties(oracle_lib):
    """With distinct values and no "empty" dequeue, a history without patterns is
    linearizable (and the pattern verdict alone decides check())."""
    rng = random.Random(7)
    n_lin = n_bad = 0
    for it in range(500):
        h = _random_history(rng, rng.choice([4, 6, 8]), rng.choice([2, 3, 4]), list(range(1, 12)))
        seen, ok = set(), True
        for r in h:
            if r["op"] == 0:
                ok &= r["arg"] not in seen
                seen.add(r["arg"])
            if r["op"] == 1 and r["ret"] == 0:
                r["op"] = 2     # no empties: turn them into no-ops
        if not ok:
            continue
        a = oracle_lib.records_from_dicts(h)
        want = oracle_lib.brute_force(a)
        assert (not oracle_lib.patterns(a)["violations"]) == want, h
        assert oracle_lib.check(a) == ("Linearizable (FIFO)" if want else "Not linearizable (FIFO)")
        n_lin += want
        n_bad += not want
    assert n_lin > 30 and n_bad > 30, (n_lin, n_bad)


def test_search_with_distinct_values_agrees_with_brute_force(oracle_lib):
    """Distinct values with "empty" dequeues: exercises the FIFO-order pruning of
    the exact search against exhaustive enumeration."""
    rng = random.Random(2024)
    counts = {True: 0, False: 0}
    for it in range(800):
        h = _random_history(rng, rng.choice([4, 6, 8]), rng.choice([2, 3, 4]), list(range(1, 12)))
        seen, ok = set(), True
        for r in h:
            if r["op"] == 0:
                ok &= r["arg"] not in seen
                seen.add(r["arg"])
        if not ok:
            continue
        a = oracle_lib.records_from_dicts(h)
        want = oracle_lib.brute_force(a)
        assert oracle_lib.search(a) == ("Linearizable (FIFO)" if want else "Not linearizable (FIFO)"), h
        assert oracle_lib.check(a) == ("Linearizable (FIFO)" if want else "Not linearizable (FIFO)"), h
        counts[want] += 1
    assert counts[True] > 40 and counts[False] > 40, counts


def synthetic_history(rng, producers, consumers, ops_per_thread, overlap=40):
    """A history that is linearizable by construction: every operation gets an
    interval and a linearisation point inside it, and the results come from a real
    FIFO applied in point order.  Producers/consumers run back to back with long,
    overlapping intervals, so there are many concurrent "empty" dequeues."""
    ops = []
    for p in range(producers + consumers):
        t = rng.randint(0, overlap)
        for i in range(ops_per_thread):
            call = t
            end = call + rng.randint(1, overlap)
            lin = rng.uniform(call, end)
            kind = 0 if p < producers else 1
            val = (p << 32) | (i + 1)
            ops.append([lin, p, kind, val, call, end])
            t = end + rng.randint(0, overlap // 4)
    ops.sort()
    q, recs = [], []
    for lin, p, kind, val, call, end in ops:
        if kind == 0:
            q.append(val)
            recs.append(dict(proc=p, op=0, arg=val, ret=1, call=call, end=end))
        else:
            ret = q.pop(0) if q else 0
            recs.append(dict(proc=p, op=1, arg=0, ret=ret, call=call, end=end))
    # distinct logical timestamps: spread ties deterministically
    stamps = sorted({(r["call"], 0, i) for i, r in enumerate(recs)} | {(r["end"], 1, i) for i, r in enumerate(recs)})
    for k, (_, is_end, i) in enumerate(stamps):
        recs[i]["end" if is_end else "call"] = k + 1
    # ties resolved call-before-end only within equal times; keep call < end per op
    for r in recs:
        assert r["call"] < r["end"]
    return recs


@pytest.mark.parametrize("producers,consumers,ops", [(8, 24, 16), (8, 24, 6), (48, 16, 16), (4, 60, 8)])
def test_synthetic_split_histories(oracle_lib, producers, consumers, ops):
    """Exact verdicts on split-mode-like histories at the sizes the split GPU tests
    use.  (The exact search is exponential in the worst case, like the reference's
    Porcupine search; much larger split histories can end "Unknown (timeout)".)"""
    import time
    rng = random.Random(producers * 1000 + consumers)
    for it in range(5):
        recs = synthetic_history(rng, producers, consumers, ops)
        a = oracle_lib.records_from_dicts(recs)
        t0 = time.time()
        assert oracle_lib.check(a, timeout_s=30) == "Linearizable (FIFO)"
        assert time.time() - t0 < 10


@pytest.mark.parametrize("producers,consumers,ops", [(64, 192, 16), (256, 256, 16)])
def test_synthetic_large_patterns(oracle_lib, producers, consumers, ops):
    """Large histories: the pattern scan finds nothing in a linearizable history and
    flags a swapped pair of dequeues."""
    rng = random.Random(producers)
    recs = synthetic_history(rng, producers, consumers, ops)
    a = oracle_lib.records_from_dicts(recs)
    assert not oracle_lib.patterns(a)["violations"]
    deqs = [i for i, r in enumerate(recs) if r["op"] == 1 and r["ret"]]
    by_val = {r["arg"]: r for r in recs if r["op"] == 0}
    for i in deqs:
        for j in deqs:
            if recs[i]["end"] < recs[j]["call"] and by_val[recs[i]["ret"]]["end"] < by_val[recs[j]["ret"]]["call"]:
                recs[i]["ret"], recs[j]["ret"] = recs[j]["ret"], recs[i]["ret"]
                b = oracle_lib.records_from_dicts(recs)
                assert oracle_lib.patterns(b)["order"] >= 1
                assert oracle_lib.check(b) == "Not linearizable (FIFO)"
                return
    pytest.fail("no swappable pair")
