"""Regenerate the golden fixtures under tests/golden/.

Two kinds of fixture live here:

* ``history_gwfq_m0_t32_o8.jsonl`` and ``history_glfq_m0_t64_o16.jsonl`` are the
  histories that gCQ ships in ``correctness/histories/``.  They were recorded by
  the reference's history harness (correctness/history.cpp:188-205, records
  written by correctness/history.cpp:249-283) and the reference documents both
  as "Linearizable (FIFO)" under its Porcupine checker
  (correctness/lincheck/main.go:138-159, README.md:139-140).  They are copied
  byte for byte so the CPU checker can be pinned against them.
* ``mutations(records)`` derives negative histories from those two in memory;
  each must be rejected as "Not linearizable (FIFO)".  The reference ships no
  negative fixtures, so these are project-written.  The tests call it directly
  instead of committing the mutated copies.

Run from the repository root:  python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = ["history_gwfq_m0_t32_o8.jsonl", "history_glfq_m0_t64_o16.jsonl"]


def _load(path):
    with open(path) as f:
        return [json.loads(line) for line in f if line.strip()]


def _dump(recs, path):
    with open(path, "w") as f:
        for r in recs:
            f.write(json.dumps(r, separators=(",", ":")) + "\n")


def mutations(recs):
    """Yield (name, records) pairs, each a history that a FIFO queue cannot produce."""
    deqs = [i for i, r in enumerate(recs) if r["op"] == 1 and r["ret"] != 0]
    enqs = [i for i, r in enumerate(recs) if r["op"] == 0 and r["ret"] == 1]

    # 1. Two successful dequeues return each other's values, where the first
    #    returned value's enqueue completed strictly before the second's began
    #    and both dequeues are ordered in real time: FIFO order is broken.
    by_val = {recs[i]["arg"]: i for i in enqs}
    best = None
    for a in deqs:
        for b in deqs:
            if recs[a]["end"] >= recs[b]["call"]:
                continue  # need deq a strictly before deq b
            ea, eb = by_val[recs[a]["ret"]], by_val[recs[b]["ret"]]
            if recs[ea]["end"] < recs[eb]["call"]:
                best = (a, b)
                break
        if best:
            break
    if best:
        out = [dict(r) for r in recs]
        a, b = best
        out[a]["ret"], out[b]["ret"] = out[b]["ret"], out[a]["ret"]
        yield "swapped_deq", out

    # 2. A value dequeued twice.
    out = [dict(r) for r in recs]
    out[deqs[-1]]["ret"] = out[deqs[0]]["ret"]
    yield "duplicate_deq", out

    # 3. A dequeue returns a value that was never enqueued.
    out = [dict(r) for r in recs]
    out[deqs[len(deqs) // 2]]["ret"] = 0xDEADBEEF0000 + 7
    yield "phantom_value", out

    # 4. A dequeue reports "empty" (ret 0) although an enqueue finished before it
    #    started and no dequeue could have taken that value: a late dequeue whose
    #    call is after every enqueue's end, with more enqueues than successful
    #    dequeues before it.  Turn the last successful dequeue into "empty" and
    #    drop nothing else; then the value it returned is never dequeued while an
    #    empty result is observed after every enqueue completed.
    last_enq_end = max(recs[i]["end"] for i in enqs)
    late = [i for i in deqs if recs[i]["call"] > last_enq_end]
    if late:
        out = [dict(r) for r in recs]
        out[late[-1]]["ret"] = 0
        yield "empty_while_nonempty", out


def main(ref_root):
    manifest = {}
    for name in FIXTURES:
        src = os.path.join(ref_root, "correctness", "histories", name)
        with open(src, "rb") as f:
            data = f.read()
        with open(os.path.join(HERE, name), "wb") as f:
            f.write(data)
        recs = _load(os.path.join(HERE, name))
        manifest[name] = {
            "sha256": hashlib.sha256(data).hexdigest(),
            "records": len(recs),
            "ok_enq": sum(1 for r in recs if r["op"] == 0 and r["ret"] == 1),
            "valued_deq": sum(1 for r in recs if r["op"] == 1 and r["ret"] != 0),
            "expect": "Linearizable (FIFO)",
        }
        manifest[name]["negatives"] = [m for m, _ in mutations(recs)]
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(json.dumps(manifest, indent=1, sort_keys=True))


if __name__ == "__main__":
    # the reference checkout: the first argument, else $GCQ_REFERENCE_DIR
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GCQ_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout>  (or set GCQ_REFERENCE_DIR)")
    main(ref)
