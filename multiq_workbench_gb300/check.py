"""Self-checks of the batch path (chsim check.rs:1-121): a batch must give every ion exactly the
final state it gets when its job runs alone (``check_case``), and a fixed set of jobs hashes to
fixed values (``hash_ions``, FNV-1a over the final states, as ``chsim hash`` does with its own
state layout)."""
from __future__ import annotations

import numpy as np

from .channel import ION_FIELDS, IonStates


def compare(a: IonStates, b: IonStates) -> dict:
    """Ions whose final states differ, per field and overall (bitwise, like check.rs:8-20)."""
    n = len(a)
    diff = {"n": n}
    any_d = np.zeros(n, bool)
    for name, _ in ION_FIELDS:
        x, y = getattr(a, name), getattr(b, name)
        d = (x.view(np.uint8).reshape(n, -1) != y.view(np.uint8).reshape(n, -1)).any(axis=1)
        diff[name] = int(d.sum())
        any_d |= d
    diff["differ"] = int(any_d.sum())
    return diff


def check_case(engine, jobs, dc, ph) -> dict:
    """Each job run alone, then all jobs as one batch: the per-ion final states must agree bit for
    bit (check.rs:25-38).  Returns the comparison (``differ`` = ions that differ)."""
    parts = [engine.run_batch_ions([j], dc, ph)[0] for j in jobs]
    alone = IonStates.empty(sum(len(p) for p in parts))
    off = 0
    for p in parts:
        for name, _ in ION_FIELDS:
            getattr(alone, name)[off:off + len(p)] = getattr(p, name)
        off += len(p)
    # a lone job is job 0 of its batch; renumber to the batch's job ids before comparing
    off = 0
    for k, p in enumerate(parts):
        alone.jid[off:off + len(p)] = k
        off += len(p)
    batch, _ = engine.run_batch_ions(jobs, dc, ph)
    return compare(batch, alone)


def hash_ions(ions: IonStates) -> int:
    """FNV-1a 64 over every ion's final state, field by field in ``ION_FIELDS`` order (check.rs:95-99),
    computed by the native library (``mq_fnv1a64``)."""
    from . import _native as N
    h = 1469598103934665603
    for name, _ in ION_FIELDS:
        a = np.ascontiguousarray(getattr(ions, name))
        h = int(N.lib().mq_fnv1a64(a.ctypes.data, a.nbytes, h))
    return h
