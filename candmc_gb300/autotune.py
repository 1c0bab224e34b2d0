"""Project-written autotuner for the batched least-squares schedule.

The knobs are the number of streams the batch is dealt onto and the target
rows per TSQR leaf (candmc_set_tuning("leaf_rows")).  `tune_batched` times
every combination on a sample of the problem set with CUDA events and keeps
the fastest; results are cached in a JSON database keyed by the width mix and
the (log2-bucketed) row range, at $CANDMC_TUNING_DB or
~/.cache/candmc_gb300/tuning.json.
"""
import json
import math
import os

DEFAULT = {"nstreams": 16, "leaf_rows": 64}
GRID = {"nstreams": (4, 8, 16, 32), "leaf_rows": (64, 128, 256)}


def db_path():
    return os.environ.get("CANDMC_TUNING_DB",
                          os.path.join(os.path.expanduser("~"), ".cache", "candmc_gb300", "tuning.json"))


def _load():
    try:
        with open(db_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    path = db_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def key_for(ms, ns):
    widths = sorted(set(int(n) for n in ns))
    lo = int(math.log2(max(1, min(ms))))
    hi = int(math.log2(max(1, max(ms))))
    return f"batched_ls:n={','.join(map(str, widths))}:m=2^{lo}..2^{hi}"


def lookup(ms, ns):
    return _load().get(key_for(ms, ns), dict(DEFAULT))


def tune_batched(make_batch, ms, ns, reps=2):
    """make_batch() -> (As, Bs) fresh device copies of a sample batch.
    Times every knob combination and records the best in the database."""
    import torch

    import candmc_gb300 as cm
    best, best_ms, trials = None, float("inf"), []
    for leaf in GRID["leaf_rows"]:
        cm.set_tuning("leaf_rows", leaf)
        for nst in GRID["nstreams"]:
            times = []
            for _ in range(reps):
                As, Bs = make_batch()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                cm.batched_ls(As, Bs, nstreams=nst)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            t = min(times)
            trials.append({"leaf_rows": leaf, "nstreams": nst, "ms": t})
            if t < best_ms:
                best, best_ms = {"leaf_rows": leaf, "nstreams": nst}, t
    cm.set_tuning("leaf_rows", best["leaf_rows"])
    db = _load()
    db[key_for(ms, ns)] = dict(best, ms=best_ms)
    _store(db)
    return best, trials
