"""Autotuner for the scheduled navigation step.

Times the step on a caller-provided batch for each (schedule flags, sort-key Morton bits,
work-queue blocks per SM) candidate, keeps the fastest, applies its knobs to the geometry
and persists the choice as JSON keyed by the geometry's size and the batch size, so a later
process with the same geometry can apply it without re-timing. The knobs change only the
order in which the device visits tracks; results are identical for every candidate (the
tests check this), so tuning can never change physics output.
"""
import json
import os

from . import NAV_QUEUE, NAV_SORT, PREC_MIXED

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "vecgeom_gb300", "tuning.json")

CANDIDATES = [
    (PREC_MIXED | NAV_SORT | NAV_QUEUE, 0, 1),
    (PREC_MIXED | NAV_SORT | NAV_QUEUE, 0, 2),
    (PREC_MIXED | NAV_SORT | NAV_QUEUE, 7, 1),
    (PREC_MIXED | NAV_SORT | NAV_QUEUE, 5, 1),
    (PREC_MIXED | NAV_SORT, 0, 1),
    (PREC_MIXED | NAV_QUEUE, 0, 1),
]


def geometry_key(geo, n):
    i = geo.info()
    return "shapes%d_lv%d_pv%d_depth%d_nav%d_n%d" % (i["n_shapes"], i["n_lv"], i["n_pv"], i["max_depth"],
                                                      i["nav_words"], n)


def _time(torch, geo, t, st, out, step, flags, reps, warmup):
    for _ in range(warmup):
        geo.compute_step_and_next_volume(*t, st, out, step, flags=flags)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        geo.compute_step_and_next_volume(*t, st, out, step, flags=flags)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def autotune(geo, t, st, candidates=CANDIDATES, reps=3, warmup=1, cache=DEFAULT_CACHE, use_cache=True):
    """Pick the fastest candidate for step inputs `t` (x, y, z, dx, dy, dz CUDA tensors) and
    states `st`; apply it to `geo` and return {"flags", "cell_bits", "queue_blocks", "ms",
    "timings"}."""
    import torch
    n = t[0].numel()
    key = geometry_key(geo, n)
    table = {}
    if cache and os.path.exists(cache):
        try:
            with open(cache) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
    if use_cache and key in table:
        best = table[key]
        geo.set_tuning(best["cell_bits"], best["queue_blocks"])
        return dict(best, cached=True)
    out = torch.empty_like(st)
    step = torch.empty(n, dtype=torch.float64, device=t[0].device)
    timings = []
    for flags, bits, qb in candidates:
        geo.set_tuning(bits, qb)
        ms = _time(torch, geo, t, st, out, step, flags, reps, warmup)
        timings.append({"flags": flags, "cell_bits": bits, "queue_blocks": qb, "ms": ms})
    best = min(timings, key=lambda r: r["ms"])
    geo.set_tuning(best["cell_bits"], best["queue_blocks"])
    result = dict(best, timings=timings)
    if cache:
        table[key] = {k: best[k] for k in ("flags", "cell_bits", "queue_blocks", "ms")}
        try:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
        except OSError:
            pass
    return dict(result, cached=False)
