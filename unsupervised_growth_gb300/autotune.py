"""Launch-shape autotuner for group runs, the serving loop and single-network growth trials.

The group kernels run persistent, occupancy-sized grids over device work lists
(``ug_run_group``).  Three knobs decide how a round's work meets the SMs: the
blocks per SM of the HVC(RA) and HVC(I) integrators' grids, and whether the
interneuron kernel runs beside the RA kernel on a second stream.  Which shape
is fastest depends on the mix -- a few large networks fill the GPU in one wave
at occupancy, many small latency-bound ones prefer the kernels side by side,
a huge test batch prefers them back to back -- so it is measured.

The tuner is online: it times real rounds of the caller's own work under each
candidate shape (coordinate descent from the occupancy shape), keeps the
fastest, and caches it per device and mix signature.  Results do not depend on
the shape, so the tuning rounds are ordinary rounds of the run.
"""
from __future__ import annotations

import json
import math
import os
import time

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")

# (ra_blocks_per_sm, i_blocks_per_sm, overlap); 0 = the occupancy limit
START = (0, 0, True)


def signature(device_name: str, members) -> str:
    """Mix signature: device, kinds, member count and RA-neuron total on a log2 scale.
    members: iterable of (n_ra, kind, batch)."""
    members = list(members)
    kinds = "".join(sorted({k[0] for _, k, _ in members}))
    neurons = sum(n * b for n, _, b in members)
    return f"{device_name}|{kinds}|m{2 ** int(math.log2(max(len(members), 1)))}|n{int(math.log2(max(neurons, 1)))}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def tune(engine, run_round, sig: str | None = None, cache_path: str | None = DEFAULT_CACHE, repeats: int = 1,
         max_rounds: int | None = None):
    """Chooses the launch shape for `run_round` (a callable that runs one round of the
    caller's group work through `engine` and returns when it is done).

    With a cached entry for `sig`, applies it without timing.  Otherwise times
    `repeats` rounds per candidate: the start shape, then the overlap flag, then the
    RA grid (2, 1 blocks per SM), then the interneuron grid, keeping each change
    that made the round faster.  Returns {"shape", "table", "rounds", "cached"}."""
    cache = _load(cache_path) if (cache_path and sig) else {}
    if sig and sig in cache:
        ra, ii, ov = cache[sig]["shape"]
        engine.set_group_launch(ra, ii, bool(ov))
        return {"shape": (ra, ii, bool(ov)), "table": cache[sig].get("table", []), "rounds": 0, "cached": True}

    table = []
    rounds = [0]

    def measure(shape):
        engine.set_group_launch(shape[0], shape[1], shape[2])
        best = math.inf
        for _ in range(repeats):
            t0 = time.perf_counter()
            run_round()
            best = min(best, time.perf_counter() - t0)
            rounds[0] += 1
        table.append({"shape": list(shape), "seconds": best})
        return best

    best_shape = START
    best_t = measure(best_shape)
    steps = [("overlap", [not START[2]]), ("ra", [2, 1]), ("i", [2, 1])]
    for knob, values in steps:
        for v in values:
            if max_rounds is not None and rounds[0] + repeats > max_rounds:
                break
            ra, ii, ov = best_shape
            cand = (v, ii, ov) if knob == "ra" else (ra, v, ov) if knob == "i" else (ra, ii, v)
            t = measure(cand)
            if t < best_t:
                best_t, best_shape = t, cand
    engine.set_group_launch(*best_shape)
    if cache_path and sig:
        cache[sig] = {"shape": [best_shape[0], best_shape[1], int(best_shape[2])], "seconds": best_t,
                      "table": table}
        _store(cache_path, cache)
    return {"shape": best_shape, "table": table, "rounds": rounds[0], "cached": False}


# Integrating threads per block of the one-launch growth trial's HVC(RA) and HVC(I)
# roles (ug_set_growth_trial_shape); 0 = the build's default.
TRIAL_WIDTHS = (256, 128, 64, 32)


def trial_signature(device_name: str, n_ra: int, n_i: int, precision: int) -> str:
    """Signature of a single-network growth run: device, precision and both neuron counts
    on a log2 scale."""
    return (f"{device_name}|trial{precision}|ra{int(math.log2(max(n_ra, 1)))}"
            f"|i{int(math.log2(max(n_i, 1)))}")


def tune_growth_trial(engine, run_trial, sig: str | None = None, cache_path: str | None = DEFAULT_CACHE,
                      widths=TRIAL_WIDTHS, repeats: int = 1):
    """Chooses the block shape of the one-launch growth trial for `run_trial` (a callable
    that runs the caller's next growth trial(s) through `engine` and returns when done).

    A single network's trial is a chain of sync intervals separated by grid barriers, so
    its time is the latency of the slowest block per interval: how many integrating warps
    share an SM scheduler decides it, not occupancy.  Because an interval waits for the
    slower of the two roles, narrowing one role alone can show no gain; so the search
    first tries equal widths for both roles, then refines the HVC(RA) width and then the
    HVC(I) width from the best of those, keeping each faster shape.  With a cached entry
    for `sig` the shape is applied without timing.  The results are the same bits for
    every shape, so the timed trials are ordinary trials of the run.  Returns
    {"shape", "table", "trials", "cached"}."""
    cache = _load(cache_path) if (cache_path and sig) else {}
    if sig and sig in cache:
        ra, ii = cache[sig]["shape"]
        engine.set_growth_trial_shape(ra, ii)
        return {"shape": (ra, ii), "table": cache[sig].get("table", []), "trials": 0, "cached": True}
    table = []
    trials = [0]

    def measure(shape):
        engine.set_growth_trial_shape(*shape)
        run_trial()   # the first trial of a shape captures its graph
        trials[0] += 1
        best = math.inf
        for _ in range(repeats):
            t0 = time.perf_counter()
            run_trial()
            best = min(best, time.perf_counter() - t0)
            trials[0] += 1
        table.append({"shape": list(shape), "seconds": best})
        return best

    best_shape = (0, 0)
    best_t = measure(best_shape)
    tried = {best_shape}
    for knob in ("both", "ra", "i"):
        for w in widths:
            cand = (w, w) if knob == "both" else (w, best_shape[1]) if knob == "ra" else (best_shape[0], w)
            if cand in tried:
                continue
            tried.add(cand)
            t = measure(cand)
            if t < best_t:
                best_t, best_shape = t, cand
    engine.set_growth_trial_shape(*best_shape)
    if cache_path and sig:
        cache[sig] = {"shape": list(best_shape), "seconds": best_t, "table": table}
        _store(cache_path, cache)
    return {"shape": best_shape, "table": table, "trials": trials[0], "cached": False}
