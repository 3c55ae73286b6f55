"""Spike-train comparison used to state the single-precision error against the
double-precision build: spikes of one trial as (neuron, step) rows, and the
fraction of one train matched within a number of 0.02 ms steps by the other."""
import numpy as np


def sorted_spikes(neuron, step):
    """(neuron, step) rows sorted by neuron, then step."""
    neuron, step = np.asarray(neuron), np.asarray(step)
    order = np.lexsort((step, neuron))
    return np.stack([neuron[order], step[order]], axis=1)


def match_within(a, b, tol_steps=1):
    """Fraction of the spikes of a matched (greedily, nearest first) to a spike of b
    of the same neuron within tol_steps, over the larger count, and the largest
    matched distance in steps."""
    if len(a) == 0 and len(b) == 0:
        return 1.0, 0
    matched = 0
    worst = 0
    bi = {}
    for n, s in b:
        bi.setdefault(int(n), []).append(int(s))
    for n, s in a:
        cand = bi.get(int(n), [])
        best = None
        for k, t in enumerate(cand):
            if abs(t - int(s)) <= tol_steps and (best is None or abs(t - int(s)) < abs(cand[best] - int(s))):
                best = k
        if best is not None:
            worst = max(worst, abs(cand[best] - int(s)))
            cand.pop(best)
            matched += 1
    return matched / max(len(a), len(b)), worst
