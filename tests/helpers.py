"""Shared helpers of the parity tests: small seeded networks and comparisons."""
import numpy as np

from unsupervised_growth_gb300.network import synthetic_chain_network, synthetic_growth_network


def small_chain(seed=5, n_ra=60, n_i=20, groups=5, group=10, weight=500.0, num_steps=25000, delay_cap=2.0, **kw):
    return synthetic_chain_network(n_ra=n_ra, n_i=n_i, n_groups=groups, group_size=group, weight=weight, seed=seed,
                                   delay_cap=delay_cap, num_steps=num_steps, **kw)


def small_growth(seed=7, n_ra=40, n_i=14, n_tr=6, num_steps=25000, **kw):
    return synthetic_growth_network(n_ra=n_ra, n_i=n_i, n_tr=n_tr, seed=seed, num_steps=num_steps, **kw)


def sorted_spikes(neuron, step):
    order = np.lexsort((step, neuron))
    return np.stack([neuron[order], step[order]], axis=1)


def oracle_trial_spikes(onet, which):
    n, s = onet.spikes(which)
    return sorted_spikes(n, s)


def match_within(a, b, tol_steps=1):
    """Fraction of spikes of a matched to a spike of b of the same neuron within tol_steps (greedy)."""
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
