"""Seeded synthetic workloads of the batched and served forms: many growing
networks of uneven size in one group, and a Poisson stream of growth and
test-trial requests of mixed network size.

There is no public dataset for this simulator; these generators stand in for
the reference's own network-creation programs (createNetworkForGrowth) with
its spatial connectivity rule (synthetic_growth_network) and a synthetic
chain for test trials (synthetic_chain_network).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .network import Network, synthetic_chain_network, synthetic_growth_network

DELAY_WIDTHS = (0.0, 1.0, 3.0, 6.0, 10.0)   # ms, uniform delays 0..w, round-robin over the networks


def log_uniform_sizes(rng, n, lo=200, hi=8000):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).round().astype(int)


def uneven_networks(n_nets=64, seed=4, lo=200, hi=8000, widths=DELAY_WIDTHS, n_tr=10) -> list[Network]:
    """Growing networks with HVC(RA) counts log-uniform in [lo, hi], HVC(I) = RA / 4,
    uniform axonal delays 0..w with w taken round-robin from `widths`."""
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(rng, n_nets, lo, hi)
    return [growth_member(int(s), seed * 1000 + k, widths[k % len(widths)], k, n_tr) for k, s in enumerate(sizes)]


def growth_member(n_ra, seed, width, net_id, n_tr=10) -> Network:
    return synthetic_growth_network(n_ra=n_ra, n_i=max(n_ra // 4, 1), n_tr=min(n_tr, n_ra), seed=seed,
                                    delays="uniform", delay_width=width, net_id=net_id)


def chain_member(n_ra, seed, net_id) -> Network:
    """A grown network for test trials: a synfire chain over about half the neurons
    (groups of up to 100), lognormal delays mean 3 ms."""
    group = max(min(100, n_ra // 20), 2)
    groups = max(min(20, n_ra // (2 * group)), 2)
    net = synthetic_chain_network(n_ra=n_ra, n_i=max(n_ra // 4, 1), n_groups=groups, group_size=group,
                                  weight=500.0, seed=seed)
    net.net_id = net_id
    return net


@dataclass
class Request:
    arrival: float        # seconds after the stream starts
    kind: str             # "growth" or "test"
    n_ra: int
    n_trials: int
    seed: int

    def network(self) -> Network:
        if self.kind == "growth":
            return growth_member(self.n_ra, self.seed, DELAY_WIDTHS[self.seed % len(DELAY_WIDTHS)], self.seed)
        return chain_member(self.n_ra, self.seed, self.seed)


def request_stream(n_requests=48, rate_hz=2.0, seed=5, lo=200, hi=8000, max_trials=50,
                   growth_fraction=0.5) -> list[Request]:
    """Poisson arrivals at rate_hz; network size log-uniform in [lo, hi]; trials
    uniform in 1..max_trials; growth or test with probability growth_fraction."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = log_uniform_sizes(rng, n_requests, lo, hi)
    trials = rng.integers(1, max_trials + 1, n_requests)
    kinds = np.where(rng.random(n_requests) < growth_fraction, "growth", "test")
    return [Request(float(a), str(k), int(s), int(t), seed * 10000 + i)
            for i, (a, k, s, t) in enumerate(zip(arrivals, kinds, sizes, trials))]


# ------------------------------------------------------------ named configurations
# Config 1: a plain growth trial of 300 HVC(RA) / 100 HVC(I) on a sphere, uniform
# 0-2 ms delays, white noise sigma 0.1 / 0.2, ten mature training neurons, the STDP
# set of the network defaults (tau 30 ms, A_P = 1.05 A_D, supersynapse threshold
# 0.035, Nss 3).
def config1_network(seed: int = 1) -> Network:
    return synthetic_growth_network(n_ra=300, n_i=100, n_tr=10, seed=seed, delays="uniform", delay_width=2.0)


# Config 2: growth at scale, 2000 / 550 with log-normal delays (mean 3, sd 1.5, cap 10 ms).
def config2_network(seed: int = 2, syn=None, mat=None) -> Network:
    extra = {}
    if syn:
        extra["syn"] = syn
    if mat:
        extra["mat"] = mat
    return synthetic_growth_network(n_ra=2000, n_i=550, n_tr=10, seed=seed, delays="lognormal", lognormal_mean=3.0,
                                    lognormal_sigma=1.5, delay_cap=10.0, **extra)


# Config 3: the fixed grown 2000 / 550 network for batched test trials: a synfire chain
# of 20 groups x 100 neurons, 0.05 mS/cm^2 per synapse between consecutive groups
# (500 in the reference's weight units, which raiseExcWeight divides by the
# 10000 um^2 dendritic area), log-normal delays mean 3 ms.
CONFIG3 = dict(n_ra=2000, n_i=550, n_groups=20, group_size=100, weight=500.0, seed=3)


def config3_network(num_steps: int = 25000) -> Network:
    return synthetic_chain_network(delays="lognormal", lognormal_mean=3.0, lognormal_sigma=1.5, delay_cap=10.0,
                                   num_steps=num_steps, **CONFIG3)


def network_fingerprint(net: Network) -> str:
    """SHA-256 over every array and parameter of a network, so a result stored for a
    seeded network can be matched to the network rebuilt on another machine."""
    import hashlib
    h = hashlib.sha256()
    for k in sorted(vars(net)):
        v = getattr(net, k)
        if isinstance(v, np.ndarray):
            h.update(k.encode())
            h.update(np.ascontiguousarray(v).tobytes())
        elif isinstance(v, dict):
            h.update(repr(sorted(v.items())).encode())
        else:
            h.update(repr((k, v)).encode())
    return h.hexdigest()
