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
