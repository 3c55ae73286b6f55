"""Shared helpers of the parity tests: small seeded networks and comparisons."""
import numpy as np

from unsupervised_growth_gb300.compare import match_within, sorted_spikes  # noqa: F401  (re-exported)
from unsupervised_growth_gb300.network import synthetic_chain_network, synthetic_growth_network

# Fast-growing synapses: supersynapses form within a few trials on a 40/14 network.
FAST_SYN = dict(Nss=2, A_P=20.0, A_D=20.0 / 1.05, T_0=0.0, T_P=10.0, T_D=10.0, TAU_P=30.0, TAU_D=30.0, BETA=0.2,
                BETA_SUPERSYNAPSE=0.2, ACTIVATION_THRESHOLD=10.0, SUPERSYNAPSE_THRESHOLD=40.0, WEIGHT_MAX=160.0)
FAST_MAT = dict(RATE_WINDOW_LONG=1000, E_REST_IMMATURE=-65.0, GCA_IMMATURE=25.0, DEATH_RATE_THRESHOLD=0.01)


def small_chain(seed=5, n_ra=60, n_i=20, groups=5, group=10, weight=500.0, num_steps=25000, delay_cap=2.0, **kw):
    return synthetic_chain_network(n_ra=n_ra, n_i=n_i, n_groups=groups, group_size=group, weight=weight, seed=seed,
                                   delay_cap=delay_cap, num_steps=num_steps, **kw)


def small_growth(seed=7, n_ra=40, n_i=14, n_tr=6, num_steps=25000, **kw):
    return synthetic_growth_network(n_ra=n_ra, n_i=n_i, n_tr=n_tr, seed=seed, num_steps=num_steps, **kw)


def growth_net(seed=7, replace_ids=(), syn=None):
    """The 40/14 fast-growth network of the growth parity tests; neurons in replace_ids
    are made older than the 1000-trial robustness window, so silence replaces them."""
    net = small_growth(seed=seed, n_ra=40, n_i=14, n_tr=8, syn=syn or FAST_SYN, mat=FAST_MAT, delays="uniform",
                       delay_width=2.0)
    net.training_spread = np.linspace(0.0, 15.0, len(net.training))
    for r in replace_ids:
        net.trials_after_replacement[r] = 1001
    net.trials_after_replacement[net.training] = 0
    return net


def oracle_trial_spikes(onet, which):
    n, s = onet.spikes(which)
    return sorted_spikes(n, s)


def heavy_growth_net(seed, width, delays="uniform", n_tr=20):
    """A 1100 / 275 fast-growth network: at least 1024 HVC(RA), so in a group its spiking
    rows take the block-per-row delivery path.  Twenty training neurons spread over
    15 ms, so training rows potentiate onto one another within a trial."""
    net = small_growth(seed=seed, n_ra=1100, n_i=275, n_tr=n_tr, syn=FAST_SYN, mat=FAST_MAT, delays=delays,
                       delay_width=width)
    net.training_spread = np.linspace(0.0, 15.0, len(net.training))
    net.trials_after_replacement[net.training] = 0
    return net
