"""GB300 trial engine for the songbird-HVC network-growth simulator.

The CUDA library (``_lib/libugrowth.so``, C ABI in ``include/ugrowth.h``) runs
the per-trial hot path of Sawndip/unsupervised_growth; ``engine`` binds it,
``network`` builds network descriptions.
"""
from .network import Network, synthetic_chain_network, synthetic_growth_network  # noqa: F401

__all__ = ["Network", "synthetic_chain_network", "synthetic_growth_network"]
