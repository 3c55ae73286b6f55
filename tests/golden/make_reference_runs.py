"""Generate tests/golden/reference_runs.npz: results of the reference's own
simulator (NetworkGrowthSimulator, c++/src/NetworkGrowthSimulator.cpp, built
unmodified by oracle/Makefile target `refsim` and driven by
oracle/ref_harness/sim_harness.cpp) on the workload configurations, for the GPU
parity tests to compare against where the reference tree is absent.

Cases (networks rebuilt from their seeds by unsupervised_growth_gb300.workloads /
tests.helpers; each stored with the network's fingerprint so a test can tell
whether it rebuilt the same network):
  config3  the 2000 / 550 synfire-chain network of the batched test trials,
           one full 500 ms test trial (trial_no_stdp_fixedSpread), trial index 0;
  config1  300 / 100 growth network with the config-1 STDP set, growth trials 0-4
           with their per-trial tail (trial_1stSoma_pre_1stSoma_post_delays_fixedSpread
           and chain_growth's bookkeeping);
  heavy0, heavy1  1100 / 275 fast-growth networks (zero and 0.5 ms delays), growth
           trials 0-2: networks of at least 1024 HVC(RA), whose spiking rows take the
           block-per-row delivery path in a group.

Per trial: spikes (neuron, step) of soma, dendrite and interneurons sorted by
neuron then step; for growth also the nonzero RA->RA weights, the ordered active
and super lists and the per-neuron maturation state.

Run: python tests/golden/make_reference_runs.py  (about six minutes on one core)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.helpers import heavy_growth_net, sorted_spikes  # noqa: E402
from unsupervised_growth_gb300.workloads import config1_network, config3_network, network_fingerprint  # noqa: E402

OUT = os.path.join(HERE, "reference_runs.npz")

CASES = [
    ("config3", config3_network, "test", [0]),
    ("config1", config1_network, "growth", [0, 1, 2, 3, 4]),
    ("heavy0", lambda: heavy_growth_net(41, 0.0), "growth", [0, 1, 2]),
    ("heavy1", lambda: heavy_growth_net(42, 0.5), "growth", [0, 1, 2]),
]

PROPS = ("rest_potential", "gca", "mature", "maturation_scale", "remodeled", "trials_after_replacement",
         "firing_rate_long")


def lists_csr(lists):
    off = np.zeros(len(lists) + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(x) for x in lists])
    tgt = np.array([j for x in lists for j in x], dtype=np.int32)
    return off, tgt


def main():
    if not O.build_ref_sim():
        sys.exit("the reference tree is needed (set UG_REFERENCE_DIR)")
    out = {}
    for name, make, kind, trials in CASES:
        net = make()
        out[f"{name}__fingerprint"] = np.array(network_fingerprint(net))
        out[f"{name}__trials"] = np.array(trials, dtype=np.int32)
        r = O.RefSimNet(net)
        for t in trials:
            t0 = time.time()
            assert r.run_trial(kind == "growth", t) == 0
            pre = f"{name}__t{t}__"
            for w in (0, 1, 2):
                out[pre + f"spk{w}"] = sorted_spikes(*r.spikes(w)).astype(np.int32)
            if kind == "growth":
                r.after_growth_trial(t)
                W = r.weights()
                idx = np.flatnonzero(W)
                out[pre + "w_idx"] = idx.astype(np.int64)
                out[pre + "w_val"] = W.ravel()[idx]
                for which, tag in ((0, "act"), (1, "sup")):
                    off, tgt = lists_csr(r.synapse_list(which))
                    out[pre + tag + "_off"], out[pre + tag + "_tgt"] = off, tgt
                p = r.neuron_props()
                for k in PROPS:
                    out[pre + k] = p[k]
                out[pre + "replaced"] = r.replaced().astype(np.int32)
            print(f"{name} trial {t}: {time.time() - t0:.1f} s, soma spikes {len(out[pre + 'spk0'])}", flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
