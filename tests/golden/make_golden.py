"""Generates tests/golden/neuron_golden.npz from the reference's own neuron classes.

Runs c++/src/HH2_test.cpp and c++/src/HHI_buffer.cpp, compiled unmodified from
the reference tree into oracle/_ref/libref.so (see oracle/Makefile), through
the trial path's per-step calls with the Philox noise streams of
oracle/ugo_noise.h, and stores subsampled state traces and every spike step.
Run from the repository root where the reference tree exists:

    python tests/golden/make_golden.py [/path/to/reference/c++]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

SUB = 25
N_STEPS = 24999

# (name, kind, kwargs)
SCENARIOS = [
    ("ra_mature_kicked", "ra", dict(erest=-80.0, gca=55.0, noise=(0.0, 0.1, 0.0, 0.2), seed=11, trial=0, neuron=3,
                                    kicks=[(5000, 3.0, 0.0), (9000, 0.0, 0.8), (15000, 0.4, 0.0), (15010, 0.4, 0.3)])),
    ("ra_immature", "ra", dict(erest=-55.0, gca=0.0, noise=(0.0, 0.1, 0.0, 0.2), seed=12, trial=7, neuron=101,
                               kicks=[(2000, 1.5, 0.0), (20000, 3.0, 0.0)])),
    ("ra_partly_mature_mu", "ra", dict(erest=-70.0, gca=30.0, noise=(0.05, 0.3, -0.02, 0.4), seed=13, trial=2,
                                       neuron=7, kicks=[(100, 0.0, 2.0), (12000, 3.0, 0.0)])),
    ("i_noise_only", "i", dict(seed=21, trial=0, neuron=0, kicks=[])),
    ("i_kicked", "i", dict(seed=22, trial=5, neuron=42, kicks=[(1000, 2.0, 0.0), (8000, 0.0, 3.0), (8001, 1.0, 0.0)])),
]


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    if O.build_ref(ref_dir) is None:
        raise SystemExit(f"reference tree {ref_dir} not found")
    out = {}
    for name, kind, kw in SCENARIOS:
        fn = O.ra_single if kind == "ra" else O.i_single
        tr, fired = fn(N_STEPS, use_ref=True, **kw)
        out[name + "/trace"] = tr[::SUB].copy()
        out[name + "/final"] = tr[-1].copy()
        if kind == "ra":
            out[name + "/soma"] = np.nonzero(fired[:, 0])[0].astype(np.int32)
            out[name + "/dend"] = np.nonzero(fired[:, 1])[0].astype(np.int32)
        else:
            out[name + "/fired"] = np.nonzero(fired)[0].astype(np.int32)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "neuron_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
