"""The command-line programs (ug_growth chainGrowth / continueChainGrowth /
chainTest, the reference's three mains) on a small network written in the
reference's topology format: they run, write the reference's files, and give
the results of the same calls through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import small_growth
from tests.helpers import FAST_MAT as MAT
from unsupervised_growth_gb300 import build as B
from unsupervised_growth_gb300 import files as F

pytestmark = pytest.mark.gpu

SYN6 = dict(Nss=2, A_P=20.0, A_D=19.0, T_0=0.0, T_P=10.0, T_D=10.0, TAU_P=30.0, TAU_D=30.0, BETA=0.2,
            BETA_SUPERSYNAPSE=0.2, ACTIVATION_THRESHOLD=10.0, SUPERSYNAPSE_THRESHOLD=40.0, WEIGHT_MAX=160.0)


def cli(*args):
    r = subprocess.run([B.CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


@pytest.fixture(scope="module")
def topology(tmp_path_factory):
    """A topology directory as createNetworkForGrowth writes it, a training file and a growth config."""
    B.build()
    root = tmp_path_factory.mktemp("cli")
    net = small_growth(seed=9, n_ra=60, n_i=16, n_tr=8, syn=SYN6, mat=MAT, delays="uniform", delay_width=2.0)
    conn = dict(net.conn, model_interneuron_distance=net.conn["model_interneuron_distance"] or 0.5,
                delay_constant=1.0)
    topo = root / "topology"
    topo.mkdir()
    F.write_coordinates(str(topo / "RA_xy.bin"), net.ra_xyz.reshape(-1, 3), conn["model_interneuron_distance"])
    F.write_coordinates(str(topo / "I_xy.bin"), net.i_xyz.reshape(-1, 3), conn["model_interneuron_distance"])
    split = lambda off, a: [a[off[i]:off[i + 1]] for i in range(len(off) - 1)]
    F.write_connections(str(topo / "RA_I_connections.bin"), split(net.ra2i_off, net.ra2i_tgt),
                        split(net.ra2i_off, net.ra2i_w), split(net.ra2i_off, net.ra2i_len),
                        split(net.ra2i_off, net.ra2i_d))
    F.write_connections(str(topo / "I_RA_connections.bin"), split(net.i2ra_off, net.i2ra_tgt),
                        split(net.i2ra_off, net.i2ra_w), split(net.i2ra_off, net.i2ra_len),
                        split(net.i2ra_off, net.i2ra_d))
    F.write_num_neurons(str(topo / "num_neurons.bin"), net.n_ra, net.n_i)
    F.write_topology_cfg(str(topo / "network_parameters.cfg"), "sphere", conn["A_RA2I"], conn["SIGMA_RA2I"],
                         conn["B_I2RA"], conn["SIGMA_I2RA"])
    train = root / "training_neurons.bin"
    F.write_training(str(train), str(root / "unused_spread.bin"), net.training, np.zeros(len(net.training)))
    cfg = root / "growth_parameters.cfg"
    F.write_growth_cfg(str(cfg), SYN6, MAT, net.noise, conn)
    return root, topo, train, cfg


def test_chain_growth_continue_and_test(topology):
    from unsupervised_growth_gb300.engine import Engine
    root, topo, train, cfg = topology
    eng = Engine(precision=32, spike_capacity_per_neuron=256)   # as the programs record spikes
    out, out2, tout = root / "out", root / "out2", root / "test"
    for d in (out, out2, tout):
        d.mkdir()
    cli("chainGrowth", f"{topo}/", train, cfg, f"{out}/", "--trials", 3, "--save-short", 1, "--save-long", 2)
    # the reference's set-up files and saves
    for name in ("network_parameters.cfg", "growth_parameters.cfg", "I_xy.bin", "training_neurons.bin",
                 "training_spread.bin", "num_neurons.bin", "RA_xy_initial.bin", "weights_0.bin", "weights_2.bin",
                 "spike_times_soma.bin", "RA_RA_super_connections.bin", "activity_history_2.bin"):
        assert (out / name).exists(), name
    assert (out / "growth_parameters.cfg").read_text() == cfg.read_text()
    assert (out / "network_parameters.cfg").read_text() == (topo / "network_parameters.cfg").read_text()
    rec = np.fromfile(out / "num_synapses.bin", dtype="<i4").reshape(-1, 3)
    assert rec[:, 0].tolist() == [0, 1, 2]
    # continue from trial 2 for two trials, against the same through the C ABI
    cli("continueChainGrowth", f"{out}/", f"{out2}/", 2, "--trials", 2, "--save-short", 1, "--save-long", 1)
    rn = eng.load_network_dir(f"{out}/", 2, seed=15000)
    rn.run_growth_trials(3, 2, True)
    W, trial = F.read_weights(str(out2 / "weights_4.bin"))
    assert trial == 4 and np.array_equal(W, rn.weights())
    assert F.read_synapse_lists(str(out2 / "RA_RA_active_connections_4.bin"))[0] == rn.synapse_list(0)
    rn.free()
    # test trials of the trial-2 network
    cli("chainTest", f"{out}/", 2, 4, f"{tout}/")
    for k in range(4):
        for kind in ("soma", "dend", "interneuron"):
            assert (tout / f"test_spike_times_{kind}_{k}.bin").exists()
    rn = eng.load_network_dir(f"{out}/", 2, seed=15000)
    rn.run_test_trials(0, 4)
    p = str(root / "jitter_abi.bin")
    rn.write_jitter(p)
    assert open(p, "rb").read() == (tout / "jitter.bin").read_bytes()
    times, trial, _ = F.read_spike_times(str(tout / "test_spike_times_soma_3.bin"))
    n, s = rn.spikes(3, 0)
    assert trial == 2 and sum(len(t) for t in times) == len(n)
    rn.free()
    eng.close()
