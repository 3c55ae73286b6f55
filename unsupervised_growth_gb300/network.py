"""Network description for the growth / test-trial path.

A ``Network`` holds every array that the simulator reads on the per-trial path,
in the layout the reference keeps on its master rank
(c++/include/NetworkGrowthSimulator.h:100-260): RA->I and I->RA connection
lists (CSR here, in the reference's per-source order), the dense RA->RA weight
and axonal-delay matrices, the ordered active and super synapse lists, and the
per-neuron maturation state.  The same object feeds the CUDA library (through
``unsupervised_growth_gb300.engine``) and the test oracle.

``synthetic_*`` build the workloads the benchmark and the parity tests use.
There is no public dataset for this simulator, so every input is generated
from a seed with the sizes and distributions of the workloads:

* ``synthetic_growth_network`` -- HVC(RA) and HVC(I) on a sphere, distance
  dependent RA<->I connectivity ``A*exp(-d^2/lambda^2)`` with exponential
  weights, RA->RA weights 0, uniform or log-normal axonal delays.
* ``synthetic_chain_network`` -- a grown network carrying a synfire chain of
  groups with a fixed weight between consecutive groups (active synapses).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

TIMESTEP = 0.02
TRIAL_DURATION = 500.0
DEFAULT_NUM_STEPS = int(TRIAL_DURATION / TIMESTEP)   # 25000 -> 24999 integration steps

# Defaults of the reference's parameter structs (c++/include/ConfigurationNetworkGrowth.h:30-104);
# synaptic parameters default to zero there, the values below are the ones the growth workloads use.
DEFAULT_SYN = dict(Nss=3, A_P=0.0025, A_D=0.0025 / 1.05, T_0=0.0, T_P=10.0, T_D=10.0, TAU_P=30.0, TAU_D=30.0,
                   BETA=0.0001, BETA_SUPERSYNAPSE=0.0001, ACTIVATION_THRESHOLD=0.005,
                   SUPERSYNAPSE_THRESHOLD=0.035, WEIGHT_MAX=0.05)
DEFAULT_MAT = dict(E_REST_MATURE=-80.0, E_REST_IMMATURE=-55.0, GCA_MATURE=55.0, GCA_IMMATURE=0.0,
                   DEATH_RATE_THRESHOLD=0.01, RATE_WINDOW_LONG=1000)
DEFAULT_NOISE = dict(white_noise_mean_soma=0.0, white_noise_std_soma=0.1, white_noise_mean_dend=0.0,
                     white_noise_std_dend=0.2)
DEFAULT_CONN = dict(Gei_max=0.25, Gie_max=0.1, delay_constant=1.0, A_RA2I=0.1, SIGMA_RA2I=0.0,
                    B_I2RA=0.1, SIGMA_I2RA=0.0, model_interneuron_distance=0.0)

MATURATION_SCALE_SPONTANEOUS = 100000.0
MATURATION_SCALE_DRIVEN = 1000.0


def fibonacci_model_distance(n_i: int) -> float:
    """Distance between the first two points of the Fibonacci sphere of n_i
    interneurons, the model interneuron spacing the reference derives in
    sample_coordinates (c++/src/NetworkGrowthSimulator.cpp:296-312)."""
    dphi = math.pi * (3.0 - math.sqrt(5.0))
    dz = 2 / float(n_i)
    z = 1 - dz / 2.0
    x1, y1 = math.cos(0.0) * math.sqrt(1.0 - z * z), math.sin(0.0) * math.sqrt(1.0 - z * z)
    x2 = math.cos(dphi) * math.sqrt(1.0 - (z - dz) * (z - dz))
    y2 = math.sin(dphi) * math.sqrt(1.0 - (z - dz) * (z - dz))
    tmp = x1 * x2 + y1 * y2 + z * (z - dz)
    return 0.0 if tmp > 1.0 else math.acos(tmp)


def sphere_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Great-circle distance between unit vectors (distance_on_sphere,
    NetworkGrowthSimulator.cpp:37-45)."""
    tmp = a @ b.T
    out = np.arccos(np.clip(tmp, -1.0, 1.0))
    out[tmp > 1.0] = 0.0
    return out


def _csr_from_lists(lists, n_src):
    off = np.zeros(n_src + 1, dtype=np.int32)
    for i, l in enumerate(lists):
        off[i + 1] = off[i] + len(l)
    tgt = np.array([t for l in lists for t in l], dtype=np.int32)
    return off, tgt


@dataclass
class Network:
    n_ra: int
    n_i: int
    seed: int = 1
    net_id: int = 0
    num_steps: int = DEFAULT_NUM_STEPS
    syn: dict = field(default_factory=lambda: dict(DEFAULT_SYN))
    mat: dict = field(default_factory=lambda: dict(DEFAULT_MAT))
    noise: dict = field(default_factory=lambda: dict(DEFAULT_NOISE))
    conn: dict = field(default_factory=lambda: dict(DEFAULT_CONN))
    ra2i_off: np.ndarray = None
    ra2i_tgt: np.ndarray = None
    ra2i_w: np.ndarray = None
    ra2i_d: np.ndarray = None
    ra2i_len: np.ndarray = None
    i2ra_off: np.ndarray = None
    i2ra_tgt: np.ndarray = None
    i2ra_w: np.ndarray = None
    i2ra_d: np.ndarray = None
    i2ra_len: np.ndarray = None
    w_rara: np.ndarray = None
    d_rara: np.ndarray = None
    len_rara: np.ndarray = None
    active_off: np.ndarray = None
    active_tgt: np.ndarray = None
    super_off: np.ndarray = None
    super_tgt: np.ndarray = None
    rest_potential: np.ndarray = None
    gca: np.ndarray = None
    mature: np.ndarray = None
    maturation_scale: np.ndarray = None
    remodeled: np.ndarray = None
    trials_after_replacement: np.ndarray = None
    activity_history: np.ndarray = None
    training: np.ndarray = None
    training_spread: np.ndarray = None
    ra_xyz: np.ndarray = None
    i_xyz: np.ndarray = None

    def set_lists(self, active, supers):
        self.active_off, self.active_tgt = _csr_from_lists(active, self.n_ra)
        self.super_off, self.super_tgt = _csr_from_lists(supers, self.n_ra)

    def lists(self, which: str):
        off, tgt = (self.active_off, self.active_tgt) if which == "active" else (self.super_off, self.super_tgt)
        return [tgt[off[i]:off[i + 1]].tolist() for i in range(self.n_ra)]

    def max_delay(self) -> float:
        m = 0.0
        for a in (self.ra2i_d, self.i2ra_d, self.d_rara):
            if a is not None and a.size:
                m = max(m, float(np.max(a)))
        return m

    def validate(self):
        assert self.w_rara.shape == (self.n_ra, self.n_ra)
        assert self.d_rara.shape == (self.n_ra, self.n_ra)
        assert self.ra2i_off.shape == (self.n_ra + 1,) and self.i2ra_off.shape == (self.n_i + 1,)
        assert int(self.mat["RATE_WINDOW_LONG"]) >= 1000
        assert self.activity_history.shape == (self.n_ra, int(self.mat["RATE_WINDOW_LONG"]))
        return self


def _sphere_points(rng, n):
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * math.pi, n)
    s = np.sqrt(1 - z * z)
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def _fibonacci_sphere(rng, n, jitter):
    dphi = math.pi * (3.0 - math.sqrt(5.0))
    dz = 2.0 / n
    k = np.arange(n)
    z = 1 - dz / 2.0 - k * dz
    phi = k * dphi
    r = np.sqrt(1 - z * z)
    p = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    p = p + rng.normal(0.0, jitter, p.shape)
    return p / np.linalg.norm(p, axis=1, keepdims=True)


def synthetic_growth_network(n_ra=300, n_i=100, n_tr=10, seed=1, delays="uniform", delay_width=2.0,
                             lognormal_mean=3.0, lognormal_sigma=1.5, delay_cap=10.0, p0=0.1,
                             weight_mean=0.1, num_steps=DEFAULT_NUM_STEPS, syn=None, mat=None, noise=None,
                             conn=None, net_id=0) -> Network:
    """Sphere network for growth trials.

    Connection probability ``p0*exp(-d^2/lambda^2)`` with d the model-space
    great-circle distance in microns and lambda = 3 interneuron spacings
    (written in the reference's ``A*exp(-d^2/(2 sigma^2))`` form with
    sigma = lambda/sqrt(2)); exponential weights with the given mean;
    RA->RA weights start at 0 with no active or super synapses.
    Delays: ``uniform`` in [0, delay_width] ms or ``lognormal`` with the
    given mean and standard deviation, capped at delay_cap ms.
    """
    rng = np.random.default_rng(seed)
    net = Network(n_ra=n_ra, n_i=n_i, seed=seed, num_steps=num_steps, net_id=net_id)
    if syn:
        net.syn.update(syn)
    if mat:
        net.mat.update(mat)
    if noise:
        net.noise.update(noise)
    model_dist = fibonacci_model_distance(n_i)
    lam = 3 * 40.0
    sigma = lam / math.sqrt(2.0)
    net.conn.update(dict(A_RA2I=p0, B_I2RA=p0, SIGMA_RA2I=sigma, SIGMA_I2RA=sigma,
                         model_interneuron_distance=model_dist))
    if conn:
        net.conn.update(conn)
    net.i_xyz = _fibonacci_sphere(rng, n_i, 0.15 * model_dist)
    net.ra_xyz = _sphere_points(rng, n_ra)

    def draw_delays(shape):
        if delays == "uniform":
            return rng.uniform(0.0, delay_width, shape)
        mu = math.log(lognormal_mean ** 2 / math.sqrt(lognormal_mean ** 2 + lognormal_sigma ** 2))
        s = math.sqrt(math.log(1 + (lognormal_sigma / lognormal_mean) ** 2))
        return np.minimum(rng.lognormal(mu, s, shape), delay_cap)

    d_ri = sphere_distance(net.ra_xyz, net.i_xyz) * 40.0 / model_dist
    p = p0 * np.exp(-d_ri ** 2 / lam ** 2)
    conn_ri = rng.random(p.shape) < p
    lists = [np.nonzero(conn_ri[i])[0] for i in range(n_ra)]
    net.ra2i_off, net.ra2i_tgt = _csr_from_lists(lists, n_ra)
    e = len(net.ra2i_tgt)
    net.ra2i_w = rng.exponential(weight_mean, e)
    net.ra2i_d = draw_delays(e)
    net.ra2i_len = np.array([d_ri[i, j] for i in range(n_ra) for j in lists[i]], dtype=np.float64)

    conn_ir = rng.random(p.T.shape) < p.T
    lists = [np.nonzero(conn_ir[i])[0] for i in range(n_i)]
    net.i2ra_off, net.i2ra_tgt = _csr_from_lists(lists, n_i)
    e = len(net.i2ra_tgt)
    net.i2ra_w = rng.exponential(weight_mean, e)
    net.i2ra_d = draw_delays(e)
    net.i2ra_len = np.array([d_ri[j, i] for i in range(n_i) for j in lists[i]], dtype=np.float64)

    net.w_rara = np.zeros((n_ra, n_ra))
    net.d_rara = draw_delays((n_ra, n_ra))
    np.fill_diagonal(net.d_rara, 0.0)
    net.len_rara = sphere_distance(net.ra_xyz, net.ra_xyz) * 40.0 / model_dist
    np.fill_diagonal(net.len_rara, 0.0)
    net.set_lists([[] for _ in range(n_ra)], [[] for _ in range(n_ra)])

    net.training = np.sort(rng.choice(n_ra, n_tr, replace=False)).astype(np.int32)
    net.training_spread = np.zeros(n_tr)
    net.rest_potential = np.full(n_ra, net.mat["E_REST_IMMATURE"])
    net.gca = np.full(n_ra, net.mat["GCA_IMMATURE"])
    net.mature = np.zeros(n_ra, dtype=np.int32)
    net.rest_potential[net.training] = net.mat["E_REST_MATURE"]
    net.gca[net.training] = net.mat["GCA_MATURE"]
    net.mature[net.training] = 1
    net.maturation_scale = np.full(n_ra, MATURATION_SCALE_SPONTANEOUS)
    net.remodeled = np.zeros(n_ra, dtype=np.int32)
    net.trials_after_replacement = np.zeros(n_ra, dtype=np.int32)
    net.activity_history = np.zeros((n_ra, int(net.mat["RATE_WINDOW_LONG"])), dtype=np.int32)
    return net.validate()


def synthetic_chain_network(n_ra=2000, n_i=550, n_groups=20, group_size=100, weight=0.05, seed=3,
                            delays="lognormal", lognormal_mean=3.0, lognormal_sigma=1.5, delay_cap=10.0,
                            num_steps=DEFAULT_NUM_STEPS, **kw) -> Network:
    """A grown network for test trials: RA->RA synfire chain of n_groups x
    group_size mature neurons, ``weight`` on every synapse between consecutive
    groups (active synapses, and super synapses up to Nss), the first group
    the training set."""
    net = synthetic_growth_network(n_ra=n_ra, n_i=n_i, n_tr=group_size, seed=seed, delays=delays,
                                   lognormal_mean=lognormal_mean, lognormal_sigma=lognormal_sigma,
                                   delay_cap=delay_cap, num_steps=num_steps, **kw)
    rng = np.random.default_rng(seed + 1000)
    order = rng.permutation(n_ra)[: n_groups * group_size].reshape(n_groups, group_size)
    active = [[] for _ in range(n_ra)]
    supers = [[] for _ in range(n_ra)]
    for g in range(n_groups - 1):
        for i in order[g]:
            for j in order[g + 1]:
                net.w_rara[i, j] = weight
                active[i].append(int(j))
                if len(supers[i]) < int(net.syn["Nss"]):
                    supers[i].append(int(j))
    net.set_lists(active, supers)
    net.training = np.sort(order[0]).astype(np.int32)
    net.training_spread = np.zeros(len(net.training))
    net.rest_potential[:] = net.mat["E_REST_MATURE"]
    net.gca[:] = net.mat["GCA_MATURE"]
    net.mature[:] = 1
    net.remodeled[:] = 0
    return net.validate()
