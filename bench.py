"""Benchmark of the per-trial hot path on GB300.

Workload (one step = one batch): the batched test-trial mix -- a fixed grown
network of 2000 HVC(RA) and 550 HVC(I) neurons on a sphere, carrying a synfire
chain of 20 groups x 100 neurons with 0.05 mS/cm^2 per synapse between
consecutive groups (reference weight 500: raiseExcWeight divides by the 10000
um^2 dendritic area), log-normal axonal delays (mean 3 ms, sd 1.5 ms, capped at
10 ms), run as 1024 independent 500 ms test trials (trial_no_stdp_fixedSpread,
24999 steps of 0.02 ms each) that differ only in their Philox noise streams.
Single precision on the device; spikes are checked against the double build.

value: trials/s of the device-resident batch (CUDA events).  e2e: the same
through the C ABI with the host copies of every step's inputs and results.
--impl reference: the CPU restatement of the reference (oracle/), on every
host core, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trials/s & neuron-RK4-steps/s vs plain FP64 GPU at \u22641-step spike err; p99 lat"
N_RA, N_I, GROUPS, GROUP, WEIGHT = 2000, 550, 20, 100, 500.0
NUM_STEPS = 25000
BATCH = 1024
SEED = 3
# Work per neuron-step of the single-precision integrators, counted from their
# source (csrc/ug_ra_f32x2.cuh, csrc/ug_i_f32.cuh): FP32 lane operations (a packed
# f32x2 operation counts 2) and SFU operations (ex2, rcp).
#   RA: 4 stages x 82 packed ops + 122 packed ops of stage sums and noise = 450 FP32 ops;
#       4 x (8 ex2 + 2 rcp) = 40 SFU
#   I : 12 stages x 63 ops + 376 ops of the DP8 tableau sums      = 1132 FP32 ops; 12 x (4 ex2 + 1 rcp) = 60 SFU
FP32_RA, FP32_I = 450, 1132
MUFU_RA, MUFU_I = 40, 60
# DRAM bytes per launch from ncu captures of the integrators at 128 trials (RA 16.4 MB and
# interneurons 21.8 MB read, ~0 written; the fused launch 38.2 MB), scaled to a launch of
# BATCH trials: the state read grows with the trials.
DRAM_BYTES_RA_PER_TRIAL = 16.4e6 / 128
DRAM_BYTES_I_PER_TRIAL = 21.8e6 / 128
CPU_WINDOWS = 8   # the headline's CPU baseline advances every core's trial in 8 equal windows
FP64_BATCH = 64   # test trials per batch of the batched double-precision figure
SERVE_REQUESTS, SERVE_RATE, SERVE_MAX_TRIALS = 16, 4.0, 10   # the latency leg of the headline


def make_network(num_steps=NUM_STEPS):
    from unsupervised_growth_gb300.network import synthetic_chain_network
    return synthetic_chain_network(n_ra=N_RA, n_i=N_I, n_groups=GROUPS, group_size=GROUP, weight=WEIGHT, seed=SEED,
                                   delays="lognormal", lognormal_mean=3.0, lognormal_sigma=1.5, delay_cap=10.0,
                                   num_steps=num_steps)


def workload_config():
    return {"workload": "batched test trials, 2000 HVC-RA + 550 HVC-I synfire-chain network (20x100, 0.05 mS/cm^2), "
                        "lognormal delays mean 3 ms, 1024 Philox-seeded 500 ms trials per step",
            "n_ra": N_RA, "n_i": N_I, "trials_per_step": BATCH, "steps_per_trial": NUM_STEPS - 1, "dt_ms": 0.02,
            "l2": "state+rings of a batch exceed L2 (129 MB); L2 also flushed between steps"}


# ---------------------------------------------------------------- CPU baseline
def _cpu_proc(conn, first_trial):
    """One CPU process: the oracle holding the config-3 network, advancing its own
    test trials window by window on command (None ends it)."""
    sys.path.insert(0, ROOT)
    from oracle.oracle import OracleNet
    onet = OracleNet(make_network())
    trial = first_trial
    onet.trial_begin(False, trial)
    conn.send("ready")
    while True:
        n = conn.recv()
        if n is None:
            break
        t0 = time.perf_counter()
        done = 0
        while done < n:
            k = onet.trial_advance(n - done)
            if k == 0:   # the trial ended inside this window: the next one starts
                onet.trial_end()
                trial += 1
                onet.trial_begin(False, trial)
                continue
            done += k
        conn.send(time.perf_counter() - t0)
    onet.trial_end()


class CpuArm:
    """`cores` processes (spawned, so none inherits a CUDA context), each running its
    own test trials of the config-3 network in the oracle.  A step advances every
    process by the same number of integration steps; over ceil(24999 / window) steps
    each process completes a whole trial, so the rate needs no extrapolation."""

    def __init__(self, cores: int, first_trial: int):
        from oracle import oracle as O
        O.build()
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for c in range(cores):
            a, b = ctx.Pipe()
            p = ctx.Process(target=_cpu_proc, args=(b, first_trial + 1000 * c), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        for a in self.conns:
            assert a.recv() == "ready"
        self.cores = cores

    def step(self, n_steps: int) -> float:
        """Wall seconds for every process to advance n_steps integration steps."""
        t0 = time.perf_counter()
        for a in self.conns:
            a.send(n_steps)
        for a in self.conns:
            a.recv()
        return time.perf_counter() - t0

    def close(self):
        for a in self.conns:
            a.send(None)
        for p in self.procs:
            p.join(timeout=60)


def cpu_sample(cores: int, windows: int = 8, first_trial: int = 5_000_000):
    """Trials/s of the oracle on `cores` processes, each integrating one whole 24999-step
    trial of the config-3 network in `windows` equal windows."""
    arm = CpuArm(cores, first_trial)
    w = -(-(NUM_STEPS - 1) // windows)
    times = [arm.step(w) for _ in range(windows)]
    arm.close()
    steps = w * windows
    return cores * steps / (NUM_STEPS - 1) / sum(times), times


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------- GPU arm
def _fp64_plain(net, device, trial, rn32):
    """Times one trial of the plain double-precision path (no batching, no graph)
    and compares the single build's spikes of the same trial with it."""
    from unsupervised_growth_gb300.compare import match_within, sorted_spikes
    from unsupervised_growth_gb300.engine import Engine
    eng64 = Engine(precision=64, device=device, use_graphs=False)
    rn64 = eng64.load_network(net)
    rn64.run_test_trials(trial, 1)
    eng64.synchronize()
    t0 = time.perf_counter()
    rn64.run_test_trials(trial, 1)
    eng64.synchronize()
    fp64_s = time.perf_counter() - t0
    rn32.run_test_trials(trial, 1)
    acc = {}
    for w, name in ((0, "soma"), (1, "dend"), (2, "interneuron")):
        a = sorted_spikes(*rn32.spikes(0, w))
        b = sorted_spikes(*rn64.spikes(0, w))
        frac, worst = match_within(a, b, 1)
        acc[name] = {"spikes_fp32": int(len(a)), "spikes_fp64": int(len(b)), "matched_within_1_step": frac,
                     "max_step_error": worst}
    rn64.free()
    eng64.close()
    return fp64_s, acc


def _fp64_batched(net, device, first, batch=FP64_BATCH):
    """Seconds for one batch of `batch` test trials of the double build with graph replay
    (after one untimed batch)."""
    from unsupervised_growth_gb300.engine import Engine
    eng64 = Engine(precision=64, device=device, use_graphs=True)
    rn64 = eng64.load_network(net)
    rn64.run_test_trials(first, batch)
    eng64.synchronize()
    t0 = time.perf_counter()
    rn64.run_test_trials(first + batch, batch)
    eng64.synchronize()
    secs = time.perf_counter() - t0
    rn64.free()
    eng64.close()
    return batch, secs


def serve_stream(eng, reqs, nets, clk_index=None):
    """Submit reqs at their arrival times to a started server, adopt and free each
    network when its request ends; returns the poll records in request order."""
    ids = [None] * len(reqs)
    t_start = time.perf_counter()

    def submitter():
        for k, (r, net) in enumerate(zip(reqs, nets)):
            delay = t_start + r.arrival - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids[k] = eng.submit(net, r.kind, 0, r.n_trials, True)

    th = threading.Thread(target=submitter)
    th.start()
    infos = [None] * len(reqs)
    pending = set(range(len(reqs)))
    while pending:
        for k in list(pending):
            if ids[k] is None:
                continue
            info = eng.poll(ids[k])
            if info["state"] in ("done", "failed"):
                infos[k] = info
                pending.discard(k)
                if info["net_id"] >= 0:
                    eng.adopt(nets[k], info["net_id"], reqs[k].kind, reqs[k].n_trials).free()
        time.sleep(0.002)
    th.join()
    return infos


def _warm_server(eng, request_cls):
    """One small request of each kind (captures both group graphs)."""
    for kind in ("growth", "test"):
        w = request_cls(0.0, kind, 300, 2, 7)
        info = eng.poll(eng.submit(w.network(), kind, 0, 2, True), 300.0)
        eng.adopt(w.network(), info["net_id"], kind, 2).free()


def serve_leg(device):
    """The latency part of the metric: a short Poisson stream of growth and test-trial
    requests through the serving loop (a fresh engine, so the headline engine's state
    is untouched).  Returns p50/p99 request latency."""
    import numpy as np

    from unsupervised_growth_gb300.engine import Engine
    from unsupervised_growth_gb300.workloads import Request, request_stream
    reqs = request_stream(n_requests=SERVE_REQUESTS, rate_hz=SERVE_RATE, max_trials=SERVE_MAX_TRIALS)
    nets = [r.network() for r in reqs]
    eng = Engine(precision=32, device=device)
    eng.server_start(max_members=64)
    _warm_server(eng, Request)
    infos = serve_stream(eng, reqs, nets)
    eng.server_stop()
    eng.close()
    lat = np.array([i["t_done"] - i["t_submit"] for i in infos])
    t0 = min(i["t_submit"] for i in infos)
    t1 = max(i["t_done"] for i in infos)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "served_trials_per_s": sum(r.n_trials for r in reqs) / (t1 - t0),
            "failed": sum(1 for i in infos if i["state"] != "done"),
            "workload": f"{SERVE_REQUESTS} requests, Poisson arrivals at {SERVE_RATE}/s, HVC-RA log-uniform "
                        f"200-8000, HVC-I = RA/4, 1-{SERVE_MAX_TRIALS} trials each, growth or test with p = 0.5, "
                        f"continuous batching in the serving loop (bench.py --workload serve runs the full stream)"}


TRIALS_PER_RANK = 1_000_000   # rank r draws the noise streams of trials [r * 1e6, (r + 1) * 1e6)


def replica_first_trial(rank: int) -> int:
    """First trial index of a replica: replicas never share a noise stream."""
    return rank * TRIALS_PER_RANK


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest replica's time (the job finishes with it)."""
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, rank, world, local_rank):
    import torch

    global BATCH
    BATCH = args.batch

    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine, calibrate_pipes

    B.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    net = make_network()
    eng = Engine(precision=32, device=local_rank, spike_capacity_per_neuron=16, use_graphs=not args.no_graphs)
    # a dedicated stream: the engine's kernels and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    rn = eng.load_network(net)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    first = replica_first_trial(rank)
    if (args.warmup + 2 * args.steps + 1) * BATCH > TRIALS_PER_RANK:
        raise SystemExit("too many trials per replica for its range of noise streams")

    for w in range(args.warmup):
        rn.run_test_trials(first + w * BATCH, BATCH)
    torch.cuda.synchronize()

    launches0 = eng.launch_count()
    step_ms = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rn.run_test_trials(first + (args.warmup + k) * BATCH, BATCH)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    total_ms = sum(step_ms)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, "cuda")
        dist.barrier()

    # e2e through the C ABI: trial list H2D, batch, per-neuron spike statistics D2H
    e2e_s = []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rn.run_test_trials(first + (args.warmup + args.steps + k) * BATCH, BATCH)
        stats = [rn.trial_stats(w) for w in (0, 1, 2)]
        e2e_s.append(time.perf_counter() - t0)
    h2d = BATCH * (4 + 8)
    d2h = sum(a.nbytes + b.nbytes for a, b in stats)
    spikes_per_trial = float(stats[0][0].sum()) / BATCH

    result = None
    if rank == 0:
        trials = BATCH * args.steps * world
        value = trials / (total_ms / 1e3)
        e2e_value = BATCH * args.steps * world / max(sum(e2e_s), 1e-9)
        mufu_peak, fma_peak = calibrate_pipes(local_rank)
        # per-kernel device time: one more batch with every launch bracketed by events, in
        # the shape the timed steps ran (both integrators of an interval fused in one
        # launch), then one with the integrators launched apart, for their split
        avg_steps = (NUM_STEPS - 1) / 2000.0   # integration steps per interval launch
        ra_ns, i_ns = BATCH * N_RA * avg_steps, BATCH * N_I * avg_steps
        work = {"k_interval_x": (ra_ns * FP32_RA + i_ns * FP32_I, ra_ns * MUFU_RA + i_ns * MUFU_I),
                "k_interval_ra": (ra_ns * FP32_RA, ra_ns * MUFU_RA), "k_interval_i": (i_ns * FP32_I, i_ns * MUFU_I)}
        kernels = {}
        for fused, names in ((True, ("k_interval_x",)), (False, ("k_interval_ra", "k_interval_i"))):
            eng.set_interval_fusion(fused)
            eng.set_kernel_timing(True)
            rn.run_test_trials(first, BATCH)
            kt = {k: eng.kernel_timing(k) for k in names + ("k_trial_init", "k_noise_events")}
            eng.set_kernel_timing(False)
            total_kernel_ms = max(sum(v[0] for v in kt.values()), 1e-9)
            for k in names:
                ms, cnt = kt[k]
                avg_ms = ms / max(cnt, 1)
                sec = max(avg_ms, 1e-9) * 1e-3
                ops, sfu = work[k]
                kernels[k] = {"launches": cnt, "avg_launch_ms": avg_ms, "share": ms / total_kernel_ms,
                              "fp32_ops_per_launch": ops, "fp32_frac": ops / sec / fma_peak,
                              "sfu_ops_per_launch": sfu, "sfu_frac": sfu / sec / mufu_peak}
        eng.set_interval_fusion(True)
        dom = "k_interval_x"   # the timed steps' kernel: 2001 of their 2003 launches per batch
        per_launch = kernels[dom]["fp32_ops_per_launch"]
        achieved = per_launch / (kernels[dom]["avg_launch_ms"] * 1e-3)

        # plain double-precision GPU path: one trial per run, no batching, no graph;
        # and the double build batched, to split the speed-up into batching and precision
        fp64 = None if args.skip_fp64 else _fp64_plain(net, local_rank, first, rn)
        fp64_batched = None if args.skip_fp64 else _fp64_batched(net, local_rank, first + 500_000)
        latency = None if args.skip_serve else serve_leg(local_rank)
        cores = os.cpu_count() or 1
        cpu_rate, cpu_times = cpu_sample(cores, CPU_WINDOWS) if not args.skip_cpu else (None, [])
        result = {
            "metric": METRIC,
            "value": value, "unit": "trials/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded network and Philox noise)",
            "config": dict(workload_config(), parallelism=f"replicas{world}"),
            "neuron_steps_per_s": value * (N_RA + N_I) * (NUM_STEPS - 1),
            "e2e": {"value": e2e_value, "unit": "trials/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fma_peak / 1e12, "unit": "T FP32 ops/s",
                         "frac": achieved / fma_peak, "kernel": dom,
                         "traffic": (DRAM_BYTES_RA_PER_TRIAL + DRAM_BYTES_I_PER_TRIAL) * BATCH,
                         "traffic_source": "ncu captures of the integrators at 128 trials, scaled by the trials "
                                           "per launch",
                         "split": "k_interval_ra and k_interval_i: the same batch with the integrators launched "
                                  "apart (ug_set_interval_fusion 0)",
                         "peak_source": "FP32 FMA throughput loop (ug_calibrate_pipes), measured in this run; "
                                        "SFU peak (ex2+rcp loop) also measured",
                         "sfu_peak_gops": mufu_peak / 1e9, "kernels": kernels,
                         "algorithmic_per_launch": f"{per_launch:.4g} FP32 ops (RA {FP32_RA}, I {FP32_I} per "
                                                   f"neuron-step x neurons x {avg_steps:.4f} steps x {BATCH} trials)"},
            "soma_spikes_per_trial": spikes_per_trial,
            "clocks": clk.summary(),
        }
        if fp64 is not None:
            fp64_s, acc = fp64
            result["fp64_plain_gpu"] = {"trials_per_s": 1.0 / fp64_s, "speedup_of_value": value * fp64_s,
                                        "how": "one trial per run, no batching, no graph, double precision"}
            result["accuracy_vs_fp64"] = acc
        if fp64_batched is not None:
            b64, s64 = fp64_batched
            result["fp64_batched_gpu"] = {"trials_per_s": b64 / s64, "trials_per_batch": b64,
                                          "speedup_of_value": value / (b64 / s64),
                                          "how": "the double build with the production batching and graph replay: "
                                                 "value / this = the single-precision gain, this / fp64_plain_gpu "
                                                 "= the batching gain"}
        if latency is not None:
            result["latency"] = latency
        if cpu_rate is not None:
            result["cpu_baseline"] = {"value": cpu_rate, "unit": "trials/s", "cores": cores, "kind": "port",
                                      "sample": f"oracle/ (the double-precision CPU port, bit-identical to the "
                                                f"reference's NetworkGrowthSimulator on the pinned cases) on all "
                                                f"{cores} host cores, one process per core, each integrating one "
                                                f"whole 24999-step trial of this network in {CPU_WINDOWS} windows; "
                                                f"no extrapolation",
                                      "wall_s": sum(cpu_times)}
    rn.free()
    eng.close()
    if dist:
        dist.destroy_process_group()
    return result


# Fast-growing synaptic and maturation parameters (the growth parity tests' set): the
# active and super topology change within a few trials, so single and double precision
# can be compared on a topology that has grown.
FAST_SYN = dict(Nss=2, A_P=20.0, A_D=20.0 / 1.05, T_0=0.0, T_P=10.0, T_D=10.0, TAU_P=30.0, TAU_D=30.0, BETA=0.2,
                BETA_SUPERSYNAPSE=0.2, ACTIVATION_THRESHOLD=10.0, SUPERSYNAPSE_THRESHOLD=40.0, WEIGHT_MAX=160.0)
FAST_MAT = dict(RATE_WINDOW_LONG=1000, E_REST_IMMATURE=-65.0, GCA_IMMATURE=25.0, DEATH_RATE_THRESHOLD=0.01)


def make_growth_network(num_steps=NUM_STEPS, fast=False):
    """The config-2 network; `fast`: fast-growing synapses, with the ten training neurons
    spread over 15 ms so that they potentiate onto one another and supersynapses form."""
    import numpy as np

    from unsupervised_growth_gb300.network import synthetic_growth_network
    extra = dict(syn=FAST_SYN, mat=FAST_MAT) if fast else {}
    net = synthetic_growth_network(n_ra=N_RA, n_i=N_I, n_tr=10, seed=2, delays="lognormal", lognormal_mean=3.0,
                                   lognormal_sigma=1.5, delay_cap=10.0, num_steps=num_steps, **extra)
    if fast:
        net.training_spread = np.linspace(0.0, 15.0, len(net.training))
    return net


def run_growth(args, local_rank):
    """Growth at scale: one network, consecutive growth trials (a step is one trial
    together with its between-trial bookkeeping).  Single-precision neurons with
    double-precision weights, against the plain double-precision path."""
    import torch

    from unsupervised_growth_gb300 import autotune
    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine
    B.build()
    torch.cuda.set_device(local_rank)
    net = make_growth_network(num_steps=args.num_steps)
    eng = Engine(precision=32, device=local_rank, use_graphs=not args.no_graphs)
    rn = eng.load_network(net)
    rn.run_growth_trials(0, args.warmup, True)
    eng.synchronize()
    eng.set_kernel_timing(False)
    # the block shape of the one-launch trial, tuned on the run's own next trials
    nxt = [args.warmup]

    def one_trial():
        rn.run_growth_trials(nxt[0], 1, True)
        eng.synchronize()
        nxt[0] += 1

    cache = autotune.DEFAULT_CACHE if args.autotune_cache is None else (args.autotune_cache or None)
    tuned = autotune.tune_growth_trial(eng, one_trial,
                                       sig=autotune.trial_signature(_device_name(local_rank), N_RA, N_I, 32),
                                       cache_path=cache)
    first = nxt[0]
    l0 = eng.launch_count()
    with ClockSampler(local_rank) as clk:
        t0 = time.perf_counter()
        rn.run_growth_trials(first, args.steps, True)
        eng.synchronize()
        wall = time.perf_counter() - t0
    launches = eng.launch_count() - l0
    rep_events, rep_neurons = rn.replacement_count()
    sup32 = [sorted(x) for x in rn.synapse_list(1)]
    per_interval, kt = None, {}
    if not args.skip_compare:
        # the same network's next trials with per-interval launches (the shape the
        # one-launch trial replaces), for comparison
        eng.set_growth_launch(False)
        n_cmp = 3
        nxt = first + args.steps
        rn.run_growth_trials(nxt, 1, True)   # captures that shape's graph
        eng.synchronize()
        t0 = time.perf_counter()
        rn.run_growth_trials(nxt + 1, n_cmp, True)
        eng.synchronize()
        per_interval = n_cmp / (time.perf_counter() - t0)
        eng.set_growth_launch(True)
        eng.set_kernel_timing(True)   # kernel timing runs the per-interval launches, one kernel at a time
        rn.run_growth_trials(nxt + 1 + n_cmp, 1, True)
        names = ("k_interval_ra", "k_interval_i", "k_growth_rows", "k_growth_newpost", "k_growth_ltp",
                 "k_growth_epilogue", "k_trial_init", "k_noise_events", "k_growth_reset")
        kt = {k: eng.kernel_timing(k) for k in names}
        eng.set_kernel_timing(False)
    trial_ms = (args.num_steps - 1) * 0.02
    result = {"metric": f"growth trials/s ({trial_ms:g} ms growth trials, 2000 RA + 550 I network, one network)",
              "value": args.steps / wall, "unit": "trials/s", "n_gpus": 1, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
              "dtype": "f32 neurons, f64 weights", "data": "synthetic (seeded network and Philox noise)",
              "config": {"workload": "growth trials of one 2000 HVC-RA + 550 HVC-I sphere network, lognormal "
                                     "delays mean 3 ms capped 10 ms, 10 training neurons", "trial_ms": trial_ms},
              "neuron_steps_per_s": args.steps / wall * (N_RA + N_I) * (args.num_steps - 1),
              "gpu_launches": launches, "clocks": clk.summary(),
              "replacements": {"events": rep_events, "neurons": rep_neurons,
                               "supersynapses_at_end": sum(len(x) for x in sup32)},
              "launch": "one cooperative kernel per trial (all sync intervals, bounded grid barriers)",
              "trial_shape": {"ra_threads": tuned["shape"][0], "i_threads": tuned["shape"][1],
                              "cached": tuned["cached"],
                              "table": [[t["shape"][0], t["shape"][1], round(1e3 * t["seconds"], 2)]
                                        for t in tuned["table"]],
                              "how": "autotuned [ra, i, ms per trial]; 0 = default (32 threads)"},
              "per_interval_launches_trials_per_s": per_interval,
              "kernel_ms_per_trial": {k: round(v[0], 3) for k, v in kt.items()},
              "kernel_ms_how": "per-interval launches timed one kernel at a time"}
    if not args.skip_fp64:
        eng64 = Engine(precision=64, device=local_rank, use_graphs=False)
        eng64.set_growth_launch(False)   # the plain path: per-interval launches, no graph
        rn64 = eng64.load_network(net)
        t0 = time.perf_counter()
        rn64.run_growth_trials(0, args.warmup + args.steps, True)
        eng64.synchronize()
        fp64_wall = time.perf_counter() - t0
        sup64 = [sorted(x) for x in rn64.synapse_list(1)]
        result["fp64_plain_gpu"] = {"trials_per_s": (args.warmup + args.steps) / fp64_wall,
                                    "how": "double precision, no graph, same trials"}
        result["same_supersynapse_topology_as_fp64"] = sup32 == sup64
        rn64.free()
        eng64.close()
    rn.free()
    eng.close()
    return result


def _device_name(device):
    import torch
    return torch.cuda.get_device_name(device).replace(" ", "_")


def _fp64_plain_seconds(nets, device, kind):
    """Seconds per trial of the plain double-precision path (one trial, no batching,
    no graph) for each network."""
    from unsupervised_growth_gb300.engine import Engine
    eng = Engine(precision=64, device=device, use_graphs=False)
    eng.set_growth_launch(False)   # the plain path: per-interval launches, no graph
    out = []
    for net in nets:
        rn = eng.load_network(net)
        t0 = time.perf_counter()
        if kind == "growth":
            rn.run_growth_trials(0, 1, True)
        else:
            rn.run_test_trials(0, 1)
        eng.synchronize()
        out.append(time.perf_counter() - t0)
        rn.free()
    eng.close()
    return out


def _interp_loglog(xs, ys, x):
    import numpy as np
    order = np.argsort(xs)
    lx, ly = np.log(np.asarray(xs, float)[order]), np.log(np.asarray(ys, float)[order])
    if len(lx) == 1:
        return float(ys[0] * x / xs[0])
    k = int(np.clip(np.searchsorted(lx, np.log(x)) - 1, 0, len(lx) - 2))
    slope = (ly[k + 1] - ly[k]) / (lx[k + 1] - lx[k]) if lx[k + 1] > lx[k] else 1.0
    return float(np.exp(ly[k] + slope * (np.log(x) - lx[k])))


def run_uneven(args, local_rank):
    """Batched growth of many networks of uneven size: one step = one group round,
    i.e. one growth trial of every network, all stepped by the same launches."""
    from unsupervised_growth_gb300 import autotune
    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine
    from unsupervised_growth_gb300.workloads import uneven_networks
    B.build()
    nets = uneven_networks(args.members)
    eng = Engine(precision=32, device=local_rank)
    rns = [eng.load_network(n) for n in nets]
    trial = [0]

    def one_round():
        eng.run_group([(rn, "growth", trial[0], 1, True) for rn in rns])
        trial[0] += 1

    one_round()   # first round: growth state set-up and graph capture
    sig = autotune.signature(_device_name(local_rank), [(n.n_ra, "growth", 1) for n in nets])
    cache = autotune.DEFAULT_CACHE if args.autotune_cache is None else (args.autotune_cache or None)
    tuned = autotune.tune(eng, one_round, sig=sig, max_rounds=max(args.warmup, 6), cache_path=cache)
    while trial[0] < args.warmup:
        one_round()
    l0 = eng.launch_count()
    with ClockSampler(local_rank) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            one_round()
        wall = time.perf_counter() - t0
    launches = eng.launch_count() - l0
    eng.set_kernel_timing(True)
    one_round()
    names = ("k_trial_init", "k_noise_events", "k_growth_reset", "k_interval_ra", "k_interval_i",
             "k_growth_rows_heavy", "k_growth_rows", "k_growth_newpost", "k_growth_ltp", "k_growth_epilogue",
             "k_check_bad")
    kt = {k: round(eng.kernel_timing(k)[0], 3) for k in names}
    eng.set_kernel_timing(False)
    neurons = sum(n.n_ra + n.n_i for n in nets)
    res = {"metric": f"growth trials/s ({len(nets)} growing networks of uneven size, one group)",
           "value": len(nets) * args.steps / wall, "unit": "trials/s", "n_gpus": 1, "steps": args.steps,
           "warmup": trial[0] - args.steps - 1, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
           "dtype": "f32 neurons, f64 weights", "data": "synthetic (seeded networks and Philox noise)",
           "config": {"workload": f"{len(nets)} growing networks, HVC-RA log-uniform 200-8000 (seed 4), HVC-I = RA/4, "
                                  "uniform delays 0-w, w in {0,1,3,6,10} ms round-robin; a step is one growth trial "
                                  "of every network",
                      "ra_total": int(sum(n.n_ra for n in nets)), "ra_min": int(min(n.n_ra for n in nets)),
                      "ra_max": int(max(n.n_ra for n in nets))},
           "neuron_steps_per_s": neurons * (NUM_STEPS - 1) * args.steps / wall,
           "gpu_launches": launches, "clocks": clk.summary(),
           "autotune": {"shape": list(tuned["shape"]), "cached": tuned["cached"], "rounds": tuned["rounds"],
                        "table": tuned["table"]},
           "kernel_ms_per_round": kt}
    if not args.skip_sequential:
        # the same trials one network at a time on the single-network path
        seq = 0.0
        for rn in rns:
            rn.run_growth_trials(trial[0], 1, True)   # captures the network's graph
            eng.synchronize()
            t0 = time.perf_counter()
            rn.run_growth_trials(trial[0] + 1, 1, True)
            eng.synchronize()
            seq += time.perf_counter() - t0
        res["one_network_at_a_time"] = {"s_per_round": seq, "group_speedup": seq / (wall / args.steps)}
    if not args.skip_fp64:
        order = sorted(range(len(nets)), key=lambda k: nets[k].n_ra)
        pick = [order[0], order[len(order) // 2], order[-1]]
        secs = _fp64_plain_seconds([nets[k] for k in pick], local_rank, "growth")
        est = sum(_interp_loglog([nets[k].n_ra for k in pick], secs, n.n_ra) for n in nets)
        res["fp64_plain_gpu"] = {"sampled_networks_ra": [nets[k].n_ra for k in pick], "s_per_trial": secs,
                                 "est_s_per_round": est, "est_speedup_of_value": est / (wall / args.steps),
                                 "how": "double precision, one network and one trial at a time, no graph; the "
                                        "round time is interpolated (log-log in HVC-RA count) from 3 sampled networks"}
    for rn in rns:
        rn.free()
    eng.close()
    return res


def run_create(args, local_rank):
    """createNetworkForGrowth on the device: a step generates one network topology
    (coordinates with minimum-distance rejection, RA<->I connections, training
    arrangements) of the given size on the sphere, each step from its own seed.
    value: networks/s of device time; e2e: networks/s through ug_generate_topology
    (host arrays out, device-to-host copies included); cpu_baseline: the sequential
    oracle on one core, a few networks of the same size."""
    import math

    import torch

    from oracle import oracle as O
    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine
    B.build()
    torch.cuda.set_device(local_rank)
    n_ra, n_i = (int(x) for x in args.create_size.split("x"))
    p = dict(A_RA2I=0.1, SIGMA_RA2I=120 / math.sqrt(2.0), B_I2RA=0.1, SIGMA_I2RA=120 / math.sqrt(2.0))
    eng = Engine(precision=32, device=local_rank)
    for s in range(args.warmup):
        eng.generate_topology(p, n_ra, n_i, 10, seed=1000 + s).free()
    dev_ms, walls, edges, launches, stages = [], [], 0, 0, [0.0, 0.0, 0.0]
    d2h = 0
    with ClockSampler(local_rank) as clk:
        for s in range(args.steps):
            t0 = time.perf_counter()
            t = eng.generate_topology(p, n_ra, n_i, 10, seed=s)
            walls.append(time.perf_counter() - t0)
            i = t.info
            dev_ms.append(i["device_ms"])
            edges += i["n_ra2i"] + i["n_i2ra"]
            launches += i["launches"]
            stages = [a + b for a, b in zip(stages, (i["interneuron_ms"], i["placement_ms"], i["connection_ms"]))]
            d2h = 24 * (n_ra + n_i) + 4 * (n_ra + n_i + 2) + 12 * (i["n_ra2i"] + i["n_i2ra"])
            t.free()
    value = 1e3 * args.steps / sum(dev_ms)
    e2e = args.steps / sum(walls)
    # the oracle on one core, a bounded sample
    ncpu = max(1, min(args.steps, 5 if n_ra <= 4000 else 1))
    t0 = time.perf_counter()
    for s in range(ncpu):
        O.generate_topology(p, n_ra, n_i, 10, seed=s)
    cpu = ncpu / (time.perf_counter() - t0)
    return {"metric": f"networks/s (createNetworkForGrowth topology, {n_ra} RA + {n_i} I on the sphere)",
            "value": value, "unit": "networks/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sum(dev_ms) / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (f32 prefilters)", "data": "synthetic (seeded topology streams)",
            "config": {"workload": f"topology generation, {n_ra} HVC-RA + {n_i} HVC-I on the sphere, A = 0.1, "
                                   f"sigma = 120/sqrt(2) um, 10 training neurons, a new seed per step",
                       "stage_ms": {"interneurons": stages[0] / args.steps, "placement": stages[1] / args.steps,
                                    "connections": stages[2] / args.steps},
                       "edges_per_network": edges / args.steps, "l2": "inputs are a few MB; not flushed"},
            "e2e": {"value": e2e, "unit": "networks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk.summary(),
            "cpu_baseline": {"value": cpu, "unit": "networks/s", "cores": 1, "kind": "port",
                             "sample": f"{ncpu} networks of the same size from the sequential oracle"}}


def run_serve(args, local_rank):
    """Serving: growth and test-trial requests of mixed network size arrive as a
    Poisson stream; the engine's scheduler admits them by device footprint into the
    running group rounds.  Reports latency percentiles and trials/s."""
    import numpy as np

    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine
    from unsupervised_growth_gb300.workloads import Request, request_stream
    B.build()
    reqs = request_stream(n_requests=args.requests, rate_hz=args.rate)
    nets = [r.network() for r in reqs]
    eng = Engine(precision=32, device=local_rank)
    eng.server_start(max_members=args.members)
    _warm_server(eng, Request)
    with ClockSampler(local_rank) as clk:
        infos = serve_stream(eng, reqs, nets)
    eng.server_stop()
    failed = [i for i in infos if i["state"] != "done"]
    lat = np.array([i["t_done"] - i["t_submit"] for i in infos])
    wait = np.array([i["t_admit"] - i["t_submit"] for i in infos])
    t0 = min(i["t_submit"] for i in infos)
    t1 = max(i["t_done"] for i in infos)
    trials = sum(r.n_trials for r in reqs)
    nsteps = sum(r.n_trials * (r.n_ra + max(r.n_ra // 4, 1)) * (NUM_STEPS - 1) for r in reqs)
    res = {"metric": "served trials/s and request latency (Poisson stream of growth and test-trial requests)",
           "value": trials / (t1 - t0), "unit": "trials/s", "n_gpus": 1, "steps": len(reqs), "warmup": 2,
           "ms_per_step": 1e3 * (t1 - t0) / len(reqs), "higher_is_better": True, "dtype": "f32 neurons, f64 weights",
           "data": "synthetic (seeded request stream, networks and Philox noise)",
           "config": {"workload": f"{len(reqs)} requests, Poisson arrivals at {args.rate}/s, HVC-RA log-uniform "
                                  "200-8000, HVC-I = RA/4, 1-50 trials per request, growth or test with p = 0.5",
                      "trials": trials, "max_members": args.members},
           "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                         "max": float(lat.max())},
           "queue_wait_s": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
           "neuron_steps_per_s": nsteps / (t1 - t0), "failed": len(failed), "clocks": clk.summary()}
    if not args.skip_fp64:
        est = 0.0
        sample = {}
        for kind in ("growth", "test"):
            sizes = [r.n_ra for r in reqs if r.kind == kind]
            if not sizes:
                continue
            pick = sorted({min(sizes), int(np.median(sizes)), max(sizes)})
            from unsupervised_growth_gb300.workloads import Request
            secs = _fp64_plain_seconds([Request(0.0, kind, n, 1, 99).network() for n in pick], local_rank, kind)
            sample[kind] = {"ra": pick, "s_per_trial": secs}
            est += sum(r.n_trials * _interp_loglog(pick, secs, r.n_ra) for r in reqs if r.kind == kind)
        res["fp64_plain_serial"] = {"est_seconds": est, "est_trials_per_s": trials / est,
                                    "speedup_of_value": (trials / (t1 - t0)) / (trials / est), "sample": sample,
                                    "how": "every request alone, one trial at a time, double precision, no graph; "
                                           "per-trial times interpolated (log-log in HVC-RA count) from sampled sizes"}
    eng.close()
    return res


def run_topology(args, local_rank):
    """Single precision against the double build over consecutive growth trials of
    the 2000/550 growth network: per trial, the grown supersynapse and active
    topology, the weights and the spikes; reports the first trial whose topology
    differs, if any.  A step is one growth trial of both builds."""
    import numpy as np

    from unsupervised_growth_gb300.compare import match_within, sorted_spikes
    from unsupervised_growth_gb300 import build as B
    from unsupervised_growth_gb300.engine import Engine
    B.build()
    net = make_growth_network(num_steps=args.num_steps, fast=args.fast_growth)
    e32, e64 = Engine(precision=32, device=local_rank), Engine(precision=64, device=local_rank)
    r32, r64 = e32.load_network(net), e64.load_network(net)
    first_div = {"super": None, "active": None}
    worst_w, worst_rel, min_match, worst_step, spikes = 0.0, 0.0, 1.0, 0, 0
    t32 = t64 = 0.0
    for t in range(args.steps):
        t0 = time.perf_counter()
        r32.run_growth_trials(t, 1, True)
        e32.synchronize()
        t32 += time.perf_counter() - t0
        t0 = time.perf_counter()
        r64.run_growth_trials(t, 1, True)
        e64.synchronize()
        t64 += time.perf_counter() - t0
        for which, key in ((1, "super"), (0, "active")):
            a = [sorted(x) for x in r32.synapse_list(which)]
            b = [sorted(x) for x in r64.synapse_list(which)]
            if a != b and first_div[key] is None:
                first_div[key] = t
        w32, w64 = r32.weights(), r64.weights()
        d = np.abs(w32 - w64)
        worst_w = max(worst_w, float(d.max()))
        worst_rel = max(worst_rel, float((d / np.maximum(np.abs(w64), 1e-300))[w64 != 0].max(initial=0.0)))
        a, b = sorted_spikes(*r32.spikes(0, 0)), sorted_spikes(*r64.spikes(0, 0))
        frac, worst = match_within(a, b, 1)
        spikes += len(b)
        min_match, worst_step = min(min_match, frac), max(worst_step, worst)
    sup = sum(len(x) for x in r64.synapse_list(1))
    res = {"metric": "growth topology agreement, single vs double precision (consecutive growth trials)",
           "value": args.steps if first_div["super"] is None else first_div["super"], "unit": "trials",
           "n_gpus": 1, "steps": args.steps, "warmup": 0, "higher_is_better": True,
           "dtype": "f32 neurons, f64 weights vs f64", "data": "synthetic (seeded network and Philox noise)",
           "config": {"workload": "growth trials of one 2000 HVC-RA + 550 HVC-I sphere network, lognormal delays "
                                  "mean 3 ms capped 10 ms, 10 training neurons"
                                  + (", fast-growing synapses (A_P 20, thresholds 10/40, Nss 2)" if args.fast_growth
                                     else ""),
                      "trial_ms": (args.num_steps - 1) * 0.02},
           "first_divergent_trial": first_div, "supersynapses_at_end": sup,
           "max_weight_abs_error": worst_w, "max_weight_rel_error": worst_rel,
           "soma_spikes_fp64": spikes, "min_fraction_matched_within_1_step": min_match, "max_step_error": worst_step,
           "s_per_trial": {"f32": t32 / args.steps, "f64": t64 / args.steps},
           "value_means": "trials before the supersynapse topology first differs (= steps if never)"}
    for r in (r32, r64):
        r.free()
    e32.close()
    e64.close()
    return res


def run_reference(args, rank):
    """The CPU path of the reference on the host cores, for the config-3 workload: every
    core runs its own test trials of the 2000 / 550 chain network in the double-precision
    CPU port (oracle/), which tests/test_reference_sim.py shows bit-identical to the
    reference's own NetworkGrowthSimulator.  The reference's trial code itself needs the
    reference tree, which is not on the GPU host.  A step advances every core by
    ceil(24999 / steps) integration steps, so the timed steps cover one whole trial per
    core; the warm-up steps advance a separate warm-up trial by 200 steps each."""
    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    window = -(-(NUM_STEPS - 1) // max(args.steps, 1))
    warm = CpuArm(cores, 6_000_000)
    for _ in range(args.warmup):
        warm.step(200)
    warm.close()
    arm = CpuArm(cores, 7_000_000)
    times = [arm.step(window) for _ in range(args.steps)]
    arm.close()
    trials = cores * window * args.steps / (NUM_STEPS - 1)
    value = trials / sum(times)
    sample = (f"all {cores} host cores, one process per core, each advancing its own 24999-step test trial of the "
              f"config-3 network by {window} steps per step; {args.steps} steps = {trials / cores:.3f} trial per core; "
              f"oracle/ (the double-precision CPU port, bit-identical to the reference's NetworkGrowthSimulator on "
              f"the pinned cases)")
    return {"impl": "reference", "metric": METRIC, "value": value,
            "unit": "trials/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded network and Philox noise)",
            "config": dict(workload_config(), parallelism=f"cpu{cores}", trials_per_step=trials / args.steps),
            "cpu_baseline": {"value": value, "unit": "trials/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "trials/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="test",
                    choices=["test", "growth", "uneven", "serve", "topology", "create"],
                    help="test: batched test trials (the headline); growth: consecutive growth trials of one "
                         "network; uneven: one group of growing networks of uneven size; serve: a Poisson stream "
                         "of requests through the serving loop; topology: single vs double precision over "
                         "consecutive growth trials; create: network topology generation (createNetworkForGrowth)")
    ap.add_argument("--create-size", default="2000x550", help="create: HVC(RA) x HVC(I)")
    ap.add_argument("--num-steps", type=int, default=NUM_STEPS,
                    help="growth, topology: steps per trial + 1 (25000: 500 ms trials; profiling runs use fewer)")
    ap.add_argument("--fast-growth", action="store_true",
                    help="topology: fast-growing synaptic parameters, so that supersynapses form within a few trials")
    ap.add_argument("--members", type=int, default=64, help="uneven: networks in the group; serve: member slots")
    ap.add_argument("--requests", type=int, default=48, help="serve: requests in the stream")
    ap.add_argument("--rate", type=float, default=2.0, help="serve: arrivals per second")
    ap.add_argument("--skip-sequential", action="store_true", help="uneven: skip the one-network-at-a-time timing")
    ap.add_argument("--autotune-cache", default=None,
                    help="uneven, growth: autotuner cache file ('' to tune every run; default: the package's cache)")
    ap.add_argument("--batch", type=int, default=BATCH, help="test trials per step (profiling runs use fewer)")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernels directly instead of graph replay")
    ap.add_argument("--skip-cpu", action="store_true", help="do not time the CPU baseline")
    ap.add_argument("--skip-fp64", action="store_true", help="do not time the plain double-precision GPU path")
    ap.add_argument("--skip-compare", action="store_true",
                    help="growth: do not time the per-interval launches and their per-kernel split")
    ap.add_argument("--skip-serve", action="store_true", help="do not run the serving-latency leg of the headline")
    args = ap.parse_args()
    if args.gpus > 1 and "RANK" not in os.environ:
        # one process per GPU: relaunch under torch.distributed.run on this node
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
        raise SystemExit(subprocess.call(cmd))
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        res = run_reference(args, rank)
    elif args.workload == "growth":
        res = run_growth(args, local_rank) if rank == 0 else None
    elif args.workload == "uneven":
        res = run_uneven(args, local_rank) if rank == 0 else None
    elif args.workload == "serve":
        res = run_serve(args, local_rank) if rank == 0 else None
    elif args.workload == "topology":
        res = run_topology(args, local_rank) if rank == 0 else None
    elif args.workload == "create":
        res = run_create(args, local_rank) if rank == 0 else None
    else:
        res = run_ours(args, rank, world, local_rank)
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
