"""Benchmark of the UJ step on the random-cloud workload (N = 2^20 particles,
X ~ U[0,1]^3, Gamma ~ N(0, 1e-3), sigma ~ U[0.01, 0.03], Gaussian-erf kernel,
FP32-comp form).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one all-pairs UJ evaluation (U and J of every particle from every
particle: N^2 pair slots).  `value` times steps on device-resident inputs
(vpm_uj_dev); `e2e` times the reference-facing drop-in (vpm_uj on the host
46-row particle matrix, host<->device copies included).  One JSON line is
printed by rank 0.  Under torchrun each rank evaluates its own field
(independent replicas, weak scaling, no collective on the data path).

--impl reference times the oracle port of the reference's CPU UJ_direct
(oracle/, OpenMP over every host core) on a bounded sample of the same
workload: the reference itself (Julia + FastMultipole.jl) cannot be installed
here.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "flowvpm.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

N_PARTICLES = 1 << 20
KERNEL = 2            # gaussianerf
FLOP_PER_PAIR = 74    # VPM_FLOP_PER_UJ_PAIR
FLOP_PER_ADJ_PAIR = 186   # VPM_FLOP_PER_UJ_ADJ_PAIR
# DRAM bytes of one uj_mixed_kernel<gaussianerf> launch at N = 2^20, measured by ncu
# (`ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#  --clock-control none -k regex:uj_mixed_kernel -c 1 python bench.py --kernel-only --n 1048576
#  --warmup 0 --steps 1`): 405,746,944 read + 181,722,112 written.  The compulsory traffic is
# ~0.16 GB (56 B in, 96 B out a particle); the rest is re-reads of the 50 MB source pack that
# miss L2.  Either way it is ~0.42 GB/s over the 1.41 s launch: the kernel is FP32-bound.
UJ_DRAM_BYTES_2P20 = 405_746_944 + 181_722_112
# (warp, 32-source tile) pairs within reach that one estr_mixed_kernel<gaussianerf> launch
# loads on the 200,000-particle leapfrog rings: one cp.async commit (LDGDEPBAR) per loaded tile
# in ncu's per-opcode counts of `python bench.py --kernel-only --estr --cloud rings --n 200000
# --warmup 0 --steps 1` (2,967,977 commits, 4 LDGSTS each), of the 6,250 x 6,250 tile pairs.
# The reach depends on the positions and core sizes only, which the workload fixes.
ESTR_TILES_IN_REACH_RINGS200K = 2_967_977
# the headline metric as the reference's benchmark definition names it; `value` is the
# FP32-comp rate, `fp64_gpu` / `mixed_over_fp64` and `adjoint` carry the other two parts
METRIC = "UJ pair-interactions/s, FP32-comp vs FP64 GPU @≤1e-6 rel err; adjoint/fwd ratio"
WORKLOAD = "random cloud UJ: N=2^20, X~U[0,1]^3, Gamma~N(0,1e-3), sigma~U[0.01,0.03], gaussianerf"


def random_cloud(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(0.0, 1.0, (n, 3)), rng.normal(0.0, 1e-3, (n, 3)), rng.uniform(0.01, 0.03, n))


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- helpers
def max_over_ranks(ms: float, dist, device: str) -> float:
    """The slowest rank's time (every rank gets it); `dist` None = one process."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, units_per_step: float, steps: int, elapsed_ms: float) -> float:
    """Whole-job rate of `world` independent replicas, each doing `units_per_step`
    per step, timed by the slowest rank."""
    return world * units_per_step * steps / (elapsed_ms / 1e3)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def cpu_baseline(X, G, s, budget_s=12.0):
    """The oracle (FP64 reference formula) on every host core, on a bounded
    sample: all N sources against a prefix of the targets."""
    import oracle
    cores = os.cpu_count() or 1
    nt = 64
    t0 = time.perf_counter()
    oracle.uj_pairs(X[:nt], X, G, s, KERNEL)
    dt = time.perf_counter() - t0
    rate0 = nt * X.shape[0] / dt
    nt = int(min(X.shape[0], max(cores * 16, rate0 * budget_s / X.shape[0])))
    nt -= nt % (cores * 16) or 0
    nt = max(nt, cores * 16)
    t0 = time.perf_counter()
    oracle.uj_pairs(X[:nt], X, G, s, KERNEL)
    dt = time.perf_counter() - t0
    return {"value": nt * X.shape[0] / dt, "unit": "pairs/s", "cores": cores, "kind": "port",
            "sample": f"{nt} targets x {X.shape[0]} sources ({nt * X.shape[0]:.3e} pairs) in {dt:.1f} s; "
                      "oracle/vpm_oracle.c oracle_uj_pairs, FP64 reference formula, OpenMP"}


def run_reference(args, rank, world):
    """--impl reference: the oracle port of UJ_direct on the host cores."""
    if rank != 0:
        return
    X, G, s = random_cloud(N_PARTICLES, seed=0)
    import oracle
    cores = os.cpu_count() or 1
    # bounded sample per step: all sources against `nt` targets (~5 s of CPU work)
    nt = cores * 32
    for _ in range(max(0, args.warmup)):
        oracle.uj_pairs(X[:cores * 4], X, G, s, KERNEL)
    times = []
    for k in range(args.steps):
        sl = slice((k * nt) % (N_PARTICLES - nt), (k * nt) % (N_PARTICLES - nt) + nt)
        t0 = time.perf_counter()
        oracle.uj_pairs(X[sl], X, G, s, KERNEL)
        times.append(time.perf_counter() - t0)
    pairs = nt * N_PARTICLES
    value = pairs * len(times) / sum(times)
    # the small configuration in full: all pairs of a 2^14 cloud, median of 5 after one warm-up
    Xs, Gs, ss = random_cloud(1 << 14, seed=0)
    oracle.uj_pairs(Xs, Xs, Gs, ss, KERNEL)
    small = []
    for _ in range(5):
        t0 = time.perf_counter()
        oracle.uj_pairs(Xs, Xs, Gs, ss, KERNEL)
        small.append(time.perf_counter() - t0)
    small_rate = float(1 << 28) / statistics.median(small)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_per_step": f"{nt} targets x {N_PARTICLES} sources"},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                             "sample": f"{nt} targets x {N_PARTICLES} sources per step, {args.steps} steps"},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "n_2p14_all_pairs": {"value": small_rate, "unit": "pairs/s", "ms": 1e3 * statistics.median(small),
                                 "note": "all 2^28 pairs of a 2^14 cloud, median of 5"},
            "note": "oracle port (oracle/vpm_oracle.c) of UJ_direct's pair loop: the reference (Julia + "
                    "FastMultipole.jl) cannot be installed in this environment"}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world):
    import torch
    import vpm_gb300 as vpm

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    ctx = vpm.Context(dev)
    n = N_PARTICLES
    X, G, s = random_cloud(n, seed=1000 * rank)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    xt, gs, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    flush = torch.empty(64 << 20, device="cuda", dtype=torch.float32)   # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream()

    def step():
        U.zero_()
        J.zero_()
        ctx.uj_dev(xt, xt, gs, sg, U, J, KERNEL, vpm.FP32COMP)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(dev) as clk:
        barrier()
        t_start = time.perf_counter()
        total = torch.cuda.Event(enable_timing=True)
        total_end = torch.cuda.Event(enable_timing=True)
        total.record(stream)
        for k in range(args.steps):
            flush.fill_(float(k))            # L2 flush between timed steps
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        total_end.record(stream)
        barrier()
        wall = time.perf_counter() - t_start
    launches = ctx.launches - launches0
    elapsed_ms = total.elapsed_time(total_end)
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    elapsed_ms = max_over_ranks(elapsed_ms, dist, "cuda")
    pairs_per_step = float(n) * n
    value = replica_rate(world, pairs_per_step, args.steps, elapsed_ms)
    # dominant kernel: the UJ launch (pack is O(N), microseconds); flops per launch / avg duration
    avg_kernel_s = statistics.mean(kernel_ms) / 1e3
    achieved_tflops = FLOP_PER_PAIR * pairs_per_step / avg_kernel_s / 1e12

    # FP32 FFMA peak of this GPU, measured now (the driver's peaks file has HBM and bf16 only)
    ffma = vpm.Context(dev)
    peak_tflops = measure_ffma_peak(ffma)

    # ---- end to end through the reference-facing call (host 46-row matrix)
    P = np.zeros((46, n), order="F")
    P[0:3] = X.T
    P[3:6] = G.T
    P[6] = s
    ctx.set_stream(None)
    ctx.uj(P, n, KERNEL, vpm.FP32COMP, vpm._lib.RESET)   # warm (allocations)
    e2e_times = []
    for _ in range(args.steps):   # as many calls as timed device steps
        t0 = time.perf_counter()
        ctx.uj(P, n, KERNEL, vpm.FP32COMP, vpm._lib.RESET)
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * pairs_per_step / statistics.mean(e2e_times)

    out = None
    if rank == 0:
        # accuracy of this very run against the oracle on a seeded subset of targets
        import oracle
        sub = np.sort(np.random.default_rng(5).choice(n, 256, replace=False))
        Ur, Jr = oracle.uj_pairs(X[sub], X, G, s, KERNEL)
        Uh, Jh = U.cpu().numpy()[sub], J.cpu().numpy()[sub]
        err = {"U_max_rel": float(np.abs(Uh - Ur).max() / np.abs(Ur).max()),
               "J_max_rel": float(np.abs(Jh - Jr).max() / np.abs(Jr).max()),
               "U_rms_rel": float(np.linalg.norm(Uh - Ur) / np.linalg.norm(Ur)),
               "J_rms_rel": float(np.linalg.norm(Jh - Jr) / np.linalg.norm(Jr)),
               "targets_checked": 256}
        dfma_peak = measure_dfma_peak(ffma)
        fp64 = fp64_rate(ctx, vpm, torch, X, G, s, dfma_peak)
        wnk = winckelmans_rate(ctx, vpm, torch, X, G, s)
        adjoint = adjoint_ratio(ctx, vpm, torch, peak_tflops, dfma_peak)
        estr_b, lf_b = rings_blocks(ctx, vpm, torch, peak_tflops)
        jet_b = jet_block(ctx, vpm, torch, peak_tflops)
        base = cpu_baseline(X, G, s)
        mp = measured_peaks()
        out = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 positions/accumulation)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_particles": n, "kernel": "gaussianerf",
                       "precision": "fp32comp", "pairs_per_step": pairs_per_step,
                       "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": 8 * 8 * n,
                    "d2h_bytes_per_step": 12 * 8 * n, "ms_per_step": 1e3 * statistics.mean(e2e_times),
                    "call": "vpm_uj(ctx, host 46xN matrix, RESET) = UJ_gb300_mixed(pfield)"},
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak_tflops,
                         "unit": "TFLOP/s", "frac": achieved_tflops / peak_tflops,
                         "traffic": UJ_DRAM_BYTES_2P20 if n == 1 << 20 else None,
                         "traffic_unit": "bytes per launch",
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one N=2^20 launch "
                                           "(405.7 + 181.7 MB; 1 pass, --clock-control none)",
                         "kernel": "uj_mixed_kernel<gaussianerf>",
                         "flop_per_pair": FLOP_PER_PAIR,
                         "peak_source": "FFMA-loop kernel measured in this run (no FP32 figure in "
                                        "MEASURED_PEAKS.json)",
                         "peak_nominal_2070MHz": 152 * 128 * 2 * 2.07e9 / 1e12,
                         "hbm_peak_gbs_measured": mp.get("hbm_gbs")},
            "cpu_baseline": base,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "fp64_gpu": fp64,
            "winckelmans": wnk,
            "mixed_over_fp64": fp64["mixed_over_fp64_same_config"],
            "adjoint": adjoint,
            "estr": estr_b,
            "leapfrog_step": lf_b,
            "jet": jet_b,
            "error_vs_oracle": err,
            "wall_s_timed_region": wall,
        }
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


def fp64_rate(ctx, vpm, torch, X, G, s, fp64_peak):
    """The plain FP64 form and the FP32-comp form on the same configuration:
    2^15 seeded targets of the 2^20 cloud against all of its sources (one timed
    evaluation each, after a warm-up), and the FP64 form's fraction of the
    DFMA-loop peak."""
    n = X.shape[0]
    nt = 1 << 15
    sub = np.sort(np.random.default_rng(15).choice(n, nt, replace=False))
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    xt, xs, gs, sg = d(X[sub]), d(X), d(G), d(s)
    U = torch.zeros(nt, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(nt, 9, device="cuda", dtype=torch.float64)
    out = {"targets": nt, "sources": n, "pairs": float(nt) * n}
    for prec, tag in ((vpm.FP64, "fp64"), (vpm.FP32COMP, "fp32comp")):
        ctx.uj_dev(xt[:1024], xs, gs, sg, U[:1024], J[:1024], KERNEL, prec)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ctx.uj_dev(xt, xs, gs, sg, U, J, KERNEL, prec)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out[f"ms_{tag}"] = ms
        out[f"pairs_per_s_{tag}"] = float(nt) * n / (ms / 1e3)
    out["value"] = out["pairs_per_s_fp64"]
    out["unit"] = "pairs/s"
    out["mixed_over_fp64_same_config"] = out["pairs_per_s_fp32comp"] / out["pairs_per_s_fp64"]
    ach = FLOP_PER_PAIR * out["pairs_per_s_fp64"] / 1e12
    out["roofline_fp64"] = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                            "frac": ach / fp64_peak if fp64_peak else None, "kernel": "uj_f64_kernel<gaussianerf>",
                            "peak_source": "DFMA-loop kernel measured in this run (vpm_probe_dfma)"}
    return out


def _timed_min(torch, fn, reps=3):
    """Minimum CUDA-event time (ms) of `reps` calls after one warm-up call."""
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def rings_blocks(ctx, vpm, torch, peak_tflops):
    """The leapfrogging-rings workload (two coaxial rings, R = 1 and 0.7, 10
    particles a section, 200,000 particles, Gaussian-erf, FP32-comp):
    * `estr`: one Estr pass (vpm_estr_dev, J from the field's own UJ) at 25 flop
      per pair over all N^2 pair slots;
    * `leapfrog_step`: whole device-resident rVPM RK3 steps with the dynamic SFS
      procedure, core spreading and relaxation, against the work of the
      reference's own step: per step it evaluates 5 UJ and 4 Estr passes over
      all pairs (3 stages of UJ + Estr, the test filter's UJ + Estr, the
      relaxation's UJ), 5 x 74 + 4 x 25 = 470 flop per pair slot."""
    from vpm_gb300 import device_step as ds, workloads
    X, G, s = workloads.leapfrog_rings(200_000)
    n = X.shape[0]
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    S = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    ctx.uj_dev(x, x, g, sg, U, J, KERNEL, vpm.FP32COMP)
    ms_estr = _timed_min(torch, lambda: ctx.estr_dev(x, J, x, g, sg, J, S, KERNEL, vpm.FP32COMP, True))
    ms_uj = _timed_min(torch, lambda: ctx.uj_dev(x, x, g, sg, U, J, KERNEL, vpm.FP32COMP))
    pairs = float(n) * n
    estr_tf = 25 * pairs / (ms_estr / 1e3) / 1e12
    uj_tf = FLOP_PER_PAIR * pairs / (ms_uj / 1e3) / 1e12
    in_reach = ESTR_TILES_IN_REACH_RINGS200K * 32 * 32
    estr = {"workload": "leapfrog rings, 200,000 particles, FP32-comp", "n_particles": n, "ms": ms_estr,
            "pairs_per_s": pairs / (ms_estr / 1e3), "flop_per_pair": 25, "achieved_tflops": estr_tf,
            "all_pair_slots_frac_of_ffma_peak": estr_tf / peak_tflops,
            "tile_pairs_in_reach": in_reach,
            "in_reach_frac_of_ffma_peak": 25 * in_reach / (ms_estr / 1e3) / 1e12 / peak_tflops,
            "kernel": "estr_mixed_kernel<gaussianerf>",
            "uj_ms_same_field": ms_uj, "uj_frac_of_ffma_peak": uj_tf / peak_tflops,
            "note": "pairs_per_s and all_pair_slots_frac count all N^2 pair slots, as the reference evaluates "
                    "them; tiles and 8-source sub-blocks whose every pair is past zeta/zeta(0) < 1e-13 are "
                    "skipped (their terms are below FP32 resolution), so that figure reads above 1. "
                    "tile_pairs_in_reach = the 32 x 32 pair slots of the (warp, source tile) pairs the kernel "
                    "loads (ncu count of one launch on this workload); in_reach_frac counts those at 25 flop"}
    fld = ds.DeviceField(x.clone(), g.clone(), sg.clone(), kernel=KERNEL, precision=vpm.FP32COMP)
    sfs = ds.DynamicSFSParams()
    visc = ds.CoreSpreadingParams(nu=1e-4, sgm0=0.05)
    step = lambda: ds.rk3_step(fld, 0.005, ctx, sfs=sfs, viscous=visc, relax_rlxf=0.3)
    ms_step = _timed_min(torch, step, reps=3)
    flop_step = (5 * 74 + 4 * 25) * pairs
    ach = flop_step / (ms_step / 1e3) / 1e12
    lf = {"workload": "leapfrog rings, 200,000 particles, FP32-comp, dynamic SFS, core spreading, relaxation",
          "ms_per_step": ms_step, "particle_steps_per_s": n / (ms_step / 1e3),
          "reference_flop_per_pair_slot": 470, "achieved_tflops": ach, "frac_of_ffma_peak": ach / peak_tflops,
          "note": "UJ + stretching + SFS: the reference's step evaluates 5 UJ and 4 Estr passes over all pairs "
                  "(74 and 25 flop a pair); this step evaluates 4 UJ, 3 Estr, and the test filter's differences "
                  "directly (one J-difference pass and 2 Estr), and its time includes every kernel of the step"}
    return estr, lf


def jet_block(ctx, vpm, torch, peak_tflops):
    """The jet-like cloud with the FMM near field (2^20 particles in a cylinder,
    sigma = 0.02, leaf size 64, theta = 0.4): one near-field UJ call (octree,
    lists and P2P on the GPU), and the P2P alone (lists reused)."""
    from vpm_gb300 import workloads
    X, G, s = workloads.jet_cloud(1 << 20)
    n = X.shape[0]
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    kw = dict(leaf_size=64, theta=0.4, kernel=KERNEL, precision=vpm.FP32COMP)
    st = ctx.p2p_leaflist_dev(x, g, sg, U, J, **kw)
    ms_call = _timed_min(torch, lambda: ctx.p2p_leaflist_dev(x, g, sg, U, J, **kw))
    ms_p2p = _timed_min(torch, lambda: ctx.p2p_leaflist_dev(x, g, sg, U, J, reuse=True, **kw))
    pairs = float(st[2])
    ach = FLOP_PER_PAIR * pairs / (ms_p2p / 1e3) / 1e12
    return {"workload": "jet-like cloud, 2^20 particles, near field (leaf 64, theta 0.4), FP32-comp UJ",
            "leaves": st[0], "leaf_pairs": st[1], "pairs": pairs, "ms_per_call": ms_call,
            "pairs_per_s_call": pairs / (ms_call / 1e3), "ms_p2p": ms_p2p, "pairs_per_s_p2p": pairs / (ms_p2p / 1e3),
            "achieved_tflops_p2p": ach, "frac_of_ffma_peak_p2p": ach / peak_tflops,
            "note": "ms_per_call builds the octree and lists and runs the P2P; ms_p2p reuses the lists "
                    "(VPM_REUSE_LISTS): packs + P2P"}


def winckelmans_rate(ctx, vpm, torch, X, G, s):
    """The same cloud with the Winckelmans kernel, FP32-comp: one timed
    evaluation and its error against the oracle on 256 seeded targets."""
    import oracle
    n = X.shape[0]
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    xt, gs, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    ctx.uj_dev(xt[:4096], xt, gs, sg, U[:4096], J[:4096], vpm._lib.KERNEL_WINCKELMANS, vpm.FP32COMP)
    U.zero_()
    J.zero_()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    ctx.uj_dev(xt, xt, gs, sg, U, J, vpm._lib.KERNEL_WINCKELMANS, vpm.FP32COMP)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    sub = np.sort(np.random.default_rng(6).choice(n, 256, replace=False))
    Ur, Jr = oracle.uj_pairs(X[sub], X, G, s, vpm._lib.KERNEL_WINCKELMANS)
    Uh, Jh = U.cpu().numpy()[sub], J.cpu().numpy()[sub]
    return {"value": float(n) * n / (ms / 1e3), "unit": "pairs/s", "n_particles": n, "ms": ms,
            "kernel": "uj_mixed_kernel<winckelmans>",
            "error_vs_oracle": {"U_max_rel": float(np.abs(Uh - Ur).max() / np.abs(Ur).max()),
                                "J_max_rel": float(np.abs(Jh - Jr).max() / np.abs(Jr).max()),
                                "targets_checked": 256}}


def adjoint_ratio(ctx, vpm, torch, ffma_peak, dfma_peak, n=32000):
    """FP64 UJ adjoint (vpm_uj_adjoint_dev) vs FP64 UJ forward on an n-particle
    ring (1000 sections x 32 per section, the rollout workload's size), and a
    5-step rollout gradient (with per-step recompute) vs its forward."""
    import vpm_gb300.rings as rings
    from vpm_gb300 import autodiff as ad
    X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, n // 32, 32, 0.05)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    rng = np.random.default_rng(0)
    Ub, Jb = d(rng.normal(size=(n, 3))), d(rng.normal(size=(n, 9)))
    xb, gb, sb = torch.zeros_like(x), torch.zeros_like(g), torch.zeros_like(sg)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b)
    fwd = timed(lambda: ctx.uj_dev(x, x, g, sg, U, J, KERNEL, vpm.FP64))
    adj = timed(lambda: ctx.uj_adjoint_dev(x, g, sg, Ub, Jb, xb, gb, sb, KERNEL, vpm.FP64))
    fwd32 = timed(lambda: ctx.uj_dev(x, x, g, sg, U, J, KERNEL, vpm.FP32COMP))
    adj32 = timed(lambda: ctx.uj_adjoint_dev(x, g, sg, Ub, Jb, xb, gb, sb, KERNEL, vpm.FP32COMP))
    steps = 5
    kw = dict(kernel=KERNEL, precision=vpm.FP64, vctx=ctx)

    def roll_fwd():
        with torch.no_grad():
            ad.ring_loss(*ad.rollout(x, g, sg, 0.01, steps, checkpoint=False, **kw), **kw)

    def roll_grad(mode):
        def run():
            xx, gg, ss = x.clone().requires_grad_(), g.clone().requires_grad_(), sg.clone().requires_grad_()
            ad.ring_loss(*ad.rollout(xx, gg, ss, 0.01, steps, checkpoint=mode, **kw), **kw).backward()
        return run
    t_roll = timed(roll_fwd)
    t_grad = timed(roll_grad(True))
    t_grad_rc = timed(roll_grad("recompute"))
    # the SFS stretching pass Estr and its adjoint (vpm_estr_adjoint_dev) on the same ring, J from its UJ
    Sb = d(rng.normal(size=(n, 3)))
    SFS = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    Jb2 = torch.zeros_like(J)
    estr = {}
    for prec, tag in ((vpm.FP64, "fp64"), (vpm.FP32COMP, "fp32comp")):
        U.zero_(); J.zero_()
        ctx.uj_dev(x, x, g, sg, U, J, KERNEL, prec)
        f = timed(lambda: ctx.estr_dev(x, J, x, g, sg, J, SFS, KERNEL, prec, True))
        a_ = timed(lambda: ctx.estr_adjoint_dev(x, g, sg, J, Sb, xb, gb, sb, Jb2, KERNEL, prec, True))
        estr.update({f"estr_fwd_ms_{tag}": f, f"estr_adjoint_ms_{tag}": a_, f"estr_adjoint_over_fwd_{tag}": a_ / f})
    # a 5-step rollout with the ConstantSFS term: gradient (forward + backward) over forward
    kw_sfs = dict(kw, sfs=ad.ConstantSFS(Cs=1.0))

    def roll_fwd_sfs():
        with torch.no_grad():
            ad.ring_loss(*ad.rollout(x, g, sg, 0.01, steps, checkpoint=False, **kw_sfs), **kw)

    def roll_grad_sfs():
        xx, gg, ss = x.clone().requires_grad_(), g.clone().requires_grad_(), sg.clone().requires_grad_()
        ad.ring_loss(*ad.rollout(xx, gg, ss, 0.01, steps, checkpoint=True, **kw_sfs), **kw).backward()
    t_roll_sfs = timed(roll_fwd_sfs)
    t_grad_sfs = timed(roll_grad_sfs)
    estr.update({"sfs_rollout_fwd_ms": t_roll_sfs, "sfs_rollout_grad_ms": t_grad_sfs,
                 "sfs_rollout_grad_over_fwd": t_grad_sfs / t_roll_sfs})
    def roof(ms, peak, pipe):
        ach = FLOP_PER_ADJ_PAIR * n * n / (ms / 1e3) / 1e12
        return {"bound": pipe, "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "flop_per_pair": FLOP_PER_ADJ_PAIR}
    return {"n_particles": n, "uj_fwd_ms": fwd, "uj_adjoint_ms": adj, "uj_adjoint_over_fwd": adj / fwd,
            "uj_fwd_ms_fp32comp": fwd32, "uj_adjoint_ms_fp32comp": adj32,
            "uj_adjoint_over_fwd_fp32comp": adj32 / fwd32,
            "uj_adjoint_roofline_fp64": roof(adj, dfma_peak, "fp64"),
            "uj_adjoint_roofline_fp32comp": roof(adj32, ffma_peak, "fp32"), **estr,
            "rollout_steps": steps, "rollout_fwd_ms": t_roll, "rollout_grad_ms": t_grad,
            "rollout_grad_over_fwd": t_grad / t_roll, "rollout_backward_over_fwd": (t_grad - t_roll) / t_roll,
            "rollout_grad_recompute_ms": t_grad_rc, "rollout_grad_recompute_over_fwd": t_grad_rc / t_roll,
            "note": "FP64 forward and adjoint, Gaussian-erf.  rollout_grad = forward + backward with per-step "
                    "checkpointing that keeps each step's UJ values; backward = rollout_grad - forward; "
                    "_recompute re-runs each step's UJ evaluations in the backward pass; estr_* = the Estr pass "
                    "(vpm_estr_dev) and its adjoint (vpm_estr_adjoint_dev, gradients w.r.t. x, Gamma, sigma, J); "
                    "sfs_rollout_* = the FP64 rollout with the ConstantSFS term (Cs = 1)"}


def measure_dfma_peak(ctx) -> float:
    """TFLOP/s of a pure DFMA loop (vpm_probe_dfma in the library)."""
    out = np.zeros(1)
    rc = ctx._L.vpm_probe_dfma(ctx._h, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(ctx._L.vpm_last_error(ctx._h).decode())
    return float(out[0])


def measure_ffma_peak(ctx) -> float:
    """TFLOP/s of a pure FFMA loop (vpm_probe_ffma in the library)."""
    import vpm_gb300._lib as L
    out = np.zeros(1)
    rc = ctx._L.vpm_probe_ffma(ctx._h, out.ctypes.data)
    if rc != 0:
        raise RuntimeError(ctx._L.vpm_last_error(ctx._h).decode())
    return float(out[0])


def run_kernel_only(args):
    """Profiling helper: only the UJ (or Estr, or with --adjoint the UJ adjoint)
    kernels on an n-particle cloud -- for --adjoint, the 32,000-particle ring of
    the rollout workload -- `warmup` + `steps` evaluations, no other work (for
    ncu captures)."""
    import torch
    import vpm_gb300 as vpm
    n = args.n
    prec = vpm.FP64 if args.precision == "fp64" else vpm.FP32COMP
    kern = {"singular": 0, "gaussian": 1, "gaussianerf": 2, "winckelmans": 3}[args.kernel]
    ctx = vpm.Context(0)
    if args.adjoint:
        import vpm_gb300.rings as rings
        X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, 1000, 32, 0.05)
        n = X.shape[0]
    elif args.cloud == "rings":   # the leapfrogging rings of n particles
        from vpm_gb300 import workloads
        X, G, s = workloads.leapfrog_rings(n)
        n = X.shape[0]
    else:
        X, G, s = random_cloud(n, seed=1)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    xt, gs, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    SFS = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    if args.estr:      # Estr reads the field's own J
        ctx.uj_dev(xt, xt, gs, sg, U, J, kern, prec)
    if args.adjoint:   # cotangents of U and J: seeded, O(1)
        rng = np.random.default_rng(7)
        U.copy_(torch.from_numpy(rng.normal(size=(n, 3))))
        J.copy_(torch.from_numpy(rng.normal(size=(n, 9))))
        xb, gb, sb = torch.zeros_like(xt), torch.zeros_like(gs), torch.zeros_like(sg)
    times = []
    for k in range(args.warmup + args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        if args.adjoint:
            ctx.uj_adjoint_dev(xt, gs, sg, U, J, xb, gb, sb, kern, prec)
        elif args.estr:
            ctx.estr_dev(xt, J, xt, gs, sg, J, SFS, kern, prec, True)
        else:
            ctx.uj_dev(xt, xt, gs, sg, U, J, kern, prec)
        b.record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            times.append(a.elapsed_time(b))
    ms = statistics.mean(times) if times else float("nan")
    print(json.dumps({"mode": "kernel-only", "n": n, "precision": args.precision, "kernel": args.kernel,
                      "estr": bool(args.estr), "adjoint": bool(args.adjoint), "ms": ms,
                      "pairs_per_s": n * n / (ms / 1e3),
                      "launches": ctx.launches}))


def _device_field(X, G, s, precision, torch, ds):
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    return ds.DeviceField(d(X), d(G), d(s), kernel=KERNEL, precision=precision)


def _leapfrog_run(ctx, X, G, s, precision, nsteps, dt, monitor_every, torch, ds, with_sfs=True):
    """nsteps device-resident RK3 steps with dynamic SFS (with_sfs), core
    spreading and relaxation; impulse and energy (fresh UJ) every
    `monitor_every` steps.  Returns (ms per step, monitor rows [(step, t, I, E)], field)."""
    fld = _device_field(X, G, s, precision, torch, ds)
    sfs = ds.DynamicSFSParams() if with_sfs else None
    visc = ds.CoreSpreadingParams(nu=1e-4, sgm0=0.05)
    mon = []

    def monitor(k):
        ds.uj(fld, ctx)
        mon.append((k, fld.t, ds.impulse(fld).cpu().numpy().tolist(), ds.energy(fld)))
    monitor(0)
    step_ms = 0.0
    for k in range(1, nsteps + 1):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ds.rk3_step(fld, dt, ctx, sfs=sfs, viscous=visc, relax_rlxf=0.3)
        b.record()
        torch.cuda.synchronize()
        step_ms += a.elapsed_time(b)
        if k % monitor_every == 0 or k == nsteps:
            monitor(k)
    return step_ms / nsteps, mon, fld


def _drift(mon):
    I0, E0 = np.array(mon[0][2]), mon[0][3]
    return {"impulse_rel_drift": float(np.linalg.norm(np.array(mon[-1][2]) - I0) / np.linalg.norm(I0)),
            "energy_rel_drift": float((mon[-1][3] - E0) / abs(E0))}


def run_leapfrog(args):
    """Leapfrogging coaxial rings: R=1 and R=0.7, 0.3 apart axially, Gamma=1
    each, a=0.1R, 10 particles per section, sigma=a/2 (~200k particles),
    Gaussian-erf, rVPM, dynamic SFS (two-level, no backscatter), core spreading
    nu=1e-4, Pedrizzetti relaxation, RK3 with dt=0.005.

    * FP32-comp at full size for --lf-steps steps: ms/step, particle-steps/s,
      impulse I = 1/2 sum x x Gamma and energy E = 1/2 sum U.(x x Gamma) drift;
    * FP64 against FP32-comp at full size over --lf-f64-steps steps (state
      difference), and over the whole run at --lf-small particles (monitor
      trajectories of both precisions)."""
    import torch
    import vpm_gb300 as vpm
    from vpm_gb300 import device_step as ds, workloads
    ctx = vpm.Context(0)
    dt = 0.005
    out = {"mode": "leapfrog", "steps": args.lf_steps, "dt": dt, "precision": "fp32comp"}
    # pair passes per FP32-comp step: 3 stage UJ + Estr, the relaxation UJ, and the dynamic
    # procedure's differences (one filter-difference pass over the J term, two Estr passes)
    passes = {"uj": 4, "estr": 5, "filter_difference": 1}
    if args.lf_n > 0:
        X, G, s = workloads.leapfrog_rings(args.lf_n, nper=10)
        n = X.shape[0]
        ms32, mon32, f32 = _leapfrog_run(ctx, X, G, s, vpm.FP32COMP, args.lf_steps, dt, 20, torch, ds)
        out.update({"n_particles": n, "ms_per_step": ms32, "particle_steps_per_s": n / (ms32 / 1e3),
                    "pairs_per_s": sum(passes.values()) * float(n) * n / (ms32 / 1e3),
                    "pair_passes_per_step": passes,
                    "drift_fp32comp": _drift(mon32), "monitor_fp32comp": mon32})
    # FP64 vs FP32-comp on the full-size field over a few steps
    k64 = args.lf_f64_steps if args.lf_n > 0 else 0
    if k64 > 0:
        ms64, m64, f64 = _leapfrog_run(ctx, X, G, s, vpm.FP64, k64, dt, k64, torch, ds)
        _, m32s, f32s = _leapfrog_run(ctx, X, G, s, vpm.FP32COMP, k64, dt, k64, torch, ds)
        rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
        out["fp64_full_size"] = {"steps": k64, "ms_per_step_fp64": ms64, "fp32comp_speedup": ms64 / ms32,
                                 "x_max_rel": rel(f32s.x, f64.x), "gamma_max_rel": rel(f32s.gam, f64.gam),
                                 "sigma_max_rel": rel(f32s.sig, f64.sig), "U_max_rel": rel(f32s.U, f64.U),
                                 "J_max_rel": rel(f32s.J, f64.J),
                                 "energy_rel_diff": (m32s[-1][3] - m64[-1][3]) / abs(m64[-1][3])}
    # whole run, both precisions, at reduced size, with two controls: the same
    # comparison without the SFS model, and FP64 against FP64 started from
    # strengths perturbed by 1e-7 (relative, seeded) -- the size of the
    # FP32-comp UJ error
    if args.lf_small > 0:
        Xs, Gs, ss = workloads.leapfrog_rings(args.lf_small, nper=10)
        Gp = Gs * (1.0 + 1e-7 * np.random.default_rng(9).standard_normal(Gs.shape))

        def diff(ma, mb):
            dI = max(np.linalg.norm(np.array(a[2]) - np.array(b[2])) / np.linalg.norm(np.array(b[2]))
                     for a, b in zip(ma, mb))
            dE = max(abs(a[3] - b[3]) / abs(b[3]) for a, b in zip(ma, mb))
            return {"impulse_max_rel_diff": float(dI), "energy_max_rel_diff": float(dE)}
        run = lambda prec, G_, sfs_: _leapfrog_run(ctx, Xs, G_, ss, prec, args.lf_steps, dt, 20, torch, ds, sfs_)
        ms64s, mon64, _ = run(vpm.FP64, Gs, True)
        ms32s, mon32s, _ = run(vpm.FP32COMP, Gs, True)
        _, mon64p, _ = run(vpm.FP64, Gp, True)
        _, mon64n, _ = run(vpm.FP64, Gs, False)
        _, mon32n, _ = run(vpm.FP32COMP, Gs, False)
        out["fp64_vs_fp32comp_small"] = {"n_particles": Xs.shape[0], "steps": args.lf_steps,
                                         "ms_per_step_fp64": ms64s, "ms_per_step_fp32comp": ms32s,
                                         "drift_fp64": _drift(mon64), "drift_fp32comp": _drift(mon32s),
                                         "fp32comp_vs_fp64": diff(mon32s, mon64),
                                         "control_fp64_perturbed_1e-7_vs_fp64": diff(mon64p, mon64),
                                         "control_no_sfs_fp32comp_vs_fp64": diff(mon32n, mon64n),
                                         "drift_no_sfs_fp64": _drift(mon64n),
                                         "monitor_fp64": mon64, "monitor_fp32comp": mon32s}
    print(json.dumps(out), flush=True)


def run_jet(args):
    """Round-jet-like cloud with the FMM near field: 2^20 particles uniform in
    a cylinder (radius 0.5, length 4), Gamma = vol * curl A of a seeded random
    Fourier field with a Gaussian spectrum, sigma = 0.02, Gaussian-erf.  The
    octree (leaf size 64, theta = 0.4) and its leaf-pair lists are built on the
    GPU at every UJ call, and every near leaf pair is evaluated by P2P in
    FP32-comp (UJ, and Estr where the step asks for it).  The far field is not
    computed.  Reported: the tree build alone, one UJ (+Estr) call, one call of
    the dynamic procedure's near-field differences, and whole rVPM RK3 steps
    with dynamic SFS and relaxation (4 near-field UJ calls, 3 with Estr, and
    the differences)."""
    import torch
    import vpm_gb300 as vpm
    from vpm_gb300 import device_step as ds, workloads
    ctx = vpm.Context(0)
    X, G, s = workloads.jet_cloud(args.jet_n)
    n = X.shape[0]
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    S = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    leaf, theta = 64, 0.4

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            out = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps, out
    import vpm_gb300._lib as L
    sizes = np.zeros(3, dtype=np.int64)

    def tree_only():
        rc = ctx._L.vpm_leaflist_dev(ctx._h, n, x.data_ptr(), leaf, theta, None, None, None, None, None,
                                     sizes.ctypes.data)
        if rc != 0:
            raise L.VPMError(rc, ctx._L.vpm_last_error(ctx._h).decode())
    ms_tree, _ = timed(tree_only, 5)
    kw = dict(leaf_size=leaf, theta=theta, kernel=KERNEL, precision=vpm.FP32COMP)
    ms_uj, st = timed(lambda: ctx.p2p_leaflist_dev(x, g, sg, U, J, **kw), 5)
    ms_ujs, _ = timed(lambda: ctx.p2p_leaflist_dev(x, g, sg, U, J, S, sfs=True, **kw), 5)
    dJ, dS = torch.zeros_like(J), torch.zeros_like(S)
    ms_dyn, _ = timed(lambda: ctx.dynamic_diff_leaflist_dev(x, g, sg, J, 0.999, dJ, dS, **kw), 5)
    ms_uj64, _ = timed(lambda: ctx.p2p_leaflist_dev(x, g, sg, U, J, leaf_size=leaf, theta=theta, kernel=KERNEL,
                                                    precision=vpm.FP64), 1)
    # accuracy of the FP32-comp near field against the FP64 near field over the same lists
    U32, J32 = torch.zeros_like(U), torch.zeros_like(J)
    U64, J64 = torch.zeros_like(U), torch.zeros_like(J)
    ctx.p2p_leaflist_dev(x, g, sg, U32, J32, **kw)
    ctx.p2p_leaflist_dev(x, g, sg, U64, J64, leaf_size=leaf, theta=theta, kernel=KERNEL, precision=vpm.FP64)
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
    pairs = st[2]
    # whole steps
    fld = ds.DeviceField(x.clone(), g.clone(), sg.clone(), kernel=KERNEL, precision=vpm.FP32COMP)
    fld.leaflist = (leaf, theta)
    sfs = ds.DynamicSFSParams()
    ds.rk3_step(fld, 1e-3, ctx, sfs=sfs, relax_rlxf=0.3)        # warm-up
    torch.cuda.synchronize()
    nst = args.jet_steps
    t0 = time.perf_counter()
    for _ in range(nst):
        ds.rk3_step(fld, 1e-3, ctx, sfs=sfs, relax_rlxf=0.3)
    torch.cuda.synchronize()
    ms_step = (time.perf_counter() - t0) * 1e3 / nst
    out = {"mode": "jet", "n_particles": n, "leaf_size": leaf, "theta": theta, "leaves": st[0], "leaf_pairs": st[1],
           "particle_pairs_per_uj": pairs, "pairs_per_particle": pairs / n,
           "tree_build_ms": ms_tree,
           "uj_call_ms": ms_uj, "uj_pairs_per_s": pairs / (ms_uj / 1e3),
           "uj_estr_call_ms": ms_ujs, "uj_estr_pairs_per_s": 2 * pairs / (ms_ujs / 1e3),
           "dynamic_diff_call_ms": ms_dyn,
           "uj_call_ms_fp64": ms_uj64, "fp32comp_over_fp64": ms_uj64 / ms_uj,
           "err_fp32comp_vs_fp64": {"U_max_rel": rel(U32, U64), "J_max_rel": rel(J32, J64)},
           "step_ms": ms_step, "steps_timed": nst, "particle_steps_per_s": n / (ms_step / 1e3),
           "step": "rVPM RK3 + dynamic SFS + Pedrizzetti relaxation: 4 near-field UJ calls (3 with Estr) and "
                   "the near-field test-filter differences; the tree is built at each UJ call and reused by "
                   "the differences",
           "far_field": "not computed (FastMultipole.jl's multipole part is outside this library)"}
    print(json.dumps(out), flush=True)


def run_rollout(args):
    """Adjoint of a rollout: the isolated ring at 1000 sections x 32 particles
    (32,000 particles, R=1, a=0.1R, sigma=a/2, Gaussian-erf), rVPM RK3 with
    Pedrizzetti relaxation, --ro-steps steps of dt=0.01; loss = kinetic-energy
    estimate + strength-weighted axial centroid at the final step.  FP64
    forward and its gradient with per-step checkpointing (each step's UJ values
    kept, the adjoint kernel in the backward pass), checked against central
    differences (h = each of --ro-h, 1e-6 by default) along --ro-dirs seeded random unit
    directions in (X, Gamma, sigma); the FP32-comp forward is timed beside it."""
    import torch
    import vpm_gb300 as vpm
    import vpm_gb300.rings as rings
    from vpm_gb300 import autodiff as ad
    ctx = vpm.Context(0)
    X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, 1000, 32, 0.05)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x0, g0, s0 = d(X), d(G), d(s)
    steps, dt = args.ro_steps, 0.01
    sfs = ad.ConstantSFS(Cs=args.ro_sfs) if args.ro_sfs > 0 else None
    kw = dict(kernel=KERNEL, precision=vpm.FP64, vctx=ctx)
    kw_step = dict(kw, sfs=sfs)

    def loss_at(x, g, sg, prec=vpm.FP64):
        k2 = dict(kernel=KERNEL, precision=prec, vctx=ctx)
        with torch.no_grad():
            return float(ad.ring_loss(*ad.rollout(x, g, sg, dt, steps, checkpoint=False, sfs=sfs, **k2), **k2))

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, out
    ms_fwd, L0 = timed(lambda: loss_at(x0, g0, s0))
    ms_fwd32, L32 = timed(lambda: loss_at(x0, g0, s0, vpm.FP32COMP))

    def grad():
        x, g, sg = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
        ad.ring_loss(*ad.rollout(x, g, sg, dt, steps, checkpoint=True, **kw_step), **kw).backward()
        return x.grad, g.grad, sg.grad
    ms_grad, (gx, gg, gs) = timed(grad)
    # the same gradient with the FP32-comp forward and adjoints, against the FP64 one

    def grad32():
        k32 = dict(kernel=KERNEL, precision=vpm.FP32COMP, vctx=ctx)
        x, g, sg = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
        ad.ring_loss(*ad.rollout(x, g, sg, dt, steps, checkpoint=True, sfs=sfs, **k32), **k32).backward()
        return x.grad, g.grad, sg.grad
    ms_grad32, g32 = timed(grad32)
    g32_rel = max(float((a - b).abs().max() / b.abs().max()) for a, b in zip(g32, (gx, gg, gs)))
    rng = np.random.default_rng(3)
    hs = [float(t) for t in args.ro_h.split(",")]
    h = hs[0]
    worst = 0.0
    worst_by_h = {f"{t:g}": 0.0 for t in hs}
    checks = []
    # with two or more steps, the Richardson combination of the last two, (r^2 fd(h2) - fd(h1)) /
    # (r^2 - 1) with r = h1/h2, cancels the h^2 term of the central differences' error
    worst_rich = 0.0
    for _ in range(args.ro_dirs):
        v = [d(rng.normal(size=t.shape)) for t in (x0, g0, s0)]
        nrm = math.sqrt(sum(float((t * t).sum()) for t in v))
        v = [t / nrm for t in v]
        an = float((gx * v[0]).sum() + (gg * v[1]).sum() + (gs * v[2]).sum())
        fds = []
        for t in hs:
            fd = (loss_at(x0 + t * v[0], g0 + t * v[1], s0 + t * v[2]) -
                  loss_at(x0 - t * v[0], g0 - t * v[1], s0 - t * v[2])) / (2 * t)
            fds.append(fd)
            rel = abs(fd - an) / max(abs(an), 1e-300)
            worst_by_h[f"{t:g}"] = max(worst_by_h[f"{t:g}"], rel)
            if t == h:
                worst = max(worst, rel)
            checks.append({"h": t, "fd": fd, "adjoint": an, "rel": rel})
        if len(hs) >= 2:
            r2 = (hs[-2] / hs[-1]) ** 2
            rich = (r2 * fds[-1] - fds[-2]) / (r2 - 1.0)
            worst_rich = max(worst_rich, abs(rich - an) / max(abs(an), 1e-300))
    print(json.dumps({"mode": "rollout", "n_particles": X.shape[0], "steps": steps, "dt": dt,
                      "sfs": None if sfs is None else f"ConstantSFS(Cs={sfs.Cs})",
                      "gradient_ms_fp32comp": ms_grad32, "fp32comp_gradient_vs_fp64_max_rel": g32_rel,
                      "loss_fp64": L0, "loss_fp32comp": L32, "forward_ms_fp64": ms_fwd,
                      "forward_ms_fp32comp": ms_fwd32, "gradient_ms_fp64": ms_grad,
                      "gradient_over_forward": ms_grad / ms_fwd,
                      "backward_over_forward": (ms_grad - ms_fwd) / ms_fwd,
                      "fd_directions": args.ro_dirs, "fd_h": h, "fd_max_rel_err": worst,
                      "fd_max_rel_err_by_h": worst_by_h,
                      "fd_richardson_max_rel_err": worst_rich if len(hs) >= 2 else None, "fd_checks": checks,
                      "note": "gradient = forward + backward with per-step checkpointing that keeps each step's "
                              "UJ values; central differences of the FP64 forward"}), flush=True)


def run_kernel_only_jet(args):
    """Profiling helper: `warmup` + `steps` near-field UJ (+Estr with --estr)
    calls -- or, with --jet-call dynamic, calls of the dynamic procedure's
    near-field differences (alpha = 0.999) -- on the jet cloud of --n particles
    at the density of the 2^20 case (the cylinder is shortened in proportion),
    nothing else."""
    import torch
    import vpm_gb300 as vpm
    from vpm_gb300 import workloads
    n = args.n
    X, G, s = workloads.jet_cloud(n, length=4.0 * n / (1 << 20))
    ctx = vpm.Context(0)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    S = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    prec = vpm.FP64 if args.precision == "fp64" else vpm.FP32COMP
    times, st = [], None
    if args.jet_call == "dynamic":
        ctx.p2p_leaflist_dev(x, g, sg, U, J, leaf_size=64, theta=0.4, kernel=KERNEL, precision=prec)
        dJ, dS = torch.zeros_like(J), torch.zeros_like(S)
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if args.jet_call == "dynamic":
            st = ctx.dynamic_diff_leaflist_dev(x, g, sg, J, 0.999, dJ, dS, leaf_size=64, theta=0.4, kernel=KERNEL,
                                               precision=prec)
        else:
            st = ctx.p2p_leaflist_dev(x, g, sg, U, J, S, leaf_size=64, theta=0.4, kernel=KERNEL, precision=prec,
                                      sfs=bool(args.estr))
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times) if times else float("nan")
    print(json.dumps({"mode": "kernel-only-jet", "call": args.jet_call, "n": n, "precision": args.precision,
                      "estr": bool(args.estr), "ms": ms, "leaves": st[0], "leaf_pairs": st[1], "pairs": st[2],
                      "pairs_per_s": st[2] / (ms / 1e3), "launches": ctx.launches}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    # profiling helpers (not the bench line): kernels alone on a smaller cloud
    ap.add_argument("--kernel-only", action="store_true")
    ap.add_argument("--n", type=int, default=1 << 16)
    ap.add_argument("--precision", default="fp32comp", choices=["fp64", "fp32comp"])
    ap.add_argument("--kernel", default="gaussianerf", choices=["singular", "gaussian", "gaussianerf", "winckelmans"])
    ap.add_argument("--estr", action="store_true")
    ap.add_argument("--cloud", default="random", choices=["random", "rings"],
                    help="--kernel-only: the random cloud or the leapfrogging rings of --n particles")
    ap.add_argument("--jet-call", default="uj", choices=["uj", "dynamic"])
    ap.add_argument("--adjoint", action="store_true")
    # the other workloads (one JSON line each, not the bench line)
    ap.add_argument("--workload", default="cloud", choices=["cloud", "leapfrog", "jet", "rollout"])
    ap.add_argument("--lf-n", type=int, default=200_000)
    ap.add_argument("--lf-steps", type=int, default=200)
    ap.add_argument("--lf-f64-steps", type=int, default=2)
    ap.add_argument("--lf-small", type=int, default=20_000)
    ap.add_argument("--jet-n", type=int, default=1 << 20)
    ap.add_argument("--jet-steps", type=int, default=3)
    ap.add_argument("--ro-steps", type=int, default=50)
    ap.add_argument("--ro-dirs", type=int, default=4)
    ap.add_argument("--ro-sfs", type=float, default=0.0, help="Cs of a ConstantSFS term in the rollout (0: none)")
    ap.add_argument("--ro-h", default="1e-6", help="central-difference steps of the rollout check, comma-separated")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.impl == "reference" else 1)))
    if args.kernel_only and args.workload == "jet":
        run_kernel_only_jet(args)
    elif args.workload == "leapfrog":
        run_leapfrog(args)
    elif args.workload == "jet":
        run_jet(args)
    elif args.workload == "rollout":
        run_rollout(args)
    elif args.kernel_only:
        run_kernel_only(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
