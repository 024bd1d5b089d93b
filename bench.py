#!/usr/bin/env python
"""TDVP steps/s on 3D N=343 Lennard-Jones bosons with 65,536 walkers.

Workload (one "step" = one RK4 TDVP time step = 4 stages, each: 2 Metropolis
sweeps per walker (686 single-particle moves), local energy + O_k + adjoint
dE_loc/d alpha per walker, walker reduction to <O>, S, force, FP64 Cholesky
solve and stage update):
  D=3, N=343 on a 7x7x7 simple-cubic start with 10% jitter, density 0.365
  (L = 9.7949), LJ eps = sigma = 1, hbar^2/2m = 0.09, 30 uniform knots on
  [0, L/2] (P = 30), McMillan-like initial Jastrow u(r) = -(1.1/r)^5 / 2
  (flat below 0.5 sigma), Gaussian moves of width 0.24 (~53% acceptance),
  dt = 5e-4, real time.
  Synthetic inputs (no dataset exists for this metric).  The walker array
  (270 MB in FP32) is larger than L2, so no flush is needed between steps.

Arms:
  default             mixed precision (FP32 pairs, FP64 centring/solve/RK4)
  --impl reference    the reference algorithm on the host cores: the FP64 CPU
                      port in oracle/ (the reference sources themselves are not
                      on the GPU host), bounded sample, extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, N, P, RHO = 3, 343, 30, 0.365
L = (N / RHO) ** (1.0 / DIM)
NW = 65536
DT = 5e-4
SWEEPS = 2
MOVES = SWEEPS * N
MC_STEP = 0.24
HBAR2_2M = 0.09
METRIC = "TDVP steps/s (3D N=343, 64k walkers): mixed+adjoint vs FP64 GPU, |ΔE/N|<1e-5"

# algorithmic FLOP convention (per pair evaluation; FMA = 2 FLOP)
FLOP_MOVE_PAIR = 32     # one Metropolis pair evaluation
FLOP_ELOC_PAIR = 110    # one unordered pair of the local-energy pass
FLOP_ADJ_PAIR = 90      # one unordered pair of the reverse (adjoint) sweep


def flop_sample_launch(nw=NW):
    return float(nw) * MOVES * 2 * (N - 1) * FLOP_MOVE_PAIR


def flop_eloc_launch(nw=NW, adjoint=True):
    pairs = float(nw) * N * (N - 1) / 2
    return pairs * (FLOP_ELOC_PAIR + (FLOP_ADJ_PAIR if adjoint else 0))


def flop_step(nw=NW):
    return 4 * (flop_sample_launch(nw) + flop_eloc_launch(nw))


def initial_params():
    """McMillan-like pair Jastrow u(r) = -(b/r)^5 / 2, b = 1.1 sigma, on the knot abscissae."""
    r = np.linspace(0.0, L / 2, P)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    return uR, np.zeros(P)


def initial_walkers(nw, seed=20261203):
    """7x7x7 simple-cubic lattice, jitter U(-1/2, 1/2) * spacing / 10 (TDVMC.cpp:725-739)."""
    m = 7
    l = L / m
    idx = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    R = idx[None, :, :] * l + (rng.uniform(size=(nw, N, DIM)) - 0.5) * l / 10.0 - L / 2
    return np.ascontiguousarray(np.transpose(R, (0, 2, 1)))


class Clocks:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "%s_traffic.txt" % kernel)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch_full_workload:"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


def cpu_port_rate(threads, walkers_per_thread=1, seed=11, mirrored=False):
    """The reference algorithm (FP64 CPU port) on a bounded sample: one stage
    (sampling pass + evaluation + adjoint) of threads*walkers_per_thread walkers.
    mirrored: the NUBosonsBulkPB workload (pb_system).
    Returns (steps/s extrapolated to the full workload, seconds, walkers)."""
    from oracle import oracle as orc
    if mirrored:
        s = orc.OracleSystem(DIM, N, P, L, user_knots=PB_KNOTS, pot_kind=orc.POT_SQUARE, pot=PB_SYSP,
                             hbar2_2m=HBAR2_2M, variant=orc.SYS_NU_PB)
    else:
        s = orc.OracleSystem(DIM, N, P, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0), hbar2_2m=HBAR2_2M)
    nws = threads * walkers_per_thread
    R = initial_walkers(nws, seed=seed)
    uR, uI = initial_params()
    t0 = time.perf_counter()
    s.stage(uR, uI, R, MOVES, MC_STEP, seed=1, pass_id=0, threads=threads, adjoint=True)
    t = time.perf_counter() - t0
    walker_stages_per_s = nws / t
    return walker_stages_per_s / (4.0 * NW), t, nws


def run_reference(args):
    threads = os.cpu_count() or 1
    rates = []
    t_probe = 2.0
    for _ in range(args.warmup):
        _, t_probe, _ = cpu_port_rate(threads, 2)
    # at least about 10 s of CPU work per measured step (one RK stage of wpt walkers per
    # thread); the probe's time per walker still carries part of a fixed start-up cost
    # (with one walker per thread the steps came out at about half the target), hence 15 s
    wpt = int(min(2048, max(1, np.ceil(15.0 / max(t_probe / 2.0, 1e-3)))))
    t_all = 0.0
    nws = 0
    for k in range(args.steps):
        r, t, nws = cpu_port_rate(threads, wpt, seed=100 + k)
        rates.append(r)
        t_all += t
    v = float(np.mean(rates))
    line = {"metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "3D N=343 LJ bosons rho=0.365, P=30, 65536 walkers, RK4 dt=5e-4, "
                                   "2 sweeps/stage, adjoint", "walkers": NW, "particles": N, "params": P},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": "per step: one RK stage (686 moves + E_loc + adjoint) of %d walkers "
                                       "on %d threads (%.1f s of CPU work per step on average), extrapolated "
                                       "x4 stages x65536 walkers" % (nws, threads, t_all / max(args.steps, 1))},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# batched trapped drops: 512 drops in 3D harmonic traps (omega = 1), Gaussian pair
# repulsion v0 = 1, sigma = 0.5, particle numbers drawn uniformly from {3, 6, 10, 20}
# (seed 4), a 12-knot pair spline plus a one-body Gaussian width each, 4,096 walkers
# per drop, units hbar = m = omega = 1 (hbar^2 / 2m = 0.5)
DROPS, DROP_WALKERS, DROP_P, DROP_RMAX = 512, 4096, 12, 4.0
DROP_NS = (3, 6, 10, 20)
DROP_DT, DROP_SWEEPS, DROP_STEP = 1e-3, 2, 0.6


def drops_workload(precision="mixed", walkers=DROP_WALKERS):
    import tdvmc_gb300 as T
    rng = np.random.default_rng(4)
    ns = rng.choice(DROP_NS, size=DROPS)
    d = T.TrappedDrops(ns, DROP_P, DROP_RMAX, walkers, omega=1.0, v0=1.0, sigma=0.5, hbar2_2m=0.5,
                       precision=precision)
    r = np.linspace(0.0, DROP_RMAX, DROP_P)
    uR = np.tile(np.concatenate([0.3 * np.exp(-r / 0.7), [-0.45]]), (DROPS, 1))
    d.SetParameters(uR, np.zeros_like(uR))
    wr = np.random.default_rng(5)
    d.SetWalkers([wr.normal(scale=0.7, size=(walkers, 3, n)) for n in ns])
    return d, ns


def run_drops(sync, steps, warmup, walkers=DROP_WALKERS):
    """The batched-drops workload: RK4 steps of all 512 drops, each stage one graph
    replay (prep, sample, evaluate + adjoint, per-drop reduce, per-drop solve), tiles
    chosen by the autotuner."""
    import tdvmc_gb300 as T
    d, ns = drops_workload(walkers=walkers)
    d.DoMetropolisSteps(10, DROP_STEP, seed=9, pass_id=0xFFFFFF00)  # thermalise
    tiles = d.Autotune(DROP_SWEEPS, DROP_STEP)
    td = T.DropsTDVP(d, DROP_DT, DROP_SWEEPS, DROP_STEP, seed=3, use_adjoint=1)
    td.time_steps(warmup)
    sync()
    l0 = d.LaunchCount()
    ms = td.time_steps(steps)
    launches = d.LaunchCount() - l0
    prof = td.profile_stage()
    out = td.step(1)
    e = out["energy"][:, 0]
    d.close()
    return {"value": steps / (ms / 1000.0), "unit": "steps/s", "drops": DROPS, "walkers_per_drop": walkers,
            "particles": {str(n): int((ns == n).sum()) for n in DROP_NS}, "spline_params": DROP_P,
            "dt": DROP_DT, "sweeps_per_stage": DROP_SWEEPS, "ms_per_step": ms / steps,
            "kernels_ms_per_stage": {k: v for k, v in prof}, "tiles": tiles,
            "gpu_launches_per_step": launches // steps, "status_ok": bool((out["status"] == 0).all()),
            "energy_per_particle_mean": float(np.mean(e / ns))}


# mirrored-distance system (NUBosonsBulkPB): the headline's bosons, walkers, moves and
# time step with every pair beyond r_max = L/2 entering at 2 r_max - r, the system's
# square well (a = sigma, b = 1) and its boundary fold; knots given (as the system
# requires) on the headline's uniform grid
PB_KNOTS = np.linspace(0.0, L / 2, P)
PB_SYSP = (1.0, 1.0)
PB_GATE_WALKERS = 8192


def run_pb(sync, steps, warmup, nw=NW, cpu=True):
    """RK4 steps/s of the mirrored-distance system in mixed precision, its kernels
    per stage, the |dE/N| gate against an FP64 evaluation of the same walkers, and
    the FP64 CPU port of the same system on the host cores."""
    import tdvmc_gb300 as T
    uR, uI = initial_params()
    s = T.NUBosonsBulkPB(DIM, N, P, L, nw, user_knots=PB_KNOTS, system_params=PB_SYSP, hbar2_2m=HBAR2_2M,
                         precision="mixed")
    s.SetParameters(uR, uI)
    s.SetWalkers(initial_walkers(nw))
    td = T.TDVP(s, DT, MOVES, MC_STEP, seed=1, use_adjoint=1)
    td.time_steps(warmup)
    sync()
    l0 = s.LaunchCount()
    ms = td.time_steps(steps)
    launches = s.LaunchCount() - l0
    prof = td.profile_stage()
    out = td.step(1)
    nsub = min(nw, PB_GATE_WALKERS)
    Rm = s.GetWalkers()[:nsub]
    fm = s.CalculateExpectationValues()
    gp = s.GetParameters()
    tiles = s.Tiles()
    s.close()
    s64 = T.NUBosonsBulkPB(DIM, N, P, L, nsub, user_knots=PB_KNOTS, system_params=PB_SYSP, hbar2_2m=HBAR2_2M,
                           precision="fp64")
    s64.SetParameters(*gp)
    s64.SetWalkers(Rm)
    f64 = s64.CalculateExpectationValues()
    s64.close()
    dE = abs(fm["eloc"][:nsub, 0].mean() - f64["eloc"][:, 0].mean()) / N
    res = {"value": steps / (ms / 1000.0), "unit": "steps/s", "walkers": nw, "ms_per_step": ms / steps,
           "kernels_ms_per_stage": {k: v for k, v in prof}, "gpu_launches_per_step": launches // steps,
           "tiles": tiles, "status": int(out["status"]), "accept_rate": out["accept_rate"],
           "gate": {"dE_per_N": dE, "pass": bool(dE < 1e-5), "walkers": nsub,
                    "against": "FP64 GPU evaluation of the same FP32-held walkers"},
           "workload": "NUBosonsBulkPB: 3D N=343 rho=0.365, P=30 knots on [0, L/2], square well a=1 b=1, "
                       "65536 walkers, RK4 dt=5e-4, 2 sweeps/stage, adjoint"}
    if cpu:
        threads = os.cpu_count() or 1
        _, t_probe, _ = cpu_port_rate(threads, 2, mirrored=True)
        wpt = int(min(1024, max(2, np.ceil(2 * 6.0 / max(t_probe, 1e-3)))))  # about 6 s of CPU work
        v, t, w = cpu_port_rate(threads, wpt, mirrored=True)
        res["cpu_port"] = {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                           "sample": "one RK stage of %d walkers on %d threads (%.1f s), extrapolated x4 stages "
                                     "x65536 walkers" % (w, threads, t)}
    return res


# large bulk: N = 1,000 on a 10x10x10 start, LJ at density 0.365, 64 knots,
# 262,144 walkers; imaginary-time preparation driven by the adjoint dE_loc/d alpha,
# then a density quench (0.365 -> 0.40, box and walkers rescaled, parameters kept
# per knot) and real-time RK4 steps dt = 2.5e-4, with an FP64 evaluation of the same
# walkers every 10 steps
C5_N, C5_P, C5_RHO, C5_RHO_Q, C5_NW = 1000, 64, 0.365, 0.40, 262144
C5_DT_IMAG, C5_DT = 1e-3, 2.5e-4
C5_STEP = 0.17
C5_CHECK_WALKERS = 8192


def c5_walkers(nw, L, seed=5):
    m = 10
    l = L / m
    idx = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    R = np.empty((nw, 3, C5_N))
    for w0 in range(0, nw, 8192):
        w1 = min(nw, w0 + 8192)
        x = idx[None] * l + (rng.uniform(size=(w1 - w0, C5_N, 3)) - 0.5) * l / 10.0 - L / 2
        R[w0:w1] = np.transpose(x, (0, 2, 1))
    return R


def c5_gate(sysm, L, nsub):
    """|dE/N| between the mixed evaluation and an FP64 evaluation of the same
    (FP32-held) walkers, first nsub walkers."""
    import tdvmc_gb300 as T
    Rm = sysm.GetWalkers()[:nsub]
    fm = sysm.CalculateExpectationValues()
    gp = sysm.GetParameters()
    s64 = T.BosonsBulk(3, C5_N, C5_P, L, nsub, system_params=(1.0, 1.0), potential="lj", hbar2_2m=HBAR2_2M,
                       precision="fp64")
    s64.SetParameters(*gp)
    s64.SetWalkers(Rm)
    f64 = s64.CalculateExpectationValues()
    s64.close()
    return abs(fm["eloc"][:nsub, 0].mean() - f64["eloc"][:, 0].mean()) / C5_N


def run_c5(sync, imag_steps, real_steps, timed_steps, check_every=10, nw=C5_NW, log=None):
    """Imaginary-time preparation (use_adjoint = 2), density quench, real-time RK4
    steps; returns the timed real-time steps/s and the FP64 gate at every check."""
    import tdvmc_gb300 as T
    L0 = (C5_N / C5_RHO) ** (1.0 / 3.0)
    L1 = (C5_N / C5_RHO_Q) ** (1.0 / 3.0)
    r = np.linspace(0.0, L0 / 2, C5_P)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    R = c5_walkers(nw, L0)
    s0 = T.BosonsBulk(3, C5_N, C5_P, L0, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=HBAR2_2M,
                      precision="mixed")
    s0.SetParameters(uR, np.zeros(C5_P))
    s0.SetWalkers(R)
    del R
    gates = []
    t0 = time.perf_counter()
    ti = T.TDVP(s0, C5_DT_IMAG, 2 * C5_N, C5_STEP, seed=5, imaginary_time=1, use_adjoint=2)
    e_imag = []
    sync()
    t_imag = time.perf_counter()
    for k in range(imag_steps):
        out = ti.step(1)
        e_imag.append(out["energy"][0] / C5_N)
        if log:
            log("imag step %d E/N %.6f acc %.3f status %d" % (k, e_imag[-1], out["accept_rate"], out["status"]))
    sync()
    t_imag = time.perf_counter() - t_imag
    gp = s0.GetParameters()
    Rq = s0.GetWalkers() * (L1 / L0)
    s0.close()
    s1 = T.BosonsBulk(3, C5_N, C5_P, L1, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=HBAR2_2M,
                      precision="mixed")
    s1.SetParameters(*gp)
    s1.SetWalkers(Rq)
    del Rq
    tr = T.TDVP(s1, C5_DT, 2 * C5_N, C5_STEP, seed=6, use_adjoint=1)
    e_real = []
    t_real, t_gate = time.perf_counter(), 0.0
    for k in range(real_steps - timed_steps):
        out = tr.step(1)
        e_real.append(out["energy"][0] / C5_N)
        if check_every and (k + 1) % check_every == 0:
            t_g = time.perf_counter()
            g = c5_gate(s1, L1, min(C5_CHECK_WALKERS, nw))
            t_gate += time.perf_counter() - t_g
            gates.append({"step": k + 1, "dE_per_N": g})
            if log:
                log("real step %d E/N %.6f acc %.3f status %d gate %.2e"
                    % (k + 1, e_real[-1], out["accept_rate"], out["status"], g))
    sync()
    t_real = time.perf_counter() - t_real - t_gate
    ms_timed = None
    if timed_steps > 0:
        sync()
        ms_timed = tr.time_steps(timed_steps)  # CUDA events on the library's stream
    res = {"imag_steps": imag_steps, "real_steps": real_steps, "walkers": nw, "particles": C5_N, "params": C5_P,
           "rho": [C5_RHO, C5_RHO_Q], "dt_imag": C5_DT_IMAG, "dt": C5_DT, "moves_per_stage": 2 * C5_N,
           "energy_per_particle_imag": e_imag[-3:], "energy_per_particle_real": e_real[-3:],
           "gates": gates, "gate_pass": bool(all(g["dE_per_N"] < 1e-5 for g in gates)),
           "gate_walkers": min(C5_CHECK_WALKERS, nw),
           "imag_steps_per_s_wall": imag_steps / t_imag if imag_steps else None,
           "real_steps_per_s_wall": (real_steps - timed_steps) / t_real if real_steps > timed_steps else None,
           "wall_s": time.perf_counter() - t0}
    if ms_timed is not None:
        res["value"] = timed_steps / (ms_timed / 1000.0)
        res["unit"] = "steps/s"
        res["ms_per_step"] = ms_timed / timed_steps
        res["gate_after_timed"] = c5_gate(s1, L1, min(C5_CHECK_WALKERS, nw))
        res["kernels_ms_per_stage"] = {k: v for k, v in tr.profile_stage()}
        res["tiles"] = s1.Tiles()
    s1.close()
    return res


class Ranks:
    """Replica ranks under torchrun (one process per GPU, each running the whole
    workload): a barrier and the maximum over ranks; no-ops for one rank."""

    def __init__(self, world, backend="nccl"):
        self.dist = None
        self.device = "cuda" if backend == "nccl" else "cpu"
        if world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x):
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


def run_ours(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    try:
        import torch
        torch.cuda.set_device(local)
        sync = torch.cuda.synchronize
    except Exception:
        torch = None

        def sync():
            pass
    ranks = Ranks(world, "nccl")
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as Nat

    lib = Nat.load()
    uR, uI = initial_params()
    nw = args.walkers
    R0 = initial_walkers(nw)
    sysm = T.BosonsBulk(DIM, N, P, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=HBAR2_2M,
                        precision="mixed")
    sysm.SetParameters(uR, uI)
    sysm.SetWalkers(R0)
    if args.stored and args.no_extras:
        # profiling runs of the stored-sample path: RK4 (3) or the predictor-corrector (5)
        # on stored samples, a rotating quarter of the walkers resampled per step
        td = T.TDVP(sysm, DT, MOVES, MC_STEP, seed=1, use_adjoint=1, ode_solver=3 if args.stored == "rk4" else 5,
                    update_every=1, update_percent=25.0)
    else:
        td = T.TDVP(sysm, DT, MOVES, MC_STEP, seed=1, use_adjoint=1)
    if args.autotune:
        sysm.Autotune(MOVES, MC_STEP)
    launches0 = sysm.LaunchCount()
    # warm-up steps (thermalise the walkers, build and warm the graphs)
    td.time_steps(args.warmup)
    sync()
    ranks.barrier()
    sync()
    clocks = Clocks()
    clocks.start()
    launches_a = sysm.LaunchCount()
    ms = td.time_steps(args.steps)  # CUDA events on the library's stream around the K steps
    sync()
    ranks.barrier()
    sync()
    launches_b = sysm.LaunchCount()
    clk = clocks.stop()
    ms = ranks.max(ms)
    if args.no_extras:
        # profiling runs: the timed steps only
        if rank == 0:
            print(json.dumps({"walkers": nw, "steps": args.steps, "ms_per_step": ms / args.steps}))
        return

    # per-kernel device times of one eager stage (CUDA events around each kernel)
    prof = td.profile_stage()
    kt = {k: v for k, v in prof}
    top = max(prof, key=lambda kv: kv[1])

    # end-to-end through the C ABI with host buffers: parameters in, statistics
    # and parameters out, every step
    uRh, uIh, pRh, pIh = sysm.GetParameters()
    sync()
    ranks.barrier()
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        sysm.SetParameters(uRh, uIh, pRh, pIh)
        last = td.step(1)
        uRh, uIh, pRh, pIh = sysm.GetParameters()
    sync()
    e2e_s = ranks.max(time.perf_counter() - t0)
    e2e = args.steps / e2e_s
    h2d = (2 * P + 2) * 8 * 2 + 4
    d2h = (3 * P + 12) * 8 + 24 + (2 * P + 2) * 8

    # |dE/N| gate: FP64 evaluation of all the walkers the mixed path holds (its FP32
    # coordinates) against the mixed evaluation
    Rm = sysm.GetWalkers()
    fm = sysm.CalculateExpectationValues()
    gp = sysm.GetParameters()
    s64 = T.BosonsBulk(DIM, N, P, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=HBAR2_2M,
                       precision="fp64")
    s64.SetParameters(gp[0], gp[1], gp[2], gp[3])
    s64.SetWalkers(Rm)
    f64 = s64.CalculateExpectationValues()
    dE_per_N = abs(fm["eloc"][:, 0].mean() - f64["eloc"][:, 0].mean()) / N
    del Rm

    # plain FP64 GPU path, same kernels in double, at the full walker count
    s64.SetWalkers(R0)
    s64.SetParameters(uR, uI)
    td64 = T.TDVP(s64, DT, MOVES, MC_STEP, seed=1, use_adjoint=1)
    td64.time_steps(1)
    ms64 = td64.time_steps(1)
    fp64_steps_s = 1000.0 / ms64
    s64.close()

    # RK4 on stored samples (ODE_SOLVER_TYPE 3, correlated-sampling reuse): the
    # first stage of every step resamples a rotating quarter of the walkers, the
    # other three stages re-evaluate the stored samples
    td3 = T.TDVP(sysm, DT, MOVES, MC_STEP, seed=1, use_adjoint=1, ode_solver=3, update_every=1,
                 update_percent=25.0)
    td3.time_steps(2)  # stores every walker, then one refresh step
    ms3 = td3.time_steps(args.steps)
    prof3 = {k: v for k, v in td3.profile_stage()}
    # predictor-corrector on stored samples (ODE_SOLVER_TYPE 5): Euler predictor and
    # 6 corrector passes, each re-evaluating the stored samples
    td5 = T.TDVP(sysm, DT, MOVES, MC_STEP, seed=1, use_adjoint=1, ode_solver=5, update_every=1,
                 update_percent=25.0)
    td5.time_steps(1)
    ms5 = td5.time_steps(args.steps)

    # batched trapped drops (512 drops of 3-20 particles, 4,096 walkers each)
    drops = run_drops(sync, args.steps, args.warmup) if args.extras_drops else None
    # large bulk (N = 1,000, 262,144 walkers): one imaginary-time step driven by the
    # adjoint, the density quench, one real-time step, then two timed real-time steps
    c5 = run_c5(sync, 1, 3, 2, check_every=0) if args.extras_c5 else None
    # the mirrored-distance system (NUBosonsBulkPB) on the headline's shape
    pb = run_pb(sync, args.steps, args.warmup, cpu=(world == 1)) if args.extras_pb else None
    if c5:
        c5["workload"] = ("3D N=1000 LJ bosons rho=0.365 -> 0.40 quench, P=64, 262144 walkers, "
                          "RK4 dt=2.5e-4, 2 sweeps/stage")

    # FP32 pipe ceiling and roofline of the dominant kernel
    import ctypes as C
    pk = C.c_double()
    Nat.check(lib.tdvmc_measure_fp32_peak(C.byref(pk)), "tdvmc_measure_fp32_peak")
    fp32_peak = pk.value
    if top[0] == "k_sample":
        fl = flop_sample_launch()
    elif top[0] == "k_eloc_rev":
        fl = float(NW) * N * (N - 1) / 2 * FLOP_ADJ_PAIR
    elif top[0].startswith("k_eloc"):
        fl = flop_eloc_launch(adjoint=False)  # the forward kernel; the adjoint pass is k_eloc_rev
    else:
        fl = 0.0
    achieved = fl / (top[1] * 1e-3) / 1e12
    traffic = ncu_traffic(top[0])

    # CPU baseline: the reference algorithm (FP64 port) on the host cores, bounded
    # sample; one GPU only (replica ranks would share the host's cores)
    threads = os.cpu_count() or 1
    cpu_baseline = None
    if world == 1:
        _, t_probe, _ = cpu_port_rate(threads, 4)
        wpt = int(min(1024, max(4, np.ceil(4 * 12.0 / max(t_probe, 1e-3)))))  # about 12 s of CPU work
        cpu_v, cpu_t, cpu_w = cpu_port_rate(threads, wpt)
        cpu_baseline = {"value": cpu_v, "unit": "steps/s", "cores": threads, "kind": "port",
                        "sample": "one RK stage (686 moves + E_loc + adjoint) of %d walkers on %d threads "
                                  "(%.1f s), extrapolated x4 stages x65536 walkers" % (cpu_w, threads, cpu_t)}

    value = world * args.steps / (ms / 1000.0)
    peaks = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "3D N=343 LJ bosons rho=0.365, P=30, 65536 walkers, RK4 dt=5e-4, 2 sweeps/stage, "
                               "adjoint", "walkers": NW, "particles": N, "params": P, "moves_per_stage": MOVES,
                   "mc_step": MC_STEP, "l2": "inputs larger than L2 (walkers 270 MB)",
                   "parallelism": "single GPU" if world == 1 else "replicas"},
        "e2e": {"value": e2e * world, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches_b - launches_a),
        "roofline": {"bound": "fp32", "kernel": top[0], "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak if fp32_peak else None,
                     "peak_source": "measured FP32 FMA loop (tdvmc_measure_fp32_peak)",
                     "traffic": traffic, "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "kernels_ms_per_stage": kt,
        "fp64_gpu": {"value": fp64_steps_s, "unit": "steps/s", "walkers_timed": nw, "steps_timed": 1,
                     "speedup_mixed_over_fp64": value / world / fp64_steps_s},
        "gate": {"dE_per_N": dE_per_N, "pass": bool(dE_per_N < 1e-5), "walkers": nw,
                 "against": "FP64 GPU evaluation of the same FP32-held walkers"},
        "batched_drops": drops,
        "large_bulk": c5,
        "mirrored_distance": pb,
        "stored_sample_rk4": {"value": args.steps / (ms3 / 1000.0), "unit": "steps/s", "update_every": 1,
                              "update_percent": 25.0, "kernels_ms_refresh_stage": prof3},
        "stored_sample_pc": {"value": args.steps / (ms5 / 1000.0), "unit": "steps/s", "update_every": 1,
                             "update_percent": 25.0, "correctors": 6},
        "cpu_baseline": cpu_baseline,
        "algorithmic_tflop_per_step": flop_step() / 1e12,
        "achieved_tflops_step": flop_step() / (ms / args.steps * 1e-3) / 1e12,
        "clocks": clk,
        "energy_per_particle": float(fm["eloc"][:, 0].mean() / N),
        "accept_rate": last["accept_rate"] if last else None,
        "tiles": sysm.Tiles(),
    }
    if rank == 0:
        print(json.dumps(line))


def run_workload(args):
    """One of the other workloads alone, one JSON line (not the headline metric)."""
    import torch
    torch.cuda.set_device(0)
    sync = torch.cuda.synchronize
    if args.workload == "pb":
        out = run_pb(sync, args.steps, args.warmup, nw=args.walkers)
    elif args.workload == "drops":
        out = run_drops(sync, args.steps, args.warmup, walkers=args.drop_walkers)
        out["workload"] = ("512 trapped 3D drops, N in {3,6,10,20}, 12-knot spline + one-body width, "
                           "4096 walkers/drop, RK4 dt=1e-3, 2 sweeps/stage, adjoint, autotuned tiles")
    else:
        def log(msg):
            print(msg, file=sys.stderr, flush=True)
        if args.walkers != NW:
            # a short run at another walker count (profiler runs): one imaginary-time and one
            # real-time step, no FP64 checks
            out = run_c5(sync, 1, 1, 0, check_every=0, nw=args.walkers, log=log)
        else:
            out = run_c5(sync, 50, 200, 10, check_every=10, log=log)
        out["workload"] = ("3D N=1000 LJ bosons rho=0.365, P=64, %d walkers: %d imaginary-time steps "
                           "(adjoint force), quench to rho=0.40, %d real-time RK4 steps dt=2.5e-4"
                           % (out["walkers"], out["imag_steps"], out["real_steps"]))
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--autotune", type=int, default=0)
    ap.add_argument("--walkers", type=int, default=NW,
                    help="walkers (default: the 65,536 of the workload; with --workload c5 another count runs "
                         "one imaginary-time and one real-time step, for profiler runs)")
    ap.add_argument("--no-extras", action="store_true",
                    help="time the steps only (no e2e, FP64, CPU or gate legs): for profiler runs on a small case")
    ap.add_argument("--stored", choices=["rk4", "pc"], default=None,
                    help="with --no-extras: time steps on stored samples (RK4 or the predictor-corrector)")
    ap.add_argument("--extras-drops", type=int, default=1, help="time the batched-drops workload as an extra")
    ap.add_argument("--extras-c5", type=int, default=1, help="time the large-bulk workload as an extra")
    ap.add_argument("--extras-pb", type=int, default=1,
                    help="time the mirrored-distance system (NUBosonsBulkPB) on the headline shape as an extra")
    ap.add_argument("--drop-walkers", type=int, default=DROP_WALKERS,
                    help="with --workload drops: walkers per drop (smaller for profiler runs)")
    ap.add_argument("--workload", choices=["bulk", "drops", "c5", "pb"], default="bulk",
                    help="drops: the batched-drops workload alone; c5: the full large-bulk run (50 imaginary-"
                         "time steps, quench, 200 real-time steps, FP64 check every 10 steps)")
    args = ap.parse_args()
    if args.workload != "bulk":
        run_workload(args)
        return
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
