"""GPU: the workloads as stated, against the FP64 oracle.

  1D bulk (N = 20, L = 20, Gaussian soft core 2 exp(-r^2 / (2 0.5^2)) quenched to
      4 exp(...), 10 uniform knots, coefficients N(0, 0.01), 1,000 walkers, 200
      sweeps per step): one RK4 step at dt = 1e-3 after the quench; FP64 against
      the oracle running the same Philox stream, parameters relative 1e-9 and
      walkers 1e-9; the mixed path's step against the FP64 step to a quarter of
      the parameter increment (different chains).  The step size is tuned by
      bisection toward 50 % acceptance; with coefficients of 0.01 the wave
      function is nearly flat, so the acceptance stays above 90 % for any step up
      to the box length, and the tuner ends at the largest step it tries (L / 2).
  3D benchmark system (N = 343, LJ at density 0.365, 30 knots): the mixed
      chain's sampled averages of E^R, E^I and O_k against the FP64 oracle's own
      chain (Philox, 128 walkers) within 3 sigma (E) and 4 sigma (each O_k),
      sigma from the scatter over independent walkers.
  Autotuner on the benchmark system at 16,384 walkers: the walkers are left
      bit-identical, and the tiles it picks give the same evaluation as the
      default tiles at the mixed tolerance (1e-5).
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def c1_setup(precision, step=None):
    import tdvmc_gb300 as T
    n, p, L, nw = 20, 10, 20.0, 1000
    rng = np.random.default_rng(101)
    uR = rng.normal(0.0, 0.01, size=p)
    uI = rng.normal(0.0, 0.01, size=p)
    sysp = (0.5, 2.0, 0.0, 0.5, 4.0)  # b = 2 -> 4 at t >= 0: the quench is active
    R0 = rng.uniform(-L / 2, L / 2, size=(nw, 1, n))
    s = T.BosonsBulk(1, n, p, L, nw, system_params=sysp, potential="gauss", hbar2_2m=1.0, precision=precision)
    s.SetTime(0.0)
    s.SetParameters(uR, uI)
    s.SetWalkers(R0)
    return s, uR, uI, R0, sysp


def tune_step(s, n, lo=0.05, hi=10.0):
    """Bisection of the Gaussian move width for 50 % acceptance (one sweep per trial;
    the walkers are restored)."""
    R = s.GetWalkers()
    for k in range(30):
        mid = np.sqrt(lo * hi)
        acc = s.DoMetropolisSteps(n, mid, seed=999, pass_id=1000 + k) / (n * s.nw)
        s.SetWalkers(R)
        if acc > 0.5:
            lo = mid
        else:
            hi = mid
    return np.sqrt(lo * hi)


def test_c1_quench_rk4_step_matches_oracle():
    import tdvmc_gb300 as T
    n, p, L, dt, seed, pass0 = 20, 10, 20.0, 1e-3, 17, 5
    s, uR, uI, R0, sysp = c1_setup("fp64")
    step = tune_step(s, n)
    acc = s.DoMetropolisSteps(n, step, seed=999, pass_id=2000) / (n * s.nw)
    s.SetWalkers(R0)
    # 50 % where it can be reached; else the largest step tried, at high acceptance
    assert abs(acc - 0.5) < 0.03 or (step > 0.99 * 10.0 and acc > 0.5), (step, acc)
    moves = 200 * n
    s.DoMetropolisSteps(0, step, seed, pass0)  # sets the Philox pass counter
    td = T.TDVP(s, dt, moves, step, seed=seed)
    out = td.step()
    assert out["status"] == 0
    gR, gI, gpR, gpI = s.GetParameters()
    o = orc.OracleSystem(1, n, p, L, pot_kind=orc.POT_GAUSS, pot=sysp, time=0.0, hbar2_2m=1.0)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    cur, Ro, ks = base.copy(), R0.copy(), []
    for k in range(4):
        st = o.stage(cur[:p], cur[p:2 * p], Ro, moves, step, seed, pass0 + k, threads=8, adjoint=False)
        m = orc.centred(st["O"], st["eloc"])
        dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"])
        kv = np.concatenate([dR, dI, [pR, pI]])
        ks.append(kv)
        if k < 3:
            cur = base + kv * (dt / 2 if k < 2 else dt)
    new = orc.rk4_combine(base, ks, dt)
    assert np.abs(s.GetWalkers() - Ro).max() < 1e-9
    got = np.concatenate([gR, gI, [gpR, gpI]])
    assert relmax(got, new) < 1e-9
    # the mixed path walks its own chain: the step's increment agrees statistically
    sm, *_ = c1_setup("mixed")
    sm.DoMetropolisSteps(0, step, seed, pass0)
    T.TDVP(sm, dt, moves, step, seed=seed).step()
    mR, mI, _, _ = sm.GetParameters()
    inc64 = np.concatenate([gR - uR, gI - uI])
    incm = np.concatenate([mR - uR, mI - uI])
    assert np.abs(incm - inc64).max() < 0.25 * np.abs(inc64).max(), (incm, inc64)


def test_benchmark_system_sampled_averages_match_oracle_chain():
    import tdvmc_gb300 as T
    import bench as B
    n, p, L = B.N, B.P, B.L
    uR, uI = B.initial_params()
    uI = 0.02 * np.random.default_rng(3).normal(size=p)
    step, therm, nsamp = B.MC_STEP, 10 * n, 8
    # FP64 oracle chain: 128 walkers from the lattice start, Philox stream
    nwo = 128
    o = orc.OracleSystem(3, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0), hbar2_2m=B.HBAR2_2M)
    Ro = B.initial_walkers(nwo, seed=77)
    o.stage(uR, uI, Ro, therm, step, 11, 0, threads=16, adjoint=False)  # thermalisation
    rows = []
    for k in range(nsamp):
        st = o.stage(uR, uI, Ro, 2 * n, step, 11, k + 1, threads=16, adjoint=False)
        rows.append(np.concatenate([st["eloc"], st["O"]], axis=1))
    per_o = np.array(rows).mean(0)
    # mixed GPU chain: 4,096 walkers, its own stream
    nw = 4096
    s = T.BosonsBulk(3, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=B.HBAR2_2M,
                     precision="mixed")
    s.SetParameters(uR, uI)
    s.SetWalkers(B.initial_walkers(nw, seed=78))
    s.DoMetropolisSteps(therm, step, seed=12, pass_id=0)
    rows = []
    for k in range(nsamp):
        s.DoMetropolisSteps(2 * n, step, seed=12, pass_id=k + 1)
        f = s.CalculateExpectationValues()
        rows.append(np.concatenate([f["eloc"], f["O"]], axis=1))
    per_g = np.array(rows).mean(0)
    mo, mg = per_o.mean(0), per_g.mean(0)
    eo = per_o.std(0, ddof=1) / np.sqrt(nwo)
    eg = per_g.std(0, ddof=1) / np.sqrt(nw)
    comb = np.sqrt(eo ** 2 + eg ** 2)
    dev = np.abs(mo - mg) / np.where(comb > 0, comb, 1.0)
    assert np.all(np.abs(mo - mg)[comb == 0] < 1e-9)
    assert dev[0] < 3 and dev[1] < 3, dev[:2]
    assert np.all(dev[2:] < 4), dev


def test_autotune_keeps_walkers_and_results():
    import tdvmc_gb300 as T
    import bench as B
    nw = 16384
    s = T.BosonsBulk(3, B.N, B.P, B.L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=B.HBAR2_2M,
                     precision="mixed")
    uR, uI = B.initial_params()
    s.SetParameters(uR, uI)
    R0 = B.initial_walkers(nw)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(2 * B.N, B.MC_STEP, seed=1, pass_id=0)
    before = s.GetWalkers()
    ref = s.CalculateExpectationValues()
    dref = s.CalculateLocalEnergyAdjoint()
    tiles = s.Autotune(2 * B.N, B.MC_STEP)
    assert tiles["sample_lanes"] in (8, 16, 32) and tiles["eval_lanes"] in (8, 16, 32)
    assert np.array_equal(s.GetWalkers(), before)
    got = s.CalculateExpectationValues()
    dgot = s.CalculateLocalEnergyAdjoint()
    for key in ("O", "eloc", "other"):
        assert relmax(got[key], ref[key]) < 1e-5, key
    assert relmax(dgot, dref) < 1e-5
    # a step with the tuned tiles runs
    out = T.TDVP(s, B.DT, 2 * B.N, B.MC_STEP, seed=2, use_adjoint=1).step(1)
    assert out["status"] == 0
