"""GPU: correlated-sampling reuse (stored samples, ODE_SOLVER_TYPE 3 and 5).

Tolerances (stated per test):
  RK4 / predictor-corrector on stored samples, mixed vs FP64 with fixed walkers:
      parameter increments 2e-4 of their largest magnitude;
  stored vs direct evaluation at the same walkers and parameters: FP64
      relative 1e-11, mixed 1e-5 on ln psi, O_k, E_loc, the kinetic sums and
      dE/d alpha (scaled by the largest magnitude of each quantity);
  RK4 on stored samples vs the FP64 oracle (sampling at the first stage,
      evaluation of the fixed samples at the three others, a rotating
      refresh window on later steps): parameters relative 1e-9, walkers 1e-9;
  the predictor-corrector on stored samples likewise (1e-9).
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def soa(cfgs):
    return np.ascontiguousarray(np.transpose(np.asarray(cfgs), (0, 2, 1)))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
@pytest.mark.parametrize("golden,pot", [("eval_d3_n343_p30", "square"), ("eval_d2_n64_k20", "lj"),
                                        ("eval_d1_n20_p10", "gauss")])
def test_stored_eval_matches_direct_eval(precision, tol, golden, pot):
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, golden + ".npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    kn = z["knots"] if z["knots"].size else None
    sysp = {"square": z["sysp"], "lj": (1.0, 1.0), "gauss": (0.5, 2.0)}[pot]
    cfgs = soa(z["cfgs"])
    nw = 4 * len(cfgs)
    rng = np.random.default_rng(3)
    R = np.concatenate([cfgs] * 4) + rng.normal(0, 0.01, size=(nw, dim, n))
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=sysp, potential=pot, user_knots=kn, hbar2_2m=0.09,
                     precision=precision)
    s.SetTime(float(z["time"]))
    uR, uI = np.asarray(z["uR"]), np.asarray(z["uI"])
    s.SetParameters(uR, uI)
    s.SetWalkers(R)
    s.FillCorrelatedSamplingData()
    for k, (a, b) in enumerate([(uR, uI), (1.1 * uR + 0.01, 0.5 * uI - 0.02)]):
        s.SetParameters(a, b)
        got = s.CalculateExpectationValuesForStoredSamples(adjoint=True)
        ref = s.CalculateExpectationValues()
        ref["dE"] = s.CalculateLocalEnergyAdjoint()
        for key in ("lnpsi", "O", "eloc", "other", "dE"):
            assert relmax(got[key], ref[key]) < tol, (k, key, relmax(got[key], ref[key]))


def test_stored_eval_n1000_tracks_direct():
    """The large bulk system: N = 1000 on a jittered 10x10x10 start at density
    0.365, LJ, 64 knots (66 splines).  The stored evaluation (larger store tiles,
    16-byte loads over particles) equals the direct one to 1e-11 in FP64; in
    mixed precision, on FP32-representable coordinates, the direct and the
    stored evaluations both match the FP64 evaluation to 1e-5 relative on ln psi,
    O_k, E_loc, the kinetic sums and dE/d alpha."""
    import tdvmc_gb300 as T
    dim, n, p, nw = 3, 1000, 64, 32
    L = (n / 0.365) ** (1.0 / 3.0)
    rng = np.random.default_rng(5)
    m = 10
    idx = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    R = idx[None] * (L / m) + (rng.uniform(size=(nw, n, 3)) - 0.5) * (L / m) * 0.3 - L / 2
    R = np.ascontiguousarray(np.transpose(R, (0, 2, 1))).astype(np.float32).astype(np.float64)
    r = np.linspace(0.0, L / 2, p)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    uI = 0.01 * rng.normal(size=p)
    out = {}
    for prec in ("fp64", "mixed"):
        s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09,
                         precision=prec)
        s.SetParameters(uR, uI)
        s.SetWalkers(R)
        s.FillCorrelatedSamplingData()
        got = s.CalculateExpectationValuesForStoredSamples(adjoint=True)
        ref = s.CalculateExpectationValues()
        ref["dE"] = s.CalculateLocalEnergyAdjoint()
        out[prec] = (got, ref)
        s.close()
    truth = out["fp64"][1]
    for key in ("lnpsi", "O", "eloc", "other", "dE"):
        assert relmax(out["fp64"][0][key], truth[key]) < 1e-11, key
        assert relmax(out["mixed"][0][key], truth[key]) < 1e-5, (key, relmax(out["mixed"][0][key], truth[key]))
        assert relmax(out["mixed"][1][key], truth[key]) < 1e-5, (key, relmax(out["mixed"][1][key], truth[key]))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_stored_eval_more_than_32_splines(precision, tol):
    """P = 40 (42 splines, more than the FP32 evaluation keeps as register sums):
    the stored evaluation with 16-byte loads over particles, N = 45 (two
    32-particle chunks, the second mostly padding), equal-width knots.  FP64:
    stored equals direct at 1e-11.  Mixed, on FP32-representable walkers: the
    stored and the direct evaluation each match the FP64 evaluation at 1e-5."""
    import tdvmc_gb300 as T
    dim, n, p, L = 3, 45, 40, 4.2
    nw = 96
    rng = np.random.default_rng(5)
    R = rng.uniform(0.0, L, size=(nw, dim, n)).astype(np.float32).astype(np.float64)
    uR = -0.3 * np.exp(-np.linspace(0.0, 3.0, p)) + 0.01 * rng.normal(size=p)
    uI = 0.02 * rng.normal(size=p)
    pars = [(uR, uI), (1.2 * uR - 0.01, 0.7 * uI + 0.01)]
    out = {}
    for prec in sorted({precision, "fp64"}):
        s = T.BosonsBulk(dim, n, p, L, nw, system_params=(0.5, 2.0), potential="gauss", hbar2_2m=0.09,
                         precision=prec)
        s.SetParameters(uR, uI)
        s.SetWalkers(R)
        s.FillCorrelatedSamplingData()
        out[prec] = []
        for a, b in pars:
            s.SetParameters(a, b)
            got = s.CalculateExpectationValuesForStoredSamples(adjoint=True)
            ref = s.CalculateExpectationValues()
            ref["dE"] = s.CalculateLocalEnergyAdjoint()
            out[prec].append((got, ref))
        s.close()
    for k in range(len(pars)):
        got, ref = out[precision][k]
        truth = out["fp64"][k][1]
        for key in ("lnpsi", "O", "eloc", "other", "dE"):
            if precision == "fp64":
                assert relmax(got[key], ref[key]) < tol, (k, key, relmax(got[key], ref[key]))
            else:
                assert relmax(got[key], truth[key]) < tol, (k, key, relmax(got[key], truth[key]))
                assert relmax(ref[key], truth[key]) < tol, (k, key, relmax(ref[key], truth[key]))


def test_stored_sample_rk4_matches_oracle_fp64():
    """Three RK4 steps on stored samples: the first samples every walker, the
    next two refresh windows [0, nw/4) and [nw/4, nw/2) (UpdateSamplesConsecutive)."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw, moves, step, dt, seed, pass0 = 64, 2 * n, 0.35, 1e-3, 21, 5
    q = nw // 4
    rng = np.random.default_rng(19)
    R0 = np.repeat(z["R0"].T[None], nw, axis=0) + rng.normal(0, 0.05, size=(nw, dim, n))
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    uR, uI = np.asarray(z["uR"]), np.asarray(z["uI"])
    sysp = tuple(z["sysp"])  # the square well the fixture was sampled with
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=sysp, potential="square", hbar2_2m=0.09, precision="fp64")
    s.SetParameters(uR, uI, 0.0, 0.0)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(0, step, seed, pass0)  # sets the Philox pass counter
    td = T.TDVP(s, dt, moves, step, seed=seed, ode_solver=3, update_every=1, update_percent=25.0)

    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_SQUARE, pot=sysp, hbar2_2m=0.09)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    Ro = R0.copy()
    windows = [(0, nw), (0, q), (q, 2 * q)]
    for st, (w0, w1) in enumerate(windows):
        before = s.GetWalkers()
        td.step()
        after = s.GetWalkers()
        moved = np.any(np.abs(after - before).reshape(nw, -1) > 0, axis=1)
        assert not moved[:w0].any() and not moved[w1:].any()
        pass_id = pass0 + 4 * st
        o.sample(base[:p], Ro, moves, step, seed, pass_id, w0=w0, nw=w1 - w0) if st else \
            o.sample(base[:p], Ro, moves, step, seed, pass_id)
        cur = base.copy()
        ks = []
        for k in range(4):
            out = o.stage(cur[:p], cur[p:2 * p], Ro, 0, step, seed, 0, threads=4, adjoint=False)
            m = orc.centred(out["O"], out["eloc"])
            dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"])
            kv = np.concatenate([dR, dI, [pR, pI]])
            ks.append(kv)
            if k < 3:
                cur = base + kv * (dt / 2 if k < 2 else dt)
        base = orc.rk4_combine(base, ks, dt)
        assert np.all(np.isfinite(base))
        assert np.abs(after - Ro).max() < 1e-9, st
        gR, gI, gpR, gpI = s.GetParameters()
        assert relmax(np.concatenate([gR, gI, [gpR, gpI]]), base) < 1e-9, st


def test_stored_sample_pc_matches_oracle_fp64():
    """Three predictor-corrector steps on stored samples (ODE_SOLVER_TYPE 5,
    CalculateNextParametersPCReuseSamples, TDVMC.cpp:1912-1967): Euler predictor,
    then 6 passes u <- u + (u'(u) + u'(trial)) dt / 2, every pass evaluating the
    stored samples; the first step samples every walker, the next two refresh
    windows [0, nw/4) and [nw/4, nw/2).  Parameters and walkers to 1e-9."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw, moves, step, dt, seed, pass0 = 64, 2 * n, 0.35, 1e-3, 23, 5
    q = nw // 4
    rng = np.random.default_rng(29)
    R0 = np.repeat(z["R0"].T[None], nw, axis=0) + rng.normal(0, 0.05, size=(nw, dim, n))
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    uR, uI = np.asarray(z["uR"]), np.asarray(z["uI"])
    sysp = tuple(z["sysp"])
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=sysp, potential="square", hbar2_2m=0.09, precision="fp64")
    s.SetParameters(uR, uI, 0.0, 0.0)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(0, step, seed, pass0)  # sets the Philox pass counter
    td = T.TDVP(s, dt, moves, step, seed=seed, ode_solver=5, update_every=1, update_percent=25.0)

    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_SQUARE, pot=sysp, hbar2_2m=0.09)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    Ro = R0.copy()

    def rhs(cur):
        out = o.stage(cur[:p], cur[p:2 * p], Ro, 0, step, seed, 0, threads=4, adjoint=False)
        m = orc.centred(out["O"], out["eloc"])
        dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"])
        return np.concatenate([dR, dI, [pR, pI]])

    windows = [(0, nw), (0, q), (q, 2 * q)]
    for st, (w0, w1) in enumerate(windows):
        before = s.GetWalkers()
        td.step()
        after = s.GetWalkers()
        moved = np.any(np.abs(after - before).reshape(nw, -1) > 0, axis=1)
        assert not moved[:w0].any() and not moved[w1:].any()
        pass_id = pass0 + 7 * st  # one pass per stage: predictor and 6 correctors
        o.sample(base[:p], Ro, moves, step, seed, pass_id, w0=w0, nw=w1 - w0) if st else \
            o.sample(base[:p], Ro, moves, step, seed, pass_id)
        k0 = rhs(base)
        trial = base + k0 * dt
        for _ in range(6):
            trial = base + (k0 + rhs(trial)) * (dt / 2)
        base = trial
        assert np.all(np.isfinite(base))
        assert np.abs(after - Ro).max() < 1e-9, st
        gR, gI, gpR, gpI = s.GetParameters()
        assert relmax(np.concatenate([gR, gI, [gpR, gpI]]), base) < 1e-9, st


@pytest.mark.parametrize("ode", [3, 5])
def test_stored_sample_steps_mixed_track_fp64(ode):
    """RK4 (3) and the predictor-corrector (5) on stored samples in mixed precision
    against FP64, with no Metropolis moves, so both evaluate the same walkers:
    N = 64, P = 30 (32 splines: the staged FP32 evaluation and the equal-width
    store), Gaussian pair potential, real time, 256 walkers, three steps with
    refresh windows of a quarter.  The parameter increments (about 1e-2) agree
    to 2e-4 of their largest magnitude (FP32 pair sums and the 3xTF32 S through
    the regularised solves; measured 1.7e-5); RK4 and the predictor-corrector
    differ from each other by about 8e-3 on the same case."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "eval_d3_n64_p10.npz"))
    dim, n, L = int(z["dim"]), int(z["n"]), float(z["L"])
    p, nw = 30, 256
    rng = np.random.default_rng(23)
    cfgs = soa(z["cfgs"])
    R = np.concatenate([cfgs] * (nw // len(cfgs) + 1))[:nw] + rng.normal(0, 0.02, size=(nw, dim, n))
    uR = -0.4 * np.exp(-np.linspace(0.0, 4.0, p)) + 0.005 * rng.normal(size=p)
    uI = 0.01 * rng.normal(size=p)
    out = {}
    for prec in ("fp64", "mixed"):
        s = T.BosonsBulk(dim, n, p, L, nw, system_params=(0.5, 2.0), potential="gauss", hbar2_2m=0.09,
                         precision=prec)
        s.SetParameters(uR, uI, 0.0, 0.0)
        s.SetWalkers(R)
        td = T.TDVP(s, 1e-3, 0, 0.3, seed=3, imaginary_time=0, use_adjoint=1, ode_solver=ode, update_every=1,
                    update_percent=25.0)
        st = td.step(3)
        assert st["status"] == 0, st
        gp = s.GetParameters()
        out[prec] = np.concatenate([gp[0] - uR, gp[1] - uI])
    d64, dmx = out["fp64"], out["mixed"]
    assert np.abs(d64).max() > 0
    assert np.abs(dmx - d64).max() < 2e-4 * np.abs(d64).max(), np.abs(dmx - d64).max() / np.abs(d64).max()


def test_store_state_rules():
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    z = np.load(os.path.join(GOLD, "eval_d3_n64_p10.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw = 8
    s = T.BosonsBulk(dim, n, p, L, nw, precision="fp64")
    s.SetParameters(z["uR"], z["uI"])
    R = np.concatenate([soa(z["cfgs"])] * 2)[:nw]
    s.SetWalkers(R)
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateExpectationValuesForStoredSamples()
    assert e.value.code == N.ERR_STATE
    s.FillCorrelatedSamplingData()
    s.CalculateExpectationValuesForStoredSamples()
    s.DoMetropolisSteps(4, 0.2, seed=1, pass_id=0)  # moving the walkers invalidates the store
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateExpectationValuesForStoredSamples()
    assert e.value.code == N.ERR_STATE
    s.FillCorrelatedSamplingData()
    s.SetWalkers(R)
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateExpectationValuesForStoredSamples()
    assert e.value.code == N.ERR_STATE
    with pytest.raises(N.TdvmcError) as e:
        T.TDVP(s, 0.01, 4, 0.2, ode_solver=3, update_every=1, update_percent=150.0).step()
    assert e.value.code == N.ERR_ARG
