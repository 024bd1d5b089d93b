"""GPU: batched trapped drops of uneven particle number (all drops in one
launch per kernel) against the FP64 oracle restatement.

Tolerances (stated per test):
  evaluation and adjoint vs the oracle: FP64 relative 1e-12, mixed 1e-5 (each
      quantity scaled by its largest magnitude over the drop's walkers; mixed
      walkers are FP32-representable, the coordinates the mixed path holds);
  known answer (no interaction, exact Gaussian): E_loc = (3/2) omega n for
      every walker, FP64 1e-12 relative, mixed 1e-6;
  FP64 sampler chain vs the oracle chain (same Philox stream): positions
      1e-9, identical acceptance counts;
  per-drop reduction and solve vs numpy / the oracle solve: 1e-10;
  one RK4 step of every drop vs the oracle step: parameters 1e-9;
  an adjoint-driven imaginary-time Euler step vs the oracle: parameters 1e-9.
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

NS = [3, 6, 10, 20, 2, 32]  # particle numbers of the drops (both limits included)
P = 12
RMAX = 4.0


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def params(rng, S, aP=-0.45):
    r = np.linspace(0.0, RMAX, P)
    base = 0.3 * np.exp(-r / 0.7)  # a repulsive-core-like pair Jastrow (u decreasing in r)
    uR = np.array([np.concatenate([base + 0.02 * rng.normal(size=P), [aP + 0.02 * rng.normal()]]) for _ in range(S)])
    uI = 0.01 * rng.normal(size=(S, P + 1))
    return uR, uI


def walkers(rng, ns, nw, f32):
    out = []
    for n in ns:
        w = rng.normal(scale=1.0, size=(nw, 3, n))
        out.append(w.astype(np.float32).astype(np.float64) if f32 else w)
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_drops_eval_and_adjoint_match_oracle(precision, tol):
    import tdvmc_gb300 as T
    rng = np.random.default_rng(4)
    nw = 37  # not a multiple of any block size: ragged last work item
    d = T.TrappedDrops(NS, P, RMAX, nw, omega=1.0, v0=1.0, sigma=0.5, hbar2_2m=0.5, precision=precision)
    uR, uI = params(rng, len(NS))
    d.SetParameters(uR, uI)
    W = walkers(rng, NS, nw, precision == "mixed")
    d.SetWalkers(W)
    out = d.CalculateExpectationValues(adjoint=True)
    for s, n in enumerate(NS):
        o = orc.OracleDrop(n, P, RMAX, v0=1.0, sigma=0.5, omega=1.0, hbar2_2m=0.5)
        refs = [o.eval(uR[s], uI[s], W[s][w].T, adjoint=True) for w in range(nw)]
        for key in ("O", "eloc", "other", "dE"):
            ref = np.array([r[key] for r in refs])
            assert rel(out[key][s], ref) < tol, (n, key, rel(out[key][s], ref))
        lp = np.array([r["lnpsi"] for r in refs])
        assert np.abs(out["lnpsi"][s] - lp).max() <= tol * max(np.abs(lp).max(), 1.0)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_drops_known_answer_exact_gaussian(precision, tol):
    """No interaction and the exact trap ground state: E_loc = (3/2) omega n,
    zero variance, for every configuration of every drop in the batch."""
    import tdvmc_gb300 as T
    rng = np.random.default_rng(44)
    nw, omega, c = 64, 1.3, 0.5
    d = T.TrappedDrops(NS, P, RMAX, nw, omega=omega, v0=0.0, sigma=0.5, hbar2_2m=c, precision=precision)
    S = len(NS)
    uR = np.zeros((S, P + 1))
    uR[:, P] = -omega / (4.0 * c)
    d.SetParameters(uR, np.zeros((S, P + 1)))
    d.SetWalkers(walkers(rng, NS, nw, precision == "mixed"))
    d.DoMetropolisSteps(4, 0.6, seed=5, pass_id=0)
    out = d.CalculateExpectationValues(adjoint=True)
    for s, n in enumerate(NS):
        e = 1.5 * omega * n
        assert np.abs(out["eloc"][s][:, 0] - e).max() < tol * e, (n, out["eloc"][s][:, 0][:4])
        assert np.abs(out["eloc"][s][:, 1]).max() < tol * e
    st = d.ReduceStatistics()
    assert np.allclose(st["energy"][:, 0], 1.5 * omega * np.array(NS), rtol=tol)
    # the force vanishes at the exact ground state: cov(O, E) = 0
    assert np.abs(st["cov_OER"]).max() < 1e-5 * np.abs(st["S"]).max()


def test_drops_fp64_chain_matches_oracle_chain():
    import tdvmc_gb300 as T
    rng = np.random.default_rng(7)
    nw = 40
    d = T.TrappedDrops(NS, P, RMAX, nw, v0=1.0, sigma=0.5, precision="fp64")
    uR, uI = params(rng, len(NS))
    d.SetParameters(uR, uI)
    W = walkers(rng, NS, nw, False)
    d.SetWalkers(W)
    acc = d.DoMetropolisSteps(3, 0.5, seed=11, pass_id=6)
    got = d.GetWalkers()
    tot = 0
    for s, n in enumerate(NS):
        o = orc.OracleDrop(n, P, RMAX, v0=1.0, sigma=0.5)
        R = np.ascontiguousarray(W[s])
        tot += o.sample(uR[s], R, 3 * n, 0.5, seed=11, pass_id=6, walker0=s * nw)
        assert np.abs(got[s] - R).max() < 1e-9, n
    assert acc == tot
    assert 0.05 < acc / (3 * nw * sum(NS)) < 0.95


def test_drops_reduction_and_solve_match_oracle():
    import tdvmc_gb300 as T
    rng = np.random.default_rng(8)
    nw = 300
    d = T.TrappedDrops(NS, P, RMAX, nw, v0=1.0, sigma=0.5, precision="fp64")
    uR, uI = params(rng, len(NS))
    d.SetParameters(uR, uI)
    d.SetWalkers(walkers(rng, NS, nw, False))
    d.DoMetropolisSteps(5, 0.5, seed=3, pass_id=1)
    out = d.CalculateExpectationValues(adjoint=True)
    st = d.ReduceStatistics()
    for imag in (0, 1):
        uRd, uId, pRd, pId, status = d.SolveForParametersDot(imaginary_time=imag)
        for s in range(len(NS)):
            c = orc.centred(out["O"][s], out["eloc"][s])
            assert rel(st["O"][s], c["O"]) < 1e-10
            assert rel(st["S"][s], c["S"]) < 1e-10
            assert rel(st["cov_OER"][s], c["cOER"]) < 1e-10
            assert rel(st["dE"][s], out["dE"][s].mean(0)) < 1e-10
            r = orc.solve_centred(c["O"], c["ER"], c["EI"], c["S"], c["cOER"], c["cOEI"], imag=imag)
            assert rel(uRd[s], r[0]) < 1e-10 and rel(uId[s], r[1]) < 1e-10
            assert abs(pRd[s] - r[2]) <= 1e-10 * max(abs(r[2]), 1.0)
            assert int(status[s]) == (5 if r[4] else 0)


def test_drops_rk4_step_matches_oracle():
    """One RK4 step of every drop: four stages of sampling (the oracle walks the
    same Philox stream), evaluation, per-drop reduction and solve, then the RK4
    combination, FP64 against the oracle run the same way."""
    import tdvmc_gb300 as T
    rng = np.random.default_rng(9)
    ns = [3, 6, 10, 20]
    nw, dt, sweeps, step, seed = 96, 2e-3, 2, 0.5, 21
    d = T.TrappedDrops(ns, P, RMAX, nw, v0=1.0, sigma=0.5, precision="fp64")
    uR, uI = params(rng, len(ns))
    W = walkers(rng, ns, nw, False)
    d.SetParameters(uR, uI)
    d.SetWalkers(W)
    td = T.DropsTDVP(d, dt, sweeps, step, seed=seed, use_adjoint=1)
    res = d.GetParameters()  # pass counter 0 at creation
    out = td.step(1)
    assert (out["status"] == 0).all()
    gR, gI, gpR, gpI = d.GetParameters()
    for s, n in enumerate(ns):
        o = orc.OracleDrop(n, P, RMAX, v0=1.0, sigma=0.5)
        R = np.ascontiguousarray(W[s])
        u = np.concatenate([uR[s], uI[s], [0.0, 0.0]])
        p1 = P + 1
        ks = []
        cur = u.copy()
        for k in range(4):
            o.sample(cur[:p1], R, sweeps * n, step, seed=seed, pass_id=k, walker0=s * nw)
            ev = [o.eval(cur[:p1], cur[p1:2 * p1], R[w].T, adjoint=True) for w in range(nw)]
            c = orc.centred(np.array([e["O"] for e in ev]), np.array([e["eloc"] for e in ev]))
            r = orc.solve_centred(c["O"], c["ER"], c["EI"], c["S"], c["cOER"], c["cOEI"], imag=0)
            kk = np.concatenate([r[0], r[1], [r[2], r[3]]])
            ks.append(kk)
            cur = u + kk * (dt / 2.0 if k < 2 else dt)
        new = orc.rk4_combine(u, ks, dt)
        assert rel(gR[s], new[:p1]) < 1e-9, n
        assert rel(gI[s], new[p1:2 * p1]) < 1e-9, n
        assert abs(gpR[s] - new[2 * p1]) < 1e-9 * max(abs(new[2 * p1]), 1.0)
    del res


def test_drops_adjoint_imaginary_time_step_matches_oracle():
    """An imaginary-time Euler step of every drop driven by the adjoint
    (F_k = -(cov(O_k, E^R) + <dE_loc/d uR_k> / 2)), FP64 against the oracle run
    the same way: parameters relative 1e-9."""
    import tdvmc_gb300 as T
    rng = np.random.default_rng(19)
    ns = [3, 6, 10, 20]
    nw, dt, sweeps, step, seed = 128, 5e-3, 2, 0.5, 23
    d = T.TrappedDrops(ns, P, RMAX, nw, v0=1.0, sigma=0.5, precision="fp64")
    uR, uI = params(rng, len(ns))
    uI[:] = 0.0
    W = walkers(rng, ns, nw, False)
    d.SetParameters(uR, uI)
    d.SetWalkers(W)
    out = T.DropsTDVP(d, dt, sweeps, step, seed=seed, imaginary_time=1, ode_solver=0, use_adjoint=2).step(1)
    assert (out["status"] == 0).all()
    gR, gI, gpR, gpI = d.GetParameters()
    p1 = P + 1
    for s, n in enumerate(ns):
        o = orc.OracleDrop(n, P, RMAX, v0=1.0, sigma=0.5)
        R = np.ascontiguousarray(W[s])
        o.sample(uR[s], R, sweeps * n, step, seed=seed, pass_id=0, walker0=s * nw)
        ev = [o.eval(uR[s], uI[s], R[w].T, adjoint=True) for w in range(nw)]
        c = orc.centred(np.array([e["O"] for e in ev]), np.array([e["eloc"] for e in ev]))
        dER = np.array([e["dE"][:, 0] for e in ev]).mean(0)
        r = orc.solve_centred(c["O"], c["ER"], c["EI"], c["S"], c["cOER"] + 0.5 * dER, c["cOEI"], imag=1)
        new = np.concatenate([uR[s], uI[s], [0.0, 0.0]]) + np.concatenate([r[0], r[1], [r[2], r[3]]]) * dt
        assert rel(gR[s], new[:p1]) < 1e-9, n
        assert rel(gI[s], new[p1:2 * p1]) < 1e-9 or np.abs(new[p1:2 * p1]).max() < 1e-300
        assert abs(gpR[s] - new[2 * p1]) < 1e-9 * max(abs(new[2 * p1]), 1.0)


def test_drops_autotune_keeps_walkers_and_results():
    import tdvmc_gb300 as T
    rng = np.random.default_rng(13)
    nw = 512
    d = T.TrappedDrops(NS, P, RMAX, nw, v0=1.0, sigma=0.5, precision="mixed")
    uR, uI = params(rng, len(NS))
    d.SetParameters(uR, uI)
    d.SetWalkers(walkers(rng, NS, nw, True))
    before = d.GetWalkers()
    ref = d.CalculateExpectationValues(adjoint=True)
    tiles = d.Autotune(2, 0.5)
    assert tiles["sample_walkers_per_block"] in (32, 64, 128) and tiles["eval_walkers_per_block"] in (32, 64, 128)
    after = d.GetWalkers()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    got = d.CalculateExpectationValues(adjoint=True)
    for key in ("lnpsi", "O", "eloc", "dE"):
        assert np.array_equal(got[key], ref[key]), key  # each walker is computed by one thread either way


def test_drops_argument_errors():
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    with pytest.raises(N.TdvmcError):
        T.TrappedDrops([3, 33], P, RMAX, 8)
    with pytest.raises(N.TdvmcError):
        T.TrappedDrops([3, 1], P, RMAX, 8)
    with pytest.raises(N.TdvmcError):
        T.TrappedDrops([3], 40, RMAX, 8)
    d = T.TrappedDrops([3, 4], P, RMAX, 8)
    with pytest.raises(N.TdvmcError) as e:
        d.CalculateExpectationValues()
    assert e.value.code == N.ERR_STATE
