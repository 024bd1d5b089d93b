"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Tolerances (stated per test):
  FP64 path   relative 1e-12 on ln psi, O_k, E_loc, the kinetic sums and
              dE_loc/d alpha (scaled by the largest magnitude of the vector);
  mixed path  relative 1e-5 per walker on the same quantities (FP32 pairs),
              evaluated on FP32-representable coordinates (the walkers the
              mixed path holds; the oracle sees the same configuration);
  sampler     FP64: the same Philox stream gives the same chain as the oracle
              (positions to 1e-9, identical acceptance counts); mixed: the
              sampled averages agree with the reference's own chain within 3
              sigma (E^R, E^I) and 4 sigma per O_k.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
EVAL_FILES = sorted(glob.glob(os.path.join(GOLD, "eval_*.npz")))

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def gpu_system(z, nw, precision, potential="square", sysp=None, hbar2_2m=1.0):
    import tdvmc_gb300 as T
    kn = z["knots"] if z["knots"].size else None
    s = T.BosonsBulk(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), nw,
                     system_params=z["sysp"] if sysp is None else sysp, potential=potential, user_knots=kn,
                     hbar2_2m=hbar2_2m, precision=precision)
    s.SetTime(float(z["time"]))
    return s


def oracle_system(z, pot_kind=orc.POT_SQUARE, sysp=None, hbar2_2m=1.0):
    kn = z["knots"] if z["knots"].size else None
    return orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), user_knots=kn, pot_kind=pot_kind,
                            pot=z["sysp"] if sysp is None else sysp, time=float(z["time"]), hbar2_2m=hbar2_2m)


def soa(cfgs):
    """(ncfg, n, dim) particle-major -> walker SoA (ncfg, dim, n)."""
    return np.ascontiguousarray(np.transpose(np.asarray(cfgs), (0, 2, 1)))


def min_pair_distance(R, L):
    d = R[:, None, :] - R[None, :, :]
    d -= L * np.trunc(d / L + np.where(d >= 0, 0.5, -0.5))
    r = np.sqrt((d * d).sum(-1))
    return r[np.triu_indices(len(R), 1)].min()


CASES = [(f, prec, pot) for f in EVAL_FILES for prec in ("fp64", "mixed") for pot in ("square", "lj", "gauss")]


@pytest.mark.parametrize("path,precision,pot", CASES,
                         ids=["%s-%s-%s" % (os.path.basename(c[0])[5:-4], c[1], c[2]) for c in CASES])
def test_eval_and_adjoint_match_oracle(path, precision, pot):
    z = np.load(path)
    cfgs = z["cfgs"]
    if precision == "mixed":
        cfgs = cfgs.astype(np.float32).astype(np.float64)
    nw = len(cfgs)
    # LJ in reduced units; square well and Gaussian soft core with the file's parameters
    # (including the quench branch of eval_d1_n20_p10_quench)
    sysp = np.array([1.0, 1.0]) if pot == "lj" else z["sysp"]
    s = gpu_system(z, nw, precision, potential=pot, sysp=sysp, hbar2_2m=0.09)
    kind = {"square": orc.POT_SQUARE, "lj": orc.POT_LJ, "gauss": orc.POT_GAUSS}[pot]
    o = oracle_system(z, pot_kind=kind, sysp=sysp, hbar2_2m=0.09)
    s.SetParameters(z["uR"], z["uI"], float(z["phiR"]), float(z["phiI"]))
    s.SetWalkers(soa(cfgs))
    fwd = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    tol = 1e-12 if precision == "fp64" else 1e-5
    for c, R in enumerate(cfgs):
        if precision == "mixed" and pot == "lj" and min_pair_distance(R, float(z["L"])) < 0.7:
            # overlapping particles (V ~ 1e20): FP32 coordinates resolve r only to
            # ~1e-6 absolute, which (sigma/r)^12 turns into a relative error far
            # above 1e-5; such configurations have zero weight in any chain
            continue
        r = o.eval(z["uR"], z["uI"], R, adjoint=True)
        scale_lnpsi = max(abs(r["lnpsi"]), np.abs(z["uR"]).max() * len(R))
        assert abs(fwd["lnpsi"][c] - r["lnpsi"]) < tol * scale_lnpsi
        assert relmax(fwd["O"][c], r["O"]) < tol
        scaleE = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(fwd["eloc"][c] - r["eloc"]).max() < tol * scaleE
        assert np.abs(fwd["other"][c] - r["other"]).max() < tol * scaleE
        scaled = max(np.abs(r["dE"]).max(), 1.0)
        assert np.abs(dE[c] - r["dE"]).max() < tol * scaled


def test_sampler_follows_oracle_chain_fp64():
    """Same Philox stream, same move rule: the FP64 chain equals the oracle's."""
    z = np.load(os.path.join(GOLD, "eval_d3_n64_p10.npz"))
    nw = 24
    rng = np.random.default_rng(8)
    R0 = np.concatenate([soa(z["cfgs"])] * 2)[:nw] + rng.normal(0, 0.01, size=(nw, 3, 64))
    R0 = np.array([[[orc.lib().orc_nic_coord(v, float(z["L"])) for v in row] for row in w] for w in R0])
    s = gpu_system(z, nw, "fp64")
    o = oracle_system(z)
    uR = np.asarray(z["uR"]) * 0.5
    s.SetParameters(uR, z["uI"])
    s.SetWalkers(R0)
    acc_gpu = s.DoMetropolisSteps(2 * 64, 0.3, seed=1234, pass_id=7)
    Ro = R0.copy()
    acc_orc = o.sample(uR, Ro, 2 * 64, 0.3, seed=1234, pass_id=7)
    assert acc_gpu == acc_orc
    assert np.abs(s.GetWalkers() - Ro).max() < 1e-9


def test_sampler_matches_reference_chain_mixed():
    """FP32 chain vs the reference's mt19937 chain (tests/golden/sample_d3_n27.npz)."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    blocks = z["blocks"]
    ref_mean = blocks.mean(0)
    ref_err = blocks.std(0, ddof=1) / np.sqrt(len(blocks))
    nw = 4096
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=z["sysp"], potential="square", precision="mixed")
    s.SetParameters(z["uR"], z["uI"])
    R = np.repeat(z["R0"].T[None], nw, axis=0) + np.random.default_rng(2).normal(0, 0.05, size=(nw, dim, n))
    s.SetWalkers(R)
    s.DoMetropolisSteps(50 * n, float(z["step"]), seed=5, pass_id=0)
    rows = []
    acc = 0
    nsamp = 8
    for k in range(nsamp):
        acc += s.DoMetropolisSteps(n, float(z["step"]), seed=5, pass_id=k + 1)
        f = s.CalculateExpectationValues()
        rows.append(np.concatenate([f["eloc"], f["O"]], axis=1))
    per_walker = np.array(rows).mean(0)
    mean = per_walker.mean(0)
    err = per_walker.std(0, ddof=1) / np.sqrt(nw)
    comb = np.sqrt(err ** 2 + ref_err[1:3 + p] ** 2)
    diff = np.abs(mean - ref_mean[1:3 + p])
    assert np.all(diff[comb == 0] < 1e-6)
    dev = np.where(comb > 0, diff / np.where(comb > 0, comb, 1), 0)
    assert dev[0] < 3 and dev[1] < 3, dev
    assert np.all(dev[2:] < 4), dev
    rate = acc / (nsamp * n * nw)
    assert abs(rate - ref_mean[0]) < 3 * ref_err[0] + 0.01


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reduction_and_solve_match_oracle(precision):
    z = np.load(os.path.join(GOLD, "eval_d3_n64_p10.npz"))
    nw = 1000
    rng = np.random.default_rng(4)
    R = np.concatenate([soa(z["cfgs"])] * (nw // len(z["cfgs"]) + 1))[:nw] + rng.normal(0, 0.05, size=(nw, 3, 64))
    s = gpu_system(z, nw, precision, potential="lj", sysp=(1.0, 1.0), hbar2_2m=0.09)
    s.SetParameters(z["uR"], z["uI"], 0.3, -0.1)
    s.SetWalkers(R)
    f = s.CalculateExpectationValues()
    st = s.ReduceStatistics()
    O, E = f["O"], f["eloc"]
    Oc = O - O.mean(0)
    tolS = 1e-12 if precision == "fp64" else 2e-6
    assert relmax(st["O"], O.mean(0)) < 1e-12
    assert abs(st["energy"][0] - E[:, 0].mean()) < 1e-12 * np.abs(E[:, 0]).max()
    assert relmax(st["S"], Oc.T @ Oc / nw) < tolS
    assert relmax(st["cov_OER"], Oc.T @ (E[:, 0] - E[:, 0].mean()) / nw) < 1e-10
    assert relmax(st["cov_OEI"], Oc.T @ (E[:, 1] - E[:, 1].mean()) / nw) < 1e-10
    for imag in (0, 1):
        for pre in (0, 1):
            for lin in (0, 1):
                g = s.SolveForParametersDot(imag, pre, lin)
                # the device solve against the oracle's, on the device's own moments: 1e-10
                r = orc.solve_centred(st["O"], st["energy"][0], st["energy"][1], st["S"], st["cov_OER"],
                                      st["cov_OEI"], imag, pre, lin)
                assert relmax(g[0], r[0]) < 1e-10
                assert relmax(g[1], r[1]) < 1e-10
                assert abs(g[2] - r[2]) < 1e-10 * max(1, abs(r[2]))
                assert abs(g[3] - r[3]) < 1e-10 * max(1, abs(r[3]))
                assert g[4] == r[4]


@pytest.mark.parametrize("ode,norm", [(2, 0), (0, 0), (2, 1)])
def test_tdvp_step_matches_oracle_fp64(ode, norm):
    """A full RK4 (or Euler) step: sampling, evaluation, reduction, solve, update.
    With USE_NORMALIZE_WF the step ends with phi^R = -ln psi of the last sampled
    configuration of walker 0 at the last stage's parameters (NormalizeWavefunction,
    TDVMC.cpp:2525-2529, 3760-3766), against the oracle's value at 1e-12."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw, moves, step, dt, seed, pass0 = 64, 2 * n, 0.35, 0.01, 77, 3
    rng = np.random.default_rng(9)
    R0 = np.repeat(z["R0"].T[None], nw, axis=0) + rng.normal(0, 0.05, size=(nw, dim, n))
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    uR, uI = np.asarray(z["uR"]), np.asarray(z["uI"])
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09, precision="fp64")
    s.SetParameters(uR, uI, 0.0, 0.0)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(0, step, seed, pass0)  # sets the Philox pass counter
    td = T.TDVP(s, dt, moves, step, seed=seed, ode_solver=ode, normalize_wf=norm)
    td.step()
    gR, gI, gpR, gpI = s.GetParameters()

    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0), hbar2_2m=0.09)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    cur = base.copy()
    Ro = R0.copy()
    ks = []
    nst = 4 if ode == 2 else 1
    for k in range(nst):
        out = o.stage(cur[:p], cur[p:2 * p], Ro, moves, step, seed, pass0 + k, threads=4, adjoint=False)
        lnpsi0 = out["lnpsi"][0]
        m = orc.centred(out["O"], out["eloc"])
        dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"])
        kv = np.concatenate([dR, dI, [pR, pI]])
        ks.append(kv)
        if ode == 2 and k < 3:
            cur = base + kv * (dt / 2 if k < 2 else dt)
    if ode == 2:
        new = orc.rk4_combine(base, ks, dt)
    else:
        new = base + ks[0] * dt
    if norm:
        new[2 * p] = -lnpsi0
        assert abs(gpR + lnpsi0) < 1e-12 * max(abs(lnpsi0), 1.0)
    assert np.abs(s.GetWalkers() - Ro).max() < 1e-9
    got = np.concatenate([gR, gI, [gpR, gpI]])
    assert relmax(got, new) < 1e-9


def test_errors_and_call_order():
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    with pytest.raises(N.TdvmcError):
        T.BosonsBulk(3, 8, 3, 4.0, 4)  # too few parameters
    with pytest.raises(N.TdvmcError):
        T.BosonsBulk(4, 8, 10, 4.0, 4)  # DIM out of range
    s = T.BosonsBulk(3, 8, 10, 4.0, 4)
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateExpectationValues()  # no walkers yet
    assert e.value.code == N.ERR_STATE
    with pytest.raises(AssertionError):
        s.SetWalkers(np.zeros((5, 3, 8)))


@pytest.mark.parametrize("nw,n,dim", [(1, 2, 1), (3, 5, 2), (37, 33, 3), (5, 97, 3)])
def test_ragged_sizes_match_oracle(nw, n, dim):
    """Walker counts that do not fill a block, particle counts that do not fill a lane group."""
    import tdvmc_gb300 as T
    p, L = 8, 3.0 + n ** (1.0 / dim)
    rng = np.random.default_rng(n)
    uR, uI = rng.normal(0, 0.2, p), rng.normal(0, 0.1, p)
    R = rng.uniform(-L / 2, L / 2, size=(nw, dim, n))
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", precision="fp64")
    s.SetParameters(uR, uI)
    s.SetWalkers(R)
    f = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0))
    for w in range(nw):
        r = o.eval(uR, uI, R[w].T, adjoint=True)
        assert relmax(f["O"][w], r["O"]) < 1e-12 or np.abs(r["O"]).max() == 0
        sc = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(f["eloc"][w] - r["eloc"]).max() < 1e-12 * sc
        assert np.abs(dE[w] - r["dE"]).max() < 1e-12 * max(np.abs(r["dE"]).max(), 1.0)


@pytest.mark.parametrize("dim,n", [(3, 65), (3, 80), (3, 96), (3, 111), (3, 337), (1, 70), (2, 70)])
def test_half_sweep_slot_edges_mixed(dim, n):
    """FP32 32-lane evaluation (the half sweep of the forward kernel and the rotated
    own slot of the adjoint) at particle counts that leave the last slot of 32 rows
    with 1, 16, 32, 15, 17 and 6 rows, in 3D and at N = 70 in 1D and 2D, on
    FP32-representable coordinates; tolerance as in the fixture cases (1e-5)."""
    import tdvmc_gb300 as T
    p, nw = 12, 9
    L = (n / 0.4) ** (1.0 / dim)
    rng = np.random.default_rng(n)
    R = rng.uniform(-L / 2, L / 2, size=(nw, dim, n)).astype(np.float32).astype(np.float64)
    uR, uI = rng.normal(0, 0.2, p), rng.normal(0, 0.1, p)
    sysp = (0.5, 2.0)
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=sysp, potential="gauss", hbar2_2m=0.09, precision="mixed")
    assert s.Tiles()["eval_lanes"] == 32
    s.SetParameters(uR, uI)
    s.SetWalkers(R)
    f = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_GAUSS, pot=sysp, hbar2_2m=0.09)
    tol = 1e-5
    for w in range(nw):
        r = o.eval(uR, uI, R[w].T, adjoint=True)
        assert abs(f["lnpsi"][w] - r["lnpsi"]) < tol * max(abs(r["lnpsi"]), np.abs(uR).max() * n)
        assert relmax(f["O"][w], r["O"]) < tol
        sc = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(f["eloc"][w] - r["eloc"]).max() < tol * sc
        assert np.abs(f["other"][w] - r["other"]).max() < tol * sc
        assert np.abs(dE[w] - r["dE"]).max() < tol * max(np.abs(r["dE"]).max(), 1.0)


def test_adjoint_driven_imaginary_time_step_matches_oracle_fp64():
    """Imaginary-time Euler step with the adjoint in the force:
    F_k = -(cov(O_k, E^R) + <dE_loc/d uR_k> / 2), i.e. -1/2 d<E>/d uR_k."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw, moves, step, dt, seed, pass0 = 96, 2 * n, 0.35, 0.01, 5, 11
    rng = np.random.default_rng(12)
    R0 = np.repeat(z["R0"].T[None], nw, axis=0) + rng.normal(0, 0.05, size=(nw, dim, n))
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    uR, uI = np.asarray(z["uR"]), np.zeros(p)
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09, precision="fp64")
    s.SetParameters(uR, uI, 0.0, 0.0)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(0, step, seed, pass0)
    td = T.TDVP(s, dt, moves, step, seed=seed, ode_solver=0, imaginary_time=1, use_adjoint=2)
    td.step()
    gR, gI, gpR, gpI = s.GetParameters()

    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0), hbar2_2m=0.09)
    Ro = R0.copy()
    out = o.stage(uR, uI, Ro, moves, step, seed, pass0, threads=4, adjoint=True)
    m = orc.centred(out["O"], out["eloc"])
    dER = out["dE"][:, :, 0].mean(0)
    dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"] + 0.5 * dER, m["cOEI"],
                                          imag=1)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    new = base + np.concatenate([dR, dI, [pR, pI]]) * dt
    got = np.concatenate([gR, gI, [gpR, gpI]])
    assert relmax(got, new) < 1e-9
    # and it differs from the plain covariance force
    dR0 = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"], imag=1)[0]
    assert relmax(dR0, dR) > 1e-9


@pytest.mark.parametrize("mode", ["fp64", "mixed", "mixed-scalar"])
@pytest.mark.parametrize("dim,n", [(1, 20), (2, 40), (3, 150), (3, 300), (3, 600)])
def test_sampler_padded_slots_follow_oracle_chain(dim, n, mode):
    """Particle counts whose register slots run past n (the slot count is rounded
    up to a compiled one: N = 20 on 8 lanes in 4 slots, 40 on 16 lanes in 4, 150
    on 32 lanes in 8, 300 on 32 lanes in 11, 600 on 32 lanes in 32, whose packed
    FP32 sampler reads the lane's coordinates from shared memory) in 1D, 2D and 3D.  FP64: the chain
    equals the oracle's (same Philox stream; positions 1e-9, identical
    acceptance).  FP32, packed and scalar samplers: the same moves on at least
    90 % of the walkers (a decision within FP32 rounding of its threshold may
    send a walker its own way), positions within 1e-4, acceptance within 1 %."""
    import tdvmc_gb300 as T
    precision = "fp64" if mode == "fp64" else "mixed"
    L = (n / 0.5) ** (1.0 / dim)
    nw, p, moves, step = 32, 10, 2 * n, 0.5
    rng = np.random.default_rng(100 * dim + n)
    uR, uI = 0.3 * rng.normal(size=p), 0.1 * rng.normal(size=p)
    R0 = rng.uniform(-L / 2, L / 2, size=(nw, dim, n))
    if precision == "mixed":
        R0 = R0.astype(np.float32).astype(np.float64)
    if mode == "mixed-scalar":
        os.environ["TDVMC_SAMPLER"] = "scalar"
    try:
        s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", precision=precision)
    finally:
        os.environ.pop("TDVMC_SAMPLER", None)
    s.SetParameters(uR, uI)
    s.SetWalkers(R0)
    acc = s.DoMetropolisSteps(moves, step, seed=21, pass_id=4)
    Rg = s.GetWalkers()
    s.close()
    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0))
    Ro = np.ascontiguousarray(R0.copy())
    acc_o = o.sample(uR, Ro, moves, step, seed=21, pass_id=4)
    assert 0.1 < acc_o / (moves * nw) < 0.95
    if precision == "fp64":
        assert acc == acc_o
        assert np.abs(Rg - Ro).max() < 1e-9
    else:
        d = np.abs(Rg - Ro).reshape(nw, -1).max(1)
        assert (d < 1e-4).mean() >= 0.9, d
        assert abs(acc - acc_o) <= 0.01 * acc_o, (acc, acc_o)


def test_packed_sampler_with_shared_coordinates_follows_scalar_chain():
    """N = 600 (32 slots of 32 lanes: the packed sampler that reads the lane's
    own coordinates from shared memory at each move) walks the scalar FP32
    sampler's chain bit for bit: identical walkers and acceptance counts."""
    import tdvmc_gb300 as T
    n, p, nw = 600, 20, 256
    L = (n / 0.365) ** (1.0 / 3.0)
    rng = np.random.default_rng(17)
    m = 9
    idx = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    R0 = idx[None] * (L / m) + (rng.uniform(size=(nw, n, 3)) - 0.5) * (L / m) * 0.3 - L / 2
    R0 = np.ascontiguousarray(np.transpose(R0, (0, 2, 1))).astype(np.float32).astype(np.float64)
    r = np.linspace(0.0, L / 2, p)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    out = {}
    for mode in ("packed", "scalar"):
        if mode == "scalar":
            os.environ["TDVMC_SAMPLER"] = "scalar"
        try:
            s = T.BosonsBulk(3, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09,
                             precision="mixed")
        finally:
            os.environ.pop("TDVMC_SAMPLER", None)
        assert s.Tiles()["sample_lanes"] == 32
        s.SetParameters(uR, np.zeros(p))
        s.SetWalkers(R0)
        acc = s.DoMetropolisSteps(2 * n, 0.17, seed=5, pass_id=9)
        out[mode] = (acc, s.GetWalkers())
        s.close()
    (a_p, R_p), (a_s, R_s) = out["packed"], out["scalar"]
    assert a_p == a_s
    assert np.array_equal(R_p, R_s)
    assert 0.2 < a_p / (2 * n * nw) < 0.9


def test_packed_sampler_follows_scalar_chain_mixed():
    """The f32x2 FP32 sampler (uniform knots) walks the scalar FP32 sampler's
    chain bit for bit: same Philox stream and update arithmetic, and every pair
    term and partial sum rounded the same way.  Tolerance: identical walkers
    and acceptance counts."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "eval_d3_n343_p30.npz"))
    nw, n = 512, int(z["n"])
    rng = np.random.default_rng(11)
    R0 = np.concatenate([soa(z["cfgs"])] * (nw // len(z["cfgs"]))) + rng.normal(0, 0.02, size=(nw, 3, n))
    uR = np.asarray(z["uR"])
    out = {}
    for mode in ("packed", "scalar"):
        if mode == "scalar":
            os.environ["TDVMC_SAMPLER"] = "scalar"
        try:
            s = T.BosonsBulk(3, n, int(z["p"]), float(z["L"]), nw, system_params=z["sysp"], precision="mixed")
        finally:
            os.environ.pop("TDVMC_SAMPLER", None)
        s.SetParameters(uR, z["uI"])
        s.SetWalkers(R0)
        acc = s.DoMetropolisSteps(2 * n, 0.2, seed=99, pass_id=3)
        out[mode] = (acc, s.GetWalkers())
        s.close()
    (a_p, R_p), (a_s, R_s) = out["packed"], out["scalar"]
    same = np.all(R_p.reshape(nw, -1) == R_s.reshape(nw, -1), axis=1)
    assert same.mean() == 1.0, same.mean()
    assert a_p == a_s
    assert 0.05 < a_p / (2 * n * nw) < 0.95


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_maximum_size_matches_oracle(precision, tol):
    """N = 1024 (the largest N the C ABI accepts) with p = 64: evaluation and
    adjoint against the oracle, and for FP64 the sampler chain (positions 1e-9,
    identical acceptance).  FP64: relative 1e-12 throughout.  Mixed, on
    FP32-representable coordinates: relative 1e-5 on ln psi, O_k, E_loc, the
    kinetic sums and dE/d alpha."""
    import tdvmc_gb300 as T
    dim, n, p = 3, 1024, 64
    L = float((n / 0.365) ** (1.0 / 3.0))
    nw = 3
    rng = np.random.default_rng(1024)
    m = int(np.ceil(n ** (1 / 3)))
    idx = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    cfgs = np.array([idx * (L / m) + rng.uniform(-0.1, 0.1, size=(n, 3)) * (L / m) - L / 2 for _ in range(nw)])
    cfgs = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(cfgs)  # inside the box, as the sampler keeps them
    if precision == "mixed":
        cfgs = cfgs.astype(np.float32).astype(np.float64)
    r = np.linspace(0.0, L / 2, p)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    uI = 0.01 * rng.normal(size=p)
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09,
                     precision=precision)
    s.SetParameters(uR, uI)
    s.SetWalkers(soa(cfgs))
    f = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    o = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_LJ, pot=(1.0, 1.0), hbar2_2m=0.09)
    for w in range(nw):
        ref = o.eval(uR, uI, cfgs[w], adjoint=True)
        assert relmax(f["O"][w], ref["O"]) < tol
        assert relmax(f["eloc"][w], ref["eloc"]) < tol, (f["eloc"][w], ref["eloc"])
        assert relmax(f["other"][w], ref["other"]) < tol, (f["other"][w], ref["other"])
        assert relmax(dE[w], ref["dE"]) < tol, relmax(dE[w], ref["dE"])
        assert abs(f["lnpsi"][w] - ref["lnpsi"]) <= tol * max(abs(ref["lnpsi"]), 1.0)
    if precision == "fp64":
        R0 = soa(cfgs)
        s.SetWalkers(R0)
        acc = s.DoMetropolisSteps(256, 0.1, seed=3, pass_id=2)
        Ro = R0.copy()
        acc_o = o.sample(uR, Ro, 256, 0.1, seed=3, pass_id=2)
        assert acc == acc_o
        assert np.abs(s.GetWalkers() - Ro).max() < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("env", [{"TDVMC_HIST": "0"}, {"TDVMC_HIST": "1"}, {"TDVMC_HIST": "2"},
                                 {"TDVMC_EVAL_WALKERS_PER_BLOCK": "1"}, {"TDVMC_EVAL_WALKERS_PER_BLOCK": "4"}],
                         ids=["hist0", "hist1", "hist2", "wpb1", "wpb4"])
def test_evaluation_variants_match_oracle(precision, env):
    """The evaluation kernels' histogram update modes (lane-private records,
    float4 slots, shared-memory atomics) and forced walkers per block, selected
    through the environment when the context is created: same results as the
    oracle at the tolerances of the fixture cases."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "eval_d3_n343_p30.npz"))
    cfgs = z["cfgs"]
    if precision == "mixed":
        cfgs = cfgs.astype(np.float32).astype(np.float64)
    nw = len(cfgs)
    sysp = np.array([1.0, 1.0])
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        s = gpu_system(z, nw, precision, potential="lj", sysp=sysp, hbar2_2m=0.09)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    o = oracle_system(z, pot_kind=orc.POT_LJ, sysp=sysp, hbar2_2m=0.09)
    s.SetParameters(z["uR"], z["uI"], float(z["phiR"]), float(z["phiI"]))
    s.SetWalkers(soa(cfgs))
    fwd = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    tol = 1e-12 if precision == "fp64" else 1e-5
    for c, R in enumerate(cfgs):
        if precision == "mixed" and min_pair_distance(R, float(z["L"])) < 0.7:
            continue  # overlapping particles: see test_eval_and_adjoint_match_oracle
        r = o.eval(z["uR"], z["uI"], R, adjoint=True)
        assert relmax(fwd["O"][c], r["O"]) < tol
        scaleE = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(fwd["eloc"][c] - r["eloc"]).max() < tol * scaleE
        assert np.abs(fwd["other"][c] - r["other"]).max() < tol * scaleE
        scaled = max(np.abs(r["dE"]).max(), 1.0)
        assert np.abs(dE[c] - r["dE"]).max() < tol * scaled


def test_profile_stage_leaves_the_step_boundary():
    """tdvmc_profile_stage runs one stage eagerly and then puts the parameters and
    the stage index back to the step boundary: the parameters are unchanged, and
    after one more step the evaluation uses that step's final parameters (a fresh
    context given the same walkers and parameters evaluates identically)."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw = 64
    rng = np.random.default_rng(5)
    R0 = np.repeat(z["R0"].T[None], nw, axis=0) + rng.normal(0, 0.05, size=(nw, dim, n))
    mk = lambda: T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09,  # noqa
                              precision="fp64")
    s = mk()
    s.SetParameters(z["uR"], z["uI"], 0.0, 0.0)
    s.SetWalkers(R0)
    td = T.TDVP(s, 1e-3, n, 0.35, seed=3)
    before = np.concatenate(s.GetParameters()[:2])
    td.profile_stage()
    assert np.array_equal(np.concatenate(s.GetParameters()[:2]), before)
    td.step()
    got = s.CalculateExpectationValues()
    f = mk()
    f.SetParameters(*s.GetParameters())
    f.SetWalkers(s.GetWalkers())
    ref = f.CalculateExpectationValues()
    for key in ("lnpsi", "O", "eloc", "other"):
        assert np.array_equal(got[key], ref[key]), key
