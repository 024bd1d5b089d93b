"""GPU parity of the mirrored-distance system (PhysicalSystems::NUBosonsBulkPB)
through the C ABI, against the FP64 oracle's NUBosonsBulkPB variant and the
reference's own values in the pb_eval_* fixtures.

Tolerances (stated per test):
  FP64 path   relative 1e-12 against the oracle (ln psi, O_k, E_loc, the kinetic
              sums, dE_loc/d alpha), and the fixtures' tolerance 5e-9 against the
              reference's own numbers;
  mixed path  relative 1e-5 per walker on FP32-representable coordinates;
  sampler     FP64: the oracle's chain (positions 1e-9, identical acceptance);
              FP32: the same moves on at least 90 % of the walkers;
  steps       FP64 RK4 step (direct and on stored samples): parameters 1e-9.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
PB_FILES = sorted(glob.glob(os.path.join(GOLD, "pb_eval_*.npz")))
RTOL_REF = 5e-9

pytestmark = pytest.mark.gpu


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def soa(cfgs):
    return np.ascontiguousarray(np.transpose(np.asarray(cfgs), (0, 2, 1)))


def gpu_pb(z, nw, precision, hbar2_2m=1.0, exact=False):
    import tdvmc_gb300 as T
    s = T.NUBosonsBulkPB(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), nw, user_knots=z["knots"],
                         system_params=z["sysp"], hbar2_2m=hbar2_2m, precision=precision, exact_derivatives=exact)
    s.SetTime(float(z["time"]))
    return s


def oracle_pb(z, hbar2_2m=1.0, exact=False):
    return orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), user_knots=z["knots"],
                            pot_kind=orc.POT_SQUARE, pot=z["sysp"], time=float(z["time"]), hbar2_2m=hbar2_2m,
                            variant=orc.SYS_NU_PB_EXACT if exact else orc.SYS_NU_PB)


CASES = [(f, prec, form) for f in PB_FILES for prec in ("fp64", "mixed") for form in ("reference", "exact")]


@pytest.mark.parametrize("path,precision,form", CASES,
                         ids=["%s-%s-%s" % (os.path.basename(c[0])[8:-4], c[1], c[2]) for c in CASES])
def test_pb_eval_and_adjoint_match_oracle(path, precision, form):
    """Both forms of the mirrored pairs' derivative terms (the reference's and
    the exact one) against the oracle; the reference's form also against the
    reference's own numbers."""
    z = np.load(path)
    cfgs = z["cfgs"]
    if precision == "mixed":
        cfgs = cfgs.astype(np.float32).astype(np.float64)
    nw = len(cfgs)
    exact = form == "exact"
    s = gpu_pb(z, nw, precision, exact=exact)
    o = oracle_pb(z, exact=exact)
    s.SetParameters(z["uR"], z["uI"], float(z["phiR"]), float(z["phiI"]))
    s.SetWalkers(soa(cfgs))
    fwd = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    tol = 1e-12 if precision == "fp64" else 1e-5
    for c, R in enumerate(cfgs):
        r = o.eval(z["uR"], z["uI"], R, adjoint=True)
        scale_lnpsi = max(abs(r["lnpsi"]), np.abs(z["uR"]).max() * len(R))
        assert abs(fwd["lnpsi"][c] - r["lnpsi"]) < tol * scale_lnpsi
        assert relmax(fwd["O"][c], r["O"]) < tol
        scaleE = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(fwd["eloc"][c] - r["eloc"]).max() < tol * scaleE
        assert np.abs(fwd["other"][c] - r["other"]).max() < tol * scaleE
        scaled = max(np.abs(r["dE"]).max(), 1.0)
        assert np.abs(dE[c] - r["dE"]).max() < tol * scaled
        if precision == "fp64" and not exact:
            # the reference's own evaluation of the same configuration
            assert relmax(fwd["lnpsi"][c], z["ref_lnpsi"][c]) < RTOL_REF
            assert relmax(fwd["O"][c], z["ref_O"][c]) < RTOL_REF
            sE = max(abs(z["ref_other"][c][0]), abs(z["ref_other"][c][1]), 1.0)
            assert abs(fwd["eloc"][c][0] - z["ref_ER"][c]) < RTOL_REF * sE
            assert abs(fwd["eloc"][c][1] - z["ref_EI"][c]) < RTOL_REF * sE
            assert fwd["other"][c][1] == z["ref_other"][c][1]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["d1_n20_p10", "d2_n64_k20", "d3_n64_p10"])
def test_pb_sampler_follows_oracle_chain(name, precision):
    """Metropolis moves with mirrored distances (NUBosonsBulkPB.cpp:684-740) on
    32 lanes per walker, whose padded register slots hold phantoms: FP64 the
    oracle's chain; FP32 the same moves on at least 90 % of the walkers,
    acceptance within 1 %."""
    z = np.load(os.path.join(GOLD, "pb_eval_%s.npz" % name))
    dim, n, L = int(z["dim"]), int(z["n"]), float(z["L"])
    nw, moves, step = 32, 2 * n, 0.4 if dim > 1 else 1.0
    rng = np.random.default_rng(7 + dim)
    R0 = np.concatenate([soa(z["cfgs"])] * (nw // len(z["cfgs"]) + 1))[:nw]
    R0 = R0 + rng.normal(0, 0.02, size=R0.shape)
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    if precision == "mixed":
        R0 = R0.astype(np.float32).astype(np.float64)
    uR = 0.5 * np.asarray(z["uR"])
    s = gpu_pb(z, nw, precision)
    s.SetParameters(uR, z["uI"])
    s.SetWalkers(R0)
    acc = s.DoMetropolisSteps(moves, step, seed=55, pass_id=9)
    Rg = s.GetWalkers()
    s.close()
    o = oracle_pb(z)
    Ro = np.ascontiguousarray(R0.copy())
    acc_o = o.sample(uR, Ro, moves, step, seed=55, pass_id=9)
    assert 0.05 < acc_o / (moves * nw) < 0.98
    if precision == "fp64":
        assert acc == acc_o
        assert np.abs(Rg - Ro).max() < 1e-9
    else:
        d = np.abs(Rg - Ro).reshape(nw, -1).max(1)
        assert (d < 1e-4).mean() >= 0.9, d
        assert abs(acc - acc_o) <= 0.01 * acc_o, (acc, acc_o)


@pytest.mark.parametrize("ode,exact", [(2, False), (3, False), (2, True), (3, True)])
def test_pb_tdvp_step_matches_oracle_fp64(ode, exact):
    """One RK4 step of the mirrored-distance system, direct (ODE_SOLVER_TYPE 2)
    and on stored samples (3), in both forms of the derivative terms: sampling,
    evaluation, reduction, solve, update."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "pb_eval_d3_n64_p10.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    nw, moves, step, dt, seed, pass0 = 64, n, 0.3, 1e-3, 13, 2
    rng = np.random.default_rng(4)
    R0 = np.concatenate([soa(z["cfgs"])] * 4)[:nw] + rng.normal(0, 0.02, size=(nw, dim, n))
    R0 = np.vectorize(lambda v: orc.lib().orc_nic_coord(v, L))(R0)
    uR, uI = 0.5 * np.asarray(z["uR"]), np.asarray(z["uI"])
    s = gpu_pb(z, nw, "fp64", hbar2_2m=0.09, exact=exact)
    s.SetParameters(uR, uI, 0.0, 0.0)
    s.SetWalkers(R0)
    s.DoMetropolisSteps(0, step, seed, pass0)  # sets the Philox pass counter
    kw = dict(update_every=1, update_percent=25.0) if ode == 3 else {}
    td = T.TDVP(s, dt, moves, step, seed=seed, ode_solver=ode, **kw)
    td.step()
    gR, gI, gpR, gpI = s.GetParameters()

    o = oracle_pb(z, hbar2_2m=0.09, exact=exact)
    base = np.concatenate([uR, uI, [0.0, 0.0]])
    cur = base.copy()
    Ro = R0.copy()
    if ode == 3:
        o.sample(uR, Ro, moves, step, seed, pass0)
    ks = []
    for k in range(4):
        if ode == 3:
            out = o.stage(cur[:p], cur[p:2 * p], Ro, 0, step, seed, 0, threads=4, adjoint=False)
        else:
            out = o.stage(cur[:p], cur[p:2 * p], Ro, moves, step, seed, pass0 + k, threads=4, adjoint=False)
        m = orc.centred(out["O"], out["eloc"])
        dR, dI, pR, pI, _ = orc.solve_centred(m["O"], m["ER"], m["EI"], m["S"], m["cOER"], m["cOEI"])
        kv = np.concatenate([dR, dI, [pR, pI]])
        ks.append(kv)
        if k < 3:
            cur = base + kv * (dt / 2 if k < 2 else dt)
    new = orc.rk4_combine(base, ks, dt)
    assert np.abs(s.GetWalkers() - Ro).max() < 1e-9
    assert relmax(np.concatenate([gR, gI, [gpR, gpI]]), new) < 1e-9


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_pb_stored_eval_matches_direct_eval(precision, tol, exact):
    """The stored-sample columns (k_cs_store) of the mirrored distances give the
    direct evaluation at the stored parameters and at others."""
    z = np.load(os.path.join(GOLD, "pb_eval_d2_n64_k20.npz"))
    cfgs = soa(z["cfgs"])
    nw = 2 * len(cfgs)
    rng = np.random.default_rng(12)
    R = np.concatenate([cfgs] * 2) + rng.normal(0, 0.01, size=(nw,) + cfgs.shape[1:])
    s = gpu_pb(z, nw, precision, hbar2_2m=0.09, exact=exact)
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


def test_pb_pair_distribution_weight():
    """g(r) of NUBosonsBulkPB adds 1 per pair (NUBosonsBulkPB.cpp:602-612) where
    BosonsBulk adds D/(N-1): same walkers, same bins, ratio (N-1)/D."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "pb_eval_d3_n64_p10.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    R = soa(z["cfgs"])
    nw = len(R)
    pb = gpu_pb(z, nw, "fp64")
    bulk = T.BosonsBulk(dim, n, p, L, nw, system_params=z["sysp"], user_knots=z["knots"], precision="fp64")
    out = []
    for s in (pb, bulk):
        s.SetParameters(z["uR"], z["uI"])
        s.SetWalkers(R)
        out.append(s.CalculateAdditionalSystemProperties(100)["gr"])
    assert out[0].size == out[1].size == 100
    assert np.abs(out[0] - out[1] * (n - 1) / dim).max() <= 1e-12 * np.abs(out[0]).max()


@pytest.mark.parametrize("mode", ["fp64", "mixed", "mixed-scalar"])
@pytest.mark.parametrize("n", [150, 343, 600])
def test_pb_sampler_padded_slots_follow_oracle_chain(n, mode):
    """Mirrored-distance moves with register slots past N (150 particles on 32
    lanes in 8 slots, 343 in 11, 600 in 32 read from shared memory), uniform
    knots: FP64 the oracle's chain; FP32 packed (f32x2) and scalar samplers the
    same moves on at least 90 % of the walkers, acceptance within 1 %."""
    import tdvmc_gb300 as T
    dim, p, nw = 3, 10, 32
    L = (n / 0.5) ** (1.0 / dim)
    knots = np.linspace(0.0, L / 2, p)
    moves, step = 2 * n, 0.5
    rng = np.random.default_rng(n)
    uR, uI = 0.3 * rng.normal(size=p), 0.1 * rng.normal(size=p)
    R0 = rng.uniform(-L / 2, L / 2, size=(nw, dim, n))
    precision = "fp64" if mode == "fp64" else "mixed"
    if precision == "mixed":
        R0 = R0.astype(np.float32).astype(np.float64)
    if mode == "mixed-scalar":
        os.environ["TDVMC_SAMPLER"] = "scalar"
    try:
        s = T.NUBosonsBulkPB(dim, n, p, L, nw, user_knots=knots, system_params=(0.8, 1.0), precision=precision)
    finally:
        os.environ.pop("TDVMC_SAMPLER", None)
    s.SetParameters(uR, uI)
    s.SetWalkers(R0)
    acc = s.DoMetropolisSteps(moves, step, seed=31, pass_id=2)
    Rg = s.GetWalkers()
    s.close()
    o = orc.OracleSystem(dim, n, p, L, user_knots=knots, pot_kind=orc.POT_SQUARE, pot=(0.8, 1.0),
                         variant=orc.SYS_NU_PB)
    Ro = np.ascontiguousarray(R0.copy())
    acc_o = o.sample(uR, Ro, moves, step, seed=31, pass_id=2)
    assert 0.1 < acc_o / (moves * nw) < 0.95
    if precision == "fp64":
        assert acc == acc_o
        assert np.abs(Rg - Ro).max() < 1e-9
    else:
        d = np.abs(Rg - Ro).reshape(nw, -1).max(1)
        assert (d < 1e-4).mean() >= 0.9, d
        assert abs(acc - acc_o) <= 0.01 * acc_o, (acc, acc_o)


def test_pb_autotune_stays_on_its_kernels():
    """The autotuner on the mirrored-distance system: its kernels exist for 32
    lanes and histogram mode 0 only, so every other candidate is skipped; the
    walkers are restored and the results equal those of the default tiles."""
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "pb_eval_d3_n64_p10.npz"))
    nw = 1024
    R = np.concatenate([soa(z["cfgs"])] * (nw // len(z["cfgs"])))
    s = gpu_pb(z, nw, "mixed")
    s.SetParameters(z["uR"], z["uI"])
    s.SetWalkers(R.astype(np.float32).astype(np.float64))
    s.DoMetropolisSteps(64, 0.3, seed=1, pass_id=0)
    before = s.GetWalkers()
    ref = s.CalculateExpectationValues()
    dref = s.CalculateLocalEnergyAdjoint()
    tiles = s.Autotune(64, 0.3)
    assert tiles["sample_lanes"] == 32 and tiles["eval_lanes"] == 32
    assert np.array_equal(s.GetWalkers(), before)
    got = s.CalculateExpectationValues()
    for key in ("lnpsi", "O", "eloc", "other"):
        assert np.array_equal(got[key], ref[key]), key
    assert np.array_equal(s.CalculateLocalEnergyAdjoint(), dref)


@pytest.mark.parametrize("exact", [False, True])
def test_pb_mixed_tracks_fp64_at_the_benchmark_shape(exact):
    """3D N=343, rho=0.365, P=30 knots on [0, L/2] (the benchmark's shape), 16
    jittered-lattice walkers held in FP32: the mixed evaluation against the FP64
    evaluation of the same walkers within 1e-5 (ln psi, O_k, E_loc, the kinetic
    sums, dE/d alpha), in both forms of the derivative terms.  Every pair with
    r > L/2 is mirrored here (about half of them), including the pairs across
    the minimum-image wrap where the mirrored form's gradient changes sign."""
    import tdvmc_gb300 as T
    import bench as B
    nw = 16
    R = B.initial_walkers(nw, seed=77).astype(np.float32).astype(np.float64)
    knots = np.linspace(0.0, B.L / 2, B.P)
    uR, uI = B.initial_params()
    uI = 0.01 * np.random.default_rng(3).normal(size=B.P)
    out = {}
    for prec in ("fp64", "mixed"):
        s = T.NUBosonsBulkPB(B.DIM, B.N, B.P, B.L, nw, user_knots=knots, system_params=(1.0, 1.0),
                             hbar2_2m=B.HBAR2_2M, precision=prec, exact_derivatives=exact)
        s.SetParameters(uR, uI)
        s.SetWalkers(R)
        f = s.CalculateExpectationValues()
        f["dE"] = s.CalculateLocalEnergyAdjoint()
        out[prec] = f
        s.close()
    a, b = out["mixed"], out["fp64"]
    for c in range(nw):
        assert abs(a["lnpsi"][c] - b["lnpsi"][c]) < 1e-5 * max(abs(b["lnpsi"][c]), 1.0)
        assert relmax(a["O"][c], b["O"][c]) < 1e-5
        sc = max(np.abs(b["other"][c]).max(), 1.0)
        assert np.abs(a["eloc"][c] - b["eloc"][c]).max() < 1e-5 * sc
        assert np.abs(a["other"][c] - b["other"][c]).max() < 1e-5 * sc
        assert np.abs(a["dE"][c] - b["dE"][c]).max() < 1e-5 * max(np.abs(b["dE"][c]).max(), 1.0)


def test_pb_sampler_matches_reference_chain_mixed():
    """The mixed sampler's chain against the reference's own mt19937 chain for the
    mirrored-distance system (tests/golden/sample_pb_d3_n27.npz: block averages of
    the reference's DoMetropolisStep / UpdateExpectationValues on NUBosonsBulkPB,
    3D N=27, knots to L/2): O_k within 4 sigma, acceptance within 3 sigma, E^I
    within 3 sigma, E^R within 4 sigma (its local energy is heavy-tailed: the FP64
    oracle's chain lands 2.2 sigma from the reference's on the same seeds)."""
    z = np.load(os.path.join(GOLD, "sample_pb_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    blocks = z["blocks"]
    ref_mean = blocks.mean(0)
    ref_err = blocks.std(0, ddof=1) / np.sqrt(len(blocks))
    import tdvmc_gb300 as T
    nw = 4096
    s = T.NUBosonsBulkPB(dim, n, p, L, nw, user_knots=z["knots"], system_params=z["sysp"], precision="mixed")
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
    assert dev[0] < 4 and dev[1] < 3, dev
    assert np.all(dev[2:] < 4), dev
    rate = acc / (nsamp * n * nw)
    assert abs(rate - ref_mean[0]) < 3 * ref_err[0] + 0.01


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim,n", [(1, 2), (3, 3), (2, 5), (3, 33), (3, 65)])
def test_pb_ragged_sizes_match_oracle(dim, n, precision):
    """Particle counts that leave the 32-lane groups of the mirrored-distance kernels
    partly empty (N = 2, 3, 5), one slot and one particle more (33), two slots and one
    more (65): evaluation, adjoint and a sampling pass against the oracle (FP64 1e-12
    and the same chain; mixed 1e-5 on FP32-held walkers)."""
    import tdvmc_gb300 as T
    p, nw = 8, 5
    L = (n / 0.4) ** (1.0 / dim)
    knots = np.linspace(0.0, L / 2, p)
    rng = np.random.default_rng(10 * n + dim)
    uR, uI = 0.3 * rng.normal(size=p), 0.1 * rng.normal(size=p)
    R = rng.uniform(-L / 2, L / 2, size=(nw, dim, n))
    if precision == "mixed":
        R = R.astype(np.float32).astype(np.float64)
    s = T.NUBosonsBulkPB(dim, n, p, L, nw, user_knots=knots, system_params=(0.5, 1.0), precision=precision)
    s.SetParameters(uR, uI)
    s.SetWalkers(R)
    f = s.CalculateExpectationValues()
    dE = s.CalculateLocalEnergyAdjoint()
    o = orc.OracleSystem(dim, n, p, L, user_knots=knots, pot_kind=orc.POT_SQUARE, pot=(0.5, 1.0),
                         variant=orc.SYS_NU_PB)
    tol = 1e-12 if precision == "fp64" else 1e-5
    for w in range(nw):
        r = o.eval(uR, uI, R[w].T, adjoint=True)
        assert abs(f["lnpsi"][w] - r["lnpsi"]) < tol * max(abs(r["lnpsi"]), np.abs(uR).max() * n)
        assert relmax(f["O"][w], r["O"]) < tol
        sc = max(np.abs(r["other"]).max(), 1.0)
        assert np.abs(f["eloc"][w] - r["eloc"]).max() < tol * sc
        assert np.abs(f["other"][w] - r["other"]).max() < tol * sc
        assert np.abs(dE[w] - r["dE"]).max() < tol * max(np.abs(r["dE"]).max(), 1.0)
    if precision == "fp64":
        acc = s.DoMetropolisSteps(4 * n, 0.5, seed=8, pass_id=3)
        Ro = np.ascontiguousarray(R.copy())
        acc_o = o.sample(uR, Ro, 4 * n, 0.5, seed=8, pass_id=3)
        assert acc == acc_o
        assert np.abs(s.GetWalkers() - Ro).max() < 1e-9
