"""Pin the FP64 oracle against outputs of the reference itself.

The fixtures in tests/golden/ were produced by the unmodified reference
sources (oracle/ref/build_ref.sh + oracle/ref/harness.cpp, driven by
tests/golden/make_golden.py).

Tolerances: the reference evaluates its B-splines from closed-form monomial
weights in absolute r (SplineFactory.cpp:54-101).  Those weights carry
rounding errors of order 1e-9 in the spline values themselves, which
test_reference_weights_roundoff demonstrates through the partition of
unity; the oracle evaluates the same polynomials in local coordinates
(exact to ~1e-15).  Agreement with the reference is therefore asserted at
the level of the reference's own roundoff (RTOL_REF below), and every
quantity that does not involve the weights (minimum image, knots, solve) is
asserted at 1e-12 or tighter.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
RTOL_REF = 5e-9


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def load_system(z):
    kn = z["knots"] if z["knots"].size else None
    return orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), user_knots=kn,
                            pot_kind=orc.POT_SQUARE, pot=z["sysp"], time=float(z["time"]))


EVAL_FILES = sorted(glob.glob(os.path.join(GOLD, "eval_*.npz")))


def test_nic_known_answers():
    """The 48 minimum-image checks of src/test/Tests.h:76-156 (tolerance 1e-9 as there)."""
    z = np.load(os.path.join(GOLD, "nic_kat.npz"))
    assert len(z["inputs"]) == 48
    for inp, exp, ref in zip(z["inputs"], z["expected"], z["reference"]):
        L, dim = inp[0], int(inp[1])
        ri, rj = inp[2:2 + dim], inp[5:5 + dim]
        r, d = orc.nic_disp(ri, rj, L)
        assert abs(r - exp[0]) < 1e-9
        assert np.all(np.abs(d - exp[1:1 + dim]) < 1e-9)
        # and bit-for-bit the reference's own output on the same input
        assert r == ref[0]
        assert np.array_equal(d, ref[1:1 + dim])


@pytest.mark.parametrize("path", EVAL_FILES, ids=[os.path.basename(p)[5:-4] for p in EVAL_FILES])
def test_knots_and_weights(path):
    z = np.load(path)
    s = load_system(z)
    assert np.array_equal(s.knots(), z["ref_nodes"])
    W = s.abs_weights().reshape(-1, 4)
    RW = z["ref_weights"].reshape(-1, 4)
    scale = np.abs(RW).max(1, keepdims=True)
    assert (np.abs(W - RW) / scale).max() < 1e-12


@pytest.mark.parametrize("path", EVAL_FILES, ids=[os.path.basename(p)[5:-4] for p in EVAL_FILES])
def test_reference_weights_roundoff(path):
    """Partition of unity: the oracle's local pieces are exact to 1e-14; the
    reference's closed-form weights are not, which bounds parity with it."""
    z = np.load(path)
    s = load_system(z)
    kn = s.knots()
    loc = s.local_weights()
    W = z["ref_weights"].reshape(-1, 4, 4).astype(np.longdouble)
    rng = np.random.default_rng(1)
    worst_o, worst_r = 0.0, 0.0
    for r in rng.uniform(1e-6, s.rmax, 2000):
        b = np.searchsorted(kn, r, side="left") - 1
        t = (r - kn[b]) / (kn[b + 1] - kn[b])
        so = sum(np.polyval(loc[b, q][::-1], t) for q in range(4))
        rl = np.longdouble(r)
        sr = sum(W[b - q, q, 0] + W[b - q, q, 1] * rl + W[b - q, q, 2] * rl ** 2 + W[b - q, q, 3] * rl ** 3
                 for q in range(4))
        worst_o = max(worst_o, abs(so - 1.0))
        worst_r = max(worst_r, abs(float(sr) - 1.0))
    assert worst_o < 1e-14
    assert worst_r < RTOL_REF


@pytest.mark.parametrize("path", EVAL_FILES, ids=[os.path.basename(p)[5:-4] for p in EVAL_FILES])
def test_eval_matches_reference(path):
    """ln psi, O_k, E_loc and the kinetic partial sums on fixed configurations
    (BosonsBulk.cpp:179-218, 220-336, 349-458, 522-545)."""
    z = np.load(path)
    s = load_system(z)
    p = int(z["p"])
    for c, R in enumerate(z["cfgs"]):
        r = s.eval(z["uR"], z["uI"], R)
        assert relmax(r["lnpsi"], z["ref_lnpsi"][c]) < RTOL_REF
        assert relmax(r["O"], z["ref_O"][c]) < RTOL_REF
        scaleE = max(abs(z["ref_other"][c][0]), abs(z["ref_other"][c][1]), 1.0)
        assert abs(r["eloc"][0] - z["ref_ER"][c]) < RTOL_REF * scaleE
        assert abs(r["eloc"][1] - z["ref_EI"][c]) < RTOL_REF * scaleE
        # other: kineticR, V_int (reference slots 0,1) and the partial sums (slots 4..8)
        assert abs(r["other"][0] - z["ref_other"][c][0]) < RTOL_REF * scaleE
        assert r["other"][1] == z["ref_other"][c][1]
        assert relmax(r["other"][2:7], z["ref_other"][c][4:9]) < RTOL_REF
        # exponent slot and wf slot of the reference's other-values
        assert relmax(r["lnpsi"], z["ref_other"][c][3]) < RTOL_REF
        assert relmax(np.exp(r["lnpsi"] + float(z["phiR"])), z["ref_wf"][c]) < RTOL_REF * max(1.0, abs(r["lnpsi"]))
        assert r["O"].shape == (p,)


@pytest.mark.parametrize("path", EVAL_FILES, ids=[os.path.basename(p)[5:-4] for p in EVAL_FILES])
def test_lj_pair_sum_matches_reference(path):
    """Lennard-Jones pair sum (Potentials/LJ.cpp:16-22) over pairs inside the cut-off."""
    z = np.load(path)
    kn = z["knots"] if z["knots"].size else None
    s = orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), user_knots=kn,
                         pot_kind=orc.POT_LJ, pot=(1.0, 1.0), time=0.0)
    for c, R in enumerate(z["cfgs"]):
        r = s.eval(z["uR"], z["uI"], R)
        assert relmax(r["other"][1], z["ref_lj"][c]) < 1e-12


@pytest.mark.parametrize("path", EVAL_FILES, ids=[os.path.basename(p)[5:-4] for p in EVAL_FILES])
def test_move_matches_reference(path):
    """Exponent change of a single-particle move (BosonsBulk.cpp:553-657)."""
    z = np.load(path)
    s = load_system(z)
    for R, part, new, ref in zip(z["move_cfg"], z["move_part"], z["move_new"], z["ref_move"]):
        d = s.move_delta(z["uR"], R, int(part), new)
        scale = max(abs(ref[0]), abs(ref[1]), 1.0)
        assert abs(d - (ref[1] - ref[0])) < RTOL_REF * scale
        assert np.isclose(np.exp(2.0 * d), ref[2], rtol=1e-6)


def test_solve_matches_reference():
    """SolveForParametersDot, Cholesky and QR variants, real and imaginary time,
    with and without preconditioning (TDVMC.cpp:1713-1828)."""
    z = np.load(os.path.join(GOLD, "solve.npz"))
    for i in range(len(z["p"])):
        p = int(z["p"][i])
        uR, uI, pR, pI, bad = orc.solve(z["O_%d" % i], z["ER_%d" % i], z["EI_%d" % i], z["OO_%d" % i],
                                        z["OER_%d" % i], z["OEI_%d" % i], imag=int(z["imag"][i]),
                                        precond=int(z["pre"][i]), solver=int(z["solver"][i]))
        out = z["out_%d" % i]
        tol = 1e-12 if int(z["solver"][i]) == 0 else 1e-9
        assert relmax(uR, out[:p]) < tol
        assert relmax(uI, out[p:2 * p]) < tol
        assert abs(pR - out[2 * p]) < tol * max(1.0, abs(out[2 * p]))
        assert abs(pI - out[2 * p + 1]) < tol * max(1.0, abs(out[2 * p + 1]))
        assert bad == bool(out[2 * p + 2])


@pytest.mark.parametrize("name", ["d1_n20", "d2_n64", "d3_n343"])
def test_oracle_observables_match_reference(name):
    """g(r) and S(k) of fixed configurations against the reference's own
    CalculateAdditionalSystemProperties (tests/golden/obs_*.npz), 1e-13."""
    z = np.load(os.path.join(GOLD, "obs_%s.npz" % name))
    o = orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]))
    for c, R in enumerate(z["cfgs"]):
        gr, sk = o.observables(R, int(z["gr_bins"]), z["shell_off"], z["kvec"])
        assert gr.shape == z["ref_gr"][c].shape
        assert np.abs(gr - z["ref_gr"][c]).max() <= 1e-13 * np.abs(z["ref_gr"][c]).max()
        assert np.abs(sk - z["ref_sk"][c]).max() <= 1e-13 * np.abs(z["ref_sk"][c]).max()
    # the k grid of the structure factor is the shell norm
    kn = np.sqrt((z["kvec"][z["shell_off"][:-1]] ** 2).sum(1))
    assert np.allclose(kn, z["ref_kgrid"], rtol=1e-14)


PB_FILES = sorted(glob.glob(os.path.join(GOLD, "pb_eval_*.npz")))


def load_pb(z):
    return orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"]), user_knots=z["knots"],
                            pot_kind=orc.POT_SQUARE, pot=z["sysp"], time=float(z["time"]), variant=orc.SYS_NU_PB)


@pytest.mark.parametrize("path", PB_FILES, ids=[os.path.basename(p)[8:-4] for p in PB_FILES])
def test_pb_eval_matches_reference(path):
    """The mirrored-distance system (NUBosonsBulkPB.cpp): ln psi, O_k, E_loc,
    the potential and the kinetic partial sums on fixed configurations, against
    the reference's own evaluation at the tolerance of its spline weights."""
    z = np.load(path)
    s = load_pb(z)
    for c, R in enumerate(z["cfgs"]):
        r = s.eval(z["uR"], z["uI"], R)
        assert relmax(r["lnpsi"], z["ref_lnpsi"][c]) < RTOL_REF
        assert relmax(r["O"], z["ref_O"][c]) < RTOL_REF
        scaleE = max(abs(z["ref_other"][c][0]), abs(z["ref_other"][c][1]), 1.0)
        assert abs(r["eloc"][0] - z["ref_ER"][c]) < RTOL_REF * scaleE
        assert abs(r["eloc"][1] - z["ref_EI"][c]) < RTOL_REF * scaleE
        assert abs(r["other"][0] - z["ref_other"][c][0]) < RTOL_REF * scaleE
        assert r["other"][1] == z["ref_other"][c][1]
        assert relmax(r["other"][2:7], z["ref_other"][c][4:9]) < RTOL_REF


def test_pb_fixtures_exercise_the_mirror():
    """The 3D fixture holds pairs beyond r_max (entering at 2 r_max - r) and pairs
    whose mirrored distance lies inside the square well (a potential the
    BosonsBulk convention would not count)."""
    z = np.load(os.path.join(GOLD, "pb_eval_d3_n64_p10.npz"))
    L, rmax, a = float(z["L"]), float(z["knots"][-1]), float(z["sysp"][0])
    beyond = well = 0
    for R in z["cfgs"]:
        for i in range(len(R)):
            for j in range(i):
                r, _ = orc.nic_disp(R[i], R[j], L)
                beyond += r >= rmax
                well += r >= rmax and 2 * rmax - r < a
    assert beyond > 1000 and well > 0
    assert any(v > 0 for v in z["ref_other"][:, 1])


@pytest.mark.parametrize("path", PB_FILES, ids=[os.path.basename(p)[8:-4] for p in PB_FILES])
def test_pb_move_matches_reference(path):
    """Exponent change of a single-particle move of the mirrored-distance system
    (NUBosonsBulkPB.cpp:612-690: r < r_max for the old and the new position)."""
    z = np.load(path)
    s = load_pb(z)
    for R, part, new, ref in zip(z["move_cfg"], z["move_part"], z["move_new"], z["ref_move"]):
        d = s.move_delta(z["uR"], R, int(part), new)
        assert abs(d - (ref[1] - ref[0])) < RTOL_REF * max(abs(ref[0]), 1.0)


@pytest.mark.parametrize("path", PB_FILES, ids=[os.path.basename(p)[8:-4] for p in PB_FILES])
def test_pb_adjoint_is_the_derivative_of_the_local_energy(path):
    """dE_loc/d uR_k of the mirrored-distance system (the reference has no
    adjoint for it): E_loc is quadratic in uR, so central differences with step
    h are exact up to rounding; relative 1e-7 of the largest component."""
    z = np.load(path)
    s = load_pb(z)
    uR, uI = np.asarray(z["uR"], dtype=np.float64), np.asarray(z["uI"], dtype=np.float64)
    R = z["cfgs"][0]
    dE = s.eval(uR, uI, R, adjoint=True)["dE"].reshape(-1, 2)
    h = 1e-3
    fd = np.zeros_like(dE)
    for k in range(len(uR)):
        e = np.zeros_like(uR)
        e[k] = h
        fd[k] = (s.eval(uR + e, uI, R)["eloc"] - s.eval(uR - e, uI, R)["eloc"]) / (2 * h)
    assert np.abs(dE - fd).max() < 1e-7 * np.abs(fd).max()


def test_pb_exact_derivatives_are_those_of_ln_psi():
    """The exact form of the mirrored-distance system (ORC_SYS_NU_PB_EXACT): the
    kinetic sums sum_a |grad_a ln psi|^2 and sum_a lap_a ln psi (real part from
    uR, imaginary part from uI) agree with central differences of ln psi, on
    configurations with no pair within 2e-4 of r_max or of the minimum-image
    wrap |d_a| = L/2, where ln psi has kinks.  The reference's form (d / r', no
    sign flip) does not: its sums differ from the derivatives of its own ln psi."""
    z = np.load(os.path.join(GOLD, "pb_eval_d3_n64_p10.npz"))
    L, rmax = float(z["L"]), float(z["knots"][-1])
    uR, uI = np.asarray(z["uR"]), np.asarray(z["uI"])
    systems = {v: orc.OracleSystem(int(z["dim"]), int(z["n"]), int(z["p"]), L, user_knots=z["knots"],
                                   pot_kind=orc.POT_SQUARE, pot=z["sysp"], variant=v)
               for v in (orc.SYS_NU_PB, orc.SYS_NU_PB_EXACT)}
    h1, h2 = 1e-6, 1e-4
    checked = 0
    for R in z["cfgs"]:
        d = R[:, None, :] - R[None, :, :]
        d -= L * np.round(d / L)
        iu = np.triu_indices(len(R), 1)
        r = np.sqrt((d * d).sum(-1))[iu]
        if np.abs(r - rmax).min() < 2 * h2 or np.abs(np.abs(d[iu]) - L / 2).min() < 2 * h2:
            continue
        checked += 1
        for v, s in systems.items():
            res = s.eval(uR, uI, R)
            for u, kg, kl in ((uR, 2, 4), (uI, 3, 5)):
                f = lambda X: s.eval(u, uI, X)["lnpsi"]  # noqa: E731
                f0, g2, lap = f(R), 0.0, 0.0
                for a in range(len(R)):
                    for k in range(R.shape[1]):
                        e = np.zeros_like(R)
                        e[a, k] = h1
                        g2 += ((f(R + e) - f(R - e)) / (2 * h1)) ** 2
                        e[a, k] = h2
                        lap += (f(R + e) - 2 * f0 + f(R - e)) / h2 ** 2
                if v == orc.SYS_NU_PB_EXACT:
                    assert abs(res["other"][kg] - g2) < 1e-7 * abs(g2)
                    assert abs(res["other"][kl] - lap) < 1e-5 * max(abs(lap), abs(g2))
                else:
                    assert abs(res["other"][kg] - g2) > 1e-3 * abs(g2)
        if checked == 2:
            break
    assert checked >= 1
