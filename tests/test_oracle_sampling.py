"""Oracle checks that have no fixed reference output: the adjoint against
central finite differences, the Philox generator against its published
known-answer vectors, and the oracle's Metropolis chain against the
reference's own chain (tests/golden/sample_d3_n27.npz) within 3 sigma."""
import os

import numpy as np

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _system(kind=orc.POT_LJ, dim=3, n=27, p=10, L=3.6):
    return orc.OracleSystem(dim, n, p, L, pot_kind=kind, pot=(1.0, 1.0), time=0.0, hbar2_2m=0.09)


def test_adjoint_matches_finite_differences():
    """dE_loc/d uR_k and, by holomorphy, dE_loc/d uI_k = i dE_loc/d uR_k."""
    rng = np.random.default_rng(3)
    for dim, n, p, L in ((3, 27, 10, 3.6), (2, 16, 8, 5.0), (1, 12, 6, 12.0)):
        s = _system(dim=dim, n=n, p=p, L=L)
        R = rng.uniform(-L / 2, L / 2, size=(n, dim))
        uR = rng.normal(0, 0.3, p)
        uI = rng.normal(0, 0.2, p)
        dE = s.eval(uR, uI, R, adjoint=True)["dE"]
        h = 1e-5

        def kin(a, b):
            # the pair potential does not depend on alpha; differencing the
            # kinetic part keeps the finite difference free of its roundoff
            r = s.eval(a, b, R)
            return np.array([r["other"][0], r["eloc"][1]])

        for k in range(p):
            e = np.zeros(p)
            e[k] = h
            fdR = (kin(uR + e, uI) - kin(uR - e, uI)) / (2 * h)
            fdI = (kin(uR, uI + e) - kin(uR, uI - e)) / (2 * h)
            scale = max(1.0, np.abs(dE).max())
            assert abs(fdR[0] - dE[k, 0]) < 1e-6 * scale
            assert abs(fdR[1] - dE[k, 1]) < 1e-6 * scale
            # d/d uI = i d/d uR  ->  (dE_R, dE_I)/duI = (-Im, Re)
            assert abs(fdI[0] + dE[k, 1]) < 1e-6 * scale
            assert abs(fdI[1] - dE[k, 0]) < 1e-6 * scale


def test_oracle_chain_matches_reference_chain():
    """Sampled averages of the oracle's Philox chain vs the reference's mt19937
    chain on the same system agree within 3 sigma (E_R, E_I, acceptance) and
    4 sigma per component of <O_k>."""
    z = np.load(os.path.join(GOLD, "sample_d3_n27.npz"))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    s = orc.OracleSystem(dim, n, p, L, pot_kind=orc.POT_SQUARE, pot=z["sysp"], time=0.0)
    blocks = z["blocks"]  # [acceptance, ER, EI, O[p], other[9]]
    ref_mean = blocks.mean(0)
    ref_err = blocks.std(0, ddof=1) / np.sqrt(len(blocks))

    nw, nsamp = 128, 40
    R = np.repeat(z["R0"].T[None, :, :], nw, axis=0).copy()
    rng = np.random.default_rng(5)
    R += rng.normal(0, 0.05, size=R.shape)
    step = float(z["step"])
    s.sample(z["uR"], R, 50 * n, step, seed=99, pass_id=0)
    acc_tot = 0
    rows = []
    for k in range(nsamp):
        out = s.stage(z["uR"], z["uI"], R, n, step, seed=99, pass_id=k + 1, threads=4, adjoint=False)
        acc_tot += out["accepted"]
        rows.append(np.concatenate([out["eloc"], out["O"]], axis=1))
    rows = np.array(rows)  # [sample, walker, 2+p]
    per_walker = rows.mean(0)
    mean = per_walker.mean(0)
    err = per_walker.std(0, ddof=1) / np.sqrt(nw)
    acc = acc_tot / (nsamp * n * nw)
    comb = np.sqrt(err ** 2 + ref_err[1:3 + p] ** 2)
    diff = np.abs(mean - ref_mean[1:3 + p])
    # an O_k without any pair in its support is exactly zero in both chains
    assert np.all(diff[comb == 0] == 0)
    dev = np.where(comb > 0, diff / np.where(comb > 0, comb, 1.0), 0.0)
    assert dev[0] < 3.0, dev
    assert dev[1] < 3.0, dev
    assert np.all(dev[2:] < 4.0), dev
    assert abs(acc - ref_mean[0]) < 3.0 * ref_err[0] + 0.01
