"""GPU: pair distribution g(r) and structure factor S(k) against the reference.

Fixtures tests/golden/obs_*.npz hold the reference's own
CalculateAdditionalSystemProperties (BosonsBulk.cpp:474-520) of fixed
configurations; the GPU evaluates the same configurations as walkers and
averages them, as the reference averages its samples.

Tolerances: FP64 relative 1e-12 (g(r)) and 1e-11 (S(k)), scaled by the largest
value.  Mixed: FP32 distances can move a pair across a bin edge, so g(r) is
compared as pair counts per bin (at most 4 pairs per configuration may move)
and S(k) at 1e-4 relative to the largest value.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

pytestmark = pytest.mark.gpu


def shell_volumes(dim, rmax, bins):
    h = rmax / bins
    cnt = int((rmax - 0.0) / h)
    i = np.arange(1, cnt + 1)
    if dim == 1:
        return np.full(cnt, h)
    v = 4.0 * np.pi * (h * i) ** 3 / 3.0 if dim == 3 else np.pi * (h * i) ** 2
    return np.diff(np.concatenate([[0.0], v]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["d1_n20", "d2_n64", "d3_n343"])
def test_observables_match_reference(name, precision):
    import tdvmc_gb300 as T
    z = np.load(os.path.join(GOLD, "obs_%s.npz" % name))
    dim, n, p, L = int(z["dim"]), int(z["n"]), int(z["p"]), float(z["L"])
    cfgs = np.ascontiguousarray(np.transpose(z["cfgs"], (0, 2, 1)))
    nw = len(cfgs)
    s = T.BosonsBulk(dim, n, p, L, nw, precision=precision)
    s.SetWalkers(cfgs)
    out = s.CalculateAdditionalSystemProperties(int(z["gr_bins"]), z["shell_off"], z["kvec"])
    ref_gr = z["ref_gr"].mean(0)
    ref_sk = z["ref_sk"].mean(0)
    assert out["gr"].shape == ref_gr.shape and out["sk"].shape == ref_sk.shape
    if precision == "fp64":
        assert np.abs(out["gr"] - ref_gr).max() <= 1e-12 * np.abs(ref_gr).max()
        assert np.abs(out["sk"] - ref_sk).max() <= 1e-11 * np.abs(ref_sk).max()
    else:
        vol = shell_volumes(dim, L / 2, int(z["gr_bins"]))
        to_pairs = vol * nw * (n - 1) / dim
        moved = np.abs((out["gr"] - ref_gr) * to_pairs).sum()
        assert moved <= 4 * 2 * nw + 1e-6, moved
        assert np.abs(out["sk"] - ref_sk).max() <= 1e-4 * np.abs(ref_sk).max()


def test_observables_argument_checks():
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    z = np.load(os.path.join(GOLD, "obs_d3_n343.npz"))
    s = T.BosonsBulk(3, int(z["n"]), int(z["p"]), float(z["L"]), 2, precision="fp64")
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateAdditionalSystemProperties(50)
    assert e.value.code == N.ERR_STATE  # no walkers yet
    s.SetWalkers(np.ascontiguousarray(np.transpose(z["cfgs"][:2], (0, 2, 1))))
    g = s.CalculateAdditionalSystemProperties(50)  # g(r) only
    assert g["gr"].size == 50 and g["sk"].size == 0
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateAdditionalSystemProperties(0)
    assert e.value.code == N.ERR_ARG
    bad = np.array([0, 3, 2], dtype=np.int32)  # decreasing offsets
    with pytest.raises(N.TdvmcError) as e:
        s.CalculateAdditionalSystemProperties(50, bad, z["kvec"][:3])
    assert e.value.code == N.ERR_ARG
