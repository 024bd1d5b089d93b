"""GPU: the failure path of the bounded hardware waits, without a GPU fault.

The tensor-core contraction of S (k_gram_tf32, waits on tcgen05 commits) and
the stored-sample evaluation (k_cs_eval_st, waits on TMA bulk copies) bound
every wait in time.  TDVMC_TEST_WAIT_NS=0 at context creation makes the first
(status) wait of each completion give up at once; the kernel records the
failure, waits for the same completion with its drain limit (so no copy or
MMA is in flight when it moves on or exits) and reports NaN, which the step
returns as TDVMC_ERR_NONFINITE.  A context created afterwards without the
setting runs normally.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(nw=2048, n=64, p=12, L=6.0):
    import tdvmc_gb300 as T
    rng = np.random.default_rng(0)
    s = T.BosonsBulk(3, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09, precision="mixed")
    r = np.linspace(0, L / 2, p)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    s.SetParameters(uR, 0.01 * rng.normal(size=p))
    m = 4
    idx = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    R = idx[None] * (L / m) + (rng.uniform(size=(nw, n, 3)) - 0.5) * (L / m) / 10 - L / 2
    s.SetWalkers(np.ascontiguousarray(np.transpose(R, (0, 2, 1))))
    return s


@pytest.mark.parametrize("ode", [2, 3])
def test_wait_time_out_reports_nonfinite(ode):
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    os.environ["TDVMC_TEST_WAIT_NS"] = "0"
    try:
        s = _system()
    finally:
        os.environ.pop("TDVMC_TEST_WAIT_NS", None)
    td = T.TDVP(s, 1e-3, 64, 0.25, seed=3, ode_solver=ode, update_every=1 if ode == 3 else 0,
                update_percent=25.0)
    out = td.step(1)
    assert out["status"] == N.ERR_NONFINITE, out
    s.close()
    # the GPU and a fresh context are unaffected
    s2 = _system()
    td2 = T.TDVP(s2, 1e-3, 64, 0.25, seed=3, ode_solver=ode, update_every=1 if ode == 3 else 0,
                 update_percent=25.0)
    out2 = td2.step(1)
    assert out2["status"] == N.OK and np.isfinite(out2["energy"][0])
    s2.close()
