"""The tensor-core Gram contraction S = Oc^T Oc / N_w (3xTF32, FP32 accumulate)
against the FP64 contraction of the same per-walker O_k.

Tolerance: 3xTF32 keeps ~21 significant bits per product and FP32
accumulation over at most a few hundred walkers per CTA; S is compared
relative to its largest entry at 2e-6.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import sys, numpy as np
sys.path.insert(0, %r)
import tdvmc_gb300 as T
rng = np.random.default_rng(0)
out = []
for dim, n, p, L, nw in ((3, 64, 10, 4.0, 1000), (3, 64, 30, 4.0, 4099), (2, 40, 48, 9.0, 777), (3, 27, 100, 3.6, 2000)):
    R = rng.uniform(-L / 2, L / 2, size=(nw, dim, n))
    uR, uI = rng.normal(0, 0.2, p), rng.normal(0, 0.1, p)
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", precision="mixed")
    s.SetParameters(uR, uI)
    s.SetWalkers(R)
    f = s.CalculateExpectationValues()
    st = s.ReduceStatistics()
    O = f["O"]
    Oc = O - O.mean(0)
    S = Oc.T @ Oc / nw
    out.append(np.abs(st["S"] - S).max() / np.abs(S).max())
    assert np.allclose(st["S"], st["S"].T, rtol=0, atol=1e-12 * np.abs(S).max())
print("ERR", " ".join("%%.3e" %% e for e in out))
'''


def run(env_gram):
    env = dict(os.environ)
    env["TDVMC_GRAM"] = env_gram
    r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("ERR")][0]
    return [float(x) for x in line.split()[1:]]


def test_tensor_core_gram_matches_fp64():
    errs = run("tc")
    assert max(errs) < 2e-6, errs


def test_fp64_gram_is_exact():
    errs = run("fp64")
    assert max(errs) < 1e-12, errs
