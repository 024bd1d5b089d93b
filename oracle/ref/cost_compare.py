"""Per-sample CPU cost of the reference and of the oracle port on the benchmark
system (3D, N = 343, density 0.365, P = 30, square-well pair potential of the
harness), one thread each.

TEST INFRASTRUCTURE ONLY: it times the reference harness built by
``oracle/ref/build_ref.sh`` (the unmodified reference sources) and the FP64
oracle, so that the CPU baseline of the benchmark (which runs the port on the
GPU host, where the reference is not built) can be related to the reference
itself.  One sample is what one RK stage does per walker: 2N single-particle
moves, then the local energy and the local operators.

    python oracle/ref/cost_compare.py [samples] [reference-root]   (default /root/reference)
"""
from __future__ import annotations

import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
N, P, RHO, STEP = 343, 30, 0.365, 0.17
L = (N / RHO) ** (1.0 / 3.0)
SYSP = (0.9, 1.0)


def fmt(a):
    return " ".join("%.17g" % v for v in np.asarray(a, dtype=np.float64).reshape(-1))


def start(rng):
    m = 7
    idx = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    return idx * (L / m) + (rng.uniform(size=(N, 3)) - 0.5) * (L / m) * 0.3 - L / 2


def reference_seconds(samples, uR, uI, R, ref_root):
    """Wall time of the harness's SAMPLE command (one chain: 2N moves, then one
    UpdateExpectationValues, per sample); the start-up is taken out by a run of
    one sample."""
    def run(ns):
        script = "SYSTEM 3 %d %d %.17g 0 2 %s 0\n" % (N, P, L, fmt(SYSP))
        script += "PARAMS %s %s 0 0\n" % (fmt(uR), fmt(uI))
        script += "SAMPLE 7 %.17g 0 %d %d 1\n%s\n" % (STEP, ns, 2 * N, fmt(R))
        t = time.perf_counter()
        subprocess.run([HARNESS, os.path.join(ref_root, "config", "")], input=script, capture_output=True, text=True, check=True)
        return time.perf_counter() - t
    return run(samples) - run(1), samples - 1


def port_seconds(samples, uR, uI, R):
    """Wall time of the oracle's stage (2N moves and one evaluation per walker,
    no adjoint), one thread, ``samples`` walkers."""
    o = orc.OracleSystem(3, N, P, L, pot_kind=orc.POT_SQUARE, pot=SYSP)
    Rs = np.ascontiguousarray(np.repeat(R.T[None], samples, axis=0))
    t = time.perf_counter()
    o.stage(uR, uI, Rs, 2 * N, STEP, 7, 0, threads=1, adjoint=False)
    return time.perf_counter() - t, samples


def main():
    samples = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    ref_root = sys.argv[2] if len(sys.argv) > 2 else "/root/reference"
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: oracle/ref/build_ref.sh")
    rng = np.random.default_rng(3)
    r = np.linspace(0.0, L / 2, P)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    uI = 0.01 * rng.normal(size=P)
    R = start(rng)
    tr, nr = reference_seconds(samples, uR, uI, R, ref_root)
    tp, npt = port_seconds(samples, uR, uI, R)
    print("reference: %.2f ms per sample (%d samples, %.2f s)" % (1e3 * tr / nr, nr, tr))
    print("port:      %.2f ms per sample (%d samples, %.2f s)" % (1e3 * tp / npt, npt, tp))
    print("port / reference: %.2f" % ((tp / npt) / (tr / nr)))


if __name__ == "__main__":
    main()
