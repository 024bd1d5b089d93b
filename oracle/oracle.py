"""ctypes front end of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module.  The product package ``tdvmc_gb300`` never
does: its compute runs in the CUDA library and fails loudly without it.

The C sources (``oracle/tdvmc_oracle.c``) restate the reference algorithm of
mathiasgartner/TDVMC (``PhysicalSystems::BosonsBulk`` and the TDVP driver in
``src/TDVMC.cpp``); their parity with the reference is pinned by
``tests/test_oracle_golden.py`` against fixtures produced by the reference
itself (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtdvmc_oracle.so")
SRC = os.path.join(HERE, "tdvmc_oracle.c")

POT_NONE, POT_SQUARE, POT_GAUSS, POT_LJ = 0, 1, 2, 3
# BosonsBulk, NUBosonsBulkPB, NUBosonsBulkPB with exact derivatives (tdvmc_oracle.h)
SYS_BOSONS_BULK, SYS_NU_PB, SYS_NU_PB_EXACT = 0, 1, 2

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build_oracle(force: bool = False) -> str:
    """Compile the oracle shared library with gcc (seconds)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "tdvmc_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-pthread",
                           "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_int,
                                 C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_set_variant.argtypes = [C.c_void_p, C.c_int]
        L.orc_num_knots.argtypes = [C.c_void_p]
        L.orc_num_splines.argtypes = [C.c_void_p]
        L.orc_rmax.argtypes = [C.c_void_p]
        L.orc_rmax.restype = C.c_double
        L.orc_knots.argtypes = [C.c_void_p, _dp]
        L.orc_abs_weights.argtypes = [C.c_void_p, _dp]
        L.orc_local_weights.argtypes = [C.c_void_p, _dp]
        L.orc_nic_coord.argtypes = [C.c_double, C.c_double]
        L.orc_nic_coord.restype = C.c_double
        L.orc_nic_disp.argtypes = [_dp, _dp, C.c_int, C.c_double, _dp]
        L.orc_nic_disp.restype = C.c_double
        L.orc_eval.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_void_p]
        L.orc_move_delta.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp]
        L.orc_move_delta.restype = C.c_double
        L.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_sample.argtypes = [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, C.c_int64, C.c_int,
                                 C.c_double, C.c_uint64, C.c_uint32]
        L.orc_sample.restype = C.c_int64
        L.orc_stage_threads.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int64, C.c_int, C.c_double,
                                        C.c_uint64, C.c_uint32, C.c_int, _dp, _dp, _dp, _dp, C.c_void_p]
        L.orc_stage_threads.restype = C.c_int64
        L.orc_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_double, C.c_double,
                                _dp, _dp, _dp, _dp, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_solve.restype = C.c_int
        L.orc_solve_centred.argtypes = L.orc_solve.argtypes
        L.orc_solve_centred.restype = C.c_int
        L.orc_observables.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_void_p, _dp, _dp, _dp]
        L.orc_observables.restype = C.c_int
        L.orc_drop_create.restype = C.c_void_p
        L.orc_drop_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_drop_free.argtypes = [C.c_void_p]
        L.orc_drop_eval.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_void_p]
        L.orc_drop_sample.argtypes = [C.c_void_p, _dp, _dp, C.c_int64, C.c_int64, C.c_int, C.c_double,
                                      C.c_uint64, C.c_uint32]
        L.orc_drop_sample.restype = C.c_int64
        _lib = L
    return _lib


def nic_disp(ri, rj, L):
    ri = np.ascontiguousarray(ri, dtype=np.float64)
    rj = np.ascontiguousarray(rj, dtype=np.float64)
    d = np.zeros_like(ri)
    r = lib().orc_nic_disp(ri, rj, ri.size, float(L), d)
    return r, d


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return [int(o[i]) for i in range(4)]


class OracleSystem:
    """One periodic pair-spline Bose system (BosonsBulk semantics) in FP64."""

    def __init__(self, dim, n, p, L, user_knots=None, pot_kind=POT_SQUARE, pot=(0.5, 2.0),
                 time=0.0, hbar2_2m=1.0, variant=SYS_BOSONS_BULK):
        self.dim, self.n, self.p, self.L = int(dim), int(n), int(p), float(L)
        uk = None if user_knots is None else np.ascontiguousarray(user_knots, dtype=np.float64)
        pv = np.ascontiguousarray(pot, dtype=np.float64)
        self._uk, self._pv = uk, pv
        h = lib().orc_create(self.dim, self.n, self.p, self.L,
                             None if uk is None else uk.ctypes.data, 0 if uk is None else uk.size,
                             int(pot_kind), pv.ctypes.data, pv.size, float(time), float(hbar2_2m))
        if not h:
            raise ValueError("oracle rejected the system (parameter count or sizes)")
        self.h = h
        if variant != SYS_BOSONS_BULK:
            lib().orc_set_variant(h, int(variant))
        self.nk = lib().orc_num_knots(h)
        self.ns = lib().orc_num_splines(h)
        self.rmax = lib().orc_rmax(h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def knots(self):
        out = np.zeros(self.nk)
        lib().orc_knots(self.h, out)
        return out

    def abs_weights(self):
        out = np.zeros(self.ns * 16)
        lib().orc_abs_weights(self.h, out)
        return out.reshape(self.ns, 4, 4)

    def local_weights(self):
        out = np.zeros(self.nk * 16)
        lib().orc_local_weights(self.h, out)
        return out.reshape(self.nk, 4, 4)

    def eval(self, uR, uI, R, adjoint=False):
        """R: (n, dim) particle-major.  Returns dict of FP64 results."""
        uR = np.ascontiguousarray(uR, dtype=np.float64)
        uI = np.ascontiguousarray(uI, dtype=np.float64)
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(-1)
        lnpsi = np.zeros(1)
        O = np.zeros(self.p)
        eloc = np.zeros(2)
        other = np.zeros(7)
        dE = np.zeros(2 * self.p) if adjoint else None
        lib().orc_eval(self.h, uR, uI, R, lnpsi, O, eloc, other, None if dE is None else dE.ctypes.data)
        res = dict(lnpsi=lnpsi[0], O=O, eloc=eloc, other=other)
        if adjoint:
            res["dE"] = dE.reshape(self.p, 2)
        return res

    def observables(self, R, gr_bins, shell_off, kvec):
        """g(r) and S(k) of one configuration R (n, dim).  Returns (gr, sk)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(-1)
        off = np.ascontiguousarray(shell_off, dtype=np.int32)
        kv = np.ascontiguousarray(kvec, dtype=np.float64).reshape(-1)
        gr = np.zeros(int(gr_bins) + 1)
        sk = np.zeros(max(len(off) - 1, 1))
        cnt = lib().orc_observables(self.h, R, int(gr_bins), len(off) - 1, off.ctypes.data, kv, gr, sk)
        return gr[:cnt], sk[:len(off) - 1]

    def move_delta(self, uR, R, p, newpos):
        return lib().orc_move_delta(self.h, np.ascontiguousarray(uR, dtype=np.float64),
                                    np.ascontiguousarray(R, dtype=np.float64).reshape(-1), int(p),
                                    np.ascontiguousarray(newpos, dtype=np.float64))

    def sample(self, uR, Rsoa, moves, step, seed, pass_id, w0=0, nw=None):
        """In-place sampling of walkers stored SoA (nw, dim, n).  Returns accepted moves."""
        assert Rsoa.dtype == np.float64 and Rsoa.flags["C_CONTIGUOUS"]
        nwt = Rsoa.shape[0]
        nw = nwt - w0 if nw is None else nw
        return lib().orc_sample(self.h, np.ascontiguousarray(uR, dtype=np.float64), Rsoa, nwt, int(w0), int(nw),
                                int(moves), float(step), int(seed), int(pass_id) & 0xFFFFFFFF)

    def stage(self, uR, uI, Rsoa, moves, step, seed, pass_id, threads=1, adjoint=True):
        """Sampling pass plus per-walker evaluation (the CPU baseline workload)."""
        nw = Rsoa.shape[0]
        lnpsi = np.zeros(nw)
        O = np.zeros((nw, self.p))
        eloc = np.zeros((nw, 2))
        other = np.zeros((nw, 7))
        dE = np.zeros((nw, self.p, 2)) if adjoint else None
        acc = lib().orc_stage_threads(self.h, np.ascontiguousarray(uR, dtype=np.float64),
                                      np.ascontiguousarray(uI, dtype=np.float64), Rsoa, nw, int(moves),
                                      float(step), int(seed), int(pass_id) & 0xFFFFFFFF, int(threads),
                                      lnpsi, O, eloc, other, None if dE is None else dE.ctypes.data)
        out = dict(lnpsi=lnpsi, O=O, eloc=eloc, other=other, accepted=acc)
        if adjoint:
            out["dE"] = dE
        return out


class OracleDrop:
    """One trapped drop (open boundaries, pair spline + one-body Gaussian) in FP64.
    Parameter vectors have p + 1 entries (the pair spline, then alpha_p)."""

    def __init__(self, n, p, rmax, v0=1.0, sigma=0.5, omega=1.0, hbar2_2m=0.5):
        self.n, self.p = int(n), int(p)
        h = lib().orc_drop_create(self.n, self.p, float(rmax), float(v0), float(sigma), float(omega),
                                  float(hbar2_2m))
        if not h:
            raise ValueError("oracle rejected the drop")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_drop_free(self.h)
            self.h = None

    def eval(self, uR, uI, R, adjoint=False):
        """R: (n, 3) particle-major."""
        p1 = self.p + 1
        uR = np.ascontiguousarray(uR, dtype=np.float64)
        uI = np.ascontiguousarray(uI, dtype=np.float64)
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(-1)
        lnpsi, O, eloc, other = np.zeros(1), np.zeros(p1), np.zeros(2), np.zeros(7)
        dE = np.zeros(2 * p1) if adjoint else None
        lib().orc_drop_eval(self.h, uR, uI, R, lnpsi, O, eloc, other, None if dE is None else dE.ctypes.data)
        res = dict(lnpsi=lnpsi[0], O=O, eloc=eloc, other=other)
        if adjoint:
            res["dE"] = dE.reshape(p1, 2)
        return res

    def sample(self, uR, Rsoa, moves, step, seed, pass_id, walker0=0):
        """In-place moves of walkers stored SoA (nw, 3, n); Philox walker index walker0 + w."""
        assert Rsoa.dtype == np.float64 and Rsoa.flags["C_CONTIGUOUS"]
        return lib().orc_drop_sample(self.h, np.ascontiguousarray(uR, dtype=np.float64), Rsoa, Rsoa.shape[0],
                                     int(walker0), int(moves), float(step), int(seed), int(pass_id) & 0xFFFFFFFF)


def solve(O, ER, EI, OO, OER, OEI, imag=0, precond=0, solver=0):
    """SolveForParametersDot from raw moments.  Returns (uDotR, uDotI, phiDotR, phiDotI, rejected)."""
    P = len(O)
    uR = np.zeros(P)
    uI = np.zeros(P)
    pR = C.c_double(0.0)
    pI = C.c_double(0.0)
    bad = lib().orc_solve(P, int(imag), int(precond), int(solver), np.ascontiguousarray(O, dtype=np.float64),
                          float(ER), float(EI), np.ascontiguousarray(OO, dtype=np.float64).reshape(-1),
                          np.ascontiguousarray(OER, dtype=np.float64), np.ascontiguousarray(OEI, dtype=np.float64),
                          uR, uI, C.byref(pR), C.byref(pI))
    return uR, uI, pR.value, pI.value, bool(bad)


def solve_centred(O, ER, EI, S, covOER, covOEI, imag=0, precond=0, solver=0):
    """The solve from centred moments (S, cov(O,E^R), cov(O,E^I))."""
    P = len(O)
    uR = np.zeros(P)
    uI = np.zeros(P)
    pR = C.c_double(0.0)
    pI = C.c_double(0.0)
    bad = lib().orc_solve_centred(P, int(imag), int(precond), int(solver), np.ascontiguousarray(O, dtype=np.float64),
                                  float(ER), float(EI), np.ascontiguousarray(S, dtype=np.float64).reshape(-1),
                                  np.ascontiguousarray(covOER, dtype=np.float64),
                                  np.ascontiguousarray(covOEI, dtype=np.float64), uR, uI, C.byref(pR), C.byref(pI))
    return uR, uI, pR.value, pI.value, bool(bad)


def moments(O, eloc):
    """Raw sample moments as accumulated in UpdateExpectationValues (TDVMC.cpp:1103-1108)."""
    O = np.asarray(O, dtype=np.float64)
    ER = eloc[:, 0]
    EI = eloc[:, 1]
    n = O.shape[0]
    return dict(O=O.mean(0), ER=ER.mean(), EI=EI.mean(), OO=O.T @ O / n,
                OER=(O * ER[:, None]).mean(0), OEI=(O * EI[:, None]).mean(0))


def centred(O, eloc):
    """Two-pass centred moments: <O>, <E^R>, <E^I>, S, cov(O,E^R), cov(O,E^I)."""
    O = np.asarray(O, dtype=np.float64)
    E = np.asarray(eloc, dtype=np.float64)
    n = O.shape[0]
    Om = O.mean(0)
    Em = E.mean(0)
    Oc = O - Om
    Ec = E - Em
    return dict(O=Om, ER=Em[0], EI=Em[1], S=Oc.T @ Oc / n, cOER=Oc.T @ Ec[:, 0] / n, cOEI=Oc.T @ Ec[:, 1] / n)


def rk4_combine(u, k, dt):
    """Classical RK4 update of a parameter vector (TDVMC.cpp:2030-2033)."""
    k = [np.asarray(x, dtype=np.float64) for x in k]
    return np.asarray(u, dtype=np.float64) + ((k[0] + 2.0 * k[1] + 2.0 * k[2] + k[3]) / 6.0) * dt
