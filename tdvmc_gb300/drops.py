"""Batched trapped drops: many independent 3D systems of uneven particle number
on one GPU (the C ABI's ``tdvmc_drops_*`` entry points).

Each drop follows the reference's plugin interface for one system
(``IPhysicalSystem``, src/PhysicalSystems/IPhysicalSystem.h:98-122) with its
own parameters, walkers, walker statistics and TDVP solve; every kernel runs
once over all drops.  The wave function of a drop is the BosonsBulk pair
spline (without the minimum image, as the open-boundary cluster systems,
BosonCluster.cpp:14) plus a one-body Gaussian width: parameter vectors have
``p + 1`` entries, the last one multiplying sum_i |r_i|^2.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class TrappedDrops:
    """``n``: particles per drop (2..32); ``p``: pair-spline parameters; ``rmax``:
    spline range per drop (scalar or per drop); trap ``omega``; Gaussian pair
    repulsion ``v0``, ``sigma``; ``walkers``: walkers per drop."""

    def __init__(self, n, p, rmax, walkers, omega=1.0, v0=1.0, sigma=0.5, hbar2_2m=0.5, precision="fp64"):
        self.lib = N.load()
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.S = int(self.n.size)
        self.p, self.p1 = int(p), int(p) + 1
        self.nw = int(walkers)
        self.rmax = _f64(np.broadcast_to(np.asarray(rmax, dtype=np.float64), (self.S,)))
        d = N.DropsDesc()
        d.n_systems = self.S
        d.n = self.n.ctypes.data_as(C.POINTER(C.c_int32))
        d.p = self.p
        d.rmax = self.rmax.ctypes.data_as(C.POINTER(C.c_double))
        d.omega, d.v0, d.sigma, d.hbar2_2m = float(omega), float(v0), float(sigma), float(hbar2_2m)
        d.precision = {"fp64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]
        d.walkers_per_system = self.nw
        self.precision = precision
        h = C.c_void_p()
        N.check(self.lib.tdvmc_drops_create(C.byref(d), C.byref(h)), "tdvmc_drops_create")
        self.h = h
        self.offsets = np.concatenate([[0], np.cumsum(self.nw * 3 * self.n.astype(np.int64))])

    def close(self):
        if getattr(self, "h", None):
            self.lib.tdvmc_drops_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- state ----------------------------------------------------------------
    def SetParameters(self, uR, uI, phiR=None, phiI=None):
        """uR, uI: (S, p + 1); phiR, phiI: (S,) or None."""
        uR = _f64(uR).reshape(self.S, self.p1)
        uI = _f64(uI).reshape(self.S, self.p1)
        pR = None if phiR is None else _f64(np.broadcast_to(phiR, (self.S,)))
        pI = None if phiI is None else _f64(np.broadcast_to(phiI, (self.S,)))
        N.check(self.lib.tdvmc_drops_set_params(self.h, _ptr(uR), _ptr(uI), _ptr(pR), _ptr(pI)),
                "tdvmc_drops_set_params")

    def GetParameters(self):
        uR, uI = np.zeros((self.S, self.p1)), np.zeros((self.S, self.p1))
        pR, pI = np.zeros(self.S), np.zeros(self.S)
        N.check(self.lib.tdvmc_drops_get_params(self.h, _ptr(uR), _ptr(uI), _ptr(pR), _ptr(pI)),
                "tdvmc_drops_get_params")
        return uR, uI, pR, pI

    def SetWalkers(self, walkers):
        """walkers: list of S arrays (walkers, 3, n_s)."""
        flat = np.concatenate([_f64(w).reshape(-1) for w in walkers])
        assert flat.size == self.offsets[-1]
        N.check(self.lib.tdvmc_drops_set_walkers(self.h, _ptr(flat)), "tdvmc_drops_set_walkers")

    def GetWalkers(self):
        flat = np.zeros(int(self.offsets[-1]))
        N.check(self.lib.tdvmc_drops_get_walkers(self.h, _ptr(flat)), "tdvmc_drops_get_walkers")
        return [flat[self.offsets[s]:self.offsets[s + 1]].reshape(self.nw, 3, int(self.n[s])) for s in range(self.S)]

    # --- hot path ---------------------------------------------------------------
    def DoMetropolisSteps(self, moves_per_particle, mc_step, seed, pass_id):
        acc = C.c_int64()
        N.check(self.lib.tdvmc_drops_sample(self.h, int(moves_per_particle), float(mc_step), int(seed),
                                            int(pass_id) & 0xFFFFFFFF, C.byref(acc)), "tdvmc_drops_sample")
        return acc.value

    def CalculateExpectationValues(self, adjoint=False):
        S, W, p1 = self.S, self.nw, self.p1
        out = dict(lnpsi=np.zeros((S, W)), O=np.zeros((S, W, p1)), eloc=np.zeros((S, W, 2)),
                   other=np.zeros((S, W, 7)))
        dE = np.zeros((S, W, p1, 2)) if adjoint else None
        N.check(self.lib.tdvmc_drops_eval(self.h, _ptr(out["lnpsi"]), _ptr(out["O"]), _ptr(out["eloc"]),
                                          _ptr(out["other"]), _ptr(dE)), "tdvmc_drops_eval")
        if adjoint:
            out["dE"] = dE
        return out

    def ReduceStatistics(self):
        S, p1 = self.S, self.p1
        r = dict(O=np.zeros((S, p1)), energy=np.zeros((S, 2)), S=np.zeros((S, p1, p1)), cov_OER=np.zeros((S, p1)),
                 cov_OEI=np.zeros((S, p1)), dE=np.zeros((S, p1, 2)), accepted=np.zeros(S))
        N.check(self.lib.tdvmc_drops_reduce(self.h, _ptr(r["O"]), _ptr(r["energy"]), _ptr(r["S"]), _ptr(r["cov_OER"]),
                                            _ptr(r["cov_OEI"]), _ptr(r["dE"]), _ptr(r["accepted"])),
                "tdvmc_drops_reduce")
        return r

    def SolveForParametersDot(self, imaginary_time=0, precondition=0, lin_solver=0):
        S, p1 = self.S, self.p1
        uR, uI, pR, pI = np.zeros((S, p1)), np.zeros((S, p1)), np.zeros(S), np.zeros(S)
        st = np.zeros(S, dtype=np.int32)
        code = self.lib.tdvmc_drops_tdvp_rhs(self.h, int(imaginary_time), int(precondition), int(lin_solver),
                                             _ptr(uR), _ptr(uI), _ptr(pR), _ptr(pI), _ptr(st))
        if code not in (N.OK, N.ERR_NOT_PD, N.ERR_NONFINITE):
            N.check(code, "tdvmc_drops_tdvp_rhs")
        return uR, uI, pR, pI, st

    def Autotune(self, moves_per_particle, mc_step):
        N.check(self.lib.tdvmc_drops_autotune(self.h, int(moves_per_particle), float(mc_step)), "tdvmc_drops_autotune")
        return self.Tiles()

    def Tiles(self):
        a, b = C.c_int32(), C.c_int32()
        N.check(self.lib.tdvmc_drops_get_tiles(self.h, C.byref(a), C.byref(b)), "tdvmc_drops_get_tiles")
        return dict(sample_walkers_per_block=a.value, eval_walkers_per_block=b.value)

    def LaunchCount(self):
        return int(self.lib.tdvmc_drops_launch_count(self.h))


class DropsTDVP:
    """TDVP steps of every drop (ODE_SOLVER_TYPE 2 = RK4 or 0 = Euler);
    ``sweeps``: Metropolis moves per particle of each sampling pass."""

    def __init__(self, drops: TrappedDrops, dt, sweeps, mc_step, seed=1, imaginary_time=0, ode_solver=2,
                 lin_solver=0, precondition=0, normalize_wf=0, use_adjoint=0):
        self.d = drops
        o = N.StepOpts()
        o.dt = float(dt)
        o.imaginary_time = int(imaginary_time)
        o.ode_solver = int(ode_solver)
        o.lin_solver = int(lin_solver)
        o.precondition = int(precondition)
        o.normalize_wf = int(normalize_wf)
        o.moves_per_stage = int(sweeps)
        o.mc_step = float(mc_step)
        o.seed = int(seed)
        o.use_adjoint = int(use_adjoint)
        o.update_every = 0
        o.update_percent = 100.0
        self.opts = o

    def step(self, nsteps=1):
        S = self.d.S
        energy = np.zeros((S, 2))
        st = np.zeros(S, dtype=np.int32)
        code = self.d.lib.tdvmc_drops_run_steps(self.d.h, C.byref(self.opts), int(nsteps), _ptr(energy), _ptr(st))
        if code not in (N.OK, N.ERR_NOT_PD, N.ERR_NONFINITE):
            N.check(code, "tdvmc_drops_run_steps")
        return dict(energy=energy, status=st, code=code)

    def time_steps(self, nsteps):
        ms = C.c_float()
        N.check(self.d.lib.tdvmc_drops_time_steps(self.d.h, C.byref(self.opts), int(nsteps), C.byref(ms)),
                "tdvmc_drops_time_steps")
        return ms.value

    def profile_stage(self):
        ms = (C.c_float * 16)()
        names = (C.c_char_p * 16)()
        cnt = C.c_int32()
        N.check(self.d.lib.tdvmc_drops_profile_stage(self.d.h, C.byref(self.opts), ms, names, C.byref(cnt)),
                "tdvmc_drops_profile_stage")
        return [(names[i].decode(), ms[i]) for i in range(cnt.value)]
