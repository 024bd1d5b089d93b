"""Batched GPU sibling of the reference's physics plugin and TDVP driver step.

``BosonsBulk`` mirrors ``PhysicalSystems::BosonsBulk``
(src/PhysicalSystems/BosonsBulk.{h,cpp}) behind the ``IPhysicalSystem``
method names (src/PhysicalSystems/IPhysicalSystem.h:98-122), evaluated for
all walkers at once through the C ABI of include/tdvmc_gpu.h.  Where the
reference works on one configuration ``R`` (N x DIM), these methods work on
the walker array ``R[w, d, i]`` held on the device.

``TDVP`` wraps the driver step: sampling (DoMetropolisStep /
UpdateExpectationValues, TDVMC.cpp:858-1150), the walker reduction
(ParallelUpdateExpectationValues, 1152-1220), SolveForParametersDot
(1713-1828) and the Euler / RK4 integrators (1834-1858, 1969-2035).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

_POT = {"none": N.POT_NONE, "square": N.POT_SQUARE, "gauss": N.POT_GAUSS, "lj": N.POT_LJ}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class BosonsBulk:
    """Periodic Bose system with a cubic-B-spline pair Jastrow, batched over walkers.

    Parameters follow the reference's globals: ``dim`` (DIM), ``n`` (N),
    ``n_param`` (N_PARAM), ``box_length`` (LBOX), ``system_params``
    (SYSTEM_PARAMS: [a, b] or [a, b, t_quench, a', b']), ``user_knots``
    (NURBS_GRID with USE_NURBS=1), ``hbar2_2m`` (HBAR2_2M).
    """

    SYSTEM_TYPE = N.SYS_BOSONS_BULK

    def __init__(self, dim, n, n_param, box_length, n_walkers, system_params=(0.5, 2.0), potential="square",
                 user_knots=None, hbar2_2m=1.0, precision="fp64"):
        self.lib = N.load()
        self.dim, self.n, self.p, self.L, self.nw = int(dim), int(n), int(n_param), float(box_length), int(n_walkers)
        d = N.SystemDesc()
        d.dim, d.n, d.p = self.dim, self.n, self.p
        self._knots = None if user_knots is None else _f64(user_knots)
        d.n_user_knots = 0 if self._knots is None else self._knots.size
        d.user_knots = (C.POINTER(C.c_double)() if self._knots is None
                        else self._knots.ctypes.data_as(C.POINTER(C.c_double)))
        d.box_length = self.L
        d.pot_kind = _POT[potential] if isinstance(potential, str) else int(potential)
        sp = list(system_params)[:5]
        d.n_pot = len(sp)
        for i, v in enumerate(sp):
            d.pot[i] = float(v)
        d.hbar2_2m = float(hbar2_2m)
        d.precision = {"fp64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]
        d.n_walkers = self.nw
        d.system_type = self.SYSTEM_TYPE
        self.precision = precision
        h = C.c_void_p()
        N.check(self.lib.tdvmc_create(C.byref(d), C.byref(h)), "tdvmc_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.tdvmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- IPhysicalSystem-style state ---------------------------------------
    def InitSystem(self):
        """Knots, spline tables and boundary conditions are built at creation."""

    def SetTime(self, t):
        N.check(self.lib.tdvmc_set_time(self.h, float(t)), "tdvmc_set_time")

    def SetParameters(self, uR, uI, phiR=0.0, phiI=0.0):
        uR, uI = _f64(uR), _f64(uI)
        assert uR.size == self.p and uI.size == self.p
        N.check(self.lib.tdvmc_set_params(self.h, _ptr(uR), _ptr(uI), float(phiR), float(phiI)), "tdvmc_set_params")

    def GetParameters(self):
        uR = np.zeros(self.p)
        uI = np.zeros(self.p)
        pR, pI = C.c_double(), C.c_double()
        N.check(self.lib.tdvmc_get_params(self.h, _ptr(uR), _ptr(uI), C.byref(pR), C.byref(pI)), "tdvmc_get_params")
        return uR, uI, pR.value, pI.value

    def SetWalkers(self, R):
        """R: array (n_walkers, dim, n)."""
        R = _f64(R)
        assert R.shape == (self.nw, self.dim, self.n)
        N.check(self.lib.tdvmc_set_walkers(self.h, _ptr(R), self.nw), "tdvmc_set_walkers")

    def GetWalkers(self):
        R = np.zeros((self.nw, self.dim, self.n))
        N.check(self.lib.tdvmc_get_walkers(self.h, _ptr(R), self.nw), "tdvmc_get_walkers")
        return R

    # --- hot path ------------------------------------------------------------
    def DoMetropolisSteps(self, moves, mc_step, seed, pass_id):
        """`moves` single-particle moves per walker; returns accepted moves."""
        acc = C.c_int64()
        N.check(self.lib.tdvmc_sample(self.h, int(moves), float(mc_step), int(seed), int(pass_id) & 0xFFFFFFFF,
                                      C.byref(acc)), "tdvmc_sample")
        return acc.value

    def CalculateExpectationValues(self):
        """Forward pass: ln psi, O_k, (E^R, E^I) and the 7 kinetic/potential values per walker."""
        lnpsi = np.zeros(self.nw)
        O = np.zeros((self.nw, self.p))
        eloc = np.zeros((self.nw, 2))
        other = np.zeros((self.nw, 7))
        N.check(self.lib.tdvmc_eval_local(self.h, _ptr(lnpsi), _ptr(O), _ptr(eloc), _ptr(other)), "tdvmc_eval_local")
        return dict(lnpsi=lnpsi, O=O, eloc=eloc, other=other)

    def CalculateLocalEnergyAdjoint(self):
        """Backward pass: dE_loc/d uR_k per walker, shape (n_walkers, p, 2) = (Re, Im)."""
        dE = np.zeros((self.nw, self.p, 2))
        N.check(self.lib.tdvmc_eval_local_adjoint(self.h, _ptr(dE)), "tdvmc_eval_local_adjoint")
        return dE

    def FillCorrelatedSamplingData(self):
        """Store every walker's parameter-independent data (correlated sampling)."""
        N.check(self.lib.tdvmc_store_samples(self.h), "tdvmc_store_samples")

    def CalculateExpectationValuesForStoredSamples(self, adjoint=False):
        """Local quantities of the stored samples at the current parameters (no
        resampling); with adjoint=True also dE (n_walkers, p, 2)."""
        lnpsi = np.zeros(self.nw)
        O = np.zeros((self.nw, self.p))
        eloc = np.zeros((self.nw, 2))
        other = np.zeros((self.nw, 7))
        dE = np.zeros((self.nw, self.p, 2)) if adjoint else None
        N.check(self.lib.tdvmc_eval_stored(self.h, _ptr(lnpsi), _ptr(O), _ptr(eloc), _ptr(other),
                                           _ptr(dE) if adjoint else None), "tdvmc_eval_stored")
        out = dict(lnpsi=lnpsi, O=O, eloc=eloc, other=other)
        if adjoint:
            out["dE"] = dE
        return out

    def CalculateAdditionalSystemProperties(self, gr_bins, shell_off=None, kvec=None):
        """g(r) (GR_BIN_COUNT bins on [0, r_max)) and S(k) per k shell, averaged over
        the walkers.  kvec: (nvec, dim) k vectors scaled by 2 pi / L; shell s owns
        rows shell_off[s]:shell_off[s+1]."""
        off = np.zeros(1, dtype=np.int32) if shell_off is None else np.ascontiguousarray(shell_off, dtype=np.int32)
        nshell = len(off) - 1
        kv = _f64(np.zeros((1, self.dim)) if kvec is None else kvec)
        gr = np.zeros(int(gr_bins))
        sk = np.zeros(max(nshell, 1))
        cnt = C.c_int32()
        N.check(self.lib.tdvmc_observables(self.h, int(gr_bins), nshell, off.ctypes.data_as(C.c_void_p), _ptr(kv),
                                           _ptr(gr), C.byref(cnt), _ptr(sk)), "tdvmc_observables")
        return dict(gr=gr[:cnt.value], sk=sk[:nshell])

    def ReduceStatistics(self):
        st = N.Stats()
        P = self.p
        Om, S, cR, cI, dE = np.zeros(P), np.zeros((P, P)), np.zeros(P), np.zeros(P), np.zeros(2 * P)
        N.check(self.lib.tdvmc_reduce_stats(self.h, C.byref(st), _ptr(Om), _ptr(S), _ptr(cR), _ptr(cI), _ptr(dE)),
                "tdvmc_reduce_stats")
        return dict(energy=(st.energy_re, st.energy_im), other=np.array(st.other[:]), accept_rate=st.accept_rate,
                    O=Om, S=S, cov_OER=cR, cov_OEI=cI, dE=dE.reshape(P, 2))

    def SolveForParametersDot(self, imaginary_time=0, precondition=0, lin_solver=0):
        P = self.p
        uR, uI = np.zeros(P), np.zeros(P)
        pR, pI = C.c_double(), C.c_double()
        code = self.lib.tdvmc_tdvp_rhs(self.h, int(imaginary_time), int(precondition), int(lin_solver), _ptr(uR),
                                       _ptr(uI), C.byref(pR), C.byref(pI))
        if code not in (N.OK, N.ERR_NOT_PD):
            N.check(code, "tdvmc_tdvp_rhs")
        return uR, uI, pR.value, pI.value, code == N.ERR_NOT_PD

    def Autotune(self, moves, mc_step):
        N.check(self.lib.tdvmc_autotune(self.h, int(moves), float(mc_step)), "tdvmc_autotune")
        return self.Tiles()

    def Tiles(self):
        v = [C.c_int32() for _ in range(4)]
        N.check(self.lib.tdvmc_get_tiles(self.h, *[C.byref(x) for x in v]), "tdvmc_get_tiles")
        return dict(sample_lanes=v[0].value, sample_walkers_per_block=v[1].value, eval_lanes=v[2].value,
                    eval_walkers_per_block=v[3].value)

    def LaunchCount(self):
        return int(self.lib.tdvmc_launch_count(self.h))

    def Stream(self):
        s = C.c_void_p()
        N.check(self.lib.tdvmc_get_stream(self.h, C.byref(s)), "tdvmc_get_stream")
        return s.value


class NUBosonsBulkPB(BosonsBulk):
    """``PhysicalSystems::NUBosonsBulkPB`` (src/PhysicalSystems/NUBosonsBulkPB.cpp),
    batched over walkers: the BosonsBulk methods with every pair at r >= r_max
    entering at the mirrored distance 2 r_max - r (counted iff it lies below
    r_max), gradient terms d / r' with the sign of d, the square-well potential
    and the fold O_k = S_{k+1}, O_1 += S_0, O_{p-1} += S_{p+1}.  ``user_knots``
    (NURBS_GRID) is required: the reference reads r_max from them before it
    would build default knots (NUBosonsBulkPB.cpp:76, 91-97).

    ``exact_derivatives=True`` switches the derivative terms of the mirrored
    pairs from the reference's form (d / r', the sign flip of
    NUBosonsBulkPB.cpp:387 commented out) to the exact derivatives of
    u(2 r_max - r): -u'(r') d / r in the gradient, -(D-1)/r u'(r') in the
    Laplacian."""

    SYSTEM_TYPE = N.SYS_NU_BOSONS_BULK_PB

    def __init__(self, dim, n, n_param, box_length, n_walkers, user_knots, system_params=(0.5, 2.0),
                 hbar2_2m=1.0, precision="fp64", exact_derivatives=False):
        self.SYSTEM_TYPE = N.SYS_NU_BOSONS_BULK_PB_EXACT if exact_derivatives else N.SYS_NU_BOSONS_BULK_PB
        super().__init__(dim, n, n_param, box_length, n_walkers, system_params=system_params, potential="square",
                         user_knots=user_knots, hbar2_2m=hbar2_2m, precision=precision)


class TDVP:
    """One TDVP time step per call (ODE_SOLVER_TYPE 2 = RK4, 0 = Euler; on stored
    samples 3 = RK4 (CalculateNextParametersRK4ReuseSamples) and 5 = predictor-corrector
    (CalculateNextParametersPCReuseSamples), with update_every / update_percent as
    UPDATE_SAMPLES_EVERY_NTH_STEP / UPDATE_SAMPLES_PERCENT)."""

    def __init__(self, system: BosonsBulk, dt, moves_per_stage, mc_step, seed=1, imaginary_time=0, ode_solver=2,
                 lin_solver=0, precondition=0, normalize_wf=0, use_adjoint=0, update_every=0, update_percent=100.0):
        self.sys = system
        o = N.StepOpts()
        o.dt = float(dt)
        o.imaginary_time = int(imaginary_time)
        o.ode_solver = int(ode_solver)
        o.lin_solver = int(lin_solver)
        o.precondition = int(precondition)
        o.normalize_wf = int(normalize_wf)
        o.moves_per_stage = int(moves_per_stage)
        o.mc_step = float(mc_step)
        o.seed = int(seed)
        o.use_adjoint = int(use_adjoint)
        o.update_every = int(update_every)
        o.update_percent = float(update_percent)
        self.opts = o

    def time_steps(self, nsteps):
        """Device time (ms) of `nsteps` graph-launched steps."""
        ms = C.c_float()
        N.check(self.sys.lib.tdvmc_time_steps(self.sys.h, C.byref(self.opts), int(nsteps), C.byref(ms)),
                "tdvmc_time_steps")
        return ms.value

    def profile_stage(self):
        """Per-kernel device times (ms) of one eagerly launched stage."""
        ms = (C.c_float * 16)()
        names = (C.c_char_p * 16)()
        cnt = C.c_int32()
        N.check(self.sys.lib.tdvmc_profile_stage(self.sys.h, C.byref(self.opts), ms, names, C.byref(cnt)),
                "tdvmc_profile_stage")
        return [(names[i].decode(), ms[i]) for i in range(cnt.value)]

    def step(self, nsteps=1):
        st = N.Stats()
        code = self.sys.lib.tdvmc_run_steps(self.sys.h, C.byref(self.opts), int(nsteps), C.byref(st))
        if code not in (N.OK, N.ERR_NOT_PD, N.ERR_NONFINITE):
            N.check(code, "tdvmc_run_steps")
        return dict(energy=(st.energy_re, st.energy_im), other=np.array(st.other[:]), accept_rate=st.accept_rate,
                    status=code)
