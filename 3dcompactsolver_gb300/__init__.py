"""GB300 implementation of the per-RK-stage path of 3DCompactSolver.

The compute runs in libcs3d_gb300.so (hand-written sm_103a kernels behind the
C ABI of include/cs3d.h).  This module binds that ABI with ctypes and mirrors
the reference's C++ interface for the path under the same names:

    Domain(Nx, Ny, Nz, Lx, Ly, Lz)                      Domain.hpp:16
    BC(bcXType, bcX0, bcX1, bcYType, ...)               BC.hpp:16
    TimeStepping(type, CFL, maxTimeStep, maxTime, ...)  TimeStepping.hpp:20
    CSolver_GB300(dom, bc, ts, alphaF, mu_ref, ...)     CSolver_AWS.hpp:119
    RK4(cs), TVDRK3(cs)                                 RK4.hpp:7, TVDRK3.hpp:7
    Derivatives(dom, bcType, dir), Filter(alphaF, ...)  Derivatives.hpp:54, Filter.hpp:31

There is no CPU fallback: if the library is missing or no GPU is visible, the
constructors raise.
"""
import ctypes
import os

import numpy as np

from . import _abi
from ._abi import (  # noqa: F401  (re-exported constants)
    Config, make_config, PERIODIC_SOLVE, DIRICHLET_SOLVE, PERIODIC, SPONGE, ADIABATIC_WALL,
    MOVING_ADIABATIC_WALL, INLET, DIRX, DIRY, DIRZ, RK4 as RK4_KIND, TVDRK3 as TVDRK3_KIND, FP64,
    FP32_MIXED, SPONGE_REFERENCE, SPONGE_BANDS)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("CS3D_LIB_PATH") or os.path.join(HERE, "libcs3d_gb300.so")

OPT_STORE_INCREMENTS = 1
OPT_STORE_DIAGNOSTICS = 2
OPT_KERNEL_TIMING = 3
OPT_ADJ_RECOMPUTE = 4
OP_DERIV1, OP_DERIV2, OP_FILTER = 1, 2, 3  # kinds of the operator-only handle
ADJ_SEED = 0       # cs3d_adjoint_backward: dJ/dq of the final state given
ADJ_KE_MEAN = 1    # J = mean over points of rho |u|^2 / 2 of the final state
KERNEL_CLASSES = ("sweep_x", "sweep_y", "sweep_z", "filter", "boundary", "cfl", "sponge", "other")

_lib = None
_DP = ctypes.POINTER(ctypes.c_double)
_H = ctypes.c_void_p


class CS3DError(RuntimeError):
    """A status code other than CS3D_OK returned by the C ABI."""

    def __init__(self, code, msg):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; "
                              "g.build()'` (or 3dcompactsolver_gb300/build.py) first")
        L = ctypes.CDLL(LIB_PATH)
        L.cs3d_last_error.restype = ctypes.c_char_p
        L.cs3d_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(_H)]
        L.cs3d_destroy.argtypes = [_H]
        L.cs3d_set_initial_conditions.argtypes = [_H, _DP, _DP, _DP, _DP, _DP]
        for name in ("cs3d_step", "cs3d_pre_step", "cs3d_post_step", "cs3d_sync"):
            getattr(L, name).argtypes = [_H]
        L.cs3d_run.argtypes = [_H, ctypes.c_int]
        L.cs3d_sub_step.argtypes = [_H, ctypes.c_int, ctypes.c_int]
        L.cs3d_get_field.argtypes = [_H, ctypes.c_int, _DP]
        L.cs3d_set_field.argtypes = [_H, ctypes.c_int, _DP]
        L.cs3d_field_ptr.argtypes = [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.cs3d_get_conserved.argtypes = [_H, ctypes.POINTER(_DP)]
        L.cs3d_set_conserved.argtypes = [_H, ctypes.POINTER(_DP)]
        L.cs3d_get_scalars.argtypes = [_H, _DP, _DP, ctypes.POINTER(ctypes.c_int)]
        L.cs3d_get_stream.argtypes = [_H, ctypes.POINTER(ctypes.c_void_p)]
        L.cs3d_launch_count.argtypes = [_H, ctypes.POINTER(ctypes.c_longlong)]
        L.cs3d_set_option.argtypes = [_H, ctypes.c_int, ctypes.c_int]
        for name in ("cs3d_deriv1", "cs3d_deriv2", "cs3d_filter"):
            getattr(L, name).argtypes = [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.cs3d_tgv_quantities.argtypes = [_H, _DP]
        L.cs3d_turbulence_quantities.argtypes = [_H, _DP]
        L.cs3d_dump_solution.argtypes = [_H, ctypes.c_char_p]
        L.cs3d_aero_optics.argtypes = [_H, ctypes.c_int, ctypes.c_double, _DP]
        L.cs3d_vorticity_q.argtypes = [_H, _DP, _DP]
        L.cs3d_load_solution.argtypes = [_H, ctypes.c_char_p, ctypes.c_int, ctypes.c_double]
        L.cs3d_shear_layer_info.argtypes = [_H, _DP]
        L.cs3d_kernel_times.argtypes = [_H, _DP, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int,
                                        ctypes.c_int]
        L.cs3d_version.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3
        L.cs3d_adjoint_record.argtypes = [_H, ctypes.c_int, ctypes.c_int]
        L.cs3d_adjoint_backward.argtypes = [_H, ctypes.c_int, _DP, _DP, _DP]
        L.cs3d_rhs_eval.argtypes = [_H, _DP, _DP]
        L.cs3d_rhs_vjp.argtypes = [_H, _DP, _DP, _DP]
        L.cs3d_op_create.argtypes = [ctypes.POINTER(Config), ctypes.c_int, ctypes.POINTER(_H)]
        L.cs3d_op_destroy.argtypes = [_H]
        L.cs3d_op_apply.argtypes = [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.cs3d_op_apply_host.argtypes = [_H, ctypes.c_int, _DP, _DP]
        L.cs3d_op_get_stream.argtypes = [_H, ctypes.POINTER(ctypes.c_void_p)]
        _lib = L
    return _lib


def check(rc):
    if rc != 0:
        raise CS3DError(rc, lib().cs3d_last_error().decode(errors="replace"))


def _dptr(a):
    return a.ctypes.data_as(_DP)


class Solver:
    """One solver handle on the current CUDA device (the C ABI, 1:1)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.shape = (cfg.Nz, cfg.Ny, cfg.Nx)
        h = _H()
        check(lib().cs3d_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().cs3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_initial_conditions(self, rho0, p0, U0, V0, W0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (rho0, p0, U0, V0, W0)]
        for a in arrs:
            if a.size != self.cfg.npts:
                raise ValueError(f"initial field has {a.size} points, expected {self.cfg.npts}")
        check(lib().cs3d_set_initial_conditions(self.h, *[_dptr(a) for a in arrs]))

    def step(self):
        check(lib().cs3d_step(self.h))

    def run(self, n):
        check(lib().cs3d_run(self.h, int(n)))

    def pre_step(self):
        check(lib().cs3d_pre_step(self.h))

    def sub_step(self, rk_step, rk_last):
        check(lib().cs3d_sub_step(self.h, int(rk_step), int(bool(rk_last))))

    def post_step(self):
        check(lib().cs3d_post_step(self.h))

    def sync(self):
        check(lib().cs3d_sync(self.h))

    def set_option(self, option, value=1):
        check(lib().cs3d_set_option(self.h, option, int(value)))

    def get(self, field):
        out = np.empty(self.shape, np.float64)
        check(lib().cs3d_get_field(self.h, int(field), _dptr(out)))
        return out

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        check(lib().cs3d_set_field(self.h, int(field), _dptr(a)))

    def field_ptr(self, field):
        p = ctypes.c_void_p()
        check(lib().cs3d_field_ptr(self.h, int(field), ctypes.byref(p)))
        return p.value

    def conserved(self):
        """q1 as a (5, Nz, Ny, Nx) array."""
        out = np.empty((5,) + tuple(self.shape), np.float64)
        ptrs = (_DP * 5)(*[_dptr(out[f]) for f in range(5)])
        check(lib().cs3d_get_conserved(self.h, ptrs))
        return out

    def set_conserved(self, q):
        """Set q1 from a (5, Nz, Ny, Nx) array (all five fields, one call)."""
        a = [np.ascontiguousarray(q[f], dtype=np.float64) for f in range(5)]
        ptrs = (_DP * 5)(*[_dptr(x) for x in a])
        check(lib().cs3d_set_conserved(self.h, ptrs))

    def scalars(self):
        dt, t, ts = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        check(lib().cs3d_get_scalars(self.h, ctypes.byref(dt), ctypes.byref(t), ctypes.byref(ts)))
        return dt.value, t.value, ts.value

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().cs3d_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def launch_count(self):
        c = ctypes.c_longlong()
        check(lib().cs3d_launch_count(self.h, ctypes.byref(c)))
        return c.value

    def kernel_times(self, reset=False):
        """{class: (total_ms, launches)} accumulated while OPT_KERNEL_TIMING was on."""
        n = len(KERNEL_CLASSES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        check(lib().cs3d_kernel_times(self.h, ms, cnt, n, int(reset)))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}

    def tgv_quantities(self):
        out = np.zeros(7)
        check(lib().cs3d_tgv_quantities(self.h, _dptr(out)))
        return out

    # -- discrete adjoint (periodic, RK4 or TVD-RK3, fixed dt) ----------------
    def _q5(self, q):
        a = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        if a.size != 5 * self.cfg.npts:
            raise ValueError(f"expected 5 fields of {self.cfg.npts} points, got {a.size} values")
        return a

    def rhs_eval(self, q):
        """R(q), the stage right-hand side from its 48 stored pointwise inputs."""
        qa = self._q5(q)
        out = np.empty((5,) + self.shape)
        check(lib().cs3d_rhs_eval(self.h, _dptr(qa), _dptr(out)))
        return out

    def rhs_vjp(self, q, lam):
        """(dR/dq)^T lam at the state q (both (5, Nz, Ny, Nx))."""
        qa, la = self._q5(q), self._q5(lam)
        out = np.empty((5,) + self.shape)
        check(lib().cs3d_rhs_vjp(self.h, _dptr(qa), _dptr(la), _dptr(out)))
        return out

    def adjoint_record(self, nsteps, checkpoint_every=0):
        """Run nsteps from the current state, keeping checkpoints for the adjoint."""
        check(lib().cs3d_adjoint_record(self.h, int(nsteps), int(checkpoint_every)))

    def adjoint_backward(self, objective=ADJ_KE_MEAN, seed=None):
        """(dJ/dq0 as (5, Nz, Ny, Nx), J) for the recorded steps."""
        grad = np.empty((5,) + self.shape)
        J = ctypes.c_double(0.0)
        keep = self._q5(seed) if seed is not None else None
        sp = _dptr(keep) if keep is not None else None
        check(lib().cs3d_adjoint_backward(self.h, int(objective), sp, _dptr(grad), ctypes.byref(J)))
        return grad, J.value

    def vorticity_q(self):
        """(|curl u|, Q-criterion) of the current state, each (Nz, Ny, Nx)."""
        v = np.empty(self.shape)
        q = np.empty(self.shape)
        check(lib().cs3d_vorticity_q(self.h, _dptr(v), _dptr(q)))
        return v, q

    def aero_optics(self, num_angles=5, max_angle=70.0):
        """Optical-path integrals of the density, shape (num_angles, Nz, Nx)."""
        out = np.zeros((num_angles, self.cfg.Nz, self.cfg.Nx))
        check(lib().cs3d_aero_optics(self.h, int(num_angles), float(max_angle), _dptr(out)))
        return out

    def dump_solution(self, prefix=""):
        """Write q1 in dumpSolution's format: <prefix>rho.out.<step> ... rhoE."""
        check(lib().cs3d_dump_solution(self.h, prefix.encode()))

    def load_solution(self, prefix, time_step, time):
        """Restart from dumpSolution files of step time_step (the time is not in them)."""
        check(lib().cs3d_load_solution(self.h, prefix.encode(), int(time_step), float(time)))

    def turbulence_quantities(self):
        """The turbdata.out row of calcTurbulenceQuantities (11 values)."""
        out = np.zeros(11)
        check(lib().cs3d_turbulence_quantities(self.h, _dptr(out)))
        return out

    def shear_layer_info(self):
        """(17, Ny) per-plane statistics of shearLayerInfoCalc (rows as in cs3d.h)."""
        out = np.zeros((17, self.cfg.Ny))
        check(lib().cs3d_shear_layer_info(self.h, _dptr(out)))
        return out

    def line_op(self, kind, direction, in_ptr, out_ptr):
        """kind 1/2/3 = deriv1/deriv2/filter on device arrays in the direction's
        contiguous layout."""
        fn = {1: lib().cs3d_deriv1, 2: lib().cs3d_deriv2, 3: lib().cs3d_filter}[kind]
        check(fn(self.h, int(direction), ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr)))


class Operator:
    """An operator-only handle (cs3d_op_*): the 1st-derivative, 2nd-derivative
    and filter operators of one direction of the grid in cfg, with no solver
    state.  kind 1/2/3 = OP_DERIV1 / OP_DERIV2 / OP_FILTER."""

    def __init__(self, cfg, direction):
        h = _H()
        check(lib().cs3d_op_create(ctypes.byref(cfg), int(direction), ctypes.byref(h)))
        self.h = h
        self.npts = cfg.Nx * cfg.Ny * cfg.Nz

    def close(self):
        if getattr(self, "h", None):
            lib().cs3d_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply(self, kind, in_ptr, out_ptr):
        """Device arrays (integer addresses), queued on stream()."""
        check(lib().cs3d_op_apply(self.h, int(kind), ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr)))

    def apply_host(self, kind, data_in, data_out=None):
        """Host arrays, synchronous; returns data_out (allocated if None)."""
        a = np.ascontiguousarray(data_in, dtype=np.float64)
        if a.size != self.npts:
            raise ValueError(f"field has {a.size} points, expected {self.npts}")
        out = np.empty_like(a) if data_out is None else data_out
        if not (out.flags.c_contiguous and out.dtype == np.float64 and out.size == self.npts):
            raise ValueError("data_out must be a C-contiguous float64 array of the field's size")
        check(lib().cs3d_op_apply_host(self.h, int(kind), _dptr(a), _dptr(out)))
        return out

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().cs3d_op_get_stream(self.h, ctypes.byref(s)))
        return s.value


def ic_velocity_gradient(grad_q0, rho0, U0, V0, W0):
    """dJ/dU0, dJ/dV0, dJ/dW0 from dJ/dq0 through the initial state
    q0 = (rho0, rho0 U0, rho0 V0, rho0 W0, p0/(gamma-1) + rho0 |u0|^2 / 2)
    of setInitialConditions (CSolver_AWS.cpp:199-504) on periodic grids."""
    g = np.asarray(grad_q0).reshape((5,) + np.shape(rho0))
    return (rho0 * (g[1] + U0 * g[4]), rho0 * (g[2] + V0 * g[4]), rho0 * (g[3] + W0 * g[4]))


# ---------------------------------------------------------------------------
# reference-named interface
# ---------------------------------------------------------------------------
class Domain:
    """Grid of Domain.hpp:16-52: x_i = i*L/(N-1)."""

    def __init__(self, Nx, Ny, Nz, Lx, Ly, Lz):
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.N = self.Nx * self.Ny * self.Nz
        self.Lx, self.Ly, self.Lz = float(Lx), float(Ly), float(Lz)
        self.x = np.array([(float(i) / (float(self.Nx) - 1.0)) * self.Lx for i in range(self.Nx)])
        self.y = np.array([(float(j) / (float(self.Ny) - 1.0)) * self.Ly for j in range(self.Ny)])
        self.z = np.array([(float(k) / (float(self.Nz) - 1.0)) * self.Lz for k in range(self.Nz)])
        self.dx = self.x[1] - self.x[0]
        self.dy = self.y[1] - self.y[0]
        self.dz = self.z[1] - self.z[0]


class BC:
    """Boundary types and kinds of BC.hpp:10-31."""
    PERIODIC_SOLVE, DIRICHLET_SOLVE = PERIODIC_SOLVE, DIRICHLET_SOLVE
    PERIODIC, SPONGE, ADIABATIC_WALL, MOVING_ADIABATIC_WALL, INLET = (
        PERIODIC, SPONGE, ADIABATIC_WALL, MOVING_ADIABATIC_WALL, INLET)

    def __init__(self, bcXType, bcX0, bcX1, bcYType, bcY0, bcY1, bcZType, bcZ0, bcZ1):
        self.bcXType, self.bcYType, self.bcZType = bcXType, bcYType, bcZType
        self.bcX0, self.bcX1, self.bcY0, self.bcY1, self.bcZ0, self.bcZ1 = (
            bcX0, bcX1, bcY0, bcY1, bcZ0, bcZ1)


class TimeStepping:
    """TimeStepping.hpp:10-40.  The reference always steps at constant CFL
    (CSolver_AWS.cpp:530); dt_fixed > 0 freezes dt instead."""
    CONST_DT, CONST_CFL = 0, 1

    def __init__(self, timeSteppingType, CFL, maxTimeStep, maxTime, filterStep, checkStep=1,
                 dumpStep=1 << 30, dt_fixed=0.0):
        self.timeSteppingType = timeSteppingType
        self.CFL = float(CFL)
        self.maxTimeStep = int(maxTimeStep)
        self.maxTime = float(maxTime)
        self.filterStep = int(filterStep)
        self.checkStep = int(checkStep)
        self.dumpStep = int(dumpStep)
        self.dt_fixed = float(dt_fixed)
        self.dt = 0.0


class CSolver_GB300:
    """Drop-in for CSolver_AWS (CSolver_AWS.hpp:119) on one GPU.

    The reference's five stage virtuals run as one fused launch sequence, which
    is issued by updateData(), the last of them; preSubStep, solveEqnSet and
    postSubStep only record the call.  Public state arrays (rho1 ... rhoE2,
    U, V, W, p, T, mu, sos) are read from the device on access."""

    def __init__(self, dom, bc, ts, alphaF, mu_ref, blocksize=16, useTiming=False, rk=_abi.RK4,
                 precision=FP64, sponge_mode=SPONGE_REFERENCE, sponge_frac=(0.0,) * 6,
                 wall_vel=(0.0,) * 12):
        self.dom, self.bc, self.ts = dom, bc, ts
        self.alphaF, self.mu_ref = float(alphaF), float(mu_ref)
        self.blocksize, self.useTiming = blocksize, useTiming
        cfg = make_config(
            (dom.Nx, dom.Ny, dom.Nz), (dom.Lx, dom.Ly, dom.Lz),
            bc_type=(bc.bcXType, bc.bcYType, bc.bcZType),
            bc_kind=(bc.bcX0, bc.bcX1, bc.bcY0, bc.bcY1, bc.bcZ0, bc.bcZ1), alphaF=alphaF,
            mu_ref=mu_ref, CFL=ts.CFL, filter_step=ts.filterStep, rk=rk, precision=precision,
            sponge_mode=sponge_mode, sponge_frac=sponge_frac, wall_vel=wall_vel,
            dt_fixed=ts.dt_fixed)
        self.solver = Solver(cfg)
        shape = (dom.Nz, dom.Ny, dom.Nx)
        self.rho0 = np.ones(shape)
        self.p0 = np.ones(shape)
        self.U0 = np.zeros(shape)
        self.V0 = np.zeros(shape)
        self.W0 = np.zeros(shape)
        self.rkStep, self.rkLast, self.endFlag = 1, False, False
        self.timeStep, self.time = 0, 0.0

    # AbstractCSolver.hpp:36-43
    def initializeSolverData(self):
        pass  # device arrays are allocated by the constructor

    def setInitialConditions(self):
        self.solver.set_initial_conditions(self.rho0, self.p0, self.U0, self.V0, self.W0)

    def preStep(self):
        self.solver.pre_step()
        self.timeStep += 1

    def preSubStep(self):
        pass

    def solveEqnSet(self):
        pass

    def postSubStep(self):
        pass

    def updateData(self):
        self.solver.sub_step(self.rkStep, self.rkLast)

    def postStep(self):
        self.solver.post_step()
        if self.timeStep >= self.ts.maxTimeStep:
            self.endFlag = True
        elif self.ts.maxTime < 1e300:
            _, t, _ = self.solver.scalars()
            self.time = t
            if t >= self.ts.maxTime:
                self.endFlag = True

    def __getattr__(self, name):
        fields = {"rho1": 0, "rhoU1": 1, "rhoV1": 2, "rhoW1": 3, "rhoE1": 4, "rhok": 5, "rhoUk": 6,
                  "rhoVk": 7, "rhoWk": 8, "rhoEk": 9, "rho2": 10, "rhoU2": 11, "rhoV2": 12,
                  "rhoW2": 13, "rhoE2": 14, "rhok2": 15, "rhoUk2": 16, "rhoVk2": 17, "rhoWk2": 18,
                  "rhoEk2": 19, "U": 20, "V": 21, "W": 22, "p": 23, "T": 24, "mu": 25, "sos": 26}
        if name in fields:
            return self.__dict__["solver"].get(fields[name])
        raise AttributeError(name)


class _RKBase:
    nstages = 4

    def __init__(self, cs):
        self.cs = cs

    def updateConservedData(self):
        pass  # fused into the stage launched by cs.updateData()

    def executeSolverLoop(self):
        """RK4.hpp:120-170 / TVDRK3.hpp:98-139."""
        cs = self.cs
        cs.setInitialConditions()
        while not cs.endFlag:
            cs.rkLast = False
            cs.preStep()
            for s in range(1, self.nstages + 1):
                cs.rkStep = s
                cs.rkLast = s == self.nstages
                cs.preSubStep()
                cs.solveEqnSet()
                cs.postSubStep()
                self.updateConservedData()
                cs.updateData()
            cs.postStep()


class RK4(_RKBase):
    nstages = 4


class TVDRK3(_RKBase):
    nstages = 3


class Derivatives:
    """Derivatives(dom, bcType, dir) (Derivatives.hpp:54): calc1stDerivField /
    calc2ndDerivField (Derivatives.cpp:3-96) on fields in the direction's
    contiguous layout -- numpy arrays (synchronous, as the reference's host
    arrays; dataOut is written in place) or integer device addresses (queued
    on the operator handle's stream).  Backed by an operator-only handle."""
    DIRX, DIRY, DIRZ = DIRX, DIRY, DIRZ

    def __init__(self, dom, bcType, currentDir, alphaF=0.49):
        bt = [PERIODIC_SOLVE] * 3
        bt[currentDir] = bcType
        cfg = make_config((dom.Nx, dom.Ny, dom.Nz), (dom.Lx, dom.Ly, dom.Lz), bc_type=tuple(bt),
                          alphaF=alphaF)
        self.op = Operator(cfg, currentDir)
        self.currentDir = currentDir

    def _apply(self, kind, dataIn, dataOut):
        if isinstance(dataIn, np.ndarray):
            self.op.apply_host(kind, dataIn, dataOut)
        else:
            self.op.apply(kind, dataIn, dataOut)

    def calc1stDerivField(self, dataIn, dataOut):
        self._apply(OP_DERIV1, dataIn, dataOut)

    def calc2ndDerivField(self, dataIn, dataOut):
        self._apply(OP_DERIV2, dataIn, dataOut)


class Filter(Derivatives):
    """Filter(alphaF, dom, bcType, dir).filterField (Filter.hpp:31, Filter.cpp:129-171)."""

    def __init__(self, alphaF, dom, bcType, currentDir):
        super().__init__(dom, bcType, currentDir, alphaF=alphaF)

    def filterField(self, dataIn, dataOut):
        self._apply(OP_FILTER, dataIn, dataOut)
