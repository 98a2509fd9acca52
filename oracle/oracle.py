"""ctypes access to the test oracle.  TEST INFRASTRUCTURE ONLY.

Two implementations with one interface:
  * OraclePort  -- oracle/cs3d_oracle.c, the C restatement of the reference
                   algorithm (built by `make -C oracle`), available everywhere;
  * RefSolver   -- the reference's own sources linked with oracle/ref_harness.cpp
                   (built by `make -C oracle ref` where the reference checkout
                   exists), used to pin the restatement and to make the
                   committed golden vectors.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this.
"""
import ctypes
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
_abi = importlib.import_module("3dcompactsolver_gb300._abi")
Config = _abi.Config

_DP = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_DP)


def reference_dir():
    """The reference checkout that oracle/Makefile compiles from (its REF,
    which $CS3D_REFERENCE overrides), or None where that directory does not
    exist (the GPU machines carry no reference checkout)."""
    import subprocess
    out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    d = out.stdout.strip()
    return d if out.returncode == 0 and d and os.path.isdir(d) else None


def build(ref=False, quiet=True):
    """Compile the restatement (and, with ref=True and a reference checkout
    present, the reference harness)."""
    import subprocess
    targets = ["all"]
    if ref and reference_dir():
        targets.append("ref")
    out = subprocess.run(["make", "-C", HERE] + targets, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _load(path):
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    return ctypes.CDLL(path)


_PORT = {}


def port_lib(flavour="strict"):
    if flavour not in _PORT:
        lib = _load(os.path.join(HERE, f"liboracle_{flavour}.so"))
        lib.or_create.restype = _VP
        lib.or_create.argtypes = [ctypes.POINTER(Config)]
        lib.or_destroy.argtypes = [_VP]
        lib.or_set_initial_conditions.argtypes = [_VP, _DP, _DP, _DP, _DP, _DP]
        lib.or_step.argtypes = [_VP]
        lib.or_run.argtypes = [_VP, ctypes.c_int]
        lib.or_pre_step.argtypes = [_VP]
        lib.or_sub_step.argtypes = [_VP, ctypes.c_int, ctypes.c_int]
        lib.or_post_step.argtypes = [_VP]
        lib.or_get_named.argtypes = [_VP, ctypes.c_char_p, _DP]
        lib.or_set_named.argtypes = [_VP, ctypes.c_char_p, _DP]
        lib.or_get_scalars.argtypes = [_VP, _DP, _DP, ctypes.POINTER(ctypes.c_int)]
        lib.or_tgv_quantities.argtypes = [_VP, _DP]
        lib.or_turbulence_quantities.argtypes = [_VP, _DP]
        lib.or_shear_layer_info.argtypes = [_VP, _DP]
        lib.or_aero_optics.argtypes = [_VP, ctypes.c_int, ctypes.c_double, _DP]
        lib.or_vorticity_q.argtypes = [_VP, _DP, _DP]
        lib.or_line_op.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_long, _DP, _DP]
        lib.or_num_threads.restype = ctypes.c_int
        _PORT[flavour] = lib
    return _PORT[flavour]


_REF = {}


def ref_available(flavour="strict"):
    return os.path.exists(os.path.join(HERE, "_ref", f"libref3d_{flavour}.so"))


def ref_lib(flavour="strict"):
    if flavour not in _REF:
        lib = _load(os.path.join(HERE, "_ref", f"libref3d_{flavour}.so"))
        lib.ref_create.restype = _VP
        lib.ref_create.argtypes = [ctypes.POINTER(Config)]
        lib.ref_set_ic.argtypes = [_VP, _DP, _DP, _DP, _DP, _DP]
        lib.ref_step.argtypes = [_VP]
        lib.ref_pre_step.argtypes = [_VP]
        lib.ref_sub_step.argtypes = [_VP, ctypes.c_int, ctypes.c_int]
        lib.ref_post_step.argtypes = [_VP]
        lib.ref_get_field.argtypes = [_VP, ctypes.c_int, _DP]
        lib.ref_get_named.argtypes = [_VP, ctypes.c_char_p, _DP]
        lib.ref_get_scalars.argtypes = [_VP, _DP, _DP, ctypes.POINTER(ctypes.c_int)]
        lib.ref_destroy.argtypes = [_VP]
        lib.ref_turbulence_quantities.argtypes = [_VP]
        lib.ref_shear_layer_info.argtypes = [_VP]
        lib.ref_dump_solution.argtypes = [_VP]
        lib.ref_aero_optics.argtypes = [_VP, ctypes.c_int, ctypes.c_double, _DP]
        lib.ref_line_op.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, _DP, _DP]
        _REF[flavour] = lib
    return _REF[flavour]


_FIELD_NAMES = ["rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1", "rhok", "rhoUk", "rhoVk", "rhoWk",
                "rhoEk", "rho2", "rhoU2", "rhoV2", "rhoW2", "rhoE2", "rhok2", "rhoUk2", "rhoVk2",
                "rhoWk2", "rhoEk2", "U", "V", "W", "p", "T", "mu", "sos", "spongeRhoAvg",
                "spongeRhoUAvg", "spongeRhoVAvg", "spongeRhoWAvg", "spongeRhoEAvg", "sigma"]


class _Base:
    def __init__(self, cfg):
        self.cfg = cfg
        self.shape = (cfg.Nz, cfg.Ny, cfg.Nx)

    def conserved(self):
        """q1 as a (5, Nz, Ny, Nx) array."""
        return np.stack([self.get(n) for n in ("rho1", "rhoU1", "rhoV1", "rhoW1", "rhoE1")])

    def run(self, n):
        for _ in range(n):
            self.step()


class OraclePort(_Base):
    """The C restatement (oracle/cs3d_oracle.c)."""

    def __init__(self, cfg, flavour="strict"):
        super().__init__(cfg)
        self.lib = port_lib(flavour)
        self.h = self.lib.or_create(ctypes.byref(cfg))
        if not self.h:
            raise ValueError("or_create rejected the configuration")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_destroy(self.h)
            self.h = None

    def set_initial_conditions(self, rho0, p0, U0, V0, W0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (rho0, p0, U0, V0, W0)]
        self.lib.or_set_initial_conditions(self.h, *[_ptr(a) for a in arrs])

    def step(self):
        self.lib.or_step(self.h)

    def run(self, n):
        self.lib.or_run(self.h, n)

    def pre_step(self):
        self.lib.or_pre_step(self.h)

    def sub_step(self, s, last):
        self.lib.or_sub_step(self.h, s, int(last))

    def post_step(self):
        self.lib.or_post_step(self.h)

    def get(self, name):
        out = np.empty(self.shape, np.float64)
        if self.lib.or_get_named(self.h, name.encode(), _ptr(out)):
            raise KeyError(name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if self.lib.or_set_named(self.h, name.encode(), _ptr(a)):
            raise KeyError(name)

    def scalars(self):
        dt, t, ts = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self.lib.or_get_scalars(self.h, ctypes.byref(dt), ctypes.byref(t), ctypes.byref(ts))
        return dt.value, t.value, ts.value

    def tgv_quantities(self):
        out = np.zeros(7)
        self.lib.or_tgv_quantities(self.h, _ptr(out))
        return out

    def turbulence_quantities(self):
        """The turbdata.out row of calcTurbulenceQuantities (11 values)."""
        out = np.zeros(11)
        self.lib.or_turbulence_quantities(self.h, _ptr(out))
        return out

    def shear_layer_info(self):
        """(17, Ny) per-plane statistics of shearLayerInfoCalc (see the C source)."""
        out = np.zeros((17, self.cfg.Ny))
        self.lib.or_shear_layer_info(self.h, _ptr(out))
        return out

    def vorticity_q(self):
        """(|curl u|, Q-criterion) of the state, each (Nz, Ny, Nx)."""
        v = np.zeros(self.shape)
        q = np.zeros(self.shape)
        self.lib.or_vorticity_q(self.h, _ptr(v), _ptr(q))
        return v, q

    def aero_optics(self, num_angles=5, max_angle=70.0):
        """OPL integrals of the density of q1, shape (num_angles, Nz, Nx)."""
        out = np.zeros((num_angles, self.cfg.Nz, self.cfg.Nx))
        self.lib.or_aero_optics(self.h, num_angles, max_angle, _ptr(out))
        return out


class RefSolver(_Base):
    """The reference's own CSolver_AWS + RK4/TVDRK3 (oracle/_ref)."""

    def __init__(self, cfg, flavour="strict"):
        super().__init__(cfg)
        self.lib = ref_lib(flavour)
        self.h = self.lib.ref_create(ctypes.byref(cfg))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def set_initial_conditions(self, rho0, p0, U0, V0, W0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (rho0, p0, U0, V0, W0)]
        self.lib.ref_set_ic(self.h, *[_ptr(a) for a in arrs])

    def step(self):
        self.lib.ref_step(self.h)

    def pre_step(self):
        self.lib.ref_pre_step(self.h)

    def sub_step(self, s, last):
        self.lib.ref_sub_step(self.h, s, int(last))

    def post_step(self):
        self.lib.ref_post_step(self.h)

    def get(self, name):
        out = np.empty(self.shape, np.float64)
        if name in _FIELD_NAMES:
            rc = self.lib.ref_get_field(self.h, _FIELD_NAMES.index(name), _ptr(out))
        else:
            rc = self.lib.ref_get_named(self.h, name.encode(), _ptr(out))
        if rc:
            raise KeyError(name)
        return out

    def scalars(self):
        dt, t, ts = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self.lib.ref_get_scalars(self.h, ctypes.byref(dt), ctypes.byref(t), ctypes.byref(ts))
        return dt.value, t.value, ts.value

    def _in_tmpdir(self, fn):
        import tempfile
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                fn()
                return {f: open(os.path.join(d, f)).read() for f in os.listdir(d)}
            finally:
                os.chdir(cwd)

    def dump_solution(self):
        """The reference's dumpSolution: {file name: bytes} of what it writes."""
        import tempfile
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                self.lib.ref_dump_solution(self.h)
                return {f: open(os.path.join(d, f), "rb").read() for f in os.listdir(d)}
            finally:
                os.chdir(cwd)

    def aero_optics(self, num_angles=5, max_angle=70.0):
        """The reference's AeroOptics::computeAO on rho2: (OPL array, {file: bytes})."""
        out = np.zeros((num_angles, self.cfg.Nz, self.cfg.Nx))
        files = self._in_tmpdir_bytes(lambda: self.lib.ref_aero_optics(self.h, num_angles, max_angle, _ptr(out)))
        return out, files

    def _in_tmpdir_bytes(self, fn):
        import tempfile
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as d:
            os.chdir(d)
            try:
                fn()
                return {f: open(os.path.join(d, f), "rb").read() for f in os.listdir(d)}
            finally:
                os.chdir(cwd)

    def turbulence_quantities(self):
        """The reference's calcTurbulenceQuantities: its turbdata.out row."""
        files = self._in_tmpdir(lambda: self.lib.ref_turbulence_quantities(self.h))
        return np.array([float(x) for x in files["turbdata.out"].split()])

    def shear_layer_info(self):
        """The reference's shearLayerInfoCalc, read back from its .out files, in
        the row order of the restatement (rows 2, 3, 4, 5, 15, 16 are not
        written by the reference and come back as NaN)."""
        files = self._in_tmpdir(lambda: self.lib.ref_shear_layer_info(self.h))
        names = {0: "rhoAvg", 1: "uAvg", 6: "rhoprime2", 7: "uprime2", 8: "vprime2", 9: "wprime2",
                 10: "pprime2", 11: "tprime2", 12: "uvprime", 13: "uwprime", 14: "vwprime"}
        out = np.full((17, self.cfg.Ny), np.nan)
        for k, nm in names.items():
            vals = [float(x) for x in files[nm + ".out"].split()]
            out[k] = vals[1:]  # the first value is the time
        return out


def line_op_port(kind, bc_type, N, dh, alphaF, lines, flavour="strict"):
    """Apply operator kind (1: d/dx, 2: d2/dx2, 3: filter) to contiguous lines
    (array of shape (..., N))."""
    a = np.ascontiguousarray(lines, dtype=np.float64)
    out = np.empty_like(a)
    nl = a.size // N
    port_lib(flavour).or_line_op(kind, bc_type, N, dh, alphaF, nl, _ptr(a), _ptr(out))
    return out


def line_op_ref(kind, direction, bc_type, N3, L3, alphaF, field, flavour="strict"):
    """The reference's calc1stDerivField / calc2ndDerivField / filterField on a
    field in the direction's contiguous layout."""
    a = np.ascontiguousarray(field, dtype=np.float64)
    out = np.empty_like(a)
    ref_lib(flavour).ref_line_op(kind, direction, bc_type, N3[0], N3[1], N3[2], L3[0], L3[1],
                                 L3[2], alphaF, _ptr(a), _ptr(out))
    return out
