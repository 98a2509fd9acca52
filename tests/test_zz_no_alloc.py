"""cs3d_kinetic_energy_noalloc, the allocation-free entry point, against the
KEsum column of cs3d_tgv_quantities on the same state: two calls in a row,
then again after another step.  Kept in its own file, collected last, so that
it also runs after every other GPU test has used the device."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

_DP = ctypes.POINTER(ctypes.c_double)


def _fn(pkg):
    f = pkg.lib().cs3d_kinetic_energy_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_longlong, ctypes.c_void_p, _DP]
    return f


def _ke(pkg, f, ptrs, npts, stream):
    ke = ctypes.c_double(0.0)
    rc = f(*ptrs, npts, stream, ctypes.byref(ke))
    assert rc == 0, pkg.lib().cs3d_last_error().decode()
    return ke.value


def test_noalloc_kinetic_energy_matches_tgv_quantities(gpu_pkg, cases):
    cfg, ic = cases.tgv(32)
    s = gpu_pkg.Solver(cfg)
    s.set_option(gpu_pkg.OPT_STORE_DIAGNOSTICS, 1)
    s.set_initial_conditions(*ic)
    f = _fn(gpu_pkg)
    npts = 32 ** 3
    ptrs = [s.field_ptr(i) for i in range(4)]
    stream = s.stream()
    for _ in range(2):
        s.step()
        ref = s.tgv_quantities()[1]
        a = _ke(gpu_pkg, f, ptrs, npts, stream)
        b = _ke(gpu_pkg, f, ptrs, npts, stream)
        assert a == b
        assert abs(a - ref) <= 1e-14 * abs(ref), (a, ref)


def test_noalloc_kinetic_energy_rejects_bad_sizes(gpu_pkg, cases):
    cfg, ic = cases.tgv(16)
    s = gpu_pkg.Solver(cfg)
    s.set_initial_conditions(*ic)
    f = _fn(gpu_pkg)
    ptrs = [s.field_ptr(i) for i in range(4)]
    ke = ctypes.c_double(0.0)
    assert f(*ptrs, 0, s.stream(), ctypes.byref(ke)) == 2
    assert f(*ptrs, 1 << 31, s.stream(), ctypes.byref(ke)) == 2
    assert b"2^31-1" in gpu_pkg.lib().cs3d_last_error()
    assert f(None, *ptrs[1:], 16, s.stream(), ctypes.byref(ke)) == 1
