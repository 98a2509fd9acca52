"""The FP64 viscosity power T^0.76 of the sweeps (`visc_pow`, csrc/cs3d_dev.cuh),
restated in numpy: an FP32 estimate exp2(0.76 log2 T), then one Halley step on
y^25 = T^19 written as y + y (c - a) / (13 a + 12 c), a = y^25 and c = T^19 by
repeated squaring.  Pins the accuracy the kernels rely on against the C
library's pow (which the reference's IdealGas uses for mu = mu_ref T^0.76)."""
import numpy as np


def _visc_pow(T):
    y = np.exp2(np.float32(0.76) * np.log2(T.astype(np.float32))).astype(np.float64)
    t2 = T * T
    t4 = t2 * t2
    t8 = t4 * t4
    t16 = t8 * t8
    c = t16 * t2 * T
    y2 = y * y
    y4 = y2 * y2
    y8 = y4 * y4
    y16 = y8 * y8
    a = y16 * y8 * y
    return y + y * ((c - a) / (13.0 * a + 12.0 * c))


def _ulps(r, ref):
    return np.abs(r - ref) / np.spacing(ref)


def test_within_two_ulp_over_the_fast_range():
    rng = np.random.default_rng(7)
    T = 10.0 ** rng.uniform(-6.0, 6.0, 400_000)
    assert _ulps(_visc_pow(T), np.power(T, 0.76)).max() <= 2.0


def test_within_one_ulp_near_unit_temperature():
    # nondimensional flows sit near T = 1 (Taylor-Green, HIT, shear layer)
    rng = np.random.default_rng(8)
    T = 10.0 ** rng.uniform(-1.0, 1.0, 400_000)
    assert _ulps(_visc_pow(T), np.power(T, 0.76)).max() <= 1.0


def test_cubic_step_error_scale():
    # the step leaves ~ (n^2 - 1)/12 e^3 = 52 e^3 of an estimate error e
    # (n = 25): e = 1e-6, the FP32 estimate's worst case on [1e-6, 1e6], lands
    # within 2 ulp; e = 1e-5 would leave 5e-14, so the estimate needs the
    # accuracy of FP32 log2 and exp2
    rng = np.random.default_rng(9)
    T = 10.0 ** rng.uniform(-3.0, 3.0, 100_000)
    ref = np.power(T, 0.76)
    sign = rng.choice([-1.0, 1.0], T.size)
    c = T ** 19
    for e, bound in ((1e-6, 2.0), (1e-5, 600.0)):
        y = ref * (1.0 + e * sign)
        a = y ** 25
        r = y + y * ((c - a) / (13.0 * a + 12.0 * c))
        err = np.abs(r / ref - 1.0).max()
        assert _ulps(r, ref).max() <= bound
        assert err <= 60.0 * e ** 3 + 4e-16
