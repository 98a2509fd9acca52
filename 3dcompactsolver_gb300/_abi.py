"""ctypes mirror of include/cs3d.h: the config struct and the constants.

The values of the enumerations equal the reference's enums: BC::BCType and
BC::BCKind (BC.hpp:10-11), Derivatives::Direct (Derivatives.hpp:48).
"""
import ctypes

OK, ERR_ARG, ERR_SHAPE, ERR_CUDA, ERR_NAN, ERR_ALLOC, ERR_STATE, ERR_NODEV = range(8)
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_SHAPE", 3: "ERR_CUDA", 4: "ERR_NAN",
                5: "ERR_ALLOC", 6: "ERR_STATE", 7: "ERR_NODEV", 8: "ERR_IO"}

PERIODIC_SOLVE, DIRICHLET_SOLVE = 0, 1
PERIODIC, SPONGE, ADIABATIC_WALL, MOVING_ADIABATIC_WALL, INLET = 0, 1, 2, 3, 4
DIRX, DIRY, DIRZ = 0, 1, 2
RK4, TVDRK3 = 0, 1
FP64, FP32_MIXED = 0, 1
SPONGE_REFERENCE, SPONGE_BANDS = 0, 1

# field indices of cs3d_get_field / cs3d_set_field
F_RHO1, F_RHOK, F_RHO2, F_RHOK2, F_U, F_SPONGE_AVG, F_SIGMA = 0, 5, 10, 15, 20, 27, 32
CONSERVED = ("rho", "rhoU", "rhoV", "rhoW", "rhoE")
PRIMITIVES = ("U", "V", "W", "p", "T", "mu", "sos")
NUM_FIELDS = 33


class Config(ctypes.Structure):
    """struct cs3d_config (include/cs3d.h)."""
    _fields_ = [
        ("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
        ("bc_type", ctypes.c_int * 3),
        ("bc_kind", ctypes.c_int * 6),
        ("alphaF", ctypes.c_double),
        ("mu_ref", ctypes.c_double),
        ("CFL", ctypes.c_double),
        ("dt_fixed", ctypes.c_double),
        ("filter_step", ctypes.c_int),
        ("rk", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("sponge_mode", ctypes.c_int),
        ("sponge_frac", ctypes.c_double * 6),
        ("wall_vel", ctypes.c_double * 12),
    ]

    @property
    def shape(self):
        """Array shape of one field in XYZ layout, as numpy sees it: (Nz, Ny, Nx)."""
        return (self.Nz, self.Ny, self.Nx)

    @property
    def npts(self):
        return self.Nx * self.Ny * self.Nz

    def copy(self, **changes):
        c = Config()
        ctypes.pointer(c)[0] = self
        for k, v in changes.items():
            setattr(c, k, v)
        return c


def make_config(N, L, bc_type=(PERIODIC_SOLVE,) * 3, bc_kind=(PERIODIC,) * 6, alphaF=0.49,
                mu_ref=1.0e-4, CFL=0.5, filter_step=1, rk=RK4, precision=FP64,
                sponge_mode=SPONGE_REFERENCE, sponge_frac=(0.0,) * 6, wall_vel=(0.0,) * 12,
                dt_fixed=0.0):
    """Build a Config; N and L are 3-tuples (x, y, z) or scalars."""
    if isinstance(N, int):
        N = (N, N, N)
    if isinstance(L, (int, float)):
        L = (float(L),) * 3
    c = Config()
    c.Nx, c.Ny, c.Nz = N
    c.Lx, c.Ly, c.Lz = L
    c.bc_type[:] = list(bc_type)
    c.bc_kind[:] = list(bc_kind)
    c.alphaF = alphaF
    c.mu_ref = mu_ref
    c.CFL = CFL
    c.dt_fixed = dt_fixed
    c.filter_step = filter_step
    c.rk = rk
    c.precision = precision
    c.sponge_mode = sponge_mode
    c.sponge_frac[:] = list(sponge_frac)
    c.wall_vel[:] = list(wall_vel)
    return c
