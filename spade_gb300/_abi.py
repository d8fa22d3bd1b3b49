"""ctypes mirror of include/gbns.h: descriptor structs and constants.

The structs here are byte-for-byte the C structs of the C ABI; the Python
API fills them and passes pointers to libgbns.so.
"""
import ctypes

ABI_VERSION = 1

OK = 0
ERR_INVALID = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_NONFINITE = -4
ERR_CAPACITY = -5
ERR_TIMEOUT = -6

COORDS_IDENTITY = 0
COORDS_TANH_Y = 1
COORDS_INTEGRATED_TANH_Y = 2

CONV_NONE = 0
CONV_CENT_KEEP = 1
CONV_TOTANI = 2
CONV_FWENO = 3
CONV_WENO5 = 4
CONV_HYBRID = 5
HYBRID_FULL_FLUX = 0
HYBRID_DISS_FLUX = 1

DISS_NONE = 0
DISS_PRESSURE = 1

SENSOR_CONST = 0
SENSOR_DUCROS = 1

VISC_NONE = 0
VISC_LR = 1

LAW_CONSTANT = 0
LAW_POWER = 1
LAW_SUTHERLAND = 2

PREC_FP64 = 0
PREC_FP32_FLUX = 1
PREC_FP64_FMA = 2

BC_PERIODIC = 0
BC_NONE = 1
BC_ISOTHERMAL_NOSLIP = 2
BC_SLIP_ADIABATIC = 3

RED_MAX_WAVESPEED = 0
RED_KINETIC = 1
RED_CONSERVED = 2
RED_HEALTH = 3


class GridDesc(ctypes.Structure):
    _fields_ = [
        ("nblk", ctypes.c_int32 * 3),
        ("ncell", ctypes.c_int32 * 3),
        ("ng", ctypes.c_int32),
        ("coords", ctypes.c_int32),
        ("bounds", ctypes.c_double * 6),
        ("coord_param", ctypes.c_double * 4),
    ]


class GasDesc(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("R", ctypes.c_double)]


class SchemeDesc(ctypes.Structure):
    _fields_ = [
        ("convective", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("weno_smooth", ctypes.c_int32),
        ("dissipation", ctypes.c_int32),
        ("sensor", ctypes.c_int32),
        ("viscous", ctypes.c_int32),
        ("visc_law", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("tile_variant", ctypes.c_int32),
        ("hybrid_flux", ctypes.c_int32),
        ("eps_p", ctypes.c_double),
        ("eps_T", ctypes.c_double),
        ("sensor_alpha", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("prandtl", ctypes.c_double),
        ("T_ref", ctypes.c_double),
        ("power", ctypes.c_double),
        ("S", ctypes.c_double),
        ("prandtl_inv", ctypes.c_double),
        ("gas", GasDesc),
        ("hybrid_sensor", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("hybrid_param", ctypes.c_double),
    ]


DEV_OK = 0
DEV_TMA_TIMEOUT = 1

SOURCE_CONST = 0
SOURCE_BODY_FORCE = 1
SOURCE_BODY_ACCEL = 2


class SourceDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("c", ctypes.c_double * 5),
        ("gas", GasDesc),
    ]


class BcDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32 * 6), ("t_wall", ctypes.c_double * 6)]


def grid_desc(nblk, ncell, ng, bounds, coords=COORDS_IDENTITY, coord_param=(0.0, 0.0, 0.0, 0.0)):
    g = GridDesc()
    for d in range(3):
        g.nblk[d] = int(nblk[d])
        g.ncell[d] = int(ncell[d])
    g.ng = int(ng)
    g.coords = int(coords)
    for i in range(6):
        g.bounds[i] = float(bounds[i])
    for i in range(4):
        g.coord_param[i] = float(coord_param[i])
    return g


def bc_desc(kinds, t_wall=(0.0,) * 6):
    b = BcDesc()
    for i in range(6):
        b.kind[i] = int(kinds[i])
        b.t_wall[i] = float(t_wall[i])
    return b
