"""ctypes mirror of the plain-data structs declared in include/rsg.h.

These are the input records of the C ABI (fluid tables, Corey parameters,
sources, initial values, run specification).  They carry no behaviour; the
helpers below build them from numpy arrays and keep the arrays alive for as
long as the struct is used.
"""
import ctypes as C

import numpy as np

MAX_COMPONENTS = 8

# rsg_status values (include/rsg.h)
STATUS = {
    0: "OK",
    1: "NOT_CONVERGED_ITERATIONS",
    2: "NOT_CONVERGED_DIVERGENCE",
    3: "NOT_CONVERGED_BREAKDOWN",
    4: "ZERO_PIVOT",
    5: "MISSING_DIAGONAL",
    6: "OUT_OF_PATTERN",
    7: "NONPOSITIVE_PRESSURE",
    8: "NEGATIVE_MOLES",
    9: "BAD_ARG",
    10: "CUDA_ERROR",
    11: "TIMEOUT",
    12: "UNSUPPORTED",
    13: "NEWTON_NOT_CONVERGED",
    14: "SINGULAR",
    15: "PHYSICS",
}
(OK, NOT_CONVERGED_ITERATIONS, NOT_CONVERGED_DIVERGENCE, NOT_CONVERGED_BREAKDOWN, ZERO_PIVOT, MISSING_DIAGONAL,
 OUT_OF_PATTERN, NONPOSITIVE_PRESSURE, NEGATIVE_MOLES, BAD_ARG, CUDA_ERROR, TIMEOUT, UNSUPPORTED,
 NEWTON_NOT_CONVERGED, SINGULAR, PHYSICS) = range(16)

CG, BICGSTAB, GMRES, FGMRES_MIXED = 0, 1, 2, 3
PC_NONE, PC_DIAGONAL, PC_ILU, PC_SSOR, PC_AMG = 0, 1, 2, 3, 4
FN_CONSTANT, FN_TABLE, FN_EVEN_TABLE = 0, 1, 2
SOURCE_FIXED, SOURCE_REGULAR = 0, 1

_dptr = C.POINTER(C.c_double)
_iptr = C.POINTER(C.c_int32)


class rsg_function(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("dim", C.c_int32),
        ("value", C.c_double),
        ("n", C.c_int32 * 3),
        ("coord", _dptr * 3),
        ("data", _dptr),
    ]


class rsg_blackoil(C.Structure):
    _fields_ = [
        ("nc", C.c_int32),
        ("molecular_weight", C.c_double * MAX_COMPONENTS),
        ("group", C.c_int32 * MAX_COMPONENTS),
        ("water_density", rsg_function),
        ("water_viscosity", rsg_function),
        ("water_enthalpy", rsg_function),
        ("bubble_point", rsg_function),
        ("dew_point", rsg_function),
        ("oil_density", rsg_function),
        ("gas_density", rsg_function),
        ("oil_viscosity", rsg_function),
        ("gas_viscosity", rsg_function),
        ("oil_enthalpy", rsg_function),
        ("gas_enthalpy", rsg_function),
    ]


RF_COREY, RF_TABULAR, RF_THREE_PHASE_TABULAR = 0, 1, 2


class rsg_rock_tables(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("krw", rsg_function),
        ("krg", rsg_function),
        ("krow", rsg_function),
        ("krog", rsg_function),
        ("kro", rsg_function),
        ("pcow", rsg_function),
        ("pcgo", rsg_function),
    ]


class rsg_corey(C.Structure):
    _fields_ = [
        ("Sr", C.c_double * 3),
        ("n", C.c_double * 3),
        ("ke", C.c_double * 3),
        ("cw", C.c_double),
        ("cow", C.c_double),
        ("cg", C.c_double),
        ("cog", C.c_double),
        ("aw", C.c_double),
        ("aow", C.c_double),
        ("ag", C.c_double),
        ("aog", C.c_double),
    ]


class rsg_source(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("num_elements", C.c_int32),
        ("elements", _iptr),
        ("q", C.c_double * MAX_COMPONENTS),
        ("temperature", C.c_double),
        ("fraction", C.c_double * MAX_COMPONENTS),
    ]


class rsg_initial(C.Structure):
    _fields_ = [
        ("datum_depth", C.c_double),
        ("datum_pressure", C.c_double),
        ("temperature", rsg_function),
        ("fraction", rsg_function * MAX_COMPONENTS),
    ]


class rsg_runspec(C.Structure):
    _fields_ = [
        ("max_nonlinear_pressure_iterations", C.c_int32),
        ("pressure_tolerance", C.c_double),
        ("linear_solver", C.c_int32),
        ("preconditioner", C.c_int32),
        ("max_linear_iterations", C.c_int32),
        ("relative_tolerance", C.c_double),
        ("absolute_tolerance", C.c_double),
        ("divergence_tolerance", C.c_double),
        ("truncate_negative_moles", C.c_int32),
        ("newton_stop_rule", C.c_int32),
        ("omega", C.c_double),
        ("ax", C.c_double),
        ("ay", C.c_double),
        ("gmres_restart", C.c_int32),
        ("inner_iterations", C.c_int32),
        ("inner_tolerance", C.c_double),
    ]


EOS_PR, EOS_SRK = 0, 1


class rsg_cubic_fluid(C.Structure):
    _fields_ = [
        ("nc", C.c_int32),
        ("eos", C.c_int32),
        ("Tc", C.c_double * MAX_COMPONENTS),
        ("pc", C.c_double * MAX_COMPONENTS),
        ("omega", C.c_double * MAX_COMPONENTS),
        ("Mw", C.c_double * MAX_COMPONENTS),
        ("Vc", C.c_double * MAX_COMPONENTS),
        ("shift", C.c_double * MAX_COMPONENTS),
        ("bic", C.c_double * (MAX_COMPONENTS * MAX_COMPONENTS)),
        ("flash_criteria", C.c_double),
        ("flash_tolerance", C.c_double),
        ("flash_max_iterations", C.c_int32),
        ("lbc", C.c_double * 5),
        ("water_density", rsg_function),
        ("water_viscosity", rsg_function),
    ]


def cubic_fields(nc):
    """Doubles per phase and cell in the rsg_cubic_phase_state layout."""
    return 6 + 2 * nc


class rsg_dt_control(C.Structure):
    _fields_ = [
        ("lambda_", C.c_double),
        ("target_residual_volume", C.c_double),
        ("target_nonlinear_iterations", C.c_int32),
        ("target_throughput", C.c_double),
        ("dt_min", C.c_double),
        ("dt_max", C.c_double),
    ]


def dt_control(dt_min, dt_max, lam=0.5, target_residual_volume=1e-2, target_nonlinear_iterations=5,
               target_throughput=0.5):
    """RunSpec's time-step keys with RunSpec's defaults."""
    c = rsg_dt_control()
    c.lambda_ = lam
    c.target_residual_volume = target_residual_volume
    c.target_nonlinear_iterations = target_nonlinear_iterations
    c.target_throughput = target_throughput
    c.dt_min = dt_min
    c.dt_max = dt_max
    return c


class rsg_dt_factors(C.Structure):
    _fields_ = [
        ("residual_volume", C.c_double),
        ("pressure_iterations", C.c_double),
        ("throughput", C.c_double),
        ("limit", C.c_int32),
    ]


class rsg_adjoint_info(C.Structure):
    _fields_ = [
        ("steps", C.c_int32),
        ("newton_iterations", C.c_int32),
        ("linear_iterations", C.c_int32),
        ("recomputed_steps", C.c_int32),
        ("backward_steps", C.c_int32),
        ("adjoint_linear_iterations", C.c_int32),
        ("objective", C.c_double),
    ]


class rsg_step_to_info(C.Structure):
    _fields_ = [
        ("steps", C.c_int32),
        ("retries", C.c_int32),
        ("newton_iterations", C.c_int32),
        ("linear_iterations", C.c_int32),
        ("time", C.c_double),
        ("status", C.c_int32),
    ]


class rsg_step_info(C.Structure):
    _fields_ = [
        ("newton_iterations", C.c_int32),
        ("linear_iterations", C.c_int32),
        ("dp_max", C.c_double),
        ("dp0", C.c_double),
        ("mass_balance_error", C.c_double),
        ("status", C.c_int32),
    ]


class rsg_solve_info(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("reason", C.c_int32),
        ("residual", C.c_double),
        ("initial_residual", C.c_double),
        ("inner_iterations", C.c_int32),
        ("refinements", C.c_int32),
    ]


def dptr(a):
    """Pointer to a contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return _dptr()
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError(f"expected a C-contiguous float64 array, got {a.dtype}")
    return a.ctypes.data_as(_dptr)


def iptr(a):
    if a is None:
        return _iptr()
    if a.dtype != np.int32 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError(f"expected a C-contiguous int32 array, got {a.dtype}")
    return a.ctypes.data_as(_iptr)


class Keep:
    """Holds numpy arrays referenced by raw pointers inside ctypes structs."""

    def __init__(self):
        self.arrays = []

    def f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.arrays.append(a)
        return a

    def i32(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.arrays.append(a)
        return a


def constant(value, dim=1):
    """util/ConstantValue"""
    f = rsg_function()
    f.kind = FN_CONSTANT
    f.dim = dim
    f.value = float(value)
    return f


def table(keep, coords, data):
    """util/LookupTable: coords is a list of 1-3 sorted axes, data has shape
    (n0, n1, n2) and is stored axis 0 fastest as LookupTable's "data" key."""
    f = rsg_function()
    f.kind = FN_TABLE
    f.dim = len(coords)
    data = np.asarray(data, dtype=np.float64)
    if data.shape != tuple(len(c) for c in coords):
        raise ValueError(f"table data of shape {data.shape} does not match axes of {[len(c) for c in coords]} points")
    for d, c in enumerate(coords):
        arr = keep.f64(c)
        f.n[d] = len(arr)
        f.coord[d] = dptr(arr)
    flat = keep.f64(data.reshape(-1, order="F"))
    f.data = dptr(flat)
    return f


def even_table(keep, ranges, data):
    """util/EvenLookupTable as its configuration gives it: per axis (xMin,
    xMax) and data of shape (n0, n1, n2); the knots are xMin + j (xMax - xMin)
    / (n - 1), summed one spacing at a time (EvenLookupTable.java:86-162)."""
    f = rsg_function()
    f.kind = FN_EVEN_TABLE
    f.dim = len(ranges)
    data = np.asarray(data, dtype=np.float64)
    if data.ndim != len(ranges):
        raise ValueError(f"table data has {data.ndim} axes, ranges give {len(ranges)}")
    for d, (lo, hi) in enumerate(ranges):
        arr = keep.f64([lo, hi])
        f.n[d] = data.shape[d]
        f.coord[d] = dptr(arr)
    flat = keep.f64(data.reshape(-1, order="F"))
    f.data = dptr(flat)
    return f
