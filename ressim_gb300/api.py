"""Python host binding of libresgpu (include/rsg.h), named after the
reference interfaces it replaces:

* ``CompRowMatrix``  - mtj sparse/CompRowMatrix (mult, multAdd, transMult, zeroRows)
* ``CG``, ``BiCGstab``, ``GMRES`` - mtj sparse iterative solvers, each with a
  preconditioner kind (``ILU``, ``SSOR``, ``DIAGONAL``, ``NONE``) and
  DefaultIterationMonitor tolerances
* ``Mesh``           - RS structured mesh + TransmissibilityComputer (O-MPFA)
* ``Discretisation`` - RS Field + Discretisation.solve(dt)

There is no CPU path: constructing a ``Context`` fails loudly when the CUDA
library or a Blackwell GPU is missing.
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libresgpu.so")
_lib = None


class RSGError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{abi.STATUS.get(status, status)}: {msg}")
        self.status = status


class IterativeSolverNotConvergedException(RSGError):
    """mtj sparse/IterativeSolverNotConvergedException: reason, residual, iterations."""

    def __init__(self, status, msg, residual, iterations):
        super().__init__(status, msg)
        self.reason = {1: "Iterations", 2: "Divergence", 3: "Breakdown"}.get(status, "Other")
        self.residual = residual
        self.iterations = iterations


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (there is no CPU fallback)")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    vp, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    P = C.POINTER
    PP = lambda: P(vp)  # noqa: E731
    sigs = {
        "rsg_abi_version": (i32, []),
        "rsg_sweep_mode": (i32, []),
        "rsg_sweep_plan_check": (i32, [i32, P(i32), P(i32), i32, i32, P(i64), C.c_char_p, i32]),
        "rsg_status_string": (C.c_char_p, [i32]),
        "rsg_context_create": (i32, [i32, PP()]),
        "rsg_context_destroy": (i32, [vp]),
        "rsg_context_last_error": (C.c_char_p, [vp]),
        "rsg_context_kernel_launches": (i64, [vp]),
        "rsg_context_synchronize": (i32, [vp]),
        "rsg_context_set_profiling": (i32, [vp, i32]),
        "rsg_context_profile_read": (i32, [vp, i32, P(d), P(i64), C.c_char_p, i32, P(i32)]),
        "rsg_context_profile_reset": (i32, [vp]),
        "rsg_context_timer_record": (i32, [vp, i32]),
        "rsg_context_timer_elapsed": (i32, [vp, i32, i32, P(d)]),
        "rsg_host_alloc": (i32, [C.c_size_t, P(vp)]),
        "rsg_host_free": (i32, [vp]),
        "rsg_csr_create": (i32, [vp, i32, i32, P(i32), P(i32), PP()]),
        "rsg_csr_destroy": (i32, [vp]),
        "rsg_csr_set_values": (i32, [vp, P(d)]),
        "rsg_csr_get_values": (i32, [vp, P(d)]),
        "rsg_csr_mult": (i32, [vp, P(d), P(d)]),
        "rsg_csr_mult_add": (i32, [vp, d, P(d), P(d)]),
        "rsg_csr_trans_mult": (i32, [vp, P(d), P(d)]),
        "rsg_csr_zero_rows": (i32, [vp, d, i32, P(i32)]),
        "rsg_csr_device_arrays": (i32, [vp, P(vp), P(vp), P(vp)]),
        "rsg_solver_create": (i32, [vp, i32, i32, PP()]),
        "rsg_solver_destroy": (i32, [vp]),
        "rsg_solver_set_monitor": (i32, [vp, d, d, d, i32]),
        "rsg_solver_set_restart": (i32, [vp, i32]),
        "rsg_solver_set_ssor": (i32, [vp, d, d, i32]),
        "rsg_solver_set_inner": (i32, [vp, i32, d]),
        "rsg_solver_setup": (i32, [vp, vp]),
        "rsg_solver_solve": (i32, [vp, vp, P(d), P(d), P(abi.rsg_solve_info)]),
        "rsg_solver_solve_device": (i32, [vp, vp, vp, vp, P(abi.rsg_solve_info)]),
        "rsg_precond_apply": (i32, [vp, P(d), P(d)]),
        "rsg_precond_trans_apply": (i32, [vp, P(d), P(d)]),
        "rsg_solver_history": (i32, [vp, i32, P(d), P(i32)]),
        "rsg_solver_amg_levels": (i32, [vp, P(i32)]),
        "rsg_solver_amg_level": (i32, [vp, i32, P(i32), P(i32), P(i32), P(d), P(i32), P(i32), P(i32), P(d)]),
        "rsg_cg_diagonal_noalloc": (i32, [i32, vp, i32, i32, vp, vp, vp, vp, vp, d, d, d, i32,
                                            P(abi.rsg_solve_info)]),
        "rsg_mesh_create_structured": (i32, [vp, i32, i32, i32, i32, P(d), d, d, d, d, d, d, P(d), PP()]),
        "rsg_mesh_destroy": (i32, [vp]),
        "rsg_mesh_compute_mpfa": (i32, [vp, d]),
        "rsg_mesh_compute_tpfa": (i32, [vp]),
        "rsg_mesh_get_counts": (i32, [vp, P(i64)]),
        "rsg_mesh_get_geometry": (i32, [vp, P(d), P(d)]),
        "rsg_mesh_get_connections": (i32, [vp, P(i32)]),
        "rsg_mesh_get_transmissibilities": (i32, [vp, P(i32), P(i32), P(d)]),
        "rsg_mesh_get_pattern": (i32, [vp, i32, P(i32), P(i32), P(i64)]),
        "rsg_mesh_assemble_potential": (i32, [vp, vp]),
        "rsg_mesh_compute_lmpfa": (i32, [vp]),
        "rsg_mesh_connection_flux": (i32, [vp, P(d), P(d)]),
        "rsg_mesh_get_interface_centers": (i32, [vp, P(d)]),
        "rsg_upscale_pressure": (i32, [vp, i32, P(i32), P(d), P(d), P(abi.rsg_solve_info)]),
        "rsg_mesh_transmissibility_adjoint": (i32, [vp, i32, P(d), P(d), P(d)]),
        "rsg_potential_adjoint": (i32, [vp, vp, vp, i32, P(i32), P(d), P(d), P(d), P(d), P(abi.rsg_solve_info)]),
        "rsg_sim_create": (i32, [vp, vp, P(abi.rsg_blackoil), P(abi.rsg_corey), P(d), P(d), i32, P(abi.rsg_source),
                                 P(abi.rsg_initial), P(abi.rsg_runspec), PP()]),
        "rsg_sim_destroy": (i32, [vp]),
        "rsg_sim_create_cubic": (i32, [vp, vp, P(abi.rsg_cubic_fluid), P(abi.rsg_corey), P(d), P(d), i32,
                                       P(abi.rsg_source), P(abi.rsg_initial), P(abi.rsg_runspec), PP()]),
        "rsg_sim_step": (i32, [vp, d, P(abi.rsg_step_info)]),
        "rsg_sim_retract": (i32, [vp]),
        "rsg_sim_save_state": (i32, [vp]),
        "rsg_sim_restore_state": (i32, [vp]),
        "rsg_sim_get_state": (i32, [vp, P(d), P(d), P(d)]),
        "rsg_sim_set_state": (i32, [vp, P(d), P(d)]),
        "rsg_sim_get_jacobian": (i32, [vp, P(d), P(d)]),
        "rsg_sim_get_residual_volume": (i32, [vp, P(d), P(d)]),
        "rsg_sim_get_time": (i32, [vp, P(d)]),
        "rsg_sim_forward": (i32, [vp, i32, P(d), i32, i32, P(i32), P(d), P(d), P(d), P(abi.rsg_adjoint_info)]),
        "rsg_sim_backward": (i32, [vp, d, P(d), P(d), P(d), P(abi.rsg_adjoint_info)]),
        "rsg_ensemble_step": (i32, [i32, P(vp), P(d), i32, P(abi.rsg_step_info), P(i32)]),
        "rsg_ensemble_step_batched": (i32, [i32, P(vp), P(d), i32, P(abi.rsg_step_info), P(i32)]),
        "rsg_solver_set_walk_shape": (i32, [vp, i32]),
        "rsg_solver_walk_shapes": (i32, [vp, P(i32)]),
        "rsg_sim_walk_shapes": (i32, [vp, P(i32)]),
        "rsg_solver_solve_batched": (i32, [i32, P(vp), P(vp), P(vp), P(vp), i32, P(abi.rsg_solve_info), P(i32)]),
        "rsg_sim_set_rock_tables": (i32, [vp, P(abi.rsg_rock_tables)]),
        "rsg_sim_write_restart": (i32, [vp, C.c_char_p]),
        "rsg_sim_read_restart": (i32, [vp, C.c_char_p]),
        "rsg_mm_read_matrix_size": (i32, [C.c_char_p, P(i32), P(i32), P(C.c_int64)]),
        "rsg_mm_read_csr": (i32, [C.c_char_p, i32, C.c_int64, P(i32), P(i32), P(d)]),
        "rsg_mm_write_csr": (i32, [C.c_char_p, i32, i32, P(i32), P(i32), P(d)]),
        "rsg_mm_read_vector_size": (i32, [C.c_char_p, P(i32)]),
        "rsg_mm_read_vector": (i32, [C.c_char_p, i32, P(d)]),
        "rsg_mm_write_vector": (i32, [C.c_char_p, i32, P(d)]),
        "rsg_cubic_phase_state": (i32, [vp, P(abi.rsg_cubic_fluid), i32, P(d), P(d), P(d), P(d), P(i32)]),
        "rsg_cubic_phase_state_cells": (i32, [vp, P(abi.rsg_cubic_fluid), i32, P(d), P(d), P(d), P(d), P(i32),
                                              P(i32)]),
        "rsg_sim_calculate_dt": (i32, [vp, d, P(abi.rsg_dt_control), P(d), P(abi.rsg_dt_factors)]),
        "rsg_sim_throughput_factor": (i32, [vp, P(abi.rsg_dt_control), P(d)]),
        "rsg_sim_step_to": (i32, [vp, d, P(abi.rsg_dt_control), P(d), P(abi.rsg_step_to_info)]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One CUDA device and one stream (rsg_context_*)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        st = lib().rsg_context_create(device, C.byref(h))
        if st != 0:
            raise RSGError(st, "rsg_context_create failed (a Blackwell GPU and libresgpu.so are required)")
        self.h = h
        # handles created from this context; destroyed before the context is
        self.children = weakref.WeakSet()

    def adopt(self, obj):
        self.children.add(obj)

    def check(self, st, what=""):
        if st != 0:
            raise RSGError(st, f"{what}: {lib().rsg_context_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            for child in list(getattr(self, "children", ())):
                child.release()
            lib().rsg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def kernel_launches(self):
        return lib().rsg_context_kernel_launches(self.h)

    def synchronize(self):
        self.check(lib().rsg_context_synchronize(self.h), "synchronize")

    def set_profiling(self, on):
        self.check(lib().rsg_context_set_profiling(self.h, int(on)), "set_profiling")

    def profile_reset(self):
        self.check(lib().rsg_context_profile_reset(self.h), "profile_reset")

    def timer_record(self, slot):
        self.check(lib().rsg_context_timer_record(self.h, slot), "timer_record")

    def timer_elapsed_ms(self, a, b):
        ms = C.c_double(0)
        self.check(lib().rsg_context_timer_elapsed(self.h, a, b, C.byref(ms)), "timer_elapsed")
        return ms.value

    def profile(self):
        ms = (C.c_double * 256)()
        ln = (C.c_int64 * 256)()
        names = C.create_string_buffer(16384)
        k = C.c_int32(0)
        self.check(lib().rsg_context_profile_read(self.h, 256, ms, ln, names, 16384, C.byref(k)), "profile_read")
        keys = names.value.decode().split("\n")[: k.value]
        return {keys[i]: (ms[i], ln[i]) for i in range(k.value)}


class CompRowMatrix:
    """mtj CompRowMatrix with the pattern resident on the GPU."""

    def __init__(self, ctx, n, rowptr, col, values=None):
        self.ctx = ctx
        self.n = int(n)
        self.rowptr = _i32(rowptr)
        self.col = _i32(col)
        h = C.c_void_p()
        ctx.check(lib().rsg_csr_create(ctx.h, self.n, len(self.col), abi.iptr(self.rowptr), abi.iptr(self.col),
                                       C.byref(h)), "rsg_csr_create")
        self.h = h
        ctx.adopt(self)
        if values is not None:
            self.set_values(values)

    def release(self):
        if getattr(self, "h", None):
            if self.ctx.h is not None:
                lib().rsg_csr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @property
    def nnz(self):
        return len(self.col)

    def set_values(self, values):
        v = _f64(values)
        if len(v) != self.nnz:
            raise ValueError(f"{len(v)} values for a pattern of {self.nnz} entries")
        self.ctx.check(lib().rsg_csr_set_values(self.h, abi.dptr(v)), "set_values")

    def get_values(self):
        v = np.zeros(self.nnz)
        self.ctx.check(lib().rsg_csr_get_values(self.h, abi.dptr(v)), "get_values")
        return v

    def mult(self, x):
        x = _f64(x)
        y = np.zeros(self.n)
        self.ctx.check(lib().rsg_csr_mult(self.h, abi.dptr(x), abi.dptr(y)), "mult")
        return y

    def mult_add(self, alpha, x, y):
        x = _f64(x)
        y = _f64(y).copy()
        self.ctx.check(lib().rsg_csr_mult_add(self.h, alpha, abi.dptr(x), abi.dptr(y)), "multAdd")
        return y

    def trans_mult(self, x):
        x = _f64(x)
        y = np.zeros(self.n)
        self.ctx.check(lib().rsg_csr_trans_mult(self.h, abi.dptr(x), abi.dptr(y)), "transMult")
        return y

    def device_arrays(self):
        """Device pointers (row_ptr, col, values) of the matrix."""
        rp, col, val = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self.ctx.check(lib().rsg_csr_device_arrays(self.h, C.byref(rp), C.byref(col), C.byref(val)), "device_arrays")
        return rp.value, col.value, val.value

    def zero_rows(self, diagonal, rows):
        r = _i32(rows)
        self.ctx.check(lib().rsg_csr_zero_rows(self.h, diagonal, len(r), abi.iptr(r)), "zeroRows")


class IterativeSolver:
    """IterativeSolver + Preconditioner pair (rsg_solver_*)."""

    method = None

    def __init__(self, ctx, precond=abi.PC_ILU, rtol=1e-5, atol=1e-50, dtol=1e5, max_iter=100000, restart=None):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(lib().rsg_solver_create(ctx.h, self.method, precond, C.byref(h)), "rsg_solver_create")
        self.h = h
        ctx.adopt(self)
        self.set_monitor(rtol, atol, dtol, max_iter)
        if restart is not None:
            ctx.check(lib().rsg_solver_set_restart(self.h, restart), "setRestart")
        self.last_info = None

    def release(self):
        if getattr(self, "h", None):
            if self.ctx.h is not None:
                lib().rsg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def set_monitor(self, rtol, atol, dtol, max_iter):
        self.ctx.check(lib().rsg_solver_set_monitor(self.h, rtol, atol, dtol, max_iter), "set_monitor")

    def set_inner(self, iterations, rtol):
        """Inner FP32 BiCGstab steps per outer step of the mixed-precision solver."""
        self.ctx.check(lib().rsg_solver_set_inner(self.h, iterations, rtol), "set_inner")

    def set_ssor(self, omega_f, omega_r, reverse=True):
        self.ctx.check(lib().rsg_solver_set_ssor(self.h, omega_f, omega_r, int(reverse)), "set_ssor")

    def set_matrix(self, A):
        """Preconditioner.setMatrix(A)"""
        self.ctx.check(lib().rsg_solver_setup(self.h, A.h), "setMatrix")

    def set_walk_shape(self, ctas):
        """ILU(0) level-walk cluster: 16 or 8 CTAs, 0 for the autotuner's timed
        choice (applied at the next set_matrix)."""
        self.ctx.check(lib().rsg_solver_set_walk_shape(self.h, int(ctas)), "set_walk_shape")

    def walk_shapes(self):
        """Clusters of the ILU(0) walks in use: FP64 lower, upper, FP32 lower,
        upper (0: no cluster walk)."""
        v = np.zeros(4, np.int32)
        self.ctx.check(lib().rsg_solver_walk_shapes(self.h, abi.iptr(v)), "walk_shapes")
        return v.tolist()

    def solve(self, A, b, x0, raise_on_fail=True):
        """IterativeSolver.solve(A, b, x): returns the new x."""
        b = _f64(b)
        x = _f64(x0).copy()
        info = abi.rsg_solve_info()
        st = lib().rsg_solver_solve(self.h, A.h, abi.dptr(b), abi.dptr(x), C.byref(info))
        self.last_info = info
        if st in (1, 2, 3) and raise_on_fail:
            raise IterativeSolverNotConvergedException(st, lib().rsg_context_last_error(self.ctx.h).decode(),
                                                       info.residual, info.iterations)
        if st not in (0, 1, 2, 3):
            self.ctx.check(st, "solve")
        return x

    def apply(self, b, x0=None, trans=False):
        """Preconditioner.apply / transApply on host vectors."""
        b = _f64(b)
        x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
        f = lib().rsg_precond_trans_apply if trans else lib().rsg_precond_apply
        self.ctx.check(f(self.h, abi.dptr(b), abi.dptr(x)), "apply")
        return x

    def amg_levels(self):
        n = C.c_int32(0)
        self.ctx.check(lib().rsg_solver_amg_levels(self.h, C.byref(n)), "amg_levels")
        return n.value

    def amg_level_sizes(self, k):
        """(rows, operator entries, coarse rows, interpolation entries) of AMG level k."""
        sz = np.zeros(4, np.int32)
        self.ctx.check(lib().rsg_solver_amg_level(self.h, k, abi.iptr(sz), *([None] * 7)), "amg_level")
        return tuple(int(v) for v in sz)

    def amg_level(self, k):
        """Level k of the AMG hierarchy: operator (CSR), aggregates and the
        interpolation operator by columns."""
        sz = np.zeros(4, np.int32)
        self.ctx.check(lib().rsg_solver_amg_level(self.h, k, abi.iptr(sz), *([None] * 7)), "amg_level")
        n, nnz, c, pn = (int(v) for v in sz)
        rp = np.zeros(n + 1, np.int32)
        col = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1))
        pt = np.zeros(max(n, 1), np.int32)
        cp = np.zeros(c + 1, np.int32)
        ri = np.zeros(max(pn, 1), np.int32)
        iv = np.zeros(max(pn, 1))
        self.ctx.check(lib().rsg_solver_amg_level(self.h, k, abi.iptr(sz), abi.iptr(rp), abi.iptr(col), abi.dptr(val),
                                                  abi.iptr(pt), abi.iptr(cp), abi.iptr(ri), abi.dptr(iv)),
                       "amg_level")
        out = {"n": n, "rowptr": rp, "col": col[:nnz], "val": val[:nnz], "c": c}
        if c:
            out.update(pt=pt[:n], colptr=cp, rowind=ri[:pn], Idata=iv[:pn])
        return out

    def history(self):
        n = C.c_int32(0)
        lib().rsg_solver_history(self.h, 0, abi.dptr(None), C.byref(n))
        out = np.zeros(max(n.value, 1))
        self.ctx.check(lib().rsg_solver_history(self.h, len(out), abi.dptr(out), C.byref(n)), "history")
        return out[: n.value]


class CG(IterativeSolver):
    method = abi.CG


class BiCGstab(IterativeSolver):
    method = abi.BICGSTAB


class GMRES(IterativeSolver):
    method = abi.GMRES


class MixedFGMRES(IterativeSolver):
    """FP64 flexible GMRES with an FP32 BiCGstab + FP32 preconditioner inside."""

    method = abi.FGMRES_MIXED


class Mesh:
    """Structured RS mesh; compute_mpfa() = O_MPFA.calculateTransmissibilities."""

    def __init__(self, ctx, dim, ni, nj, nk, perm, coords=None, x0=0.0, y0=0.0, z0=0.0, dx=1.0, dy=1.0, dz=-1.0):
        self.ctx = ctx
        self._perm = _f64(perm)
        self._coords = _f64(coords) if coords is not None else None
        h = C.c_void_p()
        ctx.check(lib().rsg_mesh_create_structured(ctx.h, dim, ni, nj, nk, abi.dptr(self._coords), x0, y0, z0, dx,
                                                   dy, dz, abi.dptr(self._perm), C.byref(h)), "mesh_create")
        self.h = h
        ctx.adopt(self)

    def release(self):
        if getattr(self, "h", None):
            if self.ctx.h is not None:
                lib().rsg_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def compute_mpfa(self, continuity=1.0):
        self.ctx.check(lib().rsg_mesh_compute_mpfa(self.h, continuity), "compute_mpfa")

    def compute_tpfa(self):
        """TPFA.calculateTransmissibilities: the two-point alternative to MPFA-O."""
        self.ctx.check(lib().rsg_mesh_compute_tpfa(self.h), "compute_tpfa")

    def compute_lmpfa(self):
        """L_MPFA.calculateTransmissibilities: the L-method (3-D)."""
        self.ctx.check(lib().rsg_mesh_compute_lmpfa(self.h), "compute_lmpfa")

    def counts(self):
        c = (C.c_int64 * 5)()
        self.ctx.check(lib().rsg_mesh_get_counts(self.h, c), "counts")
        return dict(elements=c[0], connections=c[1], md=c[2], points=c[3], pattern_nnz=c[4])

    def geometry(self):
        k = self.counts()
        centers = np.zeros((k["elements"], 3))
        vols = np.zeros(k["elements"])
        self.ctx.check(lib().rsg_mesh_get_geometry(self.h, abi.dptr(centers), abi.dptr(vols)), "geometry")
        return centers, vols

    def connections(self):
        k = self.counts()
        conn = np.zeros((k["connections"], 2), dtype=np.int32)
        self.ctx.check(lib().rsg_mesh_get_connections(self.h, abi.iptr(conn)), "connections")
        return conn

    def transmissibilities(self):
        k = self.counts()
        ptr = np.zeros(k["connections"] + 1, dtype=np.int32)
        el = np.zeros(k["md"], dtype=np.int32)
        kk = np.zeros(k["md"])
        self.ctx.check(lib().rsg_mesh_get_transmissibilities(self.h, abi.iptr(ptr), abi.iptr(el), abi.dptr(kk)),
                       "transmissibilities")
        return ptr, el, kk

    def pattern(self, which=0):
        nnz = C.c_int64(0)
        self.ctx.check(lib().rsg_mesh_get_pattern(self.h, which, abi.iptr(None), abi.iptr(None), C.byref(nnz)),
                       "pattern")
        n = self.counts()["elements"]
        rp = np.zeros(n + 1, dtype=np.int32)
        col = np.zeros(nnz.value, dtype=np.int32)
        self.ctx.check(lib().rsg_mesh_get_pattern(self.h, which, abi.iptr(rp), abi.iptr(col), C.byref(nnz)),
                       "pattern")
        return rp, col

    def assemble_potential(self, A):
        self.ctx.check(lib().rsg_mesh_assemble_potential(self.h, A.h), "assemble_potential")

    def connection_flux(self, p):
        """flux[c] = sum_k t_k p[el_k] per connection (PotentialCalculator.calculateFlux,
        LocalFlowRateAverage.computeDarcyFlux)."""
        p = _f64(p)
        out = np.zeros(self.counts()["connections"])
        self.ctx.check(lib().rsg_mesh_connection_flux(self.h, abi.dptr(p), abi.dptr(out)), "connection_flux")
        return out

    def interface_centers(self):
        """Centre of each connection's here interface, (connections, 3)."""
        out = np.zeros((self.counts()["connections"], 3))
        self.ctx.check(lib().rsg_mesh_get_interface_centers(self.h, abi.dptr(out)), "interface_centers")
        return out

    def transmissibility_adjoint(self, conn_weights, cell_potentials):
        """sum_k sum_c mu_k[c] d(sum_m t_cm phi_k[el_m]) / d log K_e for every element e."""
        mu = np.ascontiguousarray(np.atleast_2d(_f64(conn_weights)))
        phi = np.ascontiguousarray(np.atleast_2d(_f64(cell_potentials)))
        if mu.shape[0] != phi.shape[0]:
            raise ValueError("one potential vector per weight vector")
        out = np.zeros(self.counts()["elements"])
        self.ctx.check(lib().rsg_mesh_transmissibility_adjoint(self.h, mu.shape[0], abi.dptr(mu), abi.dptr(phi),
                                                               abi.dptr(out)), "transmissibility_adjoint")
        return out

    def potential_adjoint(self, solver, A, fixed, p, dJdp):
        """Gradient of J(p) with respect to per-element log-permeability for the
        steady potential problem A(theta) p = b (fixed rows identity).
        Returns (dJ/dlogk, lambda); solver.last_info holds the transposed solve."""
        fixed = np.ascontiguousarray(fixed, dtype=np.int32)
        n = self.counts()["elements"]
        p, w = _f64(p), _f64(dJdp)
        lam = np.zeros(n)
        grad = np.zeros(n)
        info = abi.rsg_solve_info()
        st = lib().rsg_potential_adjoint(self.h, solver.h, A.h, len(fixed), abi.iptr(fixed), abi.dptr(p),
                                         abi.dptr(w), abi.dptr(lam), abi.dptr(grad), C.byref(info))
        solver.last_info = info
        self.ctx.check(st, "potential_adjoint")
        return grad, lam


class Discretisation:
    """RS Field + Discretisation on the GPU: step(dt) = Discretisation.solve(dt)."""

    def __init__(self, ctx, mesh, fluid, corey, porosity, compaction, sources, init, spec):
        self.ctx = ctx
        self.mesh = mesh
        self._keep = (fluid, corey, _f64(porosity), _f64(compaction), sources, init, spec)
        h = C.c_void_p()
        create = lib().rsg_sim_create_cubic if isinstance(fluid, abi.rsg_cubic_fluid) else lib().rsg_sim_create
        ctx.check(create(ctx.h, mesh.h, C.byref(fluid), C.byref(corey), abi.dptr(self._keep[2]), abi.dptr(self._keep[3]),
                         len(sources), sources, C.byref(init), C.byref(spec), C.byref(h)), "sim_create")
        self.h = h
        ctx.adopt(self)
        self.n = mesh.counts()["elements"]
        self.nc = fluid.nc

    def release(self):
        if getattr(self, "h", None):
            if self.ctx.h is not None:
                lib().rsg_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def step(self, dt, raise_on_fail=True):
        info = abi.rsg_step_info()
        st = lib().rsg_sim_step(self.h, dt, C.byref(info))
        if st != 0 and raise_on_fail:
            self.ctx.check(st, "Discretisation.solve")
        return info

    def save_state(self):
        """Keeps a device-side copy of the whole state (rsg_sim_save_state)."""
        self.ctx.check(lib().rsg_sim_save_state(self.h), "save_state")

    def restore_state(self):
        """Returns to the state kept by save_state; the same steps then repeat bit for bit."""
        self.ctx.check(lib().rsg_sim_restore_state(self.h), "restore_state")

    def retract(self):
        self.ctx.check(lib().rsg_sim_retract(self.h), "retract")

    def set_rock_tables(self, tables):
        """TabularRockFluid / ThreePhaseTabularRockFluid (abi.rsg_rock_tables)
        in place of the Corey model; the tables are copied."""
        self.ctx.check(lib().rsg_sim_set_rock_tables(self.h, C.byref(tables)), "set_rock_tables")

    def walk_shapes(self):
        """Clusters of the pressure solver's ILU(0) walks (see
        IterativeSolver.walk_shapes)."""
        v = np.zeros(4, np.int32)
        self.ctx.check(lib().rsg_sim_walk_shapes(self.h, abi.iptr(v)), "walk_shapes")
        return v.tolist()

    def write_restart(self, path):
        """The primary state (time, p, reference p, T, N) to a restart file."""
        self.ctx.check(lib().rsg_sim_write_restart(self.h, os.fsencode(path)), "write_restart")

    def read_restart(self, path):
        """Restart from a file written by write_restart (Field(Field, ...))."""
        self.ctx.check(lib().rsg_sim_read_restart(self.h, os.fsencode(path)), "read_restart")

    def time(self):
        """Field.getTime [s]."""
        t = C.c_double(0)
        self.ctx.check(lib().rsg_sim_get_time(self.h, C.byref(t)), "time")
        return t.value

    def calculate_dt(self, dt, ctl):
        """Discretisation.calculateDt: (next dt, rsg_dt_factors)."""
        out = C.c_double(0)
        f = abi.rsg_dt_factors()
        self.ctx.check(lib().rsg_sim_calculate_dt(self.h, dt, C.byref(ctl), C.byref(out), C.byref(f)), "calculateDt")
        return out.value, f

    def throughput_factor(self, ctl):
        out = C.c_double(0)
        self.ctx.check(lib().rsg_sim_throughput_factor(self.h, C.byref(ctl), C.byref(out)), "throughputFactor")
        return out.value

    def step_to(self, end_time, ctl, dt):
        """TimeStepper.stepTo: (status, dt carried to the next call, rsg_step_to_info).
        A status other than 0 is a failure the time step could not be reduced past."""
        d = C.c_double(dt)
        info = abi.rsg_step_to_info()
        st = lib().rsg_sim_step_to(self.h, end_time, C.byref(ctl), C.byref(d), C.byref(info))
        if st not in (0, 1, 2, 3, 7, 8, 13):
            self.ctx.check(st, "stepTo")
        return st, d.value, info

    def forward(self, dts, checkpoint_every, cells, component_weights, cell_weights=None):
        """Recorded forward run for the adjoint: returns (J, rsg_adjoint_info),
        J = sum over steps, listed cells and components of
        cell_weight * component_weight * dN (moles into the cell before locking)."""
        dts = _f64(np.atleast_1d(dts))
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        cw = _f64(np.ones(len(cells)) if cell_weights is None else cell_weights)
        comp = np.zeros(self.nc)
        comp[:len(component_weights)] = component_weights
        J = C.c_double(0)
        info = abi.rsg_adjoint_info()
        self.ctx.check(lib().rsg_sim_forward(self.h, len(dts), abi.dptr(dts), checkpoint_every, len(cells),
                                             abi.iptr(cells), abi.dptr(cw), abi.dptr(comp), C.byref(J),
                                             C.byref(info)), "forward")
        return J.value, info

    def backward(self, rtol=1e-12):
        """Adjoint sweep of the last forward(): (dJ/dlogk, dJ/dp0, dJ/dN0, rsg_adjoint_info)."""
        grad = np.zeros(self.mesh.counts()["elements"])
        dp0 = np.zeros(self.n)
        dN0 = np.zeros((self.nc, self.n))
        info = abi.rsg_adjoint_info()
        self.ctx.check(lib().rsg_sim_backward(self.h, rtol, abi.dptr(grad), abi.dptr(dp0), abi.dptr(dN0),
                                              C.byref(info)), "backward")
        return grad, dp0, dN0, info

    def state(self):
        p = np.zeros(self.n)
        N = np.zeros(self.nc * self.n)
        S = np.zeros(3 * self.n)
        self.ctx.check(lib().rsg_sim_get_state(self.h, abi.dptr(p), abi.dptr(N), abi.dptr(S)), "state")
        return p, N.reshape(self.nc, self.n), S.reshape(3, self.n)

    def set_state(self, p, N):
        p = _f64(p)
        N = _f64(N).reshape(-1)
        self.ctx.check(lib().rsg_sim_set_state(self.h, abi.dptr(p), abi.dptr(N)), "set_state")

    def enable_jacobian_capture(self):
        st = lib().rsg_sim_get_jacobian(self.h, abi.dptr(None), abi.dptr(None))
        return st

    def jacobian(self, nnz):
        v = np.zeros(nnz)
        r = np.zeros(self.n)
        self.ctx.check(lib().rsg_sim_get_jacobian(self.h, abi.dptr(v), abi.dptr(r)), "jacobian")
        return v, r

    def residual_volume(self):
        R = np.zeros(self.n)
        d = np.zeros(self.n)
        self.ctx.check(lib().rsg_sim_get_residual_volume(self.h, abi.dptr(R), abi.dptr(d)), "residual_volume")
        return R, d


class PinnedArray:
    """numpy float64 view of page-locked host memory (rsg_host_alloc)."""

    def __init__(self, count):
        p = C.c_void_p()
        st = lib().rsg_host_alloc(max(1, count) * 8, C.byref(p))
        if st != 0:
            raise RSGError(st, "rsg_host_alloc")
        self.p = p
        self.array = np.ctypeslib.as_array((C.c_double * max(1, count)).from_address(p.value))[:count]

    def __del__(self):
        if getattr(self, "p", None):
            lib().rsg_host_free(self.p)
            self.p = None


def ensemble_step(sims, dts, max_concurrent=0):
    """Steps every Discretisation of `sims` (each on its own Context)
    concurrently; returns (per-member rsg_step_info list, statuses)."""
    n = len(sims)
    hs = (C.c_void_p * n)(*[s.h for s in sims])
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(dts, np.float64), (n,)))
    infos = (abi.rsg_step_info * n)()
    sts = np.zeros(n, np.int32)
    st = lib().rsg_ensemble_step(n, hs, abi.dptr(d), max_concurrent, infos, abi.iptr(sts))
    if st not in (0, 1, 2, 3, 7, 8, 13):
        raise RSGError(st, "ensemble_step")
    return list(infos), sts


def solve_batched(solvers, matrices, bs, x0s, precision=0):
    """IterativeSolver.solve for many systems in one persistent launch
    (rsg_solver_solve_batched): each solver (BiCGstab + ILU(0)) must have
    been set up with its matrix.  Returns (solutions, infos, statuses)."""
    n = len(solvers)
    xs = [np.array(x, dtype=np.float64, copy=True) for x in x0s]
    bs = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
    hs = (C.c_void_p * n)(*[s.h for s in solvers])
    hm = (C.c_void_p * n)(*[m.h for m in matrices])
    hb = (C.c_void_p * n)(*[b.ctypes.data for b in bs])
    hx = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
    infos = (abi.rsg_solve_info * n)()
    sts = np.zeros(n, np.int32)
    st = lib().rsg_solver_solve_batched(n, hs, hm, hb, hx, int(precision), infos, abi.iptr(sts))
    if st != 0 and not (sts == st).any():
        raise RSGError(st, "solve_batched")
    return xs, list(infos), sts


def read_matrix_market(path):
    """CompRowMatrix(MatrixVectorReader): (rows, cols, row_ptr, col, val) of a
    Matrix Market coordinate file."""
    rows, cols, nnz = C.c_int32(), C.c_int32(), C.c_int64()
    st = lib().rsg_mm_read_matrix_size(os.fsencode(path), C.byref(rows), C.byref(cols), C.byref(nnz))
    if st != 0:
        raise RSGError(st, f"read_matrix_market({path})")
    rp = np.zeros(rows.value + 1, np.int32)
    col = np.zeros(max(nnz.value, 1), np.int32)
    val = np.zeros(max(nnz.value, 1))
    st = lib().rsg_mm_read_csr(os.fsencode(path), rows.value, nnz.value, abi.iptr(rp), abi.iptr(col), abi.dptr(val))
    if st != 0:
        raise RSGError(st, f"read_matrix_market({path})")
    return rows.value, cols.value, rp, col[:nnz.value], val[:nnz.value]


def write_matrix_market(path, rows, cols, rowptr, col, val):
    """MatrixVectorWriter output of a CSR matrix (coordinate real general)."""
    rp, cl, v = _i32(rowptr), _i32(col), np.ascontiguousarray(val, np.float64)
    st = lib().rsg_mm_write_csr(os.fsencode(path), int(rows), int(cols), abi.iptr(rp), abi.iptr(cl), abi.dptr(v))
    if st != 0:
        raise RSGError(st, f"write_matrix_market({path})")


def read_matrix_market_vector(path):
    """DenseVector(MatrixVectorReader)."""
    n = C.c_int32()
    st = lib().rsg_mm_read_vector_size(os.fsencode(path), C.byref(n))
    if st != 0:
        raise RSGError(st, f"read_matrix_market_vector({path})")
    x = np.zeros(max(n.value, 1))
    st = lib().rsg_mm_read_vector(os.fsencode(path), n.value, abi.dptr(x))
    if st != 0:
        raise RSGError(st, f"read_matrix_market_vector({path})")
    return x[:n.value]


def write_matrix_market_vector(path, x):
    """MatrixVectorWriter output of a dense vector (array real)."""
    v = np.ascontiguousarray(x, np.float64)
    st = lib().rsg_mm_write_vector(os.fsencode(path), len(v), abi.dptr(v))
    if st != 0:
        raise RSGError(st, f"write_matrix_market_vector({path})")


def ensemble_step_batched(sims, dts, precision=0):
    """One time step of every Discretisation of `sims` in lockstep, with the
    pressure solves of all members in one persistent launch per Newton
    iteration (rsg_ensemble_step_batched).  precision 0: FP64 BiCGstab +
    ILU(0); 1: the mixed-precision solver (FP64 flexible GMRES around FP32
    BiCGstab + FP32 ILU(0)).  Returns (per-member rsg_step_info list,
    statuses)."""
    n = len(sims)
    hs = (C.c_void_p * n)(*[s.h for s in sims])
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(dts, np.float64), (n,)))
    infos = (abi.rsg_step_info * n)()
    sts = np.zeros(n, np.int32)
    st = lib().rsg_ensemble_step_batched(n, hs, abi.dptr(d), int(precision), infos, abi.iptr(sts))
    if st != 0 and not (sts == st).any():  # a failure of the call itself, not of one member's step
        raise RSGError(st, "ensemble_step_batched")
    return list(infos), sts


def cubic_phase_state(ctx, fluid, p, T, N, phases=None, per_cell=False):
    """CubicEquationOfState.calculatePhaseState for every cell on the GPU.
    N is (nc, n); phases (3, 6 + 2 nc, n) is in/out (zeros: no previous
    phases).  Returns (phases, flash iterations per cell); with per_cell,
    also the status of each cell instead of raising on the first failure."""
    p, T, N = _f64(p), _f64(T), _f64(N)
    n = len(p)
    nf = abi.cubic_fields(fluid.nc)
    ph = np.zeros((3, nf, n)) if phases is None else _f64(phases).copy()
    its = np.zeros(n, np.int32)
    if per_cell:
        sts = np.zeros(n, np.int32)
        ctx.check(lib().rsg_cubic_phase_state_cells(ctx.h, C.byref(fluid), n, abi.dptr(p), abi.dptr(T), abi.dptr(N),
                                                    abi.dptr(ph), abi.iptr(its), abi.iptr(sts)), "cubic_phase_state")
        return ph, its, sts
    ctx.check(lib().rsg_cubic_phase_state(ctx.h, C.byref(fluid), n, abi.dptr(p), abi.dptr(T), abi.dptr(N),
                                          abi.dptr(ph), abi.iptr(its)), "cubic_phase_state")
    return ph, its
