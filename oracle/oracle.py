"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a C++ restatement of the RS + MTJ Java code on the pressure
path (see mtj.hpp, mesh.hpp and physics.hpp for the per-file citations).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
it, always as the checker; the GPU product never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from ressim_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    d, i, vp = C.c_double, C.c_int, C.c_void_p
    P = C.POINTER
    L.orc_solve.restype = i
    L.orc_ilu.restype = i
    L.orc_ssor.restype = i
    L.orc_csr_op.restype = i
    L.orc_zero_rows.restype = i
    L.orc_dgesv.restype = i
    L.orc_mesh_create.restype = vp
    L.orc_mesh_create.argtypes = [i, i, i, i, P(d), d, d, d, d, d, d, P(d), P(i), C.c_char_p, i]
    L.orc_mesh_destroy.argtypes = [vp]
    L.orc_mesh_mpfa.argtypes = [vp, d, i, C.c_char_p, i]
    L.orc_mesh_test.argtypes = [vp, C.c_char_p, i]
    L.orc_mesh_counts.argtypes = [vp, P(C.c_longlong)]
    L.orc_mesh_geometry.argtypes = [vp, P(d), P(d), P(d), P(d), P(d), P(d)]
    L.orc_mesh_connections.argtypes = [vp, P(C.c_int32)]
    L.orc_mesh_md.argtypes = [vp, P(C.c_int32), P(C.c_int32), P(d)]
    L.orc_mesh_set_md.argtypes = [vp, P(C.c_int32), P(C.c_int32), P(d)]
    L.orc_mesh_pattern.argtypes = [vp, i, P(C.c_int32), P(C.c_int32), P(C.c_longlong)]
    L.orc_sim_create.restype = vp
    L.orc_sim_create.argtypes = [vp, P(abi.rsg_blackoil), P(abi.rsg_corey), P(d), P(d), i, P(abi.rsg_source),
                                 P(abi.rsg_initial), P(abi.rsg_runspec), P(i), C.c_char_p, i]
    L.orc_sim_destroy.argtypes = [vp]
    L.orc_sim_create_cubic.restype = vp
    L.orc_sim_create_cubic.argtypes = [vp, P(abi.rsg_cubic_fluid), P(abi.rsg_corey), P(d), P(d), i,
                                       P(abi.rsg_source), P(abi.rsg_initial), P(abi.rsg_runspec), P(i), C.c_char_p, i]
    L.orc_sim_step.argtypes = [vp, d, P(abi.rsg_step_info), C.c_char_p, i]
    L.orc_sim_retract.argtypes = [vp]
    L.orc_sim_set_rock_tables.argtypes = [vp, P(abi.rsg_rock_tables), C.c_char_p, i]
    L.orc_sim_set_rock_tables.restype = i
    L.orc_sim_state.argtypes = [vp, P(d), P(d), P(d)]
    L.orc_sim_jacobian.argtypes = [vp, P(d), P(d)]
    L.orc_sim_residual_volume.argtypes = [vp, P(d), P(d)]
    L.orc_sim_eval_cells.argtypes = [vp, P(d), P(d), P(d), P(d), P(d)]
    L.orc_sim_eval_cells.restype = i
    L.orc_sim_time.restype = d
    L.orc_sim_time.argtypes = [vp]
    L.orc_sim_last_dn.argtypes = [vp, P(d)]
    L.orc_function_eval.argtypes = [P(abi.rsg_function), i, i, P(d), P(d)]
    L.orc_sim_calculate_dt.argtypes = [vp, d, P(abi.rsg_dt_control), P(d), P(abi.rsg_dt_factors)]
    L.orc_sim_throughput_factor.restype = d
    L.orc_sim_throughput_factor.argtypes = [vp, P(abi.rsg_dt_control)]
    L.orc_sim_step_to.argtypes = [vp, d, P(abi.rsg_dt_control), P(d), P(abi.rsg_step_to_info), C.c_char_p, i]
    L.orc_cubic_roots.argtypes = [d, d, d, P(d)]
    L.orc_cubic_phase_state.argtypes = [P(abi.rsg_cubic_fluid), i, P(d), P(d), P(d), P(d), P(i), C.c_char_p, i]
    L.orc_amg_create.restype = vp
    L.orc_amg_create.argtypes = [i, i, P(C.c_int32), P(C.c_int32), P(d), P(i), C.c_char_p, i]
    L.orc_amg_destroy.argtypes = [vp]
    L.orc_amg_levels.argtypes = [vp]
    L.orc_amg_levels.restype = i
    L.orc_amg_level_sizes.argtypes = [vp, i, P(C.c_int32)]
    L.orc_amg_level_get.argtypes = [vp, i, P(C.c_int32), P(C.c_int32), P(d), P(C.c_int32), P(C.c_int32),
                                    P(C.c_int32), P(d)]
    L.orc_amg_apply.argtypes = [vp, P(d), P(d), i, C.c_char_p, i]
    L.orc_amg_apply.restype = i


class OracleError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS.get(status, status)}: {msg}")
        self.status = status


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def solve(method, precond, rowptr, col, val, b, x0, rtol=1e-5, atol=1e-50, dtol=1e5, maxit=100000, restart=30,
          omega=(1.0, 1.0), raise_on_fail=True):
    """IterativeSolver.solve on the CPU; returns (x, iterations, residual, history, status)."""
    rowptr, col, val, b = _i32(rowptr), _i32(col), _f64(val), _f64(b)
    x = _f64(x0).copy()
    n = len(b)
    it = C.c_int(0)
    res = C.c_double(0)
    hist = np.zeros(maxit * 2 + 64)
    hl = C.c_int(0)
    err = C.create_string_buffer(512)
    st = lib().orc_solve(method, precond, n, len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(val), abi.dptr(b),
                         abi.dptr(x), C.c_double(rtol), C.c_double(atol), C.c_double(dtol), maxit, restart,
                         C.c_double(omega[0]), C.c_double(omega[1]), C.byref(it), C.byref(res), abi.dptr(hist),
                         len(hist), C.byref(hl), err, 512)
    if st != 0 and raise_on_fail:
        raise OracleError(st, err.value.decode())
    return x, it.value, res.value, hist[: min(hl.value, len(hist))].copy(), st


def ilu(rowptr, col, val, b=None, trans=False):
    """ILU(0) factors (and optionally apply / transApply to b)."""
    rowptr, col, val = _i32(rowptr), _i32(col), _f64(val)
    n = len(rowptr) - 1
    LU = np.zeros(len(col))
    x = np.zeros(n)
    bb = _f64(b) if b is not None else None
    err = C.create_string_buffer(512)
    st = lib().orc_ilu(n, len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(val), abi.dptr(bb),
                       abi.dptr(x) if b is not None else abi.dptr(None), int(trans), abi.dptr(LU), err, 512)
    if st != 0:
        raise OracleError(st, err.value.decode())
    return LU, (x if b is not None else None)


def ssor(rowptr, col, val, b, x0, omega_f=1.0, omega_r=1.0, reverse=True):
    rowptr, col, val, b = _i32(rowptr), _i32(col), _f64(val), _f64(b)
    x = _f64(x0).copy()
    err = C.create_string_buffer(512)
    st = lib().orc_ssor(len(b), len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(val), abi.dptr(b), abi.dptr(x),
                        C.c_double(omega_f), C.c_double(omega_r), int(reverse), err, 512)
    if st != 0:
        raise OracleError(st, err.value.decode())
    return x


def csr_op(kind, rowptr, col, val, x, y=None, alpha=1.0):
    rowptr, col, val, x = _i32(rowptr), _i32(col), _f64(val), _f64(x)
    n = len(rowptr) - 1
    y = np.zeros(n) if y is None else _f64(y).copy()
    lib().orc_csr_op(kind, n, len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(val), C.c_double(alpha),
                     abi.dptr(x), abi.dptr(y))
    return y


def zero_rows(rowptr, col, val, diagonal, rows):
    rowptr, col, rows = _i32(rowptr), _i32(col), _i32(rows)
    v = _f64(val).copy()
    st = lib().orc_zero_rows(len(rowptr) - 1, len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(v),
                             C.c_double(diagonal), len(rows), abi.iptr(rows))
    if st != 0:
        raise OracleError(st, "zeroRows")
    return v


def dgesv(A, B):
    A = np.asfortranarray(A, dtype=np.float64).copy(order="F")
    B = np.asfortranarray(B, dtype=np.float64).copy(order="F")
    n = A.shape[0]
    nrhs = B.shape[1] if B.ndim == 2 else 1
    info = lib().orc_dgesv(n, nrhs, A.ctypes.data_as(C.POINTER(C.c_double)), B.ctypes.data_as(C.POINTER(C.c_double)))
    return info, B


class Mesh:
    """Structured RS mesh with geometry, topology and transmissibilities."""

    def __init__(self, dim, ni, nj, nk, coords=None, perm=None, x0=0.0, y0=0.0, z0=0.0, dx=1.0, dy=1.0, dz=-1.0):
        st = C.c_int(0)
        err = C.create_string_buffer(512)
        self._coords = _f64(coords) if coords is not None else None
        self._perm = _f64(perm) if perm is not None else None
        self.h = lib().orc_mesh_create(dim, ni, nj, nk, abi.dptr(self._coords), x0, y0, z0, dx, dy, dz,
                                       abi.dptr(self._perm), C.byref(st), err, 512)
        if not self.h:
            raise OracleError(st.value, err.value.decode())
        self.dim = dim

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None

    def mpfa(self, continuity=1.0, tpfa=False, lmethod=False):
        """O-method MPFA (default), TPFA, or the L-method (3-D)."""
        err = C.create_string_buffer(512)
        st = lib().orc_mesh_mpfa(self.h, continuity, 2 if lmethod else int(tpfa), err, 512)
        if st != 0:
            raise OracleError(st, err.value.decode())

    def test(self):
        err = C.create_string_buffer(512)
        st = lib().orc_mesh_test(self.h, err, 512)
        if st != 0:
            raise OracleError(st, err.value.decode())

    def counts(self):
        c = (C.c_longlong * 5)()
        lib().orc_mesh_counts(self.h, c)
        return dict(elements=c[0], connections=c[1], md=c[2], points=c[3], interfaces=c[4])

    def geometry(self):
        k = self.counts()
        centers = np.zeros((k["elements"], 3))
        vols = np.zeros(k["elements"])
        pts = np.zeros((k["points"], 3))
        inorm = np.zeros((k["interfaces"], 3))
        icen = np.zeros((k["interfaces"], 3))
        iarea = np.zeros(k["interfaces"])
        lib().orc_mesh_geometry(self.h, abi.dptr(centers), abi.dptr(vols), abi.dptr(pts), abi.dptr(inorm),
                                abi.dptr(icen), abi.dptr(iarea))
        return dict(centers=centers, volumes=vols, points=pts, inormal=inorm, icenter=icen, iarea=iarea)

    def connections(self):
        k = self.counts()
        conn = np.zeros((k["connections"], 2), dtype=np.int32)
        lib().orc_mesh_connections(self.h, abi.iptr(conn))
        return conn

    def transmissibilities(self):
        k = self.counts()
        ptr = np.zeros(k["connections"] + 1, dtype=np.int32)
        el = np.zeros(k["md"], dtype=np.int32)
        kk = np.zeros(k["md"])
        lib().orc_mesh_md(self.h, abi.iptr(ptr), abi.iptr(el), abi.dptr(kk))
        return ptr, el, kk

    def set_transmissibilities(self, ptr, el, kk):
        self._md = (_i32(ptr), _i32(el), _f64(kk))
        lib().orc_mesh_set_md(self.h, abi.iptr(self._md[0]), abi.iptr(self._md[1]), abi.dptr(self._md[2]))

    def pattern(self, which=0):
        nnz = C.c_longlong(0)
        lib().orc_mesh_pattern(self.h, which, abi.iptr(None), abi.iptr(None), C.byref(nnz))
        n = self.counts()["elements"]
        rp = np.zeros(n + 1, dtype=np.int32)
        col = np.zeros(nnz.value, dtype=np.int32)
        lib().orc_mesh_pattern(self.h, which, abi.iptr(rp), abi.iptr(col), C.byref(nnz))
        return rp, col


def function_eval(fn, x, nd=-1):
    """util/Function.get (nd < 0) or deriv(nd, ...) at the rows of x (m x dim)."""
    x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64)
    out = np.zeros(len(x))
    lib().orc_function_eval(C.byref(fn), nd, len(x), abi.dptr(x), abi.dptr(out))
    return out


def potential_matrix(mesh, rowptr, col):
    """PotentialCalculator.discretizeFlux (numerics/PotentialCalculator.java:319-333)
    as plain numpy over the oracle's MD lists (pattern from which=1)."""
    ptr, el, kk = mesh.transmissibilities()
    conn = mesh.connections()
    val = np.zeros(len(col))
    for c in range(len(conn)):
        i, j = conn[c]
        for q in range(ptr[c], ptr[c + 1]):
            k = el[q]
            a = rowptr[i] + np.searchsorted(col[rowptr[i]:rowptr[i + 1]], k)
            bpos = rowptr[j] + np.searchsorted(col[rowptr[j]:rowptr[j + 1]], k)
            val[a] += kk[q]
            val[bpos] += -kk[q]
    return val


def connection_flux(mesh, p):
    """PotentialCalculator.calculateFlux (numerics/PotentialCalculator.java:
    265-280) and LocalFlowRateAverage.computeDarcyFlux (upscale/
    LocalFlowRateAverage.java:123-137): flux[c] = 0 + t_1 p[el_1] + t_2 p[el_2]
    + ... in MD list order, one product and one sum rounded at a time."""
    ptr, el, kk = mesh.transmissibilities()
    p = _f64(p)
    flux = np.zeros(len(ptr) - 1)
    lens = np.diff(ptr)
    for q in range(int(lens.max()) if len(lens) else 0):
        m = lens > q
        idx = ptr[:-1][m] + q
        flux[m] += kk[idx] * p[el[idx]]
    return flux


def pressure_discretisation(mesh, bc):
    """upscale/PressureDiscretisation(mesh, bc) (upscale/
    PressureDiscretisation.java:59-187): the potential pattern and matrix,
    boundary rows e_i with b_i = p_i, GMRES(30) + ILU(0) from x = 0 with
    maxIterations 10000, rtol 1e-50, atol 1e-10, dtol 1e5.  bc: {cell: p}.
    Returns (x, iterations, matrix values, b)."""
    rp, col = mesh.pattern(1)
    cells = np.fromiter(bc.keys(), dtype=np.int32, count=len(bc))
    vals = np.fromiter(bc.values(), dtype=np.float64, count=len(bc))
    val = potential_matrix(mesh, rp, col)
    if len(cells):
        val = zero_rows(rp, col, val, 1.0, cells)
    b = np.zeros(len(rp) - 1)
    b[cells] = vals
    x, it, _, _, _ = solve(abi.GMRES, abi.PC_ILU, rp, col, val, b, np.zeros(len(b)), rtol=1e-50, atol=1e-10,
                           dtol=1e5, maxit=10000, restart=30)
    return x, it, val, b


class Simulator:
    """Field + Discretisation on the CPU."""

    def __init__(self, mesh, fluid, corey, porosity, compaction, sources, init, spec):
        self.mesh = mesh
        self._keep = (fluid, corey, _f64(porosity), _f64(compaction), sources, init, spec)
        st = C.c_int(0)
        err = C.create_string_buffer(512)
        create = lib().orc_sim_create_cubic if isinstance(fluid, abi.rsg_cubic_fluid) else lib().orc_sim_create
        self.h = create(mesh.h, C.byref(fluid), C.byref(corey), abi.dptr(self._keep[2]), abi.dptr(self._keep[3]),
                        len(sources), sources, C.byref(init), C.byref(spec), C.byref(st), err, 512)
        if not self.h:
            raise OracleError(st.value, err.value.decode())
        self.n = mesh.counts()["elements"]
        self.nc = fluid.nc

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    def step(self, dt, raise_on_fail=True):
        info = abi.rsg_step_info()
        err = C.create_string_buffer(512)
        st = lib().orc_sim_step(self.h, dt, C.byref(info), err, 512)
        if st != 0 and raise_on_fail:
            raise OracleError(st, err.value.decode())
        return info

    def time(self):
        return lib().orc_sim_time(self.h)

    def last_dn(self):
        """The last step's molar changes (nc x n) before the locked cells are reset."""
        out = np.zeros((self.nc, self.n))
        lib().orc_sim_last_dn(self.h, abi.dptr(out))
        return out

    def calculate_dt(self, dt, ctl):
        out = C.c_double(0)
        f = abi.rsg_dt_factors()
        lib().orc_sim_calculate_dt(self.h, dt, C.byref(ctl), C.byref(out), C.byref(f))
        return out.value, f

    def throughput_factor(self, ctl):
        return lib().orc_sim_throughput_factor(self.h, C.byref(ctl))

    def step_to(self, end_time, ctl, dt):
        """TimeStepper.stepTo; returns (status, dt carried to the next call, info)."""
        d = C.c_double(dt)
        info = abi.rsg_step_to_info()
        err = C.create_string_buffer(512)
        st = lib().orc_sim_step_to(self.h, end_time, C.byref(ctl), C.byref(d), C.byref(info), err, 512)
        return st, d.value, info

    def retract(self):
        lib().orc_sim_retract(self.h)

    def set_rock_tables(self, tables):
        """TabularRockFluid / ThreePhaseTabularRockFluid in place of Corey."""
        self._tables = tables
        err = C.create_string_buffer(512)
        st = lib().orc_sim_set_rock_tables(self.h, C.byref(tables), err, 512)
        if st != 0:
            raise OracleError(st, err.value.decode())

    def state(self):
        p = np.zeros(self.n)
        N = np.zeros(self.nc * self.n)
        S = np.zeros(3 * self.n)
        lib().orc_sim_state(self.h, abi.dptr(p), abi.dptr(N), abi.dptr(S))
        return p, N.reshape(self.nc, self.n), S.reshape(3, self.n)

    def jacobian(self, nnz):
        v = np.zeros(nnz)
        r = np.zeros(self.n)
        lib().orc_sim_jacobian(self.h, abi.dptr(v), abi.dptr(r))
        return v, r

    def residual_volume(self):
        R = np.zeros(self.n)
        d = np.zeros(self.n)
        lib().orc_sim_residual_volume(self.h, abi.dptr(R), abi.dptr(d))
        return R, d

    def eval_cells(self, p, N):
        """Re-evaluate every cell at pressures p (n) and moles N (nc x n):
        returns R, dR/dp and dR/dN (nc x n); the simulator keeps that state."""
        p, N = _f64(p), _f64(N)
        R, dRdp, dRdN = np.zeros(self.n), np.zeros(self.n), np.zeros_like(N)
        st = lib().orc_sim_eval_cells(self.h, abi.dptr(p), abi.dptr(N), abi.dptr(R), abi.dptr(dRdp), abi.dptr(dRdN))
        if st != 0:
            raise OracleError(st, "CV secondaries")
        return R, dRdp, dRdN


class AMG:
    """MTJ AMG() on the CPU: hierarchy (per level: A, aggregates pt,
    interpolation I in CompColMatrix form) and the V-cycle apply."""

    def __init__(self, rowptr, col, val):
        rowptr, col, val = _i32(rowptr), _i32(col), _f64(val)
        st = C.c_int(0)
        err = C.create_string_buffer(512)
        self.h = lib().orc_amg_create(len(rowptr) - 1, len(col), abi.iptr(rowptr), abi.iptr(col), abi.dptr(val),
                                      C.byref(st), err, 512)
        if not self.h:
            raise OracleError(st.value, err.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_amg_destroy(self.h)
            self.h = None

    def levels(self):
        return lib().orc_amg_levels(self.h)

    def level(self, k):
        sz = np.zeros(4, np.int32)
        lib().orc_amg_level_sizes(self.h, k, abi.iptr(sz))
        n, nnz, c, pn = (int(v) for v in sz)
        rp = np.zeros(n + 1, np.int32)
        col = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1))
        pt = np.zeros(max(n, 1), np.int32) if c else None
        cp = np.zeros(c + 1, np.int32) if c else None
        ri = np.zeros(max(pn, 1), np.int32) if c else None
        iv = np.zeros(max(pn, 1)) if c else None
        lib().orc_amg_level_get(self.h, k, abi.iptr(rp), abi.iptr(col), abi.dptr(val), abi.iptr(pt), abi.iptr(cp),
                                abi.iptr(ri), abi.dptr(iv))
        out = {"n": n, "rowptr": rp, "col": col[:nnz], "val": val[:nnz], "c": c}
        if c:
            out.update(pt=pt[:n], colptr=cp, rowind=ri[:pn], Idata=iv[:pn])
        return out

    def apply(self, b, x0, trans=False):
        x = _f64(x0).copy()
        err = C.create_string_buffer(512)
        st = lib().orc_amg_apply(self.h, abi.dptr(_f64(b)), abi.dptr(x), int(trans), err, 512)
        if st != 0:
            raise OracleError(st, err.value.decode())
        return x


def cubic_roots(a0, a1, a2):
    """CubicEquation(a0, a1, a2): (smallest, middle, largest) root."""
    z = np.zeros(3)
    lib().orc_cubic_roots(a0, a1, a2, abi.dptr(z))
    return tuple(z)


def cubic_phase_state(fluid, p, T, N, phases=None):
    """CubicEquationOfState.calculatePhaseState per cell; returns (phases,
    flash iterations) in the rsg_cubic_phase_state layout."""
    p, T, N = _f64(p), _f64(T), _f64(N)
    n = len(p)
    nf = abi.cubic_fields(fluid.nc)
    ph = np.zeros((3, nf, n)) if phases is None else _f64(phases).copy()
    its = np.zeros(n, np.int32)
    err = C.create_string_buffer(512)
    st = lib().orc_cubic_phase_state(C.byref(fluid), n, abi.dptr(p), abi.dptr(T), abi.dptr(N), abi.dptr(ph),
                                     its.ctypes.data_as(C.POINTER(C.c_int)), err, 512)
    if st != 0:
        raise OracleError(st, err.value.decode())
    return ph, its
