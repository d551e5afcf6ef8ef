"""The no-allocation CG entry point (rsg_cg_diagonal_noalloc) against the
regular solver entry point (rsg_solver_* with CG and the diagonal
preconditioner) and against the oracle's CG + DiagonalPreconditioner
(mtj/src/no/uib/cipr/matrix/sparse/CG.java:58-87), through the C ABI.

The no-allocation variant serves callers that cannot allocate device memory
while they run: its workspace is a fixed static device array, so it must give
the same answer as the allocating solver on consecutive calls (the array keeps
the previous call's contents), report the same failures, fill the whole array
at its largest size, and refuse systems larger than the array.  This file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api

pytestmark = pytest.mark.gpu

MAX_ROWS = 1048576  # RSG_NOALLOC_MAX_ROWS


def spd_banded(n, band, seed):
    """Symmetric, strictly diagonally dominant banded matrix in CSR form."""
    g = np.random.Generator(np.random.PCG64(seed))
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - band), i):
            A[i, j] = A[j, i] = -g.random()
    A[np.arange(n), np.arange(n)] = -A.sum(axis=1) + 1.0 + g.random(n)
    rp, col, val = [0], [], []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        col += nz.tolist()
        val += A[i, nz].tolist()
        rp.append(len(col))
    return np.array(rp, np.int32), np.array(col, np.int32), np.array(val)


def tridiagonal(n, seed):
    """Tridiagonal, strictly diagonally dominant, symmetric, in CSR form."""
    g = np.random.Generator(np.random.PCG64(seed))
    off = -g.random(n - 1)
    diag = 2.5 + g.random(n)
    rows = np.concatenate([np.arange(n - 1), np.arange(n), np.arange(1, n)])
    cols = np.concatenate([np.arange(1, n), np.arange(n), np.arange(n - 1)])
    vals = np.concatenate([off, diag, off])
    o = np.lexsort((cols, rows))
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols[o].astype(np.int32), vals[o]


def need_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def noalloc(M, b, x0, rtol=1e-10, atol=1e-50, dtol=1e5, max_iter=100000):
    """One call through the C ABI on device copies of b and x0."""
    torch = need_cuda()
    d_rp, d_col, d_val = M.device_arrays()
    tb = torch.tensor(b, dtype=torch.float64, device="cuda")
    tx = torch.tensor(x0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    info = abi.rsg_solve_info()
    st = api.lib().rsg_cg_diagonal_noalloc(0, None, M.n, M.nnz, d_rp, d_col, d_val, tb.data_ptr(), tx.data_ptr(),
                                           rtol, atol, dtol, max_iter, C.byref(info))
    return st, tx.cpu().numpy(), info


def test_noalloc_cg_matches_regular_solver_and_oracle(ctx):
    need_cuda()
    n = 4000
    rp, col, val = spd_banded(n, 6, 11)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    for call in range(2):  # the second call reuses the array the first one left behind
        b = np.random.Generator(np.random.PCG64(100 + call)).standard_normal(n)
        ref = api.CG(ctx, abi.PC_DIAGONAL, rtol=1e-10)
        ref.set_matrix(M)
        x_ref = ref.solve(M, b, np.zeros(n))
        st, x, info = noalloc(M, b, np.zeros(n))
        assert st == 0, abi.STATUS.get(st, st)
        assert info.iterations == ref.last_info.iterations
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))
        assert np.linalg.norm(b - M.mult(x)) <= 1.01e-10 * np.linalg.norm(b)
        xo, it, _, _, sto = O.solve(abi.CG, abi.PC_DIAGONAL, rp, col, val, b, np.zeros(n), rtol=1e-10)
        assert sto == 0 and abs(info.iterations - it) <= 1
        assert np.max(np.abs(x - xo)) <= 1e-9 * np.max(np.abs(xo))


def test_noalloc_failure_statuses_match_regular_solver(ctx):
    """Iteration limit and divergence give the regular solver's status and
    monitor values, and a converging call right after a failed one (which
    left its state in the array) is unaffected."""
    need_cuda()
    n = 3000
    rp, col, val = spd_banded(n, 4, 12)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    b = np.random.Generator(np.random.PCG64(7)).standard_normal(n)
    for kw, want in ((dict(max_iter=2), abi.NOT_CONVERGED_ITERATIONS),
                     (dict(dtol=0.5), abi.NOT_CONVERGED_DIVERGENCE)):
        ref = api.CG(ctx, abi.PC_DIAGONAL, rtol=1e-10, dtol=kw.get("dtol", 1e5), max_iter=kw.get("max_iter", 100000))
        ref.set_matrix(M)
        x_ref = ref.solve(M, b, np.zeros(n), raise_on_fail=False)
        st, x, info = noalloc(M, b, np.zeros(n), **kw)
        assert st == want, abi.STATUS.get(st, st)
        assert info.reason == want
        assert info.iterations == ref.last_info.iterations
        assert info.residual == pytest.approx(ref.last_info.residual, rel=1e-12)
        assert np.max(np.abs(x - x_ref)) <= 1e-12 * max(np.max(np.abs(x_ref)), 1e-300)
        st, x, info = noalloc(M, b, np.zeros(n))
        assert st == 0 and np.linalg.norm(b - M.mult(x)) <= 1.01e-10 * np.linalg.norm(b)


def test_noalloc_zero_diagonal_is_reported_even_when_converged(ctx):
    """A zero diagonal fails like DiagonalPreconditioner.setMatrix, also when
    the starting vector already solves the system."""
    need_cuda()
    n = 500
    rp, col, val = tridiagonal(n, 3)
    d = [q for q in range(rp[17], rp[18]) if col[q] == 17][0]
    val[d] = 0.0
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    x0 = np.random.Generator(np.random.PCG64(4)).standard_normal(n)
    b = M.mult(x0)
    st, _, info = noalloc(M, b, x0)
    assert st == abi.ZERO_PIVOT and info.reason == abi.ZERO_PIVOT
    st, _, _ = noalloc(M, np.random.Generator(np.random.PCG64(5)).standard_normal(n), np.zeros(n))
    assert st == abi.ZERO_PIVOT


def test_noalloc_at_largest_size_matches_regular_solver(ctx):
    """n = RSG_NOALLOC_MAX_ROWS fills the five vectors of the static array."""
    need_cuda()
    n = MAX_ROWS
    rp, col, val = tridiagonal(n, 9)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    b = np.random.Generator(np.random.PCG64(10)).standard_normal(n)
    ref = api.CG(ctx, abi.PC_DIAGONAL, rtol=1e-10)
    ref.set_matrix(M)
    x_ref = ref.solve(M, b, np.zeros(n))
    for _ in range(2):
        st, x, info = noalloc(M, b, np.zeros(n))
        assert st == 0, abi.STATUS.get(st, st)
        assert info.iterations == ref.last_info.iterations
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))


def test_noalloc_rejects_oversized_systems(ctx):
    """A system with one row more than the array holds is refused before any
    GPU work.  The matrix and vectors passed are real device arrays of that
    size, so every pointer handed over is valid for the sizes given."""
    torch = need_cuda()
    n = MAX_ROWS + 1
    rp, col, val = tridiagonal(n, 1)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    d_rp, d_col, d_val = M.device_arrays()
    tb = torch.ones(n, dtype=torch.float64, device="cuda")
    tx = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    info = abi.rsg_solve_info()
    st = api.lib().rsg_cg_diagonal_noalloc(0, None, n, M.nnz, d_rp, d_col, d_val, tb.data_ptr(), tx.data_ptr(),
                                           1e-8, 0.0, 1e5, 10, C.byref(info))
    assert st == abi.BAD_ARG
    assert not tx.any().item()
