"""The no-allocation CG entry point (rsg_cg_diagonal_noalloc) against the
regular solver entry point (rsg_solver_* with CG and the diagonal
preconditioner), through the C ABI.

The no-allocation variant serves callers that cannot allocate device memory
while they run: its workspace is a fixed static device array, so it must give
the same answer as the allocating solver on consecutive calls (the array keeps
the previous call's contents) and must refuse systems larger than the array.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from ressim_gb300 import abi, api

pytestmark = pytest.mark.gpu


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


def test_noalloc_cg_matches_regular_solver(ctx):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = 4000
    rp, col, val = spd_banded(n, 6, 11)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    d_rp, d_col, d_val = M.device_arrays()
    L = api.lib()
    for call in range(2):
        b = np.random.Generator(np.random.PCG64(100 + call)).standard_normal(n)
        ref = api.CG(ctx, abi.PC_DIAGONAL, rtol=1e-10)
        ref.set_matrix(M)
        x_ref = ref.solve(M, b, np.zeros(n))
        tb = torch.tensor(b, dtype=torch.float64, device="cuda")
        tx = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        info = abi.rsg_solve_info()
        st = L.rsg_cg_diagonal_noalloc(0, None, n, len(col), d_rp, d_col, d_val, tb.data_ptr(), tx.data_ptr(),
                                       1e-10, 1e-50, 1e5, 100000, C.byref(info))
        assert st == 0, api.abi.STATUS.get(st, st)
        x = tx.cpu().numpy()
        assert info.iterations == ref.last_info.iterations
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))
        assert np.linalg.norm(b - M.mult(x)) <= 1.01e-10 * np.linalg.norm(b)


def test_noalloc_rejects_oversized_systems(ctx):
    info = abi.rsg_solve_info()
    st = api.lib().rsg_cg_diagonal_noalloc(0, None, (1 << 20) + 1, 1, 1, 1, 1, 1, 1, 1e-8, 0.0, 1e5, 10,
                                           C.byref(info))
    assert st == 9  # RSG_BAD_ARG: the static workspace holds at most RSG_NOALLOC_MAX_ROWS rows
