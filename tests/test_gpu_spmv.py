"""The SELL-32 SpMV + dot kernels of the Krylov solvers (k_spmv_dot,
k_f32_spmv_dot) inside BiCGstab and the mixed-precision solver, against
the oracle's solves on 27-point, ragged (slices of mixed row lengths, n
not a multiple of 32), empty-row and wide-row patterns."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import oracle as O  # noqa: E402
from ressim_gb300 import abi, api  # noqa: E402
from test_gpu_sweeps import pattern27  # noqa: E402

pytestmark = pytest.mark.gpu


def random_pattern(n, maxlen, seed, empty_every=0):
    """Random rows of up to maxlen entries (diagonal dominant), every
    empty_every-th row with its diagonal only."""
    g = np.random.Generator(np.random.PCG64(seed))
    rp, col, val = [0], [], []
    for i in range(n):
        if empty_every and i % empty_every == 0:
            cs = np.array([i])
        else:
            k = int(g.integers(1, maxlen))
            cs = np.unique(np.concatenate([[i], g.integers(0, n, k - 1)]))
        v = -g.random(len(cs))
        v[cs == i] = 2.0 * maxlen
        col.extend(cs.tolist())
        val.extend(v.tolist())
        rp.append(len(col))
    return np.array(rp, np.int32), np.array(col, np.int32), np.array(val)


def _solve(ctx, rp, col, val, b, cls=api.BiCGstab):
    n = len(rp) - 1
    A = api.CompRowMatrix(ctx, n, rp, col, val)
    s = cls(ctx, abi.PC_ILU, rtol=1e-10, max_iter=5000)
    s.set_matrix(A)
    ctx.set_profiling(True)
    ctx.profile_reset()
    x = s.solve(A, b, np.zeros(n))
    prof = ctx.profile()
    ctx.set_profiling(False)
    return x, s.last_info, prof, A


@pytest.mark.parametrize("case", ["27pt", "ragged", "empty_rows", "wide"])
def test_spmv_kernels_in_bicgstab(ctx, case):
    """BiCGstab + ILU(0) to 1e-10 against the oracle: iteration counts within
    two, solutions within 1e-8 of the largest entry, the fused SpMV + dot
    kernel on every pattern."""
    if case == "27pt":
        rp, col, val = pattern27(24, 20, 9, seed=4)
    elif case == "ragged":
        rp, col, val = random_pattern(1000, 32, 5)
    elif case == "empty_rows":
        rp, col, val = random_pattern(777, 20, 6, empty_every=3)
    else:
        rp, col, val = random_pattern(600, 48, 7)
    n = len(rp) - 1
    b = np.random.Generator(np.random.PCG64(8)).standard_normal(n)
    x, info, prof, _ = _solve(ctx, rp, col, val, b)
    xo, it, _, _, _ = O.solve(abi.BICGSTAB, abi.PC_ILU, rp, col, val, b, np.zeros(n), rtol=1e-10, maxit=5000)
    assert info.reason == 0
    assert abs(info.iterations - it) <= 2, (info.iterations, it)
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))
    assert "spmv_dot" in prof, sorted(prof)


def test_fp32_spmv_in_mixed_solver(ctx):
    """The FP32 SpMV + dot inside the mixed-precision solver: the FP64 outer
    iteration meets 1e-10 on the true residual."""
    rp, col, val = pattern27(40, 36, 10, seed=9)
    n = len(rp) - 1
    b = np.random.Generator(np.random.PCG64(10)).standard_normal(n)
    x, info, prof, A = _solve(ctx, rp, col, val, b, cls=api.MixedFGMRES)
    assert info.reason == 0
    assert "inner_spmv_dot" in prof
    r = b - A.mult(x)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(b)
