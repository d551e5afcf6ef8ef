"""The distributed-shared-memory schedule of the ILU(0) level walks
(precond.cu, k_sweep_ring), built on the host and checked against each
pattern without a GPU: every row is placed once, every slot and entry index
stays inside its array, every operand of a row is computed in an earlier
level within the ring's depth and is either the reading CTA's own value or
pushed to it, and each CTA's per-level receive count equals the values pushed
to it.  The walk it schedules is MTJ's UnitLowerCompRowMatrix.solve /
UpperCompRowMatrix.solve (mtj/src/no/uib/cipr/matrix/sparse/ILU.java:54-140)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from test_gpu_sweeps import pattern27  # noqa: E402

from ressim_gb300 import abi  # noqa: E402


@pytest.fixture(scope="module")
def L():
    from ressim_gb300 import api, build

    if not os.path.exists(build.LIB):
        try:
            build.build()
        except FileNotFoundError:
            pytest.skip("nvcc not available to build libresgpu.so")
    return api.lib()


def check(L, rp, col, sweep, ctas):
    stats = np.zeros(4, np.int64)
    msg = C.create_string_buffer(256)
    st = L.rsg_sweep_plan_check(len(rp) - 1, abi.iptr(rp), abi.iptr(col), sweep, ctas,
                                stats.ctypes.data_as(C.POINTER(C.c_int64)), msg, 256)
    return st, stats, msg.value.decode()


def csr(n, rows, cols):
    """Sorted CSR pattern with the diagonal."""
    r = np.concatenate([rows, np.arange(n)])
    c = np.concatenate([cols, np.arange(n)])
    key = np.unique(r.astype(np.int64) * n + c)
    r, c = key // n, key % n
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp).astype(np.int32), c.astype(np.int32)


def transpose(rp, col):
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    return csr(n, col.astype(np.int64), rows)


@pytest.mark.parametrize("ctas", [16, 8])
@pytest.mark.parametrize("sweep", [0, 1])
def test_headline_pattern(L, sweep, ctas):
    """The 27-point pattern of the 128 x 128 x 32 grid: 506 levels, a ring of
    lookback 7 + 2 levels, each CTA (a block of 32 or 64 k-planes' worth of
    rows) exchanging with its two neighbours at most, and only the edge plane
    of each block pushed once."""
    rp, col, _ = pattern27(128, 128, 32, seed=1)
    st, stats, msg = check(L, rp, col, sweep, ctas)
    assert st == abi.OK, msg
    nlev, R, pushed, nbr = stats
    assert nlev == 506 and R == 12  # lookback 7, 2 levels of reuse margin, 3 of slack
    assert nbr <= 2
    assert pushed <= (ctas - 1) * 128 * 128 + 2 * 506 * ctas


@pytest.mark.parametrize("dims", [(4, 3, 2), (16, 16, 8), (48, 40, 12), (64, 64, 16), (7, 5, 33)])
def test_27_point_patterns(L, dims):
    rp, col, _ = pattern27(*dims, seed=3)
    for sweep in (0, 1):
        for ctas in (8, 16):
            st, _, msg = check(L, rp, col, sweep, ctas)
            assert st == abi.OK, (dims, sweep, ctas, msg)


def test_nine_point_2d_and_transposed_patterns(L):
    """The 64 x 64 potential pattern (9 points) and a non-symmetric random
    pattern with its transpose (the transposed ILU sweeps of transApply)."""
    rp, col, _ = pattern27(64, 64, 1, seed=4)
    for sweep in (0, 1):
        st, _, msg = check(L, rp, col, sweep, 16)
        assert st == abi.OK, msg
    # the 27-point pattern without its (+1, +1, 0) and (-1, 0, +1) couplings
    # in one direction: non-symmetric, still with uniform levels
    ni, nj, nk = 24, 20, 10
    rp, col, _ = pattern27(ni, nj, nk, seed=5)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    keep = (col - rows != ni + 1) & (col - rows != ni * nj - 1)
    rp, col = csr(n, rows[keep], col[keep].astype(np.int64))
    rpt, colt = transpose(rp, col)
    assert not np.array_equal(col, colt)
    for p in ((rp, col), (rpt, colt)):
        for sweep in (0, 1):
            for ctas in (8, 16):
                st, _, msg = check(L, *p, sweep, ctas)
                assert st == abi.OK, msg
    # a random banded pattern: a schedule exists only when the ring's depth
    # fits in shared memory; either way the status says which
    g = np.random.Generator(np.random.PCG64(8))
    n = 3000
    rows = g.integers(0, n, 6 * n)
    rp, col = csr(n, rows, np.clip(rows + g.integers(-3, 4, len(rows)), 0, n - 1))
    for sweep in (0, 1):
        st, _, msg = check(L, rp, col, sweep, 16)
        assert st in (abi.OK, abi.UNSUPPORTED), msg


def test_level_splitting(L):
    """A level with more rows in one CTA than its warps hold is split into
    consecutive plan levels (rows of one level are independent)."""
    n = 5000  # a diagonal matrix: one level of 5000 rows
    rp, col = csr(n, np.zeros(0, np.int64), np.zeros(0, np.int64))
    st, stats, msg = check(L, rp, col, 0, 16)
    assert st == abi.OK, msg
    assert stats[0] == -(-(n // 16 + 1) // 128)  # ceil(rows of the largest block / 128)
    # an arrow of dependencies: row 0 feeds every other row, across all CTAs
    rows = np.arange(1, n)
    rp, col = csr(n, rows, np.zeros(n - 1, np.int64))
    st, stats, msg = check(L, rp, col, 0, 16)
    assert st == abi.OK, msg
    assert stats[3] == 15


def test_long_chains_have_no_ring_schedule(L):
    """A tridiagonal matrix has one row per level: padding every level to a
    full slot set would cost too much, so it gets no ring schedule."""
    n = 200000
    rp, col = csr(n, np.arange(1, n), np.arange(n - 1))
    st, _, msg = check(L, rp, col, 0, 16)
    assert st == abi.UNSUPPORTED, msg
    assert check(L, rp, col, 2, 16)[0] == abi.BAD_ARG
