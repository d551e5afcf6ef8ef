"""ILU(0) level walks on 27-point structured patterns (the pressure pattern
of a hexahedral grid with MPFA-O).  The default walk exchanges computed
values through distributed shared memory; RSG_SWEEP=pipelined selects the
walk with a cluster barrier per level.  Both must reproduce the oracle's
UnitLowerCompRowMatrix.solve / UpperCompRowMatrix.solve
(mtj/src/no/uib/cipr/matrix/sparse/ILU.java:54-140) bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def pattern27(ni, nj, nk, seed):
    """CSR of the 27-point stencil in natural i-fastest order, random values
    with a dominant diagonal."""
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    i, j, k = i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")
    n = ni * nj * nk
    rows, cols = [], []
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                a, b, c = i + di, j + dj, k + dk
                ok = (a >= 0) & (a < ni) & (b >= 0) & (b < nj) & (c >= 0) & (c < nk)
                rows.append(np.nonzero(ok)[0])
                cols.append((a + ni * (b + nj * c))[ok])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    o = np.lexsort((c, r))
    r, c = r[o], c[o]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    g = np.random.Generator(np.random.PCG64(seed))
    val = -g.random(len(c))
    val[r == c] = 30.0 + g.random(n)
    return rp, c.astype(np.int32), val


@pytest.mark.parametrize("dims", [(4, 3, 2), (16, 16, 8), (64, 64, 16), (128, 128, 8)])
def test_ilu_27pt_bitexact(ctx, dims):
    rp, col, val = pattern27(*dims, seed=sum(dims))
    n = len(rp) - 1
    A = api.CompRowMatrix(ctx, n, rp, col, val)
    s = api.BiCGstab(ctx, abi.PC_ILU)
    s.set_matrix(A)
    b = np.random.Generator(np.random.PCG64(5)).standard_normal(n)
    _, xo = O.ilu(rp, col, val, b)
    for _ in range(2):  # two applications in a row reuse the ring's barriers
        assert np.array_equal(s.apply(b), xo)
    assert api.lib().rsg_sweep_mode() == 2


SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from test_gpu_sweeps import pattern27
from oracle import oracle as O
from ressim_gb300 import abi, api
ctx = api.Context(0)
rp, col, val = pattern27(64, 64, 16, seed=96)
n = len(rp) - 1
A = api.CompRowMatrix(ctx, n, rp, col, val)
s = api.BiCGstab(ctx, abi.PC_ILU)
s.set_matrix(A)
b = np.random.Generator(np.random.PCG64(5)).standard_normal(n)
_, xo = O.ilu(rp, col, val, b)
ok = np.array_equal(s.apply(b), xo)
print("mode", api.lib().rsg_sweep_mode(), "bitexact", ok)
s.release(); A.release(); ctx.close()
sys.exit(0 if ok else 1)
"""


def test_ilu_27pt_pipelined_walk_bitexact():
    env = dict(os.environ, RSG_SWEEP="pipelined")
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, tests=HERE)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mode 1 bitexact True" in r.stdout


SCRIPT_CTAS = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from test_gpu_sweeps import pattern27
from oracle import oracle as O
from ressim_gb300 import abi, api
ctx = api.Context(0)
rp, col, val = pattern27(48, 40, 12, seed=7)
n = len(rp) - 1
A = api.CompRowMatrix(ctx, n, rp, col, val)
s = api.BiCGstab(ctx, abi.PC_ILU)
s.set_matrix(A)
b = np.random.Generator(np.random.PCG64(5)).standard_normal(n)
_, xo = O.ilu(rp, col, val, b)
ok64 = np.array_equal(s.apply(b), xo)
m = api.MixedFGMRES(ctx, abi.PC_ILU, rtol=1e-10)  # FP32 level walks inside
m.set_matrix(A)
x = m.solve(A, b, np.zeros(n))
res = np.linalg.norm(b - A.mult(x)) / np.linalg.norm(b)
print("mode", api.lib().rsg_sweep_mode(), "fp64 bitexact", ok64, "fp32 residual", res)
m.release(); s.release(); A.release(); ctx.close()
sys.exit(0 if ok64 and res <= 1e-9 else 1)
"""


@pytest.mark.parametrize("ctas", ["8", "16"])
def test_ring_walk_cluster_sizes(ctas):
    """FP64 and FP32 walks on 8- and 16-CTA clusters, each with its table of
    expected pushed values (values travel two at a time)."""
    env = dict(os.environ, RSG_RING_CTAS=ctas)
    r = subprocess.run([sys.executable, "-c", SCRIPT_CTAS.format(root=ROOT, tests=HERE)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mode 2 fp64 bitexact True" in r.stdout, r.stdout


@pytest.mark.parametrize("cls", [api.BiCGstab, api.MixedFGMRES])
def test_walk_shapes_give_identical_results(ctx, cls):
    """The walk autotuner chooses between 16-CTA and 8-CTA cluster schedules
    per sweep and precision; every choice sums the rows in CSR order, so the
    solutions with either shape forced and with the timed choice are
    bit-identical, and walk_shapes reports the forced shape."""
    rp, col, val = pattern27(48, 40, 12, seed=3)
    n = len(rp) - 1
    A = api.CompRowMatrix(ctx, n, rp, col, val)
    b = np.random.Generator(np.random.PCG64(5)).random(n)
    xs = []
    for shape in (16, 8, 0):
        s = cls(ctx, abi.PC_ILU, rtol=1e-10, max_iter=2000)
        s.set_walk_shape(shape)
        s.set_matrix(A)
        xs.append(s.solve(A, b, np.zeros(n)))
        got = s.walk_shapes()
        assert all(v in (8, 16) for v in got), got
        if shape:
            assert got == [shape] * 4
        s.release()
    assert np.array_equal(xs[0], xs[1]) and np.array_equal(xs[0], xs[2])
