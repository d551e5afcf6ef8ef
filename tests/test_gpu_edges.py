"""Edge cases through the C ABI against the oracle: 1 x 1 systems, zero
right-hand sides, invalid patterns and missing diagonals, single-cell and
line-shaped meshes (no or one connection), and a two-phase run without
injectors."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

METHODS = [(abi.CG, api.CG), (abi.BICGSTAB, api.BiCGstab), (abi.GMRES, api.GMRES)]


@pytest.mark.parametrize("method,cls", METHODS)
@pytest.mark.parametrize("pc", [abi.PC_NONE, abi.PC_DIAGONAL, abi.PC_ILU])
def test_one_by_one_system(ctx, method, cls, pc):
    rp, col, val = np.array([0, 1], np.int32), np.array([0], np.int32), np.array([4.0])
    A = api.CompRowMatrix(ctx, 1, rp, col, val)
    s = cls(ctx, pc, rtol=1e-12)
    s.set_matrix(A)
    x = s.solve(A, np.array([2.0]), np.array([0.0]))
    xo, it, _, _, _ = O.solve(method, pc, rp, col, val, np.array([2.0]), np.array([0.0]), rtol=1e-12)
    assert x[0] == xo[0] == 0.5
    assert s.last_info.iterations == it


@pytest.mark.parametrize("method,cls", METHODS)
def test_zero_right_hand_side(ctx, method, cls):
    """MTJ's monitor sees r0 = 0 and stops at once; x0 = 0 stays 0."""
    from test_gpu_parity import banded

    rp, col, val, _ = banded(50, 3, 5)
    A = api.CompRowMatrix(ctx, 50, rp, col, val)
    s = cls(ctx, abi.PC_ILU, rtol=1e-10)
    s.set_matrix(A)
    x = s.solve(A, np.zeros(50), np.zeros(50))
    xo, it, _, _, _ = O.solve(method, abi.PC_ILU, rp, col, val, np.zeros(50), np.zeros(50), rtol=1e-10)
    assert np.array_equal(x, xo) and not x.any()
    assert s.last_info.iterations == it


def test_invalid_patterns_are_rejected(ctx):
    cases = [
        (np.array([0, 2, 3], np.int32), np.array([1, 0, 1], np.int32)),  # unsorted columns
        (np.array([0, 1, 2], np.int32), np.array([0, 2], np.int32)),     # column out of range
        (np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32)),     # decreasing row pointers
        (np.array([0, 2, 2], np.int32), np.array([0, 0], np.int32)),     # duplicate column
    ]
    for rp, col in cases:
        with pytest.raises(api.RSGError) as e:
            api.CompRowMatrix(ctx, 2, rp, col, np.ones(len(col)))
        assert e.value.status == abi.BAD_ARG


def test_missing_diagonal_and_zero_pivot(ctx):
    # row 1 has no diagonal entry: ILU(0) cannot be formed
    rp, col = np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32)
    A = api.CompRowMatrix(ctx, 2, rp, col, np.array([1.0, 2.0]))
    s = api.BiCGstab(ctx, abi.PC_ILU)
    with pytest.raises(api.RSGError) as e:
        s.set_matrix(A)
    assert e.value.status == abi.MISSING_DIAGONAL
    # a zero on the diagonal: ILU.factor's zero pivot
    rp, col = np.array([0, 2, 4], np.int32), np.array([0, 1, 0, 1], np.int32)
    val = np.array([0.0, 1.0, 1.0, 1.0])
    B = api.CompRowMatrix(ctx, 2, rp, col, val)
    with pytest.raises(api.RSGError) as e:
        s.set_matrix(B)
    assert e.value.status == abi.ZERO_PIVOT
    with pytest.raises(O.OracleError):
        O.ilu(rp, col, val)


@pytest.mark.parametrize("dim,ni,nj,nk", [(2, 1, 1, 0), (2, 5, 1, 0), (2, 1, 4, 0), (3, 1, 1, 1), (3, 3, 1, 1),
                                          (3, 1, 1, 4), (3, 2, 2, 1)])
def test_degenerate_meshes(ctx, dim, ni, nj, nk):
    """A single cell (no connections) and lines of cells: MPFA-O lists and
    both patterns bit-exact vs the oracle."""
    n = ni * nj * (nk if dim == 3 else 1)
    perm = np.tile([1.0e-13, 2.0e-13, 0.5e-13, 0.2e-13, 0.0, 0.0], (n, 1))
    gm = api.Mesh(ctx, dim, ni, nj, nk, perm)
    gm.compute_mpfa()
    om = O.Mesh(dim, ni, nj, nk, perm=perm)
    om.mpfa()
    assert gm.counts()["connections"] == om.counts()["connections"]
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    for which in (0, 1):
        for a, b in zip(gm.pattern(which), om.pattern(which)):
            assert np.array_equal(a, b)


def test_two_phase_without_injectors(ctx):
    """Only the Fixed producer column: depletion steps match the oracle."""
    case = W.two_phase_case(ni=6, nj=5, nk=3, seed=9)
    case["injectors"] = []
    keep = abi.Keep()
    fluid, co = W.two_phase_fluid(keep), W.corey()
    srcs, init, spec = W.build_sources(keep, case), W.build_initial(case), W.runspec(rtol=1e-11)
    gm = api.Mesh(ctx, 3, 6, 5, 3, case["perm"], coords=case["nodes"])
    gm.compute_mpfa()
    om = O.Mesh(3, 6, 5, 3, coords=case["nodes"], perm=case["perm"])
    om.mpfa()
    gs = api.Discretisation(ctx, gm, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    os_ = O.Simulator(om, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    for _ in range(2):
        gi, oi = gs.step(case["dt"]), os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, _ = gs.state()
    op, oN, _ = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-300)) <= 1e-10
