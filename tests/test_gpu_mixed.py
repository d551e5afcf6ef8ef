"""Mixed-precision solver (RSG_FGMRES_MIXED): FP64 flexible GMRES around an
FP32 BiCGstab with the FP32 preconditioner (ILU(0) factors, the AMG
hierarchy, or the inverted diagonal, stored in FP32).  It has no counterpart in MTJ, so
its results are checked against an FP64 direct solve (LAPACK through numpy)
or the FP64 oracle solution of the same system (IterativeSolver.solve,
sparse/CG.java) at a tighter tolerance: the solution within 1e-8 relative,
and the true FP64 residual below the requested relative tolerance."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W
from test_gpu_parity import _two_phase, banded

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pc", [abi.PC_ILU, abi.PC_DIAGONAL, abi.PC_NONE])
@pytest.mark.parametrize("n,band,seed", [(1, 0, 1), (50, 4, 2), (3000, 20, 3)])
def test_mixed_matches_fp64_solution(ctx, pc, n, band, seed):
    rp, col, val, A = banded(n, band, seed, shift=10.0)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    s = api.MixedFGMRES(ctx, pc, rtol=1e-11, max_iter=2000)
    s.set_matrix(M)
    b = np.random.Generator(np.random.PCG64(seed + 50)).standard_normal(n)
    x0 = np.zeros(n)
    x = s.solve(M, b, x0)
    xo = np.linalg.solve(A, b)
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))
    r = O.csr_op(1, rp, col, val, x, b, -1.0)
    assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm(b)
    assert s.last_info.iterations > 0


def test_mixed_fp32_amg_matches_fp64_solution(ctx):
    """FP32 AMG hierarchy (MTJ's smoothed aggregation, built in FP64 and
    copied to FP32) inside the mixed solver: the solution of the 64 x 64
    MPFA-O potential system and of a two-phase pressure Jacobian within 1e-8
    of an FP64 BiCGstab + ILU(0) solution, true FP64 residual at the
    requested tolerance."""
    case = W.potential_case(rate=2e-15)
    gm = api.Mesh(ctx, 2, 64, 64, 0, case["perm"])
    gm.compute_mpfa()
    rp, col = gm.pattern(1)
    A = api.CompRowMatrix(ctx, len(rp) - 1, rp, col)
    gm.assemble_potential(A)
    A.zero_rows(1.0, case["dirichlet_cells"])
    val = A.get_values()
    b = W.potential_rhs(case)
    # x0 = b, as PotentialCalculator.solve starts (the Dirichlet rows are then
    # satisfied from the start and the relative tolerance measures the interior)
    systems = [(rp, col, val, b, b.copy())]
    c2, gm2, om2, gs2, os2, keep = _two_phase(ctx, 24, 24, 8, spec_kw=dict(ptol=1e300, rtol=1e-2))
    gs2.enable_jacobian_capture()
    gs2.step(c2["dt"])
    rp2, col2 = gm2.pattern(0)
    jv, jr = gs2.jacobian(len(col2))
    systems.append((rp2, col2, jv, jr, np.zeros(len(rp2) - 1)))
    for rp_, col_, val_, b_, x0 in systems:
        n = len(rp_) - 1
        M = api.CompRowMatrix(ctx, n, rp_, col_, val_)
        s = api.MixedFGMRES(ctx, abi.PC_AMG, rtol=1e-10, max_iter=3000)
        s.set_matrix(M)
        assert s.amg_levels() >= 2
        x = s.solve(M, b_, x0)
        # reference: FP64 BiCGstab + ILU(0), whose monitor sees the true
        # residual (MTJ's GMRES is left preconditioned: its monitor sees
        # |M^-1 r|, which says little about |r| with this AMG)
        ref = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-14, max_iter=20000)
        ref.set_matrix(M)
        xr = ref.solve(M, b_, x0)
        assert np.max(np.abs(x - xr)) <= 1e-8 * np.max(np.abs(xr))
        r = O.csr_op(1, rp_, col_, val_, x, b_, -1.0)
        r0 = O.csr_op(1, rp_, col_, val_, x0, b_, -1.0)
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(r0)


def test_mixed_repeat_solve_and_restart(ctx):
    # two solves in a row on one handle, a short restart forcing outer cycles
    rp, col, val, A = banded(800, 12, 9, shift=8.0)
    M = api.CompRowMatrix(ctx, 800, rp, col, val)
    s = api.MixedFGMRES(ctx, abi.PC_ILU, rtol=1e-10, restart=2)
    s.set_inner(3, 1e-2)
    s.set_matrix(M)
    g = np.random.Generator(np.random.PCG64(4))
    for _ in range(2):
        xt = g.random(800)
        b = A @ xt
        x = s.solve(M, b, g.random(800))
        assert np.max(np.abs(x - xt)) <= 1e-8 * np.max(np.abs(xt))


def test_mixed_iteration_limit_status(ctx):
    rp, col, val, A = banded(500, 10, 5, shift=2.0)
    M = api.CompRowMatrix(ctx, 500, rp, col, val)
    s = api.MixedFGMRES(ctx, abi.PC_NONE, rtol=1e-14, max_iter=1)
    s.set_inner(1, 1e-1)
    s.set_matrix(M)
    b = np.ones(500)
    with pytest.raises(api.IterativeSolverNotConvergedException) as e:
        s.solve(M, b, np.zeros(500))
    assert e.value.reason == "Iterations"


def test_mixed_rejects_ssor(ctx):
    with pytest.raises(api.RSGError):
        api.MixedFGMRES(ctx, abi.PC_SSOR)


def test_mixed_potential_case(ctx):
    case = W.potential_case(rate=2e-15)
    gm = api.Mesh(ctx, 2, 64, 64, 0, case["perm"])
    gm.compute_mpfa()
    rp, col = gm.pattern(1)
    A = api.CompRowMatrix(ctx, len(rp) - 1, rp, col)
    gm.assemble_potential(A)
    A.zero_rows(1.0, case["dirichlet_cells"])
    val = A.get_values()
    b = W.potential_rhs(case)
    s = api.MixedFGMRES(ctx, abi.PC_ILU, rtol=1e-10)
    s.set_matrix(A)
    x = s.solve(A, b, b)
    xo, _, _, _, _ = O.solve(abi.CG, abi.PC_ILU, rp, col, val, b, b, rtol=1e-13)
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))


def test_mixed_two_phase_steps(ctx):
    """Black-oil steps with the mixed solver in the pressure Newton loop: the
    pressures stay within 1e-6 relative of the FP64 oracle's and the mass
    balance holds to 1e-12."""
    case, gm, om, gs, os_, keep = _two_phase(ctx, 12, 12, 4, spec_kw=dict(rtol=1e-10, method=abi.FGMRES_MIXED),
                                             oracle_spec_kw=dict(rtol=1e-12))
    for _ in range(4):
        gi = gs.step(case["dt"])
        os_.step(case["dt"])
        assert gi.mass_balance_error <= 1e-12
        gp, gN, gS = gs.state()
        op, oN, oS = os_.state()
        assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-6
        assert np.max(np.abs(gS - oS)) <= 1e-6
