"""GPU parity against the CPU oracle, through the C ABI (ctypes).

Bit-exact where the GPU evaluates the same sequential arithmetic as the
reference (SpMV rows, ILU(0)/SSOR sweeps, MPFA-O, CSR patterns, property
chain and Jacobian assembly); 1e-10 relative on solutions, where the GPU's
reductions sum in a different order than the Java loops.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def banded(n, band, seed, spd=False, shift=100.0):
    """Seeded analogue of MTJ's IterativeSolverTest matrices
    (sparse/test/IterativeSolverTest.java:87-112): random entries within a
    band, diagonal shifted by 100."""
    g = np.random.Generator(np.random.PCG64(seed))
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - band), min(n, i + band + 1)):
            if g.random() < 0.7 or i == j:
                A[i, j] = g.random()
    if spd:
        A = A + A.T
    A[np.arange(n), np.arange(n)] += shift
    rp = [0]
    col = []
    val = []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        col.extend(nz.tolist())
        val.extend(A[i, nz].tolist())
        rp.append(len(col))
    return np.array(rp, np.int32), np.array(col, np.int32), np.array(val), A


def test_csr_products_bitexact(ctx):
    rp, col, val, _ = banded(300, 7, 1)
    A = api.CompRowMatrix(ctx, 300, rp, col, val)
    x = np.random.Generator(np.random.PCG64(2)).standard_normal(300)
    y0 = np.random.Generator(np.random.PCG64(3)).standard_normal(300)
    assert np.array_equal(A.mult(x), O.csr_op(0, rp, col, val, x))
    assert np.array_equal(A.mult_add(-1.0, x, y0), O.csr_op(1, rp, col, val, x, y0, -1.0))
    assert np.array_equal(A.trans_mult(x), O.csr_op(2, rp, col, val, x))


def test_zero_rows_matches(ctx):
    rp, col, val, _ = banded(64, 4, 4)
    A = api.CompRowMatrix(ctx, 64, rp, col, val)
    rows = np.array([0, 5, 63, 17], np.int32)
    A.zero_rows(1.0, rows)
    assert np.array_equal(A.get_values(), O.zero_rows(rp, col, val, 1.0, rows))


@pytest.mark.parametrize("n,band,seed", [(1, 0, 1), (10, 2, 2), (200, 9, 3), (2000, 30, 4)])
def test_ilu_apply_bitexact(ctx, n, band, seed):
    rp, col, val, _ = banded(n, band, seed)
    A = api.CompRowMatrix(ctx, n, rp, col, val)
    s = api.BiCGstab(ctx, abi.PC_ILU)
    s.set_matrix(A)
    b = np.random.Generator(np.random.PCG64(seed + 7)).standard_normal(n)
    _, xo = O.ilu(rp, col, val, b)
    assert np.array_equal(s.apply(b), xo)
    _, xt = O.ilu(rp, col, val, b, trans=True)
    xg = s.apply(b, trans=True)
    assert np.allclose(xg, xt, rtol=1e-12, atol=1e-14)


def test_ilu_exact_on_tridiagonal(ctx):
    # ILUTest / IncompleteFactorizationTest: ILU(0) of a band matrix is exact
    for n in range(1, 11):
        for penta in (False, True):
            A = np.diag(np.full(n, 4.0 if penta else 2.0))
            for i in range(n - 1):
                A[i, i + 1] = A[i + 1, i] = -1
            if penta:
                for i in range(n - 2):
                    A[i, i + 2] = A[i + 2, i] = -1
            rp, col, val = [0], [], []
            for i in range(n):
                nz = np.nonzero(A[i])[0]
                col += nz.tolist()
                val += A[i, nz].tolist()
                rp.append(len(col))
            M = api.CompRowMatrix(ctx, n, rp, col, val)
            s = api.CG(ctx, abi.PC_ILU)
            s.set_matrix(M)
            x = np.ones(n)
            b = A @ x
            r = b - A @ s.apply(b)
            assert np.linalg.norm(r) <= 1e-5


def test_ssor_apply_bitexact(ctx):
    rp, col, val, _ = banded(500, 6, 11)
    A = api.CompRowMatrix(ctx, 500, rp, col, val)
    s = api.CG(ctx, abi.PC_SSOR)
    s.set_ssor(1.3, 0.7, True)
    s.set_matrix(A)
    b = np.random.Generator(np.random.PCG64(12)).standard_normal(500)
    x0 = np.random.Generator(np.random.PCG64(13)).standard_normal(500)
    assert np.array_equal(s.apply(b, x0), O.ssor(rp, col, val, b, x0, 1.3, 0.7, True))


SOLVERS = [(api.CG, abi.CG), (api.BiCGstab, abi.BICGSTAB), (api.GMRES, abi.GMRES)]
PCS = [abi.PC_NONE, abi.PC_DIAGONAL, abi.PC_ILU, abi.PC_SSOR]


@pytest.mark.parametrize("cls,method", SOLVERS)
@pytest.mark.parametrize("pc", PCS)
def test_krylov_recovers_solution(ctx, cls, method, pc):
    # IterativeSolverTest.testSolve / testRepeatSolve (tol 1e-4), seeded
    for seed in range(3):
        n = 5 + 15 * seed
        rp, col, val, A = banded(n, min(10, n - 1), 100 + seed, spd=(method == abi.CG))
        M = api.CompRowMatrix(ctx, n, rp, col, val)
        s = cls(ctx, pc)
        s.set_matrix(M)
        g = np.random.Generator(np.random.PCG64(seed))
        xt = g.random(n)
        b = A @ xt
        for _ in range(2):
            x = s.solve(M, b, g.random(n))
            assert np.max(np.abs(x - xt)) < 1e-4


@pytest.mark.parametrize("cls,method", SOLVERS)
def test_krylov_trajectory_matches_oracle(ctx, cls, method):
    n = 400
    # diagonally dominant, so SPD when symmetrised (CG needs it)
    rp, col, val, A = banded(n, 12, 7, spd=(method == abi.CG), shift=40.0 if method == abi.CG else 3.0)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    s = cls(ctx, abi.PC_ILU, rtol=1e-12)
    s.set_matrix(M)
    b = np.random.Generator(np.random.PCG64(8)).standard_normal(n)
    x = s.solve(M, b, np.zeros(n))
    xo, it, res, hist, _ = O.solve(method, abi.PC_ILU, rp, col, val, b, np.zeros(n), rtol=1e-12)
    assert abs(s.last_info.iterations - it) <= 1
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    h = s.history()
    k = min(len(h), len(hist), 5)
    assert np.allclose(h[:k], hist[:k], rtol=1e-9)


def test_failure_statuses(ctx):
    n = 50
    rp, col, val, A = banded(n, 3, 21)
    M = api.CompRowMatrix(ctx, n, rp, col, val)
    s = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-30, atol=0.0, max_iter=1)
    s.set_matrix(M)
    with pytest.raises(api.IterativeSolverNotConvergedException) as e:
        s.solve(M, np.ones(n), np.zeros(n))
    assert e.value.reason == "Iterations"
    # zero pivot: ILU(0) of a matrix with a zero diagonal entry
    v2 = val.copy()
    d0 = [q for q in range(rp[3], rp[4]) if col[q] == 3][0]
    v2[d0] = 0.0
    for q in range(rp[3], rp[4]):
        if col[q] < 3:
            v2[q] = 0.0
    M2 = api.CompRowMatrix(ctx, n, rp, col, v2)
    s2 = api.CG(ctx, abi.PC_ILU)
    with pytest.raises(api.RSGError) as e2:
        s2.set_matrix(M2)
    assert e2.value.status == 4
    # the context is still usable afterwards
    assert np.array_equal(M.mult(np.ones(n)), O.csr_op(0, rp, col, val, np.ones(n)))


def _mpfa_pair(ctx, dim, ni, nj, nk, case_perm, coords=None):
    gm = api.Mesh(ctx, dim, ni, nj, nk, case_perm, coords=coords)
    gm.compute_mpfa()
    om = O.Mesh(dim, ni, nj, nk, coords=coords, perm=case_perm)
    om.mpfa()
    return gm, om


def test_mpfa_2d_bitexact(ctx):
    case = W.potential_case(ni=24, nj=20, seed=5, corr_len=4.0)
    gm, om = _mpfa_pair(ctx, 2, 24, 20, 0, case["perm"])
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    for w in (0, 1):
        for a, b in zip(gm.pattern(w), om.pattern(w)):
            assert np.array_equal(a, b)
    c, v = gm.geometry()
    og = om.geometry()
    assert np.array_equal(c, og["centers"]) and np.array_equal(v, og["volumes"])


def test_mpfa_3d_perturbed_bitexact(ctx):
    case = W.two_phase_case(ni=9, nj=7, nk=5, seed=3)
    perm = case["perm"].copy()
    g = np.random.Generator(np.random.PCG64(4))
    perm[:, 3] = 0.2 * perm[:, 0] * g.uniform(-1, 1, len(perm))
    perm[:, 4] = 0.1 * perm[:, 0] * g.uniform(-1, 1, len(perm))
    perm[:, 5] = 0.1 * perm[:, 0] * g.uniform(-1, 1, len(perm))
    gm, om = _mpfa_pair(ctx, 3, 9, 7, 5, perm, case["nodes"])
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    for a, b in zip(gm.pattern(0), om.pattern(0)):
        assert np.array_equal(a, b)
    assert np.array_equal(gm.connections(), om.connections())


def test_potential_case_matches_oracle(ctx):
    """64 x 64 single-phase MPFA-O potential problem, CG + ILU(0), rtol 1e-10, x0 = b."""
    case = W.potential_case(rate=2e-15)
    gm, om = _mpfa_pair(ctx, 2, 64, 64, 0, case["perm"])
    rp, col = gm.pattern(1)
    assert len(col) == 36100
    A = api.CompRowMatrix(ctx, len(rp) - 1, rp, col)
    gm.assemble_potential(A)
    A.zero_rows(1.0, case["dirichlet_cells"])
    val = O.zero_rows(rp, col, O.potential_matrix(om, rp, col), 1.0, case["dirichlet_cells"])
    assert np.array_equal(A.get_values(), val)
    b = W.potential_rhs(case)
    s = api.CG(ctx, abi.PC_ILU, rtol=1e-10)
    s.set_matrix(A)
    x = s.solve(A, b, b)
    xo, it, _, _, _ = O.solve(abi.CG, abi.PC_ILU, rp, col, val, b, b, rtol=1e-10)
    assert abs(s.last_info.iterations - it) <= 1
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    r = b - A.mult(x)
    assert np.linalg.norm(r) <= 1.1e-10 * np.linalg.norm(b - A.mult(b))


def _two_phase(ctx, ni, nj, nk, seed=1, spec_kw=None, oracle_spec_kw=None, even=False):
    case = W.two_phase_case(ni=ni, nj=nj, nk=nk, seed=seed)
    keep = abi.Keep()
    fluid = W.two_phase_fluid(keep, even=even)
    co = W.corey()
    srcs = W.build_sources(keep, case)
    init = W.build_initial(case)
    spec = W.runspec(**(spec_kw or {}))
    gm, om = _mpfa_pair(ctx, 3, ni, nj, nk, case["perm"], case["nodes"])
    gs = api.Discretisation(ctx, gm, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    ospec = spec if oracle_spec_kw is None else W.runspec(**oracle_spec_kw)
    os_ = O.Simulator(om, fluid, co, case["porosity"], case["compaction"], srcs, init, ospec)
    return case, gm, om, gs, os_, keep


def test_two_phase_initial_state_bitexact(ctx):
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4)
    for a, b in zip(gs.state(), os_.state()):
        assert np.array_equal(a, b)
    for a, b in zip(gs.residual_volume(), os_.residual_volume()):
        assert np.array_equal(a, b)


def test_two_phase_first_jacobian_bitexact(ctx):
    # one Newton iteration per step (tolerance huge), Jacobian captured
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=dict(ptol=1e300, rtol=1e-12))
    gs.enable_jacobian_capture()
    gs.step(case["dt"])
    os_.step(case["dt"])
    rp, col = gm.pattern(0)
    gv, gr = gs.jacobian(len(col))
    ov, orr = os_.jacobian(len(col))
    assert np.array_equal(gv, ov)
    assert np.array_equal(gr, orr)


def test_two_phase_steps_match_oracle(ctx):
    case, gm, om, gs, os_, keep = _two_phase(ctx, 12, 12, 4, spec_kw=dict(rtol=1e-12))
    for step in range(6):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
        gp, gN, gS = gs.state()
        op, oN, oS = os_.state()
        assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
        assert np.max(np.abs(gS - oS)) <= 1e-10
        assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-10


def test_even_lookup_tables_match_oracle(ctx):
    """Density tables given as EvenLookupTables (direct interval index,
    knots summed one spacing at a time): initial state and the first
    Jacobian bit-exact, three steps within 1e-10."""
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=dict(ptol=1e300, rtol=1e-12), even=True)
    for a, b in zip(gs.state(), os_.state()):
        assert np.array_equal(a, b)
    gs.enable_jacobian_capture()
    gs.step(case["dt"])
    os_.step(case["dt"])
    rp, col = gm.pattern(0)
    for a, b in zip(gs.jacobian(len(col)), os_.jacobian(len(col))):
        assert np.array_equal(a, b)
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=dict(rtol=1e-12), even=True)
    for _ in range(3):
        gi, oi = gs.step(case["dt"]), os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-10


def _three_phase(ctx, spec_kw):
    case = W.three_phase_case()
    keep = abi.Keep()
    fluid = W.three_phase_fluid(keep)
    srcs = W.build_sources(keep, case)
    init = W.build_initial(case)
    spec = W.runspec(**spec_kw)
    gm, om = _mpfa_pair(ctx, 3, 12, 12, 4, case["perm"], case["nodes"])
    gs = api.Discretisation(ctx, gm, fluid, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    os_ = O.Simulator(om, fluid, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    return case, gm, gs, os_, keep


def test_three_phase_black_oil_matches_oracle(ctx):
    """Water, oil and gas (a single-phase gas cap over undersaturated oil, gas
    injected at the corners): the volume-balanced initial state is bit-exact,
    and a step of one unconverged Newton iteration (pressure tolerance 1e300)
    overshoots the explicit molar update into negative moles in the same
    element as the oracle (RS's MolarMassExplicit failure)."""
    case, gm, gs, os_, keep = _three_phase(ctx, dict(ptol=1e300, rtol=1e-12))
    for a, b in zip(gs.state(), os_.state()):
        assert np.array_equal(a, b)
    gs.enable_jacobian_capture()
    with pytest.raises(api.RSGError) as ge:
        gs.step(case["dt"])
    with pytest.raises(O.OracleError) as oe:
        os_.step(case["dt"])
    assert ge.value.status == oe.value.status == abi.NEGATIVE_MOLES
    assert "element 67" in str(ge.value) and "element 67" in str(oe.value)


def test_two_phase_retract_restores_state(ctx):
    case, gm, om, gs, os_, keep = _two_phase(ctx, 6, 6, 3)
    p0, N0, S0 = gs.state()
    gs.step(case["dt"])
    gs.retract()
    p1, N1, S1 = gs.state()
    assert np.array_equal(p0, p1) and np.array_equal(N0, N1) and np.array_equal(S0, S1)


def test_step_to_adaptive_dt_matches_oracle(ctx):
    """TimeStepper.stepTo with Discretisation.calculateDt: the same accepted
    steps, retries and final time as the oracle.  Each dt is computed from the
    state (maxima of |R|/Vp and |dN|/N), so the rounding-level differences of
    the state (1e-12 after a fixed step) move dt by ~1e-9 relative; dt and the
    state are compared to 1e-7 and 1e-8."""
    case, gm, om, gs, os_, keep = _two_phase(ctx, 12, 12, 4, spec_kw=dict(rtol=1e-12))
    ctl = abi.dt_control(1.0, 100 * 86400.0)
    gdt = odt = 20 * 86400.0  # a first step this large fails once and is retracted and retried
    retries = 0
    for end in (40 * 86400.0, 60 * 86400.0):
        gst, gdt, gi = gs.step_to(end, ctl, gdt)
        ost, odt, oi = os_.step_to(end, ctl, odt)
        assert gst == ost == 0
        assert (gi.steps, gi.retries, gi.newton_iterations) == (oi.steps, oi.retries, oi.newton_iterations)
        retries += gi.retries
        assert gs.time() == os_.time() == end
        assert abs(gdt - odt) <= 1e-7 * odt
        gp, gN, gS = gs.state()
        op, oN, oS = os_.state()
        assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-8
        assert np.max(np.abs(gS - oS)) <= 1e-8
    assert retries >= 1
    g_new, gf = gs.calculate_dt(gdt, ctl)
    o_new, of = os_.calculate_dt(odt, ctl)
    assert gf.limit == of.limit
    assert abs(g_new - o_new) <= 1e-7 * o_new
    assert abs(gs.throughput_factor(ctl) - os_.throughput_factor(ctl)) <= 1e-7 * abs(os_.throughput_factor(ctl))


def test_cubic_phase_state_matches_oracle(ctx):
    """Peng-Robinson flash and phase properties per cell against the oracle.
    CUDA's and the C library's exp/log/pow may differ in the last bit, so
    values are compared where the flash took the same number of iterations
    (nearly every cell), to 1e-7 relative: the flash stops at a 0.1 Pa
    fugacity mismatch (1e-8 of the fugacities), so last-bit differences move
    the converged split at that level, and the volume derivatives carry it.  Cells next to the critical point (two
    phases whose molar densities agree to 1%) are excluded: there the flash's
    0.1 Pa fugacity tolerance admits visibly different splits, and the volume
    derivatives (which divide by the phase difference) amplify any last-bit
    difference."""
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    nc = f.nc
    p, T, N = W.compositional_cells(3000, nc)
    gph, gits = api.cubic_phase_state(ctx, f, p, T, N)
    oph, oits = O.cubic_phase_state(f, p, T, N)
    assert np.array_equal(gph[:, 0], oph[:, 0])  # presence of each phase
    both = (oph[1, 0] > 0) & (oph[2, 0] > 0)
    near = both & (np.abs(oph[1, 2] - oph[2, 2]) < 1e-2 * np.abs(oph[1, 2]))
    assert near.mean() <= 0.02
    same = (gits == oits) & ~near
    assert same.mean() >= 0.97
    scale = np.maximum(np.abs(oph), 1e-300)
    rel = np.abs(gph - oph) / scale
    rel[np.abs(oph) < 1e-200] = np.abs(gph - oph)[np.abs(oph) < 1e-200]
    worst = np.unravel_index(np.argmax(np.where(same[None, None, :], rel, 0)), rel.shape)
    a, fld, cell = worst
    assert np.max(rel[:, :, same]) <= 1e-7, (
        f"phase {a} field {fld} cell {cell}: gpu {gph[:, :, cell].tolist()} oracle {oph[:, :, cell].tolist()} "
        f"iterations {gits[cell]} {oits[cell]} p {p[cell]} T {T[cell]} N {N[:, cell].tolist()}")
    # warm start from the persisted phases
    gph2, gits2 = api.cubic_phase_state(ctx, f, p, T, N, gph)
    oph2, oits2 = O.cubic_phase_state(f, p, T, N, oph)
    same2 = same & (gits2 == oits2)
    rel2 = np.abs(gph2 - oph2) / np.maximum(np.abs(oph2), 1e-300)
    rel2[np.abs(oph2) < 1e-200] = 0
    assert np.max(rel2[:, :, same2]) <= 1e-6


def test_compositional_steps_match_oracle(ctx):
    """Compositional line drive with the Peng-Robinson fluid model in the
    property chain: steps on the GPU against the oracle (1e-8 relative: the
    flash's stopping tolerance bounds the agreement), mass balance 1e-12."""
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    nc = f.nc
    case = W.compositional_case(12, 12, 4)
    gm, om = _mpfa_pair(ctx, 3, 12, 12, 4, case["perm"], case["nodes"])
    srcs = W.build_compositional_sources(keep, case, nc)
    init = W.build_compositional_initial(case, nc)
    spec = W.runspec(rtol=1e-12)
    gs = api.Discretisation(ctx, gm, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    os_ = O.Simulator(om, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    for a, b in zip(gs.state(), os_.state()):
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)) <= 1e-10
    for _ in range(3):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
        gp, gN, gS = gs.state()
        op, oN, oS = os_.state()
        assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-8
        assert np.max(np.abs(gS - oS)) <= 1e-8
        assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-8


@pytest.mark.parametrize("dim", [2, 3])
def test_tpfa_bitexact(ctx, dim):
    """TPFA.calculateTransmissibilities on the GPU against the oracle: MD
    lists, values (with the reference's ||K_j n|| weighting) and patterns."""
    if dim == 2:
        case = W.potential_case(ni=20, nj=14, seed=4, corr_len=3.0)
        ni, nj, nk, coords = 20, 14, 0, None
    else:
        case = W.two_phase_case(ni=7, nj=6, nk=5, seed=2)
        ni, nj, nk, coords = 7, 6, 5, case["nodes"]
    gm = api.Mesh(ctx, dim, ni, nj, nk, case["perm"], coords=coords)
    gm.compute_tpfa()
    om = O.Mesh(dim, ni, nj, nk, coords=coords, perm=case["perm"])
    om.mpfa(tpfa=True)
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    for which in (0, 1):
        for a, b in zip(gm.pattern(which), om.pattern(which)):
            assert np.array_equal(a, b)


def test_tpfa_two_phase_steps_match_oracle(ctx):
    case = W.two_phase_case(ni=10, nj=9, nk=3, seed=6)
    keep = abi.Keep()
    fluid, co = W.two_phase_fluid(keep), W.corey()
    srcs, init, spec = W.build_sources(keep, case), W.build_initial(case), W.runspec(rtol=1e-11)
    gm = api.Mesh(ctx, 3, 10, 9, 3, case["perm"], coords=case["nodes"])
    gm.compute_tpfa()
    om = O.Mesh(3, 10, 9, 3, coords=case["nodes"], perm=case["perm"])
    om.mpfa(tpfa=True)
    gs = api.Discretisation(ctx, gm, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    os_ = O.Simulator(om, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    for _ in range(3):
        gi, oi = gs.step(case["dt"]), os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, _ = gs.state()
    op, oN, _ = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-300)) <= 1e-10


def test_three_phase_converged_steps_match_oracle(ctx):
    """Water, oil and gas with converged Newton iterations over six steps:
    the gas cap and the gas injected at the corners put cells in all three
    hydrocarbon regimes of BlackOilEquationOfState.calculatePhaseState
    (single-phase oil, single-phase gas, two-phase oil/gas:
    rs/src/no/uib/cipr/rs/fluid/BlackOilEquationOfState.java:169-547).  Newton
    counts equal, pressures and saturations within 1e-10 of the oracle, moles
    within 1e-9 of each component's largest amount (the explicit molar update
    of cells with gas accumulates the flash-free black-oil split's rounding
    over the six steps: the largest deviation is 2.4e-10), mass balance
    within 1e-12."""
    case, gm, gs, os_, keep = _three_phase(ctx, dict(rtol=1e-12))
    regimes = set()
    for _ in range(6):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
        gp, gN, gS = gs.state()
        op, oN, oS = os_.state()
        assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
        assert np.max(np.abs(gS - oS)) <= 1e-10
        # moles per component relative to that component's largest amount:
        # cells holding a trace of gas carry the absolute error of the large
        # ones, not a relative one
        scale = np.max(np.abs(oN), axis=1, keepdims=True)
        assert np.max(np.abs(gN - oN) / scale) <= 1e-9
        so, sg = oS[1], oS[2]
        regimes |= {"oil"} if np.any((so > 0) & (sg == 0)) else set()
        regimes |= {"gas"} if np.any((so == 0) & (sg > 0)) else set()
        regimes |= {"oil+gas"} if np.any((so > 0) & (sg > 0)) else set()
    assert regimes == {"oil", "gas", "oil+gas"}, regimes


def test_rotation_body_force_step_matches_oracle(ctx):
    """A rotating frame (RunSpec's omega and rotation axis): the Darcy
    potential carries rho (g z - omega^2 r^2 / 2) (rs/src/no/uib/cipr/rs/field/
    CS.java:161-170).  Two converged steps with omega = 0.5 rad/s about the
    vertical axis through (3, 2): within 1e-10 of the oracle, and different
    from the same steps without rotation."""
    kw = dict(rtol=1e-12)
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=kw)
    ref = gs
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=dict(kw, omega=0.5, ax=3.0, ay=2.0))
    for _ in range(2):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        ref.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-10
    assert np.max(np.abs(gp - ref.state()[0]) / np.abs(gp)) > 1e-6


@pytest.mark.parametrize("kind", [abi.RF_TABULAR, abi.RF_THREE_PHASE_TABULAR])
def test_tabular_rock_fluid_steps_match_oracle(ctx, kind):
    """TabularRockFluid (1D tables, kro blended from krow and krog) and
    ThreePhaseTabularRockFluid (2D tables of Sw and Sg) in the property chain
    (rs/src/no/uib/cipr/rs/rock/TabularRockFluid.java:60-91,
    ThreePhaseTabularRockFluid.java:60-78), with a tabulated capillary
    pressure: four converged two-phase steps, Newton counts equal,
    pressures and saturations within 1e-10 of the oracle, mass balance within
    1e-12."""
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4, spec_kw=dict(rtol=1e-12))
    t = W.rock_tables(keep, kind)
    gs.set_rock_tables(t)
    os_.set_rock_tables(t)
    for _ in range(4):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10


def test_three_phase_tabular_rock_fluid_matches_oracle(ctx):
    """ThreePhaseTabularRockFluid on the water-oil-gas case (gas cap, gas
    injected): converged steps against the oracle as above."""
    case, gm, gs, os_, keep = _three_phase(ctx, dict(rtol=1e-12))
    t = W.rock_tables(keep, abi.RF_THREE_PHASE_TABULAR)
    gs.set_rock_tables(t)
    os_.set_rock_tables(t)
    for _ in range(3):
        gi = gs.step(case["dt"])
        oi = os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10


def test_rock_tables_contract(ctx):
    """Relative permeability tables outside [0, 1] or of the wrong dimension
    are rejected; RSG_RF_COREY returns to the Corey model."""
    case, gm, om, gs, os_, keep = _two_phase(ctx, 10, 8, 4)
    s0 = gs.state()[2].copy()
    t = W.rock_tables(keep)
    t.krw = abi.table(keep, [[0.0, 1.0]], [0.0, 1.5])
    with pytest.raises(api.RSGError):
        gs.set_rock_tables(t)
    t = W.rock_tables(keep, abi.RF_THREE_PHASE_TABULAR)
    t.krw = abi.table(keep, [[0.0, 1.0]], [0.0, 1.0])
    with pytest.raises(api.RSGError):
        gs.set_rock_tables(t)
    back = abi.rsg_rock_tables()
    back.kind = abi.RF_COREY
    gs.set_rock_tables(back)
    assert np.array_equal(gs.state()[2], s0)
