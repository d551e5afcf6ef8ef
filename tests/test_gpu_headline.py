"""Parity at the benchmark's own sizes: the 128 x 128 x 32 two-phase case
(524,288 cells, 13,716,856 pattern entries) that bench.py times, with the
bench's seed, and the 256 x 256 x 16 compositional grid (1,048,576 cells).

Against the oracle, through the C ABI:
* MPFA-O transmissibility lists (order, values, exact zeros), geometry,
  connections and the CSR pattern (numerics/LinearSolver.java:111-168):
  bit-exact;
* the first assembled Jacobian and residual
  (numerics/Discretisation.java:365-561): bit-exact;
* ILU(0) factorisation and apply on that Jacobian (the level walk the
  benchmark's time is spent in; mtj/.../sparse/ILU.java:54-140): bit-exact;
* one converged time step (Discretisation.solve, :208-225): equal Newton
  counts, pressures, saturations and moles within 1e-10 relative, mass
  balance within 1e-12;
* the same step with the mixed-precision solver (FP32 inner, FP64 outer, to
  1e-8): pressures within 1e-6 of the oracle's FP64 step.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NI, NJ, NK = 128, 128, 32
SEED = 1  # bench.py's default seed


@pytest.fixture(scope="module")
def head(ctx):
    case = W.two_phase_case(ni=NI, nj=NJ, nk=NK, seed=SEED)
    keep = abi.Keep()
    d = dict(case=case, keep=keep, fluid=W.two_phase_fluid(keep), co=W.corey(), srcs=W.build_sources(keep, case),
             init=W.build_initial(case))
    d["gm"] = api.Mesh(ctx, 3, NI, NJ, NK, case["perm"], coords=case["nodes"])
    d["gm"].compute_mpfa()
    d["om"] = O.Mesh(3, NI, NJ, NK, coords=case["nodes"], perm=case["perm"])
    d["om"].mpfa()
    yield d
    d["gm"].release()


def sims(ctx, h, gpu_spec, oracle_spec=None):
    c = h["case"]
    gs = api.Discretisation(ctx, h["gm"], h["fluid"], h["co"], c["porosity"], c["compaction"], h["srcs"], h["init"],
                            gpu_spec)
    os_ = None
    if oracle_spec is not None:
        os_ = O.Simulator(h["om"], h["fluid"], h["co"], c["porosity"], c["compaction"], h["srcs"], h["init"],
                          oracle_spec)
    return gs, os_


def test_headline_mpfa_pattern_geometry_bitexact(head):
    gm, om = head["gm"], head["om"]
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    rp, col = gm.pattern(0)
    orp, ocol = om.pattern(0)
    assert len(col) == 13716856
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.array_equal(gm.connections(), om.connections())
    c, v = gm.geometry()
    og = om.geometry()
    assert np.array_equal(c, og["centers"]) and np.array_equal(v, og["volumes"])


def test_headline_first_jacobian_and_ilu_bitexact(ctx, head):
    """One Newton iteration (pressure tolerance 1e300; the linear tolerance
    is loose because only the assembled system is compared), Jacobian and
    residual captured; then ILU(0) of that Jacobian applied to its residual
    on the GPU's level walk against the oracle's sequential solves."""
    spec = W.runspec(ptol=1e300, rtol=1e-2)
    gs, os_ = sims(ctx, head, spec, spec)
    for a, b in zip(gs.state(), os_.state()):
        assert np.array_equal(a, b)
    gs.enable_jacobian_capture()
    dt = head["case"]["dt"]
    gs.step(dt)
    os_.step(dt)
    rp, col = head["gm"].pattern(0)
    gv, gr = gs.jacobian(len(col))
    ov, orr = os_.jacobian(len(col))
    assert np.array_equal(gv, ov)
    assert np.array_equal(gr, orr)
    gs.release()
    A = api.CompRowMatrix(ctx, len(rp) - 1, rp, col, gv)
    s = api.BiCGstab(ctx, abi.PC_ILU)
    s.set_matrix(A)
    _, xo = O.ilu(rp, col, gv, gr)
    assert np.array_equal(s.apply(gr), xo)
    assert api.lib().rsg_sweep_mode() == 2
    s.release()
    A.release()


def test_headline_step_matches_oracle(ctx, head):
    """One converged step of the benchmark's case (BiCGstab + ILU(0); the
    linear tolerance is 1e-12 on both sides so that the comparison sees the
    arithmetic, not the stopping point), then the same step with the
    mixed-precision solver at the benchmark's 1e-8."""
    dt = head["case"]["dt"]
    spec = W.runspec(rtol=1e-12)
    gs, os_ = sims(ctx, head, spec, spec)
    gi = gs.step(dt)
    oi = os_.step(dt)
    assert gi.newton_iterations == oi.newton_iterations
    assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-10
    gs.release()
    ms, _ = sims(ctx, head, W.runspec(method=abi.FGMRES_MIXED, rtol=1e-8, inner_iterations=10, inner_tolerance=1e-3))
    mi = ms.step(dt)
    assert mi.mass_balance_error <= 1e-12
    mp = ms.state()[0]
    assert np.max(np.abs(mp - op) / np.abs(op)) <= 1e-6
    ms.release()


def test_compositional_size_pattern_and_step(ctx):
    """The compositional configuration's grid, 256 x 256 x 16: MPFA-O lists
    and the 26,990,776-entry pattern bit-exact; one Peng-Robinson step of
    one Newton iteration, mass balance within 1e-12.  The flash stops at a
    0.1 Pa fugacity residual (CubicEquationOfState's flash tolerance), so two
    correct evaluations differ below that level: pressures and saturations
    within 1e-8, component moles within 1e-7 relative (the largest deviation
    over the 4 x 1,048,576 moles is 2e-8; 1e-8 holds on small grids)."""
    ni, nj, nk = 256, 256, 16
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    case = W.compositional_case(ni, nj, nk, dt=2000.0)
    gm = api.Mesh(ctx, 3, ni, nj, nk, case["perm"], coords=case["nodes"])
    gm.compute_mpfa()
    om = O.Mesh(3, ni, nj, nk, coords=case["nodes"], perm=case["perm"])
    om.mpfa()
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    rp, col = gm.pattern(0)
    orp, ocol = om.pattern(0)
    assert len(col) == 26990776
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    srcs = W.build_compositional_sources(keep, case, f.nc)
    init = W.build_compositional_initial(case, f.nc)
    spec = W.runspec(rtol=1e-12, ptol=1e300)
    spec.truncate_negative_moles = 1
    gs = api.Discretisation(ctx, gm, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    os_ = O.Simulator(om, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
    gi = gs.step(case["dt"])
    oi = os_.step(case["dt"])
    assert gi.newton_iterations == oi.newton_iterations == 1
    assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-8
    assert np.max(np.abs(gS - oS)) <= 1e-8
    assert np.max(np.abs(gN - oN) / np.maximum(np.abs(oN), 1e-30)) <= 1e-7
    gs.release()
    gm.release()
