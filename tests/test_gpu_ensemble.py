"""Ensemble stepping (rsg_ensemble_step): members on their own contexts,
stepped concurrently, give exactly the results of stepping each alone."""
import numpy as np
import pytest

from ressim_gb300 import api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SIZES = [(12, 10, 4), (16, 16, 6), (9, 13, 5), (20, 8, 3)]


def _members(seed0, rtol=1e-10, stop_rule=0):
    out = []
    for k, (ni, nj, nk) in enumerate(SIZES):
        c = api.Context(0)
        sim, case = W.build_two_phase_sim(c, ni, nj, nk, seed=seed0 + k, rtol=rtol, stop_rule=stop_rule)
        out.append((c, sim, case))
    return out


def test_ensemble_equals_serial():
    conc = _members(11)
    ser = _members(11)
    try:
        dts = [m[2]["dt"] for m in conc]
        for _ in range(3):
            infos, sts = api.ensemble_step([m[1] for m in conc], dts)
            assert not sts.any()
            for (c, sim, case), inf in zip(ser, infos):
                i = sim.step(case["dt"])
                assert i.newton_iterations == inf.newton_iterations
                assert i.linear_iterations == inf.linear_iterations
        for a, b in zip(conc, ser):
            for x, y in zip(a[1].state(), b[1].state()):
                assert np.array_equal(x, y)
        # two members on one context would race on its stream: rejected
        with pytest.raises(api.RSGError):
            api.ensemble_step([conc[0][1], conc[0][1]], [1.0, 1.0])
    finally:
        for c, sim, case in conc + ser:
            c.close()


# ---- rsg_ensemble_step_batched: all members' pressure solves in one
# persistent launch per Newton iteration

def _state_close(a, b, tol):
    (pa, Na, Sa), (pb, Nb, Sb) = a.state(), b.state()
    assert np.max(np.abs(pa - pb) / np.abs(pb)) <= tol
    assert np.max(np.abs(Sa - Sb)) <= tol
    assert np.max(np.abs(Na - Nb) / np.maximum(np.abs(Nb), 1e-30)) <= tol


def test_batched_ensemble_matches_serial_fp64():
    """FP64 walks, linear solves to 1e-12 as the oracle parity tests use, and
    the max |dp/p| Newton stop rule: the reference rule tests the signed
    pressure change of cell 0, which sits at the linear solver's rounding
    level once Newton has converged, so the number of extra iterations it
    takes follows the last bits of the dot products (measured: 4 against 6
    iterations with final pressures 6e-13 apart).  Newton counts equal the
    serial path's, linear iteration counts within two per Newton iteration,
    and pressures, saturations and moles within 1e-10 (the Krylov solver's
    dot products are summed in another order); mass balance within 1e-12."""
    bat = _members(21, rtol=1e-12, stop_rule=1)
    ser = _members(21, rtol=1e-12, stop_rule=1)
    try:
        dts = [m[2]["dt"] for m in bat]
        for _ in range(3):
            infos, sts = api.ensemble_step_batched([m[1] for m in bat], dts, precision=0)
            assert not sts.any(), sts
            for (c, sim, case), inf in zip(ser, infos):
                i = sim.step(case["dt"])
                assert i.newton_iterations == inf.newton_iterations
                assert abs(i.linear_iterations - inf.linear_iterations) <= 2 * i.newton_iterations
                assert inf.mass_balance_error <= 1e-12
        for a, b in zip(bat, ser):
            _state_close(a[1], b[1], 1e-10)
    finally:
        for c, sim, case in bat + ser:
            c.close()


def test_batched_ensemble_is_deterministic_and_order_free():
    """Each member's result depends neither on the other members nor on
    their order: the same members stepped in reverse order, and a member
    stepped alone through the batched entry point, give identical bits."""
    a = _members(31)
    b = _members(31)
    c1 = _members(31)[:1]
    try:
        dts = [m[2]["dt"] for m in a]
        for _ in range(2):
            api.ensemble_step_batched([m[1] for m in a], dts, precision=0)
            api.ensemble_step_batched([m[1] for m in b][::-1], dts[::-1], precision=0)
            api.ensemble_step_batched([c1[0][1]], dts[:1], precision=0)
        for x, y in zip(a, b):
            for u, v in zip(x[1].state(), y[1].state()):
                assert np.array_equal(u, v)
        for u, v in zip(a[0][1].state(), c1[0][1].state()):
            assert np.array_equal(u, v)
    finally:
        for c, sim, case in a + b + c1:
            c.close()


def test_batched_ensemble_mixed_precision():
    """The mixed-precision solver (FP64 flexible GMRES around FP32 BiCGstab
    and FP32 ILU(0)) in the persistent launch, max |dp/p| Newton stop rule as
    above: the same Newton counts as the serial FP64 path, pressures within
    1e-6 of it, mass balance within 1e-12."""
    bat = _members(41, stop_rule=1)
    ser = _members(41, stop_rule=1)
    try:
        dts = [m[2]["dt"] for m in bat]
        for _ in range(2):
            infos, sts = api.ensemble_step_batched([m[1] for m in bat], dts, precision=1)
            assert not sts.any(), sts
            for (c, sim, case), inf in zip(ser, infos):
                i = sim.step(case["dt"])
                assert i.newton_iterations == inf.newton_iterations
                assert inf.mass_balance_error <= 1e-12
        for x, y in zip(bat, ser):
            pa, pb = x[1].state()[0], y[1].state()[0]
            assert np.max(np.abs(pa - pb) / np.abs(pb)) <= 1e-6
    finally:
        for c, sim, case in bat + ser:
            c.close()


def test_batched_ensemble_contract():
    """Members must run BiCGstab + ILU(0); other solvers are reported as
    unsupported for that member while the others step.  A member listed
    twice, or an unknown precision, is rejected."""
    from ressim_gb300 import abi
    good = _members(51)[:1]
    c = api.Context(0)
    other, case = W.build_two_phase_sim(c, 10, 8, 4, seed=3, rtol=1e-10, method=abi.GMRES)
    try:
        infos, sts = api.ensemble_step_batched([good[0][1], other], [good[0][2]["dt"], case["dt"]])
        assert sts[0] == 0 and sts[1] == abi.UNSUPPORTED
        with pytest.raises(api.RSGError):
            api.ensemble_step_batched([good[0][1], good[0][1]], [1.0, 1.0])
        with pytest.raises(api.RSGError):
            api.ensemble_step_batched([good[0][1]], [1.0], precision=2)
    finally:
        c.close()
        for cc, sim, case in good:
            cc.close()


def _first_jacobian(ctx, ni, nj, nk, seed):
    """The first pressure Jacobian and right-hand side of a two-phase case."""
    sim, case = W.build_two_phase_sim(ctx, ni, nj, nk, seed=seed, ptol=1e300, rtol=1e-2)
    sim.enable_jacobian_capture()
    sim.step(case["dt"])
    rp, col = sim._member_keep[2].pattern(0)
    val, rhs = sim.jacobian(len(col))
    return rp, col, val, rhs


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_batched_matches_single_solves(ctx, precision):
    """rsg_solver_solve_batched against rsg_solver_solve system by system
    (BiCGstab + ILU(0) to 1e-10): FP64 walks give the single solves'
    solutions to 1e-8 of their largest entry with iteration counts within a
    few; the mixed-precision solver (precision 1) meets the tolerance on the
    true FP64 residual."""
    from ressim_gb300 import abi
    systems = [_first_jacobian(ctx, *d, seed=s) for d, s in (((10, 8, 4), 3), ((16, 16, 6), 4), ((20, 12, 5), 5))]
    mats, solvers, singles, bs = [], [], [], []
    for rp, col, val, b in systems:
        n = len(rp) - 1
        M = api.CompRowMatrix(ctx, n, rp, col, val)
        ref = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-10, max_iter=5000)
        ref.set_matrix(M)
        singles.append((ref.solve(M, b, np.zeros(n)), ref.last_info.iterations))
        s = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-10, max_iter=5000)
        s.set_matrix(M)
        mats.append(M)
        solvers.append(s)
        bs.append(b)
    xs, infos, sts = api.solve_batched(solvers, mats, bs, [np.zeros(len(b)) for b in bs], precision=precision)
    assert not sts.any(), sts
    for (x1, it1), x, inf, M, b in zip(singles, xs, infos, mats, bs):
        r = b - M.mult(x)
        assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(b)
        if precision == 0:
            assert abs(inf.iterations - it1) <= max(2, it1 // 20), (inf.iterations, it1)
            assert np.max(np.abs(x - x1)) <= 1e-8 * np.max(np.abs(x1))


SCRIPT_SHAPE = r"""
import sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
from test_gpu_ensemble import _first_jacobian
from ressim_gb300 import abi, api
ctx = api.Context(0)
mats, solvers, bs = [], [], []
for d, s in (((10, 8, 4), 3), ((16, 16, 6), 4), ((20, 12, 5), 5)):
    rp, col, val, b = _first_jacobian(ctx, *d, seed=s)
    M = api.CompRowMatrix(ctx, len(rp) - 1, rp, col, val)
    sv = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-10, max_iter=5000)
    sv.set_matrix(M)
    mats.append(M); solvers.append(sv); bs.append(b)
out = {{}}
for prec in (0, 1):
    xs, infos, sts = api.solve_batched(solvers, mats, bs, [np.zeros(len(b)) for b in bs], precision=prec)
    assert not sts.any(), sts
    for k, x in enumerate(xs):
        out["x%d_%d" % (prec, k)] = x
        out["it%d_%d" % (prec, k)] = np.array([infos[k].iterations, infos[k].inner_iterations])
np.savez({path!r}, **out)
print("shapes", solvers[0].walk_shapes())
"""


def test_solve_batched_cluster_shapes_identical(tmp_path):
    """The persistent solver sums every dot product over the same 4,096
    virtual threads in the same tree whatever the cluster shape: 16-CTA
    clusters (the default) and 8-CTA clusters (RSG_RING_CTAS=8, run in a
    child process) give bit-identical solutions and iteration counts, for
    the FP64 and the mixed-precision solver."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    here = os.path.dirname(os.path.abspath(__file__))
    res = {}
    for ctas in ("16", "8"):
        path = str(tmp_path / f"shape{ctas}.npz")
        env = dict(os.environ, RSG_RING_CTAS=ctas)
        r = subprocess.run([sys.executable, "-c", SCRIPT_SHAPE.format(root=root, tests=here, path=path)], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        assert f"shapes [{ctas}, {ctas}, {ctas}, {ctas}]" in r.stdout, r.stdout
        res[ctas] = dict(np.load(path))
    assert res["16"].keys() == res["8"].keys()
    for k in res["16"]:
        assert np.array_equal(res["16"][k], res["8"][k]), k
