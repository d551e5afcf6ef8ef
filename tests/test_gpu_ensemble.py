"""Ensemble stepping (rsg_ensemble_step): members on their own contexts,
stepped concurrently, give exactly the results of stepping each alone."""
import numpy as np
import pytest

from ressim_gb300 import api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SIZES = [(12, 10, 4), (16, 16, 6), (9, 13, 5), (20, 8, 3)]


def _members(seed0):
    out = []
    for k, (ni, nj, nk) in enumerate(SIZES):
        c = api.Context(0)
        sim, case = W.build_two_phase_sim(c, ni, nj, nk, seed=seed0 + k, rtol=1e-10)
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
    """FP64 walks: Newton counts equal the serial path's, linear iteration
    counts within one per Newton iteration, and pressures, saturations and
    moles within 1e-10 (the Krylov solver's dot products are summed in
    another order); mass balance within 1e-12."""
    bat = _members(21)
    ser = _members(21)
    try:
        dts = [m[2]["dt"] for m in bat]
        for _ in range(3):
            infos, sts = api.ensemble_step_batched([m[1] for m in bat], dts, precision=0)
            assert not sts.any(), sts
            for (c, sim, case), inf in zip(ser, infos):
                i = sim.step(case["dt"])
                assert i.newton_iterations == inf.newton_iterations
                assert abs(i.linear_iterations - inf.linear_iterations) <= i.newton_iterations
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
    """FP32 factors inside the FP64 BiCGstab: the same Newton counts as the
    serial FP64 path, pressures within 1e-6 of it, mass balance within
    1e-12."""
    bat = _members(41)
    ser = _members(41)
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
