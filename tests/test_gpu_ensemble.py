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
