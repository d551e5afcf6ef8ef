"""The L-method MPFA on the GPU (rsg_mesh_compute_lmpfa, after
geometry/flux/L_MPFA.java) against the oracle's restatement: the MD lists
bit for bit on perturbed grids with full tensors, and two-phase steps on
them within 1e-10."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import oracle as O  # noqa: E402
from ressim_gb300 import abi, api  # noqa: E402
from ressim_gb300 import workloads as W  # noqa: E402
from upscale_oracle import perturbed_coords  # noqa: E402

pytestmark = pytest.mark.gpu


def _full_tensor_perm(n, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    k = 10.0 ** (0.5 * g.standard_normal(n))
    return np.stack([k, 0.8 * k, 0.1 * k, 0.2 * k, 0.03 * k, 0.02 * k], axis=1)


@pytest.mark.parametrize("dims", [(2, 2, 2), (7, 5, 4), (16, 12, 6)])
def test_lmpfa_lists_bitexact(ctx, dims):
    ni, nj, nk = dims
    coords = perturbed_coords(3, ni, nj, nk, seed=sum(dims))
    perm = _full_tensor_perm(ni * nj * nk, 2)
    gm = api.Mesh(ctx, 3, ni, nj, nk, perm, coords=coords)
    gm.compute_lmpfa()
    om = O.Mesh(3, ni, nj, nk, coords=coords, perm=perm)
    om.mpfa(lmethod=True)
    for a, b in zip(gm.transmissibilities(), om.transmissibilities()):
        assert np.array_equal(a, b)
    for w in (0, 1):
        for a, b in zip(gm.pattern(w), om.pattern(w)):
            assert np.array_equal(a, b)
    gm.release()


def test_lmpfa_two_phase_steps_match_oracle(ctx):
    """Three two-phase steps on L-method transmissibilities: the first
    Jacobian bit-exact, Newton counts equal, states within 1e-10, mass
    balance within 1e-12."""
    ni, nj, nk = 10, 8, 4
    case = W.two_phase_case(ni=ni, nj=nj, nk=nk, seed=4)
    keep = abi.Keep()
    fluid, co = W.two_phase_fluid(keep), W.corey()
    srcs, init = W.build_sources(keep, case), W.build_initial(case)
    gm = api.Mesh(ctx, 3, ni, nj, nk, case["perm"], coords=case["nodes"])
    gm.compute_lmpfa()
    om = O.Mesh(3, ni, nj, nk, coords=case["nodes"], perm=case["perm"])
    om.mpfa(lmethod=True)

    def sims(**kw):
        spec = W.runspec(**kw)
        return (api.Discretisation(ctx, gm, fluid, co, case["porosity"], case["compaction"], srcs, init, spec),
                O.Simulator(om, fluid, co, case["porosity"], case["compaction"], srcs, init, spec))

    gs, os_ = sims(ptol=1e300, rtol=1e-12)  # one Newton iteration: the first Jacobian
    gs.enable_jacobian_capture()
    gs.step(case["dt"])
    os_.step(case["dt"])
    rp, col = gm.pattern(0)
    for a, b in zip(gs.jacobian(len(col)), os_.jacobian(len(col))):
        assert np.array_equal(a, b)
    gs, os_ = sims(rtol=1e-12)
    for _ in range(3):
        gi, oi = gs.step(case["dt"]), os_.step(case["dt"])
        assert gi.newton_iterations == oi.newton_iterations
        assert gi.mass_balance_error <= 1e-12
    gp, gN, gS = gs.state()
    op, oN, oS = os_.state()
    assert np.max(np.abs(gp - op) / np.abs(op)) <= 1e-10
    assert np.max(np.abs(gS - oS)) <= 1e-10
    gm.release()


def test_lmpfa_contract(ctx):
    """2-D meshes and the transmissibility adjoint are not built for the
    L-method: RSG_UNSUPPORTED."""
    g2 = api.Mesh(ctx, 2, 4, 4, 0, np.tile([1.0, 1.0, 1.0, 0, 0, 0], (16, 1)))
    with pytest.raises(api.RSGError) as e:
        g2.compute_lmpfa()
    assert e.value.status == abi.UNSUPPORTED
    g3 = api.Mesh(ctx, 3, 4, 4, 2, np.tile([1.0, 1.0, 1.0, 0, 0, 0], (32, 1)))
    g3.compute_lmpfa()
    n, nc = 32, g3.counts()["connections"]
    with pytest.raises(api.RSGError) as e:
        g3.transmissibility_adjoint(np.ones((1, nc)), np.ones((1, n)))
    assert e.value.status == abi.UNSUPPORTED
    g2.release()
    g3.release()
