"""The upscaling caller on the GPU (rsg_upscale_pressure, rsg_mesh_connection_flux,
rsg_mesh_get_interface_centers and ressim_gb300.upscale) against the oracle:
upscale/PressureDiscretisation.java, LocalFlowRateAverage.java,
PressureBC.java and the partition geometry of meshgen/partition."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import oracle as O  # noqa: E402
from ressim_gb300 import api  # noqa: E402
from ressim_gb300 import upscale as U  # noqa: E402
from upscale_oracle import here_interface, lognormal_perm, oracle_upscale, perturbed_coords  # noqa: E402

pytestmark = pytest.mark.gpu


def _pair(ctx, dim, ni, nj, nk, seed=3, tpfa=False):
    coords = perturbed_coords(dim, ni, nj, nk, seed)
    perm = lognormal_perm(ni * nj * max(nk, 1), seed + 1)
    gm = api.Mesh(ctx, dim, ni, nj, nk, perm, coords=coords)
    om = O.Mesh(dim, ni, nj, nk, coords=coords, perm=perm)
    if tpfa:
        gm.compute_tpfa()
        om.mpfa(tpfa=True)
    else:
        gm.compute_mpfa()
        om.mpfa()
    return gm, om, coords, perm


@pytest.mark.parametrize("dim,nk", [(2, 0), (3, 5)])
def test_connection_flux_and_interface_centers_bitexact(ctx, dim, nk):
    """flux[c] = sum_k t_k p[el_k] in MD order, and the here-interface
    centres, bit for bit."""
    gm, om, _, _ = _pair(ctx, dim, 17, 13, nk)
    n = gm.counts()["elements"]
    p = np.random.Generator(np.random.PCG64(9)).standard_normal(n)
    assert np.array_equal(gm.connection_flux(p), O.connection_flux(om, p))
    conn = om.connections()
    assert np.array_equal(gm.connections(), conn)
    assert np.array_equal(gm.interface_centers(), om.geometry()["icenter"][here_interface(dim, 17, 13, conn)])
    gm.release()


def test_pressure_discretisation_matches_oracle(ctx):
    """PressureDiscretisation: GMRES(30) + ILU(0) from 0 to the absolute
    tolerance 1e-10 on the linear Dirichlet data of a side-to-side problem.
    The GPU's dot products are summed in another order than MTJ's, so the
    iteration counts agree within two and the solutions within 1e-9."""
    gm, om, _, _ = _pair(ctx, 3, 20, 16, 6, seed=5)
    centers = om.geometry()["centers"]
    ni, nj = 20, 16
    cells = [e for e in range(len(centers)) if e % ni in (0, ni - 1)]
    bc = {e: 1.0 - centers[e, 0] / ni for e in cells}
    g = U.PressureDiscretisation(gm, bc)
    xo, it, val, b = O.pressure_discretisation(om, bc)
    assert g.info.reason == 0
    assert abs(g.info.iterations - it) <= 2, (g.info.iterations, it)
    assert np.max(np.abs(g.get_solution() - xo)) <= 1e-9 * np.max(np.abs(xo))
    assert g.get_solution(cells[0]) == pytest.approx(bc[cells[0]], abs=1e-12)
    gm.release()


def test_pressure_discretisation_contract(ctx):
    gm, om, _, _ = _pair(ctx, 2, 8, 6, 0)
    with pytest.raises(api.RSGError):
        U.PressureDiscretisation(gm, {48: 1.0})  # no such cell
    gm.release()


@pytest.mark.parametrize("bc_type,method", [("Open", "mpfa"), ("Closed", "mpfa"), ("Open", "tpfa")])
def test_local_flow_rate_average_matches_oracle(ctx, bc_type, method):
    """Every domain of a 3 x 3 partition (border 2 cells) of a perturbed
    24 x 24 x 4 grid with lognormal permeability: the same boundary cells and
    inner connections, GPU pressures and fluxes within 1e-9 of the oracle's,
    coarse tensors within 1e-8."""
    dim, ni, nj, nk = 3, 24, 24, 4
    coords = perturbed_coords(dim, ni, nj, nk, 11)
    perm = lognormal_perm(ni * nj * nk, 12)
    doms = U.partition2d(0.0, 0.0, [3], [8.0], [3], [8.0], border=2.0)
    up = U.StructuredUpscaler(ctx, dim, ni, nj, nk, perm, coords=coords, method=method)
    res = up.local_flow_rate_average(doms, bc_type)
    ref, geo = oracle_upscale(dim, ni, nj, nk, coords, perm, doms, bc_type, method)
    assert np.array_equal(up.conn, geo["conn"]) and np.array_equal(up.icenters, geo["icenters"])
    assert np.array_equal(up.centers, geo["centers"])
    for g, o in zip(res, ref):
        assert g["elements"] == o["elements"]
        assert g["bc"] == o["bc"]
        for side in U.ORIENTATIONS_2D:
            assert np.array_equal(g["inner"][side], o["inner"][side])
        for key in ("px", "py", "ux", "uy"):
            assert np.max(np.abs(g[key] - o[key])) <= 1e-9 * max(np.max(np.abs(o[key])), 1e-300), key
        assert np.allclose(g["tensor"], o["tensor"], rtol=1e-8, atol=1e-12 * np.max(np.abs(o["tensor"])))


def test_uniform_tensor_is_reproduced(ctx):
    """A homogeneous full tensor on a regular 3-D grid upscales to itself
    times the thickness (MPFA-O is exact for linear pressure), through the
    GPU pipeline."""
    ni, nj, nk = 15, 15, 2
    K = (3.0, 1.0, 0.2, -0.4, 0.0, 0.0)
    perm = np.tile(np.array(K), (ni * nj * nk, 1))
    up = U.StructuredUpscaler(ctx, 3, ni, nj, nk, perm)
    doms = U.partition2d(0.0, 0.0, [3], [5.0], [3], [5.0], border=2.0)
    r = up.local_flow_rate_average([doms[4]])[0]
    H = float(nk)
    assert np.allclose(r["tensor"], [K[0] * H, K[1] * H, 0.0, K[3] * H, 0.0, 0.0], rtol=1e-8, atol=1e-9)
    assert abs(r["k21"] - K[3] * H) <= 1e-8 * H
