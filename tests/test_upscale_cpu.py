"""Upscaling host logic (ressim_gb300.upscale): the partition geometry of
meshgen/partition (Region2D, Domain2D, Partition2D, PartitionData), the
boundary data of upscale/PressureBC and the LocalFlowRateAverage formulas,
checked on the CPU with the oracle's meshes and solvers."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from ressim_gb300 import upscale as U  # noqa: E402


def test_region_is_half_open():
    """Region2D.pointInRegion's winding rule puts the left and front edges
    inside and the right and back edges outside."""
    r = U.Region2D((0, 0, 0), (2, 0, 0), (2, 1, 0), (0, 1, 0))
    pts = np.array([[1, .5], [0, .5], [2, .5], [1, 0], [1, 1], [0, 0], [2, 1], [-1e-12, .5], [1, .999999], [3, .5]])
    assert r.contains(pts).tolist() == [True, True, False, True, False, True, False, False, True, False]


def test_closest_segment():
    r = U.Region2D((0, 0, 0), (2, 0, 0), (2, 1, 0), (0, 1, 0))
    pts = np.array([[1, .1, 0], [1.95, .5, 0], [1, .9, 0], [.05, .5, 0], [3, 3, 0], [-1, -1, 0], [1, .5, 0]])
    # the centre is as far from front as from back: the first, front, wins
    assert r.closest(pts).tolist() == ["FRONT", "RIGHT", "BACK", "LEFT", "RIGHT", "FRONT", "FRONT"]
    # a z offset shifts every distance alike
    pts[:, 2] = 5.0
    assert r.closest(pts[:4]).tolist() == ["FRONT", "RIGHT", "BACK", "LEFT"]


def test_partition2d():
    ds = U.partition2d(1.0, 2.0, [2, 1], [1.5, 3.0], [1], [4.0], border=0.5)
    assert len(ds) == 3
    assert [(d.x0, d.x1, d.y0, d.y1) for d in ds] == [(1.0, 2.5, 2.0, 6.0), (2.5, 4.0, 2.0, 6.0), (4.0, 7.0, 2.0, 6.0)]
    assert ds[1].domain.contains(np.array([[2.0, 1.5]])).tolist() == [True]
    assert ds[1].inner.contains(np.array([[2.0, 2.5]])).tolist() == [False]
    with pytest.raises(ValueError):
        U.partition2d(0, 0, [1, 2], [1.0], [1], [1.0], 0.1)
    with pytest.raises(ValueError):
        U.partition2d(0, 0, [1], [-1.0], [1], [1.0], 0.1)


def test_pressure_bc_sides():
    d = U.partition2d(0.0, 0.0, [1], [4.0], [1], [2.0], 1.0)[0]
    centers = np.array([[-0.5, 1.0, 0], [4.5, 1.0, 0], [2.0, -0.5, 0], [2.0, 2.5, 0]])
    bnd = {"LEFT": np.array([0]), "RIGHT": np.array([1]), "FRONT": np.array([2]), "BACK": np.array([3])}
    bx, by = U.pressure_bc(d, centers, bnd, "Open")
    assert bx == {0: 1.125, 1: -0.125, 2: 0.5, 3: 0.5}
    assert by == {0: 0.5, 1: 0.5, 2: 1.25, 3: -0.25}
    bx, by = U.pressure_bc(d, centers, bnd, "Closed")
    assert sorted(bx) == [0, 1] and sorted(by) == [2, 3]
    with pytest.raises(ValueError):
        U.pressure_bc(d, centers, bnd, "Periodic")


def test_domain_box():
    coords = U._tensor_coords(3, 4, 3, 2, 0, 0, 0, 1, 1, -1)
    perm = np.arange(24 * 6, dtype=float).reshape(24, 6)
    els = np.array([1 + 4 * j + 12 * k for k in range(2) for j in range(1, 3)] +
                   [2 + 4 * j + 12 * k for k in range(2) for j in range(1, 3)])
    dims, local, pts, pm = U.domain_box(3, 4, 3, 2, coords, perm, els)
    assert dims == (2, 2, 2)
    assert local.tolist() == [5, 6, 9, 10, 17, 18, 21, 22]
    assert np.array_equal(pm, perm[local])
    assert np.array_equal(pts[0], coords[1 + 5 * 1]) and len(pts) == 27
    with pytest.raises(U.RSGError):
        U.domain_box(3, 4, 3, 2, coords, perm, els[:-1])


def _grid(dim, ni, nj, nk, K, seed=None):
    n = ni * nj * (nk if dim == 3 else 1)
    perm = np.tile(np.asarray(K, float), (n, 1))
    coords = U._tensor_coords(dim, ni, nj, nk, 0.0, 0.0, 0.0, 1.0, 1.0, -1.0)
    return coords, perm


@pytest.mark.parametrize("dim,nk", [(2, 0), (3, 3)])
def test_uniform_tensor_is_reproduced_on_the_oracle(dim, nk):
    """MPFA-O reproduces linear pressure fields, so a homogeneous full tensor
    K with "Open" linear boundary data upscales to itself, times the layer
    thickness in 3D (the formulas are those of a 2-D partition): k11 = kxx H,
    k22 = kyy H, k12 = k21 = kxy H."""
    from upscale_oracle import oracle_upscale
    ni = nj = 12
    K = (2.0, 0.5, 0.1, 0.3, 0.0, 0.0)
    coords, perm = _grid(dim, ni, nj, nk, K)
    doms = U.partition2d(0.0, 0.0, [3], [4.0], [3], [4.0], border=2.0)
    res, _ = oracle_upscale(dim, ni, nj, nk, coords, perm, [doms[4]])
    H = float(nk) if dim == 3 else 1.0
    t = res[0]["tensor"]
    assert np.allclose(t, [K[0] * H, K[1] * H, 0.0, K[3] * H, 0.0, 0.0], rtol=1e-8, atol=1e-9)
    assert abs(res[0]["k21"] - K[3] * H) <= 1e-8 * H
    # the inner box is 4 x 4 cells: four connections per side and layer
    assert all(len(res[0]["inner"][o]) == 4 * max(nk, 1) for o in U.ORIENTATIONS_2D)


def test_l_method_upscaling_of_a_diagonal_tensor_on_the_oracle():
    """With the L-method lists (two-point fluxes at boundary corners, exact for
    K-orthogonal grids) a homogeneous diagonal tensor on a box grid upscales
    to itself times the thickness, with no cross term."""
    from upscale_oracle import oracle_upscale
    ni = nj = 12
    nk = 2
    K = (2.0, 0.5, 0.1, 0.0, 0.0, 0.0)
    coords, perm = _grid(3, ni, nj, nk, K)
    doms = U.partition2d(0.0, 0.0, [3], [4.0], [3], [4.0], border=2.0)
    res, _ = oracle_upscale(3, ni, nj, nk, coords, perm, [doms[4]], method="lmpfa")
    t = res[0]["tensor"]
    assert np.allclose(t, [K[0] * nk, K[1] * nk, 0.0, 0.0, 0.0, 0.0], rtol=1e-8, atol=1e-9)
