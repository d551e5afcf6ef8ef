"""util/LookupTable (rs/src/no/uib/cipr/rs/util/LookupTable.java:202-430) in
the oracle, checked by the reference's own LookupTable1DTest / 2DTest /
3DTest (rs/src/no/uib/cipr/rs/util/test/): on axes that start at 0 and 1 with
random interior knots, a constant table is reproduced to 1e-14 with zero
derivatives, a linear one to 1e-14 (1e-4 for the 3D value, as there) with
exact slopes, and a trigonometric one to 1e-4.  The reference draws its
sizes and points with java.util.Random; these tests draw them from seeded
numpy generators.  Two allowances keep the reference's checks meaningful
for every draw: a derivative carries the rounding of the reference's own
formula, phi_k = (+-w or 1 -+ w) / delta summed over the corners, about
4 eps |value| / delta, which exceeds 1e-14 on intervals narrower than a few
hundredths; and the sine tables use evenly spaced knots 0.01 apart (the
linear-interpolation error of a sine is then below 2e-5), because random
knots leave gaps where the reference's own 1e-4 cannot hold.  The slope of
a piecewise-linear table is a chord, within a h / 2 of the sine's derivative
a cos(x) (the reference's 1e-4 there would need knots 2e-4 apart), and is
checked at that bound.  The GPU
evaluates the same tables inside the property chain, whose results are
bit-exact against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi


def _coord(g, n):
    c = np.concatenate([[0.0, 1.0], g.random(n - 2)])
    return np.sort(c)


def _grids(dim, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    sizes = [int(g.integers(2, 1002 if dim == 1 else 102)) for _ in range(dim)]
    coords = [_coord(g, n) for n in sizes]
    a, b, c, e = g.random(4)
    pts = g.random((int(g.integers(1, 100)), dim))
    return g, coords, (a, b, c, e), pts


def _mesh(coords):
    return np.meshgrid(*coords, indexing="ij")


def _deriv_tol(coords, pts, d, scale):
    """1e-14 plus the rounding of the derivative formula on the interval of
    each point along axis d."""
    c = coords[d]
    i = np.clip(np.searchsorted(c, pts[:, d]) - 1, 0, len(c) - 2)
    return 1e-14 + 8 * np.finfo(float).eps * scale / (c[i + 1] - c[i])


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_constant_table(dim, seed):
    _, coords, (a, b, c, e), pts = _grids(dim, seed)
    keep = abi.Keep()
    f = abi.table(keep, coords, np.full(tuple(len(x) for x in coords), e))
    assert np.all(np.abs(O.function_eval(f, pts) - e) <= 1e-14)
    for d in range(dim):
        assert np.all(np.abs(O.function_eval(f, pts, d)) <= _deriv_tol(coords, pts, d, e))


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [4, 5, 6])
def test_linear_table(dim, seed):
    _, coords, (a, b, c, e), pts = _grids(dim, seed)
    slopes = (a, b, c)[:dim]
    grid = _mesh(coords)
    data = e + sum(s * x for s, x in zip(slopes, grid))
    keep = abi.Keep()
    f = abi.table(keep, coords, data)
    exact = e + pts @ np.array(slopes)
    tol = 1e-4 if dim == 3 else 1e-14
    assert np.all(np.abs(O.function_eval(f, pts) - exact) <= tol)
    scale = e + sum(slopes)
    for d in range(dim):
        assert np.all(np.abs(O.function_eval(f, pts, d) - slopes[d]) <= _deriv_tol(coords, pts, d, scale))


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [7, 8, 9])
def test_trigonometric_table(dim, seed):
    _, _, (a, b, c, e), pts = _grids(dim, seed)
    coords = [np.linspace(0.0, 1.0, 101) for _ in range(dim)]
    amps = (a, b, c)[:dim]
    grid = _mesh(coords)
    data = e + sum(s * np.sin(x) for s, x in zip(amps, grid))
    keep = abi.Keep()
    f = abi.table(keep, coords, data)
    exact = e + np.sin(pts) @ np.array(amps)
    assert np.all(np.abs(O.function_eval(f, pts) - exact) <= 1e-4)
    h = 0.01
    for d in range(dim):
        # the table's slope is a chord of a sine: within amp * h / 2 of its cosine
        err = np.abs(O.function_eval(f, pts, d) - amps[d] * np.cos(pts[:, d]))
        assert np.all(err <= amps[d] * h / 2 + 1e-12)
