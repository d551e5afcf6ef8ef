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
checked at that bound.  util/EvenLookupTable (EvenLookupTable.java:7-175,
the reference's EvenLookupTable1D/2D/3DTest) gets the same three tables on
evenly spaced knots, and agrees with a LookupTable on the same knots.  The
GPU evaluates the same tables inside the property chain, whose results are
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


# EvenLookupTable1DTest / 2DTest / 3DTest (rs/src/no/uib/cipr/rs/util/test/):
# the same three tables on knots 0, 1/(n-1), ... summed one spacing at a
# time, evaluated through EvenLookupTable.getIndex's direct division.  With n
# down to 2 the knots are up to 1 apart, so the sine tables are checked
# against the linear-interpolation bounds a h^2 / 8 (value) and a h / 2 (slope).

def _even(dim, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    sizes = [int(g.integers(2, 1002 if dim == 1 else 102)) for _ in range(dim)]
    coords = []
    for n in sizes:
        c = np.zeros(n)
        for i in range(1, n):
            c[i] = c[i - 1] + 1.0 / (n - 1)
        coords.append(c)
    a, b, c, e = g.random(4)
    pts = g.random((int(g.integers(1, 100)), dim))
    return coords, (a, b, c, e), pts


def _even_fn(keep, coords, data):
    return abi.even_table(keep, [(0.0, 1.0)] * len(coords), data)


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_even_constant_table(dim, seed):
    coords, (a, b, c, e), pts = _even(dim, seed)
    keep = abi.Keep()
    f = _even_fn(keep, coords, np.full(tuple(len(x) for x in coords), e))
    assert np.all(np.abs(O.function_eval(f, pts) - e) <= 1e-14)
    for d in range(dim):
        assert np.all(np.abs(O.function_eval(f, pts, d)) <= _deriv_tol(coords, pts, d, e))


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [14, 15, 16])
def test_even_linear_table(dim, seed):
    coords, (a, b, c, e), pts = _even(dim, seed)
    slopes = (a, b, c)[:dim]
    data = e + sum(s * x for s, x in zip(slopes, _mesh(coords)))
    keep = abi.Keep()
    f = _even_fn(keep, coords, data)
    exact = e + pts @ np.array(slopes)
    tol = 1e-4 if dim == 3 else 1e-14
    assert np.all(np.abs(O.function_eval(f, pts) - exact) <= tol)
    scale = e + sum(slopes)
    for d in range(dim):
        assert np.all(np.abs(O.function_eval(f, pts, d) - slopes[d]) <= _deriv_tol(coords, pts, d, scale))


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("seed", [17, 18, 19])
def test_even_trigonometric_table(dim, seed):
    coords, (a, b, c, e), pts = _even(dim, seed)
    amps = (a, b, c)[:dim]
    data = e + sum(s * np.sin(x) for s, x in zip(amps, _mesh(coords)))
    keep = abi.Keep()
    f = _even_fn(keep, coords, data)
    h = [1.0 / (len(x) - 1) for x in coords]
    exact = e + np.sin(pts) @ np.array(amps)
    bound = sum(s * hd * hd / 8 for s, hd in zip(amps, h))
    assert np.all(np.abs(O.function_eval(f, pts) - exact) <= max(bound, 1e-4) + 1e-12)
    for d in range(dim):
        # the slope along d is a chord of a sine along d, interpolated across the other axes
        other = sum(s * hd * hd / 8 for k, (s, hd) in enumerate(zip(amps, h)) if k != d)
        err = np.abs(O.function_eval(f, pts, d) - amps[d] * np.cos(pts[:, d]))
        assert np.all(err <= amps[d] * h[d] / 2 + 2 * other / h[d] + 1e-12)


def test_even_table_matches_lookup_table():
    """On the same evenly spaced knots an EvenLookupTable and a LookupTable
    interpolate the same data: the direct index and the binary search can
    pick neighbouring intervals only at a knot, where both give the knot's
    value."""
    g = np.random.Generator(np.random.PCG64(20))
    for n in (2, 3, 17, 64, 1001):
        c = np.zeros(n)
        for i in range(1, n):
            c[i] = c[i - 1] + 1.0 / (n - 1)
        data = g.standard_normal(n)
        keep = abi.Keep()
        fe, ft = abi.even_table(keep, [(0.0, 1.0)], data), abi.table(keep, [c], data)
        x = np.concatenate([g.random(200), c, [-0.5, 1.5]])[:, None]
        assert np.allclose(O.function_eval(fe, x), O.function_eval(ft, x), rtol=0, atol=1e-14)
