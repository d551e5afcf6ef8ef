"""The L-method MPFA restatement in the oracle (geometry/flux/L_MPFA.java):
agreement with TPFA and the O-method where all three are exact, and the
reference's own uniform-flow check (MPFA.testUniformFlow, MPFA.java:246-283)
on perturbed grids with a full conductivity tensor.  CPU only."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from oracle import oracle as O  # noqa: E402
from upscale_oracle import here_interface, perturbed_coords  # noqa: E402


def _md_dict(m):
    ptr, el, kk = m.transmissibilities()
    return [dict(zip(el[ptr[c]:ptr[c + 1]].tolist(), kk[ptr[c]:ptr[c + 1]].tolist())) for c in range(len(ptr) - 1)]


def test_l_method_equals_tpfa_on_k_orthogonal_grids():
    """Uniform box cells and a diagonal tensor: every multi-point method
    collapses to the two-point flux."""
    ni, nj, nk = 6, 5, 4
    perm = np.tile([2.0, 1.0, 0.5, 0, 0, 0], (ni * nj * nk, 1))
    res = {}
    for key, kw in (("l", dict(lmethod=True)), ("o", {}), ("t", dict(tpfa=True))):
        m = O.Mesh(3, ni, nj, nk, perm=perm, dx=1.5, dy=0.7, dz=-0.4)
        m.mpfa(**kw)
        res[key] = _md_dict(m)
    for a, b, c in zip(res["l"], res["o"], res["t"]):
        for e in c:
            assert a.get(e, 0.0) == pytest.approx(c[e], rel=1e-12, abs=1e-14)
            assert b.get(e, 0.0) == pytest.approx(c[e], rel=1e-12, abs=1e-14)
        assert all(abs(v) <= 1e-14 for e, v in a.items() if e not in c)


def _interior(ni, nj, nk, h, t):
    """Connections none of whose four face corners lies on the grid boundary."""
    i, j, k = h % ni, (h // ni) % nj, h // (ni * nj)
    d = t - h
    if d == 1:
        return 0 < j < nj - 1 and 0 < k < nk - 1
    if d == ni:
        return 0 < i < ni - 1 and 0 < k < nk - 1
    return 0 < i < ni - 1 and 0 < j < nj - 1


@pytest.mark.parametrize("lmethod", [True, False])
def test_uniform_flow_on_perturbed_grid(lmethod):
    """A linear potential p = g . x on a perturbed grid with a homogeneous
    full tensor K: sum_k t_k p(x_k) equals the exact flux -(K g) . n A over
    every connection away from the boundary (whose points use the two-point
    rule), within 1e-8 relative."""
    ni, nj, nk = 7, 6, 5
    coords = perturbed_coords(3, ni, nj, nk, seed=5)
    K = np.array([[2.0, 0.3, 0.1], [0.3, 1.0, 0.2], [0.1, 0.2, 0.5]])
    perm = np.tile([K[0, 0], K[1, 1], K[2, 2], K[0, 1], K[0, 2], K[1, 2]], (ni * nj * nk, 1))
    m = O.Mesh(3, ni, nj, nk, coords=coords, perm=perm)
    m.mpfa(lmethod=lmethod)
    geo = m.geometry()
    conn = m.connections()
    hi = here_interface(3, ni, nj, conn)
    g = np.array([0.7, -0.4, 0.25])
    p = geo["centers"] @ g
    ptr, el, kk = m.transmissibilities()
    checked = 0
    for c, (h, t) in enumerate(conn.tolist()):
        if not _interior(ni, nj, nk, h, t):
            continue
        f = 0.0
        for q in range(ptr[c], ptr[c + 1]):
            f += kk[q] * p[el[q]]
        exact = -(K @ g) @ geo["inormal"][hi[c]] * geo["iarea"][hi[c]]
        assert f == pytest.approx(exact, rel=1e-8, abs=1e-12), (c, f, exact)
        checked += 1
    assert checked > 100


def test_l_method_row_sums_and_sides():
    """Every connection's coefficients sum to zero and include both sides
    (Connection.check), on a perturbed grid with a lognormal tensor field."""
    ni, nj, nk = 6, 6, 4
    n = ni * nj * nk
    g = np.random.Generator(np.random.PCG64(3))
    k = 10.0 ** g.standard_normal(n)
    perm = np.stack([k, k, 0.1 * k, 0.1 * k, 0.0 * k, 0.0 * k], axis=1)
    m = O.Mesh(3, ni, nj, nk, coords=perturbed_coords(3, ni, nj, nk, seed=8), perm=perm)
    m.mpfa(lmethod=True)
    ptr, el, kk = m.transmissibilities()
    conn = m.connections()
    for c in range(len(ptr) - 1):
        row = kk[ptr[c]:ptr[c + 1]]
        assert abs(row.sum()) <= 1e-9 * np.max(np.abs(row))
        els = set(el[ptr[c]:ptr[c + 1]].tolist())
        assert conn[c][0] in els and conn[c][1] in els


def test_l_method_needs_3d():
    m = O.Mesh(2, 4, 4, 0, perm=np.tile([1.0, 1.0, 1.0, 0, 0, 0], (16, 1)))
    with pytest.raises(O.OracleError):
        m.mpfa(lmethod=True)
