"""Discrete adjoint with respect to per-element log-permeability.

The transmissibility adjoint (reverse mode through T = C A^-1 B - D of every
interaction region, O_MPFA.java:193-239) and the steady potential-problem
gradient (PotentialCalculator.java:319-333, transposed solve on the GPU) are
checked against central finite differences (step 1e-6 in log k) of the
oracle's MPFA-O forward and of the GPU forward, on seeded random elements.
A torch.autograd.Function wraps the GPU forward/backward pair here in the
test harness only."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

H = 1e-6  # central-difference step in log k


def _spd_perm(n, seed):
    """Full symmetric positive definite tensors (xx yy zz xy xz yz), ~100 mD."""
    g = np.random.Generator(np.random.PCG64(seed))
    out = np.zeros((n, 6))
    for e in range(n):
        Q, _ = np.linalg.qr(g.standard_normal((3, 3)))
        K = Q @ np.diag(10.0 ** g.uniform(1.0, 3.0, 3)) @ Q.T * W.MILLIDARCY
        out[e] = (K[0, 0], K[1, 1], K[2, 2], K[0, 1], K[0, 2], K[1, 2])
    return out


def _scaled(perm, e, s):
    p = perm.copy()
    p[e] *= np.exp(s)
    return p


def _flux_functional(ptr, el, kk, mu, phi):
    """sum_c mu_c sum_m t_cm phi[el_m] from MD lists."""
    per_entry = kk * phi[el]
    flux = np.add.reduceat(per_entry, ptr[:-1]) if len(per_entry) else np.zeros(len(mu))
    flux[ptr[:-1] == ptr[1:]] = 0
    return float(mu @ flux)


CASES = {
    "2d_12x10": dict(dim=2, ni=12, nj=10, nk=0),
    "3d_6x5x4": dict(dim=3, ni=6, nj=5, nk=4),
}


def _case(name):
    c = CASES[name]
    dim, ni, nj, nk = c["dim"], c["ni"], c["nj"], c["nk"]
    n = ni * nj * (nk if dim == 3 else 1)
    perm = _spd_perm(n, 7)
    if dim == 2:
        perm = W.potential_case(ni=ni, nj=nj, seed=3, corr_len=3.0)["perm"]
    coords = W.perturbed_nodes(ni, nj, nk, 1.0, 1.0, -1.0, 0.1, 4) if dim == 3 else None
    return dim, ni, nj, nk, n, perm, coords


@pytest.mark.parametrize("name", list(CASES))
def test_transmissibility_adjoint_matches_fd(ctx, name):
    dim, ni, nj, nk, n, perm, coords = _case(name)
    gm = api.Mesh(ctx, dim, ni, nj, nk, perm, coords=coords)
    gm.compute_mpfa()
    nconn = gm.counts()["connections"]
    g = np.random.Generator(np.random.PCG64(11))
    mu = g.standard_normal((2, nconn))
    phi = g.standard_normal((2, n)) * 1e5
    grad = gm.transmissibility_adjoint(mu, phi)
    cells = g.choice(n, size=min(16, n), replace=False)
    scale = np.max(np.abs(grad))
    for e in cells:
        vals = []
        for s in (H, -H):
            om = O.Mesh(dim, ni, nj, nk, coords=coords, perm=_scaled(perm, e, s))
            om.mpfa()
            ptr, el, kk = om.transmissibilities()
            vals.append(sum(_flux_functional(ptr, el, kk, mu[k], phi[k]) for k in range(2)))
        fd = (vals[0] - vals[1]) / (2 * H)
        assert abs(fd - grad[e]) <= 1e-6 * scale + 1e-6 * abs(fd), (e, fd, grad[e])
    # the same check against the GPU forward for two of the elements
    for e in cells[:2]:
        vals = []
        for s in (H, -H):
            m2 = api.Mesh(ctx, dim, ni, nj, nk, _scaled(perm, e, s), coords=coords)
            m2.compute_mpfa()
            ptr, el, kk = m2.transmissibilities()
            vals.append(sum(_flux_functional(ptr, el, kk, mu[k], phi[k]) for k in range(2)))
            m2.release()
        fd = (vals[0] - vals[1]) / (2 * H)
        assert abs(fd - grad[e]) <= 1e-6 * scale + 1e-6 * abs(fd)


def test_transmissibility_adjoint_linear_in_pairs(ctx):
    dim, ni, nj, nk, n, perm, coords = _case("3d_6x5x4")
    gm = api.Mesh(ctx, dim, ni, nj, nk, perm, coords=coords)
    gm.compute_mpfa()
    nconn = gm.counts()["connections"]
    g = np.random.Generator(np.random.PCG64(5))
    mu = g.standard_normal((2, nconn))
    phi = g.standard_normal((2, n))
    both = gm.transmissibility_adjoint(mu, phi)
    one = gm.transmissibility_adjoint(mu[:1], phi[:1]) + gm.transmissibility_adjoint(mu[1:], phi[1:])
    assert np.allclose(both, one, rtol=1e-12, atol=1e-12 * np.max(np.abs(both)))
    # a constant potential carries no flux (sum_m t_cm = 0), so no gradient
    flat = gm.transmissibility_adjoint(mu[:1], np.ones((1, n)))
    assert np.max(np.abs(flat)) <= 1e-6 * np.max(np.abs(both))


def _potential_problem(ctx, ni, nj, perm_scale=None):
    case = W.potential_case(ni=ni, nj=nj, seed=2, corr_len=4.0, rate=2e-15)
    perm = case["perm"] if perm_scale is None else case["perm"] * np.exp(perm_scale)[:, None]
    return case, perm


def _gpu_forward(ctx, case, perm, rtol=1e-14):
    ni, nj = case["ni"], case["nj"]
    gm = api.Mesh(ctx, 2, ni, nj, 0, perm)
    gm.compute_mpfa()
    rp, col = gm.pattern(1)
    A = api.CompRowMatrix(ctx, len(rp) - 1, rp, col)
    gm.assemble_potential(A)
    A.zero_rows(1.0, case["dirichlet_cells"])
    b = W.potential_rhs(case)
    s = api.BiCGstab(ctx, abi.PC_ILU, rtol=rtol)
    s.set_matrix(A)
    p = s.solve(A, b, np.zeros(len(b)))
    return gm, A, s, p


def _oracle_forward(case, perm):
    ni, nj = case["ni"], case["nj"]
    om = O.Mesh(2, ni, nj, 0, perm=perm)
    om.mpfa()
    rp, col = om.pattern(1)
    val = O.zero_rows(rp, col, O.potential_matrix(om, rp, col), 1.0, case["dirichlet_cells"])
    n = len(rp) - 1
    A = np.zeros((n, n))
    for r in range(n):
        A[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    return np.linalg.solve(A, W.potential_rhs(case))


def test_potential_adjoint_matches_oracle_fd(ctx):
    """J = w^T p on a 32 x 32 full-tensor potential problem; 64 seeded cells
    against central differences of the oracle forward (dense solve)."""
    case, perm = _potential_problem(ctx, 32, 32)
    n = 32 * 32
    gm, A, s, p = _gpu_forward(ctx, case, perm)
    w = np.random.Generator(np.random.PCG64(21)).standard_normal(n)
    solver = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-14)
    grad, lam = gm.potential_adjoint(solver, A, case["dirichlet_cells"], p, w)
    assert solver.last_info.iterations > 0
    # the adjoint solution satisfies A^T lambda = w
    At = np.zeros((n, n))
    rp, col = gm.pattern(1)
    vals = A.get_values()
    for r in range(n):
        At[col[rp[r]:rp[r + 1]], r] = vals[rp[r]:rp[r + 1]]
    assert np.linalg.norm(At @ lam - w) <= 1e-12 * np.linalg.norm(w) * 10
    cells = np.random.Generator(np.random.PCG64(64)).choice(n, size=64, replace=False)
    scale = np.max(np.abs(grad))
    for e in cells:
        jp = w @ _oracle_forward(case, _scaled(perm, e, H))
        jm = w @ _oracle_forward(case, _scaled(perm, e, -H))
        fd = (jp - jm) / (2 * H)
        assert abs(fd - grad[e]) <= 2e-6 * scale, (e, fd, grad[e])


def test_potential_adjoint_matches_gpu_fd_and_autograd(ctx):
    torch = pytest.importorskip("torch")
    case, perm = _potential_problem(ctx, 24, 20)
    n = 24 * 20
    w = np.random.Generator(np.random.PCG64(3)).standard_normal(n)

    class PotentialObjective(torch.autograd.Function):
        """J(theta) = w^T p(theta): forward on the GPU, backward by the adjoint."""

        @staticmethod
        def forward(ctx_, theta):
            th = theta.detach().cpu().numpy()
            gm, A, s, p = _gpu_forward(ctx, case, perm * np.exp(th)[:, None])
            solver = api.BiCGstab(ctx, abi.PC_ILU, rtol=1e-14)
            grad, _ = gm.potential_adjoint(solver, A, case["dirichlet_cells"], p, w)
            ctx_.save_for_backward(torch.from_numpy(grad))
            return torch.tensor(float(w @ p), dtype=torch.float64)

        @staticmethod
        def backward(ctx_, gout):
            (grad,) = ctx_.saved_tensors
            return gout * grad

    theta = torch.zeros(n, dtype=torch.float64, requires_grad=True)
    J = PotentialObjective.apply(theta)
    J.backward()
    grad = theta.grad.numpy()
    # directional derivative along a random direction against GPU forward FD
    v = np.random.Generator(np.random.PCG64(9)).standard_normal(n)
    jp = w @ _gpu_forward(ctx, case, perm * np.exp(H * v)[:, None])[3]
    jm = w @ _gpu_forward(ctx, case, perm * np.exp(-H * v)[:, None])[3]
    fd = (jp - jm) / (2 * H)
    assert abs(fd - grad @ v) <= 1e-6 * np.linalg.norm(grad) * np.linalg.norm(v)
    # single elements against GPU forward FD
    for e in (5, 137, 300):
        jp = w @ _gpu_forward(ctx, case, _scaled(perm, e, H))[3]
        jm = w @ _gpu_forward(ctx, case, _scaled(perm, e, -H))[3]
        assert abs((jp - jm) / (2 * H) - grad[e]) <= 2e-6 * np.max(np.abs(grad))


def test_tpfa_transmissibility_adjoint_matches_fd(ctx):
    dim, ni, nj, nk, n, perm, coords = _case("3d_6x5x4")
    gm = api.Mesh(ctx, dim, ni, nj, nk, perm, coords=coords)
    gm.compute_tpfa()
    nconn = gm.counts()["connections"]
    g = np.random.Generator(np.random.PCG64(12))
    mu = g.standard_normal((2, nconn))
    phi = g.standard_normal((2, n)) * 1e5
    grad = gm.transmissibility_adjoint(mu, phi)
    scale = np.max(np.abs(grad))
    for e in g.choice(n, size=12, replace=False):
        vals = []
        for s in (H, -H):
            om = O.Mesh(dim, ni, nj, nk, coords=coords, perm=_scaled(perm, e, s))
            om.mpfa(tpfa=True)
            ptr, el, kk = om.transmissibilities()
            vals.append(sum(_flux_functional(ptr, el, kk, mu[k], phi[k]) for k in range(2)))
        fd = (vals[0] - vals[1]) / (2 * H)
        assert abs(fd - grad[e]) <= 1e-6 * scale + 1e-6 * abs(fd), (e, fd, grad[e])


def test_potential_adjoint_releases_the_solver(ctx):
    """The transposed system exists only inside the call: afterwards the
    solver has no matrix and asks for rsg_solver_setup again."""
    case, perm = _potential_problem(ctx, 12, 10)
    gm, A, s, p = _gpu_forward(ctx, case, perm, rtol=1e-12)
    w = np.ones(len(p))
    gm.potential_adjoint(s, A, case["dirichlet_cells"], p, w)
    with pytest.raises(api.RSGError) as e:
        s.solve(A, W.potential_rhs(case), np.zeros(len(p)))
    assert e.value.status == abi.BAD_ARG
    s.set_matrix(A)
    x = s.solve(A, W.potential_rhs(case), np.zeros(len(p)))
    assert np.max(np.abs(x - p)) <= 1e-9 * np.max(np.abs(p))
