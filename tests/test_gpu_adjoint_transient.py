"""Discrete adjoint of the two-phase simulator run (sequential pressure
Newton step and explicit molar update, Discretisation.java:280-919) with
respect to per-element log-permeability, checked against central finite
differences of the GPU forward and of the oracle forward, with the objective
"oil moles produced into the Fixed producer cells".

Every difference quotient carries the forward run's own rounding: with the
Newton and Krylov tolerances at 1e-13, J is reproducible to about 1e-12 |J|
(GPU) to a few 1e-11 |J| (oracle, and the GPU on 32 x 32 x 8) under a
perturbation, i.e. that much over h in the quotient; each check allows
FD_NOISE * |J| / h (h = 1e-3) or FD_NOISE_H * |J| / h (h = 1e-6) for it.  At
h = 1e-3 in log k that noise and the O(h^2) truncation are both near 1e-6 of
the gradient, so that check is the tight one; at the step h = 1e-6 the noise
is a few 1e-5 |J|.  Measured on the 8 x 8 x 3 case: the adjoint agrees with
h = 1e-4 differences to 5 digits wherever the gradient is above 1e-2 of its
largest entry."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi, api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu

H = 1e-6        # the check step
H_FINE = 1e-3   # the accuracy step
FD_NOISE = 2e-11     # rounding of J under a perturbation, relative, at h = 1e-3
FD_NOISE_H = 5e-11   # the same at h = 1e-6 (measured up to 2.4e-11 on 32 x 32 x 8)
TIGHT = dict(rtol=1e-13, atol=1e-24, ptol=1e-13, stop_rule=1, max_newton=60)  # atol: a converged Newton leaves a zero right-hand side


def _sim(ctx, case, perm, spec_kw=TIGHT, corey=None):
    keep = abi.Keep()
    gm = api.Mesh(ctx, 3, case["ni"], case["nj"], case["nk"], perm, coords=case["nodes"])
    gm.compute_mpfa()
    co = corey if corey is not None else W.corey()
    gs = api.Discretisation(ctx, gm, W.two_phase_fluid(keep), co, case["porosity"], case["compaction"],
                            W.build_sources(keep, case), W.build_initial(case), W.runspec(**spec_kw))
    gs._adj_keep = (keep, gm)
    return gs


def _objective(ctx, case, perm, dts, spec_kw=TIGHT):
    gs = _sim(ctx, case, perm, spec_kw)
    J, _ = gs.forward(dts, len(dts), case["producer"], [0.0, 1.0])
    return J


def _oracle_objective(case, perm, dts):
    keep = abi.Keep()
    om = O.Mesh(3, case["ni"], case["nj"], case["nk"], coords=case["nodes"], perm=perm)
    om.mpfa()
    os_ = O.Simulator(om, W.two_phase_fluid(keep), W.corey(), case["porosity"], case["compaction"],
                      W.build_sources(keep, case), W.build_initial(case), W.runspec(**TIGHT))
    J = 0.0
    for dt in dts:
        os_.step(dt)
        J += float(np.sum(os_.last_dn()[1, case["producer"]]))
    return J


def _scaled(perm, e, s):
    p = perm.copy()
    p[e] *= np.exp(s)
    return p


def _case(ni=8, nj=8, nk=3):
    return W.two_phase_case(ni=ni, nj=nj, nk=nk, seed=3, dt=4 * 8640.0)


def _cells(case, count, seed):
    n = case["ni"] * case["nj"] * case["nk"]
    g = np.random.Generator(np.random.PCG64(seed))
    near = [int(case["producer"][0]) + d for d in (1, -1, case["ni"], -case["ni"])]
    return np.unique(np.concatenate([g.choice(n, size=count, replace=False), near]))


@pytest.mark.parametrize("nsteps", [1, 3])
def test_adjoint_gradient_matches_gpu_fd(ctx, nsteps):
    case = _case()
    dts = [case["dt"]] * nsteps
    gs = _sim(ctx, case, case["perm"])
    J, finfo = gs.forward(dts, 2, case["producer"], [0.0, 1.0])
    assert finfo.steps == nsteps and J > 0
    grad, dp0, dN0, binfo = gs.backward(rtol=1e-13)
    assert binfo.backward_steps == nsteps
    assert binfo.recomputed_steps == (nsteps - 1) // 2 * 2
    scale = np.max(np.abs(grad))
    assert scale > 0
    for e in _cells(case, 10, 5):
        fd = (_objective(ctx, case, _scaled(case["perm"], e, H_FINE), dts) -
              _objective(ctx, case, _scaled(case["perm"], e, -H_FINE), dts)) / (2 * H_FINE)
        assert abs(fd - grad[e]) <= FD_NOISE * J / H_FINE + 1e-5 * scale, (e, fd, grad[e], scale)
        fd = (_objective(ctx, case, _scaled(case["perm"], e, H), dts) -
              _objective(ctx, case, _scaled(case["perm"], e, -H), dts)) / (2 * H)
        assert abs(fd - grad[e]) <= FD_NOISE_H * J / H + 1e-4 * abs(fd), (e, fd, grad[e], J)


def test_adjoint_checkpointing_is_exact(ctx):
    case = _case()
    dts = [case["dt"]] * 4
    grads = []
    for every in (4, 2, 1):
        gs = _sim(ctx, case, case["perm"])
        J, _ = gs.forward(dts, every, case["producer"], [0.0, 1.0])
        g, dp0, dN0, info = gs.backward(rtol=1e-13)
        assert info.recomputed_steps == {4: 0, 2: 2, 1: 3}[every]
        grads.append((J, g, dp0, dN0))
        # the simulator is left at the end of the forward run
        p, N, S = gs.state()
        ref = _sim(ctx, case, case["perm"])
        for dt in dts:
            ref.step(dt)
        rp, rN, rS = ref.state()
        assert np.array_equal(p, rp) and np.array_equal(N, rN)
    for J, g, dp0, dN0 in grads[1:]:
        assert J == grads[0][0]
        assert np.array_equal(g, grads[0][1])
        assert np.array_equal(dN0, grads[0][3])


def test_adjoint_initial_state_sensitivity(ctx):
    """dJ/dN0 of the adjoint recursion against FD of the initial moles."""
    case = _case()
    dts = [case["dt"]] * 2
    gs = _sim(ctx, case, case["perm"])
    gs.forward(dts, 2, case["producer"], [0.0, 1.0])
    grad, dp0, dN0, _ = gs.backward(rtol=1e-13)
    base = _sim(ctx, case, case["perm"])
    p0, N0, _ = base.state()
    locked = set(int(c) for c in case["producer"])
    for e in _cells(case, 4, 9):
        if int(e) in locked:
            continue
        for nu in range(2):
            h = 1e-6 * N0[nu, e]
            vals = []
            for s in (h, -h):
                N = N0.copy()
                N[nu, e] += s
                sim = _sim(ctx, case, case["perm"])
                sim.set_state(p0, N)
                vals.append(sim.forward(dts, 2, case["producer"], [0.0, 1.0])[0])
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - dN0[nu, e]) <= 1e-5 * np.max(np.abs(dN0)) + 1e-4 * abs(fd), (e, nu, fd, dN0[nu, e])


def test_adjoint_gradient_matches_oracle_fd(ctx):
    """Finite differences of the oracle forward on a 32 x 32 x 8 grid."""
    case = _case(32, 32, 8)
    dts = [case["dt"]]
    gs = _sim(ctx, case, case["perm"])
    J, _ = gs.forward(dts, 1, case["producer"], [0.0, 1.0])
    assert abs(J - _oracle_objective(case, case["perm"], dts)) <= 1e-9 * abs(J)
    grad, _, _, _ = gs.backward(rtol=1e-13)
    scale = np.max(np.abs(grad))
    for e in _cells(case, 4, 13):
        fd = (_oracle_objective(case, _scaled(case["perm"], e, H_FINE), dts) -
              _oracle_objective(case, _scaled(case["perm"], e, -H_FINE), dts)) / (2 * H_FINE)
        assert abs(fd - grad[e]) <= FD_NOISE * J / H_FINE + 1e-5 * scale, (e, fd, grad[e], scale)
        fd = (_oracle_objective(case, _scaled(case["perm"], e, H), dts) -
              _oracle_objective(case, _scaled(case["perm"], e, -H), dts)) / (2 * H)
        assert abs(fd - grad[e]) <= FD_NOISE_H * J / H + 1e-4 * abs(fd), (e, fd, grad[e], J)


def test_adjoint_gpu_fd_64_cells(ctx):
    """Central differences with step 1e-6 of the GPU forward on 64 seeded
    cells of a 32 x 32 x 8 grid (noise-bounded, see the module docstring)."""
    case = _case(32, 32, 8)
    dts = [case["dt"]]
    gs = _sim(ctx, case, case["perm"])
    J, _ = gs.forward(dts, 1, case["producer"], [0.0, 1.0])
    grad, _, _, _ = gs.backward(rtol=1e-13)
    n = case["ni"] * case["nj"] * case["nk"]
    scale = np.max(np.abs(grad))
    cells = np.random.Generator(np.random.PCG64(64)).choice(n, size=64, replace=False)
    for q, e in enumerate(cells):
        if q % 4 == 0:  # the tight step on every fourth cell
            fd = (_objective(ctx, case, _scaled(case["perm"], e, H_FINE), dts) -
                  _objective(ctx, case, _scaled(case["perm"], e, -H_FINE), dts)) / (2 * H_FINE)
            assert abs(fd - grad[e]) <= FD_NOISE * J / H_FINE + 1e-5 * scale, (e, fd, grad[e], scale)
        fd = (_objective(ctx, case, _scaled(case["perm"], e, H), dts) -
              _objective(ctx, case, _scaled(case["perm"], e, -H), dts)) / (2 * H)
        assert abs(fd - grad[e]) <= FD_NOISE_H * J / H + 1e-4 * abs(fd), (e, fd, grad[e], J)


def test_adjoint_autograd_directional(ctx):
    """torch.autograd.Function over the forward/backward pair (harness only):
    the gradient along a random direction of all log k against central
    differences of the GPU forward."""
    torch = pytest.importorskip("torch")
    case = _case()
    dts = [case["dt"]] * 2
    n = case["ni"] * case["nj"] * case["nk"]

    class CumulativeOil(torch.autograd.Function):
        @staticmethod
        def forward(ctx_, theta):
            perm = case["perm"] * np.exp(theta.detach().numpy())[:, None]
            gs = _sim(ctx, case, perm)
            J, _ = gs.forward(dts, 1, case["producer"], [0.0, 1.0])
            grad, _, _, _ = gs.backward(rtol=1e-13)
            ctx_.save_for_backward(torch.from_numpy(grad))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx_, gout):
            (grad,) = ctx_.saved_tensors
            return gout * grad

    theta = torch.zeros(n, dtype=torch.float64, requires_grad=True)
    J = CumulativeOil.apply(theta)
    J.backward()
    grad = theta.grad.numpy()
    v = np.random.Generator(np.random.PCG64(2)).standard_normal(n)
    jp = _objective(ctx, case, case["perm"] * np.exp(H_FINE * v)[:, None], dts)
    jm = _objective(ctx, case, case["perm"] * np.exp(-H_FINE * v)[:, None], dts)
    fd = (jp - jm) / (2 * H_FINE)
    assert abs(fd - grad @ v) <= FD_NOISE * float(J.detach()) / H_FINE + 1e-5 * np.linalg.norm(grad) * np.linalg.norm(v)


def test_adjoint_contract(ctx):
    """Backward needs a recorded forward run; a second backward gives the same
    gradient; fluids with a cubic equation of state are refused."""
    case = _case()
    gs = _sim(ctx, case, case["perm"])
    with pytest.raises(api.RSGError) as e:
        gs.backward()
    assert e.value.status == abi.BAD_ARG
    dts = [case["dt"]] * 2
    gs.forward(dts, 1, case["producer"], [0.0, 1.0])
    g1 = gs.backward(rtol=1e-13)[0]
    g2 = gs.backward(rtol=1e-13)[0]
    assert np.array_equal(g1, g2)
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    cc = W.compositional_case(6, 6, 2, dt=2000.0)
    m = api.Mesh(ctx, 3, 6, 6, 2, cc["perm"], coords=cc["nodes"])
    m.compute_mpfa()
    cs = api.Discretisation(ctx, m, f, W.corey(), cc["porosity"], cc["compaction"],
                            W.build_compositional_sources(keep, cc, f.nc), W.build_compositional_initial(cc, f.nc),
                            W.runspec())
    with pytest.raises(api.RSGError) as e:
        cs.forward([2000.0], 1, [0], [1.0])
    assert e.value.status == abi.UNSUPPORTED


def test_adjoint_with_capillary_pressure(ctx):
    """Skjaevelands capillary pressures switched on (cw 2 kPa, cow 1 kPa, tens
    of kPa in the water-wet cells): the phase-potential derivatives enter the
    connection terms; central differences of the GPU forward."""
    case = _case()
    dts = [case["dt"]] * 2
    co = W.corey()
    co.cw, co.cow = 2.0e3, 1.0e3
    gs = _sim(ctx, case, case["perm"], corey=co)
    J, _ = gs.forward(dts, 1, case["producer"], [0.0, 1.0])
    grad, _, dN0, _ = gs.backward(rtol=1e-13)
    scale = np.max(np.abs(grad))
    for e in _cells(case, 6, 17):
        vals = []
        for sgn in (1, -1):
            sim = _sim(ctx, case, _scaled(case["perm"], e, sgn * H_FINE), corey=co)
            vals.append(sim.forward(dts, 1, case["producer"], [0.0, 1.0])[0])
        fd = (vals[0] - vals[1]) / (2 * H_FINE)
        assert abs(fd - grad[e]) <= FD_NOISE * J / H_FINE + 1e-5 * scale, (e, fd, grad[e], scale)


def test_adjoint_gpu_fd_headline_grid(ctx):
    """The adjoint on the 128 x 128 x 32 headline grid (524,288 parameters),
    2 steps: central differences (h = 1e-6) of the GPU forward on two seeded
    cells, one beside the producer, within the noise bound of the module
    docstring.  The absolute Krylov tolerance is 1e-17 here: on this grid a
    converged Newton iteration's residual stops near 1e-18, where BiCGstab
    breaks down before reaching the small grids' 1e-24."""
    spec = dict(TIGHT, atol=1e-17)
    case = W.two_phase_case(ni=128, nj=128, nk=32, seed=3, dt=8640.0)
    dts = [case["dt"]] * 2
    gs = _sim(ctx, case, case["perm"], spec)
    J, _ = gs.forward(dts, 1, case["producer"], [0.0, 1.0])
    grad, _, _, _ = gs.backward(rtol=1e-13)
    assert np.all(np.isfinite(grad))
    n = case["ni"] * case["nj"] * case["nk"]
    cells = [int(case["producer"][0]) + 1, int(np.random.Generator(np.random.PCG64(7)).integers(n))]
    for e in cells:
        fd = (_objective(ctx, case, _scaled(case["perm"], e, H), dts, spec) -
              _objective(ctx, case, _scaled(case["perm"], e, -H), dts, spec)) / (2 * H)
        assert abs(fd - grad[e]) <= FD_NOISE_H * abs(J) / H + 1e-4 * abs(fd), (e, fd, grad[e], J)
