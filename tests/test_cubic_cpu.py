"""Oracle checks of the cubic equation of state
(rs/src/no/uib/cipr/rs/fluid/CubicEquationOfState.java): the reference's
CubicEquationTest known answers, and invariants of the flash."""
import json
import os

import numpy as np

from oracle import oracle as O
from ressim_gb300 import abi
from ressim_gb300 import workloads as W


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cubic_equation_kats.json")


def test_cubic_equation_kats():
    # rs/src/no/uib/cipr/rs/util/test/CubicEquationTest.java, extracted by tests/golden/make_golden.py
    kats = json.load(open(GOLDEN))["kats"]
    assert len(kats) == 4
    for k in kats:
        zmin, _, zmax = O.cubic_roots(*k["coefficients"])
        assert abs(zmax - k["largest"]) <= k["tolerance"] and abs(zmin - k["smallest"]) <= k["tolerance"]


def test_flash_invariants():
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    nc = f.nc
    p, T, N = W.compositional_cells(400, nc)
    ph, its = O.cubic_phase_state(f, p, T, N)
    oil_p, gas_p = ph[1, 0] > 0, ph[2, 0] > 0
    assert (oil_p | gas_p).all()
    # hydrocarbon moles split between the phases
    tot = ph[1, 6:6 + nc] + ph[2, 6:6 + nc]
    assert np.max(np.abs(tot[1:] - N[1:]) / np.maximum(N[1:], 1e-300)) <= 1e-12
    # water phase where there is water
    assert np.array_equal(ph[0, 0] > 0, N[0] > 0)
    # both phases: molar volumes positive, gas lighter than oil
    both = oil_p & gas_p
    assert both.any()
    assert (ph[1, 2][both] > ph[2, 2][both]).all()
    assert (ph[1, 1][oil_p] > 0).all() and (ph[2, 1][gas_p] > 0).all()
    # a second call starts from the persisted phases and needs no more iterations
    ph2, its2 = O.cubic_phase_state(f, p, T, N, ph)
    assert (its2[both] <= its[both]).all()
    assert np.array_equal(ph2[1, 0], ph[1, 0])


RGAS = 8.3145  # util/Constants.java:23


def _eos_constants(eos, omega):
    """The two-parameter cubic P = RT/(V - b) - a/((V + s b)(V + e b)) with
    CubicEquationOfState's EOS constants and m(omega)
    (fluid/CubicEquationOfState.java:24-46), written as (s, e, OmegaA, OmegaB, m)."""
    if eos == abi.EOS_PR:
        return 1 + 2 ** 0.5, 1 - 2 ** 0.5, 0.457235529, 0.077796074, 0.37464 + 1.53226 * omega - 0.26992 * omega ** 2
    return 1.0, 0.0, 0.42748, 0.08664, 0.48508 + 1.55171 * omega - 0.15613 * omega ** 2


def test_single_component_volumes_follow_the_cubic():
    """Peng-Robinson and Soave-Redlich-Kwong, one hydrocarbon component: the
    phase volume equals Z R T N / p with Z the largest real root of
    Z^3 + ((s + e - 1) B - 1) Z^2 + (A + s e B^2 - (s + e) B (B + 1)) Z
    - (A B + s e B^2 (B + 1)) = 0, solved here with numpy, at supercritical
    states and at a low-pressure state with three real roots (the vapour root)."""
    Tc, pc, om = 304.13, 73.77e5, 0.225
    Tr = np.array([1.2, 1.5, 2.0, 1.1, 3.0])
    pr = np.array([2.0, 1.0, 3.0, 4.0, 0.5])
    T, p = Tr * Tc, pr * pc
    N = np.zeros((2, len(T)))
    N[1] = 7.0
    for eos in (abi.EOS_PR, abi.EOS_SRK):
        keep = abi.Keep()
        f = W.compositional_fluid(keep, nhc=1)
        f.eos = eos
        f.Tc[1], f.pc[1], f.omega[1], f.shift[1] = Tc, pc, om, 0.0
        ph, _ = O.cubic_phase_state(f, p, T, N)
        assert ((ph[1, 0] > 0) ^ (ph[2, 0] > 0)).all()  # one hydrocarbon phase
        V = np.where(ph[1, 0] > 0, ph[1, 1], ph[2, 1])
        s, e, OA, OB, m = _eos_constants(eos, om)
        for i in range(len(T)):
            alpha = (1 + m * (1 - np.sqrt(Tr[i]))) ** 2
            A = OA * RGAS ** 2 * Tc ** 2 / pc * alpha * p[i] / (RGAS * T[i]) ** 2
            B = OB * RGAS * Tc / pc * p[i] / (RGAS * T[i])
            roots = np.roots([1, (s + e - 1) * B - 1, A + s * e * B ** 2 - (s + e) * B * (B + 1),
                              -(A * B + s * e * B ** 2 * (B + 1))])
            Z = roots[np.abs(roots.imag) < 1e-10].real.max()
            assert abs(V[i] - Z * RGAS * T[i] * N[1, i] / p[i]) <= 1e-12 * V[i]


def test_two_phase_cells_are_at_equilibrium():
    """At every two-phase cell of the flash, recomputed here with numpy from
    the returned phase compositions (Peng-Robinson mixture a and b with the
    binary interaction coefficients, fugacity coefficients of the generic
    two-parameter cubic): the oil volume is the smallest real root, the gas
    volume the largest (to 1e-12 in Z), and oil and gas fugacities agree to
    the flash tolerance (CubicEquationOfState.java:871-970, |f_oil - f_gas| <
    FlashTolerance = 0.1 Pa)."""
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    nc = f.nc
    p, T, N = W.compositional_cells(400, nc)
    ph, _ = O.cubic_phase_state(f, p, T, N)
    both = np.nonzero((ph[1, 0] > 0) & (ph[2, 0] > 0))[0]
    assert len(both) >= 10
    s, e, OA, OB, _ = _eos_constants(abi.EOS_PR, 0.0)
    hc = range(1, nc)
    for c in both:
        a_i, b_i = {}, {}
        for i in hc:
            w = f.omega[i]
            m = (0.379642 + 1.48503 * w - 0.164423 * w * w + 0.016666 * w ** 3 if w > 0.49
                 else _eos_constants(abi.EOS_PR, w)[4])
            a_i[i] = OA * RGAS ** 2 * f.Tc[i] ** 2 / f.pc[i] * (1 + m * (1 - np.sqrt(T[c] / f.Tc[i]))) ** 2
            b_i[i] = OB * RGAS * f.Tc[i] / f.pc[i]
        aij = {(i, j): (1 - f.bic[i * abi.MAX_COMPONENTS + j]) * np.sqrt(a_i[i] * a_i[j]) for i in hc for j in hc}
        fug = []
        for a_ph in (1, 2):
            Nph = ph[a_ph, 6:6 + nc, c]
            x = {i: Nph[i] / Nph[1:].sum() for i in hc}
            a = sum(x[i] * x[j] * aij[i, j] for i in hc for j in hc)
            b = sum(x[i] * b_i[i] for i in hc)
            A, B = a * p[c] / (RGAS * T[c]) ** 2, b * p[c] / (RGAS * T[c])
            roots = np.roots([1, (s + e - 1) * B - 1, A + s * e * B ** 2 - (s + e) * B * (B + 1),
                              -(A * B + s * e * B ** 2 * (B + 1))])
            real = roots[np.abs(roots.imag) < 1e-8].real
            Z = p[c] * ph[a_ph, 1, c] / (RGAS * T[c] * Nph[1:].sum())
            assert abs(Z - (real.min() if a_ph == 1 else real.max())) <= 1e-12
            lnphi = {i: b_i[i] / b * (Z - 1) - np.log(Z - B)
                     - A / (B * (s - e)) * (2 * sum(x[j] * aij[i, j] for j in hc) / a - b_i[i] / b)
                     * np.log((Z + s * B) / (Z + e * B)) for i in hc}
            fug.append({i: x[i] * p[c] * np.exp(lnphi[i]) for i in hc})
        assert max(abs(fug[0][i] - fug[1][i]) for i in hc) <= f.flash_tolerance * 1.01


def test_phase_state_volume_derivatives():
    """CubicEquationOfState's total-volume derivatives dV/dp, dV/dT and dV/dN
    (the volume derivatives :621-660 and the flash sensitivities they carry
    in two-phase cells) against central differences of the phase state.  The
    step is 1e-4 relative: small enough for the truncation error, large
    enough that the warm-started flash re-equilibrates beyond its 0.1 Pa
    fugacity tolerance.  At 1e-6 a two-phase cell often takes one iteration
    and keeps its old split, and the difference then measures that frozen
    split.  Components with fewer moles than twice the step are skipped."""
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    nc = f.nc
    p, T, N = W.compositional_cells(400, nc)
    ph, _ = O.cubic_phase_state(f, p, T, N)

    def total(q, fld):
        return q[1, fld] * (q[1, 0] > 0) + q[2, fld] * (q[2, 0] > 0)

    def check(pp, TT, Np, Nm, pm, Tm, h, fld, ok):
        qp, _ = O.cubic_phase_state(f, pp, TT, Np, ph.copy())
        qm, _ = O.cubic_phase_state(f, pm, Tm, Nm, ph.copy())
        keep_regime = ok & ((qp[1, 0] > 0) == (qm[1, 0] > 0)) & ((qp[2, 0] > 0) == (qm[2, 0] > 0))
        fd = (total(qp, 1) - total(qm, 1)) / (2 * np.where(ok, h, 1.0))
        an = total(ph, fld)
        assert keep_regime.sum() >= 0.9 * ok.sum()
        err = np.abs(fd - an)[keep_regime] / np.abs(an)[keep_regime]
        assert np.max(err) <= 2e-6, (fld, np.max(err))

    everywhere = np.ones(len(p), bool)
    hp, hT = 1e-4 * p, 1e-4 * T
    check(p + hp, T, N, N, p - hp, T, hp, 3, everywhere)
    check(p, T + hT, N, N, p, T - hT, hT, 4, everywhere)
    for nu in range(1, nc):
        h = 1e-4 * N[1:].sum(axis=0)
        ok = N[nu] > 2 * h
        h = np.where(ok, h, 0.0)
        Np, Nm = N.copy(), N.copy()
        Np[nu] += h
        Nm[nu] -= h
        check(p, T, Np, Nm, p, T, h, 6 + nc + nu, ok)
