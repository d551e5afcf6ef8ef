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
