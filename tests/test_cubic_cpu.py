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
