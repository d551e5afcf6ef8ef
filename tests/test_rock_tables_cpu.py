"""TabularRockFluid and ThreePhaseTabularRockFluid on the oracle
(rs/src/no/uib/cipr/rs/rock/TabularRockFluid.java:31-93,
ThreePhaseTabularRockFluid.java:31-80)."""
import numpy as np
import pytest

from oracle import oracle as O
from ressim_gb300 import abi
from ressim_gb300 import workloads as W


def _two_phase(kind=None, tables_kw=None, corey=None, spec_kw=None):
    case = W.two_phase_case(ni=10, nj=8, nk=4, seed=1)
    keep = abi.Keep()
    m = O.Mesh(3, 10, 8, 4, coords=case["nodes"], perm=case["perm"])
    m.mpfa()
    sim = O.Simulator(m, W.two_phase_fluid(keep), corey or W.corey(), case["porosity"], case["compaction"],
                      W.build_sources(keep, case), W.build_initial(case), W.runspec(**(spec_kw or {})))
    if kind is not None:
        sim.set_rock_tables(W.rock_tables(keep, kind, **(tables_kw or {})))
    return case, sim, keep


def test_linear_tables_reproduce_linear_corey():
    """Two-point tables of the linear Corey curves (exponent 1) reproduce the
    Corey model: the same Newton counts and states within 1e-11 (the two
    evaluate the same straight lines in a different rounding order)."""
    c1 = W.corey(n=1.0)
    case, a, keep = _two_phase(corey=c1, spec_kw=dict(rtol=1e-12))
    _, b, keep2 = _two_phase(corey=c1, spec_kw=dict(rtol=1e-12))
    t = abi.rsg_rock_tables()
    t.kind = abi.RF_TABULAR
    s = [0.2, 0.8]
    t.krw = abi.table(keep2, [s], [0.0, 1.0])
    t.krow = abi.table(keep2, [s], [0.0, 1.0])
    t.krg = abi.constant(0.0)
    t.krog = abi.constant(0.0)
    t.kro = abi.constant(0.0)
    t.pcow = abi.constant(0.0)
    t.pcgo = abi.constant(0.0)
    b.set_rock_tables(t)
    for _ in range(3):
        ia, ib = a.step(case["dt"]), b.step(case["dt"])
        assert ia.newton_iterations == ib.newton_iterations
    (pa, Na, Sa), (pb, Nb, Sb) = a.state(), b.state()
    assert np.max(np.abs(pa - pb) / pa) <= 1e-11
    assert np.max(np.abs(Sa - Sb)) <= 1e-11


@pytest.mark.parametrize("kind", [abi.RF_TABULAR, abi.RF_THREE_PHASE_TABULAR])
def test_tabular_steps_balance_mass(kind):
    case, sim, keep = _two_phase(kind)
    for _ in range(3):
        info = sim.step(case["dt"])
        assert info.mass_balance_error <= 1e-12


def test_relperm_tables_are_checked():
    """getRelPermTable: relative permeabilities outside [0, 1] are rejected."""
    case, sim, keep = _two_phase()
    t = W.rock_tables(keep)
    t.krw = abi.table(keep, [[0.0, 1.0]], [0.0, 1.5])
    with pytest.raises(O.OracleError):
        sim.set_rock_tables(t)
