"""Restart files (rsg_sim_write_restart / rsg_sim_read_restart): RS saves the
Field at report times (rs/src/no/uib/cipr/rs/numerics/Main.java:86-105) and a
restarted Field keeps the primary variables only
(rs/src/no/uib/cipr/rs/field/Field.java:207-262)."""
import numpy as np
import pytest

from ressim_gb300 import api
from ressim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_restart_continues_the_run(ctx, tmp_path):
    """A simulator restarted from the file after two steps holds the same
    time and state bit for bit, and its next two steps agree with the
    uninterrupted run to 1e-12 (the restarted control volumes start without
    the phase records of earlier evaluations, as in RS)."""
    a, case = W.build_two_phase_sim(ctx, 12, 10, 4, seed=2, rtol=1e-12)
    b, _ = W.build_two_phase_sim(ctx, 12, 10, 4, seed=2, rtol=1e-12)
    for _ in range(2):
        a.step(case["dt"])
    f = tmp_path / "field.rst"
    a.write_restart(f)
    raw = f.read_bytes()
    assert raw[:8] == b"RSGRST01" and len(raw) == 8 + 16 + 8 + 8 * (3 + a.nc) * 480
    b.read_restart(f)
    assert b.time() == a.time()
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    for _ in range(2):
        ia, ib = a.step(case["dt"]), b.step(case["dt"])
        assert ia.newton_iterations == ib.newton_iterations
    (pa, Na, Sa), (pb, Nb, Sb) = a.state(), b.state()
    assert np.max(np.abs(pa - pb) / pa) <= 1e-12
    assert np.max(np.abs(Sa - Sb)) <= 1e-12


def test_restart_rejects_other_simulators(ctx, tmp_path):
    a, case = W.build_two_phase_sim(ctx, 12, 10, 4, seed=2)
    c, _ = W.build_two_phase_sim(ctx, 10, 10, 4, seed=2)
    f = tmp_path / "field.rst"
    a.write_restart(f)
    with pytest.raises(api.RSGError):
        c.read_restart(f)
    (tmp_path / "junk.rst").write_bytes(b"not a restart file")
    with pytest.raises(api.RSGError):
        a.read_restart(tmp_path / "junk.rst")
