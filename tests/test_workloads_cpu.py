"""The seeded synthetic inputs have the shapes and distributions the
benchmarks state: a Gaussian random field with the requested mean and
variance (pooled over seeds, since one correlated field has few independent
samples), lognormal permeabilities with kz = 0.1 kx, porosity in [0.2, 0.3],
nodes perturbed by at most 10% of a cell, ensemble sizes within their
bounds, and the same bytes for the same seed."""
import numpy as np

from ressim_gb300 import workloads as W


def test_grf_moments_over_seeds():
    ms, vs = [], []
    for seed in range(16):
        f = W.grf((32, 32, 8), 4.0, 2.0, 1.0, seed)
        ms.append(f.mean())
        vs.append(f.var())
    assert abs(np.mean(ms) - 2.0) <= 0.15
    assert abs(np.mean(vs) - 1.0) <= 0.15


def test_two_phase_case_fields():
    c = W.two_phase_case(ni=32, nj=24, nk=8, seed=3)
    n = 32 * 24 * 8
    assert c["perm"].shape == (n, 6) and c["porosity"].shape == (n,)
    assert np.all((c["porosity"] >= 0.2) & (c["porosity"] <= 0.3))
    assert np.array_equal(c["perm"][:, 0], c["perm"][:, 1])
    assert np.allclose(c["perm"][:, 2], 0.1 * c["perm"][:, 0], rtol=1e-15)
    assert not c["perm"][:, 3:].any()
    logk = np.log10(c["perm"][:, 0] / W.MILLIDARCY)
    assert 0.5 < logk.std() < 2.0 and 0.5 < logk.mean() < 3.5
    nodes = c["nodes"]
    k, j, i = np.meshgrid(np.arange(9), np.arange(25), np.arange(33), indexing="ij")
    for axis, ideal in ((0, i), (1, j), (2, -k)):
        assert np.max(np.abs(nodes[:, axis] - ideal.reshape(-1))) <= 0.1
    assert len(c["injectors"]) == 4 and len(c["producer"]) == 8


def test_same_seed_same_bytes():
    a = W.two_phase_case(ni=16, nj=16, nk=4, seed=7)
    b = W.two_phase_case(ni=16, nj=16, nk=4, seed=7)
    c = W.two_phase_case(ni=16, nj=16, nk=4, seed=8)
    for key in ("perm", "porosity", "nodes"):
        assert a[key].tobytes() == b[key].tobytes()
        assert a[key].tobytes() != c[key].tobytes()


def test_ensemble_sizes_within_bounds():
    sizes = W.ensemble_sizes(64)
    assert len(sizes) == 64
    for s in sizes:
        assert 32 <= s[0] <= 96 and 32 <= s[1] <= 96 and 8 <= s[2] <= 24
    assert len(set(sizes)) > 1
