"""Host-side model set-up of the package against the oracle and the
reference's sample output (CPU only)."""
import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def setup_mod():
    return importlib.import_module("da-gtm_gb300.gtm_setup")


def test_grid_and_basis_match_reference_output(setup_mod, golden):
    X, FI = setup_mod.setup_grid(3, 125, 8, 2.0)
    assert np.array_equal(X, golden["X"])
    assert np.max(np.abs(FI - golden["FI"])) <= 1e-15


@pytest.mark.parametrize("L,K,M,s", [(2, 400, 16, 1.0), (3, 8000, 64, 2.0), (1, 10, 4, 2.0)])
def test_grid_and_basis_match_oracle(setup_mod, orc, L, K, M, s):
    X, FI = setup_mod.setup_grid(L, K, M, s)
    Xo, FIo = orc.stp(L, K, M, s)
    assert np.array_equal(X, Xo)
    assert np.allclose(FI, FIo, rtol=1e-14, atol=1e-15)


def test_bad_grid_sizes_rejected(setup_mod):
    with pytest.raises(ValueError):
        setup_mod.setup_grid(3, 100, 8)
    with pytest.raises(ValueError):
        setup_mod.setup_grid(2, 400, 10)


def test_mt19937_stream_matches_oracle(setup_mod, orc):
    for seed in (0, 1, 12345):
        assert np.array_equal(setup_mod.mt19937_uniform(seed, 1000), orc.mt_uniform(seed, 1000))


def test_random_init_matches_oracle(setup_mod, orc, golden):
    T = golden["T"]
    X, FI, W, beta = setup_mod.random_init(T, 3, 125, 8, 2.0, seed=7)
    Xo, FIo, Wo, bo = orc.stp3_rnd(7, T, 3, 125, 8, 2.0)
    assert np.array_equal(X, Xo)
    # cond(FI^T FI) ~ 1e10 here: W agrees to ~1e-6 relative, the centres to ~1e-7
    assert np.max(np.abs(FI @ W - FIo @ Wo)) <= 1e-5
    assert beta == pytest.approx(bo, rel=1e-12)


def test_random_init_ill_conditioned_is_least_squares(setup_mod, orc, golden):
    # K = 11^3, M = 3^3: cond(FI^T FI) ~ 4e15, so the reference's normal-equation
    # SVD solve is rounding-dominated and two correct implementations differ in W
    # and Y; both must still be near-optimal least-squares fits of FI W = Yrnd
    # (the normal equations lose ~1e-4 of the residual here).
    T = golden["T"]
    K, M, seed = 1331, 27, 7
    X, FI, W, beta = setup_mod.random_init(T, 3, K, M, 2.0, seed=seed)
    _, _, Wo, bo = orc.stp3_rnd(seed, T, 3, K, M, 2.0)
    mu, sd = setup_mod.mean_sd(T)
    u = setup_mod.mt19937_uniform(seed, K * T.shape[1]).reshape(K, -1)
    Yr = 2 * sd * 6 * (np.ceil(u / 1e-15) * 1e-15) - sd * 6 + mu
    best = np.linalg.lstsq(FI, Yr, rcond=None)[0]
    r_best = np.linalg.norm(FI @ best - Yr)
    assert np.linalg.norm(FI @ W - Yr) <= r_best * (1 + 1e-3)
    assert np.linalg.norm(FI @ Wo - Yr) <= r_best * (1 + 1e-3)
    assert beta == bo == 0.1


def test_critical_temperature_matches_oracle(setup_mod, orc, golden):
    assert setup_mod.first_critical_temp(golden["T"]) == pytest.approx(orc.ctemp(golden["T"]),
                                                                      rel=1e-12)


def test_datasets_shapes_and_values():
    ds = importlib.import_module("da-gtm_gb300.datasets")
    T = ds.make("fp_n100k", N=5000)
    assert T.shape == (5000, 166) and set(np.unique(T)) <= {0.0, 1.0}
    frac = T.mean()
    assert 0.15 < frac < 0.45
    G = ds.make("gmm_n1k")
    assert G.shape == (1000, 12)
    assert np.array_equal(ds.make("gmm_n1k", seed=3), ds.make("gmm_n1k", seed=3))
