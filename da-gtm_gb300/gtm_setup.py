"""Host-side model set-up (runs once, before the EM loop).

Own implementation of the reference's set-up path:

* :func:`latent_grid` -- regular grid in [-1, 1]^L, x fastest
  (comm/comm.c:1453-1504, dagtm_rctg);
* :func:`basis` -- Gaussian basis functions plus a bias column
  (comm/comm.c:1506-1536, dagtm_gbf);
* :func:`setup_grid` -- X and FI for K = g^L latent points and M = h^L centres,
  width ``s`` times the centre spacing (comm/comm.c:992-1103, dagtm_stp; the
  reference hard-codes s = 2 at dagtm/dagtm.cxx:1119);
* :func:`random_init` -- W and beta from uniform random centres
  (comm/comm.c:1118-1185,1401-1448: MT19937 seeded like gsl_rng_set,
  mean +- 6 sd, least squares through the SVD of FI^T FI, beta from the
  nearest-neighbour distances when K <= 1000, else 0.1);
* :func:`first_critical_temp` -- lambda_max(cov T) * N D / sum |t - mean|^2
  (comm/mpicomm.c:511-559) and the start temperature T_c / alpha^10
  (dagtm/dagtm.cxx:1148-1158).
"""
from __future__ import annotations

import numpy as np


def latent_grid(L: int, g: int) -> np.ndarray:
    axes = np.arange(g, dtype=np.float64)
    if L == 1:
        X = axes[:, None]
    elif L == 2:
        yy, xx = np.meshgrid(axes, axes, indexing="ij")
        X = np.stack([xx.ravel(), yy.ravel()], axis=1)
    elif L == 3:
        zz, yy, xx = np.meshgrid(axes, axes, axes, indexing="ij")
        X = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)
    else:
        raise ValueError("latent dimension must be 1, 2 or 3")
    return X * (2 / float(g - 1)) + -1.0


def _sqdist(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    # the reference's distance: -2 a.b + |a|^2 + |b|^2
    return (-2.0 * (A @ B.T) + (A * A).sum(1)[:, None]) + (B * B).sum(1)[None, :]


def basis(MU: np.ndarray, X: np.ndarray, sigma: float) -> np.ndarray:
    E = np.exp(_sqdist(X, MU) * (-0.5 / sigma ** 2))
    return np.concatenate([E, np.ones((X.shape[0], 1))], axis=1)


def grid_side(n: int, L: int) -> int:
    g = int(round(n ** (1.0 / L)))
    if g ** L != n:
        raise ValueError(f"{n} is not a perfect {L}-th power")
    return g


def setup_grid(L: int, K: int, M: int, s: float = 2.0):
    if s <= 0:
        raise ValueError("basis width factor must be positive")
    gx, gf = grid_side(K, L), grid_side(M, L)
    X = latent_grid(L, gx)
    MU = latent_grid(L, gf) * (gf / (gf - 1.0))
    sigma = s * (MU[1, 0] - MU[0, 0])
    return X, basis(MU, X, sigma)


def mt19937_uniform(seed: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1) from MT19937 seeded as gsl_rng_set does (0 -> 4357)."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed) if seed != 0 else 4357)
    return bg.random_raw(n).astype(np.float64) / 4294967296.0


def _svd_solve(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    U, s, Vt = np.linalg.svd(A)
    inv = np.where(s != 0.0, 1.0 / np.where(s != 0.0, s, 1.0), 0.0)
    return Vt.T @ (inv[:, None] * (U.T @ B))


def mean_sd(T: np.ndarray):
    N = T.shape[0]
    mu = T.sum(0) * (1.0 / N)
    sd = np.sqrt(((T - mu) ** 2).sum(0) * (1.0 / (N - 1)))
    return mu, sd


def random_init(T: np.ndarray, L: int, K: int, M: int, s: float = 2.0, seed: int = 1):
    """Returns X, FI, W, beta as dagtm_stp3_rnd leaves them."""
    X, FI = setup_grid(L, K, M, s)
    mu, sd = mean_sd(np.asarray(T, dtype=np.float64))
    D = mu.shape[0]
    u = mt19937_uniform(seed, K * D).reshape(K, D)
    rnd = np.ceil(u / 1e-15) * 1e-15
    dev = sd * 6
    Yr = 2 * dev * rnd - dev + mu
    W = _svd_solve(FI.T @ FI, FI.T @ Yr)
    if K > 1000:
        beta = 0.1
    else:
        Dm = _sqdist(Yr, Yr)
        np.fill_diagonal(Dm, np.finfo(np.float64).max)
        m = Dm.min(axis=0).mean()
        beta = 2.0 / (m if m != 0 else 1.0)
    return X, FI, W, beta


def first_critical_temp(T: np.ndarray) -> float:
    T = np.asarray(T, dtype=np.float64)
    N, D = T.shape
    C = T - T.sum(0) * (1.0 / N)
    lam = np.linalg.eigvalsh(C.T @ C).max() / N
    return lam * (N * D) / (C * C).sum()


def start_temp(T: np.ndarray, alpha: float = 0.99) -> float:
    return first_critical_temp(T) / alpha ** 10
