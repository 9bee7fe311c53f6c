"""Seeded synthetic data sets with the shapes of the benchmark configurations.

The reference ships one small real data set (oil flow, N = 1000, D = 12); its
fingerprint use case (166-bit chemical fingerprints) is not available here, so
these generators stand in for it with the same shapes and value ranges.

* :func:`gaussian_mixture` -- isotropic mixture with means uniform in [0,1]^D.
* :func:`fingerprints` -- binary vectors: per-feature Bernoulli probabilities
  uniform in [p_lo, p_hi], ``nproto`` prototypes drawn from them, each point a
  copy of a random prototype with every bit flipped with probability ``flip``.
"""
from __future__ import annotations

import numpy as np


def gaussian_mixture(N: int, D: int, ncomp: int, sd: float, seed: int = 0,
                     dtype=np.float64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    means = rng.random((ncomp, D))
    comp = rng.integers(0, ncomp, size=N)
    T = means[comp] + sd * rng.standard_normal((N, D))
    return T.astype(dtype, copy=False)


def fingerprints(N: int, D: int = 166, nproto: int = 20, flip: float = 0.1,
                 p_lo: float = 0.05, p_hi: float = 0.5, seed: int = 0,
                 dtype=np.float64, chunk: int = 1 << 18) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = rng.uniform(p_lo, p_hi, size=D)
    protos = (rng.random((nproto, D)) < p).astype(np.uint8)
    out = np.empty((N, D), dtype=dtype)
    for s in range(0, N, chunk):
        e = min(N, s + chunk)
        comp = rng.integers(0, nproto, size=e - s)
        flips = (rng.random((e - s, D)) < flip).astype(np.uint8)
        out[s:e] = protos[comp] ^ flips
    return out


CONFIGS = {
    # plain FP64 on CPU-sized data (the oil-flow-sized stand-in)
    "gmm_n1k": dict(gen="gmm", N=1000, D=12, ncomp=3, sd=0.1, L=2, K=400, M=16, s=1.0),
    # fingerprint shape, FP64 / FP32 on the GPU
    "fp_n100k": dict(gen="fp", N=100_000, D=166, nproto=20, L=3, K=8000, M=64, s=2.0),
    # the headline shape
    "fp_n1m": dict(gen="fp", N=1_000_000, D=166, nproto=20, L=3, K=8000, M=64, s=2.0),
    # differentiation
    "gmm_n65k": dict(gen="gmm", N=65536, D=64, ncomp=16, sd=0.2, L=2, K=4096, M=16, s=2.0),
    # large split-precision run
    "fp_n4m": dict(gen="fp", N=4_000_000, D=166, nproto=50, L=3, K=32768, M=512, s=2.0),
}


def make(name: str, seed: int = 0, N: int | None = None, dtype=np.float64) -> np.ndarray:
    c = CONFIGS[name]
    n = c["N"] if N is None else N
    if c["gen"] == "gmm":
        return gaussian_mixture(n, c["D"], c["ncomp"], c["sd"], seed, dtype)
    return fingerprints(n, c["D"], c["nproto"], seed=seed, dtype=dtype)
