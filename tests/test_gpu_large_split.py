"""The large split-precision configuration at its full size: N = 4,000,000
binary points in D = 166 (50 prototypes), K = 32,768 (32^3), M = 512 (8^3)
basis functions + bias, split-BF16 form; then gradient projection of
1,000,000 held-out points of the same generator onto the fixed map through
the backward kernels.

The dense oracle cannot run at this size; the checks are size-independent:
every column of R sums to one, so sum_k G_k = N and sum_k RT_k = sum_n t_n
(split form: 2e-5, as at the headline size); beta and the new centres are
finite; projected points end nearer the map than they started.

Basis width factor 0.5: with the reference's 2, M = 512 basis functions on
a 32^3 grid are numerically dependent (cond(FI^T FI) = 3e19, 262 eigenvalues
below 1e-12 of the largest), W is not determined and the new centres reach
+-100 where the data lie in [0, 1].  At 0.5, cond(FI^T FI) = 6e5.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_large_split_configuration(pkg):
    ds = importlib.import_module(pkg.__name__ + ".datasets")
    st = importlib.import_module(pkg.__name__ + ".gtm_setup")
    ag = importlib.import_module(pkg.__name__ + ".autograd")
    N, D, K, M = 4_000_000, 166, 32768, 512
    T = ds.fingerprints(N, D, 50, seed=2)
    X, FI = st.setup_grid(3, K, M, 0.5)
    assert FI.shape == (K, M + 1)
    rng = np.random.default_rng(2)
    Y = T[rng.integers(0, N, K)] * 0.7 + 0.15 + 0.05 * rng.standard_normal((K, D))
    temp = st.start_temp(T[:200_000], 0.99)
    beta = 4.0
    with pkg.Context(T, FI, "bf16x3") as c:
        c.set_Y(Y)
        llh, nfree = c.estep(beta, 1, temp)
        b, _, Yn = c.mstep(want_W=False, want_Y=True)
        G, RT = c.get_stats()
    assert np.isfinite(llh) and np.isfinite(nfree)
    assert abs(G.sum() - N) / N <= 2e-5
    colsum = T.sum(axis=0)
    assert np.max(np.abs(RT.sum(axis=0) - colsum)) <= 2e-5 * np.max(colsum)
    assert np.isfinite(b) and b > 0 and np.all(np.isfinite(Yn))
    assert -2.0 <= Yn.min() and Yn.max() <= 3.0  # binary data: a smooth fit near [0, 1]
    del T
    # held-out points of the same generator, projected onto the fixed map
    Th = ds.fingerprints(1_000_000, D, 50, seed=3)
    Tt = torch.tensor(Th, dtype=torch.float32, device="cuda")
    Yt = torch.tensor(Yn, dtype=torch.float32, device="cuda")
    P = ag.project(Tt, Yt, b, steps=3)
    assert torch.isfinite(P).all()
    idx = torch.tensor(rng.integers(0, 1_000_000, 4096), device="cuda")

    def nearest(Z):
        return torch.cdist(Z[idx].double(), Yt.double()).min(dim=1).values.mean().item()

    assert nearest(P) < nearest(Tt)
