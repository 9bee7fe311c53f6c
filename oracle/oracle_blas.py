"""The reference's EM iteration restated over numpy's BLAS (FP64), threaded.

TEST INFRASTRUCTURE ONLY: the "optimised BLAS" CPU baseline of ``bench.py``
(the reference built against a tuned BLAS instead of GSL's reference cblas,
the MKL/ACML option of ``CMakeLists.comm.txt:129-174``, with its element
loops spread over all host cores the way the reference spreads them over MPI
ranks), and checked against the C oracle by the CPU tests.  The product path
never imports it.

One call of :meth:`Workspace.iteration` follows ``dagtm/dagtm.cxx:1541-1779``
with dense matrices, in the reference's order:

* ``dagtm_mpi_resp`` (``comm/mpicomm.c:316-414``): R = exp(-beta/2 D),
  column sums vgc, R = R^(1/temp), column sums vgc2, the zero-column
  fallback, R /= vgc2;
* two ``dagtm_mpi_qual`` calls (``comm/mpicomm.c:463-500``);
* the inline M-step (``dagtm/dagtm.cxx:1715-1770``): G = rowsum R,
  A = FI^T diag(G) FI, B = (FI^T R) T, W from the SVD of A with exactly-zero
  singular values dropped (``dagtm_solve2``, ``comm/comm.c:1299-1348``),
  Y = FI W;
* ``dagtm_mpi_beta`` (``comm/mpicomm.c:276-302``): D from the new Y
  (``dagtm_dist_ws``, ``comm/comm.c:560-629``: -2 Y T^T, + |y|^2, + |t|^2),
  R o= D, beta = N D / sum R o D.

The K x N matrices of the reference are held transposed (N x K, one row per
data point) so that the per-point column operations are contiguous row
blocks, one block per thread; the arithmetic is the same.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np


def dist_t(Y: np.ndarray, T: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
    """D^T (N x K): -2 t_n . y_k, then + |y_k|^2, then + |t_n|^2."""
    Dt = np.matmul(T, Y.T, out=out)
    Dt *= -2.0
    Dt += (Y * Y).sum(axis=1)[None, :]
    Dt += (T * T).sum(axis=1)[:, None]
    return Dt


def resp_rows(Dt: np.ndarray, beta: float, isDA: int, temp: float, Rt: np.ndarray):
    """dagtm_mpi_resp on a block of points (rows of D^T); returns vgc, vgc2."""
    K = Dt.shape[1]
    np.multiply(Dt, -beta / 2.0, out=Rt)
    np.exp(Rt, out=Rt)
    vgc = Rt.sum(axis=1)
    vgc2 = vgc
    if isDA:
        np.power(Rt, 1.0 / temp, out=Rt)
        vgc2 = Rt.sum(axis=1)
    zero = vgc2 == 0.0
    if zero.any():
        Rt[zero, :] = 1.0
        vgc2 = vgc2.copy()
        vgc2[zero] = float(K)
        if not isDA:
            vgc = vgc2
    Rt /= vgc2[:, None]
    return vgc, vgc2


def qual(N: int, K: int, D: int, beta: float, v: np.ndarray, isDA: int, temp: float) -> float:
    with np.errstate(divide="ignore"):
        s = float(np.log(v).sum())
    c = temp if isDA else 1.0
    return (N * (D / 2.0 * np.log(beta / (2.0 * np.pi)) - np.log(K)) + c * s) / N


def solve_svd(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """x = V S^+ U^T b with exactly-zero singular values dropped."""
    U, S, Vt = np.linalg.svd(A)
    inv = np.where(S != 0.0, 1.0 / np.where(S != 0.0, S, 1.0), 0.0)
    return Vt.T @ (inv[:, None] * (U.T @ B))


class Workspace:
    """Dense buffers of one problem; ``iteration`` runs one EM step in place."""

    def __init__(self, T, FI, Y, beta, threads: int | None = None):
        self.T = np.ascontiguousarray(T, dtype=np.float64)
        self.FI = np.ascontiguousarray(FI, dtype=np.float64)
        self.Y = np.array(Y, dtype=np.float64)
        self.N, self.D = self.T.shape
        self.K = self.FI.shape[0]
        self.beta = float(beta)
        self.threads = max(1, threads or os.cpu_count() or 1)
        self.pool = ThreadPoolExecutor(self.threads)
        step = -(-self.N // self.threads)
        self.blocks = [(s, min(self.N, s + step)) for s in range(0, self.N, step)]
        self.Dt = dist_t(self.Y, self.T)
        self.Rt = np.empty_like(self.Dt)

    def close(self):
        self.pool.shutdown()

    def _map(self, fn):
        return list(self.pool.map(lambda b: fn(*b), self.blocks))

    def iteration(self, isDA: int = 1, temp: float = 1.0):
        N, D, K = self.N, self.D, self.K
        out = self._map(lambda a, b: resp_rows(self.Dt[a:b], self.beta, isDA, temp, self.Rt[a:b]))
        vgc = np.concatenate([o[0] for o in out])
        vgc2 = np.concatenate([o[1] for o in out])
        llh = qual(N, K, D, self.beta, vgc, 0, temp)
        nfree = qual(N, K, D, self.beta, vgc2, 1, temp) if isDA else -llh
        G = np.sum(self._map(lambda a, b: self.Rt[a:b].sum(axis=0)), axis=0)
        A = self.FI.T @ (G[:, None] * self.FI)
        FIR = self.FI.T @ self.Rt.T          # (FI^T R), M1 x N
        B = FIR @ self.T
        W = solve_svd(A, B)
        self.Y = self.FI @ W
        dist_t(self.Y, self.T, out=self.Dt)
        s = sum(self._map(lambda a, b: float(np.einsum("ij,ij->", self.Rt[a:b], self.Dt[a:b]))))
        self.beta = N * D / s
        return llh, nfree, self.beta


def estep_stats(T, Y, beta: float, isDA: int, temp: float, chunk: int = 8192,
                threads: int | None = None):
    """The E-step quantities of one iteration over any number of points, in
    chunks of points (each chunk's K x chunk matrices in the reference's
    semantics; the columns are independent, so chunking changes only the
    order of the sums over points).  Returns llh, nfree (as dagtm_mpi_qual
    computes them), G = rowsum R and RT = R T (K x D), all FP64."""
    T = np.ascontiguousarray(T, dtype=np.float64)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    N, D = T.shape
    K = Y.shape[0]
    threads = max(1, threads or os.cpu_count() or 1)
    pool = ThreadPoolExecutor(threads)
    log1 = 0.0
    log2 = 0.0
    G = np.zeros(K)
    RT = np.zeros((K, D))
    Dt = np.empty((chunk, K))
    Rt = np.empty((chunk, K))
    try:
        for s in range(0, N, chunk):
            e = min(N, s + chunk)
            n = e - s
            dist_t(Y, T[s:e], out=Dt[:n])
            step = -(-n // threads)
            blocks = [(a, min(n, a + step)) for a in range(0, n, step)]
            out = list(pool.map(lambda b: resp_rows(Dt[b[0]:b[1]], beta, isDA, temp,
                                                    Rt[b[0]:b[1]]), blocks))
            vgc = np.concatenate([o[0] for o in out])
            vgc2 = np.concatenate([o[1] for o in out])
            with np.errstate(divide="ignore"):
                log1 += float(np.log(vgc).sum())
                log2 += float(np.log(vgc2).sum())
            G += Rt[:n].sum(axis=0)
            RT += Rt[:n].T @ T[s:e]
    finally:
        pool.shutdown()
    base = N * (D / 2.0 * np.log(beta / (2.0 * np.pi)) - np.log(K))
    llh = (base + log1) / N
    nfree = (base + temp * log2) / N if isDA else -llh
    return llh, nfree, G, RT


def resp_columns(T, Y, beta: float, isDA: int, temp: float) -> np.ndarray:
    """R (K x n) for the given points only: each column of the reference's R
    depends on its own point alone."""
    Dt = dist_t(np.ascontiguousarray(Y, dtype=np.float64), np.ascontiguousarray(T, dtype=np.float64))
    Rt = np.empty_like(Dt)
    resp_rows(Dt, beta, isDA, temp, Rt)
    return Rt.T.copy()
