"""ctypes bindings of the CPU FP64 oracle (``dagtm_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product path never imports it.

The oracle restates the reference's annealed EM step with its own semantics
(dense K x N matrices, unshifted exp, zero-column fallback); see
``dagtm_oracle.h`` for the reference file:line each function follows.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdagtm_oracle.so")
SRC_PATH = os.path.join(_HERE, "dagtm_oracle.c")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle into ``oracle/libdagtm_oracle.so`` (gcc + OpenMP)."""
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC_PATH)):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH + ".tmp", SRC_PATH, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i, d, u = ctypes.c_int, ctypes.c_double, ctypes.c_ulong
        sig = {
            "orc_set_threads": (None, [i]),
            "orc_get_threads": (i, []),
            "orc_dist": (None, [i, i, i, _dp, _dp, _dp]),
            "orc_resp": (None, [i, i, d, _dp, i, d, _dp, _dp, _dp]),
            "orc_qual": (d, [i, i, i, d, _dp, i, d]),
            "orc_mstep_stats": (None, [i, i, i, i, _dp, _dp, _dp, _dp, _dp, _dp]),
            "orc_solve2": (i, [i, i, _dp, _dp, _dp]),
            "orc_solve_chol": (i, [i, i, _dp, _dp, _dp]),
            "orc_fiw": (None, [i, i, i, _dp, _dp, _dp]),
            "orc_beta": (d, [i, i, i, _dp, _dp, _dp, _dp]),
            "orc_rctg": (None, [i, i, _dp]),
            "orc_gbf": (None, [i, i, i, _dp, _dp, d, _dp]),
            "orc_stp": (i, [i, i, i, d, _dp, _dp]),
            "orc_yrnd2": (None, [u, i, i, _dp, _dp, _dp]),
            "orc_solve_ls": (i, [i, i, i, _dp, _dp, _dp]),
            "orc_bi": (d, [i, i, _dp]),
            "orc_stp3_rnd": (i, [u, _dp, _dp, i, i, i, i, d, _dp, _dp, _dp, _dp]),
            "orc_mean": (None, [i, i, _dp, _dp]),
            "orc_sd": (None, [i, i, _dp, _dp, _dp]),
            "orc_ctemp": (d, [i, i, _dp]),
            "orc_eig_sym": (i, [i, _dp, _dp]),
            "orc_next_ctemp": (d, [i, i, i, _dp, _dp, _dp, _dp, d, d, d]),
            "orc_mt_uniform": (None, [u, i, _dp]),
            "orc_em_iteration": (i, [i, i, i, i, _dp, _dp, _dp, _dp, _dp, i, d,
                                     _dp, _dp, _dp, _dp, _dp, _dp, i]),
            "orc_run": (i, [i, i, i, i, _dp, _dp, _dp, _dp, _dp, _dp, i, i, d,
                            d, d, i, i, i, i, _dp, _dp, _dp, _dp, _ip, _dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _c(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def dist(Y, T):
    Y, T = _c(Y), _c(T)
    K, D = Y.shape
    N = T.shape[0]
    out = np.empty((K, N))
    lib().orc_dist(K, N, D, _p(Y), _p(T), _p(out))
    return out


def resp(Dm, beta, isDA, temp):
    """Returns (R, vgc, vgc2) exactly as dagtm_mpi_resp leaves them."""
    Dm = _c(Dm)
    K, N = Dm.shape
    R = np.empty((K, N))
    vgc = np.empty(N)
    vgc2 = np.zeros(N)
    lib().orc_resp(K, N, float(beta), _p(Dm), int(isDA), float(temp), _p(R), _p(vgc), _p(vgc2))
    return R, vgc, vgc2


def qual(N, K, D, beta, v, isDA, temp):
    v = _c(v).copy()
    return float(lib().orc_qual(int(N), int(K), int(D), float(beta), _p(v), int(isDA), float(temp)))


def mstep_stats(R, FI, T):
    R, FI, T = _c(R), _c(FI), _c(T)
    K, N = R.shape
    M1 = FI.shape[1]
    D = T.shape[1]
    G = np.empty(K)
    A = np.empty((M1, M1))
    B = np.empty((M1, D))
    lib().orc_mstep_stats(K, N, D, M1, _p(R), _p(FI), _p(T), _p(G), _p(A), _p(B))
    return G, A, B


def solve2(A, B):
    A, B = _c(A), _c(B)
    n, k = B.shape
    X = np.empty((n, k))
    lib().orc_solve2(n, k, _p(A), _p(B), _p(X))
    return X


def solve_chol(A, B):
    A, B = _c(A), _c(B)
    n, k = B.shape
    X = np.empty((n, k))
    if lib().orc_solve_chol(n, k, _p(A), _p(B), _p(X)) < 0:
        raise np.linalg.LinAlgError("non-finite pivot")
    return X


def fiw(FI, W):
    FI, W = _c(FI), _c(W)
    K, M1 = FI.shape
    D = W.shape[1]
    Y = np.empty((K, D))
    lib().orc_fiw(K, M1, D, _p(FI), _p(W), _p(Y))
    return Y


def beta_update(Y, T, R):
    """dagtm_mpi_beta: returns (beta, R o D, D)."""
    Y, T = _c(Y), _c(T)
    R = _c(R).copy()
    K, D = Y.shape
    N = T.shape[0]
    Dm = np.empty((K, N))
    b = lib().orc_beta(K, N, D, _p(Y), _p(T), _p(R), _p(Dm))
    return float(b), R, Dm


def stp(L, K, M, s=2.0):
    X = np.empty((K, L))
    FI = np.empty((K, M + 1))
    r = lib().orc_stp(int(L), int(K), int(M), float(s), _p(X), _p(FI))
    if r != 0:
        raise ValueError(f"dagtm_stp rejected L={L} K={K} M={M} s={s} (code {r})")
    return X, FI


def mt_uniform(seed, n):
    out = np.empty(int(n))
    lib().orc_mt_uniform(int(seed), int(n), _p(out))
    return out


def yrnd2(seed, K, mu, sd):
    mu, sd = _c(mu), _c(sd)
    D = mu.shape[0]
    Y = np.empty((K, D))
    lib().orc_yrnd2(int(seed), int(K), D, _p(mu), _p(sd), _p(Y))
    return Y


def solve_ls(A, B):
    A, B = _c(A), _c(B)
    m, n = A.shape
    k = B.shape[1]
    X = np.empty((n, k))
    lib().orc_solve_ls(m, n, k, _p(A), _p(B), _p(X))
    return X


def bi(Y):
    Y = _c(Y)
    return float(lib().orc_bi(Y.shape[0], Y.shape[1], _p(Y)))


def mean_sd(T):
    T = _c(T)
    N, D = T.shape
    mu = np.empty(D)
    sd = np.empty(D)
    lib().orc_mean(N, D, _p(T), _p(mu))
    lib().orc_sd(N, D, _p(T), _p(mu), _p(sd))
    return mu, sd


def stp3_rnd(seed, T, L, K, M, s=2.0):
    """dagtm_stp3_rnd after dagtm_mpi_mean/sd: returns X, FI, W, beta."""
    mu, sd = mean_sd(T)
    D = mu.shape[0]
    X = np.empty((K, L))
    FI = np.empty((K, M + 1))
    W = np.empty((M + 1, D))
    beta = ctypes.c_double(0.0)
    r = lib().orc_stp3_rnd(int(seed), _p(mu), _p(sd), D, int(L), int(K), int(M), float(s),
                           _p(X), _p(FI), _p(W), ctypes.byref(beta))
    if r != 0:
        raise ValueError("dagtm_stp3_rnd failed")
    return X, FI, W, float(beta.value)


def ctemp(T):
    T = _c(T)
    return float(lib().orc_ctemp(T.shape[0], T.shape[1], _p(T)))


def next_ctemp(T, Y, R, gg, temp, beta, eps):
    """AUTO schedule: the next critical temperature (R is K x N, gg the K weights)."""
    T, Y, R, gg = _c(T), _c(Y), _c(R), _c(np.asarray(gg, float))
    N, D = T.shape
    K = Y.shape[0]
    return float(lib().orc_next_ctemp(N, D, K, _p(T), _p(Y), _p(R), _p(gg), temp, beta, eps))


def eig_sym(S):
    S = _c(S)
    lam = np.empty(S.shape[0])
    lib().orc_eig_sym(S.shape[0], _p(S), _p(lam))
    return lam


class Workspace:
    """Dense K x N buffers for timing one reference-semantics EM iteration."""

    def __init__(self, T, FI, Y, beta):
        self.T = _c(T)
        self.FI = _c(FI)
        self.Y = _c(Y).copy()
        self.N, self.D = self.T.shape
        self.K, self.M1 = self.FI.shape
        self.W = np.empty((self.M1, self.D))
        self.Dm = dist(self.Y, self.T)
        self.R = np.empty_like(self.Dm)
        self.vgc = np.empty(self.N)
        self.vgc2 = np.empty(self.N)
        self.beta = ctypes.c_double(float(beta))
        self.llh = ctypes.c_double(0.0)
        self.nfree = ctypes.c_double(0.0)

    def iteration(self, isDA=1, temp=1.0, solver=0):
        lib().orc_em_iteration(self.N, self.D, self.K, self.M1, _p(self.T), _p(self.FI),
                               _p(self.Y), _p(self.W), ctypes.byref(self.beta), int(isDA),
                               float(temp), _p(self.Dm), _p(self.R), _p(self.vgc),
                               _p(self.vgc2), ctypes.byref(self.llh), ctypes.byref(self.nfree),
                               int(solver))
        return self.llh.value, self.nfree.value, self.beta.value


def run(T, FI, Y, beta, temp, isDA=1, schedule=0, alpha=0.99, delta=0.1, eps=1e-6,
        iter0=0, maxloop=0, solver=0, cap=100000, want_R=False):
    """Annealing loop from a restart state; returns a dict with the trace and final state."""
    T, FI = _c(T), _c(FI)
    Y = _c(Y).copy()
    N, D = T.shape
    K, M1 = FI.shape
    W = np.zeros((M1, D))
    b = ctypes.c_double(float(beta))
    t = ctypes.c_double(float(temp))
    cap = int(cap)
    tt, tn, tl, tb = (np.zeros(cap) for _ in range(4))
    nout = ctypes.c_int(0)
    R = np.empty((K, N)) if want_R else None
    ret = lib().orc_run(N, D, K, M1, _p(T), _p(FI), _p(Y), _p(W), ctypes.byref(b), ctypes.byref(t),
                        int(isDA), int(schedule), float(alpha), float(delta), float(eps),
                        int(iter0), int(maxloop), int(solver), cap, _p(tt), _p(tn), _p(tl),
                        _p(tb), ctypes.byref(nout), _p(R) if R is not None else None)
    n = min(nout.value, cap)
    return {"ret": ret, "n": nout.value, "temp_trace": tt[:n], "nfree_trace": tn[:n],
            "llh_trace": tl[:n], "beta_trace": tb[:n], "Y": Y, "W": W, "beta": b.value,
            "temp": t.value, "R": R}


def run_hda(T, FI, Y, beta, temp, L, alpha=0.99, eps=1e-6, eps2=1e-3, Kmax=32768,
            iter0=0, maxloop=0):
    """The annealing loop with the hierarchical schedule (-H, EXP cooling),
    restated over the C primitives above: E-step and qualities
    (dagtm/dagtm.cxx:1541-1605), the two stopping tests (:1690-1709), M-step
    with the Cholesky solve and beta (:1715-1779), and at the end of each
    temperature the expansion logic of :1912-2124 (ready / expand on the
    log-likelihood gain over the temperature against eps2, the next critical
    temperature against temp * alpha, K = (round(K^(1/L)) 2)^L, new FI from
    dagtm_stp with width factor 2, Y = FI W).  The weights of next_ctemp are
    the G of the last M-step at this K (the row sums of R before the first).
    Python control flow: small cases only."""
    T, FI = _c(T), _c(FI)
    Y = _c(Y).copy()
    N, D = T.shape
    K, M1 = FI.shape
    nloop = iter0
    if maxloop:
        maxloop = iter0 + maxloop
    q = 0.0
    llh = 0.0
    isLast = False
    ready = False
    W = None
    G = None
    tr = {"temp": [], "nfree": [], "llh": [], "beta": [], "K": []}
    expansions = []
    Dm = dist(Y, T)
    big = np.finfo(np.float64).max
    while True:
        if temp < 1.0:
            temp = 1.0
            isLast = True
        queue = [big] * 50
        qnext = 0
        qual_before = llh
        while True:
            R, vgc, vgc2 = resp(Dm, beta, 1, temp)
            q_old = q
            nloop += 1
            llh = qual(N, K, D, beta, vgc, 0, temp)
            nfree = qual(N, K, D, beta, vgc2, 1, temp)
            q = nfree
            diff = q - q_old
            for key, v in (("temp", temp), ("nfree", nfree), ("llh", llh), ("beta", beta),
                           ("K", K)):
                tr[key].append(v)
            if abs(diff) < eps:
                break
            if nloop > 50:
                with np.errstate(over="ignore", invalid="ignore"):
                    avg_old = sum(queue) / 50
                    queue[qnext] = q
                    qnext = (qnext + 1) % 50
                    avg = sum(queue) / 50
                    stalled = abs(avg - avg_old) < eps
                if stalled:
                    break
            G, A, B = mstep_stats(R, FI, T)
            W = solve_chol(A, B)
            Y = fiw(FI, W)
            beta, _, Dm = beta_update(Y, T, R)
            if maxloop and nloop >= maxloop:
                isLast = True
                break
        if isLast:
            break
        if K < Kmax:
            qual_diff = llh - qual_before
            expand = False
            if ready:
                if qual_diff < eps2:
                    ready = False
                else:
                    expand = True
            if not ready:
                gg = G if G is not None else R.sum(axis=1)
                if next_ctemp(T, Y, R, gg, temp, beta, eps) >= temp * alpha:
                    ready = True
            if expand:
                ready = False
                Knew = int(round(K ** (1.0 / L)) * 2) ** L
                _, FI = stp(L, Knew, M1 - 1, 2.0)
                expansions.append((nloop, K, Knew))
                K = Knew
                Y = fiw(FI, W)
                Dm = dist(Y, T)
                G = None
        temp *= alpha
    return {"n": len(tr["temp"]), "temp_trace": np.array(tr["temp"]),
            "nfree_trace": np.array(tr["nfree"]), "llh_trace": np.array(tr["llh"]),
            "beta_trace": np.array(tr["beta"]), "K_trace": np.array(tr["K"]),
            "expansions": expansions, "Y": Y, "W": W, "FI": FI, "beta": beta, "temp": temp}
