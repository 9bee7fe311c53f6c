"""GB300-native DA-GTM annealed EM step (sm_103a).

Python side of the C ABI declared in ``include/dagtm_gb300.h``: the context
that owns the device buffers of one GTM problem, the E-step and M-step that
replace ``dagtm_mpi_resp``/``dagtm_mpi_qual``/``dagtm_mpi_beta`` and the inline
M-step of ``dagtm/dagtm.cxx``, and the temperature loop of
``dagtm/dagtm.cxx:1508-2206`` (EXP, LINEAR and AUTO schedules, and the
hierarchical expansion) driving them.

The package directory is named ``da-gtm_gb300``; import it with
``importlib.import_module("da-gtm_gb300")``.  There is no CPU fallback: the
compiled library must be present (``build.build()``), and every call that
fails raises :class:`DgtmError`.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdagtm_gb300.so")

FP64, FP32, BF16X3 = 0, 1, 2
SOLVE_CHOLESKY, SOLVE_SVD = 0, 1
PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16x3": BF16X3}
SOLVERS = {"cholesky": SOLVE_CHOLESKY, "svd": SOLVE_SVD}

ERRORS = {1: "EINVAL", 2: "ECUDA", 3: "ENOTSPD", 4: "ENONFINITE", 5: "ETIMEOUT", 6: "ENOMEM",
          7: "ESTATE", 8: "ENOTSUP"}

# every symbol the header declares (checked by the CPU tests)
ABI_SYMBOLS = ("dgtm_version", "dgtm_last_error_string", "dgtm_ctx_create", "dgtm_ctx_destroy",
               "dgtm_set_solver", "dgtm_set_Y", "dgtm_get_Y", "dgtm_get_W", "dgtm_estep",
               "dgtm_mstep", "dgtm_get_stats", "dgtm_map", "dgtm_get_R_block", "dgtm_map_rd",
               "dgtm_get_RD_block", "dgtm_next_ctemp",
               "dgtm_next_ctemp_k", "dgtm_set_timing",
               "dgtm_reset_timing", "dgtm_get_timing", "dgtm_get_stream", "dgtm_get_path",
               "dgtm_selftest",
               "dgtm_fe_workspace_size", "dgtm_fe_forward", "dgtm_fe_backward",
               "dgtm_fe_forward_noalloc", "dgtm_wait_probe")
PHASES = ("estep", "estep_reduce", "mstep_pass", "mstep_solve")
PATHS = ("cuda_cores", "split_bf16", "exact_slices")


class DgtmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


def load_library(path: str = LIB_PATH):
    """Load the compiled C ABI.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with da-gtm_gb300/build.py "
                          "(there is no CPU fallback)")
    L = ctypes.CDLL(path)
    i, d, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    pp = ctypes.POINTER(vp)
    sig = {
        "dgtm_version": (i, []),
        "dgtm_last_error_string": (ctypes.c_char_p, []),
        "dgtm_ctx_create": (i, [i, i, i, i, _dp, i, _dp, i, i, pp]),
        "dgtm_ctx_destroy": (i, [vp]),
        "dgtm_set_solver": (i, [vp, i]),
        "dgtm_set_Y": (i, [vp, _dp, i]),
        "dgtm_get_Y": (i, [vp, _dp, i]),
        "dgtm_get_W": (i, [vp, _dp, i]),
        "dgtm_estep": (i, [vp, d, i, d, _dp, _dp]),
        "dgtm_mstep": (i, [vp, _dp, i, _dp, i, _dp]),
        "dgtm_get_stats": (i, [vp, _dp, _dp, i]),
        "dgtm_map": (i, [vp, _dp, i, _dp, i]),
        "dgtm_get_R_block": (i, [vp, i, i, i, i, _dp, i]),
        "dgtm_map_rd": (i, [vp, _dp, i, _dp, i]),
        "dgtm_get_RD_block": (i, [vp, i, i, i, i, _dp, i]),
        "dgtm_next_ctemp": (i, [vp, d, d, d, _dp, _dp]),
        "dgtm_next_ctemp_k": (i, [vp, d, d, d, _dp, _dp, _dp]),
        "dgtm_set_timing": (i, [vp, i]),
        "dgtm_reset_timing": (i, [vp]),
        "dgtm_get_timing": (i, [vp, _dp, ctypes.POINTER(ctypes.c_longlong),
                                ctypes.POINTER(ctypes.c_longlong)]),
        "dgtm_get_stream": (i, [vp, pp]),
        "dgtm_get_path": (i, [vp, ctypes.POINTER(i)]),
        "dgtm_selftest": (i, [_dp, i]),
        "dgtm_fe_workspace_size": (i, [i, i, i, ctypes.POINTER(ctypes.c_size_t)]),
        "dgtm_fe_forward": (i, [vp, vp, i, i, i, d, d, vp, ctypes.c_size_t, vp, vp]),
        "dgtm_fe_backward": (i, [vp, vp, i, i, i, d, d, vp, ctypes.c_size_t, vp, vp, vp, vp,
                                 vp]),
        "dgtm_fe_forward_noalloc": (i, [vp, vp, i, i, i, d, d, vp, vp]),
        "dgtm_wait_probe": (i, [ctypes.c_uint, ctypes.POINTER(i), _dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(code: int):
    if code != 0:
        msg = load_library().dgtm_last_error_string().decode(errors="replace")
        raise DgtmError(code, msg)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def selftest():
    """Largest errors of the three tensor-core operand configurations (0 = exact),
    then the number of packed double-float lanes that differ from the scalar ones."""
    errs = (ctypes.c_double * 4)()
    _check(load_library().dgtm_selftest(errs, 4))
    return list(errs)


def wait_probe(limit_ms: int = 50):
    """One bounded wait that runs out (see dgtm_wait_probe): returns the status
    code, the site the kernel recorded and the milliseconds it waited."""
    site = ctypes.c_int()
    ms = ctypes.c_double()
    code = load_library().dgtm_wait_probe(int(limit_ms), ctypes.byref(site), ctypes.byref(ms))
    return code, site.value, ms.value


class Context:
    """One GTM problem resident on the current CUDA device.

    ``T`` (N x D) and ``FI`` (K x M1) are uploaded once; ``precision`` is
    ``"fp64"``, ``"fp32"`` or ``"bf16x3"``.
    """

    def __init__(self, T, FI, precision: str = "fp64", solver: str = "cholesky"):
        lib = load_library()
        T = _f64(T)
        FI = _f64(FI)
        if T.ndim != 2 or FI.ndim != 2:
            raise ValueError("T and FI must be 2-D")
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, not {precision!r}")
        if solver not in SOLVERS:
            raise ValueError(f"solver must be one of {sorted(SOLVERS)}, not {solver!r}")
        self.N, self.D = T.shape
        self.K, self.M1 = FI.shape
        self.precision = precision
        self.solver = solver
        self._create(T, FI)

    def _create(self, T, FI):
        h = ctypes.c_void_p()
        _check(load_library().dgtm_ctx_create(self.N, self.D, self.K, self.M1, _p(T), self.D,
                                              _p(FI), self.M1, PRECISIONS[self.precision],
                                              ctypes.byref(h)))
        self._h = h
        if self.solver != "cholesky":
            self.set_solver(self.solver)

    def set_basis(self, T, FI, Y):
        """A new latent basis FI (K' x M1, same M1) on the same data T, with
        centres Y (K' x D): the context is rebuilt in place for K'.  This is
        the hierarchical schedule's grid expansion (dagtm/dagtm.cxx:2110-2144:
        new X and FI, K-sized buffers reallocated, Y = FI W)."""
        T = _f64(T)
        FI = _f64(FI)
        if T.shape != (self.N, self.D) or FI.ndim != 2 or FI.shape[1] != self.M1:
            raise ValueError("set_basis: T must be the context's data and FI K' x M1")
        self.close()
        self.K = FI.shape[0]
        self._create(T, FI)
        self.set_Y(Y)

    # life cycle
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load_library().dgtm_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # calls
    def set_solver(self, solver: str):
        """"cholesky" or "svd"; kept across set_basis."""
        if solver not in SOLVERS:
            raise ValueError(f"solver must be one of {sorted(SOLVERS)}, not {solver!r}")
        _check(load_library().dgtm_set_solver(self._h, SOLVERS[solver]))
        self.solver = solver

    def set_Y(self, Y):
        Y = _f64(Y)
        if Y.shape != (self.K, self.D):
            raise ValueError(f"Y must be {self.K} x {self.D}")
        _check(load_library().dgtm_set_Y(self._h, _p(Y), self.D))

    def get_Y(self) -> np.ndarray:
        Y = np.empty((self.K, self.D))
        _check(load_library().dgtm_get_Y(self._h, _p(Y), self.D))
        return Y

    def get_W(self) -> np.ndarray:
        W = np.empty((self.M1, self.D))
        _check(load_library().dgtm_get_W(self._h, _p(W), self.D))
        return W

    def estep(self, beta: float, isDA: int, temp: float):
        """Returns (llh, nfree) as dagtm_mpi_qual computes them."""
        llh = ctypes.c_double()
        nfree = ctypes.c_double()
        _check(load_library().dgtm_estep(self._h, float(beta), int(isDA), float(temp),
                                         ctypes.byref(llh), ctypes.byref(nfree)))
        return llh.value, nfree.value

    def mstep(self, want_W: bool = True, want_Y: bool = False):
        """Returns (beta, W or None, Y or None)."""
        b = ctypes.c_double()
        W = np.empty((self.M1, self.D)) if want_W else None
        Y = np.empty((self.K, self.D)) if want_Y else None
        _check(load_library().dgtm_mstep(self._h, _p(W) if W is not None else None, self.D,
                                         _p(Y) if Y is not None else None, self.D,
                                         ctypes.byref(b)))
        return b.value, W, Y

    def get_stats(self):
        G = np.empty(self.K)
        RT = np.empty((self.K, self.D))
        _check(load_library().dgtm_get_stats(self._h, _p(G), _p(RT), self.D))
        return G, RT

    def map(self, X) -> np.ndarray:
        X = _f64(X)
        L = X.shape[1]
        M = np.empty((self.N, L))
        _check(load_library().dgtm_map(self._h, _p(X), L, _p(M), L))
        return M

    def set_timing(self, on: bool = True):
        _check(load_library().dgtm_set_timing(self._h, int(bool(on))))

    def reset_timing(self):
        _check(load_library().dgtm_reset_timing(self._h))

    def timing(self) -> dict:
        """Per-phase device ms, kernel launches and calls since the last reset."""
        ms = (ctypes.c_double * 4)()
        nl = (ctypes.c_longlong * 4)()
        nc = (ctypes.c_longlong * 4)()
        _check(load_library().dgtm_get_timing(self._h, ms, nl, nc))
        return {p: {"ms": ms[i], "launches": nl[i], "calls": nc[i]} for i, p in enumerate(PHASES)}

    @property
    def path(self) -> str:
        """The implementation of the E-step and responsibility pass:
        "cuda_cores", "split_bf16" or "exact_slices" (dgtm_get_path)."""
        out = ctypes.c_int()
        _check(load_library().dgtm_get_path(self._h, ctypes.byref(out)))
        return PATHS[out.value]

    def stream(self) -> int:
        """cudaStream_t of the context, as an integer handle."""
        out = ctypes.c_void_p()
        _check(load_library().dgtm_get_stream(self._h, ctypes.byref(out)))
        return out.value or 0

    def R_block(self, k0: int, nk: int, n0: int, nn: int) -> np.ndarray:
        R = np.empty((nk, nn))
        _check(load_library().dgtm_get_R_block(self._h, k0, nk, n0, nn, _p(R), nn))
        return R

    def map_rd(self, X) -> np.ndarray:
        """(R o D)^T X after an M-step: the reference's MAP when it stops on
        its iteration cap (R of the last E-step times the squared distances
        to the new centres)."""
        X = _f64(X)
        L = X.shape[1]
        M = np.empty((self.N, L))
        _check(load_library().dgtm_map_rd(self._h, _p(X), L, _p(M), L))
        return M

    def RD_block(self, k0: int, nk: int, n0: int, nn: int) -> np.ndarray:
        R = np.empty((nk, nn))
        _check(load_library().dgtm_get_RD_block(self._h, k0, nk, n0, nn, _p(R), nn))
        return R

    def next_ctemp(self, temp: float, beta: float, eps: float, gg=None,
                   per_centre: bool = False):
        """Next critical temperature (AUTO cooling) from the last E-step's R;
        gg: per-centre weights (the G of the last M-step), None: row sums of R.
        per_centre: also return every centre's ctemp_k (the reference's vctemp)."""
        out = ctypes.c_double()
        g = None if gg is None else _f64(np.asarray(gg).reshape(self.K))
        ck = np.empty(self.K) if per_centre else None
        _check(load_library().dgtm_next_ctemp_k(self._h, float(temp), float(beta), float(eps),
                                                _p(g) if g is not None else None,
                                                _p(ck) if ck is not None else None,
                                                ctypes.byref(out)))
        return (out.value, ck) if per_centre else out.value


QUEUE_SIZE = 50  # dagtm/dagtm.cxx:45 INIT_QUEUE_SIZE


def _gtm_setup():
    import importlib
    return importlib.import_module(__name__ + ".gtm_setup")


@dataclass
class RunResult:
    temp_trace: list = field(default_factory=list)
    nfree_trace: list = field(default_factory=list)
    llh_trace: list = field(default_factory=list)
    beta_trace: list = field(default_factory=list)
    beta: float = 0.0
    temp: float = 1.0
    nloop: int = 0
    W: np.ndarray | None = None
    expansions: list = field(default_factory=list)  # HDA: (iteration, K before, K after)


def anneal(ctx: Context, beta: float, temp: float, isDA: int = 1, schedule: str = "exp",
           alpha: float = 0.99, delta: float = 0.1, eps: float = 1e-6, iter0: int = 0,
           maxloop: int = 0, log=None, hda: bool = False, T=None, L: int = 0,
           Kmax: int = 32768, eps2: float = 1e-3, on_expand=None) -> RunResult:
    """Temperature loop of dagtm/dagtm.cxx:1508-2206 (EXP / LINEAR / AUTO, HDA).

    AUTO (dagtm/dagtm.cxx:1919-1934): the next temperature is the critical
    temperature from ``Context.next_ctemp`` with the G of the last M-step as
    weights (the reference's vggsub), or temp * alpha when that is not below
    the current temperature.

    HDA (``hda=True``, the -H option; EXP schedule; dagtm/dagtm.cxx:1912-2124):
    at the end of a temperature with K < Kmax, a grid that is ready to expand
    either expands, if the log-likelihood rose by at least eps2 over the
    temperature, or stops being ready.  A grid that is not ready asks for the
    next critical temperature and becomes ready when it is at least
    temp * alpha.  Expanding doubles the latent grid per dimension,
    K = (round(K^(1/L)) 2)^L, rebuilds X and FI with width factor 2 and the
    same M, and sets Y = FI W (``Context.set_basis``; ``T`` must be the
    context's data, ``L`` the latent dimension).  ``on_expand(ctx, info)``
    runs before the expansion, with ``info`` holding the trace index, K, the
    new K, W, beta and the per-centre critical temperatures of the last
    ``next_ctemp`` call (the reference writes these, with the MAP, when it
    logs progress).

    Starts from the centres already loaded into ``ctx`` (a fresh set-up or a
    restart, dagtm/dagtm.cxx:1161-1232) and mirrors the reference's order:
    E-step, qualities, |diff| < eps test (before the M-step), the 50-wide
    moving-average test once nloop > 50, M-step, beta, maxloop test.
    """
    if hda and (schedule != "exp" or T is None or L < 1):
        raise ValueError("HDA needs the EXP schedule, the data T and the latent dimension L")
    res = RunResult()
    nloop = iter0
    if maxloop:
        maxloop = iter0 + maxloop
    qual = 0.0
    llh = 0.0
    isLast = False
    W = None
    G_last = None
    ready = False  # HDA: bReadyToExpand
    ctemp_k = None
    while True:
        if temp < 1.0:
            temp = 1.0
            isLast = True
        qual_before_temp = llh
        queue = [np.finfo(np.float64).max] * QUEUE_SIZE
        qnext = 0
        if log:
            log(f"\nT= {temp:.10g}\n")
        lloop = 0
        while True:
            llh, nfree = ctx.estep(beta, isDA, temp)
            qual_old = qual
            lloop += 1
            nloop += 1
            qual = nfree if isDA else llh
            diff = qual - qual_old
            res.temp_trace.append(temp)
            res.nfree_trace.append(nfree)
            res.llh_trace.append(llh)
            res.beta_trace.append(beta)
            if log:
                log("::: %15d %15d %15d %15.7f %15.7f %15.7f %15.7f\n"
                    % (nloop, lloop, ctx.K, temp, nfree, llh, diff))
            if abs(diff) < eps:
                break
            if nloop > QUEUE_SIZE:
                # a queue still holding DBL_MAX sums to inf and the test fails,
                # as in the reference (comm/comm.c:1742-1746)
                with np.errstate(over="ignore", invalid="ignore"):
                    avg_old = sum(queue) / QUEUE_SIZE
                    queue[qnext] = qual
                    qnext = (qnext + 1) % QUEUE_SIZE
                    avg = sum(queue) / QUEUE_SIZE
                    stalled = abs(avg - avg_old) < eps
                if stalled:
                    break
            beta, W, _ = ctx.mstep(want_W=True)
            if schedule == "auto" or hda:
                G_last = ctx.get_stats()[0]
            if maxloop and nloop >= maxloop:
                isLast = True
                break
        if isDA and not isLast:
            if schedule == "linear":
                temp -= delta
            elif schedule == "auto":
                ctemp = ctx.next_ctemp(temp, beta, eps, gg=G_last)
                if ctemp >= temp:
                    ctemp = temp * alpha  # no valid next critical temperature
                temp = ctemp
            else:
                if hda and ctx.K < Kmax:
                    qual_diff = llh - qual_before_temp
                    expand = False
                    if ready:
                        if qual_diff < eps2:
                            ready = False  # nothing happened at this temperature
                        else:
                            expand = True
                    if not ready:
                        cmax, ctemp_k = ctx.next_ctemp(temp, beta, eps, gg=G_last,
                                                       per_centre=True)
                        if cmax >= temp * alpha:
                            ready = True
                    if expand:
                        ready = False
                        if W is None:  # no M-step in this call: the context's last W
                            W = ctx.get_W()
                        Knew = int(round(ctx.K ** (1.0 / L)) * 2) ** L
                        if on_expand is not None:
                            on_expand(ctx, dict(index=len(res.temp_trace) - 1, K=ctx.K,
                                                K_new=Knew, W=W, beta=beta, ctemp=ctemp_k))
                        if log:
                            log(f"new K : {Knew}\n")
                        _, FI = _gtm_setup().setup_grid(L, Knew, ctx.M1 - 1, 2.0)
                        res.expansions.append((nloop, ctx.K, Knew))
                        ctx.set_basis(T, FI, FI @ W)
                        G_last = None
                temp *= alpha
        else:
            break
    res.beta = beta
    res.temp = temp
    res.nloop = nloop
    res.W = W
    return res
