"""A context stand-in served by the oracle's FP64 primitives (test scaffolding).

``anneal`` reaches its context only through estep / mstep / get_stats /
next_ctemp / get_W / set_basis; this class serves them with the oracle's
dense K x N routines in the order of the reference's loop, so host control
flow can be checked on a machine without a GPU.
"""
import numpy as np


class OracleCtx:
    """A context stand-in over the oracle's primitives (test scaffolding)."""

    def __init__(self, orc, T, FI, Y):
        self.orc = orc
        self.T = np.ascontiguousarray(T, float)
        self.FI = np.ascontiguousarray(FI, float)
        self.Y = np.ascontiguousarray(Y, float).copy()
        self.N, self.D = self.T.shape
        self.K, self.M1 = self.FI.shape
        self.Dm = orc.dist(self.Y, self.T)
        self.R = self.G = self.W = None
        self.calls = []

    def estep(self, beta, isDA, temp):
        self.calls.append("estep")
        self.R, vgc, vgc2 = self.orc.resp(self.Dm, beta, isDA, temp)
        llh = self.orc.qual(self.N, self.K, self.D, beta, vgc, 0, temp)
        nfree = self.orc.qual(self.N, self.K, self.D, beta, vgc2, 1, temp) if isDA else -llh
        return llh, nfree

    def mstep(self, want_W=True, want_Y=False):
        self.calls.append("mstep")
        self.G, A, B = self.orc.mstep_stats(self.R, self.FI, self.T)
        self.W = self.orc.solve_chol(A, B)
        self.Y = self.orc.fiw(self.FI, self.W)
        beta, _, self.Dm = self.orc.beta_update(self.Y, self.T, self.R)
        return beta, (self.W.copy() if want_W else None), (self.Y.copy() if want_Y else None)

    def get_stats(self):
        return self.G.copy(), None

    def get_W(self):
        return self.W.copy()

    def next_ctemp(self, temp, beta, eps, gg=None, per_centre=False):
        w = self.R.sum(axis=1) if gg is None else np.asarray(gg)
        c = self.orc.next_ctemp(self.T, self.Y, self.R, w, temp, beta, eps)
        self.calls.append(("ctemp", temp, c, None if gg is None else w.copy()))
        if not per_centre:
            return c
        ck = np.array([self.orc.next_ctemp(self.T, self.Y[k:k + 1], self.R[k:k + 1], w[k:k + 1],
                                           temp, beta, eps) for k in range(self.K)])
        return c, ck

    def set_basis(self, T, FI, Y):
        self.calls.append(("basis", FI.shape[0]))
        self.FI = np.ascontiguousarray(FI, float)
        self.K = self.FI.shape[0]
        self.Y = np.ascontiguousarray(Y, float).copy()
        self.Dm = self.orc.dist(self.Y, self.T)
        self.G = None
