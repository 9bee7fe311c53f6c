"""torch.autograd binding of the annealed free energy (FP32 data, FP64 reductions).

``free_energy(Y, T, beta, temp)`` returns F = N (D/2 ln(beta/2pi) - ln K) +
temp sum_n ln sum_k exp(-beta d_kn / (2 temp)) as a 0-dim float64 tensor on
the data's device; ``F.backward()`` fills the gradients of Y (K x D), T
(N x D) and beta through the hand-written kernels of ``dgtm_fe_backward``
(responsibilities recomputed tile by tile from two numbers per point kept by
the forward).  Y and T must be contiguous float32 CUDA tensors; beta may be a
float or a 0-dim tensor (which then receives a gradient).

``project(T_new, Y, beta, ...)`` moves held-out points by gradient descent on
F with the map (Y, beta) fixed: each point drifts towards its
responsibility-weighted centre sum_k R_kn y_k.
"""
from __future__ import annotations

import ctypes
import importlib

import torch

_pkg = importlib.import_module(__name__.rsplit(".", 1)[0])


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class FreeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, Y, T, beta, temp):
        if Y.dtype != torch.float32 or T.dtype != torch.float32 or not Y.is_cuda or not T.is_cuda:
            raise TypeError("Y and T must be float32 CUDA tensors")
        Y = Y.contiguous()
        T = T.contiguous()
        K, D = Y.shape
        N, D2 = T.shape
        if D != D2:
            raise ValueError("Y and T must have the same number of columns")
        b = float(beta)
        lib = _pkg.load_library()
        nbytes = ctypes.c_size_t()
        _pkg._check(lib.dgtm_fe_workspace_size(N, K, D, ctypes.byref(nbytes)))
        ws = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=Y.device)
        off = (-ws.data_ptr()) % 256
        ws_ptr = ws.data_ptr() + off
        F = torch.empty((), dtype=torch.float64, device=Y.device)
        _pkg._check(lib.dgtm_fe_forward(Y.data_ptr(), T.data_ptr(), N, K, D, b, float(temp),
                                        ws_ptr, nbytes.value, _stream(Y.device), F.data_ptr()))
        ctx.save_for_backward(Y, T, ws)
        ctx.meta = (N, K, D, b, float(temp), ws_ptr, nbytes.value)
        ctx.beta_is_tensor = torch.is_tensor(beta)
        return F

    @staticmethod
    def backward(ctx, gF):
        Y, T, ws = ctx.saved_tensors
        N, K, D, b, temp, ws_ptr, nbytes = ctx.meta
        lib = _pkg.load_library()
        g = gF.detach().to(dtype=torch.float64).contiguous()
        dY = torch.empty_like(Y) if ctx.needs_input_grad[0] else None
        dT = torch.empty_like(T) if ctx.needs_input_grad[1] else None
        want_beta = ctx.needs_input_grad[2] and ctx.beta_is_tensor
        db = torch.empty((), dtype=torch.float64, device=Y.device) if want_beta else None
        _pkg._check(lib.dgtm_fe_backward(Y.data_ptr(), T.data_ptr(), N, K, D, b, temp, ws_ptr,
                                         nbytes, _stream(Y.device), g.data_ptr(),
                                         dY.data_ptr() if dY is not None else None,
                                         dT.data_ptr() if dT is not None else None,
                                         db.data_ptr() if db is not None else None))
        return dY, dT, db, None


def free_energy(Y, T, beta, temp=1.0):
    return FreeEnergy.apply(Y, T, beta, temp)


def project(T_new, Y, beta, temp=1.0, steps=50, lr=None):
    """Gradient projection of held-out points onto a fixed map.

    Each step moves the points along -dF/dT, i.e. towards sum_k R_kn y_k, with
    step size ``lr`` (default 1/beta, which makes one step the exact
    fixed-point update t <- sum_k R_kn y_k at temp = 1).
    """
    T = T_new.detach().clone().contiguous().requires_grad_(True)
    Yd = Y.detach().contiguous()
    step = (1.0 / float(beta)) if lr is None else lr
    for _ in range(steps):
        F = free_energy(Yd, T, float(beta), temp)
        (g,) = torch.autograd.grad(F, T)
        with torch.no_grad():
            T += step * g  # F increases towards the centres: ascend
    return T.detach()
