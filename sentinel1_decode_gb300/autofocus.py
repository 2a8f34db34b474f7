"""Entropy-minimising azimuth autofocus over the hand-written adjoint of the
azimuth chain (s1g_azimuth_adjoint): a thin torch.autograd.Function whose
forward runs the chain and whose backward returns the gradients the same
library call produced.  Gradient checks and autofocus only; the product path
does not use it.
"""
from __future__ import annotations

import numpy as np
import torch


class AzimuthEntropy(torch.autograd.Function):
    """loss = AzimuthEntropy.apply(theta, centroid, decoder, swath, burst, chain):
    image entropy of `burst` focused with the phase-error polynomial theta
    (float64 tensor: coefficients of x^2, x^3, ...) and Doppler centroid
    (float64 scalar tensor, Hz).  chain "stripmap": the range-Doppler chain
    (s1g_azimuth_adjoint; centroid absolute); "tops": the TOPS chain with
    frequency unfolding (s1g_tops_adjoint; centroid = offset added to the
    burst's estimated centroid)."""

    @staticmethod
    def forward(ctx, theta, centroid, decoder, swath, burst, chain="stripmap"):
        fn = decoder.tops_adjoint if chain == "tops" else decoder.azimuth_adjoint
        loss, g_t, g_c = fn(swath, burst, theta.detach().cpu().numpy(), float(centroid.detach().cpu()), grads=True)
        ctx.save_for_backward(torch.as_tensor(g_t, dtype=theta.dtype, device=theta.device),
                              torch.as_tensor(g_c, dtype=centroid.dtype, device=centroid.device))
        return torch.as_tensor(loss, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad):
        g_t, g_c = ctx.saved_tensors
        return grad * g_t, grad * g_c, None, None, None, None


def autofocus(decoder, swath: str, burst: int, terms: int = 2, centroid: float = 0.0, fit_centroid: bool = False,
              iterations: int = 25, theta0=None, chain: str = "stripmap") -> dict:
    """Minimise the image entropy over the phase-error polynomial (and, if
    asked, the Doppler centroid, or for chain "tops" the offset to the
    estimated one) with L-BFGS.  Returns the estimates and the entropy before
    and after."""
    theta = torch.zeros(terms, dtype=torch.float64) if theta0 is None else \
        torch.as_tensor(np.asarray(theta0, dtype=np.float64)).clone()
    theta.requires_grad_(True)
    fc = torch.tensor(float(centroid), dtype=torch.float64, requires_grad=fit_centroid)
    params = [theta] + ([fc] if fit_centroid else [])
    opt = torch.optim.LBFGS(params, lr=1.0, max_iter=iterations, line_search_fn="strong_wolfe")
    start = float(AzimuthEntropy.apply(theta.detach(), fc.detach(), decoder, swath, burst, chain))
    history = []

    def closure():
        opt.zero_grad()
        loss = AzimuthEntropy.apply(theta, fc, decoder, swath, burst, chain)
        loss.backward()
        history.append(float(loss.detach()))
        return loss

    opt.step(closure)
    end = float(AzimuthEntropy.apply(theta.detach(), fc.detach(), decoder, swath, burst, chain))
    return {"theta": theta.detach().numpy().copy(), "centroid": float(fc.detach()), "entropy_start": start,
            "entropy_end": end, "evaluations": len(history)}
