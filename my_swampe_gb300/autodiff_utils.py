"""Forward-mode gradient helper, the counterpart of the reference's
``my_swampe.autodiff_utils.fwd_grad`` (``autodiff_utils.py:27-89``).

``loss_fn(theta)`` maps a 1-D parameter tensor to a scalar tensor through the
differentiable run (:func:`my_swampe_gb300.adjoint.integrate`); each
directional derivative is one forward-mode pass (``torch.autograd.forward_ad``
dual tensors), which runs the GPU tangent-linear model.

With ``batched=True`` the directions run together, as ``jax.jacfwd`` pushes
them in one vmapped pass: ``loss_fn`` then maps a (k, p) tensor -- k copies of
theta -- to k losses, computing copy i as ensemble member i of one run.  Every
member carries its own tangent, so one tangent-linear launch per step gives k
directional derivatives (``chunk`` bounds k).
"""
from __future__ import annotations

from typing import Callable, Optional

import torch
import torch.autograd.forward_ad as fwAD


def fwd_grad(loss_fn: Callable[[torch.Tensor], torch.Tensor], theta, *, chunk: Optional[int] = None,
             batched: bool = False) -> torch.Tensor:
    """Forward-mode gradient of a scalar loss with respect to a 1-D parameter vector.

    Same contract as the reference: ``theta`` must be 1-D; an empty ``theta``
    gives an empty gradient; ``chunk`` (a positive int, or None for all
    directions at once) groups directions, and a non-positive ``chunk``
    smaller than the parameter count raises ``ValueError``.  By default the
    directions run one after another (each a full primal + tangent run on the
    GPU).  ``batched=True``: ``loss_fn`` takes a (k, p) batch of parameter
    vectors and returns k losses, computing row i as ensemble member i; each
    chunk of k <= chunk directions is then one run whose member i carries
    direction i."""
    theta = torch.as_tensor(theta)
    if theta.dim() != 1:
        raise ValueError(f"theta must be 1-D, got shape {tuple(theta.shape)}.")
    p = int(theta.shape[0])
    if p == 0:
        return torch.zeros((0,), dtype=theta.dtype, device=theta.device)
    if chunk is not None and int(chunk) < p and int(chunk) <= 0:
        raise ValueError(f"chunk must be a positive int or None, got {chunk!r}.")
    eye = torch.eye(p, dtype=theta.dtype, device=theta.device)
    out = torch.empty(p, dtype=theta.dtype, device=theta.device)
    base = theta.detach()
    if batched:
        k = p if chunk is None else min(int(chunk), p)
        for i in range(0, p, k):
            n = min(k, p - i)
            rows = base.expand(n, p).clone()
            with fwAD.dual_level():
                losses = loss_fn(fwAD.make_dual(rows, eye[i: i + n]))
                tangent = fwAD.unpack_dual(losses).tangent
            if tangent is not None and tuple(tangent.shape) != (n,):
                raise ValueError(f"a batched loss_fn must return {n} losses, got shape {tuple(tangent.shape)}")
            out[i: i + n] = tangent if tangent is not None else 0.0
        return out
    for i in range(p):
        with fwAD.dual_level():
            loss = loss_fn(fwAD.make_dual(base, eye[i]))
            tangent = fwAD.unpack_dual(loss).tangent
        out[i] = tangent if tangent is not None else 0.0
    return out
