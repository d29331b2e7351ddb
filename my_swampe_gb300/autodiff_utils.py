"""Forward-mode gradient helper, the counterpart of the reference's
``my_swampe.autodiff_utils.fwd_grad`` (``autodiff_utils.py:27-89``).

``loss_fn(theta)`` maps a 1-D parameter tensor to a scalar tensor through the
differentiable run (:func:`my_swampe_gb300.adjoint.integrate`); each
directional derivative is one forward-mode pass (``torch.autograd.forward_ad``
dual tensors), which runs the GPU tangent-linear model.
"""
from __future__ import annotations

from typing import Callable, Optional

import torch
import torch.autograd.forward_ad as fwAD


def fwd_grad(loss_fn: Callable[[torch.Tensor], torch.Tensor], theta, *, chunk: Optional[int] = None) -> torch.Tensor:
    """Forward-mode gradient of a scalar loss with respect to a 1-D parameter vector.

    Same contract as the reference: ``theta`` must be 1-D; an empty ``theta``
    gives an empty gradient; ``chunk`` (a positive int, or None for all
    directions at once) only groups directions, and a non-positive ``chunk``
    smaller than the parameter count raises ``ValueError``.  Directions run one
    after another (each is a full primal + tangent run on the GPU)."""
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
    for i in range(p):
        with fwAD.dual_level():
            loss = loss_fn(fwAD.make_dual(base, eye[i]))
            tangent = fwAD.unpack_dual(loss).tangent
        out[i] = tangent if tangent is not None else 0.0
    return out
