"""Differentiable batched forward dynamics for trajectory rollouts.

``ABAFunction`` wraps the batched ABA (forward) and the batched analytical ABA
derivatives (backward) of the C ABI in a ``torch.autograd.Function``: for an
incoming gradient g on ddq, the vector-Jacobian products are
``q_bar = ddq_dq^T g``, ``v_bar = ddq_dv^T g`` and ``tau_bar = Minv g`` (Minv is
symmetric), with the Jacobians of reference algorithm/aba-derivatives.hxx:380-453.
The backward calls gb_aba_derivatives_vjp, which applies them without forming
the nv x nv Jacobians (O(nv^2) per instance instead of the O(nv^3) products).

``rollout`` integrates ``v <- v + dt * ABA(q, v, tau_k)``, ``q <- q + dt * v``
(semi-implicit Euler) for all time steps and, with ``checkpoint_every = k``,
stores only every k-th state for the backward pass and recomputes the steps
inside a segment (torch.utils.checkpoint).  The wrapper supports models whose
configuration space is a vector space (revolute and prismatic joints, nq == nv), as the
100-link chain of the rollout workload is.
"""
from __future__ import annotations

import torch
from torch.utils.checkpoint import checkpoint

from . import api
from .model import Model


class ABAFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, v, tau, model: Model, data: api.Data):
        ddq = api.aba(model, data, q.detach(), v.detach(), tau.detach())
        ctx.save_for_backward(q.detach(), v.detach(), tau.detach())
        ctx.model = model
        ctx.data = data
        return ddq

    @staticmethod
    def backward(ctx, g):
        q, v, tau = ctx.saved_tensors
        q_bar, v_bar, tau_bar = api.abaDerivativesVJP(ctx.model, ctx.data, q, v, tau, g.contiguous())
        return q_bar, v_bar, tau_bar, None, None


def aba(model: Model, data: api.Data, q, v, tau):
    """Differentiable batched ABA (q, v, tau: (batch, nv) CUDA float64 tensors)."""
    if model.nq != model.nv:
        raise ValueError("the autograd wrapper needs a vector-space configuration (revolute / prismatic joints, nq == nv)")
    return ABAFunction.apply(q, v, tau, model, data)


def _segment(model, data, dt, q, v, taus):
    for k in range(taus.shape[0]):
        v = v + dt * aba(model, data, q, v, taus[k])
        q = q + dt * v
    return q, v


def rollout(model: Model, data: api.Data, q0, v0, taus, dt: float = 1e-3, checkpoint_every: int | None = 8):
    """Semi-implicit Euler rollout; taus has shape (steps, batch, nv).  Returns (q_T, v_T)."""
    q, v = q0, v0
    steps = taus.shape[0]
    if not checkpoint_every:
        return _segment(model, data, dt, q, v, taus)
    for s in range(0, steps, checkpoint_every):
        seg = taus[s : s + checkpoint_every]
        q, v = checkpoint(_segment, model, data, dt, q, v, seg, use_reentrant=False)
    return q, v
