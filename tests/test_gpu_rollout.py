"""Differentiable rollout through the batched ABA / ABA-derivative kernels
(torch.autograd.Function, semi-implicit Euler, checkpoints every 8 steps):
the final state matches an FP64 rollout of the oracle, the gradients of
||q_T||^2 match central finite differences, and checkpointing changes nothing."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import LOCAL, OracleModel
from pinocchio_gb300 import autograd
from pinocchio_gb300 import sample_models as sm

pytestmark = pytest.mark.gpu


def _setup(n=12, B=4, T=16, seed=0):
    import torch

    model = sm.chain(n, seed, (0.1, 1.0))
    rng = np.random.default_rng(seed)
    q0 = rng.uniform(-np.pi, np.pi, (B, n))
    v0 = 0.1 * rng.standard_normal((B, n))
    taus = rng.standard_normal((T, B, n))
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    return model, q0, v0, taus, d


def test_rollout_matches_oracle_rollout():
    model, q0, v0, taus, d = _setup()
    data = pg.createData(model)
    qT, vT = autograd.rollout(model, data, d(q0), d(v0), d(taus), dt=1e-3, checkpoint_every=8)
    om = OracleModel(model)
    q, v = q0.copy(), v0.copy()
    for k in range(taus.shape[0]):
        v = v + 1e-3 * om.aba(q, v, taus[k], LOCAL)
        q = q + 1e-3 * v
    assert np.abs(qT.detach().cpu().numpy() - q).max() < 1e-12
    assert np.abs(vT.detach().cpu().numpy() - v).max() < 1e-10


def test_rollout_gradients_vs_finite_differences_and_checkpointing():
    import torch

    model, q0, v0, taus, d = _setup(n=8, B=3, T=16, seed=1)
    data = pg.createData(model)

    def loss_of(q0t, v0t, tt, ck):
        qT, _ = autograd.rollout(model, data, q0t, v0t, tt, dt=1e-3, checkpoint_every=ck)
        return (qT**2).sum()

    grads = {}
    for ck in (8, None):
        q0t, v0t, tt = (d(a).requires_grad_() for a in (q0, v0, taus))
        loss_of(q0t, v0t, tt, ck).backward()
        grads[ck] = [t.grad.detach().cpu().numpy() for t in (q0t, v0t, tt)]
    for a, b in zip(grads[8], grads[None]):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-14)
    h = 1e-6
    rng = np.random.default_rng(3)
    with torch.no_grad():
        for which, base in enumerate((q0, v0, taus)):
            for _ in range(4):
                idx = tuple(rng.integers(0, s) for s in base.shape)
                plus, minus = base.copy(), base.copy()
                plus[idx] += h
                minus[idx] -= h
                args_p = [q0, v0, taus]
                args_m = [q0, v0, taus]
                args_p[which], args_m[which] = plus, minus
                fd = (loss_of(*(d(a) for a in args_p), 8) - loss_of(*(d(a) for a in args_m), 8)).item() / (2 * h)
                an = grads[8][which][idx]
                assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (which, idx, fd, an)
