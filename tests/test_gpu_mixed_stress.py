"""Mixed precision on the configurations that are benchmarked with it: the ABA
derivatives and their vector-Jacobian products on the 100-link chain (the rollout
workload's model), and a rollout shaped like the benchmarked one (100-link chain, 64
semi-implicit Euler steps of dt = 1e-3, checkpoints every 8 steps) in mixed precision
against the FP64 oracle rollout: the final state and the gradients of ||q_T||^2 with
respect to q0, v0 and every tau_k (the oracle's gradients come from the adjoint
recursion over its analytical ABA derivatives, unittest/aba-derivatives.cpp:117-154
being the reference's own check of those derivatives).  The max and median relative
errors are printed; the bar is 1e-5."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel, rollout_with_gradients
from pinocchio_gb300 import autograd
from pinocchio_gb300 import sample_models as sm
from util import MIXED_TOL, med_rel_err, rel_err

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_mixed_aba_derivatives_chain100():
    model = sm.chain(100, 4)
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 257, 41)
    tau = 10.0 * x
    data = pg.createData(model, "mixed")
    dq, dv, Minv = (t.cpu().numpy() for t in pg.computeABADerivatives(model, data, _dev(q), _dev(v), _dev(tau)))
    ddq_o, dq_o, dv_o, Minv_o = om.aba_derivatives(q, v, tau)
    errs = {n: (rel_err(a, b), med_rel_err(a, b)) for n, a, b in
            (("ddq", data.ddq.cpu().numpy(), ddq_o), ("ddq_dq", dq, dq_o), ("ddq_dv", dv, dv_o), ("Minv", Minv, Minv_o))}
    print("chain100 mixed ABA derivatives (max, median):", errs)
    for n, (mx, _) in errs.items():
        assert mx < MIXED_TOL, (n, mx)


def test_mixed_aba_derivatives_vjp_chain100():
    model = sm.chain(100, 4)
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 257, 43)
    tau = 10.0 * x
    g = np.random.default_rng(5).standard_normal((q.shape[0], model.nv))
    data = pg.createData(model, "mixed")
    qb, vb, tb = (a.cpu().numpy() for a in pg.abaDerivativesVJP(model, data, _dev(q), _dev(v), _dev(tau), _dev(g)))
    _, dq, dv, Minv = om.aba_derivatives(q, v, tau)
    refs = (np.einsum("bk,bkc->bc", g, dq), np.einsum("bk,bkc->bc", g, dv), np.einsum("bkc,bc->bk", Minv, g))
    errs = {n: (rel_err(a, b), med_rel_err(a, b)) for n, a, b in zip(("q_bar", "v_bar", "tau_bar"), (qb, vb, tb), refs)}
    print("chain100 mixed VJP (max, median):", errs)
    for n, (mx, _) in errs.items():
        assert mx < MIXED_TOL, (n, mx)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_rollout_chain100_64_steps_vs_fp64_oracle(precision):
    import torch

    n, B, T, dt = 100, 24, 64, 1e-3
    model = sm.chain(n, 4, (0.1, 1.0))
    rng = np.random.default_rng(5)
    q0 = rng.uniform(-np.pi, np.pi, (B, n))
    v0 = 0.1 * rng.standard_normal((B, n))
    taus = rng.standard_normal((T, B, n))
    data = pg.createData(model, precision)
    q0t, v0t, tt = (_dev(a).requires_grad_() for a in (q0, v0, taus))
    qT, vT = autograd.rollout(model, data, q0t, v0t, tt, dt=dt, checkpoint_every=8)
    (qT**2).sum().backward()
    got = [qT.detach().cpu().numpy(), q0t.grad.cpu().numpy(), v0t.grad.cpu().numpy(),
           tt.grad.cpu().numpy().transpose(1, 0, 2)]
    qT_o, _, gq_o, gv_o, gt_o = rollout_with_gradients(OracleModel(model), q0, v0, taus, dt)
    refs = [qT_o, gq_o, gv_o, gt_o.transpose(1, 0, 2)]
    errs = {k: (rel_err(a, b), med_rel_err(a, b)) for k, a, b in zip(("q_T", "grad_q0", "grad_v0", "grad_taus"), got, refs)}
    print(f"rollout chain100 T=64 {precision} (max, median):", errs)
    tol = MIXED_TOL if precision == "mixed" else 1e-10
    for k, (mx, _) in errs.items():
        assert mx < tol, (k, mx)
    del torch
