"""Contact dynamics with a given constraint Jacobian, the oracle on the CPU:
forwardDynamics(q, v, tau, J, gamma, inv_damping) and impulseDynamics(q, v_before,
J, r_coeff, inv_damping) (reference algorithm/contact-dynamics.hxx:81-165,
255-327) against the identities of the reference's unittest/contact-dynamics.cpp
(test_FD 21-92, test_FD_with_damping 213-271, test_ID 273-337): the multipliers
equal -(J M^-1 J^T)^-1 (J M^-1 (tau - nle) + gamma) computed with dense inverses
here, the dynamics residual M ddq + nle - tau - J^T lambda and the constraint
residual J ddq + gamma vanish; with damping J ddq + gamma = -inv_damping lambda;
after an impact J dq_after = -r_coeff J v_before."""
import numpy as np
import pytest

from oracle.oracle import LOCAL, OracleModel, symmetrize_upper
from pinocchio_gb300 import sample_models as sm
from test_oracle import _support
from util import MODELS, rel_err


def feet_jacobian(model, om, q, joints):
    """6 rows per listed joint: its world-frame Jacobian columns (the rows of data.J that move it)."""
    Jw = om.joint_jacobians(q)  # (B, nv, 6)
    sup = _support(model)
    J = np.zeros((q.shape[0], 6 * len(joints), model.nv))
    for r, i in enumerate(joints):
        for k in sup[i]:
            J[:, 6 * r:6 * r + 6, k] = Jw[:, k]
    return J


def leaf_joints(model, n=2):
    parents = list(model.tables()["parents"])
    leaves = [i for i in range(1, len(parents)) if i not in parents]
    return leaves[-n:]


@pytest.fixture(scope="module", params=["humanoid32", "tree32ff", "mixedtree24ff", "unaligned20ff"])
def case(request):
    model = MODELS[request.param]()
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 6, 41)
    if request.param == "humanoid32":  # two feet, 6 rows each, as the reference's test_FD
        J = feet_jacobian(model, om, q, leaf_joints(model))
    else:  # full row rank: 8 random rows
        J = np.random.default_rng(43).normal(size=(6, 8, model.nv))
    gamma = np.random.default_rng(42).normal(size=(6, J.shape[1]))
    return request.param, model, om, q, v, 10.0 * x, J, gamma


def _dense(model, om, q, v):
    M = symmetrize_upper(om.crba(q, LOCAL))
    nle = om.rnea(q, v, np.zeros_like(v))
    return M, nle, np.linalg.inv(M)


def test_forward_dynamics_identities(case):
    name, model, om, q, v, tau, J, gamma = case
    ddq, lam = om.forward_dynamics(q, v, tau, J, gamma)
    M, nle, Minv = _dense(model, om, q, v)
    JMJ = J @ Minv @ J.transpose(0, 2, 1)
    rhs = np.einsum("bck,bk->bc", J @ Minv, tau - nle) + gamma
    assert rel_err(lam, -np.linalg.solve(JMJ, rhs[..., None])[..., 0]) < 1e-10
    scale = np.abs(tau).max()
    dyn = np.einsum("bij,bj->bi", M, ddq) + nle - tau - np.einsum("bck,bc->bk", J, lam)
    assert np.abs(dyn).max() < 1e-10 * scale
    assert np.abs(np.einsum("bck,bk->bc", J, ddq) + gamma).max() < 1e-10 * scale
    ddl, laml = om.forward_dynamics(q, v, tau, J, gamma, prec=1)
    assert rel_err(ddq, ddl) < 1e-11 and rel_err(lam, laml) < 1e-11


def test_forward_dynamics_with_damping_and_without_rows(case):
    name, model, om, q, v, tau, J, gamma = case
    mu = 1e-3
    ddq, lam = om.forward_dynamics(q, v, tau, J, gamma, inv_damping=mu)
    assert np.abs(np.einsum("bck,bk->bc", J, ddq) + gamma + mu * lam).max() < 1e-9 * np.abs(tau).max()
    # a repeated row makes J M^-1 J^T singular: damping keeps the solve defined
    J2 = np.concatenate([J, J[:, :1]], axis=1)
    g2 = np.concatenate([gamma, gamma[:, :1]], axis=1)
    d2, l2 = om.forward_dynamics(q, v, tau, J2, g2, inv_damping=mu)
    assert np.isfinite(d2).all() and np.isfinite(l2).all()
    # no constraint rows: the unconstrained dynamics (ABA)
    d0, l0 = om.forward_dynamics(q, v, tau, J[:, :0], gamma[:, :0])
    assert l0.shape == (q.shape[0], 0)
    assert rel_err(d0, om.aba(q, v, tau)) < 1e-11


def test_impulse_dynamics_identities(case):
    name, model, om, q, v, tau, J, gamma = case
    for r in (0.0, 0.4):
        out, imp = om.impulse_dynamics(q, v, J, r_coeff=r)
        M, _, Minv = _dense(model, om, q, v)
        JMJ = J @ Minv @ J.transpose(0, 2, 1)
        Jv = np.einsum("bck,bk->bc", J, v)
        assert rel_err(imp, np.linalg.solve(JMJ, (-(1 + r) * Jv)[..., None])[..., 0]) < 1e-10
        assert np.abs(np.einsum("bij,bj->bi", M, out - v) - np.einsum("bck,bc->bk", J, imp)).max() < 1e-10 * np.abs(v).max()
        assert np.abs(np.einsum("bck,bk->bc", J, out) + r * Jv).max() < 1e-10 * np.abs(v).max()


@pytest.mark.parametrize("mu", [0.0, 1e-3])
def test_kkt_inverse(case, mu):
    """computeKKTContactDynamicMatrixInverse against the dense inverse of [[M, J^T], [J, -mu I]]
    (unittest/contact-dynamics.cpp:94-134)"""
    name, model, om, q, v, tau, J, gamma = case
    K = om.kkt_inverse(q, J, mu)
    M, _, _ = _dense(model, om, q, v)
    nc = J.shape[1]
    KKT = np.block([[M, J.transpose(0, 2, 1)], [J, np.broadcast_to(-mu * np.eye(nc), (len(q), nc, nc))]])
    assert rel_err(K, np.linalg.inv(KKT)) < 1e-9
