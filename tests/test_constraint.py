"""The oracle's constraintDynamics (reference algorithm/constrained-dynamics.hxx:188-520) pinned by
the reference's own checks (unittest/constrained-dynamics.cpp): no constraint gives ABA (:115-180);
a frame / point contact gives forwardDynamics with the contact frame's Jacobian and drift
(computeAcceleration + getJointJacobian, :66-113 and :578-640); the KKT equations; closed loops
(:500-570) keep the constraint's acceleration at zero (central differences of the constraint
velocity along the motion); the proximal iterations with mu > 0 converge to the undamped solution
and handle redundant constraints; the Baumgarte correction; long double agreement."""
import numpy as np
import pytest

from oracle.oracle import LOCAL as CONV_LOCAL
from oracle.oracle import OracleModel
from pinocchio_gb300 import constraints as cs
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import rel_err

def _se3(x):
    return x[:9].reshape(3, 3), x[9:12]


def _actinv(R, t, m):
    """(R, t)^-1 . act(m) for a motion m = [lin; ang]."""
    return np.concatenate([R.T @ (m[:3] - np.cross(t, m[3:])), R.T @ m[3:]])


def _act(R, t, m):
    w = R @ m[3:]
    return np.concatenate([R @ m[:3] + np.cross(t, w), w])


def _rand_se3(rng, scale=0.2):
    a = rng.standard_normal(3)
    th = np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]]) / th
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
    return gm.SE3(R, scale * rng.standard_normal(3))


def _support(model, j):
    cols = []
    while j > 0:
        cols += list(range(model.idx_vs[j], model.idx_vs[j] + model.nvs[j]))
        j = model.parents[j]
    return sorted(cols)


def _leaves(model):
    par = set(model.parents[1:])
    return [j for j in range(1, model.njoints) if j not in par]


def _frame_jacobian_and_drift(model, om, q, v, c):
    """The contact's Jacobian rows and drift for a constraint to the world (joint2 = 0), built from
    the oracle's joint Jacobians and forward kinematics as the reference's test does."""
    B = q.shape[0]
    oMi, vi, ai = om.forward_kinematics(q, v, np.zeros_like(v))
    Jw = om.joint_jacobians(q)  # (B, nv, 6) world columns
    sup = _support(model, c.joint1_id)
    P = c.joint1_placement
    n = c.size()
    J = np.zeros((B, n, model.nv))
    g = np.zeros((B, n))
    for b in range(B):
        Ri, ti = _se3(oMi[b, c.joint1_id])
        Rc, tc = Ri @ P.rotation, Ri @ P.translation + ti
        for k in sup:
            col = _actinv(Rc, tc, Jw[b, k])
            if c.reference_frame == cs.LOCAL_WORLD_ALIGNED:
                col = np.concatenate([Rc @ col[:3], Rc @ col[3:]])
            J[b, :, k] = col[:n]
        vc = _actinv(P.rotation, P.translation, vi[b, c.joint1_id])
        ac = _actinv(P.rotation, P.translation, ai[b, c.joint1_id])
        if c.type == cs.CONTACT_3D:
            acc = ac[:3] + np.cross(vc[3:], vc[:3])
        else:
            acc = ac
        if c.reference_frame == cs.LOCAL_WORLD_ALIGNED:
            acc = np.concatenate([Rc @ acc[:3], Rc @ acc[3:]]) if n == 6 else Rc @ acc
        g[b] = acc[:n]
    return J, g


def _contacts(model, rng, kinds):
    leaves = _leaves(model)
    out = []
    for k, (t, f) in enumerate(kinds):
        out.append(cs.RigidConstraintModel(t, model, leaves[k % len(leaves)], _rand_se3(rng), f))
    return out


@pytest.fixture(scope="module")
def humanoid():
    model = sm.humanoid32(1)
    return model, OracleModel(model)


def test_no_constraint_is_aba(humanoid):
    model, om = humanoid
    q, v, x = sm.random_inputs(model, 16, 1)
    ddq, lam, it, res = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc([]))
    assert lam.shape == (16, 0) and np.all(it == 1)
    assert rel_err(ddq, om.aba(q, v, 10 * x, CONV_LOCAL)) < 1e-12


@pytest.mark.parametrize("kinds", [
    [(cs.CONTACT_6D, cs.LOCAL)],
    [(cs.CONTACT_6D, cs.LOCAL_WORLD_ALIGNED), (cs.CONTACT_6D, cs.LOCAL)],
    [(cs.CONTACT_3D, cs.LOCAL), (cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED), (cs.CONTACT_6D, cs.LOCAL)],
    [(cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED)] * 4,
])
def test_contacts_match_forward_dynamics_and_kkt(humanoid, kinds):
    """constraintDynamics == forwardDynamics(J, gamma) with the contact frames' Jacobians and drifts,
    and M ddq + nle - tau = J^T lambda (constrained-dynamics.cpp:578-640)."""
    model, om = humanoid
    rng = np.random.default_rng(len(kinds))
    cms = _contacts(model, rng, kinds)
    q, v, x = sm.random_inputs(model, 12, 2)
    tau = 10 * x
    ddq, lam, it, res = om.constraint_dynamics(q, v, tau, cs.stack_desc(cms))
    Js, gs = zip(*(_frame_jacobian_and_drift(model, om, q, v, c) for c in cms))
    J, g = np.concatenate(Js, axis=1), np.concatenate(gs, axis=1)
    d_ref, l_ref = om.forward_dynamics(q, v, tau, J, g)
    assert rel_err(ddq, d_ref) < 1e-10 and rel_err(lam, l_ref) < 1e-10
    nle = om.rnea(q, v, np.zeros_like(v))
    M = om.crba(q)
    M = np.triu(M) + np.swapaxes(np.triu(M, 1), 1, 2)
    lhs = np.einsum("bij,bj->bi", M, ddq) + nle - tau
    assert rel_err(lhs, np.einsum("bcj,bc->bj", J, lam)) < 1e-9
    assert np.abs(np.einsum("bcj,bj->bc", J, ddq) + g).max() < 1e-8 * max(1.0, np.abs(g).max())
    assert np.all(it == 1)


def _velocity_error(model, om, q, v, c):
    """The constraint's velocity error of a closed loop: 6D LOCAL vc1 - c1Mc2.act(vc2) in frame 1;
    3D: the world velocity difference of the two points."""
    oMi, vi, _ = om.forward_kinematics(q, v)
    out = []
    for b in range(q.shape[0]):
        fr = []
        for j, P in ((c.joint1_id, c.joint1_placement), (c.joint2_id, c.joint2_placement)):
            Ri, ti = _se3(oMi[b, j])
            Rc, tc = Ri @ P.rotation, Ri @ P.translation + ti
            vc = _actinv(P.rotation, P.translation, vi[b, j]) if j > 0 else np.zeros(6)
            fr.append((Rc, tc, vc))
        (R1, t1, v1), (R2, t2, v2) = fr
        if c.type == cs.CONTACT_6D:
            R12, t12 = R1.T @ R2, R1.T @ (t2 - t1)
            out.append(v1 - _act(R12, t12, v2))
        else:
            out.append(R1 @ v1[:3] - R2 @ v2[:3])
    return np.array(out)


@pytest.mark.parametrize("ctype", [cs.CONTACT_6D, cs.CONTACT_3D])
def test_closed_loop_keeps_constraint_acceleration_zero(humanoid, ctype):
    """A loop between two limbs: d/dt of the constraint velocity along (v, ddq) vanishes
    (central differences over q(t +- h) = integrate(q, +-h v + h^2/2 ddq), v(t +- h) = v +- h ddq)."""
    model, om = humanoid
    rng = np.random.default_rng(7)
    lv = _leaves(model)
    c = cs.RigidConstraintModel(ctype, model, lv[1], _rand_se3(rng), lv[3], _rand_se3(rng), cs.LOCAL)
    q, v, x = sm.random_inputs(model, 6, 3)
    v = 0.3 * v
    ddq, lam, it, res = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc([c]))
    h = 1e-5
    qp = om.integrate(q, h * v + 0.5 * h * h * ddq)
    qm = om.integrate(q, -h * v + 0.5 * h * h * ddq)
    dve = (_velocity_error(model, om, qp, v + h * ddq, c) - _velocity_error(model, om, qm, v - h * ddq, c)) / (2 * h)
    assert np.abs(dve).max() < 1e-5 * max(1.0, np.abs(ddq).max())


def test_proximal_iterations_converge_and_handle_redundancy(humanoid):
    """mu > 0 with enough iterations reaches the undamped solution (relative residual below the
    accuracy); a duplicated contact (singular Delassus matrix) is solved by the proximal iterations
    with the same accelerations as the single contact (constrained-dynamics.hpp: mu ~ 1e-12 hint)."""
    model, om = humanoid
    rng = np.random.default_rng(4)
    cms = _contacts(model, rng, [(cs.CONTACT_6D, cs.LOCAL), (cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED)])
    q, v, x = sm.random_inputs(model, 8, 5)
    d0, l0, _, _ = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms))
    d1, l1, it, res = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms), mu=1e-4, max_iter=200)
    assert np.all(it > 1) and np.all(it < 200) and np.all(res[:, 1] <= 1e-12)
    assert rel_err(d1, d0) < 1e-9 and rel_err(l1, l0) < 1e-9
    one = cms[:1]
    dd, ld, itd, resd = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(one + one), mu=1e-6, max_iter=500)
    ds, ls, _, _ = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(one))
    assert rel_err(dd, ds) < 1e-7
    assert rel_err(ld[:, :6] + ld[:, 6:], ls) < 1e-7  # the force splits between the two copies
    d2, _, it2, res2 = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms), mu=1e-4, max_iter=3)
    assert np.all(it2 == 3) and np.all(res2[:, 1] > 0)


def _log6(R, t):
    c = np.clip((np.trace(R) - 1) / 2, -1, 1)
    a = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2
    th = np.arctan2(np.linalg.norm(a), c)
    w = a * (th / np.sin(th)) if th > 1e-8 else a
    if th < 1e-8:
        alpha, beta = 1.0, 1.0 / 12
    else:
        alpha = th * np.sin(th) / (2 * (1 - np.cos(th)))
        beta = 1 / th**2 - np.sin(th) / (2 * th * (1 - np.cos(th)))
    return np.concatenate([alpha * t - 0.5 * np.cross(w, t) + beta * w.dot(t) * w, w])


def test_baumgarte_correction_and_desired_acceleration(humanoid):
    """A 6D LOCAL contact to a world anchor with Kp, Kd and a desired acceleration: the contact
    frame's spatial acceleration equals -Kp (-log6(c1Mc2)) - Kd vc1 + a_desired."""
    model, om = humanoid
    rng = np.random.default_rng(9)
    j = _leaves(model)[0]
    c = cs.RigidConstraintModel(cs.CONTACT_6D, model, j, _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL)
    c.corrector.Kp[:] = rng.uniform(1, 10, 6)
    c.corrector.Kd[:] = rng.uniform(1, 10, 6)
    c.desired_contact_acceleration[:] = rng.standard_normal(6)
    q, v, x = sm.random_inputs(model, 5, 6)
    ddq, lam, it, res = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc([c]))
    oMi, vi, ai = om.forward_kinematics(q, v, ddq)
    P1, P2 = c.joint1_placement, c.joint2_placement
    for b in range(q.shape[0]):
        Ri, ti = _se3(oMi[b, j])
        R1, t1 = Ri @ P1.rotation, Ri @ P1.translation + ti
        R12, t12 = R1.T @ P2.rotation, R1.T @ (P2.translation - t1)
        vc1 = _actinv(P1.rotation, P1.translation, vi[b, j])
        ac1 = _actinv(P1.rotation, P1.translation, ai[b, j])
        want = c.corrector.Kp * _log6(R12, t12) - c.corrector.Kd * vc1 + c.desired_contact_acceleration
        assert np.allclose(ac1, want, rtol=1e-9, atol=1e-9 * np.abs(want).max())


def test_long_double_agreement(humanoid):
    model, om = humanoid
    rng = np.random.default_rng(11)
    cms = _contacts(model, rng, [(cs.CONTACT_6D, cs.LOCAL), (cs.CONTACT_3D, cs.LOCAL), (cs.CONTACT_6D, cs.LOCAL_WORLD_ALIGNED)])
    cms[0].corrector.Kp[:] = 3.0
    cms[1].corrector.Kd[:] = 2.0
    q, v, x = sm.random_inputs(model, 8, 8)
    a = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms), mu=1e-6, max_iter=4)
    b = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms), mu=1e-6, max_iter=4, prec=1)
    assert rel_err(a[0], b[0]) < 1e-11 and rel_err(a[1], b[1]) < 1e-11


def test_argument_errors(humanoid):
    model, om = humanoid
    with pytest.raises(ValueError):
        cs.RigidConstraintModel(cs.CONTACT_6D, model, 3, cs.WORLD)
    with pytest.raises(ValueError):
        cs.RigidConstraintModel(cs.CONTACT_6D, model, model.njoints)
    with pytest.raises(ValueError):
        cs.ProximalSettings(1e-12, -1.0, 1)
    with pytest.raises(ValueError):
        cs.ProximalSettings(1e-12, 0.0, 0)
    c = cs.RigidConstraintModel(cs.CONTACT_3D, model, 5, gm.SE3.Identity(), cs.LOCAL_WORLD_ALIGNED)
    assert c.joint2_id == 0 and c.reference_frame == cs.LOCAL_WORLD_ALIGNED and c.size() == 3
    c = cs.RigidConstraintModel(cs.CONTACT_6D, model, 5, gm.SE3.Identity(), 7, gm.SE3.Identity(), cs.LOCAL)
    assert (c.joint1_id, c.joint2_id) == (5, 7)


def _central_differences(model, om, q, v, tau, desc, h=1e-6, **kw):
    """Central differences of constraintDynamics' (ddq, lambda_c) in q (along integrate), v and tau."""
    B, nv = q.shape[0], model.nv
    out = []
    for which in ("q", "v", "tau"):
        dd = np.zeros((B, nv, nv))
        dl = None
        for k in range(nv):
            e = np.zeros((B, nv))
            e[:, k] = h
            if which == "q":
                args_p, args_m = (om.integrate(q, e), v, tau), (om.integrate(q, -e), v, tau)
            elif which == "v":
                args_p, args_m = (q, v + e, tau), (q, v - e, tau)
            else:
                args_p, args_m = (q, v, tau + e), (q, v, tau - e)
            fp = om.constraint_dynamics(*args_p, desc, **kw)
            fm = om.constraint_dynamics(*args_m, desc, **kw)
            dd[:, :, k] = (fp[0] - fm[0]) / (2 * h)
            if dl is None:
                dl = np.zeros((B, fp[1].shape[1], nv))
            dl[:, :, k] = (fp[1] - fm[1]) / (2 * h)
        out += [dd, dl]
    return out  # ddq_dq, dl_dq, ddq_dv, dl_dv, ddq_dtau, dl_dtau


@pytest.mark.parametrize("kinds", [
    [(cs.CONTACT_6D, cs.LOCAL), (cs.CONTACT_3D, cs.LOCAL)],
    [(cs.CONTACT_6D, cs.LOCAL_WORLD_ALIGNED), (cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED)],
    [(cs.CONTACT_3D, cs.LOCAL), (cs.CONTACT_6D, cs.LOCAL_WORLD_ALIGNED), (cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED),
     (cs.CONTACT_6D, cs.LOCAL)],
])
def test_constraint_dynamics_derivatives_central_differences(humanoid, kinds):
    """computeConstraintDynamicsDerivatives (constraints to the world, no gains) against central
    differences of constraintDynamics (the check of unittest/constrained-dynamics-derivatives.cpp)."""
    model, om = humanoid
    rng = np.random.default_rng(21)
    cms = [cs.RigidConstraintModel(t, model, j, _rand_se3(rng), 0, _rand_se3(rng, 1.0), f)
           for (t, f), j in zip(kinds, _leaves(model))]
    q, v, x = sm.random_inputs(model, 4, 22)
    desc = cs.stack_desc(cms)
    got = om.constraint_dynamics_derivatives(q, v, 10 * x, desc)
    ref = om.constraint_dynamics(q, v, 10 * x, desc)
    assert rel_err(got[0], ref[0]) < 1e-14 and rel_err(got[1], ref[1]) < 1e-14
    fd = _central_differences(model, om, q, v, 10 * x, desc)
    names = ("ddq_dq", "dlambda_dq", "ddq_dv", "dlambda_dv", "ddq_dtau", "dlambda_dtau")
    analytic = (got[2], got[5], got[3], got[6], got[4], got[7])
    for name, a, f in zip(names, analytic, fd):
        assert rel_err(a, f) < 1e-6, (name, rel_err(a, f))


def test_constraint_dynamics_derivatives_with_local_contact_gains(humanoid):
    """LOCAL point and frame contacts to the world with Baumgarte gains (the corrector's derivative,
    constrained-dynamics-derivatives.hxx:753-830, with Jlog6 for the frame contact) against central
    differences, next to a world-aligned point contact without gains; the reference's same terms in
    LOCAL_WORLD_ALIGNED axes disagree with central differences and are refused."""
    model, om = humanoid
    rng = np.random.default_rng(31)
    lv = _leaves(model)
    cms = [cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[0], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[2], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_6D, model, lv[1], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[3], _rand_se3(rng), 0, _rand_se3(rng, 1.0),
                                   cs.LOCAL_WORLD_ALIGNED)]
    for c in cms[:3]:
        c.corrector.Kp[:] = rng.uniform(0.5, 5.0, c.size())
        c.corrector.Kd[:] = rng.uniform(0.5, 5.0, c.size())
    q, v, x = sm.random_inputs(model, 4, 32)
    desc = cs.stack_desc(cms)
    got = om.constraint_dynamics_derivatives(q, v, 10 * x, desc)
    fd = _central_differences(model, om, q, v, 10 * x, desc)
    names = ("ddq_dq", "dlambda_dq", "ddq_dv", "dlambda_dv", "ddq_dtau", "dlambda_dtau")
    analytic = (got[2], got[5], got[3], got[6], got[4], got[7])
    for name, a, f in zip(names, analytic, fd):
        assert rel_err(a, f) < 1e-6, (name, rel_err(a, f))
    cms[3].corrector.Kp[:] = 1.0
    with pytest.raises(ValueError):
        om.constraint_dynamics_derivatives(q, v, 10 * x, cs.stack_desc(cms))


def test_constraint_dynamics_derivatives_proximal_and_errors(humanoid):
    """With mu > 0 the derivatives follow the proximal recursion: at convergence they approach the
    undamped derivatives; closed loops and Baumgarte gains in world-aligned axes are rejected."""
    model, om = humanoid
    rng = np.random.default_rng(23)
    cms = [cs.RigidConstraintModel(cs.CONTACT_6D, model, j, _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL)
           for j in _leaves(model)[:2]]
    q, v, x = sm.random_inputs(model, 3, 24)
    desc = cs.stack_desc(cms)
    a = om.constraint_dynamics_derivatives(q, v, 10 * x, desc)
    b = om.constraint_dynamics_derivatives(q, v, 10 * x, desc, mu=1e-6, max_iter=50, absolute_accuracy=0.0,
                                           relative_accuracy=1e-14)
    assert np.all(b[8] > 1)
    for k in range(2, 8):
        assert rel_err(b[k], a[k]) < 1e-6, k
    loop = [cs.RigidConstraintModel(cs.CONTACT_6D, model, _leaves(model)[0], gm.SE3.Identity(), _leaves(model)[1],
                                    gm.SE3.Identity(), cs.LOCAL)]
    with pytest.raises(ValueError, match="world"):
        om.constraint_dynamics_derivatives(q, v, x, cs.stack_desc(loop))
    wa = [cs.RigidConstraintModel(cs.CONTACT_6D, model, _leaves(model)[0], gm.SE3.Identity(), 0, gm.SE3.Identity(),
                                  cs.LOCAL_WORLD_ALIGNED)]
    wa[0].corrector.Kp[:] = 1.0
    with pytest.raises(ValueError, match="LOCAL contacts"):
        om.constraint_dynamics_derivatives(q, v, x, cs.stack_desc(wa))


@pytest.mark.parametrize("mu", [0.0, 0.1])
def test_contact_cholesky_accessors(humanoid, mu):
    """ContactCholeskyDecomposition (unittest/contact-cholesky.cpp:270-420): matrix() is the KKT
    matrix [[-mu I, J], [J^T, M]] built from the contact frames' Jacobians and M, inverse() its
    inverse, getInverseOperationalSpaceInertiaMatrix() = J M^-1 J^T + mu I,
    getOperationalSpaceInertiaMatrix() its inverse, getInverseMassMatrix() = M^-1, getJMinv() = J M^-1."""
    model, om = humanoid
    rng = np.random.default_rng(11)
    cms = _contacts(model, rng, [(cs.CONTACT_6D, cs.LOCAL), (cs.CONTACT_3D, cs.LOCAL_WORLD_ALIGNED)])
    q, v, x = sm.random_inputs(model, 6, 12)
    out = om.contact_cholesky(q, cs.stack_desc(cms), mu=mu)
    J = np.concatenate([_frame_jacobian_and_drift(model, om, q, v, c)[0] for c in cms], axis=1)
    M = om.crba(q)
    M = np.triu(M) + np.swapaxes(np.triu(M, 1), 1, 2)
    nc, nv = J.shape[1], model.nv
    H = np.zeros((6, nc + nv, nc + nv))
    H[:, :nc, :nc] = -mu * np.eye(nc)
    H[:, :nc, nc:] = J
    H[:, nc:, :nc] = np.swapaxes(J, 1, 2)
    H[:, nc:, nc:] = M
    assert rel_err(out["matrix"], H) < 1e-12
    eye = np.broadcast_to(np.eye(nc + nv), H.shape)
    assert np.abs(np.einsum("bij,bjk->bik", out["inverse"], H) - eye).max() < 1e-9
    Minv = np.linalg.inv(M)
    JMJ = np.einsum("bij,bjk,blk->bil", J, Minv, J) + mu * np.eye(nc)
    assert rel_err(out["osim_inverse"], JMJ) < 1e-11
    assert rel_err(out["osim"], np.linalg.inv(JMJ)) < 1e-9
    assert rel_err(out["minv"], Minv) < 1e-11
    assert rel_err(out["jminv"], np.einsum("bij,bjk->bik", J, Minv)) < 1e-11


def test_jlog6_against_central_differences():
    """Jlog6 (spatial/explog.hpp) = d log6(M exp6(d)) / dd at 0, at large, small and zero angles."""
    from oracle.oracle import log6

    def exp6(d):
        rho, phi = d[:3], d[3:]
        t = np.linalg.norm(phi)
        P = np.array([[0, -phi[2], phi[1]], [phi[2], 0, -phi[0]], [-phi[1], phi[0], 0]])
        if t < 1e-12:
            return np.eye(3) + P, rho + P @ rho / 2
        R = np.eye(3) + np.sin(t) / t * P + (1 - np.cos(t)) / t**2 * P @ P
        V = np.eye(3) + (1 - np.cos(t)) / t**2 * P + (t - np.sin(t)) / t**3 * P @ P
        return R, V @ rho

    rng = np.random.default_rng(0)
    for scale in (2.5, 1.0, 1e-4, 0.0):
        R, t = exp6(np.concatenate([rng.standard_normal(3), scale * rng.standard_normal(3)]))
        _, J = log6((R, t))
        F = np.zeros((6, 6))
        for k in range(6):
            e = np.zeros(6)
            e[k] = 1e-6
            (Rp, tp), (Rm, tm) = exp6(e), exp6(-e)
            F[:, k] = (log6((R @ Rp, R @ tp + t))[0] - log6((R @ Rm, R @ tm + t))[0]) / 2e-6
        assert np.abs(J - F).max() < 1e-8, scale

