"""The CPU oracle against the reference's own identity tests and analytic known answers.

The reference's hot-path tests pin no numbers; they check identities, which are
restated here against the oracle (reference file:line on each test):
  ABA o RNEA round trip (unittest/aba.cpp:124-184), tau = M a + nle (unittest/aba.cpp:229-263),
  CRBA vs RNEA columns (unittest/crba.cpp:67-130), U D U^T = M (unittest/cholesky.cpp:31-100),
  Minv M = I (unittest/aba-derivatives.cpp:96-100), derivatives vs finite differences
  (unittest/rnea-derivatives.cpp:113-314, unittest/aba-derivatives.cpp:23-155),
  batch == serial bit-exact (unittest/parallel-aba.cpp:21-55, unittest/parallel-rnea.cpp:78-112).
"""
import copy

import numpy as np
import pytest

from oracle.oracle import LOCAL, WORLD, OracleModel, symmetrize_upper
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import MODELS, ORACLE_ONLY_MODELS, rel_err

CPU_MODELS = ["manipulator6r", "humanoid32", "tree12", "tree60ff", "chain100", "mixedtree12", "mixedtree24ff",
              "unaligned14", "unaligned20ff", "translationtree14", "multidoftree16", "unbounded15ff"]


@pytest.fixture(scope="module", params=CPU_MODELS)
def case(request):
    model = {**MODELS, **ORACLE_ONLY_MODELS}[request.param]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 16, 11)
    return request.param, model, om, q, v, a


def test_aba_rnea_roundtrip(case):
    name, model, om, q, v, a = case
    tau = om.rnea(q, v, a)
    tol = 1e-10 if name == "chain100" else 1e-12
    for conv in (LOCAL, WORLD):
        assert rel_err(om.aba(q, v, tau, conv), a) < tol


def test_mass_matrix_and_nle(case):
    name, model, om, q, v, a = case
    tau = om.rnea(q, v, a)
    nle = om.rnea(q, v, np.zeros_like(a))
    M = symmetrize_upper(om.crba(q))
    assert rel_err(np.einsum("bij,bj->bi", M, a) + nle, tau) < 1e-12


def test_crba_columns_and_conventions(case):
    name, model, om, q, v, a = case
    M = symmetrize_upper(om.crba(q, LOCAL))
    assert rel_err(symmetrize_upper(om.crba(q, WORLD)), M) < 1e-12
    # block-upper triangle only, as crba leaves it: rows of joint i, columns of its subtree
    joint_of = np.repeat(np.arange(model.njoints), model.nvs)
    lower_other = np.tril(np.ones((model.nv, model.nv), bool), -1) & (joint_of[:, None] != joint_of[None, :])
    assert np.all(om.crba(q)[:, lower_other] == 0.0)
    zero = np.zeros_like(v)
    g = om.rnea(q, zero, zero)
    for j in range(0, model.nv, max(1, model.nv // 5)):
        e = np.zeros_like(v)
        e[:, j] = 1.0
        # the difference cancels the (much larger) gravity torque: allow its rounding
        assert rel_err(om.rnea(q, zero, e) - g, M[:, :, j]) < 1e-10


def test_cholesky(case):
    name, model, om, q, v, a = case
    Mu = om.crba(q)
    U, D = om.cholesky(Mu)
    M = symmetrize_upper(Mu)
    assert np.allclose(np.diagonal(U, axis1=1, axis2=2), 1.0) and np.all(np.tril(U, -1) == 0)
    assert rel_err(np.einsum("bij,bj,bkj->bik", U, D, U), M) < 1e-12


def test_aba_derivatives_consistency(case):
    name, model, om, q, v, a = case
    tau = om.rnea(q, v, a)
    ddq, ddq_dq, ddq_dv, Minv = om.aba_derivatives(q, v, tau)
    M = symmetrize_upper(om.crba(q))
    eye = np.broadcast_to(np.eye(model.nv), M.shape)
    tol = 1e-9 if name == "chain100" else 1e-12
    assert rel_err(np.einsum("bij,bjk->bik", Minv, M), eye) < tol
    assert np.array_equal(Minv, np.swapaxes(Minv, 1, 2))
    # ddq_dq = -Minv dtau_dq(q, v, ddq) with the RNEA derivatives (aba-derivatives.hxx:451-452)
    _, dtau_dq, dtau_dv, _ = om.rnea_derivatives(q, v, ddq)
    assert rel_err(-np.einsum("bij,bjk->bik", Minv, dtau_dq), ddq_dq) < 1e-11
    assert rel_err(-np.einsum("bij,bjk->bik", Minv, dtau_dv), ddq_dv) < 1e-11


def _fd(f, x0, h, k, integrate=None):
    e = np.zeros((x0.shape[0], integrate[1] if integrate else x0.shape[1]))
    e[:, k] = h
    if integrate:
        return (f(integrate[0](x0, e)) - f(integrate[0](x0, -e))) / (2 * h)
    return (f(x0 + e) - f(x0 - e)) / (2 * h)


@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "tree12", "mixedtree24ff", "unaligned20ff",
                                  "translationtree14", "multidoftree16", "unbounded15ff"])
def test_derivatives_vs_central_fd(name):
    model = {**MODELS, **ORACLE_ONLY_MODELS}[name]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 4, 5)
    tau = om.rnea(q, v, a)
    _, dq, dv, _ = om.rnea_derivatives(q, v, a)
    _, adq, adv, Minv = om.aba_derivatives(q, v, tau)
    h = 1e-6  # central differences in the tangent space, step 1e-6
    fd = {k: np.zeros_like(dq) for k in ("rq", "rv", "aq", "av", "at")}
    for k in range(model.nv):
        fd["rq"][:, :, k] = _fd(lambda x: om.rnea(x, v, a), q, h, k, (om.integrate, model.nv))
        fd["rv"][:, :, k] = _fd(lambda x: om.rnea(q, x, a), v, h, k)
        fd["aq"][:, :, k] = _fd(lambda x: om.aba(x, v, tau), q, h, k, (om.integrate, model.nv))
        fd["av"][:, :, k] = _fd(lambda x: om.aba(q, x, tau), v, h, k)
        fd["at"][:, :, k] = _fd(lambda x: om.aba(q, v, x), tau, h, k)
    assert rel_err(dq, fd["rq"]) < 1e-6
    assert rel_err(dv, fd["rv"]) < 1e-6
    assert rel_err(adq, fd["aq"]) < 1e-6
    assert rel_err(adv, fd["av"]) < 1e-6
    assert rel_err(Minv, fd["at"]) < 1e-6


def test_unbounded_revolute_is_the_revolute_joint_in_its_angle():
    """An unbounded revolute joint at q = (cos t, sin t) (joint-revolute-unbounded.hpp) has the
    dynamics of the revolute joint about the same axis at t, in every function and derivative
    (both have nv = 1 and the same motion subspace); its integrate is the rotation of the unit
    complex by v with the first-order renormalisation (special-orthogonal.hpp:164-185)."""
    mu = MODELS["unbounded15ff"]()
    mr = copy.deepcopy(mu)
    to_rev = {gm.JT_RUBX: gm.JT_RX, gm.JT_RUBY: gm.JT_RY, gm.JT_RUBZ: gm.JT_RZ, gm.JT_RUBU: gm.JT_RU}
    mr.jtypes = [to_rev.get(j, j) for j in mu.jtypes]
    assert mr.nv == mu.nv and mu.nq == mr.nq + sum(j in to_rev for j in mu.jtypes)
    ou, orv = OracleModel(mu), OracleModel(mr)
    qu, v, a = sm.random_inputs(mu, 16, 21)
    qr = np.zeros((16, mr.nq))
    for i in range(1, mu.njoints):
        iqu, iqr, n = mu.idx_qs[i], mr.idx_qs[i], mr.nqs[i]
        if mu.jtypes[i] in to_rev:
            qr[:, iqr] = np.arctan2(qu[:, iqu + 1], qu[:, iqu])
        else:
            qr[:, iqr : iqr + n] = qu[:, iqu : iqu + n]
    tau = orv.rnea(qr, v, a)
    assert rel_err(ou.rnea(qu, v, a), tau) < 1e-12
    for conv in (LOCAL, WORLD):
        assert rel_err(ou.aba(qu, v, tau, conv), orv.aba(qr, v, tau, conv)) < 1e-12
    assert rel_err(ou.crba(qu), orv.crba(qr)) < 1e-12
    for x, y in zip(ou.rnea_derivatives(qu, v, a), orv.rnea_derivatives(qr, v, a)):
        assert rel_err(x, y) < 1e-12
    for x, y in zip(ou.aba_derivatives(qu, v, tau), orv.aba_derivatives(qr, v, tau)):
        assert rel_err(x, y) < 1e-11
    # integrate: (cos, sin) turned by v and renormalised to first order
    qn = ou.integrate(qu, v)
    for ju, iqu, ivu in zip(mu.jtypes[1:], mu.idx_qs[1:], mu.idx_vs[1:]):
        if ju in to_rev:
            c, s_ = qu[:, iqu], qu[:, iqu + 1]
            cw, sw = np.cos(v[:, ivu]), np.sin(v[:, ivu])
            z = np.stack([cw * c - sw * s_, sw * c + cw * s_], axis=1)
            z *= ((3.0 - (z * z).sum(axis=1)) / 2.0)[:, None]
            assert np.allclose(qn[:, iqu : iqu + 2], z, rtol=0, atol=1e-15)


def test_batch_equals_serial():
    model = MODELS["humanoid32"]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 64, 3)
    tau_b = om.rnea(q, v, a, nthreads=4)
    ddq_b = om.aba(q, v, tau_b, WORLD, nthreads=4)
    for b in range(0, 64, 7):
        assert np.array_equal(om.rnea(q[b : b + 1], v[b : b + 1], a[b : b + 1], nthreads=1)[0], tau_b[b])
        assert np.array_equal(om.aba(q[b : b + 1], v[b : b + 1], tau_b[b : b + 1], WORLD, nthreads=1)[0], ddq_b[b])


def test_long_double_agrees():
    model = MODELS["humanoid32"]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 8, 4)
    tau = om.rnea(q, v, a)
    assert rel_err(om.rnea(q, v, a, prec=1), tau) < 1e-14
    assert rel_err(om.aba(q, v, tau, WORLD, prec=1), om.aba(q, v, tau, WORLD)) < 1e-12


# ---- analytic known answers --------------------------------------------------------------
def pendulum(m=2.0, L=0.7, Ixx=0.05):
    """One revolute joint about x, COM hanging at (0, 0, -L)."""
    model = gm.Model()
    j = model.addJoint(0, gm.JointModelRX(), gm.SE3.Identity(), "pivot")
    model.appendBodyToJoint(j, gm.Inertia(m, [0, 0, -L], np.diag([Ixx, 0.03, 0.04])))
    return model


def test_kat_pendulum():
    m, L, Ixx, g = 2.0, 0.7, 0.05, 9.81
    om = OracleModel(pendulum(m, L, Ixx))
    rng = np.random.default_rng(0)
    q = rng.uniform(-np.pi, np.pi, (32, 1))
    v = rng.standard_normal((32, 1))
    a = rng.standard_normal((32, 1))
    tau = (Ixx + m * L * L) * a + m * g * L * np.sin(q)
    assert rel_err(om.rnea(q, v, a), tau) < 1e-13
    assert rel_err(om.aba(q, v, tau), a) < 1e-13
    assert rel_err(symmetrize_upper(om.crba(q))[:, 0, 0][:, None], np.full((32, 1), Ixx + m * L * L)) < 1e-14


def cart_pole(M=1.5, m=0.4, L=0.6, I=(0.02, 0.03, 0.01)):
    """A cart sliding along x (prismatic) carrying a pendulum about y, COM at (0, 0, -L)."""
    model = gm.Model()
    cart = model.addJoint(0, gm.JointModelPX(), gm.SE3.Identity(), "cart")
    model.appendBodyToJoint(cart, gm.Inertia(M, [0, 0, 0], np.diag([0.1, 0.2, 0.3])))
    pole = model.addJoint(cart, gm.JointModelRY(), gm.SE3.Identity(), "pole")
    model.appendBodyToJoint(pole, gm.Inertia(m, [0, 0, -L], np.diag(I)))
    return model


def test_kat_cart_pole():
    """Lagrange's equations of the cart-pole: with x_c = x - L sin t, z_c = -L cos t,
    tau_x = (M+m) x'' - m L cos t t'' + m L sin t t'^2,
    tau_t = -m L cos t x'' + (m L^2 + Iyy) t'' + m g L sin t."""
    M, m, L, Iyy, g = 1.5, 0.4, 0.6, 0.03, 9.81
    om = OracleModel(cart_pole(M, m, L))
    rng = np.random.default_rng(3)
    q = np.stack([rng.uniform(-0.5, 0.5, 32), rng.uniform(-np.pi, np.pi, 32)], axis=1)
    v, a = rng.standard_normal((32, 2)), rng.standard_normal((32, 2))
    s, c = np.sin(q[:, 1]), np.cos(q[:, 1])
    tau = np.stack([(M + m) * a[:, 0] - m * L * c * a[:, 1] + m * L * s * v[:, 1] ** 2,
                    -m * L * c * a[:, 0] + (m * L * L + Iyy) * a[:, 1] + m * g * L * s], axis=1)
    assert rel_err(om.rnea(q, v, a), tau) < 1e-13
    assert rel_err(om.aba(q, v, tau), a) < 1e-12
    Mq = symmetrize_upper(om.crba(q))
    assert np.allclose(Mq[:, 0, 0], M + m, rtol=1e-14) and np.allclose(Mq[:, 1, 1], m * L * L + Iyy, rtol=1e-14)
    assert np.allclose(Mq[:, 0, 1], -m * L * c, rtol=1e-13, atol=1e-15)


def test_kat_prismatic_slide():
    """A body on a slide (no rotation): tau = m (a + 9.81 e_z . axis), the axis in the world."""
    rng = np.random.default_rng(4)
    for joint, k in ((gm.JointModelPZ(), 2), (gm.JointModelPX(), 0), (gm.JointModelPY(), 1)):
        model = gm.Model()
        R = sm.random_rotation(rng)
        j = model.addJoint(0, joint, gm.SE3(R, [0.1, -0.2, 0.3]), "slide")
        model.appendBodyToJoint(j, gm.Inertia(2.5, [0.05, 0.0, -0.1], np.diag([0.01, 0.02, 0.03])))
        q, v, a = (rng.standard_normal((8, 1)) for _ in range(3))
        tau = 2.5 * (a + 9.81 * R[2, k])
        assert rel_err(OracleModel(model).rnea(q, v, a), tau) < 1e-13


def _rebuild(model, joint_of):
    """The same tree with joint i replaced by joint_of(i, jtype)."""
    out = gm.Model()
    for i in range(1, model.njoints):
        out.addJoint(model.parents[i], joint_of(i, model.jtypes[i]), model.jointPlacements[i], model.names[i])
        out.inertias[i] = model.inertias[i]
    return out


def test_unaligned_joints_on_coordinate_axes():
    """A revolute / prismatic unaligned joint about +e_k is JointModelR{X,Y,Z} / P{X,Y,Z};
    about -e_k it is that joint with its coordinate negated."""
    model = MODELS["mixedtree12"]()
    rng = np.random.default_rng(5)
    q, v, a = sm.random_inputs(model, 16, 6)
    ref = OracleModel(model)
    axis_of = lambda jt: np.eye(3)[(jt - gm.JT_PX) if jt in gm.PRISMATIC else (jt - gm.JT_RX)]  # noqa: E731
    kind = lambda jt: gm.JointModelPrismaticUnaligned if jt in gm.PRISMATIC else gm.JointModelRevoluteUnaligned  # noqa: E731
    plus = OracleModel(_rebuild(model, lambda i, jt: kind(jt)(axis_of(jt))))
    assert rel_err(plus.rnea(q, v, a), ref.rnea(q, v, a)) < 1e-14
    assert rel_err(plus.aba(q, v, a), ref.aba(q, v, a)) < 1e-13
    D = np.where(rng.random(model.nv) < 0.5, -1.0, 1.0)  # flip a random subset of the joints
    flip = OracleModel(_rebuild(model, lambda i, jt: kind(jt)(D[model.idx_vs[i]] * axis_of(jt))))
    assert rel_err(flip.rnea(q * D, v * D, a * D), ref.rnea(q, v, a) * D) < 1e-13


def test_kat_tilted_pendulum():
    """A point mass m at distance L from an axis a tilted by b from the vertical (COM
    perpendicular to a, down-slope at q = 0): tau = m L^2 q'' + m g L sin(b) sin q."""
    m, L, b, g = 1.3, 0.8, 0.6, 9.81
    a = np.array([np.sin(b), 0.0, np.cos(b)])  # tilted about y
    c = L * np.array([np.cos(b), 0.0, -np.sin(b)])  # perpendicular to a, down-slope
    model = gm.Model()
    j = model.addJoint(0, gm.JointModelRevoluteUnaligned(a), gm.SE3.Identity(), "pivot")
    model.appendBodyToJoint(j, gm.Inertia(m, c, np.zeros((3, 3))))
    om = OracleModel(model)
    rng = np.random.default_rng(7)
    q, v, acc = rng.uniform(-np.pi, np.pi, (16, 1)), rng.standard_normal((16, 1)), rng.standard_normal((16, 1))
    tau = m * L * L * acc + m * g * L * np.sin(b) * np.sin(q)
    assert rel_err(om.rnea(q, v, acc), tau) < 1e-13
    assert rel_err(om.aba(q, v, tau), acc) < 1e-12


def free_body(m=3.0, I=(0.2, 0.3, 0.4)):
    model = gm.Model()
    j = model.addJoint(0, gm.JointModelFreeFlyer(), gm.SE3.Identity(), "base")
    model.appendBodyToJoint(j, gm.Inertia(m, [0, 0, 0], np.diag(I)))
    return model


def test_kat_free_body_newton_euler():
    m, I = 3.0, np.diag([0.2, 0.3, 0.4])
    model = free_body(m, np.diag(I))
    om = OracleModel(model)
    q, v, _ = sm.random_inputs(model, 32, 9)
    ddq = om.aba(q, v, np.zeros((32, 6)))
    g = np.array([0.0, 0.0, -9.81])
    for b in range(32):
        R = sm.quat_to_matrix(*q[b, 3:7])
        lin, w = v[b, :3], v[b, 3:]
        exp_lin = R.T @ g - np.cross(w, lin)
        exp_ang = np.linalg.solve(I, -np.cross(w, I @ w))
        assert np.allclose(ddq[b], np.concatenate([exp_lin, exp_ang]), rtol=1e-13, atol=1e-13)


def _act_motion(M, m6):
    """oMi.act(m) for M = (R row-major, t) (reference spatial/se3-tpl.hpp:265-280)."""
    R = M[..., :9].reshape(M.shape[:-1] + (3, 3))
    t = M[..., 9:]
    w = np.einsum("...ij,...j->...i", R, m6[..., 3:])
    lin = np.einsum("...ij,...j->...i", R, m6[..., :3]) + np.cross(t, w)
    return np.concatenate([lin, w], axis=-1)


def _support(model):
    """dofs of joint i and of its ancestors, per joint (the columns of data.J that move joint i)."""
    t = model.tables()
    parents = t["parents"]
    nvs = list(model.nvs)
    idx_v = np.concatenate([[0], np.cumsum(nvs)])[: len(parents)]
    out = []
    for i in range(len(parents)):
        dofs, j = [], i
        while j > 0:
            dofs += list(range(idx_v[j], idx_v[j] + nvs[j]))
            j = parents[j]
        out.append(sorted(dofs))
    return out


def test_forward_kinematics_and_jacobians_agree(case):
    """computeJointJacobians against forwardKinematics (unittest/jacobian.cpp:19-60:
    J v is the world-frame spatial velocity of each joint), joint 0 the identity,
    and the long-double oracle."""
    name, model, om, q, v, a = case
    oMi, vi, ai = om.forward_kinematics(q, v, a)
    J = om.joint_jacobians(q)  # (B, nv, 6)
    for i, dofs in enumerate(_support(model)):
        world = _act_motion(oMi[:, i], vi[:, i])
        Jv = np.einsum("bkr,bk->br", J[:, dofs], v[:, dofs]) if dofs else np.zeros_like(world)
        assert rel_err(Jv, world) < 1e-12, i
    assert np.array_equal(oMi[:, 0], np.tile(np.eye(3).reshape(-1).tolist() + [0, 0, 0], (len(q), 1)))
    assert not vi[:, 0].any() and not ai[:, 0].any()
    oMl, vl, al = om.forward_kinematics(q, v, a, prec=1)
    Jl = om.joint_jacobians(q, prec=1)
    for x, y in ((oMi, oMl), (vi, vl), (ai, al), (J, Jl)):
        assert rel_err(x, y) < 1e-12
    # placement-only and velocity-only calls fill the same placements / velocities
    o2, v2, a2 = om.forward_kinematics(q, v)
    assert np.array_equal(o2, oMi) and np.array_equal(v2, vi) and a2 is None
    assert np.array_equal(om.forward_kinematics(q)[0], oMi)


@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "tree12", "mixedtree24ff", "unaligned20ff",
                                  "translationtree14", "multidoftree16"])
def test_forward_kinematics_acceleration_vs_fd(name):
    """data.a[i] is the time derivative of the joint-frame velocity data.v[i]
    along (q + dt v, v + dt a): central differences, step 1e-6."""
    model = {**MODELS, **ORACLE_ONLY_MODELS}[name]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 4, 21)
    _, _, ai = om.forward_kinematics(q, v, a)
    h = 1e-6
    vp = om.forward_kinematics(om.integrate(q, h * v), v + h * a)[1]
    vm = om.forward_kinematics(om.integrate(q, -h * v), v - h * a)[1]
    assert rel_err((vp - vm) / (2 * h), ai) < 1e-6


def test_oracle_rollout_gradients_vs_central_differences():
    """The adjoint recursion of the oracle's rollout (the FP64 reference of the
    differentiable rollout) against central differences of its own forward rollout."""
    from oracle.oracle import rollout_with_gradients

    model = sm.chain(6, 2, (0.1, 1.0))
    om = OracleModel(model)
    rng = np.random.default_rng(9)
    B, T, n, dt = 2, 8, model.nv, 1e-2
    q0 = rng.uniform(-np.pi, np.pi, (B, n))
    v0 = 0.1 * rng.standard_normal((B, n))
    taus = rng.standard_normal((T, B, n))
    _, _, gq, gv, gt = rollout_with_gradients(om, q0, v0, taus, dt)

    def loss(q, v, t):
        qT = rollout_with_gradients(om, q, v, t, dt)[0]
        return float((qT**2).sum())

    h = 1e-6
    for which, (base, grad) in enumerate(((q0, gq), (v0, gv), (taus, gt))):
        for _ in range(5):
            idx = tuple(rng.integers(0, s) for s in base.shape)
            args_p, args_m = [q0, v0, taus], [q0, v0, taus]
            plus, minus = base.copy(), base.copy()
            plus[idx] += h
            minus[idx] -= h
            args_p[which], args_m[which] = plus, minus
            fd = (loss(*args_p) - loss(*args_m)) / (2 * h)
            assert abs(fd - grad[idx]) <= 1e-7 * max(1.0, abs(grad[idx])), (which, idx, fd, grad[idx])


def test_kat_spherical_euler_equations():
    """A body on a spherical joint with its centre of mass at the joint, no gravity: ABA gives
    Euler's equations, dw/dt = Ic^-1 (tau - w x Ic w) in the body frame, for any orientation."""
    rng = np.random.default_rng(3)
    model = gm.Model()
    model.gravity = np.zeros(6)
    j = model.addJoint(0, gm.JointModelSpherical(), gm.SE3(), "ball")
    A = rng.standard_normal((3, 3))
    Ic = A @ A.T + 3 * np.eye(3)
    model.appendBodyToJoint(j, gm.Inertia(2.0, np.zeros(3), Ic))
    om = OracleModel(model)
    q = sm.random_unit_quaternion(rng, 8)
    w = rng.standard_normal((8, 3))
    tau = rng.standard_normal((8, 3))
    ddq = om.aba(q, w, tau)
    ref = np.linalg.solve(Ic, (tau - np.cross(w, w @ Ic.T)).T).T
    assert rel_err(ddq, ref) < 1e-13
    assert rel_err(om.rnea(q, w, ddq), tau) < 1e-13
