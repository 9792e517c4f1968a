"""Spherical ZYX joints (reference JointModelSphericalZYX, multibody/joint/joint-spherical-ZYX.hpp) on
the CPU: the oracle, which runs the joint as a chain of revolute joints about z, y and x (like the
library), against the reference's own known answers (unittest/joint-spherical.cpp:215-300) and
against a direct Newton-Euler step with the joint's closed-form transform, motion subspace S(q)
and bias c (joint-spherical-ZYX.hpp:440-470); the model's sizes, integrate and external forces.
The library's kernels run the ZYX tree on the host in test_hostsim.py and on the GPU in the tests
over util.MODELS and test_gpu_next.py."""
import numpy as np

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel, expand_spherical_zyx, symmetrize_upper
from pinocchio_gb300 import sample_models as sm
from util import rel_err


def single_joint_model(placement=None, inertia=None):
    m = pg.Model()
    j = m.addJoint(0, pg.JointModelSphericalZYX(), placement or pg.SE3.Identity(), "root")
    m.appendBodyToJoint(j, inertia or pg.Inertia(1.0, [0.5, 0.0, 0.0], np.eye(3)))
    return m


def test_reference_known_answers():
    """rnea and crba of one ZYX joint with a unit mass at (0.5, 0, 0) and unit rotational inertia
    under the default gravity: the values of the reference's unit tests."""
    om = OracleModel(single_joint_model())
    qs = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [3.0, 2.0, 1.0]])
    va = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [1.0, 1.0, 1.0]])
    tau = om.rnea(qs, va, va)
    expected = np.array([[0.0, -4.905, 0.0],
                         [-0.53611600195085, -0.74621832606188, -0.38177329067604],
                         [0.73934458094049, 2.7804530848031, 0.50684940972146]])
    assert np.allclose(tau, expected, rtol=0, atol=1e-12)
    M = symmetrize_upper(om.crba(qs))
    Mexp = np.array([[[1.25, 0, 0], [0, 1.25, 0], [0, 0, 1.0]],
                     [[1.0729816454316, 0, -0.8414709848079], [0, 1.25, 0], [-0.8414709848079, 0, 1.0]],
                     [[1.043294547392, 0, -0.90929742682568], [0, 1.25, 0], [-0.90929742682568, 0, 1.0]]])
    assert np.allclose(M, Mexp, rtol=0, atol=1e-12)


def _zyx(q):
    """R, the angular part of S and the bias c's angular part at (q, qd) as the reference writes them."""
    s0, c0 = np.sin(q[0]), np.cos(q[0])
    s1, c1 = np.sin(q[1]), np.cos(q[1])
    s2, c2 = np.sin(q[2]), np.cos(q[2])
    R = np.array([[c0 * c1, c0 * s1 * s2 - s0 * c2, c0 * s1 * c2 + s0 * s2],
                  [s0 * c1, s0 * s1 * s2 + c0 * c2, s0 * s1 * c2 - c0 * s2],
                  [-s1, c1 * s2, c1 * c2]])
    S = np.array([[-s1, 0.0, 1.0], [c1 * s2, c2, 0.0], [c1 * c2, -s2, 0.0]])

    def bias(qd):
        return np.array([-c1 * qd[0] * qd[1],
                         -s1 * s2 * qd[0] * qd[1] + c1 * c2 * qd[0] * qd[2] - s2 * qd[1] * qd[2],
                         -s1 * c2 * qd[0] * qd[1] - c1 * s2 * qd[0] * qd[2] - c2 * qd[1] * qd[2]])
    return R, S, bias


def test_chain_against_the_closed_form_joint():
    """One ZYX joint at a random placement carrying a random body: the oracle's rnea, forward
    kinematics (placement, velocity, acceleration) and joint Jacobian against a Newton-Euler step
    written with the joint's own R, S(q) and c."""
    rng = np.random.default_rng(21)
    P, Y = sm.random_placement(rng), sm.random_inertia(rng)
    om = OracleModel(single_joint_model(P, Y))
    B = 12
    q = rng.uniform(-np.pi, np.pi, (B, 3))
    q[:, 1] = rng.uniform(-1.2, 1.2, B)
    qd, qdd = rng.standard_normal((B, 3)), rng.standard_normal((B, 3))
    tau = om.rnea(q, qd, qdd)
    oMi, vi, ai = om.forward_kinematics(q, qd, qdd)
    J = om.joint_jacobians(q)
    m, c, Ic = Y.mass, Y.lever, Y.matrix3()
    g = np.array([0.0, 0.0, -9.81])
    for b in range(B):
        R, S, bias = _zyx(q[b])
        Rw = P.rotation @ R
        w = S @ qd[b]
        dw = S @ qdd[b] + bias(qd[b])
        assert np.allclose(oMi[b, 1, :9].reshape(3, 3), Rw, atol=1e-13)
        assert np.allclose(oMi[b, 1, 9:], P.translation, atol=1e-13)
        assert np.allclose(vi[b, 1], np.r_[np.zeros(3), w], atol=1e-13)
        assert np.allclose(ai[b, 1], np.r_[np.zeros(3), dw], atol=1e-12)
        # the body's acceleration with gravity (linear part Rw^T (-g)), its momentum rate
        lin, ang = Rw.T @ (-g), dw
        f_lin = m * (lin - np.cross(c, ang))
        f_ang = Ic @ ang + np.cross(c, f_lin)
        h_lin = m * (-np.cross(c, w))
        h_ang = Ic @ w + np.cross(c, h_lin)
        f_lin, f_ang = f_lin + np.cross(w, h_lin), f_ang + np.cross(w, h_ang)
        assert np.allclose(tau[b], S.T @ f_ang, rtol=0, atol=1e-11)
        ang_cols = Rw @ S
        assert np.allclose(J[b][:, 3:], ang_cols.T, atol=1e-13)
        assert np.allclose(J[b][:, :3], np.cross(P.translation, ang_cols.T), atol=1e-13)


def test_sizes_integrate_and_tables():
    model = sm.zyx_tree()
    assert (model.nq, model.nv, model.njoints) == (16, 16, 9)
    assert np.all(model.neutral() == 0.0)
    t, rows = expand_spherical_zyx(model.tables())
    assert len(t["parents"]) == 9 + 2 * 3 and rows[-1] == len(t["parents"]) - 1
    om = OracleModel(model)
    q, v, _ = sm.random_inputs(model, 8, 3)
    assert rel_err(om.integrate(q, v), q + v) < 1e-15  # a vector space
    # fext on the caller's joints reaches the same bodies: a force on the last joint is the
    # Jacobian transpose's torque
    fext = np.zeros((8, model.njoints, 6))
    fext[:, 3] = np.random.default_rng(4).standard_normal((8, 6))
    zero = np.zeros_like(v)
    dtau = om.rnea(q, zero, zero) - om.rnea(q, zero, zero, fext=fext)
    oMi, _, _ = om.forward_kinematics(q)
    J = om.joint_jacobians(q)
    for b in range(8):
        R = oMi[b, 3, :9].reshape(3, 3)
        p = oMi[b, 3, 9:]
        fl, fa = R @ fext[b, 3, :3], R @ fext[b, 3, 3:]
        fw = np.r_[fl, fa + np.cross(p, fl)]  # the force in world axes about the origin
        sub = [k for k in range(model.nv) if k < model.idx_vs[4]]  # joint 3's support
        assert np.allclose(dtau[b, sub], J[b][sub] @ fw, atol=1e-10)

