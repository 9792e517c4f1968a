"""The neighbours of the path through the C ABI:
computeMinverse (reference algorithm/aba.hxx:838-880) against the oracle's
Minv and M^-1, nonLinearEffects and computeGeneralizedGravity (rnea.hxx:221-446)
against the oracle's RNEA with zero acceleration / zero velocity,
forwardKinematics (kinematics.hxx:42-272) and computeJointJacobians
(jacobian.hxx:17-95) against the oracle's; FP64 at 1e-12 and mixed precision
at 1e-5, both output modes, both layouts."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import LOCAL, OracleModel, symmetrize_upper
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu
MIXED_MODELS = list(MODELS)  # the 100-link chain included: its mixed derivative sweeps run in double-float


@pytest.fixture(scope="module", params=list(MODELS))
def case(request):
    import torch

    model = MODELS[request.param]()
    q, v, x = sm.random_inputs(model, 301, 77)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return request.param, model, OracleModel(model), q, v, x, dev


def _tol(name, precision):
    if precision == "mixed":
        return mixed_tol(name)
    return 1e-10 if name == "chain100" else FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compute_minverse(case, precision):
    name, model, om, q, v, x, dev = case
    if precision == "mixed" and name not in MIXED_MODELS:
        pytest.skip("the mixed-precision bar applies to the benchmark models")
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    Mi = pg.computeMinverse(model, data, dev(q)).cpu().numpy()
    _, _, _, Mref = om.aba_derivatives(q, v, 10.0 * x)
    assert rel_err(Mi, Mref) < tol
    Mi_up = pg.computeMinverse(model, data, dev(q), symmetric=False).cpu().numpy()
    assert rel_err(Mi_up, np.triu(Mref)) < tol
    assert np.all(np.tril(Mi_up, -1) == 0.0)
    if precision == "fp64":  # Minv M = I (unittest/aba-derivatives.cpp:96-100)
        M = symmetrize_upper(om.crba(q, LOCAL))
        eye = np.broadcast_to(np.eye(model.nv), M.shape)
        assert np.abs(np.einsum("bij,bjk->bik", Mi, M) - eye).max() < (1e-8 if name == "chain100" else 1e-11)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonlinear_effects_and_gravity(case, precision):
    name, model, om, q, v, x, dev = case
    tol = _tol(name, precision)
    if precision == "mixed":
        tol = 1e-5
    data = pg.createData(model, precision)
    nle = pg.nonLinearEffects(model, data, dev(q), dev(v)).cpu().numpy()
    g = pg.computeGeneralizedGravity(model, data, dev(q)).cpu().numpy()
    zero = np.zeros_like(v)
    assert rel_err(nle, om.rnea(q, v, zero)) < tol
    assert rel_err(g, om.rnea(q, zero, zero)) < tol


def test_soa_layout_minverse_and_gravity():
    import torch

    model = sm.humanoid32(1)
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 77, 3)
    data = pg.createData(model)
    B, nv = q.shape[0], model.nv
    qs = torch.from_numpy(np.ascontiguousarray(q.T)).cuda()  # SoA: element-major
    Mi = torch.empty((nv * nv, B), dtype=torch.float64, device="cuda")
    g = torch.empty((nv, B), dtype=torch.float64, device="cuda")
    L = _capi.lib()
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(L.gb_compute_minverse(data.dev.h, _capi.GB_FP64, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_SOA, B, P(qs), P(Mi), None))
    _capi.check(L.gb_generalized_gravity(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, P(qs), P(g), None))
    torch.cuda.synchronize()
    _, _, _, Mref = om.aba_derivatives(q, v, x)
    assert rel_err(Mi.cpu().numpy().T.reshape(B, nv, nv), Mref) < FP64_TOL
    assert rel_err(g.cpu().numpy().T, om.rnea(q, np.zeros_like(v), np.zeros_like(v))) < FP64_TOL


def test_empty_batch_and_errors():
    model = sm.manipulator6r(0)
    data = pg.createData(model)
    L = _capi.lib()
    assert L.gb_compute_minverse(data.dev.h, _capi.GB_FP64, _capi.GB_MATRIX_UPPER, _capi.GB_LAYOUT_INSTANCE, 0, None, None, None) == 0
    assert L.gb_compute_minverse(data.dev.h, _capi.GB_FP64, 7, _capi.GB_LAYOUT_INSTANCE, 1, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_nonlinear_effects(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, 3, None, None, None, None) == _capi.GB_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_forward_kinematics(case, precision):
    """forwardKinematics (reference algorithm/kinematics.hxx:42-272): placements,
    joint-frame velocities and accelerations against the oracle; the q-only and
    (q, v) forms; the SOA layout gives the same bits."""
    import torch

    name, model, om, q, v, x, dev = case
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    oMi, vi, ai = (t.cpu().numpy() for t in pg.forwardKinematics(model, data, dev(q), dev(v), dev(x)))
    o_r, v_r, a_r = om.forward_kinematics(q, v, x)
    assert rel_err(oMi, o_r) < tol
    assert rel_err(vi, v_r) < tol
    assert rel_err(ai, a_r) < tol
    o2, v2, a2 = pg.forwardKinematics(model, data, dev(q), dev(v))
    assert np.array_equal(o2.cpu().numpy(), oMi) and np.array_equal(v2.cpu().numpy(), vi) and a2 is None
    o3, v3, a3 = pg.forwardKinematics(model, data, dev(q))
    assert np.array_equal(o3.cpu().numpy(), oMi) and v3 is None and a3 is None
    B, nj = q.shape[0], model.njoints
    outs = [torch.empty((n, B), dtype=torch.float64, device="cuda") for n in (12 * nj, 6 * nj, 6 * nj)]
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    qs, vs, xs = (dev(np.ascontiguousarray(t.T)) for t in (q, v, x))
    _capi.check(
        _capi.lib().gb_forward_kinematics(data.dev.h, _capi.GB_FP64 if precision == "fp64" else _capi.GB_MIXED,
                                          _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(xs), p(outs[0]), p(outs[1]),
                                          p(outs[2]), None)
    )
    torch.cuda.synchronize()
    for o, r in zip(outs, (oMi, vi, ai)):
        assert np.array_equal(o.cpu().numpy().T.reshape(r.shape), r)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compute_joint_jacobians(case, precision):
    """computeJointJacobians (reference algorithm/jacobian.hxx:17-95) against the
    oracle; J v equals the world-frame velocity of the last joint."""
    name, model, om, q, v, x, dev = case
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    J = pg.computeJointJacobians(model, data, dev(q)).cpu().numpy()  # (B, 6, nv)
    assert J.shape == (q.shape[0], 6, model.nv)
    assert rel_err(J, np.swapaxes(om.joint_jacobians(q), 1, 2)) < tol


def test_forward_kinematics_errors():
    model = MODELS["manipulator6r"]()
    data = pg.createData(model)
    L = _capi.lib()
    z = np.zeros((2, 12 * model.njoints))
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    q = np.zeros((2, model.nq))
    # an acceleration without a velocity, an output without its input
    assert L.gb_forward_kinematics(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, 2, p(q), None, p(q), p(z), None,
                                   None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_forward_kinematics(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, 2, p(q), None, None, p(z), p(z),
                                   None, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_forward_kinematics(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, 0, None, None, None, None, None,
                                   None, None) == _capi.GB_OK


def test_translation_joints_keep_the_callers_joint_indexing():
    """A translation joint runs as three prismatic joints inside the kernels; the C ABI still
    reports the caller's joints, and forwardKinematics writes one placement per caller joint
    (the oracle computes the translation joint natively)."""
    import ctypes as C

    from pinocchio_gb300 import _capi

    model = sm.translation_tree(9)
    data = pg.createData(model)
    nq, nv, nj = C.c_int(), C.c_int(), C.c_int()
    _capi.check(_capi.lib().gb_model_dims(data.dev.h, C.byref(nq), C.byref(nv), C.byref(nj)))
    assert (nq.value, nv.value, nj.value) == (model.nq, model.nv, model.njoints)
    q, v, a = sm.random_inputs(model, 33, 4)
    oMi, vi, ai = pg.forwardKinematics(model, data, q, v, a)  # numpy in, numpy out
    oMo, vo, ao = OracleModel(model).forward_kinematics(q, v, a)
    assert oMi.shape == oMo.shape
    assert rel_err(oMi, oMo) < FP64_TOL and rel_err(vi, vo) < FP64_TOL and rel_err(ai, ao) < FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_spherical_zyx_reference_known_answers(precision):
    """One spherical ZYX joint (three revolute joints inside the kernels) with a unit mass at (0.5,
    0, 0) and unit rotational inertia: rnea, crba and aba (M^-1 (tau - nle)) at the reference's own
    known answers (unittest/joint-spherical.cpp:215-300); the C ABI reports the caller's joint."""
    m = pg.Model()
    j = m.addJoint(0, pg.JointModelSphericalZYX(), pg.SE3.Identity(), "root")
    m.appendBodyToJoint(j, pg.Inertia(1.0, [0.5, 0.0, 0.0], np.eye(3)))
    data = pg.createData(m, precision)
    nq, nv, nj = C.c_int(), C.c_int(), C.c_int()
    _capi.check(_capi.lib().gb_model_dims(data.dev.h, C.byref(nq), C.byref(nv), C.byref(nj)))
    assert (nq.value, nv.value, nj.value) == (3, 3, 2)
    qs = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [3.0, 2.0, 1.0]])
    va = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [1.0, 1.0, 1.0]])
    tol = 1e-12 if precision == "fp64" else 1e-5
    tau = np.asarray(pg.rnea(m, data, qs, va, va))
    expected = np.array([[0.0, -4.905, 0.0],
                         [-0.53611600195085, -0.74621832606188, -0.38177329067604],
                         [0.73934458094049, 2.7804530848031, 0.50684940972146]])
    assert np.allclose(tau, expected, rtol=0, atol=tol * 10)
    M = np.asarray(pg.crba(m, data, qs))
    Mexp = np.array([[[1.25, 0, 0], [0, 1.25, 0], [0, 0, 1.0]],
                     [[1.0729816454316, 0, -0.8414709848079], [0, 1.25, 0], [-0.8414709848079, 0, 1.0]],
                     [[1.043294547392, 0, -0.90929742682568], [0, 1.25, 0], [-0.90929742682568, 0, 1.0]]])
    assert np.allclose(M, Mexp, rtol=0, atol=tol * 10)
    ddq = np.asarray(pg.aba(m, data, qs, va, expected))
    assert np.allclose(ddq, va, rtol=0, atol=tol * 100)
