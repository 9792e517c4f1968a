"""Mimic joints on the GPU against the oracle (the reference's recipe over the full model,
unittest/rnea.cpp:350-420 and unittest/crba.cpp:131-170): rnea, nonLinearEffects,
computeGeneralizedGravity, computeStaticTorque, crba (both output modes), forwardKinematics,
computeJointJacobians (6 x nvExtended), integrate and rneaInParallel; both layouts and both
precisions; the functions the reference does not take mimic joints in are refused."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import MimicOracleModel
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, rel_err

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-4  # a random tree like the joint-type models


@pytest.fixture(scope="module")
def case():
    import torch

    model = sm.mimic_tree()
    q, v, x = sm.random_inputs(model, 300, 17)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return model, MimicOracleModel(model), q, v, x, dev


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rnea_family(case, precision):
    model, om, q, v, x, dev = case
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    data = pg.createData(model, precision)
    zero = np.zeros_like(v)
    assert rel_err(pg.rnea(model, data, dev(q), dev(v), dev(x)).cpu().numpy(), om.rnea(q, v, x)) < tol
    assert rel_err(pg.nonLinearEffects(model, data, dev(q), dev(v)).cpu().numpy(), om.rnea(q, v, zero)) < tol
    assert rel_err(pg.computeGeneralizedGravity(model, data, dev(q)).cpu().numpy(), om.rnea(q, zero, zero)) < tol
    fext = np.random.default_rng(3).standard_normal((q.shape[0], model.njoints, 6))
    st = pg.computeStaticTorque(model, data, dev(q), dev(fext)).cpu().numpy()
    assert rel_err(st, om.rnea(q, zero, zero, fext=fext)) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_crba(case, precision):
    model, om, q, v, x, dev = case
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    data = pg.createData(model, precision)
    Mref = om.crba(q)
    M = pg.crba(model, data, dev(q)).cpu().numpy()
    assert M.shape == (q.shape[0], model.nv, model.nv) and rel_err(M, Mref) < tol
    Mu = pg.crba(model, data, dev(q), symmetric=False).cpu().numpy()
    assert np.all(np.tril(Mu, -1) == 0.0) and rel_err(Mu, np.triu(Mref)) < tol
    # the equation of motion of the reduced model: M a + nle = rnea
    tau = pg.rnea(model, data, dev(q), dev(v), dev(x)).cpu().numpy()
    nle = pg.nonLinearEffects(model, data, dev(q), dev(v)).cpu().numpy()
    assert rel_err(np.einsum("bij,bj->bi", M, x) + nle, tau) < (1e-11 if precision == "fp64" else 1e-4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_kinematics(case, precision):
    model, om, q, v, x, dev = case
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    data = pg.createData(model, precision)
    outs = [t.cpu().numpy() for t in pg.forwardKinematics(model, data, dev(q), dev(v), dev(x))]
    for o, r in zip(outs, om.forward_kinematics(q, v, x)):
        assert rel_err(o, r) < tol
    J = pg.computeJointJacobians(model, data, dev(q)).cpu().numpy()
    assert J.shape == (q.shape[0], 6, model.nvExtended)
    assert rel_err(J, np.swapaxes(om.joint_jacobians(q), 1, 2)) < tol


def test_integrate(case):
    model, om, q, v, x, dev = case
    out = pg.integrate(model, dev(q), dev(0.1 * v)).cpu().numpy()
    assert rel_err(out, om.integrate(q, 0.1 * v)) < 1e-15


def test_soa_layout_and_in_parallel(case):
    import torch

    model, om, q, v, x, dev = case
    data = pg.createData(model)
    B = q.shape[0]
    qs, vs, xs = (dev(np.ascontiguousarray(t.T)) for t in (q, v, x))
    tau = torch.empty((model.nv, B), dtype=torch.float64, device="cuda")
    M = torch.empty((model.nv * model.nv, B), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    L = _capi.lib()
    _capi.check(L.gb_rnea(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(xs), p(tau), None))
    _capi.check(L.gb_crba(data.dev.h, _capi.GB_FP64, _capi.GB_LOCAL, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_SOA, B,
                          p(qs), p(M), None, None, None))
    torch.cuda.synchronize()
    assert rel_err(tau.cpu().numpy().T, om.rnea(q, v, x)) < FP64_TOL
    assert rel_err(M.cpu().numpy().T.reshape(B, model.nv, model.nv), om.crba(q)) < FP64_TOL
    pool = pg.ModelPool(model, 4)  # the reference's nq x batch / nv x batch matrices
    out = np.asarray(pg.rneaInParallel(4, pool, q.T, v.T, x.T))
    assert out.shape == (model.nv, B) and rel_err(out.T, om.rnea(q, v, x)) < FP64_TOL


def test_functions_without_mimic_support_are_refused(case):
    """ABA, the derivatives, the Cholesky, Minv and the contact functions refuse mimic joints, as
    the reference's MimicChecker does (aba.hxx:250, rnea-derivatives.hxx:157, cholesky.hxx:37)."""
    model, om, q, v, x, dev = case
    data = pg.createData(model)
    for call in (
        lambda: pg.aba(model, data, dev(q), dev(v), dev(x)),
        lambda: pg.computeABADerivatives(model, data, dev(q), dev(v), dev(x)),
        lambda: pg.computeRNEADerivatives(model, data, dev(q), dev(v), dev(x)),
        lambda: pg.computeMinverse(model, data, dev(q)),
    ):
        with pytest.raises(Exception, match="mimic"):
            call()
    L = _capi.lib()
    U = np.empty((2, model.nv, model.nv))
    D = np.empty((2, model.nv))
    qq = np.ascontiguousarray(q[:2])
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = L.gb_crba(data.dev.h, _capi.GB_FP64, _capi.GB_LOCAL, _capi.GB_MATRIX_UPPER, _capi.GB_LAYOUT_INSTANCE, 2, p(qq),
                   p(U), p(U), p(D), None)
    assert rc == _capi.GB_ERR_UNSUPPORTED
    h = C.c_void_p()
    assert L.gb_constraint_set_create(data.dev.h, 0, None, C.byref(h)) == _capi.GB_ERR_UNSUPPORTED
    nve = C.c_int()
    _capi.check(L.gb_model_nv_extended(data.dev.h, C.byref(nve)))
    assert nve.value == model.nvExtended


def test_mimic_with_expanded_joints():
    """Mimic joints in a tree whose spherical ZYX and translation joints the model builder expands
    into chains: the maps from the caller's q and v to the extended tree skip the expanded joints'
    internal links (rnea, crba and the kinematics against the oracle)."""
    import torch

    rng = np.random.default_rng(12)
    m = pg.Model()
    a = m.addJoint(0, pg.JointModelSphericalZYX(), sm.random_placement(rng), "a")
    m.appendBodyToJoint(a, sm.random_inertia(rng))
    b = m.addJoint(a, pg.JointModelRZ(), sm.random_placement(rng), "b")
    m.appendBodyToJoint(b, sm.random_inertia(rng))
    c = m.addJoint(b, pg.JointModelTranslation(), sm.random_placement(rng), "c")
    m.appendBodyToJoint(c, sm.random_inertia(rng))
    d = m.addJoint(c, pg.JointModelMimic(pg.JointModelPY(), b, -0.7, 0.2), sm.random_placement(rng), "d")
    m.appendBodyToJoint(d, sm.random_inertia(rng))
    e = m.addJoint(d, pg.JointModelSphericalZYX(), sm.random_placement(rng), "e")
    m.appendBodyToJoint(e, sm.random_inertia(rng))
    assert (m.nq, m.nv, m.nvExtended) == (10, 10, 11)
    om = MimicOracleModel(m)
    q, v, x = sm.random_inputs(m, 64, 5)
    dev = lambda t: torch.from_numpy(np.ascontiguousarray(t)).cuda()  # noqa: E731
    data = pg.createData(m)
    assert rel_err(pg.rnea(m, data, dev(q), dev(v), dev(x)).cpu().numpy(), om.rnea(q, v, x)) < FP64_TOL
    assert rel_err(pg.crba(m, data, dev(q)).cpu().numpy(), om.crba(q)) < FP64_TOL
    outs = [t.cpu().numpy() for t in pg.forwardKinematics(m, data, dev(q), dev(v), dev(x))]
    for o, r in zip(outs, om.forward_kinematics(q, v, x)):
        assert rel_err(o, r) < FP64_TOL
    J = pg.computeJointJacobians(m, data, dev(q)).cpu().numpy()
    assert rel_err(J, np.swapaxes(om.joint_jacobians(q), 1, 2)) < FP64_TOL
    assert rel_err(pg.integrate(m, dev(q), dev(0.1 * v)).cpu().numpy(), om.integrate(q, 0.1 * v)) < 1e-15
