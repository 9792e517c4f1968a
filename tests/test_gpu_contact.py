"""Contact dynamics on the GPU through the C ABI: gb_forward_dynamics and
gb_impulse_dynamics (reference algorithm/contact-dynamics.hxx:81-165, 255-327)
against the oracle on the same constraint Jacobians: FP64 at 1e-11 (the FP64
parity bar widened by the conditioning of J M^-1 J^T: the oracle's double and
long-double results already differ by up to ~1e-12 on these Jacobians) and mixed
precision (FP32 bias forces) at the mixed bar, with and without damping, without
constraint rows, in both array layouts."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from test_contact import feet_jacobian, leaf_joints
from util import FP64_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["humanoid32", "tree32ff", "mixedtree24ff", "unaligned20ff"])
def case(request):
    import torch

    model = MODELS[request.param]()
    om = OracleModel(model)
    B = 157
    q, v, x = sm.random_inputs(model, B, 51)
    if request.param == "humanoid32":
        J = feet_jacobian(model, om, q, leaf_joints(model))
    else:
        J = np.random.default_rng(52).normal(size=(B, 8, model.nv))
    gamma = np.random.default_rng(53).normal(size=(B, J.shape[1]))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return request.param, model, om, q, v, 10.0 * x, J, gamma, dev


FP64_CONTACT_TOL = 10 * FP64_TOL


def _tol(name, precision):
    return mixed_tol(name) if precision == "mixed" else FP64_CONTACT_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mu", [0.0, 1e-3])
def test_forward_dynamics(case, precision, mu):
    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model, precision)
    ddq = pg.forwardDynamics(model, data, dev(q), dev(v), dev(tau), dev(J), dev(gamma), mu).cpu().numpy()
    rd, rl = om.forward_dynamics(q, v, tau, J, gamma, inv_damping=mu)
    tol = _tol(name, precision)
    assert rel_err(ddq, rd) < tol
    assert rel_err(data.lambda_c.cpu().numpy(), rl) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_impulse_dynamics(case, precision):
    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model, precision)
    out = pg.impulseDynamics(model, data, dev(q), dev(v), dev(J), 0.3).cpu().numpy()
    ro, ri = om.impulse_dynamics(q, v, J, r_coeff=0.3)
    # the impulse path reads no bias forces: FP64 in both precisions
    assert rel_err(out, ro) < FP64_CONTACT_TOL
    assert rel_err(data.impulse_c.cpu().numpy(), ri) < FP64_CONTACT_TOL


def test_no_rows_shared_jacobian_and_soa(case):
    import torch

    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model)
    B, nv, nc = q.shape[0], model.nv, J.shape[1]
    # no constraint rows: the unconstrained dynamics
    d0 = pg.forwardDynamics(model, data, dev(q), dev(v), dev(tau), np.zeros((0, nv)), np.zeros(0)).cpu().numpy()
    assert rel_err(d0, om.aba(q, v, tau)) < FP64_CONTACT_TOL
    # one Jacobian shared by the batch
    d1 = pg.forwardDynamics(model, data, dev(q), dev(v), dev(tau), J[0], gamma[0]).cpu().numpy()
    r1 = om.forward_dynamics(q, v, tau, np.broadcast_to(J[:1], J.shape), np.broadcast_to(gamma[:1], gamma.shape))[0]
    assert rel_err(d1, r1) < FP64_CONTACT_TOL
    # value-major arrays give the instance-layout results bit for bit
    ref = pg.forwardDynamics(model, data, dev(q), dev(v), dev(tau), dev(J), dev(gamma))
    ref_l = data.lambda_c
    qs, vs, ts, Js, gs = (dev(np.ascontiguousarray(t.T)) for t in (q, v, tau, J.reshape(B, -1), gamma))
    out = torch.empty((nv, B), dtype=torch.float64, device="cuda")
    lam = torch.empty((nc, B), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(_capi.lib().gb_forward_dynamics(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, nc, p(qs), p(vs), p(ts),
                                                p(Js), p(gs), 0.0, p(out), p(lam), None))
    torch.cuda.synchronize()
    assert torch.equal(out.T, ref) and torch.equal(lam.T, ref_l)


def test_contact_arguments_are_checked(case):
    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model)
    B, nv, nc = q.shape[0], model.nv, J.shape[1]
    qd, vd, td, Jd, gd, out, lam = dev(q), dev(v), dev(tau), dev(J), dev(gamma), dev(np.zeros((B, nv))), dev(np.zeros((B, nc)))
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    L, h = _capi.lib(), data.dev.h
    args = (p(qd), p(vd), p(td), p(Jd), p(gd))
    assert L.gb_forward_dynamics(h, 0, 0, B, -1, *args, 0.0, p(out), p(lam), None) == _capi.GB_ERR_SIZE
    assert L.gb_forward_dynamics(h, 0, 0, B, nc, *args, -1.0, p(out), p(lam), None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_forward_dynamics(h, 0, 0, B, nc, p(qd), p(vd), p(td), None, p(gd), 0.0, p(out), p(lam), None) == \
        _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_impulse_dynamics(h, 0, 0, B, nc, p(qd), p(vd), p(Jd), 0.0, 0.0, p(out), None, None) == \
        _capi.GB_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("mu", [0.0, 1e-3])
def test_kkt_inverse(case, mu):
    """computeKKTContactDynamicMatrixInverse against the oracle's (contact-dynamics.hxx:166-225),
    at 1e-10: its blocks carry (J M^-1 J^T)^-1, whose conditioning widens the FP64 bar further"""
    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model)
    K = pg.computeKKTContactDynamicMatrixInverse(model, data, dev(q), dev(J), mu).cpu().numpy()
    assert rel_err(K, om.kkt_inverse(q, J, mu)) < 1e-10


def test_kkt_inverse_soa_layout_and_no_constraint_rows(case):
    """The value-major (SOA) indexing of J and of the KKT inverse gives the bits of the
    instance layout; with nc == 0 (J may be NULL) the inverse is M^-1 itself, which
    computeMinverse also returns."""
    import torch

    name, model, om, q, v, tau, J, gamma, dev = case
    data = pg.createData(model)
    B, nv, nc = q.shape[0], model.nv, J.shape[1]
    n = nv + nc
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    L, h = _capi.lib(), data.dev.h
    qd, Jd = dev(q), dev(J)
    K_inst = torch.empty((B, n, n), dtype=torch.float64, device="cuda")
    _capi.check(L.gb_kkt_contact_inverse(h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, B, nc, p(qd), p(Jd), 1e-3,
                                         p(K_inst), None))
    qs, Js = dev(q.T), dev(J.reshape(B, -1).T)
    K_soa = torch.empty((n * n, B), dtype=torch.float64, device="cuda")
    _capi.check(L.gb_kkt_contact_inverse(h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, nc, p(qs), p(Js), 1e-3,
                                         p(K_soa), None))
    torch.cuda.synchronize()
    assert torch.equal(K_soa.T.reshape(B, n, n), K_inst)
    K0 = torch.empty((B, nv, nv), dtype=torch.float64, device="cuda")
    _capi.check(L.gb_kkt_contact_inverse(h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, B, 0, p(qd), None, 0.0, p(K0),
                                         None))
    Minv = pg.computeMinverse(model, data, qd)
    torch.cuda.synchronize()
    assert rel_err(K0.cpu().numpy(), Minv.cpu().numpy()) < 1e-12
    _, _, _, Minv_o = om.aba_derivatives(q, v, tau)
    assert rel_err(K0.cpu().numpy(), Minv_o) < 1e-11
