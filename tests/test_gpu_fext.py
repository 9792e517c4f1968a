"""External forces on the GPU through the C ABI: gb_rnea_fext, gb_static_torque,
gb_aba_fext, gb_rnea_derivatives_fext and gb_aba_derivatives_fext (the reference's
fext overloads, algorithm/rnea.hxx:164-218 and 448-489, aba.hxx:296-352 and
543-605, rnea-derivatives.hxx:550-633, aba-derivatives.hxx:463-541) against the
oracle with the same forces: FP64 at 1e-12 and mixed precision at the mixed bar,
on trees with free-flyer, prismatic and unaligned joints (whose forces the
kernels turn into the folded joint frame), in both array layouts."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import LOCAL, WORLD, OracleModel, symmetrize_upper
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from test_fext import random_fext
from util import FP64_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu
GPU_FEXT_MODELS = ["manipulator6r", "humanoid32", "tree32ff", "mixedtree24ff", "unaligned14", "unaligned20ff",
                   "translationtree14"]


@pytest.fixture(scope="module", params=GPU_FEXT_MODELS)
def case(request):
    import torch

    model = MODELS[request.param]()
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 203, 91)
    fext = random_fext(om.njoints, 203, 92)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return request.param, model, om, q, v, x, fext, dev


def _tol(name, precision):
    return mixed_tol(name) if precision == "mixed" else FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rnea_and_static_torque_with_fext(case, precision):
    name, model, om, q, v, a, fext, dev = case
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    tau = pg.rnea(model, data, dev(q), dev(v), dev(a), dev(fext)).cpu().numpy()
    assert rel_err(tau, om.rnea(q, v, a, fext=fext)) < tol
    z = np.zeros_like(v)
    st = pg.computeStaticTorque(model, data, dev(q), dev(fext)).cpu().numpy()
    assert rel_err(st, om.rnea(q, z, z, fext=fext)) < tol
    # one set of forces shared by the batch, as a list of njoints 6-vectors
    shared = [fext[0, i] for i in range(om.njoints)]
    tau_s = pg.rnea(model, data, dev(q), dev(v), dev(a), shared).cpu().numpy()
    assert rel_err(tau_s, om.rnea(q, v, a, fext=np.broadcast_to(fext[:1], fext.shape))) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aba_with_fext(case, precision):
    name, model, om, q, v, x, fext, dev = case
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    tau = 10.0 * x
    ref = om.aba(q, v, tau, fext=fext)
    for conv in (LOCAL, WORLD):
        ddq = pg.aba(model, data, dev(q), dev(v), dev(tau), dev(fext), conv).cpu().numpy()
        assert rel_err(ddq, ref) < tol
    if precision == "fp64":  # aba(rnea(a, fext), fext) = a (unittest/aba.cpp:186-222)
        t2 = om.rnea(q, v, x, fext=fext)
        assert rel_err(pg.aba(model, data, dev(q), dev(v), dev(t2), fext=dev(fext)).cpu().numpy(), x) < 1e-11


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_derivatives_with_fext(case, precision):
    name, model, om, q, v, x, fext, dev = case
    tol = _tol(name, precision)
    data = pg.createData(model, precision)
    rt, rq, rv, rM = om.rnea_derivatives(q, v, x, fext=fext)
    dq, dv, M = (t.cpu().numpy() for t in pg.computeRNEADerivatives(model, data, dev(q), dev(v), dev(x), dev(fext)))
    assert rel_err(dq, rq) < tol and rel_err(dv, rv) < tol and rel_err(M, symmetrize_upper(rM)) < tol
    assert rel_err(data.tau.cpu().numpy(), rt) < tol
    tau = 10.0 * x
    ref = om.aba_derivatives(q, v, tau, fext=fext)
    out = pg.computeABADerivatives(model, data, dev(q), dev(v), dev(tau), dev(fext))
    for got, r in zip((data.ddq,) + tuple(out), ref):
        assert rel_err(got.cpu().numpy(), r) < tol


def test_soa_layout_with_fext(case):
    """value-major arrays (stride batch) give the instance-layout results bit for bit"""
    import torch

    name, model, om, q, v, x, fext, dev = case
    data = pg.createData(model)
    B, nv = q.shape[0], model.nv
    tau = 10.0 * x
    # the value-major copies stay referenced until the kernels have run
    qs, vs, xs, ts, fs = (dev(np.ascontiguousarray(t.T)) for t in (q, v, x, tau, fext.reshape(B, -1)))
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    ref_tau = pg.rnea(model, data, dev(q), dev(v), dev(x), dev(fext))
    out = torch.empty((nv, B), dtype=torch.float64, device="cuda")
    _capi.check(_capi.lib().gb_rnea_fext(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(xs), p(fs),
                                         p(out), None))
    torch.cuda.synchronize()
    assert torch.equal(out.T, ref_tau)
    ref = pg.computeABADerivatives(model, data, dev(q), dev(v), dev(tau), dev(fext))
    mats = [torch.empty((nv * nv, B), dtype=torch.float64, device="cuda") for _ in range(3)]
    ddq = torch.empty((nv, B), dtype=torch.float64, device="cuda")
    _capi.check(_capi.lib().gb_aba_derivatives_fext(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, p(qs), p(vs),
                                                    p(ts), p(fs), *(p(m) for m in mats), p(ddq), None))
    torch.cuda.synchronize()
    for m, r in zip(mats, ref):
        assert torch.equal(m.T.reshape(B, nv, nv), r)
    assert torch.equal(ddq.T, data.ddq)


def test_fext_arguments_are_checked(case):
    name, model, om, q, v, x, fext, dev = case
    data = pg.createData(model)
    with pytest.raises(ValueError):
        pg.rnea(model, data, dev(q), dev(v), dev(x), dev(fext[:, 1:]))
    B = q.shape[0]
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    out = dev(np.zeros((B, model.nv)))
    qd, vd, xd = dev(q), dev(v), dev(x)
    rc = _capi.lib().gb_rnea_fext(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_INSTANCE, B, p(qd), p(vd), p(xd), None,
                                  p(out), None)
    assert rc == _capi.GB_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_torque_derivatives(case, precision):
    """computeStaticTorqueDerivatives (rnea-derivatives.hxx:185-233) against the oracle's
    RNEA derivatives at zero velocity and acceleration with the same forces"""
    name, model, om, q, v, x, fext, dev = case
    data = pg.createData(model, precision)
    z = np.zeros_like(v)
    ref = om.rnea_derivatives(q, z, z, fext=fext)[1]
    got = pg.computeStaticTorqueDerivatives(model, data, dev(q), dev(fext)).cpu().numpy()
    assert rel_err(got, ref) < _tol(name, precision)
