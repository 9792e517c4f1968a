"""GPU parity of the batched analytical derivatives through the C ABI:
computeRNEADerivatives -> (dtau_dq, dtau_dv, M) and computeABADerivatives ->
(ddq_dq, ddq_dv, Minv), FP64 against the oracle at 1e-12 (the ill-conditioned
100-link chain at 1e-10), mixed precision at 1e-5, central finite differences
(step 1e-6 in the tangent space), both layouts and the identities the
reference's tests use (unittest/aba-derivatives.cpp:96-100: Minv = M^-1)."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel, symmetrize_upper
from pinocchio_gb300 import _capi
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu

# the mixed-precision bar applies to every model: on the 100-link chain (a tree deeper than
# 32 joints) the mixed sweeps keep their column sets and dtau in double-float
MIXED_MODELS = list(MODELS)


def fp64_tol(name):
    return 1e-10 if name == "chain100" else FP64_TOL


@pytest.fixture(scope="module", params=list(MODELS))
def case(request):
    import torch

    model = MODELS[request.param]()
    q, v, x = sm.random_inputs(model, 517, 41)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return request.param, model, OracleModel(model), q, v, x, dev


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rnea_derivatives(case, precision):
    name, model, om, q, v, a, dev = case
    if precision == "mixed" and name not in MIXED_MODELS:
        pytest.skip("FP64 stress model")
    data = pg.createData(model, precision)
    dq, dv, M = (t.cpu().numpy() for t in pg.computeRNEADerivatives(model, data, dev(q), dev(v), dev(a)))
    tau_o, dq_o, dv_o, M_o = om.rnea_derivatives(q, v, a)
    tol = fp64_tol(name) if precision == "fp64" else mixed_tol(name)
    assert rel_err(dq, dq_o) < tol
    assert rel_err(dv, dv_o) < tol
    assert rel_err(M, symmetrize_upper(M_o)) < tol
    assert rel_err(data.tau.cpu().numpy(), tau_o) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aba_derivatives(case, precision):
    name, model, om, q, v, x, dev = case
    if precision == "mixed" and name not in MIXED_MODELS:
        pytest.skip("FP64 stress model")
    tau = 10.0 * x
    data = pg.createData(model, precision)
    dq, dv, Minv = (t.cpu().numpy() for t in pg.computeABADerivatives(model, data, dev(q), dev(v), dev(tau)))
    ddq_o, dq_o, dv_o, Minv_o = om.aba_derivatives(q, v, tau)
    tol = fp64_tol(name) if precision == "fp64" else mixed_tol(name)
    assert rel_err(data.ddq.cpu().numpy(), ddq_o) < tol
    assert rel_err(Minv, Minv_o) < tol
    assert rel_err(dq, dq_o) < tol
    assert rel_err(dv, dv_o) < tol
    assert np.array_equal(Minv, np.swapaxes(Minv, 1, 2))


def test_minv_is_inverse_of_crba(case):
    name, model, om, q, v, x, dev = case
    data = pg.createData(model)
    _, _, Minv = pg.computeABADerivatives(model, data, dev(q), dev(v), dev(x))
    M = pg.crba(model, data, dev(q))
    eye = np.broadcast_to(np.eye(model.nv), (q.shape[0], model.nv, model.nv))
    assert rel_err((Minv @ M).cpu().numpy(), eye) < (1e-8 if name == "chain100" else 1e-11)


@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "tree12", "mixedtree24ff"])
def test_derivatives_vs_central_fd_on_gpu(name):
    import torch

    model = MODELS[name]()
    data = pg.createData(model)
    q, v, x = sm.random_inputs(model, 16, 3)
    tau = 10.0 * x
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    dq, dv, Minv = (t.cpu().numpy() for t in pg.computeABADerivatives(model, data, dev(q), dev(v), dev(tau)))
    h = 1e-6
    fdq, fdv, fdt = np.zeros_like(dq), np.zeros_like(dq), np.zeros_like(dq)
    qd, vd, td = dev(q), dev(v), dev(tau)
    for k in range(model.nv):
        e = torch.zeros((16, model.nv), dtype=torch.float64, device="cuda")
        e[:, k] = h
        qp, qm = pg.integrate(model, qd, e), pg.integrate(model, qd, -e)
        fdq[:, :, k] = ((pg.aba(model, data, qp, vd, td) - pg.aba(model, data, qm, vd, td)) / (2 * h)).cpu().numpy()
        fdv[:, :, k] = ((pg.aba(model, data, qd, vd + e, td) - pg.aba(model, data, qd, vd - e, td)) / (2 * h)).cpu().numpy()
        fdt[:, :, k] = ((pg.aba(model, data, qd, vd, td + e) - pg.aba(model, data, qd, vd, td - e)) / (2 * h)).cpu().numpy()
    assert rel_err(dq, fdq) < 1e-6
    assert rel_err(dv, fdv) < 1e-6
    assert rel_err(Minv, fdt) < 1e-6


def test_soa_layout_derivatives(case):
    import torch

    name, model, om, q, v, x, dev = case
    data = pg.createData(model)
    B, nv = q.shape[0], model.nv
    ref = [t.clone() for t in pg.computeABADerivatives(model, data, dev(q), dev(v), dev(x))]
    qs, vs, ts = (dev(t.T) for t in (q, v, x))
    outs = [torch.empty((nv * nv, B), dtype=torch.float64, device="cuda") for _ in range(3)]
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(
        _capi.lib().gb_aba_derivatives(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(ts),
                                       p(outs[0]), p(outs[1]), p(outs[2]), None, None)
    )
    torch.cuda.synchronize()
    for o, r in zip(outs, ref):
        assert torch.equal(o.T.reshape(B, nv, nv), r)


def test_gravity_with_angular_part_is_rejected():
    model = MODELS["manipulator6r"]()
    model.gravity = np.array([0, 0, -9.81, 0.1, 0, 0])
    data = pg.createData(model)
    with pytest.raises(_capi.GBError) as err:
        pg.computeABADerivatives(model, data, np.zeros((2, 6)), np.zeros((2, 6)), np.zeros((2, 6)))
    assert err.value.code == _capi.GB_ERR_GRAVITY


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aba_derivatives_vjp(case, precision):
    """gb_aba_derivatives_vjp == g^T of the oracle's Jacobians (and Minv g)."""
    name, model, om, q, v, x, dev = case
    if precision == "mixed" and name not in MIXED_MODELS:
        pytest.skip("the mixed-precision bar applies to the benchmark models")
    tol = fp64_tol(name) if precision == "fp64" else mixed_tol(name)
    tau = 10.0 * x
    g = np.random.default_rng(5).standard_normal((q.shape[0], model.nv))
    data = pg.createData(model, precision)
    qb, vb, tb = (a.cpu().numpy() for a in pg.abaDerivativesVJP(model, data, dev(q), dev(v), dev(tau), dev(g)))
    _, dq, dv, Minv = om.aba_derivatives(q, v, tau)
    assert rel_err(qb, np.einsum("bk,bkc->bc", g, dq)) < tol
    assert rel_err(vb, np.einsum("bk,bkc->bc", g, dv)) < tol
    assert rel_err(tb, np.einsum("bkc,bc->bk", Minv, g)) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aba_derivatives_large_batch_matches_slices(precision):
    """A batch large enough that every CTA of the product kernel walks several
    blocks (both pipeline stages, many barrier phases) gives, bit for bit, the
    results of the same configurations computed in small batches; the SOA
    layout gives the same bits as the instance layout; no pipeline wait gave up."""
    import torch

    model = MODELS["humanoid32"]()
    B, nv = 3001, model.nv
    q, v, x = sm.random_inputs(model, B, 77)
    tau = 10.0 * x
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    data = pg.createData(model, precision)
    full = [t.clone() for t in pg.computeABADerivatives(model, data, dev(q), dev(v), dev(tau))]
    for lo, hi in ((0, 41), (1500, 1517), (B - 9, B)):
        part = pg.computeABADerivatives(model, data, dev(q[lo:hi]), dev(v[lo:hi]), dev(tau[lo:hi]))
        for f, p in zip(full, part):
            assert torch.equal(f[lo:hi], p)
    qs, vs, ts = (dev(t.T) for t in (q, v, tau))
    outs = [torch.empty((nv * nv, B), dtype=torch.float64, device="cuda") for _ in range(3)]
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    prec = _capi.GB_FP64 if precision == "fp64" else _capi.GB_MIXED
    _capi.check(
        _capi.lib().gb_aba_derivatives(data.dev.h, prec, _capi.GB_LAYOUT_SOA, B, ptr(qs), ptr(vs), ptr(ts),
                                       ptr(outs[0]), ptr(outs[1]), ptr(outs[2]), None, None)
    )
    torch.cuda.synchronize()
    for o, r in zip(outs, full):
        assert torch.equal(o.T.reshape(B, nv, nv), r)
    n = C.c_uint(7)
    _capi.check(_capi.lib().gb_pipeline_timeouts(C.byref(n), 0))
    assert n.value == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_staged_matrix_outputs_match_soa(precision):
    """From 1024 configurations the instance-layout matrices of computeRNEADerivatives
    and of the CRBA (with its Cholesky factors) are written into an SOA scratch and
    transposed: the same bits as the SOA layout the kernels write directly, and as a
    small batch of the same configurations."""
    import torch

    model = MODELS["humanoid32"]()
    B, nv = 1500, model.nv
    q, v, a = sm.random_inputs(model, B, 19)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    data = pg.createData(model, precision)
    prec = _capi.GB_FP64 if precision == "fp64" else _capi.GB_MIXED
    L = _capi.lib()
    inst = [torch.empty((B, nv, nv), dtype=torch.float64, device="cuda") for _ in range(3)]
    soa = [torch.empty((nv * nv, B), dtype=torch.float64, device="cuda") for _ in range(3)]
    qi, vi, ai = dev(q), dev(v), dev(a)  # kept alive until the kernels have run
    qs, vs, as_ = dev(q.T), dev(v.T), dev(a.T)
    _capi.check(L.gb_rnea_derivatives(data.dev.h, prec, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_INSTANCE, B,
                                      ptr(qi), ptr(vi), ptr(ai), ptr(inst[0]), ptr(inst[1]), ptr(inst[2]), None, None))
    _capi.check(L.gb_rnea_derivatives(data.dev.h, prec, _capi.GB_MATRIX_SYMMETRIC, _capi.GB_LAYOUT_SOA, B,
                                      ptr(qs), ptr(vs), ptr(as_), ptr(soa[0]), ptr(soa[1]), ptr(soa[2]), None, None))
    small = pg.computeRNEADerivatives(model, data, dev(q[:37]), dev(v[:37]), dev(a[:37]))
    torch.cuda.synchronize()
    for i, s, sm_ in zip(inst, soa, small):
        assert torch.equal(i, s.T.reshape(B, nv, nv))
        assert torch.equal(i[:37], sm_)
    Mi, Ui = (torch.empty((B, nv, nv), dtype=torch.float64, device="cuda") for _ in range(2))
    Di = torch.empty((B, nv), dtype=torch.float64, device="cuda")
    Ms, Us = (torch.empty((nv * nv, B), dtype=torch.float64, device="cuda") for _ in range(2))
    Ds = torch.empty((nv, B), dtype=torch.float64, device="cuda")
    for lay, qq, outs in ((_capi.GB_LAYOUT_INSTANCE, qi, (Mi, Ui, Di)), (_capi.GB_LAYOUT_SOA, qs, (Ms, Us, Ds))):
        _capi.check(L.gb_crba(data.dev.h, prec, _capi.GB_LOCAL, _capi.GB_MATRIX_UPPER, lay, B, ptr(qq), ptr(outs[0]),
                              ptr(outs[1]), ptr(outs[2]), None))
    torch.cuda.synchronize()
    assert torch.equal(Mi, Ms.T.reshape(B, nv, nv)) and torch.equal(Ui, Us.T.reshape(B, nv, nv))
    assert torch.equal(Di, Ds.T)
    _, _, _, M_o = OracleModel(model).rnea_derivatives(q[:64], v[:64], a[:64])
    assert rel_err(Mi[:64].cpu().numpy(), M_o) < (FP64_TOL if precision == "fp64" else MIXED_TOL)


def test_pipeline_wait_timeout_is_reported_and_recoverable():
    """The bounded mbarrier wait of the pipelined kernels gives up, records the
    timeout (gb_pipeline_timeouts) and leaves the context usable: a barrier that
    nothing arrives on, waited on for 2 ms."""
    import torch

    L = _capi.lib()
    n = C.c_uint(0)
    _capi.check(L.gb_pipeline_timeouts(C.byref(n), 1))  # read and reset
    _capi.check(L.gb_pipeline_wait_selftest(2000, None))
    _capi.check(L.gb_pipeline_timeouts(C.byref(n), 1))
    assert n.value == 1
    assert L.gb_pipeline_wait_selftest(0, None) == _capi.GB_ERR_INVALID_ARGUMENT
    model = MODELS["humanoid32"]()
    q, v, x = sm.random_inputs(model, 64, 2)
    data = pg.createData(model, "mixed")
    dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    dq, dv, Minv = (t.cpu().numpy() for t in pg.computeABADerivatives(model, data, dev(q), dev(v), dev(10.0 * x)))
    _, dq_o, _, _ = OracleModel(model).aba_derivatives(q, v, 10.0 * x)
    assert rel_err(dq, dq_o) < MIXED_TOL
    _capi.check(L.gb_pipeline_timeouts(C.byref(n), 0))
    assert n.value == 0
