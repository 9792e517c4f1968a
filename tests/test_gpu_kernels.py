"""GPU parity of the batched sweep kernels (RNEA, ABA, CRBA + Cholesky,
integrate) through the C ABI, against the oracle: FP64 at 1e-12 relative,
mixed precision at 1e-5, both batch layouts, ragged / empty / single batches,
the host-memory rneaInParallel / abaInParallel entry points, batch == single
evaluation (bit-exact, as unittest/parallel-aba.cpp:54 requires) and
run-to-run determinism."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from pinocchio_gb300 import _capi
from oracle.oracle import LOCAL, WORLD, OracleModel, symmetrize_upper
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=list(MODELS))
def case(request):
    import torch

    model = MODELS[request.param]()
    q, v, x = sm.random_inputs(model, 1000 + 37, 31)  # ragged: not a multiple of the CTA size
    dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    return request.param, model, OracleModel(model), q, v, x, dev


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rnea(case, precision):
    name, model, om, q, v, a, dev = case
    data = pg.createData(model, precision)
    tau = pg.rnea(model, data, dev(q), dev(v), dev(a)).cpu().numpy()
    assert rel_err(tau, om.rnea(q, v, a)) < (FP64_TOL if precision == "fp64" else mixed_tol(name))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("convention", [LOCAL, WORLD])
def test_aba(case, precision, convention):
    name, model, om, q, v, x, dev = case
    tau = 10.0 * x
    data = pg.createData(model, precision)
    ddq = pg.aba(model, data, dev(q), dev(v), dev(tau), convention).cpu().numpy()
    assert rel_err(ddq, om.aba(q, v, tau, convention)) < (FP64_TOL if precision == "fp64" else mixed_tol(name))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_crba(case, precision):
    name, model, om, q, v, x, dev = case
    data = pg.createData(model, precision)
    Mref = om.crba(q)
    M = pg.crba(model, data, dev(q)).cpu().numpy()
    assert rel_err(M, symmetrize_upper(Mref)) < (FP64_TOL if precision == "fp64" else mixed_tol(name))
    Mu = pg.crba(model, data, dev(q), symmetric=False).cpu().numpy()
    if precision == "fp64":
        # block-upper output: every entry outside the joint-diagonal blocks and below the diagonal is zero
        joint_of = np.repeat(np.arange(model.njoints), model.nvs)
        lower_other = np.tril(np.ones((model.nv, model.nv), bool), -1) & (joint_of[:, None] != joint_of[None, :])
        assert np.all(Mu[:, lower_other] == 0.0)
        assert rel_err(np.triu(Mu), np.triu(Mref)) < FP64_TOL


def test_crba_cholesky(case):
    name, model, om, q, v, x, dev = case
    data = pg.createData(model, "mixed")  # the factorisation runs in FP64 in both precisions
    M, U, D = (t.cpu().numpy() for t in pg.crbaCholesky(model, data, dev(q)))
    Uo, Do = om.cholesky(om.crba(q))
    tol = 1e-11 if name == "chain100" else FP64_TOL
    assert rel_err(U, Uo) < tol and rel_err(D, Do) < tol
    assert rel_err(np.einsum("bij,bj,bkj->bik", U, D, U), M) < 1e-12


def test_integrate(case):
    name, model, om, q, v, x, dev = case
    out = pg.integrate(model, dev(q), dev(0.1 * v)).cpu().numpy()
    assert rel_err(out, om.integrate(q, 0.1 * v)) < 1e-15


def test_soa_layout_matches_instance_layout(case):
    import torch

    name, model, om, q, v, a, dev = case
    data = pg.createData(model)
    B = q.shape[0]
    ref = pg.rnea(model, data, dev(q), dev(v), dev(a))
    qs, vs, as_ = (dev(np.ascontiguousarray(t.T)) for t in (q, v, a))
    out = torch.empty((model.nv, B), dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(_capi.lib().gb_rnea(data.dev.h, _capi.GB_FP64, _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(as_), p(out), None))
    torch.cuda.synchronize()
    assert torch.equal(out.T, ref)


def test_batch_equals_single_and_determinism(case):
    name, model, om, q, v, x, dev = case
    data = pg.createData(model)
    tau = 10.0 * x
    full = pg.aba(model, data, dev(q), dev(v), dev(tau)).cpu().numpy()
    again = pg.aba(model, data, dev(q), dev(v), dev(tau)).cpu().numpy()
    assert np.array_equal(full, again)
    for b in (0, 1, 500, q.shape[0] - 1):
        one = pg.aba(model, data, dev(q[b]), dev(v[b]), dev(tau[b])).cpu().numpy()
        assert np.array_equal(one, full[b])


def test_empty_batch_is_a_no_op():
    model = MODELS["manipulator6r"]()
    data = pg.createData(model)
    L = _capi.lib()
    assert L.gb_rnea(data.dev.h, 0, 0, 0, None, None, None, None, None) == _capi.GB_OK


@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32"])
def test_in_parallel_host_entry_points(name):
    model = MODELS[name]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 300, 8)
    pool = pg.ModelPool(model, 8)
    tau = pg.rneaInParallel(8, pool, q.T, v.T, a.T)
    assert tau.shape == (model.nv, 300)
    assert rel_err(tau.T, om.rnea(q, v, a)) < FP64_TOL
    ddq = pg.abaInParallel(4, pool, q.T, v.T, tau)
    assert rel_err(ddq.T, om.aba(q, v, tau.T, WORLD)) < FP64_TOL
    with pytest.raises(_capi.GBError) as err:
        pg.rneaInParallel(9, pool, q.T, v.T, a.T)  # num_threads > pool.size()
    assert err.value.code == _capi.GB_ERR_POOL


@pytest.mark.parametrize("name", ["humanoid32", "multidoftree16"])
def test_preallocated_outputs(name):
    """``out=`` writes the single calls' results into the caller's tensors (the same tensors are
    returned, with the bits of the allocating calls); a wrong shape, dtype or device raises."""
    import torch

    model = MODELS[name]()
    q, v, x = (torch.from_numpy(a).cuda() for a in sm.random_inputs(model, 301, 8))
    data = pg.createData(model, "mixed")
    B, nv = q.shape[0], model.nv
    vec = lambda: torch.full((B, nv), np.nan, dtype=torch.float64, device="cuda")  # noqa: E731
    mat = lambda: torch.full((B, nv, nv), np.nan, dtype=torch.float64, device="cuda")  # noqa: E731
    o = vec()
    assert pg.rnea(model, data, q, v, x, out=o) is o and torch.equal(o, pg.rnea(model, data, q, v, x))
    o = vec()
    assert pg.aba(model, data, q, v, x, out=o) is o and torch.equal(o, pg.aba(model, data, q, v, x))
    o = mat()
    assert pg.crba(model, data, q, out=o) is o and torch.equal(o, pg.crba(model, data, q))
    outs = (mat(), mat(), mat(), vec())
    got = pg.computeABADerivatives(model, data, q, v, x, out=outs)
    assert all(a is b for a, b in zip(got, outs))
    ref = pg.computeABADerivatives(model, data, q, v, x)
    assert all(torch.equal(a, b) for a, b in zip(got, ref)) and torch.equal(outs[3], data.ddq)
    outs = (mat(), mat(), mat())
    got = pg.computeRNEADerivatives(model, data, q, v, x, out=outs)
    ref = pg.computeRNEADerivatives(model, data, q, v, x)
    assert all(a is b and torch.equal(a, r) for a, b, r in zip(got, outs, ref))
    one = torch.empty(nv, dtype=torch.float64, device="cuda")
    assert torch.equal(pg.aba(model, data, q[7], v[7], x[7], out=one), pg.aba(model, data, q, v, x)[7])
    for bad in (torch.empty((B, nv + 1), dtype=torch.float64, device="cuda"),
                torch.empty((B, nv), dtype=torch.float32, device="cuda"),
                torch.empty((B, nv), dtype=torch.float64)):
        with pytest.raises(ValueError):
            pg.aba(model, data, q, v, x, out=bad)
    with pytest.raises(ValueError):
        pg.computeABADerivatives(model, data, q, v, x, out=(mat(),))


def test_copy_async_round_trip():
    """copyAsync (gb_memcpy_async): pinned host -> device -> pinned host on the current stream,
    the same bytes back; size mismatches and NULL pointers are rejected."""
    import torch

    src = torch.arange(1 << 20, dtype=torch.float64).pin_memory()
    dev = torch.empty(1 << 20, dtype=torch.float64, device="cuda")
    back = torch.empty(1 << 20, dtype=torch.float64).pin_memory()
    pg.copyAsync(dev, src)
    pg.copyAsync(back, dev)
    torch.cuda.synchronize()
    assert torch.equal(back, src)
    with pytest.raises(ValueError):
        pg.copyAsync(back[:10], dev)
    L = _capi.lib()
    assert L.gb_memcpy_async(None, C.c_void_p(dev.data_ptr()), 8, None) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_memcpy_async(None, None, 0, None) == _capi.GB_OK
