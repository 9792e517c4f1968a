"""The kernels' per-instance code, built for the host, against the oracle.

The same gb_dyn.cuh source that nvcc compiles for sm_103a is compiled by g++
here, so the arithmetic of both precisions is checked without a GPU:
FP64 at the 1e-12 parity bar, mixed precision at the 1e-5 bar."""
import numpy as np
import pytest

from hostsim import HostSim
from oracle.oracle import LOCAL, WORLD, OracleModel, symmetrize_upper
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, MODELS, rel_err


@pytest.fixture(scope="module", params=list(MODELS))
def case(request):
    model = MODELS[request.param]()
    q, v, x = sm.random_inputs(model, 64, 21)
    return request.param, model, OracleModel(model), HostSim(model), q, v, x


def test_rnea(case):
    name, model, om, hs, q, v, a = case
    ref = om.rnea(q, v, a)
    assert rel_err(hs.rnea(q, v, a), ref) < FP64_TOL
    assert rel_err(hs.rnea(q, v, a, mixed=True), ref) < MIXED_TOL


def test_aba(case):
    name, model, om, hs, q, v, x = case
    tau = 10.0 * x
    ref = om.aba(q, v, tau, LOCAL)
    assert rel_err(hs.aba(q, v, tau), ref) < FP64_TOL
    assert rel_err(hs.aba(q, v, tau), om.aba(q, v, tau, WORLD)) < FP64_TOL
    assert rel_err(hs.aba(q, v, tau, mixed=True), ref) < MIXED_TOL


def test_crba_cholesky(case):
    name, model, om, hs, q, v, x = case
    Mu = om.crba(q)
    M, U, D = hs.crba(q, symmetric=True, cholesky=True)
    Uo, Do = om.cholesky(Mu)
    assert rel_err(M, symmetrize_upper(Mu)) < FP64_TOL
    tol = 1e-11 if name == "chain100" else FP64_TOL  # U, D of the 100-link chain are ill-conditioned
    assert rel_err(U, Uo) < tol and rel_err(D, Do) < tol
    assert rel_err(hs.crba(q, mixed=True, symmetric=True), symmetrize_upper(Mu)) < MIXED_TOL
    Mup = hs.crba(q, symmetric=False)
    assert np.array_equal(Mup == 0, Mu == 0) or rel_err(Mup, Mu) < FP64_TOL


def test_integrate(case):
    name, model, om, hs, q, v, x = case
    assert rel_err(hs.integrate(q, 0.1 * v), om.integrate(q, 0.1 * v)) < 1e-15


def test_rnea_derivatives(case):
    name, model, om, hs, q, v, a = case
    ref = om.rnea_derivatives(q, v, a)
    got = hs.rnea_derivatives(q, v, a)
    tol = 1e-10 if name == "chain100" else FP64_TOL
    for g, r in zip(got[:3], ref[:3]):
        assert rel_err(g, r) < tol
    assert rel_err(got[3], symmetrize_upper(ref[3])) < tol
    if name != "chain100":
        for g, r in zip(hs.rnea_derivatives(q, v, a, mixed=True)[:3], ref[:3]):
            assert rel_err(g, r) < MIXED_TOL


def test_aba_derivatives(case):
    name, model, om, hs, q, v, x = case
    tau = 10.0 * x
    ref = om.aba_derivatives(q, v, tau)
    got = hs.aba_derivatives(q, v, tau)
    tol = 1e-10 if name == "chain100" else FP64_TOL
    for g, r in zip(got, ref):
        assert rel_err(g, r) < tol
    if name != "chain100":  # the chain is the FP64 stress model
        for g, r in zip(hs.aba_derivatives(q, v, tau, mixed=True), ref):
            assert rel_err(g, r) < MIXED_TOL
