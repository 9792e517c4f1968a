"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the FP64 oracle on seeded inputs, with its long-double run beside it).

CPU: the oracle built on this host reproduces every fixture (1e-13 relative:
the x86 and Arm builds differ only by FMA contraction and libm), and its FP64
run sits within 1e-10 of its long-double run.  GPU: the FP64 kernels match the
fixtures at 1e-12 and the mixed-precision kernels at 1e-5, through the C ABI."""
import glob
import os

import numpy as np
import pytest

from oracle.oracle import LOCAL, WORLD, OracleModel
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
FACTORIES = {
    "manipulator6r": lambda: sm.manipulator6r(0),
    "humanoid32": lambda: sm.humanoid32(1),
    "tree12": lambda: sm.random_tree(12, False, 3),
}
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _load(path):
    name = os.path.basename(path)[:-4]
    return name, FACTORIES[name](), dict(np.load(path))


def test_fixtures_present():
    assert {os.path.basename(p)[:-4] for p in FIXTURES} == set(FACTORIES)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_fixture(path):
    name, model, g = _load(path)
    om = OracleModel(model)
    q, v, a, tau = g["q"], g["v"], g["a"], g["tau_in"]
    tol = 1e-13
    assert rel_err(om.rnea(q, v, a), g["rnea"]) < tol
    assert rel_err(om.aba(q, v, tau, LOCAL), g["aba_local"]) < tol
    assert rel_err(om.aba(q, v, tau, WORLD), g["aba_world"]) < tol
    M = om.crba(q, LOCAL)
    assert rel_err(M, g["crba"]) < tol
    U, D = om.cholesky(M)
    assert rel_err(U, g["chol_U"]) < tol and rel_err(D, g["chol_D"]) < tol
    for got, key in zip(om.rnea_derivatives(q, v, a), ("rneaD_tau", "rneaD_dq", "rneaD_dv", "rneaD_M")):
        assert rel_err(got, g[key]) < tol, key
    for got, key in zip(om.aba_derivatives(q, v, tau), ("abaD_ddq", "abaD_dq", "abaD_dv", "abaD_Minv")):
        assert rel_err(got, g[key]) < 1e-12, key
    assert rel_err(om.integrate(q, v), g["integrate"]) < tol


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_fp64_fixture_agrees_with_long_double(path):
    _, _, g = _load(path)
    for key in ("rnea", "aba_local", "aba_world", "abaD_ddq", "rneaD_tau", "integrate", "chol_D"):
        assert rel_err(g[key], g[key + "_ld"]) < 1e-12, key
    for key in [k for k in g if k.startswith("maxdiff_")]:
        assert float(g[key]) <= 1e-10 * max(1.0, float(np.abs(g[key[8:]]).max())), key


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_kernels_match_fixture(path, precision):
    import torch

    import pinocchio_gb300 as pg
    from oracle.oracle import symmetrize_upper

    name, model, g = _load(path)
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    data = pg.createData(model, precision)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    q, v, a, tau = d(g["q"]), d(g["v"]), d(g["a"]), d(g["tau_in"])
    c = lambda t: t.cpu().numpy()  # noqa: E731
    assert rel_err(c(pg.rnea(model, data, q, v, a)), g["rnea"]) < tol
    assert rel_err(c(pg.aba(model, data, q, v, tau)), g["aba_local"]) < tol
    assert rel_err(c(pg.crba(model, data, q)), symmetrize_upper(g["crba"])) < tol
    dq, dv, M = pg.computeRNEADerivatives(model, data, q, v, a)
    assert rel_err(c(dq), g["rneaD_dq"]) < tol and rel_err(c(dv), g["rneaD_dv"]) < tol
    assert rel_err(c(M), symmetrize_upper(g["rneaD_M"])) < tol
    Aq, Av, Mi = pg.computeABADerivatives(model, data, q, v, tau)
    assert rel_err(c(Aq), g["abaD_dq"]) < tol and rel_err(c(Av), g["abaD_dv"]) < tol
    assert rel_err(c(Mi), g["abaD_Minv"]) < tol
    assert rel_err(c(pg.integrate(model, q, v, data)), g["integrate"]) < 1e-14
