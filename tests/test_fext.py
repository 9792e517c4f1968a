"""External forces (the reference's fext overloads of rnea, aba, computeStaticTorque,
computeRNEADerivatives and computeABADerivatives: algorithm/rnea.hxx:164-218 and
448-489, aba.hxx:296-352 and 543-605, rnea-derivatives.hxx:550-633,
aba-derivatives.hxx:463-541) on the CPU: the oracle against identities that do
not go through its own code path, and the host build of the kernel code against
the oracle.

Pins (fext_i is a force on joint i expressed in joint i's frame):
  * tau(q, v, a, fext) = tau(q, v, a) - sum_i J_i^T oMi.act(fext_i), with J_i the
    world-frame Jacobian columns of joint i's support (the reference's
    unittest/rnea.cpp:136-177 and 250-280 check rnea and computeStaticTorque
    with fext against J^T fext);
  * aba(q, v, rnea(q, v, a, fext), fext) = a in both conventions
    (unittest/aba.cpp:186-222);
  * the fext derivatives against central differences of the fext functions
    (step 1e-6 in the tangent space), Minv unchanged by fext;
  * computeStaticTorque(q, fext) = rnea(q, 0, 0, fext) (rnea.hpp:144).
"""
import numpy as np
import pytest

from oracle.oracle import LOCAL, WORLD, OracleModel
from pinocchio_gb300 import sample_models as sm
from test_oracle import _fd, _support
from util import MODELS, mixed_tol, rel_err

FEXT_MODELS = ["manipulator6r", "humanoid32", "tree12", "mixedtree24ff", "unaligned14", "unaligned20ff"]


def random_fext(njoints, B, seed):
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(B, njoints, 6))
    f[:, 0] = 0.0  # joint 0 (the universe) takes no force
    return f


def _act_force(M, f6):
    """oMi.act(f) for M = (R row-major, t) (reference spatial/force-dense.hpp:214-219)."""
    R = M[..., :9].reshape(M.shape[:-1] + (3, 3))
    t = M[..., 9:]
    lin = np.einsum("...ij,...j->...i", R, f6[..., :3])
    ang = np.einsum("...ij,...j->...i", R, f6[..., 3:]) + np.cross(t, lin)
    return np.concatenate([lin, ang], axis=-1)


@pytest.fixture(scope="module", params=FEXT_MODELS)
def case(request):
    model = MODELS[request.param]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 12, 21)
    return request.param, model, om, q, v, a, random_fext(om.njoints, 12, 22)


def test_rnea_fext_is_jacobian_transpose(case):
    name, model, om, q, v, a, fext = case
    tau0 = om.rnea(q, v, a)
    tau1 = om.rnea(q, v, a, fext=fext)
    oMi = om.forward_kinematics(q)[0]
    J = om.joint_jacobians(q)  # (B, nv, 6): world-frame columns
    expect = tau0.copy()
    for i, dofs in enumerate(_support(model)):
        if i == 0 or not dofs:
            continue
        fw = _act_force(oMi[:, i], fext[:, i])
        expect[:, dofs] -= np.einsum("bkr,br->bk", J[:, dofs], fw)
    assert rel_err(tau1, expect) < 1e-12
    # joint 0's entries are not read
    f2 = fext.copy()
    f2[:, 0] = 1e3
    assert np.array_equal(om.rnea(q, v, a, fext=f2), tau1)


def test_aba_rnea_roundtrip_with_fext(case):
    name, model, om, q, v, a, fext = case
    tau = om.rnea(q, v, a, fext=fext)
    for conv in (LOCAL, WORLD):
        assert rel_err(om.aba(q, v, tau, conv, fext=fext), a) < 1e-12


def test_static_torque_and_long_double(case):
    name, model, om, q, v, a, fext = case
    z = np.zeros_like(v)
    st = om.rnea(q, z, z, fext=fext)
    g = om.rnea(q, z, z)
    assert not np.allclose(st, g)
    tl = om.rnea(q, v, a, fext=fext, prec=1)
    assert rel_err(om.rnea(q, v, a, fext=fext), tl) < 1e-13
    dl = om.aba_derivatives(q, v, 10 * a, fext=fext, prec=1)
    for x, y in zip(om.aba_derivatives(q, v, 10 * a, fext=fext), dl):
        assert rel_err(x, y) < 1e-11


@pytest.mark.parametrize("name", ["manipulator6r", "humanoid32", "mixedtree24ff", "unaligned20ff"])
def test_fext_derivatives_vs_central_fd(name):
    model = MODELS[name]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 3, 25)
    fext = random_fext(om.njoints, 3, 26)
    tau = om.rnea(q, v, a, fext=fext)
    _, dq, dv, M = om.rnea_derivatives(q, v, a, fext=fext)
    ddq, adq, adv, Minv = om.aba_derivatives(q, v, tau, fext=fext)
    assert rel_err(ddq, a) < 1e-11
    assert rel_err(Minv, om.aba_derivatives(q, v, tau)[3]) < 1e-13  # Minv does not see fext
    h = 1e-6
    fd = {k: np.zeros_like(dq) for k in ("rq", "rv", "aq", "av")}
    integ = (om.integrate, model.nv)
    for k in range(model.nv):
        fd["rq"][:, :, k] = _fd(lambda x: om.rnea(x, v, a, fext=fext), q, h, k, integ)
        fd["rv"][:, :, k] = _fd(lambda x: om.rnea(q, x, a, fext=fext), v, h, k)
        fd["aq"][:, :, k] = _fd(lambda x: om.aba(x, v, tau, fext=fext), q, h, k, integ)
        fd["av"][:, :, k] = _fd(lambda x: om.aba(q, x, tau, fext=fext), v, h, k)
    assert rel_err(dq, fd["rq"]) < 1e-6
    assert rel_err(dv, fd["rv"]) < 1e-6
    assert rel_err(adq, fd["aq"]) < 1e-6
    assert rel_err(adv, fd["av"]) < 1e-6
    # the fext terms matter: derivatives without fext differ
    assert rel_err(om.rnea_derivatives(q, v, a)[1], dq) > 1e-6


def test_fext_size_is_checked():
    model = MODELS["tree12"]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 2, 3)
    with pytest.raises(ValueError):
        om.rnea(q, v, a, fext=np.zeros((2, om.njoints - 1, 6)))


@pytest.mark.parametrize("name", FEXT_MODELS)
def test_kernel_code_with_fext_on_host(name):
    """The per-configuration kernel code (host build) with external forces against the oracle:
    FP64 at 1e-12, mixed precision at the mixed bar."""
    hostsim = pytest.importorskip("hostsim")
    model = MODELS[name]()
    om = OracleModel(model)
    hs = hostsim.HostSim(model)
    q, v, a = sm.random_inputs(model, 24, 27)
    tau = 10.0 * a
    fext = random_fext(om.njoints, 24, 28)
    tol = mixed_tol(name)
    ref = om.rnea(q, v, a, fext=fext)
    assert rel_err(hs.rnea(q, v, a, fext=fext), ref) < 1e-12
    assert rel_err(hs.rnea(q, v, a, mixed=True, fext=fext), ref) < tol
    ref = om.aba(q, v, tau, fext=fext)
    assert rel_err(hs.aba(q, v, tau, fext=fext), ref) < 1e-12
    assert rel_err(hs.aba(q, v, tau, mixed=True, fext=fext), ref) < tol
    rt, rq, rv, rM = om.rnea_derivatives(q, v, a, fext=fext)
    for mixed, t in ((False, 1e-12), (True, tol)):
        ht, hq, hv, hM = hs.rnea_derivatives(q, v, a, mixed=mixed, symmetric=False, fext=fext)
        for x, y in ((ht, rt), (hq, rq), (hv, rv), (hM, rM)):
            assert rel_err(x, y) < t
    ref = om.aba_derivatives(q, v, tau, fext=fext)
    for mixed, t in ((False, 1e-12), (True, tol)):
        for x, y in zip(hs.aba_derivatives(q, v, tau, mixed=mixed, fext=fext), ref):
            assert rel_err(x, y) < t


def test_static_torque_derivatives_vs_central_fd():
    """d/dq of rnea(q, 0, 0, fext), which computeStaticTorqueDerivatives returns
    (rnea-derivatives.hxx:185-233), against central differences"""
    model = MODELS["unaligned20ff"]()
    om = OracleModel(model)
    q, v, a = sm.random_inputs(model, 3, 31)
    fext = random_fext(om.njoints, 3, 32)
    z = np.zeros_like(v)
    dq = om.rnea_derivatives(q, z, z, fext=fext)[1]
    fd = np.zeros_like(dq)
    for k in range(model.nv):
        fd[:, :, k] = _fd(lambda x: om.rnea(x, z, z, fext=fext), q, 1e-6, k, (om.integrate, model.nv))
    assert rel_err(dq, fd) < 1e-6
