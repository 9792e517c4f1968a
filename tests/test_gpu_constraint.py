"""GPU parity of constraintDynamics (reference algorithm/constrained-dynamics.hxx:188-520) through the
C ABI against the oracle: point and frame contacts in LOCAL and LOCAL_WORLD_ALIGNED axes, closed
loops between two limbs, Baumgarte gains and desired accelerations, the proximal iterations with
mu > 0 (iteration counts and residuals), a redundant pair of contacts, no constraint (= ABA), both
precisions and both batch layouts, every joint type, and the argument errors."""
import ctypes as C

import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import LOCAL as CONV_LOCAL
from oracle.oracle import OracleModel
from pinocchio_gb300 import _capi
from pinocchio_gb300 import constraints as cs
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MODELS, mixed_tol, rel_err

pytestmark = pytest.mark.gpu


def _rand_se3(rng, scale=0.2):
    a = rng.standard_normal(3)
    th = np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]]) / th
    return gm.SE3(np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K, scale * rng.standard_normal(3))


def _leaves(model):
    par = set(model.parents[1:])
    return [j for j in range(1, model.njoints) if j not in par]


def _exclusive_dofs(model, leaf):
    """The dofs between a leaf and its first branching ancestor (only this leaf's constraint moves them)."""
    nchild = np.bincount(np.asarray(model.parents[1:]), minlength=model.njoints)
    n, j = 0, leaf
    while j > 0:
        n += model.nvs[j]
        if nchild[model.parents[j]] > 1 or model.parents[j] == 0:
            break
        j = model.parents[j]
    return n


def _support(model, j):
    cols = []
    while j > 0:
        cols += list(range(model.idx_vs[j], model.idx_vs[j] + model.nvs[j]))
        j = model.parents[j]
    return cols


def _constraints(model, seed, gains=False):
    """Full-rank constraints: per leaf a frame contact (6 rows) when at least 6 dofs serve only that
    leaf, a point contact (3 rows) when at least 3 do, in alternating LOCAL / LOCAL_WORLD_ALIGNED
    axes, anchored to random world frames."""
    rng = np.random.default_rng(seed)
    cms = []
    for k, leaf in enumerate(_leaves(model)):
        n = _exclusive_dofs(model, leaf)
        if n < 3:
            continue
        t = cs.CONTACT_6D if n >= 6 and k % 2 == 0 else cs.CONTACT_3D
        f = cs.LOCAL if (k // 2) % 2 == 0 else cs.LOCAL_WORLD_ALIGNED
        cms.append(cs.RigidConstraintModel(t, model, leaf, _rand_se3(rng), 0, _rand_se3(rng, 1.0), f))
    if not cms:  # no leaf has three dofs of its own: one point contact on the deepest leaf
        depth = {j: len(_support(model, j)) for j in _leaves(model)}
        leaf = max(depth, key=depth.get)
        cms.append(cs.RigidConstraintModel(cs.CONTACT_3D, model, leaf, _rand_se3(rng), 0, _rand_se3(rng, 1.0),
                                           cs.LOCAL))
    if gains:
        for c in cms:
            c.corrector.Kp[:] = rng.uniform(0.5, 5.0, c.size())
            c.corrector.Kd[:] = rng.uniform(0.5, 5.0, c.size())
            c.desired_contact_acceleration[:] = rng.standard_normal(6)
    return cms


def _loop_constraints(model, seed):
    """The humanoid's limbs: a frame loop between the first two, a point contact on the third, a frame
    contact on the fourth (15 rows, each limb's six dofs serving one constraint)."""
    rng = np.random.default_rng(seed)
    lv = _leaves(model)
    return [
        cs.RigidConstraintModel(cs.CONTACT_6D, model, lv[0], _rand_se3(rng), lv[1], _rand_se3(rng), cs.LOCAL),
        cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[2], _rand_se3(rng), 0, _rand_se3(rng, 1.0),
                                cs.LOCAL_WORLD_ALIGNED),
        cs.RigidConstraintModel(cs.CONTACT_6D, model, lv[3], _rand_se3(rng), cs.LOCAL_WORLD_ALIGNED),
    ]


def _fp64_tol(om, q, v, tau, desc, **kw):
    """The FP64 bar of one case: 30 x the double oracle's own error against the long-double oracle
    (the KKT solve's conditioning), at least 1e-10."""
    a = om.constraint_dynamics(q, v, tau, desc, **kw)
    b = om.constraint_dynamics(q, v, tau, desc, prec=1, **kw)
    return a, b, max(1e-10, 30 * max(rel_err(a[0], b[0]), rel_err(a[1], b[1]) if a[1].size else 0.0))


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(MODELS) + ["humanoid32-loop"])
def test_constraint_dynamics_matches_oracle(name, precision):
    loop = name.endswith("-loop")
    model = MODELS[name.replace("-loop", "")]()
    om = OracleModel(model)
    cms = _loop_constraints(model, 4) if loop else _constraints(model, 3, gains=name in ("humanoid32", "mixedtree24ff"))
    q, v, x = sm.random_inputs(model, 333, 12)
    v = 0.3 * v
    tau = 10 * x
    data = pg.createData(model, precision)
    cds = [cs.RigidConstraintData(c) for c in cms]
    ddq = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(tau), cms, cds).cpu().numpy()
    lam = data.lambda_c.cpu().numpy()
    (d_o, l_o, it_o, res_o), (d_ld, l_ld, _, _), tol64 = _fp64_tol(om, q, v, tau, cs.stack_desc(cms))
    if precision == "fp64":
        assert rel_err(ddq, d_ld) < tol64
        assert lam.size == 0 or rel_err(lam, l_ld) < tol64
    else:
        tol = max(mixed_tol(name.replace("-loop", "")), 30 * tol64)
        if name == "chain100":
            tol = 1e-3
        assert rel_err(ddq, d_o) < tol
        assert lam.size == 0 or rel_err(lam, l_o) < tol
    assert np.array_equal(data.constraint_iterations.cpu().numpy(), it_o)
    row = 0
    for cd, c in zip(cds, cms):
        f = cd.contact_force.cpu().numpy()
        assert np.array_equal(f[:, : c.size()], lam[:, row : row + c.size()])
        assert np.all(f[:, c.size():] == 0)
        row += c.size()
    assert pg.numericStatus(data) == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_proximal_iterations(precision):
    """mu > 0: the iteration counts and residuals follow the oracle's proximal loop; a duplicated
    contact (singular Delassus matrix) gives the single contact's accelerations."""
    model = sm.humanoid32(1)
    om = OracleModel(model)
    cms = _loop_constraints(model, 5)
    q, v, x = sm.random_inputs(model, 200, 13)
    data = pg.createData(model, precision)
    st = pg.ProximalSettings(1e-10, 1e-4, 50)
    ddq = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms, None, st).cpu().numpy()
    d_o, l_o, it_o, res_o = om.constraint_dynamics(q, v, 10 * x, cs.stack_desc(cms), mu=1e-4, max_iter=50,
                                                   absolute_accuracy=1e-10, relative_accuracy=1e-10)
    it = data.constraint_iterations.cpu().numpy()
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert rel_err(ddq, d_o) < tol
    assert np.abs(it - it_o).max() <= 1 and it.max() > 1 and st.iter == it.max()
    res = data.constraint_residuals.cpu().numpy()
    assert np.all((res[:, 0] <= 1e-10) | (res[:, 1] <= 1e-10) | (it == 50))
    d1 = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms[:1]).cpu().numpy()
    st2 = pg.ProximalSettings(1e-12, 1e-6, 300)
    d2 = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms[:1] * 2, None, st2).cpu().numpy()
    assert rel_err(d2, d1) < (1e-7 if precision == "fp64" else 1e-5)


def test_no_constraint_is_aba_and_layouts():
    import torch

    model = MODELS["mixedtree24ff"]()
    q, v, x = sm.random_inputs(model, 257, 14)
    data = pg.createData(model)
    ddq = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), []).cpu().numpy()
    assert rel_err(ddq, OracleModel(model).aba(q, v, 10 * x, CONV_LOCAL)) < FP64_TOL
    assert data.lambda_c.shape == (257, 0) and torch.all(data.constraint_iterations == 1)
    # SOA layout: the same bits
    cms = _constraints(model, 6)
    assert cms
    pg.initConstraintDynamics(model, data, cms)
    ref = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms).cpu().numpy()
    lam = data.lambda_c.cpu().numpy()
    B, nv, nc = q.shape[0], model.nv, lam.shape[1]
    outs = [torch.empty((n, B), dtype=torch.float64, device="cuda") for n in (nv, nc)]
    ps = _capi.ProximalSettingsC(1e-12, 1e-12, 0.0, 1)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    qs, vs, ts = (_dev(np.ascontiguousarray(t.T)) for t in (q, v, 10 * x))
    _capi.check(_capi.lib().gb_constraint_dynamics(data.dev.h, _capi.GB_FP64, data.constraint_set.h, C.byref(ps),
                                                   _capi.GB_LAYOUT_SOA, B, p(qs), p(vs), p(ts), p(outs[0]),
                                                   p(outs[1]), None, None, None))
    torch.cuda.synchronize()
    assert np.array_equal(outs[0].cpu().numpy().T, ref) and np.array_equal(outs[1].cpu().numpy().T, lam)


def test_batch_equals_single():
    model = sm.humanoid32(1)
    cms = _loop_constraints(model, 8)
    cms[0].corrector.Kp[:] = 2.0
    q, v, x = sm.random_inputs(model, 64, 15)
    data = pg.createData(model)
    full = pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms).cpu().numpy()
    for b in (0, 31, 63):
        one = pg.constraintDynamics(model, data, _dev(q[b]), _dev(v[b]), _dev(10 * x[b]), cms).cpu().numpy()
        assert np.array_equal(one, full[b])


def test_argument_errors():
    model = sm.humanoid32(1)
    data = pg.createData(model)
    other = pg.createData(model)
    L = _capi.lib()
    arr = (_capi.ConstraintDesc * 1)()
    arr[0].type, arr[0].reference_frame, arr[0].joint1_id = _capi.GB_CONTACT_6D, _capi.GB_FRAME_WORLD, 5
    h = C.c_void_p()
    assert L.gb_constraint_set_create(data.dev.h, 1, arr, C.byref(h)) == _capi.GB_ERR_INVALID_ARGUMENT
    arr[0].reference_frame, arr[0].joint1_id = _capi.GB_FRAME_LOCAL, model.njoints
    assert L.gb_constraint_set_create(data.dev.h, 1, arr, C.byref(h)) == _capi.GB_ERR_INVALID_ARGUMENT
    arr[0].joint1_id, arr[0].type = 5, 7
    assert L.gb_constraint_set_create(data.dev.h, 1, arr, C.byref(h)) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_constraint_set_create(data.dev.h, 65, arr, C.byref(h)) == _capi.GB_ERR_SIZE
    cms = _constraints(model, 9)
    pg.initConstraintDynamics(model, data, cms)
    q, v, x = (_dev(a) for a in sm.random_inputs(model, 4, 16))
    ps = _capi.ProximalSettingsC(1e-12, 1e-12, -1.0, 1)
    out = _dev(np.zeros((4, model.nv)))
    lam = _dev(np.zeros((4, data.constraint_set.nc)))
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    args = (_capi.GB_LAYOUT_INSTANCE, 4, p(q), p(v), p(x), p(out), p(lam), None, None, None)
    assert L.gb_constraint_dynamics(data.dev.h, 0, data.constraint_set.h, C.byref(ps), *args) == _capi.GB_ERR_INVALID_ARGUMENT
    ps.mu, ps.max_iter = 0.0, 0
    assert L.gb_constraint_dynamics(data.dev.h, 0, data.constraint_set.h, C.byref(ps), *args) == _capi.GB_ERR_INVALID_ARGUMENT
    ps.max_iter = 1
    assert L.gb_constraint_dynamics(other.dev.h, 0, data.constraint_set.h, C.byref(ps), *args) == _capi.GB_ERR_INVALID_ARGUMENT
    assert L.gb_constraint_dynamics(data.dev.h, 0, data.constraint_set.h, C.byref(ps), *args) == _capi.GB_OK


def _deriv_tol(om, q, v, tau, desc, **kw):
    a = om.constraint_dynamics_derivatives(q, v, tau, desc, **kw)
    b = om.constraint_dynamics_derivatives(q, v, tau, desc, prec=1, **kw)
    errs = [rel_err(a[k], b[k]) for k in range(2, 8) if a[k].size]
    return a, b, max(1e-9, 30 * max(errs))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["humanoid32", "tree32ff", "chain100", "mixedtree24ff", "unaligned20ff",
                                  "translationtree14", "multidoftree16"])
def test_constraint_dynamics_derivatives_match_oracle(name, precision):
    """computeConstraintDynamicsDerivatives (constraints to the world, no gains) against the oracle:
    ddq_dq, ddq_dv, ddq_dtau, dlambda_dq, dlambda_dv, dlambda_dtau; FP64 at 30 x the double oracle's
    own error against long double (at least 1e-9)."""
    model = MODELS[name]()
    om = OracleModel(model)
    cms = _constraints(model, 31)
    q, v, x = sm.random_inputs(model, 129, 32)
    v = 0.3 * v
    tau = 10 * x
    data = pg.createData(model, precision)
    pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(tau), cms)
    got = [t.cpu().numpy() for t in pg.computeConstraintDynamicsDerivatives(model, data, cms)]
    (o, ld, tol64) = _deriv_tol(om, q, v, tau, cs.stack_desc(cms))
    names = ("ddq_dq", "ddq_dv", "ddq_dtau", "dlambda_dq", "dlambda_dv", "dlambda_dtau")
    for k, nm in enumerate(names):
        if precision == "fp64":
            assert rel_err(got[k], ld[2 + k]) < tol64, (nm, rel_err(got[k], ld[2 + k]), tol64)
        else:
            tol = 1e-2 if name == "chain100" else max(1e-4, 30 * tol64)
            assert rel_err(got[k], o[2 + k]) < tol, (nm, rel_err(got[k], o[2 + k]))
    assert pg.numericStatus(data) == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_constraint_dynamics_derivatives_with_local_contact_gains(precision):
    """LOCAL point and frame contacts with Baumgarte gains (the corrector's derivative, Jlog6 for the
    frame contact) next to a world-aligned point contact without gains, against the oracle; gains on
    a world-aligned contact are refused."""
    model = sm.humanoid32(1)
    om = OracleModel(model)
    rng = np.random.default_rng(41)
    lv = _leaves(model)
    cms = [cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[0], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_6D, model, lv[1], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[2], _rand_se3(rng), 0, _rand_se3(rng, 1.0), cs.LOCAL),
           cs.RigidConstraintModel(cs.CONTACT_3D, model, lv[3], _rand_se3(rng), 0, _rand_se3(rng, 1.0),
                                   cs.LOCAL_WORLD_ALIGNED)]
    for c in cms[:3]:
        c.corrector.Kp[:] = rng.uniform(0.5, 5.0, c.size())
        c.corrector.Kd[:] = rng.uniform(0.5, 5.0, c.size())
    q, v, x = sm.random_inputs(model, 97, 42)
    v = 0.3 * v
    data = pg.createData(model, precision)
    pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms)
    got = [t.cpu().numpy() for t in pg.computeConstraintDynamicsDerivatives(model, data, cms)]
    (o, ld, tol64) = _deriv_tol(om, q, v, 10 * x, cs.stack_desc(cms))
    for k in range(6):
        if precision == "fp64":
            assert rel_err(got[k], ld[2 + k]) < tol64, (k, rel_err(got[k], ld[2 + k]), tol64)
        else:
            assert rel_err(got[k], o[2 + k]) < max(1e-4, 30 * tol64), (k, rel_err(got[k], o[2 + k]))
    cms[3].corrector.Kp[:] = 1.0
    pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms)
    with pytest.raises(_capi.GBError) as e:
        pg.computeConstraintDynamicsDerivatives(model, data, cms)
    assert e.value.code == _capi.GB_ERR_UNSUPPORTED


def test_constraint_dynamics_derivatives_proximal_and_errors():
    """mu > 0 with a fixed number of iterations (accuracies 0): the derivatives follow the oracle's
    proximal recursion; no constraint gives the ABA derivatives; closed loops and Baumgarte gains are
    refused with GB_ERR_UNSUPPORTED."""
    model = sm.humanoid32(1)
    om = OracleModel(model)
    cms = _constraints(model, 33)
    q, v, x = sm.random_inputs(model, 64, 34)
    data = pg.createData(model)
    st = pg.ProximalSettings(0.0, 0.0, 1e-4, 5)
    pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), cms, None, st)
    assert st.iter == 5
    got = [t.cpu().numpy() for t in pg.computeConstraintDynamicsDerivatives(model, data, cms)]
    o = om.constraint_dynamics_derivatives(q, v, 10 * x, cs.stack_desc(cms), mu=1e-4, max_iter=5,
                                           absolute_accuracy=0.0, relative_accuracy=0.0)
    for k in range(6):
        assert rel_err(got[k], o[2 + k]) < 1e-9, k
    pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), [])
    d0 = [t.cpu().numpy() for t in pg.computeConstraintDynamicsDerivatives(model, data, [])]
    _, a_dq, a_dv, a_mi = om.aba_derivatives(q, v, 10 * x)
    assert rel_err(d0[0], a_dq) < 1e-10 and rel_err(d0[1], a_dv) < 1e-10 and rel_err(d0[2], a_mi) < 1e-10
    lv = _leaves(model)
    for bad in ([cs.RigidConstraintModel(cs.CONTACT_6D, model, lv[0], gm.SE3.Identity(), lv[1], gm.SE3.Identity(),
                                         cs.LOCAL)], _constraints(model, 35, gains=True)):
        pg.constraintDynamics(model, data, _dev(q), _dev(v), _dev(10 * x), bad)
        with pytest.raises(_capi.GBError) as e:
            pg.computeConstraintDynamicsDerivatives(model, data, bad)
        assert e.value.code == _capi.GB_ERR_UNSUPPORTED


@pytest.mark.parametrize("mu", [0.0, 0.05])
@pytest.mark.parametrize("name", [n for n in MODELS if n != "chain100"] + ["humanoid32-loop"])
def test_contact_cholesky_matches_oracle(name, mu):
    """ContactCholeskyDecomposition.compute and its accessors (contact-cholesky.hpp:168-265,
    contact-cholesky.hxx:617-759) against the oracle's restatement of the reference's KKT
    factorisation, relative to the oracle's own double / long-double gap of constraintDynamics on
    the same case; the Python class reads the configurations of the last crba call."""
    import torch

    loop = name.endswith("-loop")
    model = MODELS[name.replace("-loop", "")]()
    om = OracleModel(model)
    cms = _loop_constraints(model, 5) if loop else _constraints(model, 5)
    desc = cs.stack_desc(cms)
    q, v, x = sm.random_inputs(model, 64, 9)
    ref = om.contact_cholesky(q, desc, mu=mu)
    _, _, tol = _fp64_tol(om, q, v, 10 * x, desc, mu=mu)
    tol = max(tol, 1e-10)
    data = pg.createData(model)
    pg.crba(model, data, _dev(q))
    chol = pg.ContactCholeskyDecomposition(model, cms)
    chol.compute(model, data, cms, [cs.RigidConstraintData(c) for c in cms], mu)
    got = dict(matrix=chol.matrix(), inverse=chol.inverse(), osim_inverse=chol.getInverseOperationalSpaceInertiaMatrix(),
               osim=chol.getOperationalSpaceInertiaMatrix(), minv=chol.getInverseMassMatrix(), jminv=chol.getJMinv())
    assert chol.size() == model.nv + desc_dim(desc) and chol.constraintDim() == desc_dim(desc)
    for k, r in ref.items():
        assert rel_err(got[k].cpu().numpy(), r) < tol, k
    rhs = np.random.default_rng(2).standard_normal((64, chol.size()))
    assert rel_err(chol.solve(rhs), np.einsum("bij,bj->bi", ref["inverse"], rhs)) < tol
    if chol.constraintDim():  # the Delassus operator (DelassusCholeskyExpression) and its solve
        dx = rhs[:, : chol.constraintDim()]
        expr = chol.getDelassusCholeskyExpression()
        assert rel_err(expr @ dx, np.einsum("bij,bj->bi", ref["osim_inverse"], dx)) < tol
        assert rel_err(expr.solve(dx), np.einsum("bij,bj->bi", ref["osim"], dx)) < tol
    if mu == 0.0:  # updateDamping refactorises with another mu
        chol.updateDamping(0.05)
        r2 = om.contact_cholesky(q, desc, mu=0.05)
        assert rel_err(chol.getInverseOperationalSpaceInertiaMatrix().cpu().numpy(), r2["osim_inverse"]) < tol
    # the SOA layout through the C ABI gives the same bits
    B, n, nc, nv = q.shape[0], chol.size(), chol.constraintDim(), model.nv
    outs = [torch.empty((k, B), dtype=torch.float64, device="cuda") for k in (n * n, n * n, nc * nc, nc * nc, nv * nv, nc * nv)]
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    _capi.check(_capi.lib().gb_contact_cholesky(data.dev.h, _capi.GB_FP64, data.constraint_set.h, float(mu),
                                                _capi.GB_LAYOUT_SOA, B, P(_dev(np.ascontiguousarray(q.T))),
                                                *(P(o) for o in outs), None))
    torch.cuda.synchronize()
    for o, k in zip(outs, ("matrix", "inverse", "osim_inverse", "osim", "minv", "jminv")):
        assert np.array_equal(o.cpu().numpy().T.reshape(got[k].shape), got[k].cpu().numpy()), k


def desc_dim(desc):
    return int(sum(3 if int(d[0]) == 0 else 6 for d in desc))


def test_contact_cholesky_without_constraints_and_errors():
    """With no constraint the KKT matrix is M and its inverse M^-1; mu < 0 and a set of another
    model are refused."""
    model = MODELS["humanoid32"]()
    om = OracleModel(model)
    q, v, x = sm.random_inputs(model, 16, 3)
    data = pg.createData(model)
    chol = pg.ContactCholeskyDecomposition(model)
    chol.compute(model, data, [], None, 0.0, q=_dev(q))
    M = om.crba(q)
    M = np.triu(M) + np.swapaxes(np.triu(M, 1), 1, 2)
    assert rel_err(chol.matrix().cpu().numpy(), M) < FP64_TOL
    assert rel_err(chol.inverse().cpu().numpy(), om.aba_derivatives(q, v, x)[3]) < 1e-11
    with pytest.raises(ValueError):
        chol.compute(model, data, [], None, -1.0, q=_dev(q))
    other = pg.createData(MODELS["tree12"]())
    pg.initConstraintDynamics(MODELS["tree12"](), other, [])
    L = _capi.lib()
    qq = np.ascontiguousarray(q[:2])
    rc = L.gb_contact_cholesky(data.dev.h, _capi.GB_FP64, other.constraint_set.h, 0.0, _capi.GB_LAYOUT_INSTANCE, 2,
                               qq.ctypes.data_as(C.c_void_p), None, None, None, None, None, None, None)
    assert rc == _capi.GB_ERR_INVALID_ARGUMENT

