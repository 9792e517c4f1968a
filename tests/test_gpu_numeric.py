"""The numeric status word (gb_numeric_status / pg.numericStatus / pg.checkNumeric):
host-injected NaN inputs and a model with a massless leaf (a zero joint-space inertia,
the pivot the reference's LLT in PerformStYSInversion would fail on) are reported with
GB_ERR_NUMERIC; valid calls report nothing; the other configurations of the batch are
unaffected.  No kernel faults: the failing arithmetic only produces NaN / inf."""
import numpy as np
import pytest

import pinocchio_gb300 as pg
from oracle.oracle import OracleModel
from pinocchio_gb300 import _capi
from pinocchio_gb300 import model as gm
from pinocchio_gb300 import sample_models as sm
from util import FP64_TOL, MIXED_TOL, rel_err

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _massless_leaf_chain():
    """A 3-link revolute chain whose last link has no mass and no rotational inertia."""
    rng = np.random.default_rng(4)
    model = gm.Model()
    parent = 0
    for k, axis in enumerate((gm.JointModelRZ(), gm.JointModelRY(), gm.JointModelRX())):
        j = model.addJoint(parent, axis, sm.random_placement(rng), f"j{k}")
        Y = sm.random_inertia(rng) if k < 2 else gm.Inertia(0.0, np.zeros(3), np.zeros(6))
        model.appendBodyToJoint(j, Y)
        parent = j
    return model


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("layout", ["thread", "warp"])
def test_valid_calls_report_nothing_and_nan_inputs_are_reported(precision, layout):
    model = sm.humanoid32(1)
    data = pg.createData(model, precision)
    if layout == "warp":
        _capi.check(_capi.lib().gb_model_set_layout(data.dev.h, _capi.GB_FUNC_ABA, _capi.GB_INSTANCE_PER_WARP))
        _capi.check(_capi.lib().gb_model_set_layout(data.dev.h, _capi.GB_FUNC_RNEA, _capi.GB_INSTANCE_PER_WARP))
    q, v, x = sm.random_inputs(model, 96, 5)
    tau = 10.0 * x
    assert pg.numericStatus(data) == 0
    pg.aba(model, data, _dev(q), _dev(v), _dev(tau))
    pg.rnea(model, data, _dev(q), _dev(v), _dev(x))
    pg.computeABADerivatives(model, data, _dev(q), _dev(v), _dev(tau))
    pg.crbaCholesky(model, data, _dev(q))
    assert pg.numericStatus(data) == 0
    pg.checkNumeric(data)  # does not raise
    bad = tau.copy()
    bad[17, 5] = np.nan
    ddq = pg.aba(model, data, _dev(q), _dev(v), _dev(bad)).cpu().numpy()
    flags = pg.numericStatus(data, reset=False)
    assert flags & _capi.GB_NUMERIC_NONFINITE
    with pytest.raises(_capi.GBError) as err:
        pg.checkNumeric(data)  # reads and resets
    assert err.value.code == _capi.GB_ERR_NUMERIC
    assert pg.numericStatus(data) == 0
    ok = np.arange(96) != 17
    assert not np.isfinite(ddq[17]).all() and np.isfinite(ddq[ok]).all()
    ref = OracleModel(model).aba(q[ok], v[ok], tau[ok])
    assert rel_err(ddq[ok], ref) < (FP64_TOL if precision == "fp64" else MIXED_TOL)
    # NaN in q: the RNEA output and the derivative sweeps' ddq report it too
    qb = q.copy()
    qb[3, 9] = np.nan
    pg.rnea(model, data, _dev(qb), _dev(v), _dev(x))
    assert pg.numericStatus(data) & _capi.GB_NUMERIC_NONFINITE
    pg.computeABADerivatives(model, data, _dev(qb), _dev(v), _dev(tau))
    assert pg.numericStatus(data) != 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singular_inertia_pivot_is_reported(precision):
    model = _massless_leaf_chain()
    data = pg.createData(model, precision)
    q, v, x = sm.random_inputs(model, 8, 1)
    pg.aba(model, data, _dev(q), _dev(v), _dev(x))
    assert pg.numericStatus(data) & _capi.GB_NUMERIC_PIVOT
    pg.crbaCholesky(model, data, _dev(q))
    assert pg.numericStatus(data) & _capi.GB_NUMERIC_PIVOT
    pg.computeABADerivatives(model, data, _dev(q), _dev(v), _dev(x))
    assert pg.numericStatus(data) & _capi.GB_NUMERIC_PIVOT
    # with armature the joint-space inertia is positive again
    model.armature = np.full(model.nv, 0.1)
    data = pg.createData(model, precision)
    pg.aba(model, data, _dev(q), _dev(v), _dev(x))
    pg.computeABADerivatives(model, data, _dev(q), _dev(v), _dev(x))
    assert pg.numericStatus(data) == 0
