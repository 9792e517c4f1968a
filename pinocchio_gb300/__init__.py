"""pinocchio_gb300 -- batched rigid-body dynamics on one NVIDIA GB300 (sm_103a).

A drop-in for the batched dynamics path of Pinocchio: RNEA, ABA, CRBA (+ tree
Cholesky), the analytical RNEA / ABA derivatives and the rneaInParallel /
abaInParallel batch entry points, computed by hand-written CUDA kernels
behind the C ABI of ``include/pinocchio_gb300.h``.
"""
from .model import (  # noqa: F401
    Convention,
    Inertia,
    JointModelFreeFlyer,
    JointModelPlanar,
    JointModelPrismaticUnaligned,
    JointModelPX,
    JointModelPY,
    JointModelPZ,
    JointModelRevoluteUnaligned,
    JointModelRevoluteUnboundedUnaligned,
    JointModelMimic,
    JointModelRUBX,
    JointModelRUBY,
    JointModelRUBZ,
    JointModelRX,
    JointModelRY,
    JointModelRZ,
    JointModelSpherical,
    JointModelSphericalZYX,
    JointModelComposite,
    JointModelTranslation,
    Model,
    SE3,
)
from . import sample_models  # noqa: F401
from .constraints import (  # noqa: F401
    CONTACT_3D,
    CONTACT_6D,
    LOCAL,
    LOCAL_WORLD_ALIGNED,
    WORLD,
    BaumgarteCorrectorParameters,
    ContactType,
    ProximalSettings,
    ReferenceFrame,
    RigidConstraintData,
    RigidConstraintModel,
)
from .urdf import buildModelFromUrdf, buildModelFromXML, load_model, save_model  # noqa: F401
from .mjcf import buildModelFromMJCF, buildModelFromMJCFXML  # noqa: F401
from .api import (  # noqa: F401
    ContactCholeskyDecomposition,
    Data,
    ModelPool,
    aba,
    abaDerivativesVJP,
    abaInParallel,
    checkNumeric,
    computeABADerivatives,
    computeConstraintDynamicsDerivatives,
    computeGeneralizedGravity,
    computeJointJacobians,
    computeKKTContactDynamicMatrixInverse,
    computeMinverse,
    computeRNEADerivatives,
    computeStaticTorque,
    computeStaticTorqueDerivatives,
    constraintDynamics,
    copyAsync,
    crba,
    crbaCholesky,
    createData,
    forwardDynamics,
    forwardKinematics,
    impulseDynamics,
    initConstraintDynamics,
    integrate,
    numericStatus,
    nonLinearEffects,
    rnea,
    rneaInParallel,
)


def build(force: bool = False) -> str:
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    from . import _build

    return _build.build(force=force)
