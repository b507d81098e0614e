"""GB300 spherical vertex model: the hot path of DanielMSussman/curvedSpaceVertexModel as
hand-written sm_103a CUDA behind a C ABI (include/svm.h, libsvm.so), with host classes that mirror
the reference's model / updater / simulation interface."""
from ._lib import LIBPATH, SVMError, device_count, lib  # noqa: F401
from .model import (  # noqa: F401
    PI,
    Simulation,
    Topology,
    brownianDynamics,
    dotProducts,
    energyMinimizerFIRE,
    neighborList,
    noiseSource,
    random_cell_centres,
    random_vertex_directors,
    sphericalSelfPropelledParticle,
    sphericalVectorialVicsek,
    sphericalVertexModel,
    sphericalVertexModelBatch,
    velocityVerlet,
    warmStartNetwork,
)
from .trajectory import dynamicalFeatures, logSpacedIntegers, run_trajectory, vectorValueNetCDF  # noqa: F401

__all__ = [
    "LIBPATH", "SVMError", "device_count", "lib", "PI", "Simulation", "Topology", "brownianDynamics",
    "dotProducts", "energyMinimizerFIRE", "neighborList", "noiseSource", "random_cell_centres", "random_vertex_directors",
    "sphericalSelfPropelledParticle", "sphericalVectorialVicsek", "sphericalVertexModel",
    "sphericalVertexModelBatch", "velocityVerlet", "warmStartNetwork", "dynamicalFeatures", "logSpacedIntegers", "run_trajectory",
    "vectorValueNetCDF",
]
