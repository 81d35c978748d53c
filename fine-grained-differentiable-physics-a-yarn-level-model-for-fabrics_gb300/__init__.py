"""GB300-native yarn-level cloth step (sm_103a CUDA behind a C ABI).

The package exposes the reference's cloth interface (Cloth, Environment,
PhysicsCloth, SimStep, EigenSolver) and the batched ClothBatch, all backed by
libyarnsim.so. There is no CPU fallback: without the CUDA library every call
raises.
"""
from .buildlib import build, LIB_PATH
from .cloth import (PI, ClothBatch, ClothSpec, ClothState, Cloth, EigenSolver, Environment, InitPose,
                    PhysicsCloth, SimStep, Wind, WovenPattern, Yarn)
from ._native import YarnSimError, load as load_library, library_path

__all__ = [
    "build", "LIB_PATH", "PI", "ClothBatch", "ClothSpec", "ClothState", "Cloth", "EigenSolver", "Environment",
    "InitPose", "PhysicsCloth", "SimStep", "Wind", "WovenPattern", "Yarn", "YarnSimError", "load_library",
    "library_path",
]
