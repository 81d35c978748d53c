"""GB300-native yarn-level cloth step (sm_103a CUDA behind a C ABI).

The package exposes the reference's cloth interface (Cloth, Environment,
PhysicsCloth, SimStep, EigenSolver), the batched ClothBatch and the
parameter-learning interface (YarnSimNetHeter, differentiable rollouts), all
backed by libyarnsim.so. There is no CPU fallback: without the CUDA library every call
raises.
"""
from .buildlib import build, LIB_PATH
from .cloth import (PI, ClothBatch, ClothSpec, ClothState, Cloth, EigenSolver, Environment, InitPose,
                    PhysicsCloth, SimStep, StepStats, Wind, WovenPattern, Yarn, Adjoint, STATE_KEYS)
from ._native import YarnSimError, load as load_library, library_path
from .collide import Collider, Collision, cloth_mesh_topology
from .learn import (PARAM_NAMES, YarnSimNetHeter, YarnSimNetHomo, YarnSimNetColli, YarnSimNetControl, constraint_para, invert_constraint_para, position_loss, rollout,
                    rollout_with_jacobian, two_yarn_spec, CheckpointedRollout, rollout_adjoint,
                    two_yarn_param_grad)
from .precond import LearnedPreconditioner, train as train_preconditioner, training_specs
from .render import RenderCloth, RenderType, obj_text, render_batch_cloth
from . import h5
from . import control
from . import drivers
from .drivers import DropOnSphere, sim_collision, sim_control, sim_heter, sim_homo

__all__ = [
    "build", "LIB_PATH", "PI", "ClothBatch", "ClothSpec", "ClothState", "Cloth", "EigenSolver", "Environment",
    "InitPose", "PhysicsCloth", "SimStep", "StepStats", "Wind", "WovenPattern", "Yarn", "YarnSimError", "load_library",
    "library_path", "PARAM_NAMES", "YarnSimNetHeter", "constraint_para", "invert_constraint_para", "position_loss",
    "rollout", "rollout_with_jacobian", "two_yarn_spec", "Collider", "Collision", "cloth_mesh_topology",
    "LearnedPreconditioner", "train_preconditioner", "training_specs", "RenderCloth", "RenderType", "obj_text",
    "render_batch_cloth", "drivers", "DropOnSphere", "sim_collision", "sim_control", "sim_heter", "sim_homo",
    "Adjoint", "STATE_KEYS", "CheckpointedRollout", "rollout_adjoint", "two_yarn_param_grad", "YarnSimNetHomo",
    "YarnSimNetColli", "YarnSimNetControl",
]
