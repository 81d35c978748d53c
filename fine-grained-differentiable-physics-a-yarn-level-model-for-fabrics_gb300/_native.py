"""ctypes binding of libyarnsim.so (the C ABI declared in include/yarnsim.h).

The library is the only compute path: if it is missing or fails to load, every
entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

from . import buildlib as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

YS_OK, YS_ERR_ARG, YS_ERR_CUDA, YS_ERR_NONFINITE, YS_ERR_MAXITER = 0, 1, 2, 3, 4
YS_ON_DEVICE = 1

EXPORTED = [
    "ys_last_error", "ys_batch_create", "ys_batch_destroy", "ys_batch_get_info", "ys_cloth_node_offset",
    "ys_cloth_dim", "ys_set_state", "ys_get_state", "ys_set_wind", "ys_set_winds", "ys_assemble", "ys_export_system",
    "ys_solve", "ys_get_solution", "ys_step", "ys_apply_system", "ys_synchronize", "ys_profile",
    "ys_profile_read", "ys_apply_system_noalloc", "ys_tangent_count", "ys_tangent_enable", "ys_tangent_seed",
    "ys_tangent_set_state", "ys_tangent_get_state", "ys_step_tangent", "ys_cloth_mesh_topology",
    "ys_collider_create", "ys_collider_destroy", "ys_collider_set_positions", "ys_collider_find_pairs",
    "ys_collider_get_pairs", "ys_collider_find_impacts", "ys_collider_get_impacts", "ys_use_graphs",
    "ys_step_graphed", "ys_autotune", "ys_set_pcg_schedule", "ys_autotune_results", "ys_set_producer_threads", "ys_gnn_param_count", "ys_gnn_create", "ys_gnn_destroy", "ys_gnn_get_params",
    "ys_gnn_dims", "ys_gnn_set_objective",
    "ys_gnn_set_params", "ys_gnn_train_step", "ys_gnn_loss_grad", "ys_set_preconditioner", "ys_precond_info",
    "ys_get_system_slots", "ys_tc_gemm_bf16", "ys_precond_refresh", "ys_get_normals", "ys_collider_respond",
    "ys_collider_response_impacts", "ys_collider_respond_backward", "ys_step_tangent_ext",
    "ys_collider_set_max_zone_impacts", "ys_adjoint_create", "ys_adjoint_destroy", "ys_adjoint_step",
]
YS_PREC_JACOBI, YS_PREC_LEARNED = 0, 1
YS_TANGENT_EXACT, YS_TANGENT_REFERENCE = 0, 1
PROF_KINDS = ["geom", "edges", "bends", "faces", "gather", "shear", "finalize", "pcg_setup", "spmv", "axpy", "dir",
              "update", "misc", "gnn", "precond", "pcg_persist"]


class ClothDesc(ctypes.Structure):
    """ys_cloth_desc"""
    _fields_ = [
        ("width", ctypes.c_int32), ("length", ctypes.c_int32),
        ("height", ctypes.c_double), ("L", ctypes.c_double), ("R", ctypes.c_double),
        ("pose", ctypes.c_int32), ("weave", ctypes.c_int32),
        ("warp_rho", _dp), ("warp_Y", _dp), ("warp_B", _dp),
        ("weft_rho", _dp), ("weft_Y", _dp), ("weft_B", _dp),
        ("kc", ctypes.c_double), ("kf", ctypes.c_double), ("df", ctypes.c_double),
        ("mu", ctypes.c_double), ("S", ctypes.c_double), ("handle_stiffness", ctypes.c_double),
        ("G", ctypes.c_double * 3), ("wind_vel", ctypes.c_double * 3),
        ("wind_density", ctypes.c_double), ("wind_drag", ctypes.c_double),
        ("n_handles", ctypes.c_int32), ("handles", _ip),
    ]


class SolveOpts(ctypes.Structure):
    """ys_solve_opts"""
    _fields_ = [("tol", ctypes.c_double), ("maxiter", ctypes.c_int32), ("check_every", ctypes.c_int32)]


class Schedule(ctypes.Structure):
    _fields_ = [("graphs", ctypes.c_int32), ("check_every", ctypes.c_int32), ("ms_per_step", ctypes.c_double),
                ("pcg", ctypes.c_int32), ("pcg_threads", ctypes.c_int32), ("pcg_cluster", ctypes.c_int32),
                ("producer_threads", ctypes.c_int32)]


class ClothStats(ctypes.Structure):
    """ys_cloth_stats"""
    _fields_ = [("ok", ctypes.c_int32), ("cg_iterations", ctypes.c_int32), ("cg_error", ctypes.c_double),
                ("hit_maxiter", ctypes.c_int32)]


class BatchInfo(ctypes.Structure):
    """ys_batch_info"""
    _fields_ = [("n_cloths", ctypes.c_int32), ("total_nodes", ctypes.c_int64), ("device_bytes", ctypes.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libyarnsim.so (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    path = _build.LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libyarnsim.so is not built (%s); run build() first" % path)
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.ys_last_error.restype = ctypes.c_char_p
    L.ys_batch_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ClothDesc), ctypes.c_int32, vp, ctypes.POINTER(vp)]
    L.ys_batch_destroy.argtypes = [vp]
    L.ys_batch_destroy.restype = None
    L.ys_batch_get_info.argtypes = [vp, ctypes.POINTER(BatchInfo)]
    L.ys_cloth_node_offset.argtypes = [vp, ctypes.c_int32]
    L.ys_cloth_node_offset.restype = ctypes.c_int64
    L.ys_cloth_dim.argtypes = [vp, ctypes.c_int32]
    L.ys_cloth_dim.restype = ctypes.c_int64
    L.ys_set_state.argtypes = [vp] + [vp] * 6 + [ctypes.c_int32]
    L.ys_get_state.argtypes = [vp] + [vp] * 6 + [ctypes.c_int32]
    L.ys_set_wind.argtypes = [vp, ctypes.c_int32, _dp]
    L.ys_set_winds.argtypes = [vp, vp, ctypes.c_int32]
    L.ys_assemble.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int32]
    L.ys_export_system.argtypes = [vp, ctypes.c_int32, _dp, _dp]
    L.ys_solve.argtypes = [vp, ctypes.POINTER(SolveOpts), ctypes.POINTER(ClothStats)]
    L.ys_get_solution.argtypes = [vp, vp, ctypes.c_int32]
    L.ys_step.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int32, ctypes.POINTER(SolveOpts),
                          ctypes.POINTER(ClothStats)]
    L.ys_apply_system.argtypes = [vp, vp, vp, ctypes.c_int32]
    L.ys_apply_system_noalloc.argtypes = [vp, vp, vp]
    L.ys_tangent_count.argtypes = []
    L.ys_tangent_count.restype = ctypes.c_int32
    L.ys_tangent_enable.argtypes = [vp, ctypes.c_int32]
    L.ys_tangent_seed.argtypes = [vp, vp, vp, vp, vp, vp]
    L.ys_tangent_set_state.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.c_int32]
    L.ys_tangent_get_state.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.c_int32]
    L.ys_step_tangent.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int32, vp, ctypes.c_int32, vp]
    L.ys_step_tangent_ext.argtypes = [vp, ctypes.c_double, vp, vp, ctypes.c_int32, vp, ctypes.c_int32, vp]
    L.ys_cloth_mesh_topology.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp]
    L.ys_use_graphs.argtypes = [vp, ctypes.c_int32]
    L.ys_step_graphed.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int32, vp, vp]
    L.ys_autotune.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int32, vp]
    L.ys_set_pcg_schedule.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    L.ys_autotune_results.argtypes = [vp, vp, ctypes.c_int32]
    L.ys_set_producer_threads.argtypes = [vp, ctypes.c_int32]
    L.ys_autotune_results.restype = ctypes.c_int32
    L.ys_collider_create.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int32, ctypes.c_int32, vp,
                                     ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp, ctypes.POINTER(vp)]
    L.ys_collider_destroy.argtypes = [vp]
    L.ys_collider_destroy.restype = None
    L.ys_collider_set_positions.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int32]
    L.ys_collider_find_pairs.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.ys_collider_get_pairs.argtypes = [vp, vp, ctypes.c_int64]
    L.ys_collider_find_impacts.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.ys_collider_get_impacts.argtypes = [vp, vp, ctypes.c_int64]
    L.ys_synchronize.argtypes = [vp]
    L.ys_profile.argtypes = [vp, ctypes.c_int32]
    L.ys_profile_read.argtypes = [vp, _dp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                  ctypes.c_int32]
    L.ys_gnn_param_count.argtypes = []
    L.ys_gnn_param_count.restype = ctypes.c_int32
    L.ys_gnn_create.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.ys_gnn_dims.argtypes = [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    L.ys_gnn_dims.restype = None
    L.ys_gnn_set_objective.argtypes = [vp, ctypes.c_int32]
    L.ys_gnn_destroy.argtypes = [vp]
    L.ys_gnn_destroy.restype = None
    L.ys_gnn_get_params.argtypes = [vp, vp]
    L.ys_gnn_set_params.argtypes = [vp, vp]
    L.ys_gnn_train_step.argtypes = [vp, vp, ctypes.c_uint64, ctypes.c_float, _dp]
    L.ys_gnn_loss_grad.argtypes = [vp, vp, vp, ctypes.c_uint64, _dp, vp, vp, vp]
    L.ys_set_preconditioner.argtypes = [vp, ctypes.c_int32, vp]
    L.ys_precond_refresh.argtypes = [vp, ctypes.c_int32]
    L.ys_get_normals.argtypes = [vp, vp, ctypes.c_int32]
    L.ys_precond_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.ys_get_system_slots.argtypes = [vp, vp, vp]
    L.ys_tc_gemm_bf16.argtypes = [ctypes.c_int32, vp, vp, vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    L.ys_collider_respond.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, vp, vp,
                                      ctypes.POINTER(ResponseInfo)]
    L.ys_collider_response_impacts.argtypes = [vp, vp, ctypes.c_int64]
    L.ys_collider_set_max_zone_impacts.argtypes = [vp, ctypes.c_int32]
    L.ys_collider_respond_backward.argtypes = [vp, vp, vp, ctypes.c_int32, vp, vp, vp, vp, vp]
    L.ys_adjoint_create.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(vp)]
    L.ys_adjoint_destroy.argtypes = [vp]
    L.ys_adjoint_destroy.restype = None
    L.ys_adjoint_step.argtypes = [vp, ctypes.c_double, vp, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                  ctypes.POINTER(vp), vp, ctypes.c_int32, vp, vp]
    for name in EXPORTED:
        if name not in ("ys_batch_destroy", "ys_last_error", "ys_cloth_node_offset", "ys_cloth_dim",
                        "ys_tangent_count", "ys_collider_destroy", "ys_gnn_destroy", "ys_gnn_param_count",
                        "ys_adjoint_destroy", "ys_gnn_dims"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def last_error() -> str:
    return load().ys_last_error().decode()


class Impact(ctypes.Structure):
    """ys_impact (include/yarnsim.h)."""
    _fields_ = [("type", ctypes.c_int32), ("nodes", ctypes.c_int32 * 4), ("t", ctypes.c_double),
                ("w", ctypes.c_double * 4), ("n", ctypes.c_double * 3), ("pair", ctypes.c_int64)]


class ResponseInfo(ctypes.Structure):
    """ys_response_info (include/yarnsim.h)."""
    _fields_ = [("rounds", ctypes.c_int32), ("converged", ctypes.c_int32), ("changed", ctypes.c_int32),
                ("zones", ctypes.c_int32), ("infeasible", ctypes.c_int32), ("zone_overflow", ctypes.c_int32),
                ("impacts", ctypes.c_int64), ("projections", ctypes.c_int64), ("reverted", ctypes.c_int32),
                ("pad_", ctypes.c_int32), ("detect_ms", ctypes.c_double), ("zones_ms", ctypes.c_double)]


class YarnSimError(RuntimeError):
    def __init__(self, status, where):
        super().__init__("%s failed (status %d): %s" % (where, status, last_error()))
        self.status = status


def check(status, where):
    if status not in (YS_OK,):
        raise YarnSimError(status, where)
