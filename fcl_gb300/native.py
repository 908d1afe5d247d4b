"""ctypes binding of the C ABI in include/fclgpu.h (fcl_gb300/_build/libfclgpu.so).

There is no CPU fallback: if the native library is missing or fails to load, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfclgpu.so")

FCLGPU_OK = 0
FCLGPU_ERR_INVALID_ARGUMENT = -1
FCLGPU_ERR_CAPACITY = -4
FCLGPU_ERR_STACK_DEPTH = -6
FCLGPU_ERR_DEVICE_STATUS = -7
FCLGPU_ERR_NOT_INITIALIZED = -8
FCLGPU_ERR_UNSUPPORTED_ = -9
PLAIN_FP64 = 0
FP32_RECHECK = 1


class FclGpuError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        super().__init__(f"{where}: status {code} ({status_string(code)}) {detail}".strip())


class MeshInfo(C.Structure):
    _fields_ = [("num_vertices", C.c_int64), ("num_tris", C.c_int64), ("num_nodes", C.c_int64),
                ("max_depth", C.c_int32), ("reserved", C.c_int32), ("max_abs_coord", C.c_double),
                ("device_bytes", C.c_int64)]


class CollideRequest(C.Structure):
    _fields_ = [("num_max_contacts", C.c_int32), ("precision", C.c_int32), ("enable_statistics", C.c_int32),
                ("budget", C.c_int32)]


class FrontRequest(C.Structure):
    _fields_ = [("num_max_contacts", C.c_int32), ("precision", C.c_int32)]


class FrontResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("contact_offsets", C.c_void_p), ("contacts", C.c_void_p),
                ("contacts_capacity", C.c_int64), ("front_offsets", C.c_void_p), ("front", C.c_void_p),
                ("front_capacity", C.c_int64), ("num_bv_tests", C.c_void_p), ("num_leaf_tests", C.c_void_p),
                ("total_contacts", C.c_int64), ("total_front", C.c_int64)]


class CollideResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("offsets", C.c_void_p), ("contacts", C.c_void_p),
                ("contacts_capacity", C.c_int64), ("num_bv_tests", C.c_void_p), ("num_leaf_tests", C.c_void_p),
                ("num_rechecks", C.c_void_p), ("total_contacts", C.c_int64)]


class ContactResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("offsets", C.c_void_p), ("ids", C.c_void_p), ("pos", C.c_void_p),
                ("normal", C.c_void_p), ("depth", C.c_void_p), ("capacity", C.c_int64),
                ("total_contacts", C.c_int64)]


class CcdRequest(C.Structure):
    _fields_ = [("num_max_iterations", C.c_int64), ("toc_err", C.c_double), ("motion_type", C.c_int32),
                ("solver_type", C.c_int32), ("precision", C.c_int32), ("reserved", C.c_int32)]


class CcdResult(C.Structure):
    _fields_ = [("is_collide", C.c_void_p), ("time_of_contact", C.c_void_p), ("contact_tf1", C.c_void_p),
                ("contact_tf2", C.c_void_p), ("iterations", C.c_void_p)]


class DistanceRequest(C.Structure):
    _fields_ = [("enable_nearest_points", C.c_int32), ("precision", C.c_int32), ("enable_statistics", C.c_int32),
                ("reserved", C.c_int32)]


class DistanceResult(C.Structure):
    _fields_ = [("min_distance", C.c_void_p), ("ids", C.c_void_p), ("nearest_points", C.c_void_p),
                ("margins", C.c_void_p), ("within_margin", C.c_void_p), ("num_bv_tests", C.c_void_p),
                ("num_leaf_tests", C.c_void_p), ("num_rechecks", C.c_void_p)]


class GeometryRef(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32)]


class BpCollideRequest(C.Structure):
    _fields_ = [("num_max_contacts", C.c_int64), ("precision", C.c_int32), ("exhaustive", C.c_int32)]


class BpCollideResult(C.Structure):
    _fields_ = [("num_contacts", C.c_void_p), ("num_objects", C.c_void_p), ("first_object", C.c_void_p),
                ("total_candidates", C.c_int64), ("total_node_visits", C.c_int64)]


class BpContactsRequest(C.Structure):
    _fields_ = [("num_max_contacts", C.c_int64), ("precision", C.c_int32), ("reserved", C.c_int32)]


class BpContactsResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("offsets", C.c_void_p), ("contacts", C.c_void_p), ("capacity", C.c_int64),
                ("total_contacts", C.c_int64), ("total_candidates", C.c_int64), ("total_node_visits", C.c_int64)]


class BpSelfDistanceResult(C.Structure):
    _fields_ = [("min_distance", C.c_double), ("o1", C.c_int32), ("o2", C.c_int32), ("b1", C.c_int32),
                ("b2", C.c_int32), ("nearest_points", C.c_double * 6), ("total_candidates", C.c_int64)]


class GjkSolverParams(C.Structure):
    _fields_ = [("gjk_tolerance", C.c_double), ("epa_tolerance", C.c_double), ("gjk_max_iterations", C.c_int32),
                ("epa_max_iterations", C.c_int32)]


class BpDistanceRequest(C.Structure):
    _fields_ = [("enable_nearest_points", C.c_int32), ("precision", C.c_int32)]


class BpDistanceResult(C.Structure):
    _fields_ = [("min_distance", C.c_void_p), ("object", C.c_void_p), ("ids", C.c_void_p),
                ("nearest_points", C.c_void_p), ("total_candidates", C.c_int64), ("total_node_visits", C.c_int64)]


class RobotDesc(C.Structure):
    _fields_ = [("num_links", C.c_int32), ("joint_axis", C.c_void_p), ("link_offset", C.c_void_p),
                ("link_geometry", C.c_void_p), ("link_geometry_tf", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("max_waypoints_per_step", C.c_int64), ("memory_budget_bytes", C.c_int64),
                ("precision", C.c_int32), ("compute_clearance", C.c_int32)]


class MotionResult(C.Structure):
    _fields_ = [("first_colliding_waypoint", C.c_int32), ("clearance_waypoint", C.c_int32),
                ("clearance_link", C.c_int32), ("clearance_object", C.c_int32), ("min_clearance", C.c_double),
                ("latency_ms", C.c_double), ("queue_ms", C.c_double), ("num_steps", C.c_int32),
                ("reserved", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("waypoints", C.c_int64), ("queries", C.c_int64), ("candidates", C.c_int64),
                ("busy_ms", C.c_double), ("max_step_waypoints", C.c_int64), ("collide_ms", C.c_double),
                ("distance_ms", C.c_double)]


class MeshShapeRequest(C.Structure):
    _fields_ = [("mode", C.c_int32), ("reserved", C.c_int32), ("num_max_contacts", C.c_int64)]


class MeshShapeContactsResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("offsets", C.c_void_p), ("tris", C.c_void_p), ("capacity", C.c_int64),
                ("total_contacts", C.c_int64), ("pos", C.c_void_p), ("normal", C.c_void_p),
                ("penetration_depth", C.c_void_p)]


class MeshShapeResult(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("min_distance", C.c_void_p), ("tri", C.c_void_p),
                ("nearest_points", C.c_void_p), ("num_bv_tests", C.c_void_p), ("num_leaf_tests", C.c_void_p)]


GEOM_SHAPE = 0
GEOM_MESH = 1
FCLGPU_ERR_PENDING = -10
FCLGPU_ERR_INCORRECT_DATA = -11
FCLGPU_ERR_UNSUPPORTED = -9

_lib = None

# every function the header declares, with (restype, argtypes)
_VP = C.c_void_p
_SIGS = {
    "fclgpu_status_string": (C.c_char_p, [C.c_int]),
    "fclgpu_last_error_detail": (C.c_char_p, []),
    "fclgpu_init": (C.c_int, [C.c_int]),
    "fclgpu_mesh_create": (C.c_int, [_VP, C.c_int64, _VP, C.c_int64, C.POINTER(C.c_void_p)]),
    "fclgpu_mesh_create_on_device": (C.c_int, [_VP, C.c_int64, _VP, C.c_int64, C.POINTER(C.c_void_p), _VP]),
    "fclgpu_mesh_update_model": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, _VP]),
    "fclgpu_mesh_update_model_device": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, _VP]),
    "fclgpu_mesh_destroy": (C.c_int, [_VP]),
    "fclgpu_mesh_get_info": (C.c_int, [_VP, C.POINTER(MeshInfo)]),
    "fclgpu_mesh_get_nodes": (C.c_int, [_VP, _VP, _VP]),
    "fclgpu_mesh_update": (C.c_int, [_VP, _VP, C.c_int64, _VP]),
    "fclgpu_mesh_update_device": (C.c_int, [_VP, _VP, C.c_int64, _VP]),
    "fclgpu_mesh_replace": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, _VP]),
    "fclgpu_mesh_replace_device": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, _VP]),
    "fclgpu_collide_batch_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                              C.POINTER(CollideRequest), C.POINTER(CollideResult), _VP]),
    "fclgpu_collide_batch": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                       C.POINTER(CollideRequest), C.POINTER(CollideResult), _VP]),
    "fclgpu_collide_front_batch_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP, _VP,
                                                    _VP, C.POINTER(FrontRequest), C.POINTER(FrontResult), _VP]),
    "fclgpu_collide_front_batch": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP, _VP, _VP,
                                             C.POINTER(FrontRequest), C.POINTER(FrontResult), _VP]),
    "fclgpu_continuous_collide_batch_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                                         _VP, _VP, C.POINTER(CcdRequest), C.POINTER(CcdResult), _VP]),
    "fclgpu_continuous_collide_batch": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP, _VP,
                                                  _VP, C.POINTER(CcdRequest), C.POINTER(CcdResult), _VP]),
    "fclgpu_collide_contacts_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                                 C.POINTER(CollideRequest), C.POINTER(ContactResult), _VP]),
    "fclgpu_collide_contacts": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                          C.POINTER(CollideRequest), C.POINTER(ContactResult), _VP]),
    "fclgpu_distance_batch_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                               C.POINTER(DistanceRequest), C.POINTER(DistanceResult), _VP]),
    "fclgpu_distance_batch": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                        C.POINTER(DistanceRequest), C.POINTER(DistanceResult), _VP]),
    "fclgpu_distance_batch_noalloc": (C.c_int, [_VP, C.c_int32, _VP, C.c_int32, C.c_int64, _VP, _VP, _VP,
                                                C.POINTER(DistanceRequest), C.POINTER(DistanceResult), _VP]),
    "fclgpu_kernel_launch_count": (C.c_int64, []),
    "fclgpu_last_kernel_time": (C.c_int, [C.POINTER(C.c_double)]),
    "fclgpu_set_collide_tuning": (C.c_int, [C.c_int32, C.c_int32, C.c_int32]),
    "fclgpu_get_collide_tuning": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fclgpu_shapeset_create": (C.c_int, [_VP, C.c_int32, _VP, C.c_int64, C.POINTER(C.c_void_p)]),
    "fclgpu_shapeset_destroy": (C.c_int, [_VP]),
    "fclgpu_shape_batch_device": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "fclgpu_shape_batch": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "fclgpu_shape_collide_batch": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "fclgpu_set_gjk_solver_params": (C.c_int, [C.POINTER(GjkSolverParams)]),
    "fclgpu_set_collide_test_limits": (C.c_int, [C.c_int64, C.c_int64, C.c_int32]),
    "fclgpu_set_collide_persistent": (C.c_int, [C.c_int32, C.c_int64, C.c_int32]),
    "fclgpu_collide_persistent_fallbacks": (C.c_int64, []),
    "fclgpu_get_gjk_solver_params": (C.c_int, [C.POINTER(GjkSolverParams)]),
    "fclgpu_last_shape_kernel_time": (C.c_int, [C.POINTER(C.c_double)]),
    "fclgpu_broadphase_create": (C.c_int, [_VP, _VP, C.c_int32, _VP, C.c_int32, _VP, C.POINTER(C.c_void_p)]),
    "fclgpu_broadphase_update": (C.c_int, [_VP, _VP, C.c_int32, _VP]),
    "fclgpu_broadphase_destroy": (C.c_int, [_VP]),
    "fclgpu_broadphase_get_aabbs": (C.c_int, [_VP, _VP]),
    "fclgpu_broadphase_collide_device": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpCollideRequest),
                                                   C.POINTER(BpCollideResult), _VP]),
    "fclgpu_broadphase_collide": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpCollideRequest),
                                            C.POINTER(BpCollideResult), _VP]),
    "fclgpu_broadphase_collide_contacts_device": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpContactsRequest),
                                                            C.POINTER(BpContactsResult), _VP]),
    "fclgpu_broadphase_collide_contacts": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpContactsRequest),
                                                     C.POINTER(BpContactsResult), _VP]),
    "fclgpu_broadphase_self_collide_contacts_device": (C.c_int, [_VP, C.POINTER(BpContactsRequest),
                                                                 C.POINTER(BpContactsResult), _VP]),
    "fclgpu_broadphase_self_collide_contacts": (C.c_int, [_VP, C.POINTER(BpContactsRequest),
                                                          C.POINTER(BpContactsResult), _VP]),
    "fclgpu_broadphase_self_distance": (C.c_int, [_VP, C.POINTER(BpDistanceRequest), C.POINTER(BpSelfDistanceResult),
                                                  _VP]),
    "fclgpu_broadphase_distance_device": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpDistanceRequest),
                                                    C.POINTER(BpDistanceResult), _VP]),
    "fclgpu_broadphase_distance": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.POINTER(BpDistanceRequest),
                                             C.POINTER(BpDistanceResult), _VP]),
    "fclgpu_broadphase_last_phase_ms": (C.c_int, [_VP]),
    "fclgpu_server_create": (C.c_int, [_VP, C.POINTER(RobotDesc), C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "fclgpu_server_submit": (C.c_int, [_VP, _VP, _VP, C.c_int32, C.POINTER(C.c_int64)]),
    "fclgpu_server_wait": (C.c_int, [_VP, C.c_int64, C.c_double, C.POINTER(MotionResult)]),
    "fclgpu_server_get_stats": (C.c_int, [_VP, C.POINTER(ServerStats)]),
    "fclgpu_server_link_poses": (C.c_int, [_VP, _VP, _VP, C.c_int32, _VP]),
    "fclgpu_server_destroy": (C.c_int, [_VP]),
    "fclgpu_mesh_shape_batch_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int64, _VP, _VP, _VP, _VP,
                                                 C.POINTER(MeshShapeRequest), C.POINTER(MeshShapeResult), _VP]),
    "fclgpu_mesh_shape_batch": (C.c_int, [_VP, C.c_int32, _VP, C.c_int64, _VP, _VP, _VP, _VP,
                                          C.POINTER(MeshShapeRequest), C.POINTER(MeshShapeResult), _VP]),
    "fclgpu_mesh_shape_contacts_device": (C.c_int, [_VP, C.c_int32, _VP, C.c_int64, _VP, _VP, _VP, _VP, C.c_int64,
                                                    C.POINTER(MeshShapeContactsResult), _VP]),
    "fclgpu_mesh_shape_contacts": (C.c_int, [_VP, C.c_int32, _VP, C.c_int64, _VP, _VP, _VP, _VP, C.c_int64,
                                             C.POINTER(MeshShapeContactsResult), _VP]),
}


class Shape(C.Structure):
    _fields_ = [("type", C.c_int32), ("vertex_offset", C.c_int32), ("vertex_count", C.c_int32),
                ("reserved", C.c_int32), ("params", C.c_double * 3)]


class ShapeResult(C.Structure):
    _fields_ = [("hit", C.c_void_p), ("normal", C.c_void_p), ("point", C.c_void_p), ("depth", C.c_void_p),
                ("distance", C.c_void_p), ("p1", C.c_void_p), ("p2", C.c_void_p), ("status", C.c_void_p)]


def exported_symbols() -> list[str]:
    return list(_SIGS)


def lib():
    """Loads the native library (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(code: int) -> str:
    try:
        return lib().fclgpu_status_string(code).decode()
    except Exception:  # library not loadable
        return "?"


def check(code: int, where: str) -> None:
    if code != FCLGPU_OK:
        detail = lib().fclgpu_last_error_detail()
        raise FclGpuError(code, where, detail.decode() if detail else "")
