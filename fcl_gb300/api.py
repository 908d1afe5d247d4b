"""Python mirror of FCL's proximity-query API for BVHModel<OBBRSS> meshes.

Names, argument meaning and defaults follow FCL 0.7.0:
  BVHModel.beginModel/addSubModel/endModel  geometry/bvh/BVH_model.h:56-227
  CollisionRequest / CollisionResult / Contact  narrowphase/collision_request.h:52-106,
                                                collision_result.h:52-93, contact.h:48-91
  DistanceRequest / DistanceResult          narrowphase/distance_request.h:52-113,
                                            distance_result.h
  CollisionObject                           narrowphase/collision_object.h:50-157
  collide(o1, o2, request, result)          narrowphase/collision.h:55-66
  distance(o1, o2, request, result)         narrowphase/distance.h:51-62
plus the batched entry points collide_batch / distance_batch.  Everything runs
through the C ABI (include/fclgpu.h) on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import ClassVar

import numpy as np

from . import native as N

PRECISIONS = {"fp64": N.PLAIN_FP64, "plain": N.PLAIN_FP64, "fp32": N.FP32_RECHECK, "fp32_recheck": N.FP32_RECHECK}


def _prec(p) -> int:
    if isinstance(p, int):
        return p
    return PRECISIONS[p]


class BVHModel:
    """BVHModel<OBBRSS<double>>: triangles + vertices, BVH built by endModel() on the host
    (build="host") or on the GPU (build="device"; the same tree node for node)."""

    def __init__(self, build: str = "host"):
        self._verts: list[np.ndarray] = []
        self._tris: list[np.ndarray] = []
        self._nv = 0
        self.handle = None
        self.build_state = "empty"
        if build not in ("host", "device"):
            raise N.FclGpuError(N.FCLGPU_ERR_INVALID_ARGUMENT, "BVHModel", "build is 'host' or 'device'")
        self.build = build

    # geometry/bvh/BVH_model-inl.h:207-248
    def beginModel(self, num_tris: int = 0, num_vertices: int = 0) -> int:
        self._verts, self._tris, self._nv = [], [], 0
        self.build_state = "begun"
        return 0

    # BVH_model-inl.h:416-446
    def addSubModel(self, vertices, triangles=None) -> int:
        if self.build_state != "begun":
            return -8  # BVH_ERR_BUILD_OUT_OF_SEQUENCE
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self._verts.append(v)
        if triangles is not None:
            t = np.ascontiguousarray(triangles, dtype=np.int64).reshape(-1, 3) + self._nv
            self._tris.append(t.astype(np.int32))
        self._nv += v.shape[0]
        return 0

    def addTriangle(self, p1, p2, p3) -> int:
        return self.addSubModel(np.array([p1, p2, p3], np.float64), np.array([[0, 1, 2]], np.int32))

    # BVH_model-inl.h:450-517
    def endModel(self) -> int:
        if self.build_state != "begun":
            return -8
        V = np.concatenate(self._verts) if self._verts else np.zeros((0, 3))
        T = np.concatenate(self._tris) if self._tris else np.zeros((0, 3), np.int32)
        if V.shape[0] == 0 or T.shape[0] == 0:
            raise N.FclGpuError(-5, "endModel", "model with no triangles and vertices")
        self.vertices = np.ascontiguousarray(V)
        self.tri_indices = np.ascontiguousarray(T, dtype=np.int32)
        h = C.c_void_p()
        if self.build == "device":
            N.check(N.lib().fclgpu_mesh_create_on_device(self.vertices.ctypes.data, V.shape[0],
                                                         self.tri_indices.ctypes.data, T.shape[0], C.byref(h), None),
                    "fclgpu_mesh_create_on_device")
        else:
            N.check(N.lib().fclgpu_mesh_create(self.vertices.ctypes.data, V.shape[0], self.tri_indices.ctypes.data,
                                               T.shape[0], C.byref(h)), "fclgpu_mesh_create")
        self.handle = h
        self.build_state = "processed"
        return 0

    # BVH_model-inl.h:624-651 (beginUpdateModel), :653-701 (updateVertex, updateTriangle,
    # updateSubModel), :703-727 (endUpdateModel; the refit runs on the GPU)
    def beginUpdateModel(self) -> int:
        if self.build_state not in ("processed", "updated"):
            return -10  # BVH_ERR_BUILD_EMPTY_PREVIOUS_FRAME
        self._upd: list[np.ndarray] = []
        self._nupd = 0
        self.build_state = "update_begun"
        return 0

    def updateVertex(self, p) -> int:
        return self.updateSubModel(np.asarray(p, np.float64).reshape(1, 3))

    def updateTriangle(self, p1, p2, p3) -> int:
        return self.updateSubModel(np.array([p1, p2, p3], np.float64))

    def updateSubModel(self, ps) -> int:
        if self.build_state != "update_begun":
            return -8  # BVH_ERR_BUILD_OUT_OF_SEQUENCE
        v = np.ascontiguousarray(ps, dtype=np.float64).reshape(-1, 3)
        self._upd.append(v)
        self._nupd += v.shape[0]
        return 0

    def endUpdateModel(self, refit: bool = True, bottomup: bool = True) -> int:
        """Bottom-up only (the top-down refit is not on the GPU path): refit = True refits
        the tree on the GPU; refit = False rebuilds it on the GPU and then refits it over
        both frames, as FCL does."""
        if self.build_state != "update_begun":
            return -8
        if not bottomup:
            raise N.FclGpuError(N.FCLGPU_ERR_UNSUPPORTED, "endUpdateModel", "only the bottom-up refit")
        V = np.concatenate(self._upd) if self._upd else np.zeros((0, 3))
        if V.shape[0] != self.num_vertices:
            return -7  # BVH_ERR_INCORRECT_DATA
        self.update_vertices(V, refit=refit)
        return 0

    def update_vertices(self, vertices, stream=None, refit: bool = True) -> None:
        """beginUpdateModel + updateVertex for all vertices + endUpdateModel(refit) at once:
        numpy (host) or a CUDA torch tensor (device), (nv, 3) float64."""
        if hasattr(vertices, "data_ptr"):
            N.check(N.lib().fclgpu_mesh_update_model_device(self.handle, vertices.data_ptr(), vertices.shape[0],
                                                            int(bool(refit)), stream),
                    "fclgpu_mesh_update_model_device")
        else:
            V = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
            N.check(N.lib().fclgpu_mesh_update_model(self.handle, V.ctypes.data, V.shape[0], int(bool(refit)), stream),
                    "fclgpu_mesh_update_model")
            self.vertices = V
        self.build_state = "updated"

    # geometry/bvh/BVH_model-inl.h:521-620
    def beginReplaceModel(self) -> int:
        if self.build_state not in ("processed", "updated"):
            return -10  # BVH_ERR_BUILD_EMPTY_PREVIOUS_FRAME
        self._upd = []
        self._nupd = 0
        self.build_state = "replace_begun"
        return 0

    def replaceVertex(self, p) -> int:
        return self.replaceSubModel(np.asarray(p, np.float64).reshape(1, 3))

    def replaceTriangle(self, p1, p2, p3) -> int:
        return self.replaceSubModel(np.array([p1, p2, p3], np.float64))

    def replaceSubModel(self, ps) -> int:
        if self.build_state != "replace_begun":
            return -8  # BVH_ERR_BUILD_OUT_OF_SEQUENCE
        v = np.ascontiguousarray(ps, dtype=np.float64).reshape(-1, 3)
        self._upd.append(v)
        self._nupd += v.shape[0]
        return 0

    def endReplaceModel(self, refit: bool = True, bottomup: bool = True) -> int:
        """Bottom-up only: refit = True refits the tree on the GPU without a previous frame;
        refit = False rebuilds it on the GPU (buildTree)."""
        if self.build_state != "replace_begun":
            return -8
        if not bottomup:
            raise N.FclGpuError(N.FCLGPU_ERR_UNSUPPORTED, "endReplaceModel", "only the bottom-up refit")
        V = np.concatenate(self._upd) if self._upd else np.zeros((0, 3))
        if V.shape[0] != self.num_vertices:
            return -7  # BVH_ERR_INCORRECT_DATA
        self.replace_vertices(V, refit=refit)
        return 0

    def replace_vertices(self, vertices, stream=None, refit: bool = True) -> None:
        """beginReplaceModel + replaceVertex for all vertices + endReplaceModel(refit) at
        once: numpy (host) or a CUDA torch tensor (device), (nv, 3) float64."""
        if hasattr(vertices, "data_ptr"):
            N.check(N.lib().fclgpu_mesh_replace_device(self.handle, vertices.data_ptr(), vertices.shape[0],
                                                       int(bool(refit)), stream), "fclgpu_mesh_replace_device")
        else:
            V = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
            N.check(N.lib().fclgpu_mesh_replace(self.handle, V.ctypes.data, V.shape[0], int(bool(refit)), stream),
                    "fclgpu_mesh_replace")
            self.vertices = V
        self.build_state = "processed"

    @classmethod
    def from_arrays(cls, vertices, triangles, build: str = "host") -> "BVHModel":
        m = cls(build=build)
        m.beginModel()
        m.addSubModel(vertices, triangles)
        m.endModel()
        return m

    def info(self) -> N.MeshInfo:
        inf = N.MeshInfo()
        N.check(N.lib().fclgpu_mesh_get_info(self.handle, C.byref(inf)), "fclgpu_mesh_get_info")
        return inf

    @property
    def num_tris(self) -> int:
        return int(self.tri_indices.shape[0])

    @property
    def num_vertices(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def num_bvs(self) -> int:
        return int(self.info().num_nodes)

    def get_nodes(self):
        """(nodes (n,30) float64, first_child (n,) int32) in FCL's node order."""
        n = self.num_bvs
        out = np.empty((n, 30), np.float64)
        fc = np.empty(n, np.int32)
        N.check(N.lib().fclgpu_mesh_get_nodes(self.handle, out.ctypes.data, fc.ctypes.data), "fclgpu_mesh_get_nodes")
        return out, fc

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.fclgpu_mesh_destroy(h)
            self.handle = None


def transform(R=None, t=None) -> np.ndarray:
    tf = np.zeros((3, 4))
    tf[:, :3] = np.eye(3) if R is None else np.asarray(R, np.float64)
    if t is not None:
        tf[:, 3] = np.asarray(t, np.float64)
    return tf


@dataclass
class CollisionObject:
    geometry: "BVHModel | ShapeRef"
    tf: np.ndarray = field(default_factory=lambda: transform())

    def setTransform(self, R, t):
        self.tf = transform(R, t)


# GJKSolverType (narrowphase/gjk_solver_type.h): FCL's default is GST_LIBCCD, whose
# MPR penetration and GJK distance come from libccd; this library provides FCL's own
# solver, GST_INDEP (GJKSolver_indep).  Shape pairs asked for GST_LIBCCD are rejected
# with FCLGPU_ERR_UNSUPPORTED; mesh-mesh pairs use no GJK solver and accept either.
GST_LIBCCD = 0
GST_INDEP = 1


@dataclass
class ShapeRef:
    """A convex shape of a ShapeSet used as a CollisionObject's geometry (FCL's Box,
    Sphere, Capsule, Cylinder, Cone and Convex behind shared_ptr<CollisionGeometry>)."""
    shapes: "ShapeSet"
    index: int


@dataclass
class CollisionRequest:
    num_max_contacts: int = 1
    enable_contact: bool = False
    enable_statistics: bool = False
    precision: str = "fp32"
    gjk_solver_type: int = GST_LIBCCD
    gjk_tolerance: float = 1e-6  # CollisionRequest::gjk_tolerance (collision_request.h:94)


@dataclass
class Contact:
    NONE: ClassVar[int] = -1  # Contact::NONE, the primitive id of a shape (contact.h)
    o1: object
    o2: object
    b1: int
    b2: int
    # set when CollisionRequest.enable_contact (contact.h: pos, normal, penetration_depth)
    pos: np.ndarray | None = None
    normal: np.ndarray | None = None
    penetration_depth: float = 0.0

    def __lt__(self, other):  # contact-inl.h:98-104
        if self.b1 == other.b1:
            return self.b2 < other.b2
        return self.b1 < other.b1


@dataclass
class CollisionResult:
    contacts: list = field(default_factory=list)
    num_bv_tests: int = 0
    num_leaf_tests: int = 0

    def numContacts(self) -> int:
        return len(self.contacts)

    def isCollision(self) -> bool:
        return len(self.contacts) > 0

    def getContact(self, i: int) -> Contact:
        return self.contacts[i]

    def clear(self):
        self.contacts = []


@dataclass
class DistanceRequest:
    enable_nearest_points: bool = False
    enable_signed_distance: bool = False
    rel_err: float = 0.0
    abs_err: float = 0.0
    enable_statistics: bool = False
    precision: str = "fp32"
    gjk_solver_type: int = GST_LIBCCD
    distance_tolerance: float = 1e-6  # DistanceRequest::distance_tolerance (distance_request.h:99)


@dataclass
class DistanceResult:
    min_distance: float = float(np.finfo(np.float64).max)
    nearest_points: np.ndarray = field(default_factory=lambda: np.zeros((2, 3)))
    o1: object = None
    o2: object = None
    b1: int = -1
    b2: int = -1

    def clear(self):
        self.min_distance = float(np.finfo(np.float64).max)
        self.nearest_points = np.zeros((2, 3))
        self.o1 = self.o2 = None
        self.b1 = self.b2 = -1


def _unsupported(req):
    # enable_signed_distance needs no check: FCL's signed-distance step
    # (narrowphase/distance-inl.h:147-187) runs only when min_distance < 0, which the
    # BVHModel distance traversal never reports (triangle and RSS distances are >= 0).
    if getattr(req, "rel_err", 0.0) or getattr(req, "abs_err", 0.0):
        raise N.FclGpuError(-9, "distance", "rel_err/abs_err must be 0 on the GPU path")


SOLVER_DEFAULTS = (2.0097183471152322e-14, 2.0097183471152322e-14, 128, 255)


def set_gjk_solver_params(gjk_tolerance=SOLVER_DEFAULTS[0], epa_tolerance=SOLVER_DEFAULTS[1],
                          gjk_max_iterations=SOLVER_DEFAULTS[2], epa_max_iterations=SOLVER_DEFAULTS[3]):
    """GJKSolver_indep's parameters for every later shape, mesh-shape and broadphase
    call (process-wide; fclgpu_set_gjk_solver_params).  Defaults: the solver's own."""
    p = N.GjkSolverParams(gjk_tolerance, epa_tolerance, gjk_max_iterations, epa_max_iterations)
    N.check(N.lib().fclgpu_set_gjk_solver_params(C.byref(p)), "fclgpu_set_gjk_solver_params")


def get_gjk_solver_params():
    p = N.GjkSolverParams()
    N.check(N.lib().fclgpu_get_gjk_solver_params(C.byref(p)), "fclgpu_get_gjk_solver_params")
    return (p.gjk_tolerance, p.epa_tolerance, p.gjk_max_iterations, p.epa_max_iterations)


class _RequestSolver:
    """The solver fcl::collide / fcl::distance build for one call: the request's
    tolerance (collision-inl.h:164-170, distance-inl.h:211-215), default iteration caps;
    the previous process-wide parameters come back afterwards."""

    def __init__(self, gjk_tol, epa_tol):
        self.want = (gjk_tol, epa_tol, SOLVER_DEFAULTS[2], SOLVER_DEFAULTS[3])

    def __enter__(self):
        self.prev = get_gjk_solver_params()
        set_gjk_solver_params(*self.want)

    def __exit__(self, *exc):
        set_gjk_solver_params(*self.prev)


def _shape_solver(request, where):
    if request.gjk_solver_type != GST_INDEP:
        raise N.FclGpuError(N.FCLGPU_ERR_UNSUPPORTED_, where,
                            "GST_LIBCCD (libccd's MPR and GJK) is not provided: set gjk_solver_type = GST_INDEP "
                            "for FCL's own GJK/EPA (GJKSolver_indep)")


def _mesh_first(o1, o2):
    """(mesh object, shape object): FCL calls the BVH-shape functions mesh first
    whichever argument order it got (collision-inl.h:124-131, distance-inl.h:117-126)."""
    return (o1, o2) if isinstance(o1.geometry, BVHModel) else (o2, o1)


def _collide_shapes(o1, o2, request, result):
    """Shape x shape and mesh x shape pairs of fcl::collide (GST_INDEP)."""
    _shape_solver(request, "collide")
    g1, g2 = o1.geometry, o2.geometry
    room = max(0, request.num_max_contacts - len(result.contacts))
    if isinstance(g1, ShapeRef) and isinstance(g2, ShapeRef):
        if g1.shapes is not g2.shapes:
            raise N.FclGpuError(N.FCLGPU_ERR_INVALID_ARGUMENT, "collide", "both shapes must come from one ShapeSet")
        ia, ib = np.array([g1.index], np.int32), np.array([g2.index], np.int32)
        if not request.enable_contact:
            hit = np.zeros(1, np.int32)
            N.check(N.lib().fclgpu_shape_collide_batch(g1.shapes.handle, 1, ia.ctypes.data, ib.ctypes.data,
                                                       np.ascontiguousarray(o1.tf).ctypes.data,
                                                       np.ascontiguousarray(o2.tf).ctypes.data, hit.ctypes.data, None),
                    "fclgpu_shape_collide_batch")
            if hit[0] and room > 0:
                result.contacts.append(Contact(g1, g2, Contact.NONE, Contact.NONE))
            return result.numContacts()
        if request.num_max_contacts > 1:
            types = [int(g.shapes._types[g.index]) for g in (g1, g2)]
            if types == [0, 0]:  # boxBoxIntersect can add up to four contacts
                raise N.FclGpuError(N.FCLGPU_ERR_UNSUPPORTED_, "collide",
                                    "box-box contacts beyond the deepest one (num_max_contacts > 1)")
        out = shape_batch(g1.shapes, ia, ib, o1.tf[None], o2.tf[None])
        if out["hit"][0] and room > 0:
            result.contacts.append(Contact(g1, g2, Contact.NONE, Contact.NONE, out["point"][0].copy(),
                                           out["normal"][0].copy(), float(out["depth"][0])))
        return result.numContacts()
    om, os_ = _mesh_first(o1, o2)
    gs = os_.geometry
    out = mesh_shape_contacts_batch([om.geometry], gs.shapes, np.zeros(1, np.int32), np.array([gs.index], np.int32),
                                    om.tf[None], os_.tf[None], num_max_contacts=max(1, room),
                                    enable_contact=request.enable_contact)
    for k, t in enumerate(out["tris"][:room]):
        if request.enable_contact:  # Contact(mesh, shape, tri, NONE, contactp, -normal, penetration)
            result.contacts.append(Contact(om.geometry, gs, int(t), Contact.NONE, out["pos"][k].copy(),
                                           out["normal"][k].copy(), float(out["penetration_depth"][k])))
        else:
            result.contacts.append(Contact(om.geometry, gs, int(t), Contact.NONE))
    return result.numContacts()


def _distance_shapes(o1, o2, request, result):
    """Shape x shape and mesh x shape pairs of fcl::distance (GST_INDEP)."""
    _shape_solver(request, "distance")
    g1, g2 = o1.geometry, o2.geometry
    if isinstance(g1, ShapeRef) and isinstance(g2, ShapeRef):
        if g1.shapes is not g2.shapes:
            raise N.FclGpuError(N.FCLGPU_ERR_INVALID_ARGUMENT, "distance", "both shapes must come from one ShapeSet")
        out = shape_batch(g1.shapes, np.array([g1.index], np.int32), np.array([g2.index], np.int32), o1.tf[None],
                          o2.tf[None])
        d = float(out["dist"][0]) if not out["hit"][0] else -1.0
        cand = (d, g1, g2, Contact.NONE, Contact.NONE, np.stack([out["p1"][0], out["p2"][0]]))
    else:
        om, os_ = _mesh_first(o1, o2)
        gs = os_.geometry
        out = mesh_shape_batch([om.geometry], gs.shapes, np.zeros(1, np.int32), np.array([gs.index], np.int32),
                               om.tf[None], os_.tf[None], mode="distance")
        cand = (float(out["min_distance"][0]), om.geometry, gs, int(out["tri"][0]), Contact.NONE,
                out["nearest_points"][0].copy())
    d, a, b, b1, b2, pts = cand
    if result.min_distance > d:
        result.min_distance = d
        result.o1, result.o2, result.b1, result.b2 = a, b, b1, b2
        if request.enable_nearest_points:
            result.nearest_points = pts
    return result.min_distance


def collide(o1: CollisionObject, o2: CollisionObject, request: CollisionRequest, result: CollisionResult) -> int:
    """fcl::collide; appends to result like FCL.  Mesh x mesh (BVHModel<OBBRSS>), shape x
    shape and mesh x shape pairs (ShapeRef geometries; GJKSolver_indep)."""
    _unsupported(request)
    if request.num_max_contacts == 0:
        return 0
    if isinstance(o1.geometry, ShapeRef) or isinstance(o2.geometry, ShapeRef):
        _shape_solver(request, "collide")
        with _RequestSolver(request.gjk_tolerance, request.gjk_tolerance):
            return _collide_shapes(o1, o2, request, result)
    if request.enable_contact:
        if request.enable_statistics:
            raise N.FclGpuError(N.FCLGPU_ERR_UNSUPPORTED, "collide", "statistics are not produced with contacts")
        out = collide_contacts_batch([o1.geometry, o2.geometry], np.array([[0, 1]], np.int32), o1.tf[None],
                                     o2.tf[None], num_max_contacts=request.num_max_contacts,
                                     precision=request.precision)
        room = max(0, request.num_max_contacts - len(result.contacts))
        for i in range(min(room, out["total_contacts"])):
            b1, b2 = out["contacts"][i]
            result.contacts.append(Contact(o1.geometry, o2.geometry, int(b1), int(b2), out["pos"][i].copy(),
                                           out["normal"][i].copy(), float(out["depth"][i])))
        return result.numContacts()
    out = collide_batch([o1.geometry, o2.geometry], np.array([[0, 1]], np.int32), o1.tf[None], o2.tf[None],
                        pair_of_query=None, num_max_contacts=request.num_max_contacts, precision=request.precision,
                        statistics=request.enable_statistics)
    room = max(0, request.num_max_contacts - len(result.contacts))
    for b1, b2 in out["contacts"][:room]:
        result.contacts.append(Contact(o1.geometry, o2.geometry, int(b1), int(b2)))
    if request.enable_statistics:
        result.num_bv_tests = int(out["num_bv_tests"][0])
        result.num_leaf_tests = int(out["num_leaf_tests"][0])
    return result.numContacts()


def distance(o1: CollisionObject, o2: CollisionObject, request: DistanceRequest, result: DistanceResult) -> float:
    """fcl::distance; DistanceResult::update semantics.  Mesh x mesh, shape x shape and
    mesh x shape pairs (ShapeRef geometries; GJKSolver_indep)."""
    _unsupported(request)
    if isinstance(o1.geometry, ShapeRef) or isinstance(o2.geometry, ShapeRef):
        _shape_solver(request, "distance")
        with _RequestSolver(request.distance_tolerance, SOLVER_DEFAULTS[1]):
            return _distance_shapes(o1, o2, request, result)
    out = distance_batch([o1.geometry, o2.geometry], np.array([[0, 1]], np.int32), o1.tf[None], o2.tf[None],
                         nearest_points=request.enable_nearest_points, precision=request.precision)
    d = float(out["min_distance"][0])
    if result.min_distance > d:
        result.min_distance = d
        result.o1, result.o2 = o1.geometry, o2.geometry
        result.b1, result.b2 = int(out["ids"][0, 0]), int(out["ids"][0, 1])
        if request.enable_nearest_points:
            result.nearest_points = out["nearest_points"][0].copy()
    return result.min_distance


CCDM = {"trans": 0, "linear": 1, "screw": 2, "spline": 3}   # CCDMotionType (continuous_collision_request.h:48)
CCDC = {"naive": 0, "conservative_advancement": 1, "ray_shooting": 2, "polynomial_solver": 3}   # CCDSolverType


@dataclass
class ContinuousCollisionRequest:
    num_max_iterations: int = 10
    toc_err: float = 1e-4
    ccd_motion_type: str = "trans"
    ccd_solver_type: str = "naive"
    precision: str = "fp32"


@dataclass
class ContinuousCollisionResult:
    is_collide: bool = False
    time_of_contact: float = 1.0
    contact_tf1: np.ndarray = field(default_factory=lambda: transform())
    contact_tf2: np.ndarray = field(default_factory=lambda: transform())


def continuous_collide_batch(meshes, pairs, tf1_beg, tf1_end, tf2_beg, tf2_end, pair_of_query=None,
                             num_max_iterations=10, toc_err=1e-4, motion="trans", solver="naive", precision="fp32",
                             stream=None):
    """Batched fcl::continuousCollide on mesh pairs (solver "naive" (FCL's default) or
    "conservative_advancement"; motion "trans" (FCL's default), "linear" or "screw").
    Returns is_collide (n,), time_of_contact (n,), contact_tf1/contact_tf2 (n,3,4; zero
    where no collision) and, with conservative advancement on numpy inputs, iterations
    (n,).  numpy inputs use the host entry point, torch CUDA tensors the device one."""
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    req = N.CcdRequest(int(num_max_iterations), float(toc_err), CCDM[motion], CCDC[solver], _prec(precision), 0)
    hs = _handles(meshes)
    if _is_torch(tf2_beg):
        import torch
        dev = tf2_beg.device
        n = tf2_beg.shape[0]
        hit = torch.zeros(n, dtype=torch.int32, device=dev)
        toc = torch.zeros(n, dtype=torch.float64, device=dev)
        c1 = torch.zeros((n, 3, 4), dtype=torch.float64, device=dev)
        c2 = torch.zeros((n, 3, 4), dtype=torch.float64, device=dev)
        s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        res = N.CcdResult(hit.data_ptr(), toc.data_ptr(), c1.data_ptr(), c2.data_ptr())
        N.check(N.lib().fclgpu_continuous_collide_batch_device(
            hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
            None if pair_of_query is None else pair_of_query.data_ptr(),
            None if tf1_beg is None else tf1_beg.data_ptr(), None if tf1_end is None else tf1_end.data_ptr(),
            tf2_beg.data_ptr(), tf2_end.data_ptr(), C.byref(req), C.byref(res), s),
            "fclgpu_continuous_collide_batch_device")
        return {"is_collide": hit, "time_of_contact": toc, "contact_tf1": c1, "contact_tf2": c2}
    b0 = np.ascontiguousarray(tf2_beg, np.float64).reshape(-1, 12)
    b1 = np.ascontiguousarray(tf2_end, np.float64).reshape(-1, 12)
    n = b0.shape[0]
    a0 = None if tf1_beg is None else np.ascontiguousarray(tf1_beg, np.float64).reshape(-1, 12)
    a1 = None if tf1_end is None else np.ascontiguousarray(tf1_end, np.float64).reshape(-1, 12)
    pq = None if pair_of_query is None else np.ascontiguousarray(pair_of_query, np.int32)
    hit = np.zeros(n, np.int32)
    toc = np.zeros(n)
    c1 = np.zeros((n, 3, 4))
    c2 = np.zeros((n, 3, 4))
    its = np.zeros(n, np.int32) if solver == "conservative_advancement" else None
    res = N.CcdResult(hit.ctypes.data, toc.ctypes.data, c1.ctypes.data, c2.ctypes.data,
                      None if its is None else its.ctypes.data)
    N.check(N.lib().fclgpu_continuous_collide_batch(
        hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n, None if pq is None else pq.ctypes.data,
        None if a0 is None else a0.ctypes.data, None if a1 is None else a1.ctypes.data, b0.ctypes.data,
        b1.ctypes.data, C.byref(req), C.byref(res), stream), "fclgpu_continuous_collide_batch")
    out = {"is_collide": hit, "time_of_contact": toc, "contact_tf1": c1, "contact_tf2": c2}
    if its is not None:
        out["iterations"] = its
    return out


def continuousCollide(o1: CollisionObject, tf1_end, o2: CollisionObject, tf2_end,
                      request: ContinuousCollisionRequest, result: ContinuousCollisionResult) -> float:
    """fcl::continuousCollide(o1, tf1_end, o2, tf2_end, request, result) for two
    BVHModel<OBBRSS> objects (continuous_collision-inl.h:455-469): the motions run from the
    objects' transforms to tf1_end / tf2_end."""
    out = continuous_collide_batch([o1.geometry, o2.geometry], np.array([[0, 1]], np.int32), o1.tf[None],
                                   np.asarray(tf1_end, np.float64)[None], o2.tf[None],
                                   np.asarray(tf2_end, np.float64)[None],
                                   num_max_iterations=request.num_max_iterations, toc_err=request.toc_err,
                                   motion=request.ccd_motion_type, solver=request.ccd_solver_type,
                                   precision=request.precision)
    result.is_collide = bool(out["is_collide"][0])
    result.time_of_contact = float(out["time_of_contact"][0])
    if result.is_collide:
        result.contact_tf1 = out["contact_tf1"][0].copy()
        result.contact_tf2 = out["contact_tf2"][0].copy()
    return result.time_of_contact


def _handles(meshes):
    arr = (C.c_void_p * len(meshes))()
    for i, m in enumerate(meshes):
        arr[i] = m.handle.value if isinstance(m.handle, C.c_void_p) else m.handle
    return arr


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def collide_batch(meshes, pairs, tf1, tf2, pair_of_query=None, num_max_contacts=1, precision="fp32",
                  statistics=False, contacts=True, stream=None, budget=0):
    """Batched fcl::collide.  Host (numpy) inputs use the host entry point (copies in
    and out); torch CUDA tensors use the device entry point.  Returns a dict with
    counts, offsets, contacts (total, 2) and optional statistics."""
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    req = N.CollideRequest(int(num_max_contacts), _prec(precision), int(bool(statistics)), int(budget))
    hs = _handles(meshes)
    if _is_torch(tf2):
        return _collide_batch_torch(meshes, hs, pairs, tf1, tf2, pair_of_query, req, statistics, contacts, stream)
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(-1, 12)
    pq = None if pair_of_query is None else np.ascontiguousarray(pair_of_query, np.int32)
    counts = np.zeros(n, np.int32)
    offsets = np.zeros(n + 1, np.int64)
    st = [np.zeros(n, np.int64) for _ in range(3)] if statistics else [None] * 3
    cap = 0
    while True:
        buf = np.empty((max(cap, 1), 2), np.int32) if contacts else None
        res = N.CollideResult(counts.ctypes.data, offsets.ctypes.data, None if buf is None else buf.ctypes.data,
                              cap, *(None if a is None else a.ctypes.data for a in st), 0)
        rc = N.lib().fclgpu_collide_batch(hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
                                          None if pq is None else pq.ctypes.data,
                                          None if tf1a is None else tf1a.ctypes.data, tf2.ctypes.data,
                                          C.byref(req), C.byref(res), stream)
        if rc == N.FCLGPU_ERR_CAPACITY and contacts:
            cap = int(res.total_contacts)
            continue
        N.check(rc, "fclgpu_collide_batch")
        break
    out = {"counts": counts, "offsets": offsets, "total_contacts": int(res.total_contacts)}
    if contacts:
        out["contacts"] = buf[: res.total_contacts]
    if statistics:
        out["num_bv_tests"], out["num_leaf_tests"], out["num_rechecks"] = st
    return out


class BVHFrontList:
    """detail::BVHFrontList (geometry/bvh/detail/BVH_front.h): the (b1, b2) BV node pairs
    where the last traversal of a mesh pair stopped, to restart from at the next pose."""

    def __init__(self, nodes=None):
        self.nodes = np.zeros((0, 2), np.int32) if nodes is None else np.asarray(nodes, np.int32).reshape(-1, 2)

    def size(self) -> int:
        return int(self.nodes.shape[0])

    def clear(self):
        self.nodes = np.zeros((0, 2), np.int32)


def collide_front_batch(meshes, pairs, tf1, tf2, fronts=None, pair_of_query=None, num_max_contacts=1,
                        precision="fp32", statistics=False, stream=None):
    """Front-list collide (collide(node, front_list), collision_node-inl.h:72-82) of n
    queries: fronts is a list of n (m_i, 2) node-pair arrays from a previous call (or
    None: start from the roots).  Returns counts, contact_offsets, contacts (FCL's order
    for a front traversal), fronts (the new list per query) and optional statistics."""
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    hs = _handles(meshes)
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(-1, 12)
    pq = None if pair_of_query is None else np.ascontiguousarray(pair_of_query, np.int32)
    fin_off = fin = None
    if fronts is not None:
        if len(fronts) != n:
            raise N.FclGpuError(N.FCLGPU_ERR_INVALID_ARGUMENT, "collide_front_batch", "one front per query")
        arrs = [np.asarray(f.nodes if isinstance(f, BVHFrontList) else f, np.int32).reshape(-1, 2) for f in fronts]
        fin_off = np.concatenate([[0], np.cumsum([a.shape[0] for a in arrs])]).astype(np.int64)
        fin = np.ascontiguousarray(np.concatenate(arrs) if arrs else np.zeros((0, 2), np.int32), np.int32)
        if fin.shape[0] == 0:
            fin = np.zeros((1, 2), np.int32)
    req = N.FrontRequest(int(num_max_contacts), _prec(precision))
    counts = np.zeros(n, np.int32)
    coff = np.zeros(n + 1, np.int64)
    foff = np.zeros(n + 1, np.int64)
    st = [np.zeros(n, np.int64) for _ in range(2)] if statistics else [None] * 2
    ccap, fcap = max(16, n), max(64, 4 * n + (0 if fin is None else 2 * fin.shape[0]))
    for _ in range(3):
        cont = np.zeros((ccap, 2), np.int32)
        fr = np.zeros((fcap, 2), np.int32)
        res = N.FrontResult(counts.ctypes.data, coff.ctypes.data, cont.ctypes.data, ccap, foff.ctypes.data,
                            fr.ctypes.data, fcap, *(None if a is None else a.ctypes.data for a in st), 0, 0)
        rc = N.lib().fclgpu_collide_front_batch(hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
                                                None if pq is None else pq.ctypes.data,
                                                None if tf1a is None else tf1a.ctypes.data, tf2.ctypes.data,
                                                None if fin_off is None else fin_off.ctypes.data,
                                                None if fin is None else fin.ctypes.data, C.byref(req),
                                                C.byref(res), stream)
        if rc == N.FCLGPU_ERR_CAPACITY:
            ccap, fcap = max(ccap, int(res.total_contacts)), max(fcap, int(res.total_front))
            continue
        N.check(rc, "fclgpu_collide_front_batch")
        tf = int(res.total_front)
        out = {"counts": counts, "contact_offsets": coff, "contacts": cont[: int(res.total_contacts)],
               "front_offsets": foff, "front": fr[:tf],
               "fronts": [fr[foff[i]:foff[i + 1]].copy() for i in range(n)]}
        if statistics:
            out["num_bv_tests"], out["num_leaf_tests"] = st
        return out
    raise N.FclGpuError(N.FCLGPU_ERR_CAPACITY, "fclgpu_collide_front_batch", "totals changed between calls")


def collide_front(o1: "CollisionObject", o2: "CollisionObject", request: "CollisionRequest",
                  result: "CollisionResult", front_list: BVHFrontList) -> int:
    """collide(node, front_list) on a mesh pair (BVHModel<OBBRSS>): an empty front_list
    runs the full traversal and records the front, a non-empty one restarts from it
    (propagateBVHFrontListCollisionRecurse); front_list is updated in place."""
    if not (isinstance(o1.geometry, BVHModel) and isinstance(o2.geometry, BVHModel)):
        raise N.FclGpuError(N.FCLGPU_ERR_INVALID_ARGUMENT, "collide_front", "front lists are for mesh pairs")
    room = max(0, request.num_max_contacts - len(result.contacts))
    if room == 0:
        return result.numContacts()
    out = collide_front_batch([o1.geometry, o2.geometry], [[0, 1]], o1.tf[None], o2.tf[None],
                              fronts=[front_list.nodes], num_max_contacts=room, precision=request.precision)
    for b1, b2 in out["contacts"]:
        result.contacts.append(Contact(o1.geometry, o2.geometry, int(b1), int(b2)))
    front_list.nodes = out["fronts"][0]
    return result.numContacts()


_contacts_hint = {"cap": 1 << 16}


def collide_contacts_batch(meshes, pairs, tf1, tf2, pair_of_query=None, num_max_contacts=1, precision="fp32",
                           stream=None):
    """Batched fcl::collide with CollisionRequest::enable_contact = true.  Returns a dict
    with counts, offsets, total_contacts and per contact (query after query, in the
    reference's DFS order): contacts (b1, b2), pos (world), normal (world) and depth.
    numpy inputs use the host entry point; torch CUDA tensors the device one."""
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    req = N.CollideRequest(int(num_max_contacts), _prec(precision), 0, 0)
    hs = _handles(meshes)
    if _is_torch(tf2):
        import torch
        dev = tf2.device
        n = tf2.shape[0]
        counts = torch.zeros(n, dtype=torch.int32, device=dev)
        offsets = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        args = (hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
                None if pair_of_query is None else pair_of_query.data_ptr(),
                None if tf1 is None else tf1.data_ptr(), tf2.data_ptr(), C.byref(req))
        # buffers sized from the previous batch; a batch that outgrows them runs again
        cap = _contacts_hint["cap"]
        while True:
            ids = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=dev)
            pos = torch.empty((max(cap, 1), 3), dtype=torch.float64, device=dev)
            nrm = torch.empty((max(cap, 1), 3), dtype=torch.float64, device=dev)
            dep = torch.empty(max(cap, 1), dtype=torch.float64, device=dev)
            res = N.ContactResult(counts.data_ptr(), offsets.data_ptr(), ids.data_ptr(), pos.data_ptr(),
                                  nrm.data_ptr(), dep.data_ptr(), cap, 0)
            rc = N.lib().fclgpu_collide_contacts_device(*args, C.byref(res), s)
            if rc == N.FCLGPU_ERR_CAPACITY:
                cap = int(res.total_contacts * 1.25) + 1024
                _contacts_hint["cap"] = cap
                continue
            N.check(rc, "fclgpu_collide_contacts_device")
            break
        total = int(res.total_contacts)
        return {"counts": counts, "offsets": offsets, "total_contacts": total, "contacts": ids[:total],
                "pos": pos[:total], "normal": nrm[:total], "depth": dep[:total]}
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(-1, 12)
    pq = None if pair_of_query is None else np.ascontiguousarray(pair_of_query, np.int32)
    counts = np.zeros(n, np.int32)
    offsets = np.zeros(n + 1, np.int64)
    cap = _contacts_hint["cap"]
    while True:
        ids = np.empty((max(cap, 1), 2), np.int32)
        pos = np.empty((max(cap, 1), 3))
        nrm = np.empty((max(cap, 1), 3))
        dep = np.empty(max(cap, 1))
        res = N.ContactResult(counts.ctypes.data, offsets.ctypes.data, ids.ctypes.data, pos.ctypes.data,
                              nrm.ctypes.data, dep.ctypes.data, cap, 0)
        rc = N.lib().fclgpu_collide_contacts(hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
                                             None if pq is None else pq.ctypes.data,
                                             None if tf1a is None else tf1a.ctypes.data, tf2.ctypes.data,
                                             C.byref(req), C.byref(res), stream)
        if rc == N.FCLGPU_ERR_CAPACITY:
            cap = int(res.total_contacts)
            continue
        N.check(rc, "fclgpu_collide_contacts")
        break
    t = int(res.total_contacts)
    return {"counts": counts, "offsets": offsets, "total_contacts": t, "contacts": ids[:t], "pos": pos[:t],
            "normal": nrm[:t], "depth": dep[:t]}


def _collide_batch_torch(meshes, hs, pairs, tf1, tf2, pair_of_query, req, statistics, contacts, stream):
    """Device entry point.  The contacts buffer is sized from the previous batch (a
    batch that outgrows it is re-run once with the exact size)."""
    import torch
    dev = tf2.device
    n = tf2.shape[0]
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    offsets = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    st = [torch.zeros(n, dtype=torch.int64, device=dev) for _ in range(3)] if statistics else [None] * 3
    s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    cap = _contacts_hint["cap"] if contacts else 0
    buf = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=dev) if contacts else None
    while True:
        res = N.CollideResult(counts.data_ptr(), offsets.data_ptr(),
                              None if buf is None else buf.data_ptr(), cap,
                              *(None if a is None else a.data_ptr() for a in st), 0)
        rc = N.lib().fclgpu_collide_batch_device(
            hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
            None if pair_of_query is None else pair_of_query.data_ptr(),
            None if tf1 is None else tf1.data_ptr(), tf2.data_ptr(), C.byref(req), C.byref(res), s)
        if contacts and rc == N.FCLGPU_ERR_CAPACITY:
            cap = int(res.total_contacts * 1.25) + 1024
            _contacts_hint["cap"] = cap
            buf = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=dev)
            continue
        N.check(rc, "fclgpu_collide_batch_device")
        break
    out = {"counts": counts, "offsets": offsets, "total_contacts": int(res.total_contacts)}
    if contacts:
        out["contacts"] = buf[: res.total_contacts]
    if statistics:
        out["num_bv_tests"], out["num_leaf_tests"], out["num_rechecks"] = st
    return out


def distance_batch(meshes, pairs, tf1, tf2, pair_of_query=None, nearest_points=True, precision="fp32",
                   margins=None, statistics=False, stream=None, ids=True):
    """Batched fcl::distance.  Returns min_distance, ids (n,2), nearest_points (n,2,3)
    world frame, optional within_margin (distance <= margin) and statistics.  ids=False
    with nearest_points=False asks for the distances alone."""
    want_ids = bool(ids)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    req = N.DistanceRequest(int(bool(nearest_points)), _prec(precision), int(bool(statistics)), 0)
    hs = _handles(meshes)
    if _is_torch(tf2):
        import torch
        dev = tf2.device
        n = tf2.shape[0]
        d = torch.empty(n, dtype=torch.float64, device=dev)
        ids = torch.empty((n, 2), dtype=torch.int32, device=dev) if want_ids else None
        pts = torch.zeros((n, 2, 3), dtype=torch.float64, device=dev) if nearest_points else None
        within = torch.empty(n, dtype=torch.int32, device=dev) if margins is not None else None
        st = [torch.zeros(n, dtype=torch.int64, device=dev) for _ in range(3)] if statistics else [None] * 3
        res = N.DistanceResult(d.data_ptr(), None if ids is None else ids.data_ptr(),
                               None if pts is None else pts.data_ptr(),
                               None if margins is None else margins.data_ptr(),
                               None if within is None else within.data_ptr(),
                               *(None if a is None else a.data_ptr() for a in st))
        s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        N.check(N.lib().fclgpu_distance_batch_device(
            hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n,
            None if pair_of_query is None else pair_of_query.data_ptr(),
            None if tf1 is None else tf1.data_ptr(), tf2.data_ptr(), C.byref(req), C.byref(res), s),
            "fclgpu_distance_batch_device")
    else:
        tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
        n = tf2.shape[0]
        tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(-1, 12)
        pq = None if pair_of_query is None else np.ascontiguousarray(pair_of_query, np.int32)
        mg = None if margins is None else np.ascontiguousarray(margins, np.float64)
        d = np.empty(n, np.float64)
        ids = np.empty((n, 2), np.int32) if want_ids else None
        pts = np.zeros((n, 2, 3), np.float64) if nearest_points else None
        within = np.empty(n, np.int32) if margins is not None else None
        st = [np.zeros(n, np.int64) for _ in range(3)] if statistics else [None] * 3
        res = N.DistanceResult(d.ctypes.data, None if ids is None else ids.ctypes.data,
                               None if pts is None else pts.ctypes.data,
                               None if mg is None else mg.ctypes.data, None if within is None else within.ctypes.data,
                               *(None if a is None else a.ctypes.data for a in st))
        N.check(N.lib().fclgpu_distance_batch(
            hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n, None if pq is None else pq.ctypes.data,
            None if tf1a is None else tf1a.ctypes.data, tf2.ctypes.data, C.byref(req), C.byref(res), stream),
            "fclgpu_distance_batch")
    out = {"min_distance": d}
    if want_ids:
        out["ids"] = ids
    if nearest_points:
        out["nearest_points"] = pts
    if margins is not None:
        out["within_margin"] = within
    if statistics:
        out["num_bv_tests"], out["num_leaf_tests"], out["num_rechecks"] = st
    return out


# ---------------------------------------------------------------------------------
# Convex shapes (fcl::Box, Sphere, Capsule, Cylinder, Cone, Convex) with FCL's own
# GJK/EPA solver (GJKSolver_indep) and its closed-form pairs.
# ---------------------------------------------------------------------------------
class ShapeSet:
    """A device-resident set of convex shapes.  types/params/voff/vcnt/verts follow
    fcl_gb300.workloads.ShapeSet (params: box sides; sphere r; capsule/cylinder/cone
    r, lz; convex vertices [voff, voff+vcnt) of verts)."""

    def __init__(self, types, params, voff=None, vcnt=None, verts=None):
        types = np.ascontiguousarray(types, np.int32)
        n = types.shape[0]
        params = np.ascontiguousarray(params, np.float64).reshape(n, 3)
        voff = np.zeros(n, np.int32) if voff is None else np.asarray(voff, np.int32)
        vcnt = np.zeros(n, np.int32) if vcnt is None else np.asarray(vcnt, np.int32)
        verts = np.zeros((0, 3)) if verts is None else np.ascontiguousarray(verts, np.float64).reshape(-1, 3)
        arr = (N.Shape * n)()
        for i in range(n):
            arr[i].type = int(types[i])
            arr[i].vertex_offset = int(voff[i])
            arr[i].vertex_count = int(vcnt[i])
            for k in range(3):
                arr[i].params[k] = float(params[i, k])
        self._verts = verts if verts.shape[0] else np.zeros((1, 3))
        self._types = types
        h = C.c_void_p()
        N.check(N.lib().fclgpu_shapeset_create(arr, n, self._verts.ctypes.data, verts.shape[0], C.byref(h)),
                "fclgpu_shapeset_create")
        self.handle = h
        self.n = n

    @classmethod
    def from_workload(cls, s) -> "ShapeSet":
        return cls(s.type, s.params, s.voff, s.vcnt, s.verts)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.fclgpu_shapeset_destroy(h)
            self.handle = None


def shape_batch(shapes: ShapeSet, ia, ib, tf1, tf2, stream=None):
    """Batched fcl::collide (with contact) then, for separated pairs, fcl::distance.
    numpy inputs use the host entry point, torch CUDA tensors the device one."""
    if _is_torch(tf2):
        import torch
        dev = tf2.device
        n = tf2.shape[0]
        out = dict(hit=torch.zeros(n, dtype=torch.int32, device=dev),
                   normal=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                   point=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                   depth=torch.zeros(n, dtype=torch.float64, device=dev),
                   dist=torch.zeros(n, dtype=torch.float64, device=dev),
                   p1=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                   p2=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                   status=torch.zeros((n, 2), dtype=torch.int32, device=dev))
        res = N.ShapeResult(*(out[k].data_ptr() for k in ("hit", "normal", "point", "depth", "dist", "p1", "p2",
                                                           "status")))
        s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        N.check(N.lib().fclgpu_shape_batch_device(shapes.handle, n, ia.data_ptr(), ib.data_ptr(), tf1.data_ptr(),
                                                  tf2.data_ptr(), C.byref(res), s), "fclgpu_shape_batch_device")
        return out
    ia = np.ascontiguousarray(ia, np.int32)
    ib = np.ascontiguousarray(ib, np.int32)
    n = ia.shape[0]
    tf1 = np.ascontiguousarray(tf1, np.float64).reshape(n, 12)
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(n, 12)
    out = dict(hit=np.zeros(n, np.int32), normal=np.zeros((n, 3)), point=np.zeros((n, 3)), depth=np.zeros(n),
               dist=np.zeros(n), p1=np.zeros((n, 3)), p2=np.zeros((n, 3)), status=np.zeros((n, 2), np.int32))
    res = N.ShapeResult(*(out[k].ctypes.data for k in ("hit", "normal", "point", "depth", "dist", "p1", "p2",
                                                       "status")))
    N.check(N.lib().fclgpu_shape_batch(shapes.handle, n, ia.ctypes.data, ib.ctypes.data, tf1.ctypes.data,
                                       tf2.ctypes.data, C.byref(res), stream), "fclgpu_shape_batch")
    out["hit"] = out["hit"].astype(bool)
    return out


# ------------------------------------------------------------------ broadphase ----

class DynamicAABBTreeCollisionManager:
    """Device broadphase in the place of FCL's DynamicAABBTreeCollisionManager
    (broadphase/broadphase_dynamic_AABB_tree.h:56-157).

    Geometry comes from a registry, as CollisionObject's shared geometry does: a
    ShapeSet and a list of BVHModels.  Scene and query objects are geometry refs
    (n, 2) int32 rows (kind, index) -- kind 0 = shape set entry, 1 = mesh -- with
    3x4 poses.  registerObjects + setup build the device tree; update() takes new
    poses.  collide_batch / distance_batch run manager.collide(obj, ...,
    DefaultCollisionFunction) and manager.distance(obj, ..., DefaultDistanceFunction)
    for every query object (torch CUDA tensors stay on the device, numpy arrays go
    through the host entry points)."""

    def __init__(self, shapes: "ShapeSet | None" = None, meshes=()):
        self.shapes = shapes
        self.meshes = list(meshes)
        self.handle = None
        self._refs = None
        self._tf = None

    def registerObjects(self, refs, tf) -> None:
        self._refs = np.ascontiguousarray(refs, np.int32).reshape(-1, 2)
        self._tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
        self.setup()

    def setup(self) -> None:
        self._release()
        n = self._refs.shape[0]
        hs = (C.c_void_p * max(1, len(self.meshes)))(*[m.handle.value for m in self.meshes])
        h = C.c_void_p()
        N.check(N.lib().fclgpu_broadphase_create(self.shapes.handle if self.shapes is not None else None,
                                                 hs if self.meshes else None, len(self.meshes),
                                                 self._refs.ctypes.data, n, self._tf.ctypes.data, C.byref(h)),
                "fclgpu_broadphase_create")
        self.handle = h

    def size(self) -> int:
        return 0 if self._refs is None else int(self._refs.shape[0])

    def update(self, tf, stream=None) -> None:
        """New poses of every scene object (numpy on the host or a CUDA tensor)."""
        if _is_torch(tf):
            N.check(N.lib().fclgpu_broadphase_update(self.handle, tf.data_ptr(), 1, stream), "fclgpu_broadphase_update")
            return
        self._tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
        N.check(N.lib().fclgpu_broadphase_update(self.handle, self._tf.ctypes.data, 0, stream),
                "fclgpu_broadphase_update")

    def getAABBs(self) -> np.ndarray:
        out = np.zeros((self.size(), 6))
        N.check(N.lib().fclgpu_broadphase_get_aabbs(self.handle, out.ctypes.data), "fclgpu_broadphase_get_aabbs")
        return out

    def collide_batch(self, refs, tf, num_max_contacts: int = 1, precision: str = "fp32", exhaustive: bool = False,
                      stream=None):
        """exhaustive=False stops a query at num_max_contacts like FCL's default callback
        (num_objects / first_object then cover the evaluated pairs); True evaluates all."""
        req = N.BpCollideRequest(num_max_contacts, _prec(precision), int(exhaustive))
        if _is_torch(tf):
            import torch
            dev = tf.device
            n = tf.shape[0]
            out = dict(num_contacts=torch.empty(n, dtype=torch.int64, device=dev),
                       num_objects=torch.empty(n, dtype=torch.int32, device=dev),
                       first_object=torch.empty(n, dtype=torch.int32, device=dev))
            res = N.BpCollideResult(out["num_contacts"].data_ptr(), out["num_objects"].data_ptr(),
                                    out["first_object"].data_ptr(), 0, 0)
            s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
            N.check(N.lib().fclgpu_broadphase_collide_device(self.handle, refs.data_ptr(), n, tf.data_ptr(),
                                                             C.byref(req), C.byref(res), s),
                    "fclgpu_broadphase_collide_device")
        else:
            refs = np.ascontiguousarray(refs, np.int32).reshape(-1, 2)
            tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
            n = refs.shape[0]
            out = dict(num_contacts=np.zeros(n, np.int64), num_objects=np.zeros(n, np.int32),
                       first_object=np.zeros(n, np.int32))
            res = N.BpCollideResult(out["num_contacts"].ctypes.data, out["num_objects"].ctypes.data,
                                    out["first_object"].ctypes.data, 0, 0)
            N.check(N.lib().fclgpu_broadphase_collide(self.handle, refs.ctypes.data, n, tf.ctypes.data, C.byref(req),
                                                      C.byref(res), stream), "fclgpu_broadphase_collide")
        out["total_candidates"] = res.total_candidates
        out["node_visits"] = res.total_node_visits
        return out

    def distance_batch(self, refs, tf, nearest_points: bool = True, precision: str = "fp32", stream=None,
                       witnesses: bool = True):
        """manager.distance(obj, cdata, DefaultDistanceFunction) per query: min_distance,
        object, ids and nearest_points; witnesses=False asks for the distances and objects
        alone (the mesh-shape pairs then skip their triangle ids and points)."""
        req = N.BpDistanceRequest(int(nearest_points), _prec(precision))
        if _is_torch(tf):
            import torch
            dev = tf.device
            n = tf.shape[0]
            out = dict(min_distance=torch.empty(n, dtype=torch.float64, device=dev),
                       object=torch.empty(n, dtype=torch.int32, device=dev))
            if witnesses:
                out["ids"] = torch.empty((n, 2), dtype=torch.int32, device=dev)
                out["nearest_points"] = torch.zeros((n, 2, 3), dtype=torch.float64, device=dev)
            res = N.BpDistanceResult(out["min_distance"].data_ptr(), out["object"].data_ptr(),
                                     out["ids"].data_ptr() if witnesses else None,
                                     out["nearest_points"].data_ptr() if witnesses else None, 0, 0)
            s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
            N.check(N.lib().fclgpu_broadphase_distance_device(self.handle, refs.data_ptr(), n, tf.data_ptr(),
                                                              C.byref(req), C.byref(res), s),
                    "fclgpu_broadphase_distance_device")
        else:
            refs = np.ascontiguousarray(refs, np.int32).reshape(-1, 2)
            tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
            n = refs.shape[0]
            out = dict(min_distance=np.zeros(n), object=np.zeros(n, np.int32), ids=np.zeros((n, 2), np.int32),
                       nearest_points=np.zeros((n, 2, 3)))
            res = N.BpDistanceResult(out["min_distance"].ctypes.data, out["object"].ctypes.data,
                                     out["ids"].ctypes.data if witnesses else None,
                                     out["nearest_points"].ctypes.data if witnesses else None, 0, 0)
            if not witnesses:
                del out["ids"], out["nearest_points"]
            N.check(N.lib().fclgpu_broadphase_distance(self.handle, refs.ctypes.data, n, tf.ctypes.data,
                                                       C.byref(req), C.byref(res), stream),
                    "fclgpu_broadphase_distance")
        out["total_candidates"] = res.total_candidates
        out["node_visits"] = res.total_node_visits
        return out

    def collide_contacts(self, refs=None, tf=None, num_max_contacts: int = 1, precision: str = "fp32",
                         stream=None):
        """Contact lists of manager.collide(obj, cdata, DefaultCollisionFunction) for every
        query object (refs, tf: host numpy), or of manager.collide(cdata,
        DefaultCollisionFunction) -- the scene against itself -- when refs is None.
        Returns counts (per query; per scene object o2 in the self case), offsets and
        contacts (rows (object, b1, b2); in the self case (o1, b1, b2) with o1 < o2).  Each
        (query, object) pair is evaluated with its own cap of num_max_contacts; per query
        the objects come in ascending index order, each object's contacts in the order
        FCL's narrowphase adds them."""
        req = N.BpContactsRequest(int(num_max_contacts), _prec(precision), 0)
        if refs is not None:
            refs = np.ascontiguousarray(refs, np.int32).reshape(-1, 2)
            tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
            n = refs.shape[0]
        else:
            n = self.size()
        counts = np.zeros(n, np.int64)
        offsets = np.zeros(n + 1, np.int64)
        cap = max(64, 2 * n)
        for _ in range(2):
            contacts = np.zeros((cap, 3), np.int32)
            res = N.BpContactsResult(counts.ctypes.data, offsets.ctypes.data, contacts.ctypes.data, cap, 0, 0, 0)
            if refs is not None:
                rc = N.lib().fclgpu_broadphase_collide_contacts(self.handle, refs.ctypes.data, n, tf.ctypes.data,
                                                                C.byref(req), C.byref(res), stream)
            else:
                rc = N.lib().fclgpu_broadphase_self_collide_contacts(self.handle, C.byref(req), C.byref(res), stream)
            if rc == N.FCLGPU_ERR_CAPACITY:
                cap = int(res.total_contacts)
                continue
            N.check(rc, "fclgpu_broadphase_collide_contacts")
            return {"counts": counts, "offsets": offsets, "contacts": contacts[: int(res.total_contacts)],
                    "total_candidates": int(res.total_candidates)}
        raise N.FclGpuError(N.FCLGPU_ERR_CAPACITY, "fclgpu_broadphase_collide_contacts", "contact total changed")

    def self_distance(self, nearest_points: bool = True, precision: str = "fp32", stream=None):
        """manager.distance(cdata, DefaultDistanceFunction): the smallest distance between
        two scene objects, with o1 < o2, their triangle ids and world witness points."""
        req = N.BpDistanceRequest(int(nearest_points), _prec(precision))
        r = N.BpSelfDistanceResult()
        N.check(N.lib().fclgpu_broadphase_self_distance(self.handle, C.byref(req), C.byref(r), stream),
                "fclgpu_broadphase_self_distance")
        return {"min_distance": r.min_distance, "o1": r.o1, "o2": r.o2, "b1": r.b1, "b2": r.b2,
                "nearest_points": np.array(r.nearest_points[:]).reshape(2, 3), "total_candidates": r.total_candidates}

    def collide(self, other=None, request: "CollisionRequest | None" = None, result: "CollisionResult | None" = None):
        """FCL's three collide forms with DefaultCollisionFunction: other = None -> the
        scene against itself (collide(cdata, callback)); other = (ref, tf) of one query
        object (collide(obj, cdata, callback)); other = another manager -> every object of
        the other manager against this scene (collide(other_manager, cdata, callback)).
        Appends Contact(o1, o2, b1, b2) rows (object indices; in the other-manager form o2
        is the other manager's object) up to request.num_max_contacts in all, in the order
        collide_contacts states, and returns result.numContacts()."""
        request = request or CollisionRequest()
        result = result if result is not None else CollisionResult()
        if other is None:
            out = self.collide_contacts(None, None, request.num_max_contacts, request.precision)
            q_of = np.repeat(np.arange(self.size()), out["counts"])
        elif isinstance(other, DynamicAABBTreeCollisionManager):
            out = self.collide_contacts(other._refs, other._tf, request.num_max_contacts, request.precision)
            q_of = np.repeat(np.arange(other.size()), out["counts"])
        else:
            ref, tf = other
            out = self.collide_contacts(np.asarray(ref, np.int32).reshape(1, 2), np.asarray(tf).reshape(1, 12),
                                        request.num_max_contacts, request.precision)
            q_of = np.zeros(int(out["counts"][0]), np.int64)
        room = max(0, request.num_max_contacts - len(result.contacts))
        for (o, b1, b2), q in list(zip(out["contacts"], q_of))[:room]:
            result.contacts.append(Contact(int(o), int(q), int(b1), int(b2)))
        return result.numContacts()

    def distance(self, other=None, request: "DistanceRequest | None" = None,
                 result: "DistanceResult | None" = None) -> float:
        """FCL's distance forms with DefaultDistanceFunction: other = None -> the scene
        against itself; other = (ref, tf) of one query object; other = another manager.
        Updates result with DistanceResult's strict "<" (o1, o2 = object indices)."""
        request = request or DistanceRequest()
        result = result if result is not None else DistanceResult()
        if other is None:
            r = self.self_distance(request.enable_nearest_points, request.precision)
            cand = [(r["min_distance"], r["o1"], r["o2"], r["b1"], r["b2"], r["nearest_points"])]
        else:
            if isinstance(other, DynamicAABBTreeCollisionManager):
                refs, tf = other._refs, other._tf
            else:
                refs, tf = np.asarray(other[0], np.int32).reshape(1, 2), np.asarray(other[1]).reshape(1, 12)
            out = self.distance_batch(refs, tf, nearest_points=request.enable_nearest_points,
                                      precision=request.precision)
            q = int(np.argmin(out["min_distance"])) if len(out["min_distance"]) else 0
            cand = [(float(out["min_distance"][q]), int(out["object"][q]), q, int(out["ids"][q, 0]),
                     int(out["ids"][q, 1]), out["nearest_points"][q])] if len(out["min_distance"]) else []
        for d, o1, o2, b1, b2, pts in cand:
            if result.min_distance > d:
                result.min_distance = float(d)
                result.o1, result.o2, result.b1, result.b2 = o1, o2, b1, b2
                if request.enable_nearest_points:
                    result.nearest_points = np.asarray(pts).copy()
        return result.min_distance

    def _release(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.fclgpu_broadphase_destroy(h)
        self.handle = None

    def __del__(self):
        self._release()


# ------------------------------------------------------------- request loop ----

class NaiveCollisionManager(DynamicAABBTreeCollisionManager):
    """FCL's brute-force manager (broadphase/broadphase_bruteforce.h).  The queries run on
    the device tree; what they report (contact totals capped at num_max_contacts, the
    colliding objects, the distance of queries in no contact) does not depend on the order
    a manager meets the objects, so it equals the brute-force manager's answer."""


class SaPCollisionManager(DynamicAABBTreeCollisionManager):
    """FCL's sweep-and-prune manager (broadphase/broadphase_SaP.h), answered by the device
    tree: same order-independent results (see NaiveCollisionManager)."""


class SSaPCollisionManager(DynamicAABBTreeCollisionManager):
    """FCL's simple sweep-and-prune manager (broadphase/broadphase_SSaP.h), answered by the
    device tree: same order-independent results (see NaiveCollisionManager)."""


class IntervalTreeCollisionManager(DynamicAABBTreeCollisionManager):
    """FCL's interval-tree manager (broadphase/broadphase_interval_tree.h), answered by the
    device tree: same order-independent results (see NaiveCollisionManager)."""


class DynamicAABBTreeCollisionManager_Array(DynamicAABBTreeCollisionManager):
    """FCL's array-backed dynamic AABB tree (broadphase/broadphase_dynamic_AABB_tree_array.h),
    answered by the device tree: same order-independent results (see NaiveCollisionManager)."""


class MotionServer:
    """Continuous-batching loop of motion-checking requests over a resident
    broadphase scene (fclgpu_server_*).  robot: workloads.Robot-like (axis, offset,
    link_refs, geom_tf).  submit() queues a request (base 3x4, q (K, L)) and returns
    its id; wait(id) returns its result dict."""

    def __init__(self, scene: DynamicAABBTreeCollisionManager, robot, max_waypoints_per_step: int = 4096,
                 memory_budget_bytes: int = 0, precision: str = "fp32", clearance: bool = True):
        self.scene = scene
        self.L = int(robot.axis.shape[0])
        self._axis = np.ascontiguousarray(robot.axis, np.int32)
        self._off = np.ascontiguousarray(robot.offset, np.float64).reshape(self.L, 3)
        self._refs = np.ascontiguousarray(robot.link_refs, np.int32).reshape(self.L, 2)
        self._gtf = np.ascontiguousarray(robot.geom_tf, np.float64).reshape(self.L, 12)
        desc = N.RobotDesc(self.L, self._axis.ctypes.data, self._off.ctypes.data, self._refs.ctypes.data,
                           self._gtf.ctypes.data)
        cfg = N.ServerConfig(max_waypoints_per_step, memory_budget_bytes, _prec(precision), int(clearance))
        h = C.c_void_p()
        N.check(N.lib().fclgpu_server_create(scene.handle, C.byref(desc), C.byref(cfg), C.byref(h)),
                "fclgpu_server_create")
        self.handle = h

    def submit(self, base, q) -> int:
        base = np.ascontiguousarray(base, np.float64).reshape(12)
        q = np.ascontiguousarray(q, np.float64).reshape(-1, self.L)
        rid = C.c_int64()
        N.check(N.lib().fclgpu_server_submit(self.handle, base.ctypes.data, q.ctypes.data, q.shape[0],
                                             C.byref(rid)), "fclgpu_server_submit")
        return int(rid.value)

    def wait(self, rid: int, timeout_ms: float = -1.0):
        r = N.MotionResult()
        rc = N.lib().fclgpu_server_wait(self.handle, rid, timeout_ms, C.byref(r))
        if rc == N.FCLGPU_ERR_PENDING:
            return None
        N.check(rc, "fclgpu_server_wait")
        return dict(first_colliding_waypoint=r.first_colliding_waypoint, min_clearance=r.min_clearance,
                    clearance_waypoint=r.clearance_waypoint, clearance_link=r.clearance_link,
                    clearance_object=r.clearance_object, latency_ms=r.latency_ms, queue_ms=r.queue_ms,
                    num_steps=r.num_steps)

    def stats(self):
        s = N.ServerStats()
        N.check(N.lib().fclgpu_server_get_stats(self.handle, C.byref(s)), "fclgpu_server_get_stats")
        return {k: getattr(s, k) for k, _ in N.ServerStats._fields_}

    def link_poses(self, base, q) -> np.ndarray:
        """(K, L, 3, 4) link-geometry poses as the loop computes them."""
        base = np.ascontiguousarray(base, np.float64).reshape(12)
        q = np.ascontiguousarray(q, np.float64).reshape(-1, self.L)
        out = np.zeros((q.shape[0], self.L, 3, 4))
        N.check(N.lib().fclgpu_server_link_poses(self.handle, base.ctypes.data, q.ctypes.data, q.shape[0],
                                                 out.ctypes.data), "fclgpu_server_link_poses")
        return out

    def close(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            N._lib.fclgpu_server_destroy(h)
        self.handle = None

    def __del__(self):
        self.close()


# ---------------------------------------------------------------- mesh x shape ----

def mesh_shape_batch(meshes, shapes: ShapeSet, mesh_idx, shape_idx, tf_mesh, tf_shape, mode: str = "collide",
                     num_max_contacts: int = 1, statistics: bool = False, stream=None):
    """fcl::collide / fcl::distance of BVHModel<OBBRSS> meshes against convex shapes,
    one (mesh, shape) pair per row.  mode "collide" -> counts; "distance" ->
    min_distance, tri, nearest_points (mesh point, shape point).  Host numpy inputs."""
    hs = _handles(meshes)
    m = 0 if mode == "collide" else 1
    mesh_idx = np.ascontiguousarray(mesh_idx, np.int32)
    shape_idx = np.ascontiguousarray(shape_idx, np.int32)
    n = mesh_idx.shape[0]
    tf_mesh = np.ascontiguousarray(tf_mesh, np.float64).reshape(n, 12)
    tf_shape = np.ascontiguousarray(tf_shape, np.float64).reshape(n, 12)
    out = dict(counts=np.zeros(n, np.int32), min_distance=np.zeros(n), tri=np.zeros(n, np.int32),
               nearest_points=np.zeros((n, 2, 3)), num_bv_tests=np.zeros(n, np.int64),
               num_leaf_tests=np.zeros(n, np.int64))
    req = N.MeshShapeRequest(m, 0, num_max_contacts)
    res = N.MeshShapeResult(out["counts"].ctypes.data, out["min_distance"].ctypes.data, out["tri"].ctypes.data,
                            out["nearest_points"].ctypes.data,
                            out["num_bv_tests"].ctypes.data if statistics else None,
                            out["num_leaf_tests"].ctypes.data if statistics else None)
    N.check(N.lib().fclgpu_mesh_shape_batch(hs, len(meshes), shapes.handle, n, mesh_idx.ctypes.data,
                                            shape_idx.ctypes.data, tf_mesh.ctypes.data, tf_shape.ctypes.data,
                                            C.byref(req), C.byref(res), stream), "fclgpu_mesh_shape_batch")
    return out


def mesh_shape_contacts_batch(meshes, shapes: ShapeSet, mesh_idx, shape_idx, tf_mesh, tf_shape,
                              num_max_contacts: int = 1, enable_contact: bool = False, stream=None):
    """fcl::collide of BVHModel<OBBRSS> meshes against convex shapes with the contact
    list: per pair the triangles FCL records as Contact(mesh, shape, triangle, NONE), in
    the order its traversal adds them (at most num_max_contacts).  Returns counts,
    offsets (n + 1) and tris; with enable_contact also pos (total, 3), normal (total, 3)
    and penetration_depth (total,), the geometry FCL's leaf records.  Host numpy inputs."""
    hs = _handles(meshes)
    mesh_idx = np.ascontiguousarray(mesh_idx, np.int32)
    shape_idx = np.ascontiguousarray(shape_idx, np.int32)
    n = mesh_idx.shape[0]
    tf_mesh = np.ascontiguousarray(tf_mesh, np.float64).reshape(n, 12)
    tf_shape = np.ascontiguousarray(tf_shape, np.float64).reshape(n, 12)
    counts = np.zeros(n, np.int32)
    offsets = np.zeros(n + 1, np.int64)
    cap = max(16, 4 * n)
    for _ in range(2):
        tris = np.zeros(cap, np.int32)
        res = N.MeshShapeContactsResult(counts.ctypes.data, offsets.ctypes.data, tris.ctypes.data, cap, 0)
        if enable_contact:
            pos, nrm, dep = np.zeros((cap, 3)), np.zeros((cap, 3)), np.zeros(cap)
            res.pos, res.normal, res.penetration_depth = pos.ctypes.data, nrm.ctypes.data, dep.ctypes.data
        rc = N.lib().fclgpu_mesh_shape_contacts(hs, len(meshes), shapes.handle, n, mesh_idx.ctypes.data,
                                                shape_idx.ctypes.data, tf_mesh.ctypes.data, tf_shape.ctypes.data,
                                                int(num_max_contacts), C.byref(res), stream)
        if rc == N.FCLGPU_ERR_CAPACITY:
            cap = int(res.total_contacts)
            continue
        N.check(rc, "fclgpu_mesh_shape_contacts")
        t = int(res.total_contacts)
        out = {"counts": counts, "offsets": offsets, "tris": tris[:t]}
        if enable_contact:
            out.update(pos=pos[:t], normal=nrm[:t], penetration_depth=dep[:t])
        return out
    raise N.FclGpuError(N.FCLGPU_ERR_CAPACITY, "fclgpu_mesh_shape_contacts", "contact total changed between calls")


# ------------------------------------------------------------------- autotuner ----

def get_collide_tuning():
    b, s, v = C.c_int32(), C.c_int32(), C.c_int32()
    N.check(N.lib().fclgpu_get_collide_tuning(C.byref(b), C.byref(s), C.byref(v)), "fclgpu_get_collide_tuning")
    return int(b.value), int(s.value), int(v.value)


def set_collide_tuning(budget: int, leaf_batch_steps: int, variant: int = 0) -> None:
    N.check(N.lib().fclgpu_set_collide_tuning(int(budget), int(leaf_batch_steps), int(variant)),
            "fclgpu_set_collide_tuning")


def autotune_collide(meshes, pairs, tf1, tf2, pair_of_query=None, num_max_contacts=1, sample=65536,
                     budgets=(256, 512, 1024, 2048), steps=(2, 4, 8), variants=(0, 1), repeats=2, seed=0):
    """Picks the collide rounds' knobs (BV-test budget per item, DFS steps between warp
    leaf batches, register variant) for a workload: times the FP32 form on a uniform
    sample of its queries (torch CUDA tensors) for every combination and keeps the
    fastest.  Results do not depend on the knobs; only the time does.  Returns the
    timings (ms)."""
    import torch
    n = tf2.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    idx = torch.randperm(n, generator=g)[: min(n, sample)].sort().values.to(tf2.device)
    s_tf2 = tf2[idx].contiguous()
    s_tf1 = None if tf1 is None else tf1[idx].contiguous()
    s_pq = None if pair_of_query is None else pair_of_query[idx].contiguous()
    stream = torch.cuda.current_stream(tf2.device)
    timings = {}
    best = None
    for var in variants:
        for b in budgets:
            for st in steps:
                set_collide_tuning(b, st, var)
                collide_batch(meshes, pairs, s_tf1, s_tf2, pair_of_query=s_pq, num_max_contacts=num_max_contacts,
                              contacts=False)
                torch.cuda.synchronize()
                ms = []
                for _ in range(repeats):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    collide_batch(meshes, pairs, s_tf1, s_tf2, pair_of_query=s_pq,
                                  num_max_contacts=num_max_contacts, contacts=False, stream=stream.cuda_stream)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    ms.append(e0.elapsed_time(e1))
                key = (b, st, var)
                timings[key] = min(ms)
                if best is None or timings[key] < timings[best]:
                    best = key
    set_collide_tuning(*best)
    return {"best": list(best), "timings_ms": {f"{k[0]}/{k[1]}/{k[2]}": v for k, v in timings.items()}}
