"""ctypes front end of the FP64 CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the CPU
baseline leg of bench.py.  The shipped library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (g++ -ffp-contract=off)."""
    out = subprocess.run(["make", "-s", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_mesh_create.restype = C.c_void_p
        L.orc_mesh_create.argtypes = [_dp, C.c_int, _ip, C.c_int]
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_mesh_num_nodes.argtypes = [C.c_void_p]
        L.orc_mesh_get_nodes.argtypes = [C.c_void_p, _dp, _ip]
        L.orc_mesh_update.argtypes = [C.c_void_p, _dp]
        L.orc_mesh_replace.argtypes = [C.c_void_p, _dp]
        L.orc_mesh_rebuild.argtypes = [C.c_void_p, _dp, C.c_int]
        L.orc_collide_batch.restype = C.c_int64
        L.orc_collide_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, C.c_int64, C.c_int,
                                        _i64p, _i64p, _i64p, _ip, C.c_int64]
        L.orc_collide_contacts_batch.restype = C.c_int64
        L.orc_collide_contacts_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, C.c_int64,
                                                 C.c_int, _i64p, _ip, _dp, _dp, _dp, C.c_int64]
        L.orc_ccd_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, C.c_int64, C.c_double,
                                    C.c_int, C.c_int, _ip, _dp, _dp, _dp]
        L.orc_motion.argtypes = [C.c_int, C.c_int64, _dp, _dp, _dp, _dp]
        L.orc_ca_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, C.c_int, C.c_int, _ip, _dp,
                                   _dp, _dp, _i64p]
        L.orc_tri_contact_batch.argtypes = [C.c_int64, _dp, _dp, _ip, _dp, _dp, _dp]
        L.orc_distance_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, C.c_int, C.c_int,
                                         _dp, _ip, _dp, _i64p, _i64p]
        L.orc_rss_fit3.argtypes = [_dp, _dp]
        L.orc_rss_member_distance.restype = C.c_double
        L.orc_rss_member_distance.argtypes = [_dp, _dp]
        L.orc_rss_distance.restype = C.c_double
        L.orc_rss_distance.argtypes = [_dp, _dp, _dp]
        L.orc_obb_overlap.argtypes = [_dp, _dp, _dp]
        L.orc_tri_intersect_batch.argtypes = [C.c_int64, _dp, _dp, _dp, _ip]
        L.orc_tri_distance_batch.argtypes = [C.c_int64, _dp, _dp, _dp, _dp]
        L.orc_hardware_threads.restype = C.c_int
        L.orc_brute_collide.restype = C.c_int64
        L.orc_brute_collide.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _ip, C.c_int64]
        L.orc_brute_distance.restype = C.c_double
        L.orc_brute_distance.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _q(a):
    return a.ctypes.data_as(_i64p)


def hardware_threads() -> int:
    return int(lib().orc_hardware_threads())


class Mesh:
    """BVHModel<OBBRSS> built by the oracle (reference algorithm, MEAN split)."""

    def __init__(self, verts: np.ndarray, tris: np.ndarray):
        self.verts = np.ascontiguousarray(verts, dtype=np.float64)
        self.tris = np.ascontiguousarray(tris, dtype=np.int32)
        self.h = lib().orc_mesh_create(_d(self.verts), self.verts.shape[0], _i(self.tris), self.tris.shape[0])

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mesh_free(self.h)
            self.h = None

    def update(self, verts: np.ndarray) -> None:
        """beginUpdateModel / updateVertex / endUpdateModel() with the default
        bottom-up refit: the previous frame is the current vertices."""
        v = np.ascontiguousarray(verts, dtype=np.float64)
        assert v.shape == self.verts.shape
        lib().orc_mesh_update(self.h, _d(v))
        self.verts = v

    def replace(self, verts: np.ndarray) -> None:
        """beginReplaceModel / replaceVertex / endReplaceModel(refit = true, bottomup =
        true): no previous frame, each leaf refitted to its new triangle (fit3)."""
        v = np.ascontiguousarray(verts, dtype=np.float64)
        assert v.shape == self.verts.shape
        lib().orc_mesh_replace(self.h, _d(v))
        self.verts = v

    def rebuild(self, verts: np.ndarray, update: bool) -> None:
        """endUpdateModel(refit = false) (update) / endReplaceModel(refit = false):
        the tree rebuilt on the new vertices, then (update) the bottom-up refit over both
        frames."""
        v = np.ascontiguousarray(verts, dtype=np.float64)
        assert v.shape == self.verts.shape
        lib().orc_mesh_rebuild(self.h, _d(v), int(update))
        self.verts = v

    def nodes(self):
        n = lib().orc_mesh_num_nodes(self.h)
        out = np.empty((n, 30), np.float64)
        fc = np.empty(n, np.int32)
        lib().orc_mesh_get_nodes(self.h, _d(out), _i(fc))
        return out, fc


def collide_batch(m1: Mesh, m2: Mesh, tf2: np.ndarray, tf1: np.ndarray | None = None,
                  num_max_contacts: int = 1, nthreads: int = 1):
    """Returns (counts, contacts (total,2) int32 in per-pose DFS order, nbv, nleaf)."""
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1p = None if tf1 is None else _d(np.ascontiguousarray(tf1, np.float64).reshape(-1, 12))
    counts = np.zeros(n, np.int64)
    nbv = np.zeros(n, np.int64)
    nleaf = np.zeros(n, np.int64)
    cap = 1 << 16
    while True:
        out = np.empty((cap, 2), np.int32)
        total = lib().orc_collide_batch(m1.h, m2.h, n, tf1p, _d(tf2), num_max_contacts, nthreads,
                                        _q(counts), _q(nbv), _q(nleaf), _i(out), cap)
        if total <= cap:
            return counts, out[:total].copy(), nbv, nleaf
        cap = int(total)


def collide_front(m1: Mesh, m2: Mesh, tf2, tf1=None, front=None, num_max_contacts: int = 1):
    """collide(node, front_list) for one pose: returns (contacts (k,2), new front (m,2),
    nbv, nleaf).  front: (m,2) int32 node pairs from a previous call, or None / empty."""
    L = lib()
    L.orc_collide_front.restype = C.c_int64
    L.orc_collide_front.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, C.c_int64, _ip, C.c_int64, _ip, C.c_int64,
                                    _i64p, _ip, C.c_int64, _i64p, _i64p]
    fin = np.ascontiguousarray(np.zeros((0, 2), np.int32) if front is None else front, np.int32).reshape(-1, 2)
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(12)
    t1 = None if tf1 is None else _d(np.ascontiguousarray(tf1, np.float64).reshape(12))
    fcap, ccap = max(1024, 4 * fin.shape[0]), 1024
    while True:
        fout = np.zeros((fcap, 2), np.int32)
        cont = np.zeros((ccap, 2), np.int32)
        nf, nbv, nleaf = (np.zeros(1, np.int64) for _ in range(3))
        k = L.orc_collide_front(m1.h, m2.h, t1, _d(tf2), num_max_contacts, _i(fin), fin.shape[0], _i(fout), fcap,
                                _q(nf), _i(cont), ccap, _q(nbv), _q(nleaf))
        if nf[0] <= fcap and k <= ccap:
            return cont[:k].copy(), fout[:nf[0]].copy(), int(nbv[0]), int(nleaf[0])
        fcap, ccap = max(fcap, int(nf[0])), max(ccap, int(k))


def collide_contacts_batch(m1: Mesh, m2: Mesh, tf2: np.ndarray, tf1: np.ndarray | None = None,
                           num_max_contacts: int = 1, nthreads: int = 1):
    """fcl::collide with enable_contact = true.  Returns (counts, ids (total,2) int32,
    pos (total,3), normal (total,3), depth (total,)) in per-pose DFS order."""
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1p = None if tf1 is None else _d(np.ascontiguousarray(tf1, np.float64).reshape(-1, 12))
    counts = np.zeros(n, np.int64)
    cap = 1 << 16
    while True:
        ids = np.empty((cap, 2), np.int32)
        pos = np.empty((cap, 3), np.float64)
        nrm = np.empty((cap, 3), np.float64)
        dep = np.empty(cap, np.float64)
        total = lib().orc_collide_contacts_batch(m1.h, m2.h, n, tf1p, _d(tf2), num_max_contacts, nthreads,
                                                 _q(counts), _i(ids), _d(pos), _d(nrm), _d(dep), cap)
        if total <= cap:
            return counts, ids[:total].copy(), pos[:total].copy(), nrm[:total].copy(), dep[:total].copy()
        cap = int(total)


_MOTIONS = {"trans": 0, "linear": 1, "screw": 2}


def continuous_collide_batch(m1: Mesh, m2: Mesh, tf2_beg, tf2_end, tf1_beg=None, tf1_end=None,
                             num_max_iterations: int = 10, toc_err: float = 1e-4, nthreads: int = 1,
                             motion: str = "trans"):
    """fcl::continuousCollide, naive solver, translation / linear / screw motion.  Returns (hit, toc,
    contact_tf1 (n,3,4), contact_tf2 (n,3,4)); the transforms are zero where no hit."""
    b0 = np.ascontiguousarray(tf2_beg, np.float64).reshape(-1, 12)
    b1 = np.ascontiguousarray(tf2_end, np.float64).reshape(-1, 12)
    n = b0.shape[0]
    a0 = None if tf1_beg is None else np.ascontiguousarray(tf1_beg, np.float64).reshape(-1, 12)
    a1 = None if tf1_end is None else np.ascontiguousarray(tf1_end, np.float64).reshape(-1, 12)
    hit = np.zeros(n, np.int32)
    toc = np.zeros(n)
    c1 = np.zeros((n, 3, 4))
    c2 = np.zeros((n, 3, 4))
    lib().orc_ccd_batch(m1.h, m2.h, n, None if a0 is None else _d(a0), None if a1 is None else _d(a1), _d(b0),
                        _d(b1), num_max_iterations, toc_err, _MOTIONS[motion], nthreads, _i(hit), _d(toc), _d(c1),
                        _d(c2))
    return hit, toc, c1, c2


def ca_batch(m1: Mesh, m2: Mesh, b0, b1, a0=None, a1=None, motion: str = "trans", nthreads: int = 1):
    """continuousCollide with conservative advancement (the oriented OBBRSS node) for n
    motions -> (hit, toc, contact_tf1 (n,3,4), contact_tf2, iterations)."""
    b0 = np.ascontiguousarray(b0, np.float64).reshape(-1, 12)
    b1 = np.ascontiguousarray(b1, np.float64).reshape(-1, 12)
    n = b0.shape[0]
    a0 = None if a0 is None else np.ascontiguousarray(a0, np.float64).reshape(-1, 12)
    a1 = None if a1 is None else np.ascontiguousarray(a1, np.float64).reshape(-1, 12)
    hit = np.zeros(n, np.int32)
    toc = np.zeros(n)
    c1 = np.zeros((n, 3, 4))
    c2 = np.zeros((n, 3, 4))
    it = np.zeros(n, np.int64)
    lib().orc_ca_batch(m1.h, m2.h, n, None if a0 is None else _d(a0), None if a1 is None else _d(a1), _d(b0),
                       _d(b1), _MOTIONS[motion], nthreads, _i(hit), _d(toc), _d(c1), _d(c2), _q(it))
    return hit, toc, c1, c2, it


def motion(beg, end, t, kind: str = "trans"):
    """TranslationMotion / InterpMotion / ScrewMotion(beg, end) at times t: (n,3,4)."""
    beg = np.ascontiguousarray(beg, np.float64).reshape(-1, 12)
    end = np.ascontiguousarray(end, np.float64).reshape(-1, 12)
    t = np.ascontiguousarray(t, np.float64)
    out = np.empty((beg.shape[0], 3, 4))
    lib().orc_motion(_MOTIONS[kind], beg.shape[0], _d(beg), _d(end), _d(t), _d(out))
    return out


def translation_motion(beg, end, t):
    """TranslationMotion(beg, end) at times t: (n,3,4) transforms."""
    return motion(beg, end, t, "trans")


def tri_contact_batch(P: np.ndarray, Qm: np.ndarray):
    """Contact part of intersect_Triangle per pair: (counts, points (n,2,3), normal (n,3),
    depth (n,)); Qm is the second triangle already in the first one's frame."""
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 9)
    Qm = np.ascontiguousarray(Qm, np.float64).reshape(-1, 9)
    n = P.shape[0]
    cnt = np.empty(n, np.int32)
    pts = np.empty((n, 2, 3), np.float64)
    nrm = np.empty((n, 3), np.float64)
    dep = np.empty(n, np.float64)
    lib().orc_tri_contact_batch(n, _d(P), _d(Qm), _i(cnt), _d(pts), _d(nrm), _d(dep))
    return cnt, pts, nrm, dep


def distance_batch(m1: Mesh, m2: Mesh, tf2: np.ndarray, tf1: np.ndarray | None = None,
                   nearest: bool = True, nthreads: int = 1):
    """Returns (dist, ids (n,2), points (n,2,3) world frame, nbv, nleaf)."""
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(-1, 12)
    n = tf2.shape[0]
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(-1, 12)
    dist = np.empty(n, np.float64)
    ids = np.empty((n, 2), np.int32)
    pts = np.zeros((n, 2, 3), np.float64)
    nbv = np.zeros(n, np.int64)
    nleaf = np.zeros(n, np.int64)
    lib().orc_distance_batch(m1.h, m2.h, n, None if tf1a is None else _d(tf1a), _d(tf2), int(nearest),
                             nthreads, _d(dist), _i(ids), _d(pts), _q(nbv), _q(nleaf))
    return dist, ids, pts, nbv, nleaf


def rss_fit3(pts: np.ndarray) -> np.ndarray:
    pts = np.ascontiguousarray(pts, np.float64).reshape(9)
    out = np.empty(15, np.float64)
    lib().orc_rss_fit3(_d(pts), _d(out))
    return out


def rss_member_distance(a15: np.ndarray, b15: np.ndarray) -> float:
    a = np.ascontiguousarray(a15, np.float64)
    b = np.ascontiguousarray(b15, np.float64)
    return float(lib().orc_rss_member_distance(_d(a), _d(b)))


def rss_distance(tf: np.ndarray, a15: np.ndarray, b15: np.ndarray) -> float:
    tf = np.ascontiguousarray(tf, np.float64).reshape(12)
    a = np.ascontiguousarray(a15, np.float64)
    b = np.ascontiguousarray(b15, np.float64)
    return float(lib().orc_rss_distance(_d(tf), _d(a), _d(b)))


def obb_overlap(tf: np.ndarray, a15: np.ndarray, b15: np.ndarray) -> bool:
    tf = np.ascontiguousarray(tf, np.float64).reshape(12)
    a = np.ascontiguousarray(a15, np.float64)
    b = np.ascontiguousarray(b15, np.float64)
    return bool(lib().orc_obb_overlap(_d(tf), _d(a), _d(b)))


def tri_intersect_batch(P: np.ndarray, Q: np.ndarray, tf: np.ndarray) -> np.ndarray:
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 9)
    Q = np.ascontiguousarray(Q, np.float64).reshape(-1, 9)
    tf = np.ascontiguousarray(tf, np.float64).reshape(12)
    out = np.empty(P.shape[0], np.int32)
    lib().orc_tri_intersect_batch(P.shape[0], _d(P), _d(Q), _d(tf), _i(out))
    return out.astype(bool)


def tri_distance_batch(P: np.ndarray, Q: np.ndarray):
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 9)
    Q = np.ascontiguousarray(Q, np.float64).reshape(-1, 9)
    d = np.empty(P.shape[0], np.float64)
    pts = np.empty((P.shape[0], 2, 3), np.float64)
    lib().orc_tri_distance_batch(P.shape[0], _d(P), _d(Q), _d(d), _d(pts))
    return d, pts


def brute_collide(m1: Mesh, m2: Mesh, tf2: np.ndarray, tf1: np.ndarray | None = None) -> np.ndarray:
    """All intersecting triangle pairs (k, 2), row-major pair order."""
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(12)
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(12)
    cap = 1 << 16
    while True:
        out = np.empty((cap, 2), np.int32)
        k = lib().orc_brute_collide(m1.h, m2.h, None if tf1a is None else _d(tf1a), _d(tf2), _i(out), cap)
        if k <= cap:
            return out[:k].copy()
        cap = int(k)


def brute_distance(m1: Mesh, m2: Mesh, tf2: np.ndarray, tf1: np.ndarray | None = None) -> float:
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(12)
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(12)
    return float(lib().orc_brute_distance(m1.h, m2.h, None if tf1a is None else _d(tf1a), _d(tf2)))


SOLVER_DEFAULTS = (2.0097183471152322e-14, 2.0097183471152322e-14, 128, 255)


def set_gjk_solver_params(gjk_tolerance=SOLVER_DEFAULTS[0], epa_tolerance=SOLVER_DEFAULTS[1],
                          gjk_max_iterations=SOLVER_DEFAULTS[2], epa_max_iterations=SOLVER_DEFAULTS[3]):
    """GJKSolver_indep parameters of every later oracle GJK / EPA (process-wide)."""
    L = lib()
    L.orc_set_gjk_solver_params.argtypes = [C.c_double, C.c_double, C.c_int64, C.c_int64]
    L.orc_set_gjk_solver_params(gjk_tolerance, epa_tolerance, gjk_max_iterations, epa_max_iterations)


def shape_batch(shapes, ia, ib, tf1, tf2, nthreads: int = 1):
    """GJKSolver_indep collide (+ EPA contact) and, for separated pairs, distance.
    Returns dict: hit, normal, point, depth, dist, p1, p2, status (n,2)."""
    L = lib()
    if not hasattr(L, "_shape_sig"):
        L.orc_shape_batch.argtypes = [C.c_int, _ip, _dp, _ip, _ip, _dp, C.c_int64, _ip, _ip, _dp, _dp, C.c_int,
                                      _ip, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        L._shape_sig = True
    t = np.ascontiguousarray(shapes.type, np.int32)
    pr = np.ascontiguousarray(shapes.params, np.float64)
    vo = np.ascontiguousarray(shapes.voff, np.int32)
    vc = np.ascontiguousarray(shapes.vcnt, np.int32)
    vv = np.ascontiguousarray(shapes.verts, np.float64).reshape(-1, 3)
    if vv.shape[0] == 0:
        vv = np.zeros((1, 3))
    ia = np.ascontiguousarray(ia, np.int32); ib = np.ascontiguousarray(ib, np.int32)
    n = ia.shape[0]
    tf1 = np.ascontiguousarray(tf1, np.float64).reshape(n, 12)
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(n, 12)
    out = dict(hit=np.zeros(n, np.int32), normal=np.zeros((n, 3)), point=np.zeros((n, 3)), depth=np.zeros(n),
               dist=np.zeros(n), p1=np.zeros((n, 3)), p2=np.zeros((n, 3)), status=np.zeros((n, 2), np.int32))
    L.orc_shape_batch(t.shape[0], _i(t), _d(pr), _i(vo), _i(vc), _d(vv), n, _i(ia), _i(ib), _d(tf1), _d(tf2),
                      nthreads, _i(out["hit"]), _d(out["normal"]), _d(out["point"]), _d(out["depth"]),
                      _d(out["dist"]), _d(out["p1"]), _d(out["p2"]), _i(out["status"]))
    out["hit"] = out["hit"].astype(bool)
    return out


def project_origin(pts):
    L = lib()
    L.orc_project_origin.argtypes = [C.c_int, _dp, _ip, _dp]
    pts = np.ascontiguousarray(pts, np.float64)
    enc = C.c_int()
    out = np.zeros(5)
    L.orc_project_origin(pts.shape[0], _d(pts), C.byref(enc), _d(out))
    return enc.value, out[0], out[1:]


# ------------------------------------------------------------------ broadphase ----

def _bp_sigs(L):
    if getattr(L, "_bp_sig", False):
        return
    vp = C.c_void_p
    L.orc_geoms_create.restype = vp
    L.orc_geoms_create.argtypes = [C.c_int, _ip, _dp, _ip, _ip, _dp, C.c_int, C.POINTER(C.c_void_p)]
    L.orc_geoms_free.argtypes = [vp]
    L.orc_geoms_local.argtypes = [vp, _dp]
    L.orc_scene_create.restype = vp
    L.orc_scene_create.argtypes = [vp, C.c_int, _ip, _dp]
    L.orc_scene_free.argtypes = [vp]
    L.orc_scene_num_tree_nodes.restype = C.c_int
    L.orc_scene_num_tree_nodes.argtypes = [vp]
    L.orc_world_aabbs.argtypes = [vp, C.c_int64, _ip, _dp, _dp]
    L.orc_scene_candidates.restype = C.c_int64
    L.orc_scene_candidates.argtypes = [vp, C.c_int64, _ip, _dp, _i64p, _ip, C.c_int64]
    L.orc_scene_collide.restype = C.c_int64
    L.orc_scene_collide.argtypes = [vp, C.c_int64, _ip, _dp, C.c_int64, C.c_int, C.c_int, _i64p, _ip, _ip,
                                    C.c_int64, _i64p]
    L.orc_scene_distance.argtypes = [vp, C.c_int64, _ip, _dp, C.c_int, C.c_int, _dp, _ip, _ip, _dp, _i64p]
    L._bp_sig = True


class Geoms:
    """Geometry registry for the broadphase: ids [0, ns) are the shapes of a
    ShapeSet-like object (type, params, voff, vcnt, verts), ids [ns, ns + nm) the meshes."""

    def __init__(self, shapes=None, meshes=()):
        L = lib()
        _bp_sigs(L)
        if shapes is None:
            t = np.zeros(0, np.int32); pr = np.zeros((0, 3)); vo = np.zeros(0, np.int32); vc = np.zeros(0, np.int32)
            vv = np.zeros((1, 3))
        else:
            t = np.ascontiguousarray(shapes.type, np.int32)
            pr = np.ascontiguousarray(shapes.params, np.float64)
            vo = np.ascontiguousarray(shapes.voff, np.int32)
            vc = np.ascontiguousarray(shapes.vcnt, np.int32)
            vv = np.ascontiguousarray(shapes.verts, np.float64).reshape(-1, 3)
            if vv.shape[0] == 0:
                vv = np.zeros((1, 3))
        self._keep = (t, pr, vo, vc, vv, list(meshes))
        self.ns, self.nm = t.shape[0], len(meshes)
        mh = (C.c_void_p * max(1, self.nm))(*[m.h for m in meshes])
        self.h = L.orc_geoms_create(self.ns, _i(t), _d(pr), _i(vo), _i(vc), _d(vv), self.nm, mh)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_geoms_free(self.h)
            self.h = None

    def local(self):
        """Per geometry: aabb_local min, max, aabb_center, aabb_radius (10 doubles)."""
        out = np.zeros((self.ns + self.nm, 10))
        lib().orc_geoms_local(self.h, _d(out))
        return out

    def world_aabbs(self, gid, tf):
        gid = np.ascontiguousarray(gid, np.int32)
        tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
        out = np.zeros((gid.shape[0], 6))
        lib().orc_world_aabbs(self.h, gid.shape[0], _i(gid), _d(tf), _d(out))
        return out


class Scene:
    """A broadphase manager over scene objects (geometry ids + 3x4 poses): the dynamic
    AABB tree manager (use_tree=True) or the naive one, with FCL's default callbacks."""

    def __init__(self, geoms: Geoms, gid, tf):
        self.geoms = geoms
        self.gid = np.ascontiguousarray(gid, np.int32)
        self.tf = np.ascontiguousarray(tf, np.float64).reshape(-1, 12)
        self.h = lib().orc_scene_create(geoms.h, self.gid.shape[0], _i(self.gid), _d(self.tf))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_scene_free(self.h)
            self.h = None

    def num_tree_nodes(self) -> int:
        return int(lib().orc_scene_num_tree_nodes(self.h))

    def candidates(self, qgid, qtf):
        """Exact AABB-overlap scene objects per query: (counts, flat ids in object order)."""
        qgid = np.ascontiguousarray(qgid, np.int32)
        qtf = np.ascontiguousarray(qtf, np.float64).reshape(-1, 12)
        n = qgid.shape[0]
        counts = np.zeros(n, np.int64)
        total = lib().orc_scene_candidates(self.h, n, _i(qgid), _d(qtf), _q(counts), None, 0)
        ids = np.zeros(max(1, total), np.int32)
        lib().orc_scene_candidates(self.h, n, _i(qgid), _d(qtf), _q(counts), _i(ids), total)
        return counts, ids[:total]

    def collide(self, qgid, qtf, max_contacts: int = 1, use_tree: bool = True, nthreads: int = 1):
        qgid = np.ascontiguousarray(qgid, np.int32)
        qtf = np.ascontiguousarray(qtf, np.float64).reshape(-1, 12)
        n = qgid.shape[0]
        nc = np.zeros(n, np.int64); nh = np.zeros(n, np.int32); calls = np.zeros(n, np.int64)
        cap = max(1, 64 * n)
        hits = np.zeros(cap, np.int32)
        total = lib().orc_scene_collide(self.h, n, _i(qgid), _d(qtf), max_contacts, int(use_tree), nthreads,
                                        _q(nc), _i(nh), _i(hits), cap, _q(calls))
        if total > cap:
            hits = np.zeros(total, np.int32)
            lib().orc_scene_collide(self.h, n, _i(qgid), _d(qtf), max_contacts, int(use_tree), nthreads,
                                    _q(nc), _i(nh), _i(hits), total, _q(calls))
        return dict(num_contacts=nc, num_hits=nh, hits=hits[:total], narrow_calls=calls)

    def collide_lists(self, qgid, qtf, max_per_pair: int = 1, nthreads: int = 1):
        """The GPU broadphase contacts call's definition: per query, the overlapping
        scene objects in index order, each collided with a fresh result capped at
        max_per_pair -> (counts, (total, 3) rows (object, b1, b2))."""
        L = lib()
        L.orc_scene_collide_lists.restype = C.c_int64
        L.orc_scene_collide_lists.argtypes = [C.c_void_p, C.c_int64, _ip, _dp, C.c_int64, C.c_int, _i64p, _ip,
                                              C.c_int64]
        qgid = np.ascontiguousarray(qgid, np.int32)
        qtf = np.ascontiguousarray(qtf, np.float64).reshape(-1, 12)
        n = qgid.shape[0]
        counts = np.zeros(n, np.int64)
        cap = 64 * n + 64
        while True:
            trip = np.zeros((cap, 3), np.int32)
            total = L.orc_scene_collide_lists(self.h, n, _i(qgid), _d(qtf), max_per_pair, nthreads, _q(counts),
                                              _i(trip), cap)
            if total <= cap:
                return counts, trip[:total]
            cap = total

    def self_collide_lists(self, max_per_pair: int = 1):
        """Self-collision lists: per o2 the objects o1 < o2 in ascending order ->
        (counts per o2, rows (o1, b1, b2))."""
        L = lib()
        L.orc_scene_self_collide_lists.restype = C.c_int64
        L.orc_scene_self_collide_lists.argtypes = [C.c_void_p, C.c_int64, _i64p, _ip, C.c_int64]
        n = self.gid.shape[0]
        counts = np.zeros(n, np.int64)
        cap = 64 * n + 64
        while True:
            trip = np.zeros((cap, 3), np.int32)
            total = L.orc_scene_self_collide_lists(self.h, max_per_pair, _q(counts), _i(trip), cap)
            if total <= cap:
                return counts, trip[:total]
            cap = total

    def self_collide_count(self, max_contacts: int = 1) -> int:
        """NaiveCollisionManager::collide(cdata, DefaultCollisionFunction): numContacts()."""
        L = lib()
        L.orc_scene_self_collide_naive.restype = C.c_int64
        L.orc_scene_self_collide_naive.argtypes = [C.c_void_p, C.c_int64]
        return int(L.orc_scene_self_collide_naive(self.h, max_contacts))

    def self_distance(self):
        """NaiveCollisionManager::distance(cdata, DefaultDistanceFunction)."""
        L = lib()
        L.orc_scene_self_distance.argtypes = [C.c_void_p, _dp, _ip]
        d = np.zeros(7); ids = np.zeros(4, np.int32)
        L.orc_scene_self_distance(self.h, _d(d), _i(ids))
        return dict(min_distance=float(d[0]), o1=int(ids[0]), o2=int(ids[1]), b1=int(ids[2]), b2=int(ids[3]),
                    nearest_points=d[1:].reshape(2, 3))

    def distance(self, qgid, qtf, use_tree: bool = True, nthreads: int = 1):
        qgid = np.ascontiguousarray(qgid, np.int32)
        qtf = np.ascontiguousarray(qtf, np.float64).reshape(-1, 12)
        n = qgid.shape[0]
        out = dict(dist=np.zeros(n), obj=np.zeros(n, np.int32), b12=np.zeros((n, 2), np.int32),
                   pts=np.zeros((n, 2, 3)), narrow_calls=np.zeros(n, np.int64))
        lib().orc_scene_distance(self.h, n, _i(qgid), _d(qtf), int(use_tree), nthreads, _d(out["dist"]),
                                 _i(out["obj"]), _i(out["b12"]), _d(out["pts"]), _q(out["narrow_calls"]))
        return out


# ------------------------------------------------------------------ mesh-shape ----

def _ms_sigs(L):
    if getattr(L, "_ms_sig", False):
        return
    vp = C.c_void_p
    L.orc_mesh_shape_batch.argtypes = [vp, vp, C.c_int64, _ip, _dp, _dp, C.c_int64, C.c_int, C.c_int, _i64p, _dp,
                                       _ip, _dp, _i64p, _i64p]
    L.orc_mesh_shape_brute.argtypes = [vp, vp, C.c_int, _dp, _dp, _i64p, _dp]
    L.orc_shape_obbrss.argtypes = [vp, C.c_int, _dp, _dp]
    L._ms_sig = True


def mesh_shape_collide(mesh: Mesh, geoms: Geoms, sid, tfm, tfs, max_contacts: int = 1, nthreads: int = 1):
    """fcl::collide(mesh, shape) per query -> (counts, num_bv_tests, num_leaf_tests)."""
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    sid = np.ascontiguousarray(sid, np.int32)
    n = sid.shape[0]
    tfm = np.ascontiguousarray(tfm, np.float64).reshape(n, 12)
    tfs = np.ascontiguousarray(tfs, np.float64).reshape(n, 12)
    counts = np.zeros(n, np.int64); nbv = np.zeros(n, np.int64); nleaf = np.zeros(n, np.int64)
    dummy_d = np.zeros(1); dummy_i = np.zeros(1, np.int32)
    L.orc_mesh_shape_batch(mesh.h, geoms.h, n, _i(sid), _d(tfm), _d(tfs), max_contacts, 0, nthreads, _q(counts),
                           _d(dummy_d), _i(dummy_i), _d(dummy_d), _q(nbv), _q(nleaf))
    return counts, nbv, nleaf


def mesh_shape_contacts(mesh: Mesh, geoms: Geoms, sid, tfm, tfs, max_contacts: int = 1, nthreads: int = 1):
    """fcl::collide(mesh, shape) per query with the contact list -> (counts, tris): the
    triangle ids of every query's contacts, in the order FCL adds them, concatenated."""
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    L.orc_mesh_shape_contacts.restype = C.c_int64
    L.orc_mesh_shape_contacts.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _ip, _dp, _dp, C.c_int64, C.c_int,
                                          _i64p, _ip, C.c_int64]
    sid = np.ascontiguousarray(sid, np.int32)
    n = sid.shape[0]
    tfm = np.ascontiguousarray(tfm, np.float64).reshape(n, 12)
    tfs = np.ascontiguousarray(tfs, np.float64).reshape(n, 12)
    counts = np.zeros(n, np.int64)
    cap = 16 * n + 16
    while True:
        tris = np.zeros(cap, np.int32)
        total = L.orc_mesh_shape_contacts(mesh.h, geoms.h, n, _i(sid), _d(tfm), _d(tfs), max_contacts, nthreads,
                                          _q(counts), _i(tris), cap)
        if total <= cap:
            return counts, tris[:total]
        cap = total


def mesh_shape_contact_geometry(mesh: Mesh, geoms: Geoms, sid, tfm, tfs, tris):
    """The geometry FCL's mesh-shape leaf records with enable_contact for contact k
    (shape sid[k] at tfs[k], the mesh at tfm[k], triangle tris[k]) -> dict(pos (k, 3),
    normal (k, 3), depth (k,), ok (k,))."""
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    L.orc_mesh_shape_contact_geometry.restype = None
    L.orc_mesh_shape_contact_geometry.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, _ip, _dp, _dp, _ip, _dp, _dp,
                                                  _dp, _ip]
    sid = np.ascontiguousarray(sid, np.int32)
    n = sid.shape[0]
    tfm = np.ascontiguousarray(tfm, np.float64).reshape(n, 12)
    tfs = np.ascontiguousarray(tfs, np.float64).reshape(n, 12)
    tris = np.ascontiguousarray(tris, np.int32)
    out = dict(pos=np.zeros((n, 3)), normal=np.zeros((n, 3)), depth=np.zeros(n), ok=np.zeros(n, np.int32))
    L.orc_mesh_shape_contact_geometry(mesh.h, geoms.h, n, _i(sid), _d(tfm), _d(tfs), _i(tris), _d(out["pos"]),
                                      _d(out["normal"]), _d(out["depth"]), _i(out["ok"]))
    return out


def mesh_shape_distance(mesh: Mesh, geoms: Geoms, sid, tfm, tfs, nthreads: int = 1):
    """fcl::distance(mesh, shape) per query -> dict(dist, tri, pts (n,2,3), nbv, nleaf)."""
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    sid = np.ascontiguousarray(sid, np.int32)
    n = sid.shape[0]
    tfm = np.ascontiguousarray(tfm, np.float64).reshape(n, 12)
    tfs = np.ascontiguousarray(tfs, np.float64).reshape(n, 12)
    out = dict(dist=np.zeros(n), tri=np.zeros(n, np.int32), pts=np.zeros((n, 2, 3)), nbv=np.zeros(n, np.int64),
               nleaf=np.zeros(n, np.int64))
    dummy = np.zeros(1, np.int64)
    L.orc_mesh_shape_batch(mesh.h, geoms.h, n, _i(sid), _d(tfm), _d(tfs), 0, 1, nthreads, _q(dummy),
                           _d(out["dist"]), _i(out["tri"]), _d(out["pts"]), _q(out["nbv"]), _q(out["nleaf"]))
    return out


def mesh_shape_brute(mesh: Mesh, geoms: Geoms, sid: int, tfm, tfs):
    """(number of intersecting triangles, min triangle distance) over every triangle."""
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    tfm = np.ascontiguousarray(tfm, np.float64).reshape(12)
    tfs = np.ascontiguousarray(tfs, np.float64).reshape(12)
    c = C.c_int64(); d = C.c_double()
    L.orc_mesh_shape_brute(mesh.h, geoms.h, sid, _d(tfm), _d(tfs), C.byref(c), C.byref(d))
    return int(c.value), float(d.value)


def shape_obbrss(geoms: Geoms, sid: int, tf):
    L = lib(); _bp_sigs(L); _ms_sigs(L)
    tf = np.ascontiguousarray(tf, np.float64).reshape(12)
    out = np.zeros(30)
    L.orc_shape_obbrss(geoms.h, sid, _d(tf), _d(out))
    return out
