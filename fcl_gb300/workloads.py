"""Seeded synthetic workloads for the mesh, convex-shape and broadphase queries.

All generators are deterministic for a given seed on one machine (numpy PCG64).
Meshes are class-I geodesic icospheres (frequency n -> 20 n^2 triangles) scaled to
ellipsoids and perturbed per vertex; poses are Haar-uniform rotations (normalised
4-D Gaussian quaternions) with uniform translations.  Transforms are returned as
(N, 3, 4) float64 arrays [R | t].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_ICO_CACHE: dict[int, tuple[np.ndarray, np.ndarray]] = {}


def _icosahedron() -> tuple[np.ndarray, np.ndarray]:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def geodesic_sphere(freq: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit class-I geodesic sphere with 20*freq^2 triangles and 10*freq^2+2 vertices."""
    if freq in _ICO_CACHE:
        v, f = _ICO_CACHE[freq]
        return v.copy(), f.copy()
    n = int(freq)
    if n < 1:
        raise ValueError("freq must be >= 1")
    iv, ifc = _icosahedron()
    # grid points (a, b) with a + b <= n on each face; weights (n-a-b, a, b)
    ab = [(a, b) for a in range(n + 1) for b in range(n + 1 - a)]
    ab = np.array(ab, dtype=np.int64)
    local = {(int(a), int(b)): k for k, (a, b) in enumerate(ab)}
    npts = len(ab)
    # canonical weight vectors over the 12 icosahedron vertices for de-duplication
    W = np.zeros((20 * npts, 12), dtype=np.int64)
    for fi, (i0, i1, i2) in enumerate(ifc):
        rows = slice(fi * npts, (fi + 1) * npts)
        W[rows, i0] += n - ab[:, 0] - ab[:, 1]
        W[rows, i1] += ab[:, 0]
        W[rows, i2] += ab[:, 1]
    uniq, inv = np.unique(W, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    pos = (uniq.astype(np.float64) @ iv) / n
    pos /= np.linalg.norm(pos, axis=1, keepdims=True)
    # local triangles (orientation inherited from the face)
    tl = []
    for a in range(n):
        for b in range(n - a):
            tl.append((local[(a, b)], local[(a + 1, b)], local[(a, b + 1)]))
            if a + b < n - 1:
                tl.append((local[(a + 1, b)], local[(a + 1, b + 1)], local[(a, b + 1)]))
    tl = np.array(tl, dtype=np.int64)
    tris = np.concatenate([inv[fi * npts + tl] for fi in range(20)], axis=0)
    # make orientation outward
    p0, p1, p2 = pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]
    nrm = np.cross(p1 - p0, p2 - p0)
    flip = np.einsum("ij,ij->i", nrm, p0 + p1 + p2) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    tris = tris.astype(np.int32)
    _ICO_CACHE[freq] = (pos, tris)
    return pos.copy(), tris.copy()


def perturbed_ellipsoid(freq: int, radii, noise: float, seed: int, scale: float = 1.0):
    """Icosphere of frequency `freq`, scaled to `radii`, vertices + N(0, noise^2), times scale."""
    v, f = geodesic_sphere(freq)
    rng = np.random.default_rng(seed)
    v = v * np.asarray(radii, dtype=np.float64)[None, :]
    v = v + rng.normal(0.0, noise, size=v.shape)
    v = v * scale
    return np.ascontiguousarray(v, dtype=np.float64), np.ascontiguousarray(f, dtype=np.int32)


def haar_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def random_poses(n: int, lo, hi, seed: int) -> np.ndarray:
    """(n, 3, 4) transforms: Haar rotation, translation ~ U[lo, hi]^3."""
    rng = np.random.default_rng(seed)
    R = haar_rotations(n, rng)
    t = rng.uniform(lo, hi, size=(n, 3))
    tf = np.empty((n, 3, 4))
    tf[:, :, :3] = R
    tf[:, :, 3] = t
    return np.ascontiguousarray(tf)


def identity_poses(n: int) -> np.ndarray:
    tf = np.zeros((n, 3, 4))
    tf[:, 0, 0] = tf[:, 1, 1] = tf[:, 2, 2] = 1.0
    return tf


def grid_box(n: int, half=(0.5, 0.5, 0.5)) -> tuple[np.ndarray, np.ndarray]:
    """Surface of an axis-aligned box with half-extents `half`, each face split into
    n x n squares of two triangles (12 n^2 triangles, outward winding).  Faces meet at
    shared vertices; flat faces and parallel edges give ties in contact depths."""
    g = np.linspace(-1.0, 1.0, n + 1)
    verts, tris, index = [], [], {}

    def vid(p):
        key = tuple(np.round(p, 12))
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    for axis in range(3):
        for sign in (-1.0, 1.0):
            u, v = (axis + 1) % 3, (axis + 2) % 3
            for i in range(n):
                for j in range(n):
                    quad = []
                    for di, dj in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        p = np.zeros(3)
                        p[axis] = sign
                        p[u] = g[i + di]
                        p[v] = g[j + dj]
                        quad.append(vid(p * np.asarray(half, float)))
                    a, b, c, d = quad
                    if sign > 0:
                        tris += [(a, b, c), (a, c, d)]
                    else:
                        tris += [(a, c, b), (a, d, c)]
    return np.asarray(verts, np.float64), np.asarray(tris, np.int32)


# ---------------------------------------------------------------------------------
# Mesh-pair workloads
# ---------------------------------------------------------------------------------

@dataclass
class MeshPairWorkload:
    """meshes: list of (verts, tris); pairs: (P, 2) mesh indices; queries reference
    a pair via `pair` and carry tf1 (None = identity) and tf2."""
    meshes: list
    pairs: np.ndarray
    pair: np.ndarray      # (N,) int32
    tf2: np.ndarray       # (N, 3, 4)
    tf1: np.ndarray | None = None
    margin: np.ndarray | None = None   # (N,) tolerance for the distance check
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.pair.shape[0])


def config0(n_poses: int = 10000, seed: int = 0, freq: int = 16) -> MeshPairWorkload:
    """Plain method, 5,120-triangle perturbed ellipsoids, 10,000 poses in [-2,2]^3."""
    a = perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed)
    b = perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed + 1, scale=0.8)
    tf2 = random_poses(n_poses, -2.0, 2.0, seed + 7)
    return MeshPairWorkload(meshes=[a, b], pairs=np.array([[0, 1]], np.int32),
                            pair=np.zeros(n_poses, np.int32), tf2=tf2, name="c0")


def _loguniform_int(rng, lo, hi, size=None):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=size))


def mesh_pair_set(n_pairs: int = 64, seed: int = 1, tri_lo: int = 500, tri_hi: int = 200000):
    """64 mesh pairs: triangle counts log-uniform in [500, 200k] (geodesic frequency
    round(sqrt(T/20))), radii U[0.5,1.5]^3, N(0, 0.01^2) vertex noise."""
    rng = np.random.default_rng(seed)
    meshes = []
    for k in range(2 * n_pairs):
        T = _loguniform_int(rng, tri_lo, tri_hi)
        freq = max(1, int(round(math.sqrt(T / 20.0))))
        radii = rng.uniform(0.5, 1.5, size=3)
        meshes.append(perturbed_ellipsoid(freq, radii, 0.01, seed * 100003 + k))
    pairs = np.arange(2 * n_pairs, dtype=np.int32).reshape(n_pairs, 2)
    return meshes, pairs


def mesh_pair_set_subset(pair_ids, n_pairs: int = 64, seed: int = 1, tri_lo: int = 500, tri_hi: int = 200000):
    """Only the meshes of the listed pairs of mesh_pair_set (same draws, same meshes),
    as {mesh index: (verts, tris)}; the rest of the set is not generated."""
    rng = np.random.default_rng(seed)
    want = {2 * int(p) + j for p in pair_ids for j in (0, 1)}
    out = {}
    for k in range(2 * n_pairs):
        T = _loguniform_int(rng, tri_lo, tri_hi)
        freq = max(1, int(round(math.sqrt(T / 20.0))))
        radii = rng.uniform(0.5, 1.5, size=3)
        if k in want:
            out[k] = perturbed_ellipsoid(freq, radii, 0.01, seed * 100003 + k)
    return out


def config1(scale: float = 1.0, seed: int = 1, n_pairs: int = 64, tri_hi: int = 200000,
            pose_lo: int = 2000, pose_hi: int = 50000) -> MeshPairWorkload:
    """Exhaustive contacts: per pair log-uniform [2,000, 50,000] poses (times `scale`),
    translations U[-1.5,1.5]^3."""
    meshes, pairs = mesh_pair_set(n_pairs, seed, tri_hi=tri_hi)
    rng = np.random.default_rng(seed + 11)
    counts = np.maximum(1, np.round(_loguniform_int(rng, pose_lo, pose_hi, size=n_pairs) * scale)).astype(np.int64)
    pair = np.repeat(np.arange(n_pairs, dtype=np.int32), counts)
    tf2 = random_poses(int(counts.sum()), -1.5, 1.5, seed + 13)
    return MeshPairWorkload(meshes=meshes, pairs=pairs, pair=pair, tf2=tf2, name="c1")


def config2(total_poses: int = 1_000_000, seed: int = 1, n_pairs: int = 64, tri_hi: int = 200000
            ) -> MeshPairWorkload:
    """Distance batch over the same pair set: poses spread in proportion to the
    exhaustive-contact counts, translations U[1.5,4]^3, margins U[0.01,0.2]."""
    meshes, pairs = mesh_pair_set(n_pairs, seed, tri_hi=tri_hi)
    rng = np.random.default_rng(seed + 11)
    w = _loguniform_int(rng, 2000, 50000, size=n_pairs)
    counts = np.maximum(1, np.floor(w / w.sum() * total_poses)).astype(np.int64)
    counts[0] += total_poses - counts.sum()
    pair = np.repeat(np.arange(n_pairs, dtype=np.int32), counts)
    tf2 = random_poses(int(counts.sum()), 1.5, 4.0, seed + 17)
    margin = np.random.default_rng(seed + 19).uniform(0.01, 0.2, size=pair.shape[0])
    return MeshPairWorkload(meshes=meshes, pairs=pairs, pair=pair, tf2=tf2, margin=margin, name="c2")


def subsample_indices(total: int, n: int, seed: int = 0) -> np.ndarray:
    """The query indices subsample() keeps: n drawn uniformly without replacement, sorted."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(total, size=min(n, total), replace=False))


def subsample(w: MeshPairWorkload, n: int, seed: int = 0) -> MeshPairWorkload:
    """A uniform random subset of n queries (sorted by original order)."""
    idx = subsample_indices(w.n, n, seed)
    return MeshPairWorkload(meshes=w.meshes, pairs=w.pairs, pair=w.pair[idx], tf2=w.tf2[idx],
                            tf1=None if w.tf1 is None else w.tf1[idx],
                            margin=None if w.margin is None else w.margin[idx], name=w.name + "_sub")


# ---------------------------------------------------------------------------------
# Convex shape pairs (GJK/EPA batch)
# ---------------------------------------------------------------------------------
BOX, SPHERE, CAPSULE, CYLINDER, CONE, CONVEX = 0, 1, 2, 3, 4, 5


@dataclass
class ShapeSet:
    """Shapes as arrays: type[n], params[n,3] (box sides; sphere r; capsule/cylinder/
    cone r, lz), convex vertex ranges voff/vcnt into verts[m,3]."""
    type: np.ndarray
    params: np.ndarray
    voff: np.ndarray
    vcnt: np.ndarray
    verts: np.ndarray

    @property
    def n(self) -> int:
        return int(self.type.shape[0])


def random_shapes(n: int, seed: int) -> ShapeSet:
    """Box sides U[0.1,1]; Sphere r U[0.05,0.5]; Capsule/Cylinder/Cone r U[0.05,0.3],
    lz U[0.1,1]; Convex = hull of 32-256 points uniform in the unit ball scaled U[0.2,1]."""
    from scipy.spatial import ConvexHull
    rng = np.random.default_rng(seed)
    typ = rng.integers(0, 6, size=n).astype(np.int32)
    params = np.zeros((n, 3))
    voff = np.zeros(n, np.int32)
    vcnt = np.zeros(n, np.int32)
    verts = []
    off = 0
    for i in range(n):
        t = typ[i]
        if t == BOX:
            params[i] = rng.uniform(0.1, 1.0, 3)
        elif t == SPHERE:
            params[i, 0] = rng.uniform(0.05, 0.5)
        elif t in (CAPSULE, CYLINDER, CONE):
            params[i, 0] = rng.uniform(0.05, 0.3)
            params[i, 1] = rng.uniform(0.1, 1.0)
        else:
            m = int(rng.integers(32, 257))
            d = rng.normal(size=(m, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            pts = d * rng.uniform(0, 1, size=(m, 1)) ** (1.0 / 3.0) * rng.uniform(0.2, 1.0)
            hv = pts[np.sort(ConvexHull(pts).vertices)]
            voff[i] = off
            vcnt[i] = hv.shape[0]
            off += hv.shape[0]
            verts.append(hv)
    V = np.concatenate(verts) if verts else np.zeros((0, 3))
    return ShapeSet(typ, params, voff, vcnt, np.ascontiguousarray(V))


@dataclass
class ShapePairWorkload:
    shapes: ShapeSet
    ia: np.ndarray
    ib: np.ndarray
    tf1: np.ndarray
    tf2: np.ndarray

    @property
    def n(self) -> int:
        return int(self.ia.shape[0])


def config3(n_pairs: int = 4_000_000, n_shapes: int = 4096, seed: int = 3) -> ShapePairWorkload:
    """Convex GJK/EPA batch: pairs of random shapes, both posed by a Haar rotation and
    a translation in [-1,1]^3."""
    shapes = random_shapes(n_shapes, seed)
    rng = np.random.default_rng(seed + 1)
    ia = rng.integers(0, n_shapes, size=n_pairs).astype(np.int32)
    ib = rng.integers(0, n_shapes, size=n_pairs).astype(np.int32)
    tf1 = random_poses(n_pairs, -1.0, 1.0, seed + 2)
    tf2 = random_poses(n_pairs, -1.0, 1.0, seed + 3)
    return ShapePairWorkload(shapes, ia, ib, tf1, tf2)


# ---------------------------------------------------------------------------------
# Broadphase scene and motion-checking requests
# ---------------------------------------------------------------------------------

def concat_shapes(a: ShapeSet, b: ShapeSet) -> ShapeSet:
    """Shape set with a's shapes first, then b's (convex vertex offsets of b shifted)."""
    na_v = a.verts.shape[0]
    voff_b = np.where(b.type == CONVEX, b.voff + na_v, 0).astype(np.int32)
    return ShapeSet(np.concatenate([a.type, b.type]).astype(np.int32), np.concatenate([a.params, b.params]),
                    np.concatenate([a.voff, voff_b]).astype(np.int32),
                    np.concatenate([a.vcnt, b.vcnt]).astype(np.int32),
                    np.ascontiguousarray(np.concatenate([a.verts.reshape(-1, 3), b.verts.reshape(-1, 3)])))


@dataclass
class Robot:
    """A serial chain: joint i turns about a coordinate axis of the frame left by
    link i-1 (axis 0/1/2 = x/y/z), then link i extends by `offset[i]`.  Link i's
    geometry (`link_refs[i]`, kind/index into the registry) sits at `geom_tf[i]`
    (3x4) in the joint frame."""
    axis: np.ndarray        # (L,) int32
    offset: np.ndarray      # (L, 3)
    link_refs: np.ndarray   # (L, 2) int32
    geom_tf: np.ndarray     # (L, 3, 4)

    @property
    def n_links(self) -> int:
        return int(self.axis.shape[0])


@dataclass
class SceneWorkload:
    """Registry (shapes, meshes) shared by scene and robot; scene objects as refs + poses."""
    shapes: ShapeSet
    meshes: list
    refs: np.ndarray   # (N, 2) int32
    tf: np.ndarray     # (N, 3, 4)
    robot: Robot

    @property
    def n(self) -> int:
        return int(self.refs.shape[0])


def _rot_y90() -> np.ndarray:
    # maps the local z axis (capsule axis) onto x
    return np.array([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0]])


def scene4(n_objects: int | None = None, seed: int = 4, box: float = 20.0, n_shape_geoms: int = 1024,
           n_mesh_geoms: int = 16, mesh_fraction: float = 0.25, tri_lo: int = 500, tri_hi: int = 5000,
           n_links: int = 20, mesh_links: bool = True, link_tris: int = 2000) -> SceneWorkload:
    """Serving scene: N ~ logU[1000, 50000] objects (or n_objects), each a random convex
    primitive (the convex-pair recipe) or, with probability mesh_fraction, one of
    n_mesh_geoms perturbed icospheres of logU[tri_lo, tri_hi] triangles (radii
    U[0.3, 1.0]^3); Haar rotations, positions U[0, box]^3.  The robot has n_links
    links of length U[0.25, 0.4]; even links are capsules (r 0.06), odd links (when
    mesh_links) ellipsoid meshes of link_tris triangles along the link."""
    rng = np.random.default_rng(seed)
    if n_objects is None:
        n_objects = int(_loguniform_int(rng, 1000, 50000))
    scene_shapes = random_shapes(n_shape_geoms, seed + 1)
    meshes = []
    if mesh_fraction > 0:
        for k in range(n_mesh_geoms):
            T = _loguniform_int(rng, tri_lo, tri_hi)
            freq = max(1, int(round(math.sqrt(T / 20.0))))
            meshes.append(perturbed_ellipsoid(freq, rng.uniform(0.3, 1.0, size=3), 0.01, seed * 7919 + k))
    # robot link geometries
    lengths = rng.uniform(0.25, 0.4, size=n_links)
    link_types, link_params = [], []
    link_refs = np.zeros((n_links, 2), np.int32)
    geom_tf = np.zeros((n_links, 3, 4))
    freq_link = max(1, int(round(math.sqrt(link_tris / 20.0))))
    for i in range(n_links):
        L = lengths[i]
        geom_tf[i, :, 3] = (L / 2, 0.0, 0.0)
        if mesh_links and i % 2 == 1:
            link_refs[i] = (1, len(meshes))
            meshes.append(perturbed_ellipsoid(freq_link, (L / 2, 0.08, 0.08), 0.002, seed * 104729 + i))
            geom_tf[i, :, :3] = np.eye(3)
        else:
            link_refs[i] = (0, n_shape_geoms + len(link_types))
            link_types.append(CAPSULE)
            link_params.append((0.06, L, 0.0))
            geom_tf[i, :, :3] = _rot_y90()
    robot_shapes = ShapeSet(np.array(link_types, np.int32), np.array(link_params, np.float64).reshape(-1, 3),
                            np.zeros(len(link_types), np.int32), np.zeros(len(link_types), np.int32),
                            np.zeros((0, 3)))
    shapes = concat_shapes(scene_shapes, robot_shapes)
    n_scene_meshes = n_mesh_geoms if mesh_fraction > 0 else 0
    is_mesh = rng.uniform(size=n_objects) < mesh_fraction if n_scene_meshes else np.zeros(n_objects, bool)
    refs = np.zeros((n_objects, 2), np.int32)
    refs[:, 0] = is_mesh.astype(np.int32)
    refs[:, 1] = np.where(is_mesh, rng.integers(0, max(1, n_scene_meshes), size=n_objects),
                          rng.integers(0, n_shape_geoms, size=n_objects))
    tf = np.empty((n_objects, 3, 4))
    tf[:, :, :3] = haar_rotations(n_objects, rng)
    tf[:, :, 3] = rng.uniform(0.0, box, size=(n_objects, 3))
    axis = np.array([2 if i % 2 == 0 else 1 for i in range(n_links)], np.int32)
    offset = np.zeros((n_links, 3))
    offset[:, 0] = lengths
    robot = Robot(axis, offset, link_refs, geom_tf)
    return SceneWorkload(shapes, meshes, refs, np.ascontiguousarray(tf), robot)


def joint_rotation(axis: int, q: np.ndarray) -> np.ndarray:
    c, s = np.cos(q), np.sin(q)
    R = np.zeros(q.shape + (3, 3))
    if axis == 0:
        R[..., 0, 0] = 1; R[..., 1, 1] = c; R[..., 1, 2] = -s; R[..., 2, 1] = s; R[..., 2, 2] = c
    elif axis == 1:
        R[..., 0, 0] = c; R[..., 0, 2] = s; R[..., 1, 1] = 1; R[..., 2, 0] = -s; R[..., 2, 2] = c
    else:
        R[..., 0, 0] = c; R[..., 0, 1] = -s; R[..., 1, 0] = s; R[..., 1, 1] = c; R[..., 2, 2] = 1
    return R


def robot_fk(robot: Robot, base: np.ndarray, q: np.ndarray) -> np.ndarray:
    """World poses (K, L, 3, 4) of the link geometries for joint angles q (K, L)."""
    q = np.asarray(q, np.float64)
    K, L = q.shape
    R = np.broadcast_to(base[:3, :3], (K, 3, 3)).copy()
    t = np.broadcast_to(base[:3, 3], (K, 3)).copy()
    out = np.empty((K, L, 3, 4))
    for i in range(L):
        R = R @ joint_rotation(int(robot.axis[i]), q[:, i])
        G = robot.geom_tf[i]
        out[:, i, :, :3] = R @ G[:, :3]
        out[:, i, :, 3] = t + R @ G[:, 3]
        t = t + R @ robot.offset[i]
    return out


@dataclass
class MotionRequest:
    base: np.ndarray   # (3, 4)
    q: np.ndarray      # (K, L) joint angles per waypoint


def motion_requests(w: SceneWorkload, n_requests: int, seed: int = 5, k_lo: int = 10, k_hi: int = 500,
                    sigma: float = 0.05) -> list:
    """Requests: base pose uniform in the scene box (Haar rotation), K ~ logU[k_lo,
    k_hi] waypoints of a joint-space random walk with step N(0, sigma^2) from a start
    uniform in [-pi, pi]^L."""
    rng = np.random.default_rng(seed)
    box = float(w.tf[:, :, 3].max()) if w.n else 20.0
    out = []
    L = w.robot.n_links
    for _ in range(n_requests):
        K = int(_loguniform_int(rng, k_lo, k_hi + 1))
        K = max(k_lo, min(k_hi, K))
        base = np.zeros((3, 4))
        base[:, :3] = haar_rotations(1, rng)[0]
        base[:, 3] = rng.uniform(0.0, box, size=3)
        q0 = rng.uniform(-math.pi, math.pi, size=L)
        q = q0[None, :] + np.cumsum(rng.normal(0.0, sigma, size=(K, L)), axis=0)
        q[0] = q0
        out.append(MotionRequest(base, np.ascontiguousarray(q)))
    return out
