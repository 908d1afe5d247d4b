"""Generates tests/golden/env_rob.npz from the reference's own test fixtures.

Reads FCL's test meshes test/fcl_resources/env.obj (2,180 triangles) and rob.obj
(216 triangles) the way test/test_fcl_utility.h:193-278 (loadOBJFile) does, and the
poses of test_fcl_collision.cpp:313-328 / test_fcl_distance.cpp:95-102: n = 10
transforms from generateRandomTransforms (test_fcl_utility.h:348-372) with extents
(-3000,-3000,0)..(3000,3000,3000), Euler angles in [0, 2pi) mapped by eulerToMatrix
(:313-325), driven by glibc rand() from its default seed.

Usage:  python tests/golden/make_fixtures.py FCL_CHECKOUT
where FCL_CHECKOUT is the root of an FCL source tree (the directory holding
test/fcl_resources).
"""
import argparse
import ctypes
import math
import os

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "env_rob.npz")


def load_obj(path):
    pts, tris = [], []
    with open(path, "rb") as f:
        for raw in f:
            tok = raw.decode().replace("\r", " ").replace("\t", " ").split()
            if not tok or tok[0].startswith("#"):
                continue
            if tok[0] == "v":
                pts.append([float(tok[1]), float(tok[2]), float(tok[3])])
            elif tok[0] == "f":
                ids = [int(x.split("/")[0]) - 1 for x in tok[1:]]
                for t in range(len(ids) - 2):
                    tris.append([ids[0], ids[t + 1], ids[t + 2]])
    return np.array(pts, np.float64), np.array(tris, np.int32)


def euler_to_matrix(a, b, c):
    c1, c2, c3 = math.cos(a), math.cos(b), math.cos(c)
    s1, s2, s3 = math.sin(a), math.sin(b), math.sin(c)
    return np.array([[c1 * c2, -c2 * s1, s2],
                     [c3 * s1 + c1 * s2 * s3, c1 * c3 - s1 * s2 * s3, -c2 * s3],
                     [s1 * s3 - c1 * c3 * s2, c3 * s1 * s2 + c1 * s3, c2 * c3]])


def reference_transforms(n, extents):
    libc = ctypes.CDLL("libc.so.6")
    RAND_MAX = 2147483647

    def rand_interval(lo, hi):
        t = libc.rand() / (float(RAND_MAX) + 1)
        return t * (hi - lo) + lo

    out = np.zeros((n, 3, 4))
    for i in range(n):
        x = rand_interval(extents[0], extents[3])
        y = rand_interval(extents[1], extents[4])
        z = rand_interval(extents[2], extents[5])
        a = rand_interval(0.0, 2 * math.pi)
        b = rand_interval(0.0, 2 * math.pi)
        c = rand_interval(0.0, 2 * math.pi)
        out[i, :, :3] = euler_to_matrix(a, b, c)
        out[i, :, 3] = [x, y, z]
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("fcl_checkout", help="root of an FCL source tree (holds test/fcl_resources)")
    res = os.path.join(ap.parse_args().fcl_checkout, "test", "fcl_resources")
    ev, et = load_obj(os.path.join(res, "env.obj"))
    rv, rt = load_obj(os.path.join(res, "rob.obj"))
    tfs = reference_transforms(10, (-3000, -3000, 0, 3000, 3000, 3000))
    np.savez_compressed(OUT, env_v=ev, env_t=et, rob_v=rv, rob_t=rt, tf=tfs)
    print("wrote", OUT, ev.shape, et.shape, rv.shape, rt.shape)


if __name__ == "__main__":
    main()
