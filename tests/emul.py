"""ctypes wrapper of the test-only host build of the product traversal (tests/native)."""
import ctypes as C

import numpy as np

from tests.native import build_emul

_E = None


def lib():
    global _E
    if _E is None:
        _E = C.CDLL(build_emul.build())
        _E.emu_collide.restype = C.c_int64
        _E.emu_build.restype = C.c_int
    return _E


def _p(a):
    return C.c_void_p(a.ctypes.data)


def build(v, t):
    v = np.ascontiguousarray(v, np.float64); t = np.ascontiguousarray(t, np.int32)
    nn = 2 * t.shape[0] - 1
    out = np.empty((nn, 30)); fc = np.empty(nn, np.int32); md = C.c_int32()
    lib().emu_build(_p(v), C.c_int64(v.shape[0]), _p(t), C.c_int64(t.shape[0]), _p(out), _p(fc), C.byref(md))
    return out, fc, md.value


def refit(v0, t, frames, replace=None):
    """Device refit math run on the host: build from v0, then refit to each frame
    (replace[f] true: the frame replaces the vertices, no previous frame)."""
    v0 = np.ascontiguousarray(v0, np.float64); t = np.ascontiguousarray(t, np.int32)
    vs = np.ascontiguousarray(np.stack(frames), np.float64)
    rp = np.ascontiguousarray(np.zeros(len(frames)) if replace is None else replace, np.int32)
    nn = 2 * t.shape[0] - 1
    out = np.empty((nn, 30)); fc = np.empty(nn, np.int32)
    lib().emu_refit(_p(v0), C.c_int64(v0.shape[0]), _p(t), C.c_int64(t.shape[0]), _p(vs), C.c_int(len(frames)),
                    _p(out), _p(fc), _p(rp))
    return out, fc


def collide(prec, a, b, tf2, maxc, tf1=None):
    n = tf2.shape[0]
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(n, 12)
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(n, 12)
    counts = np.zeros(n, np.int32)
    cap = 1 << 22
    out = np.empty((cap, 2), np.int32)
    nbv = np.zeros(n, np.int64); nl = np.zeros(n, np.int64); nrc = np.zeros(n, np.int64)
    av, at = [np.ascontiguousarray(x) for x in a]
    bv, bt = [np.ascontiguousarray(x) for x in b]
    tot = lib().emu_collide(C.c_int(prec), _p(av), C.c_int64(av.shape[0]), _p(at), C.c_int64(at.shape[0]),
                            _p(bv), C.c_int64(bv.shape[0]), _p(bt), C.c_int64(bt.shape[0]), C.c_int64(n),
                            None if tf1a is None else _p(tf1a), _p(tf2), C.c_int(maxc), _p(counts), _p(out),
                            C.c_int64(cap), _p(nbv), _p(nl), _p(nrc))
    assert 0 <= tot <= cap
    return counts, out[:tot], nbv, nl, nrc


def collide_split(prec, a, b, tf2, maxc, budget, tf1=None):
    n = tf2.shape[0]
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(n, 12)
    tf1a = None if tf1 is None else np.ascontiguousarray(tf1, np.float64).reshape(n, 12)
    counts = np.zeros(n, np.int32)
    cap = 1 << 22
    out = np.empty((cap, 2), np.int32)
    nbv = np.zeros(n, np.int64); nl = np.zeros(n, np.int64); ni = C.c_int64()
    av, at = [np.ascontiguousarray(x) for x in a]
    bv, bt = [np.ascontiguousarray(x) for x in b]
    lib().emu_collide_split.restype = C.c_int64
    tot = lib().emu_collide_split(C.c_int(prec), _p(av), C.c_int64(av.shape[0]), _p(at), C.c_int64(at.shape[0]),
                                  _p(bv), C.c_int64(bv.shape[0]), _p(bt), C.c_int64(bt.shape[0]), C.c_int64(n),
                                  None if tf1a is None else _p(tf1a), _p(tf2), C.c_int(maxc), C.c_int64(budget),
                                  _p(counts), _p(out), C.c_int64(cap), _p(nbv), _p(nl), C.byref(ni))
    assert 0 <= tot <= cap
    return counts, out[:tot], nbv, nl, ni.value


def shape_batch(shapes, ia, ib, tf1, tf2):
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
    lib().emu_shape_batch(C.c_int(t.shape[0]), _p(t), _p(pr), _p(vo), _p(vc), _p(vv), C.c_int64(n), _p(ia), _p(ib),
                          _p(tf1), _p(tf2), *(_p(out[k]) for k in ("hit", "normal", "point", "depth", "dist", "p1",
                                                                    "p2", "status")))
    out["hit"] = out["hit"].astype(bool)
    return out


def tri_contact_batch(P, Qm):
    """tri_contact.cuh on the host: (counts, points (n,2,3), normal (n,3), depth (n,))."""
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 9)
    Qm = np.ascontiguousarray(Qm, np.float64).reshape(-1, 9)
    n = P.shape[0]
    cnt = np.empty(n, np.int32); pts = np.empty((n, 2, 3)); nrm = np.empty((n, 3)); dep = np.empty(n)
    lib().emu_tri_contact_batch(C.c_int64(n), _p(P), _p(Qm), _p(cnt), _p(pts), _p(nrm), _p(dep))
    return cnt, pts, nrm, dep


def motion(beg, end, t, kind="trans"):
    """motion.cuh's motions on the host: (n,3,4) transforms at times t."""
    beg = np.ascontiguousarray(beg, np.float64).reshape(-1, 12)
    end = np.ascontiguousarray(end, np.float64).reshape(-1, 12)
    t = np.ascontiguousarray(t, np.float64)
    out = np.empty((beg.shape[0], 3, 4))
    lib().emu_motion(C.c_int({"trans": 0, "linear": 1, "screw": 2}[kind]), C.c_int64(beg.shape[0]), _p(beg),
                     _p(end), _p(t), _p(out))
    return out


def translation_motion(beg, end, t):
    return motion(beg, end, t, "trans")


def distance_cert(a, b, tf2):
    """The certified FP32 distance traversal run on the host (tf1 = I)."""
    n = tf2.shape[0]
    tf2 = np.ascontiguousarray(tf2, np.float64).reshape(n, 12)
    d = np.zeros(n); ids = np.zeros((n, 2), np.int32); pts = np.zeros((n, 2, 3))
    nbv = np.zeros(n, np.int64); nl = np.zeros(n, np.int64); nrc = np.zeros(n, np.int64)
    av, at = [np.ascontiguousarray(x) for x in a]
    bv, bt = [np.ascontiguousarray(x) for x in b]
    rc = lib().emu_distance_cert(_p(av), C.c_int64(av.shape[0]), _p(at), C.c_int64(at.shape[0]), _p(bv),
                                 C.c_int64(bv.shape[0]), _p(bt), C.c_int64(bt.shape[0]), C.c_int64(n), _p(tf2),
                                 _p(d), _p(ids), _p(pts), _p(nbv), _p(nl), _p(nrc))
    assert rc == 0
    return d, ids, pts, nbv, nl, nrc
