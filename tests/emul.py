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
