"""ctypes access to oracle/_ref (the reference's own host code compiled in place
with stand-ins for its absent third-party libraries). TEST INFRASTRUCTURE:
available only where the reference tree exists."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref

_lib = None


def available() -> bool:
    return build_ref.available()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            raise RuntimeError("reference tree not available")
        L = C.CDLL(str(path))
        P = C.c_void_p
        L.ref_part_count.restype = C.c_int
        L.ref_part_sizes.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_get_part.argtypes = [C.c_int, P, P, P, P]
        L.ref_get_maps.argtypes = [P, P]
        L.ref_set_seed.argtypes = [C.c_uint]
        L.ref_clip.argtypes = [P, C.c_int, P, C.c_int, P]
        L.ref_separate_disjoint.argtypes = [P, C.c_int, P, C.c_int]
        L.ref_extract_surfaces.argtypes = [P, C.c_int, P, C.c_int, C.c_double, P, P, C.c_int]
        L.ref_candidate_planes.argtypes = [P, C.c_int, P, C.c_int, C.c_int, P]
        L.ref_compute_h.argtypes = [P, C.c_int, P, C.c_int, C.c_double, C.c_uint]
        L.ref_compute_h.restype = C.c_double
        L.ref_hull_volume.argtypes = [P, C.c_int, C.POINTER(C.c_int)]
        L.ref_hull_volume.restype = C.c_double
        L.ref_hull_bt.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, C.POINTER(C.c_int)]
        L.ref_hull_bt.restype = C.c_int
        L.ref_multimerge.argtypes = [P, P, P, P, C.c_int, C.c_double, C.c_double, C.c_uint]
        L.ref_multimerge.restype = C.c_int
        L.ref_score_trace.argtypes = [P, C.c_int]
        L.ref_score_trace.restype = C.c_int
        L.ref_process.argtypes = [P, C.c_int, P, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                  C.c_int, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _vt(v, t):
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(t, dtype=np.int32).reshape(-1, 3)
    return v, t


def parts():
    L = lib()
    out = []
    for i in range(L.ref_part_count()):
        nv, nt, ne = C.c_int(), C.c_int(), C.c_int()
        L.ref_part_sizes(i, C.byref(nv), C.byref(nt), C.byref(ne))
        v = np.zeros((nv.value, 3))
        t = np.zeros((nt.value, 3), np.int32)
        nw = np.zeros(nv.value, np.uint8)
        e = np.zeros((ne.value, 2), np.uint32)
        L.ref_get_part(i, _p(v), _p(t), _p(nw), _p(e))
        out.append({"vertices": v, "triangles": t, "is_new": nw, "edges": e})
    return out


def set_seed(seed: int) -> None:
    lib().ref_set_seed(seed)


def clip(v, t, plane):
    v, t = _vt(v, t)
    pl = np.ascontiguousarray(plane, dtype=np.float64)
    lib().ref_clip(_p(v), len(v), _p(t), len(t), _p(pl))
    m1 = np.zeros(len(v), np.int32)
    m2 = np.zeros(len(v), np.int32)
    lib().ref_get_maps(_p(m1), _p(m2))
    return parts(), m1, m2


def separate_disjoint(v, t):
    v, t = _vt(v, t)
    lib().ref_separate_disjoint(_p(v), len(v), _p(t), len(t))
    return parts()


def extract_surfaces(v, t, min_area):
    v, t = _vt(v, t)
    cap = 64
    pl = np.zeros((cap, 4))
    ar = np.zeros(cap)
    n = lib().ref_extract_surfaces(_p(v), len(v), _p(t), len(t), min_area, _p(pl), _p(ar), cap)
    return pl[:n], ar[:n]


def candidate_planes(v, edges, num):
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((num, 4))
    n = lib().ref_candidate_planes(_p(v), len(v), _p(e), len(e), num, _p(out))
    return out[:n]


def compute_h(v, t, k, res):
    v, t = _vt(v, t)
    return lib().ref_compute_h(_p(v), len(v), _p(t), len(t), k, res)


def hull_volume(v):
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    nt = C.c_int()
    vol = lib().ref_hull_volume(_p(v), len(v), C.byref(nt))
    return vol, nt.value


def hull_bt(v):
    """The reference's btConvexHullComputer hull (Mesh::compute_vch): hull
    vertices and fan-triangulated faces."""
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    cap = 2 * len(v) + 16
    ov = np.zeros((cap, 3), np.float64)
    ot = np.zeros((4 * cap, 3), np.int32)
    nv = C.c_int()
    nt = lib().ref_hull_bt(_p(v), len(v), _p(ov), cap, _p(ot), 4 * cap, C.byref(nv))
    if nt < 0:
        raise ValueError("hull buffers too small")
    return ov[: nv.value], ot[:nt]


def score_trace():
    """The reference loop's split searches since the last call: rows of
    (planes, points, edges, first float maximum, its score)."""
    out = np.zeros((4096, 5))
    n = lib().ref_score_trace(_p(out), 4096)
    return out[:n]


def multimerge(meshes, current_concavity, threshold, seed):
    """The reference's multimerge_ch on parts [(v, t), ...] (hulls from
    compute_ch, engine seeded with seed): the merged hulls."""
    v = np.ascontiguousarray(np.concatenate([p[0] for p in meshes]), dtype=np.float64)
    t = np.ascontiguousarray(np.concatenate([p[1] for p in meshes]), dtype=np.int32)
    nv = np.array([len(p[0]) for p in meshes], np.int32)
    nt = np.array([len(p[1]) for p in meshes], np.int32)
    lib().ref_multimerge(_p(v), _p(nv), _p(t), _p(nt), len(meshes), current_concavity, threshold,
                         seed)
    return parts()


def process(v, t, concavity, num_parts, seed, score_mode="concavity", return_parts=False,
            use_merging=False):
    v, t = _vt(v, t)
    set_seed(seed)
    c = C.c_double()
    n = lib().ref_process(_p(v), len(v), _p(t), len(t), concavity, num_parts,
                          int(score_mode == "edge"), int(return_parts), int(use_merging),
                          C.byref(c))
    return n, c.value, parts()
