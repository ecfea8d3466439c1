"""ctypes binding of the C ABI in include/visacd_gpu.h (libvisacd_gpu.so).

This is how Python callers (tests, benchmarks, the host driver's debugging
tools) reach the sm_103a kernels without torch types. The library must exist:
a missing or unloadable library raises ImportError — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "libvisacd_gpu.so"

EXPORTED = [
    "visacd_last_error", "visacd_abi_version",
    "visacd_ctx_create", "visacd_ctx_destroy", "visacd_ctx_synchronize",
    "visacd_ctx_set_timing", "visacd_ctx_reset_times", "visacd_ctx_kernel_times",
    "visacd_ctx_launch_count", "visacd_ctx_sm_count",
    "visacd_bvh_build", "visacd_bvh_destroy", "visacd_bvh_info",
    "visacd_visibility", "visacd_visibility_edges", "visacd_visibility_edges_device",
    "visacd_compute_intersection_matrix",
    "visacd_vis_variant_count", "visacd_ctx_set_vis_variant", "visacd_autotune_visibility",
    "visacd_score_planes", "visacd_score_planes_noalloc", "classify_and_rate_planes",
    "visacd_clip", "visacd_clip_fetch", "visacd_measure_fp32_peak", "visacd_measure_tex_peak", "visacd_face_hausdorff",
    "visacd_face_hausdorff_floor", "visacd_face_hausdorff_batch",
    "visacd_batch_create", "visacd_batch_run", "visacd_batch_results", "visacd_batch_info",
    "visacd_batch_destroy",
    "visacd_lp_param_count", "visacd_lp_create", "visacd_lp_destroy", "visacd_lp_get_params",
    "visacd_lp_features", "visacd_lp_forward", "visacd_lp_propose", "visacd_lp_grads",
    "visacd_lp_train_step",
    "visacd_sdf_remesh", "visacd_sdf_fetch", "visacd_hull_distances", "visacd_segment_triangle_tests",
    "visacd_set_blocking_sync", "visacd_lp_set_tcgen05", "visacd_ctx_set_blocking_wait",
    "visacd_candidate_planes", "visacd_split_search", "visacd_visibility_batch",
    "visacd_learned_split_search", "visacd_ctx_set_vis_trace", "visacd_ctx_vis_trace_counts",
    "visacd_ctx_set_score_k", "visacd_autotune_scoring", "visacd_convex_hulls", "visacd_radix_sort_pairs",
]

LP_POINTS = 2048
LP_FEATURES = 7
LP_PLANES = 16


class ClipResult(C.Structure):
    _fields_ = [("n_pos", C.c_int32), ("n_neg", C.c_int32), ("nv_pos", C.c_int32),
                ("nv_neg", C.c_int32), ("n_border", C.c_int32), ("n_border_edges", C.c_int32),
                ("n_touching", C.c_int32)]


class VisStats(C.Structure):
    _fields_ = [("pairs_tested", C.c_int64), ("n_edges", C.c_int64), ("self_hits", C.c_int64),
                ("cage_hits", C.c_int64), ("fp64_rechecks", C.c_int64), ("degenerate", C.c_int64),
                ("node_visits", C.c_int64), ("tri_tests", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class ScoreStats(C.Structure):
    _fields_ = [("quantum_exp", C.c_int32), ("argmax", C.c_int32), ("band_blocks", C.c_int64),
                ("skipped_edges", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class SplitInfo(C.Structure):
    _fields_ = [("best_index", C.c_int32), ("n_candidates", C.c_int32), ("draws_used", C.c_int32),
                ("pad", C.c_int32), ("best_score", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class LearnedSplitInfo(C.Structure):
    _fields_ = [("best_index", C.c_int32), ("n_refined", C.c_int32), ("n_probe", C.c_int32),
                ("draws_used", C.c_int32), ("fallback", C.c_int32), ("reserved", C.c_int32),
                ("best_score", C.c_double), ("best_proposal_score", C.c_double),
                ("best_probe_score", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


def load() -> C.CDLL:
    if not _LIB_PATH.exists():
        raise ImportError(f"{_LIB_PATH} is missing: build it with visacd_gb300.build.build_gpu()")
    lib = C.CDLL(str(_LIB_PATH))
    P = C.c_void_p
    i32, i64 = C.c_int32, C.c_int64
    lib.visacd_last_error.restype = C.c_char_p
    lib.visacd_abi_version.restype = C.c_int
    lib.visacd_ctx_create.argtypes = [C.c_int, P, C.POINTER(P)]
    lib.visacd_ctx_destroy.argtypes = [P]
    lib.visacd_ctx_synchronize.argtypes = [P]
    lib.visacd_ctx_set_timing.argtypes = [P, C.c_int]
    lib.visacd_ctx_reset_times.argtypes = [P]
    lib.visacd_ctx_kernel_times.argtypes = [P, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                            C.POINTER(i64), C.c_int, C.POINTER(C.c_int)]
    lib.visacd_ctx_launch_count.argtypes = [P]
    lib.visacd_ctx_launch_count.restype = i64
    lib.visacd_ctx_sm_count.argtypes = [P]
    lib.visacd_bvh_build.argtypes = [P, P, i32, P, i32, C.c_int, C.POINTER(P)]
    lib.visacd_bvh_destroy.argtypes = [P]
    lib.visacd_bvh_info.argtypes = [P, C.POINTER(i32), C.POINTER(i32)]
    lib.visacd_visibility.argtypes = [P, P, i32, P, C.c_int, P, P, C.POINTER(i64),
                                      C.POINTER(VisStats)]
    lib.visacd_visibility_edges.argtypes = [P, P, i64]
    lib.visacd_visibility_edges_device.argtypes = [P, C.POINTER(P), C.POINTER(i64)]
    lib.visacd_compute_intersection_matrix.argtypes = [P, P, i32, P, i32, P, P, i32, P, i32, P,
                                                       i64, C.POINTER(i64), C.POINTER(VisStats)]
    lib.visacd_vis_variant_count.restype = C.c_int
    lib.visacd_ctx_set_vis_variant.argtypes = [P, C.c_int]
    lib.visacd_autotune_visibility.argtypes = [P, P, i32, P, C.c_int, P, P, C.POINTER(C.c_int),
                                               C.POINTER(C.c_double)]
    lib.visacd_score_planes.argtypes = [P, P, i32, P, i32, P, i64, C.c_int, P,
                                        C.POINTER(ScoreStats)]
    lib.visacd_score_planes_noalloc.argtypes = [P, i32, P, i32, P, i64, P, P, P]
    lib.visacd_visibility_batch.argtypes = [P, i32, C.POINTER(P), P, C.POINTER(P), C.POINTER(P),
                                            C.POINTER(P), P, C.POINTER(VisStats)]
    lib.visacd_candidate_planes.argtypes = [P, P, i32, P, i64, P, i32, i32, P, C.POINTER(i32),
                                            C.POINTER(i32)]
    lib.visacd_split_search.argtypes = [P, P, i32, P, i64, P, i32, i32, P, i32, C.c_double, P,
                                        C.POINTER(SplitInfo)]
    lib.visacd_ctx_set_score_k.argtypes = [P, C.c_int]
    lib.visacd_autotune_scoring.argtypes = [P, P, i32, P, i32, P, i64, C.c_int, C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]
    lib.visacd_ctx_set_vis_trace.argtypes = [P, C.c_int]
    lib.visacd_ctx_vis_trace_counts.argtypes = [P, C.POINTER(i64), C.POINTER(i64)]
    lib.visacd_learned_split_search.argtypes = [P, P, i32, P, i64, P, C.c_float, C.c_double, i32, P, i32,
                                                i32, P, i32, C.c_double, C.c_double, P,
                                                C.POINTER(LearnedSplitInfo)]
    lib.visacd_clip.argtypes = [P, P, i32, P, i32, P, C.POINTER(ClipResult)]
    lib.visacd_measure_fp32_peak.argtypes = [P, C.POINTER(C.c_double)]
    lib.visacd_measure_tex_peak.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.visacd_batch_create.argtypes = [P, i32, C.POINTER(P), P, C.POINTER(P), C.POINTER(P), C.POINTER(P),
                                        P, i64, C.POINTER(P)]
    lib.visacd_batch_run.argtypes = [P, P, C.c_int]
    lib.visacd_batch_results.argtypes = [P, P, P, P, P, P, i64]
    lib.visacd_batch_info.argtypes = [P, C.POINTER(i64), C.POINTER(i64)]
    lib.visacd_batch_destroy.argtypes = [P]
    lib.visacd_face_hausdorff.argtypes = [P, P, i32, P, i32, P, P, i32, P, i32, P, i32, P, P, i32,
                                          C.POINTER(C.c_double)]
    lib.visacd_face_hausdorff_floor.argtypes = [P, P, i32, P, i32, P, P, i32, P, i32, P, i32, P, P, i32,
                                                C.c_double, C.POINTER(C.c_double)]
    lib.visacd_face_hausdorff_batch.argtypes = [P, i32, P, P, P, P, P, P, P, P, C.c_double, i32, P]
    lib.visacd_clip_fetch.argtypes = [P, P, P, P, P, P, P]
    lib.classify_and_rate_planes.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_int]
    lib.classify_and_rate_planes.restype = None
    lib.visacd_sdf_remesh.argtypes = [P, P, i32, P, i32, C.c_double, C.c_double, C.POINTER(i32), C.POINTER(i32)]
    lib.visacd_sdf_fetch.argtypes = [P, P, P]
    lib.visacd_hull_distances.argtypes = [P, P, P, i32, P, i64, C.c_double, P]
    lib.visacd_convex_hulls.argtypes = [P, P, P, i32, i32, P, P]
    lib.visacd_radix_sort_pairs.argtypes = [P, P, P, i32, C.c_int]
    lib.visacd_segment_triangle_tests.argtypes = [P, P, P, i64, P, C.POINTER(i64)]
    lib.visacd_set_blocking_sync.argtypes = [C.c_int, C.c_int]
    lib.visacd_lp_param_count.argtypes = []
    lib.visacd_lp_create.argtypes = [P, P, C.c_uint32, C.POINTER(P)]
    lib.visacd_lp_destroy.argtypes = [P]
    lib.visacd_lp_get_params.argtypes = [P, P]
    lib.visacd_lp_features.argtypes = [P, P, i32, P, i64, P, C.c_float, P]
    lib.visacd_lp_forward.argtypes = [P, P, i32, P]
    lib.visacd_lp_propose.argtypes = [P, P, i32, P, i64, P, C.c_float, P]
    lib.visacd_lp_grads.argtypes = [P, P, P, P, i32, i32, P, P]
    lib.visacd_lp_train_step.argtypes = [P, P, P, P, i32, i32, C.c_float, P]
    lib.visacd_lp_set_tcgen05.argtypes = [P, C.c_int]
    return lib


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
    return _lib


class VisacdError(RuntimeError):
    pass


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = lib().visacd_last_error()
        raise VisacdError(f"{what} failed (status {rc}): {msg.decode() if msg else ''}")


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a, cols: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    return a.reshape(-1, cols)


def _u32(a, cols: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.uint32))
    return a.reshape(-1, cols)


class Context:
    """Owns a visacd_ctx (one CUDA stream + pooled device buffers)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = C.c_void_p()
        _check(lib().visacd_ctx_create(device, stream, C.byref(self._h)), "visacd_ctx_create")

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib().visacd_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self) -> None:
        _check(lib().visacd_ctx_synchronize(self._h), "synchronize")

    def set_timing(self, on: bool) -> None:
        _check(lib().visacd_ctx_set_timing(self._h, int(on)), "set_timing")

    def reset_times(self) -> None:
        _check(lib().visacd_ctx_reset_times(self._h), "reset_times")

    def kernel_times(self) -> dict[str, tuple[float, int]]:
        cap = 64
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        n_l = (C.c_int64 * cap)()
        n = C.c_int()
        _check(lib().visacd_ctx_kernel_times(self._h, names, ms, n_l, cap, C.byref(n)), "kernel_times")
        return {names[i].decode(): (ms[i], n_l[i]) for i in range(min(n.value, cap))}

    @property
    def launches(self) -> int:
        return int(lib().visacd_ctx_launch_count(self._h))

    @property
    def sm_count(self) -> int:
        return int(lib().visacd_ctx_sm_count(self._h))

    # ---- BVH / visibility ------------------------------------------------
    def bvh(self, verts, tris) -> "Bvh":
        return Bvh(self, verts, tris)

    def visibility(self, pts, self_bvh: "Bvh", cage_bvh: "Bvh", is_new=None):
        """Edges (E, 2) uint32 in row-major order, plus the counters."""
        p = _f32(pts, 3)
        m = None if is_new is None else np.ascontiguousarray(np.asarray(is_new, dtype=np.uint8))
        ne = C.c_int64()
        st = VisStats()
        _check(lib().visacd_visibility(self._h, _ptr(p), len(p), _ptr(m), 0, self_bvh.handle,
                                       cage_bvh.handle, C.byref(ne), C.byref(st)), "visacd_visibility")
        out = np.empty((ne.value, 2), dtype=np.uint32)
        _check(lib().visacd_visibility_edges(self._h, _ptr(out), ne.value), "visibility_edges")
        return out, st.as_dict()

    def visibility_batch(self, parts):
        """Several parts in one call: parts = [(pts, self_bvh, cage_bvh, is_new or None)].
        Returns (list of per-part edge arrays, summed counters)."""
        K = len(parts)
        pts = [_f32(p[0], 3) for p in parts]
        masks = [None if p[3] is None else np.ascontiguousarray(np.asarray(p[3], dtype=np.uint8)) for p in parts]
        pp = (C.c_void_p * K)(*[x.ctypes.data for x in pts])
        mp = (C.c_void_p * K)(*[None if m is None else m.ctypes.data for m in masks])
        n = np.array([len(x) for x in pts], np.int32)
        sb = (C.c_void_p * K)(*[p[1].handle.value for p in parts])
        cb = (C.c_void_p * K)(*[p[2].handle.value for p in parts])
        ne = np.zeros(K, np.int64)
        st = VisStats()
        _check(lib().visacd_visibility_batch(self._h, K, pp, _ptr(n), mp, sb, cb, _ptr(ne), C.byref(st)),
               "visacd_visibility_batch")
        total = int(ne.sum())
        flat = np.empty((total, 2), dtype=np.uint32)
        _check(lib().visacd_visibility_edges(self._h, _ptr(flat), total), "visibility_edges")
        out, at = [], 0
        for k in range(K):
            out.append(flat[at:at + ne[k]])
            at += int(ne[k])
        return out, st.as_dict()

    def set_score_k(self, k: int) -> None:
        """Force planes per scoring thread (1, 2, 4, 8; 0 = tuned / default)."""
        _check(lib().visacd_ctx_set_score_k(self._h, int(k)), "visacd_ctx_set_score_k")

    def autotune_scoring(self, planes, points, edges):
        """Time 1, 2, 4 and 8 planes per thread on this call, cache the fastest
        for its shape class: (best, ms per choice)."""
        pl = _f32(planes, 4)
        pt = _f32(points, 3)
        ed = _u32(edges, 2)
        best = C.c_int()
        ms = (C.c_double * 4)()
        _check(lib().visacd_autotune_scoring(self._h, _ptr(pl), len(pl), _ptr(pt), len(pt), _ptr(ed), len(ed),
                                             0, C.byref(best), ms), "visacd_autotune_scoring")
        return best.value, list(ms)

    def set_vis_trace(self, on: bool) -> None:
        """Free-space walks before the cage BVH in large visibility calls."""
        _check(lib().visacd_ctx_set_vis_trace(self._h, int(bool(on))), "visacd_ctx_set_vis_trace")

    def vis_trace_counts(self) -> tuple[int, int]:
        """(segments cleared by the walk, grid cells read) of the last visibility call."""
        a, b = C.c_int64(), C.c_int64()
        _check(lib().visacd_ctx_vis_trace_counts(self._h, C.byref(a), C.byref(b)), "vis_trace_counts")
        return a.value, b.value

    def set_vis_variant(self, v: int) -> None:
        _check(lib().visacd_ctx_set_vis_variant(self._h, v), "set_vis_variant")

    def autotune_visibility(self, pts, self_bvh: "Bvh", cage_bvh: "Bvh", is_new=None):
        p = _f32(pts, 3)
        m = None if is_new is None else np.ascontiguousarray(np.asarray(is_new, dtype=np.uint8))
        nv = lib().visacd_vis_variant_count()
        ms = (C.c_double * nv)()
        best = C.c_int()
        _check(lib().visacd_autotune_visibility(self._h, _ptr(p), len(p), _ptr(m), 0, self_bvh.handle,
                                                cage_bvh.handle, C.byref(best), ms), "autotune")
        return best.value, list(ms)

    def compute_intersection_matrix(self, verts, tris, cage_verts, cage_tris, is_new=None,
                                    capacity: int | None = None):
        v = _f32(verts, 3)
        t = _u32(tris, 3)
        cv = _f32(cage_verts, 3)
        ct = _u32(cage_tris, 3)
        m = None if is_new is None else np.ascontiguousarray(np.asarray(is_new, dtype=np.uint8))
        n = len(v)
        cap = capacity if capacity is not None else max(1, n * (n - 1) // 2)
        out = np.empty((cap, 2), dtype=np.uint32)
        ne = C.c_int64()
        st = VisStats()
        _check(lib().visacd_compute_intersection_matrix(
            self._h, _ptr(v), n, _ptr(t), len(t), _ptr(m), _ptr(cv), len(cv), _ptr(ct), len(ct),
            _ptr(out), cap, C.byref(ne), C.byref(st)), "compute_intersection_matrix")
        return out[: ne.value].copy(), st.as_dict()

    def fp32_peak_tflops(self) -> float:
        t = C.c_double()
        _check(lib().visacd_measure_fp32_peak(self._h, C.byref(t)), "measure_fp32_peak")
        return t.value

    def tex_peak_gfetch(self) -> tuple[float, float]:
        """Texture fetch rate (G fetches/s): (coherent, divergent)."""
        c, d = C.c_double(), C.c_double()
        _check(lib().visacd_measure_tex_peak(self._h, C.byref(c), C.byref(d)), "measure_tex_peak")
        return c.value, d.value

    # ---- clipping ----------------------------------------------------------
    def clip(self, verts, tris, plane):
        """GPU clip without the cap: dict with pos/neg triangles (part-local),
        1-based maps, border points and border edges."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64)).reshape(-1, 3)
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.int32)).reshape(-1, 3)
        pl = np.ascontiguousarray(np.asarray(plane, dtype=np.float64)).reshape(4)
        r = ClipResult()
        _check(lib().visacd_clip(self._h, _ptr(v), len(v), _ptr(t), len(t), _ptr(pl), C.byref(r)),
               "visacd_clip")
        out = {f: getattr(r, f) for f, _ in ClipResult._fields_}
        pt = np.zeros((r.n_pos, 3), np.int32)
        nt_ = np.zeros((r.n_neg, 3), np.int32)
        m1 = np.zeros(len(v), np.int32)
        m2 = np.zeros(len(v), np.int32)
        b = np.zeros((r.n_border, 3))
        be = np.zeros((r.n_border_edges, 2), np.int32)
        _check(lib().visacd_clip_fetch(self._h, _ptr(pt), _ptr(nt_), _ptr(m1), _ptr(m2), _ptr(b), _ptr(be)),
               "visacd_clip_fetch")
        out.update(pos_tris=pt, neg_tris=nt_, pos_map=m1, neg_map=m2, border=b, border_edges=be)
        return out

    # ---- SDF remesh --------------------------------------------------------
    def sdf_remesh(self, verts, tris, scale: float, level: float):
        """Iso-surface at `level` outside the mesh (voxel 1/scale): (verts, tris)."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64)).reshape(-1, 3)
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.int32)).reshape(-1, 3)
        nv, nt = C.c_int32(), C.c_int32()
        _check(lib().visacd_sdf_remesh(self._h, _ptr(v), len(v), _ptr(t), len(t), float(scale), float(level),
                                       C.byref(nv), C.byref(nt)), "visacd_sdf_remesh")
        ov = np.empty((nv.value, 3), np.float64)
        ot = np.empty((nt.value, 3), np.int32)
        _check(lib().visacd_sdf_fetch(self._h, _ptr(ov), _ptr(ot)), "visacd_sdf_fetch")
        return ov, ot

    # ---- concavity metric --------------------------------------------------
    def face_hausdorff(self, va, ta, xa, ida, vb, tb, xb, idb, floor: float | None = None) -> float:
        """Sampled symmetric face Hausdorff distance (visacd_face_hausdorff).
        With `floor`: exact when the distance is >= floor, else some value
        below floor (visacd_face_hausdorff_floor)."""
        f = lambda a, c: np.ascontiguousarray(np.asarray(a, dtype=np.float64)).reshape(-1, c)
        g = lambda a, c: np.ascontiguousarray(np.asarray(a, dtype=np.int32)).reshape(-1, c)
        va, xa, vb, xb = f(va, 3), f(xa, 3), f(vb, 3), f(xb, 3)
        ta, tb, ida, idb = g(ta, 3), g(tb, 3), g(ida, 1), g(idb, 1)
        out = C.c_double()
        if floor is None:
            _check(lib().visacd_face_hausdorff(self._h, _ptr(va), len(va), _ptr(ta), len(ta), _ptr(xa), _ptr(ida),
                                               len(xa), _ptr(vb), len(vb), _ptr(tb), len(tb), _ptr(xb), _ptr(idb),
                                               len(xb), C.byref(out)), "visacd_face_hausdorff")
        else:
            _check(lib().visacd_face_hausdorff_floor(self._h, _ptr(va), len(va), _ptr(ta), len(ta), _ptr(xa),
                                                     _ptr(ida), len(xa), _ptr(vb), len(vb), _ptr(tb), len(tb),
                                                     _ptr(xb), _ptr(idb), len(xb), float(floor), C.byref(out)),
                   "visacd_face_hausdorff_floor")
        return out.value

    def face_hausdorff_batch(self, jobs, lower=None, floor: float = 0.0, independent: bool = True):
        """visacd_face_hausdorff_batch over jobs = [(va, ta, xa, ida, vb, tb, xb, idb), ...];
        returns one value per job."""
        f = lambda a, c: np.ascontiguousarray(np.asarray(a, dtype=np.float64)).reshape(-1, c)
        g = lambda a, c: np.ascontiguousarray(np.asarray(a, dtype=np.int32)).reshape(-1, c)
        vs, ts, xs, ids = [], [], [], []
        for va, ta, xa, ida, vb, tb, xb, idb in jobs:
            vs += [f(va, 3), f(vb, 3)]
            ts += [g(ta, 3), g(tb, 3)]
            xs += [f(xa, 3), f(xb, 3)]
            ids += [g(ida, 1).reshape(-1), g(idb, 1).reshape(-1)]
        cum = lambda arrs: np.concatenate([[0], np.cumsum([len(a) for a in arrs])]).astype(np.int64)
        voff, toff, soff = cum(vs), cum(ts), cum(xs)
        cat = lambda arrs, shape, dt: (np.ascontiguousarray(np.concatenate(arrs)) if arrs
                                       else np.zeros(shape, dt))
        V = cat(vs, (0, 3), np.float64)
        T = cat(ts, (0, 3), np.int32)
        X = cat(xs, (0, 3), np.float64)
        I = cat(ids, (0,), np.int32)
        low = None if lower is None else np.ascontiguousarray(np.asarray(lower, dtype=np.float64))
        out = np.zeros(len(jobs), dtype=np.float64)
        _check(lib().visacd_face_hausdorff_batch(self._h, len(jobs), _ptr(V), _ptr(voff), _ptr(T), _ptr(toff),
                                                 _ptr(X), _ptr(I), _ptr(soff), _ptr(low), float(floor),
                                                 int(bool(independent)), _ptr(out)),
               "visacd_face_hausdorff_batch")
        return out

    def segment_triangle_tests(self, seg, tri):
        """Independent segment-triangle decisions: (hit bool[S], FP64 re-checks)."""
        sg = np.ascontiguousarray(np.asarray(seg, dtype=np.float32)).reshape(-1, 6)
        tr = np.ascontiguousarray(np.asarray(tri, dtype=np.float32)).reshape(-1, 9)
        out = np.zeros(len(sg), np.uint8)
        n64 = C.c_int64()
        _check(lib().visacd_segment_triangle_tests(self._h, _ptr(sg), _ptr(tr), len(sg), _ptr(out), C.byref(n64)),
               "visacd_segment_triangle_tests")
        return out.astype(bool), n64.value

    # ---- device sort -------------------------------------------------------
    def radix_sort_pairs(self, keys, vals, key_bits: int):
        """Stable sort of (keys, vals) by key on the device; returns sorted copies."""
        k = np.ascontiguousarray(np.asarray(keys, dtype=np.uint64)).copy()
        v = np.ascontiguousarray(np.asarray(vals, dtype=np.uint32)).copy()
        _check(lib().visacd_radix_sort_pairs(self._h, _ptr(k), _ptr(v), len(k), int(key_bits)),
               "visacd_radix_sort_pairs")
        return k, v

    # ---- convex hulls ------------------------------------------------------
    def convex_hulls(self, point_sets, fix_normals: bool = True):
        """Hull triangles (k x 3 int32, indices into its own points) of every
        point array in point_sets, in one launch."""
        vs = [np.ascontiguousarray(np.asarray(p, dtype=np.float64)).reshape(-1, 3) for p in point_sets]
        off = np.zeros(len(vs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(v) for v in vs])
        allv = np.ascontiguousarray(np.concatenate(vs) if vs else np.zeros((0, 3)))
        tris = np.empty(6 * int(off[-1]), dtype=np.int32)
        counts = np.zeros(len(vs), dtype=np.int32)
        _check(lib().visacd_convex_hulls(self._h, _ptr(allv), _ptr(off), len(vs), int(bool(fix_normals)),
                                         _ptr(tris), _ptr(counts)), "visacd_convex_hulls")
        return [tris[6 * off[k]:6 * off[k] + 3 * counts[k]].reshape(-1, 3).copy() for k in range(len(vs))]

    # ---- hull merging ------------------------------------------------------
    def hull_distances(self, hulls, pairs, cutoff: float = np.finfo(np.float64).max):
        """Minimum vertex distance of each (a, b) in pairs between the vertex
        arrays hulls[a] and hulls[b]."""
        vs = [np.ascontiguousarray(np.asarray(h, dtype=np.float64)).reshape(-1, 3) for h in hulls]
        off = np.zeros(len(vs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(v) for v in vs])
        allv = np.ascontiguousarray(np.concatenate(vs) if vs else np.zeros((0, 3)))
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32)).reshape(-1, 2)
        out = np.empty(len(pr), dtype=np.float64)
        _check(lib().visacd_hull_distances(self._h, _ptr(allv), _ptr(off), len(vs), _ptr(pr), len(pr),
                                           float(cutoff), _ptr(out)), "visacd_hull_distances")
        return out

    # ---- scoring -----------------------------------------------------------
    def score_planes(self, planes, points, edges):
        pl = _f32(planes, 4)
        pt = _f32(points, 3)
        ed = _u32(edges, 2)
        scores = np.zeros(len(pl), dtype=np.float64)
        st = ScoreStats()
        _check(lib().visacd_score_planes(self._h, _ptr(pl), len(pl), _ptr(pt), len(pt), _ptr(ed),
                                         len(ed), 0, _ptr(scores), C.byref(st)), "visacd_score_planes")
        return scores, st.as_dict()

    def candidate_planes(self, verts, edges, draws, num_planes: int):
        """Candidate planes from the given edge draws: (planes n x 4 float64,
        draws used)."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 3))
        ed = _u32(edges, 2)
        dr = np.ascontiguousarray(np.asarray(draws, dtype=np.int32))
        out = np.zeros((max(num_planes, 1), 4), np.float64)
        got, used = C.c_int32(), C.c_int32()
        _check(lib().visacd_candidate_planes(self._h, _ptr(v), len(v), _ptr(ed), len(ed), _ptr(dr), len(dr),
                                             num_planes, _ptr(out), C.byref(got), C.byref(used)),
               "visacd_candidate_planes")
        return out[: got.value], used.value

    def split_search(self, verts, edges, draws, num_planes: int, flat_planes=None, flat_k: float = 2.0):
        """The split search: (best plane 4 float64, info dict)."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 3))
        ed = _u32(edges, 2)
        dr = np.ascontiguousarray(np.asarray(draws, dtype=np.int32))
        fl = None if flat_planes is None or len(flat_planes) == 0 else \
            np.ascontiguousarray(np.asarray(flat_planes, dtype=np.float64).reshape(-1, 4))
        best = np.zeros(4, np.float64)
        info = SplitInfo()
        _check(lib().visacd_split_search(self._h, _ptr(v), len(v), _ptr(ed), len(ed), _ptr(dr), len(dr),
                                         num_planes, _ptr(fl), 0 if fl is None else len(fl), flat_k,
                                         _ptr(best), C.byref(info)), "visacd_split_search")
        return best, info.as_dict()

    def score_planes_device(self, d_planes: int, P: int, d_points: int, N: int, d_edges: int,
                            E: int, d_scores: int, stats: bool = False):
        st = ScoreStats()
        _check(lib().visacd_score_planes(self._h, C.c_void_p(d_planes), P, C.c_void_p(d_points), N,
                                         C.c_void_p(d_edges), E, 1, C.c_void_p(d_scores),
                                         C.byref(st) if stats else None), "visacd_score_planes")
        return st.as_dict() if stats else None


class Batch:
    """visacd_batch: many parts' visibility + scoring in one launch sequence."""

    def __init__(self, ctx: "Context", parts):
        """parts: list of (points (n,3), Bvh self, Bvh cage, planes (P,4))."""
        self._ctx = ctx
        self._keep = []
        n = len(parts)
        pts_ptrs = (C.c_void_p * n)()
        sb = (C.c_void_p * n)()
        cb = (C.c_void_p * n)()
        pl_ptrs = (C.c_void_p * n)()
        npts = np.zeros(n, np.int32)
        npl = np.zeros(n, np.int32)
        for k, (pts, s, c, pl) in enumerate(parts):
            p = _f32(pts, 3)
            q = _f32(pl, 4)
            self._keep += [p, q, s, c]
            pts_ptrs[k] = p.ctypes.data
            pl_ptrs[k] = q.ctypes.data
            sb[k] = s.handle.value
            cb[k] = c.handle.value
            npts[k] = len(p)
            npl[k] = len(q)
        self.n_planes = npl
        self._h = C.c_void_p()
        _check(lib().visacd_batch_create(ctx.handle, n, pts_ptrs, _ptr(npts), sb, cb, pl_ptrs, _ptr(npl), 0,
                                         C.byref(self._h)), "visacd_batch_create")
        self.n_parts = n

    def run(self, use_graph: bool = True) -> None:
        _check(lib().visacd_batch_run(self._ctx.handle, self._h, int(use_graph)), "visacd_batch_run")

    def info(self):
        a, b = C.c_int64(), C.c_int64()
        _check(lib().visacd_batch_info(self._h, C.byref(a), C.byref(b)), "batch_info")
        return a.value, b.value

    def results(self, with_edges: bool = False):
        ne = np.zeros(self.n_parts, np.int64)
        scores = np.zeros(int(self.n_planes.sum()), np.float64)
        am = np.zeros(self.n_parts, np.int32)
        _check(lib().visacd_batch_results(self._ctx.handle, self._h, _ptr(ne), None, None, None, 0),
               "batch_results")
        edges = np.zeros((int(ne.sum()), 2), np.uint32) if with_edges else None
        _check(lib().visacd_batch_results(self._ctx.handle, self._h, _ptr(ne), _ptr(scores), _ptr(am),
                                          _ptr(edges) if with_edges else None, int(ne.sum())),
               "batch_results")
        return ne, scores, am, edges

    def close(self):
        if self._h:
            lib().visacd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Bvh:
    def __init__(self, ctx: Context, verts, tris, device_ptrs: bool = False, nv: int = 0, nt: int = 0):
        self._h = C.c_void_p()
        self._ctx = ctx
        if device_ptrs:
            _check(lib().visacd_bvh_build(ctx.handle, C.c_void_p(verts), nv, C.c_void_p(tris), nt, 1,
                                          C.byref(self._h)), "visacd_bvh_build")
        else:
            v = _f32(verts, 3)
            t = _u32(tris, 3)
            _check(lib().visacd_bvh_build(ctx.handle, _ptr(v), len(v), _ptr(t), len(t), 0,
                                          C.byref(self._h)), "visacd_bvh_build")

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> tuple[int, int]:
        nt, depth = C.c_int32(), C.c_int32()
        _check(lib().visacd_bvh_info(self._h, C.byref(nt), C.byref(depth)), "bvh_info")
        return nt.value, depth.value

    def close(self) -> None:
        if self._h:
            lib().visacd_bvh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def classify_and_rate_planes(planes, points, edges) -> np.ndarray:
    """The reference-signature entry point (float scores, default context)."""
    pl = _f32(planes, 4)
    pt = _f32(points, 3)
    ed = _u32(edges, 2)
    out = np.zeros(len(pl), dtype=np.float32)
    lib().classify_and_rate_planes(_ptr(pl), _ptr(pt), _ptr(ed), _ptr(out), len(pl), len(pt), len(ed))
    return out


class PlaneProposer:
    """The learned plane proposer (visacd_lp_*): BF16 tensor-core network over
    2048 sampled visibility edges -> 16 planes. `params` None = seeded init."""

    def __init__(self, ctx: Context, params=None, seed: int = 0):
        self._ctx = ctx
        self._h = C.c_void_p()
        self.n_params = int(lib().visacd_lp_param_count())
        p = None
        if params is not None:
            p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(-1))
            if p.size != self.n_params:
                raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        _check(lib().visacd_lp_create(ctx.handle, _ptr(p), seed, C.byref(self._h)), "visacd_lp_create")

    def set_tcgen05(self, enable: bool) -> None:
        """Forward per-edge layers on tcgen05 (tensor memory) instead of mma.sync."""
        _check(lib().visacd_lp_set_tcgen05(self._h, int(bool(enable))), "visacd_lp_set_tcgen05")

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        _check(lib().visacd_lp_get_params(self._h, _ptr(out)), "visacd_lp_get_params")
        return out

    def features(self, points, edges, center, scale) -> np.ndarray:
        pt = _f32(points, 3)
        ed = _u32(edges, 2)
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float32).reshape(3))
        out = np.empty((LP_POINTS, LP_FEATURES), dtype=np.float32)
        _check(lib().visacd_lp_features(self._h, _ptr(pt), len(pt), _ptr(ed), len(ed), _ptr(c),
                                        float(scale), _ptr(out)), "visacd_lp_features")
        return out

    def forward(self, feats) -> np.ndarray:
        f = np.ascontiguousarray(np.asarray(feats, dtype=np.float32).reshape(-1, LP_POINTS, LP_FEATURES))
        out = np.empty((len(f), LP_PLANES, 4), dtype=np.float32)
        _check(lib().visacd_lp_forward(self._h, _ptr(f), len(f), _ptr(out)), "visacd_lp_forward")
        return out

    def propose(self, points, edges, center, scale) -> np.ndarray:
        pt = _f32(points, 3)
        ed = _u32(edges, 2)
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float32).reshape(3))
        out = np.empty((LP_PLANES, 4), dtype=np.float64)
        _check(lib().visacd_lp_propose(self._h, _ptr(pt), len(pt), _ptr(ed), len(ed), _ptr(c),
                                       float(scale), _ptr(out)), "visacd_lp_propose")
        return out

    def split_search(self, verts, edges, center, scale: float, half: float, refine_k: int, draws,
                     probe_planes: int, flat_planes=None, flat_k: float = 2.0, tolerance: float = 0.01):
        """The learned split search of one part in one call
        (visacd_learned_split_search): (best plane 4 float64, info dict)."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 3))
        ed = _u32(edges, 2)
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float32).reshape(3))
        dr = np.ascontiguousarray(np.asarray(draws, dtype=np.int32))
        fl = None if flat_planes is None or len(flat_planes) == 0 else \
            np.ascontiguousarray(np.asarray(flat_planes, dtype=np.float64).reshape(-1, 4))
        best = np.zeros(4, np.float64)
        info = LearnedSplitInfo()
        _check(lib().visacd_learned_split_search(self._h, _ptr(v), len(v), _ptr(ed), len(ed), _ptr(c),
                                                 float(scale), float(half), int(refine_k), _ptr(dr), len(dr),
                                                 int(probe_planes), _ptr(fl), 0 if fl is None else len(fl),
                                                 float(flat_k), float(tolerance), _ptr(best),
                                                 C.byref(info)), "visacd_learned_split_search")
        return best, info.as_dict()

    @staticmethod
    def _batch(feats, labels, weights):
        f = np.ascontiguousarray(np.asarray(feats, dtype=np.float32).reshape(-1, LP_POINTS, LP_FEATURES))
        lab = np.ascontiguousarray(np.asarray(labels, dtype=np.float32).reshape(len(f), -1, 4))
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float32).reshape(len(f), lab.shape[1]))
        return f, lab, w

    def grads(self, feats, labels, weights):
        f, lab, w = self._batch(feats, labels, weights)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        _check(lib().visacd_lp_grads(self._h, _ptr(f), _ptr(lab), _ptr(w), len(f), lab.shape[1], _ptr(g),
                                     C.byref(loss)), "visacd_lp_grads")
        return float(loss.value), g

    def train_step(self, feats, labels, weights, lr: float) -> float:
        f, lab, w = self._batch(feats, labels, weights)
        loss = C.c_float()
        _check(lib().visacd_lp_train_step(self._h, _ptr(f), _ptr(lab), _ptr(w), len(f), lab.shape[1],
                                          float(lr), C.byref(loss)), "visacd_lp_train_step")
        return float(loss.value)

    def close(self) -> None:
        if self._h:
            lib().visacd_lp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
