"""Benchmark of the visibility-edge hot path on one GB300.

Workload (the large concave blob): icosphere subdivision 5 (10242 vertices,
20480 triangles) displaced by 8 seeded Gaussian bumps, all 52,444,161 vertex
pairs segment-tested against the part and a 0.03 offset cage, then 2500
candidate planes scored against the resulting visibility edges.

One step = BVH builds (part + cage) + visibility over every pair + edge
compaction + scoring of the candidate planes + argmax — the GPU hot path of one
decomposition split (reference: compute_intersection_matrix,
lib/src/intersections.cpp:327; classify_and_rate_planes,
lib/cuda/plane_intersections.cu:71).

value: pairs/s with inputs resident in device memory.
e2e:   the same through the C ABI with host buffers (copies inside the timing).
Prints one JSON line (rank 0). --impl reference times the CPU restatement of
the same path (FP64, OpenMP, all host threads) on a bounded sample of rows.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "decomps/sec batched+learned vs plain on 1 GB300 at <=1% concavity gap; pairs/s"
UNIT = "pairs/s"
N_PLANES = 2500
L2_BYTES = 129 * 1024 * 1024
# Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) that
# ncu measured for a kernel on a workload, one "workload kernel bytes" line
# each; written from the ncu capture whose command the matching summary in
# profiles/ gives.
TRAFFIC_FILE = ROOT / "profiles" / "dram_traffic.txt"


THROUGHPUT_FILE = ROOT / "profiles" / "visibility_throughput.txt"


def measured_throughput(workload_name: str, kernel: str) -> dict:
    """ncu's L1 / L2 throughput, issue activity and occupancy of a kernel on a
    workload ("workload kernel l1 l2 issue occupancy" lines, percent)."""
    if not THROUGHPUT_FILE.exists():
        return {}
    for line in THROUGHPUT_FILE.read_text().splitlines():
        f = line.split()
        if len(f) == 6 and not line.startswith("#") and f[0] == workload_name and f[1] == kernel:
            return {"l1_pct": float(f[2]), "l2_pct": float(f[3]), "issue_active_pct": float(f[4]),
                    "achieved_occupancy_pct": float(f[5]),
                    "survey_roofline_max_l1_l2_pct": max(float(f[2]), float(f[3])),
                    "source": f"ncu --set full of this launch (profiles/{kernel}_blob_s5_full.md)"}
    return {}


def measured_traffic(workload_name: str, kernel: str):
    if not TRAFFIC_FILE.exists():
        return None
    for line in TRAFFIC_FILE.read_text().splitlines():
        f = line.split()
        if len(f) == 3 and not line.startswith("#") and f[0] == workload_name and f[1] == kernel:
            return int(f[2])
    return None


WORKLOADS = {"blob_s5": 5, "blob_s4": 4, "blob_s3": 3}


def workload(seed: int = 2026, name: str = "blob_s5"):
    from visacd_gb300 import meshgen

    v, t = meshgen.displaced_blob(WORKLOADS[name], seed=seed)
    cv, ct = meshgen.offset_cage(v, t, 0.03)
    return v, t, cv, ct


def bisector_planes(v: np.ndarray, edges: np.ndarray, n: int, seed: int) -> np.ndarray:
    """Perpendicular-bisector planes of randomly drawn edges (setup only)."""
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, len(edges), size=n)
    p1, p2 = v[edges[idx, 0]], v[edges[idx, 1]]
    nrm = p2 - p1
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = -(nrm * (p1 + p2) * 0.5).sum(1)
    return np.concatenate([nrm, d[:, None]], 1).astype(np.float32)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.rows: list[list[str]] = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 3 + k and r[3 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args) -> dict:
    import torch

    from visacd_gb300 import _native, build

    world, rank, local = dist_setup()
    build.build_gpu()
    # A dedicated stream: the library launches on it and the CUDA events below
    # are recorded on it (torch's default stream would have handle 0, which the
    # library treats as "make your own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = _native.Context(local, stream.cuda_stream)
    v, t, cv, ct = workload(name=args.workload)
    n = len(v)
    n_pairs = n * (n - 1) // 2
    dev = torch.device("cuda", local)
    d_v = torch.from_numpy(v.astype(np.float32)).to(dev)
    d_t = torch.from_numpy(t.astype(np.int32)).to(dev)
    d_cv = torch.from_numpy(cv.astype(np.float32)).to(dev)
    d_ct = torch.from_numpy(ct.astype(np.int32)).to(dev)
    lib = _native.lib()
    import ctypes as C

    # Setup: one pass to get edges for the candidate planes.
    sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
    edges0, st0 = ctx.visibility(v, sb, cb)
    walk_cleared, walk_reads = ctx.vis_trace_counts()
    bvh_depth = (sb.info()[1], cb.info()[1])
    # Autotune the visibility launch shape for this shape class (setup, untimed).
    tuned_variant, tuned_ms = ctx.autotune_visibility(v, sb, cb)
    sb.close()
    cb.close()
    planes = bisector_planes(v, edges0, N_PLANES, seed=1)
    # Autotune the scoring kernel's planes per thread for this shape class.
    score_k, score_k_ms = ctx.autotune_scoring(planes, v, edges0)
    d_planes = torch.from_numpy(planes).to(dev)
    d_scores = torch.empty(N_PLANES, dtype=torch.float64, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def step_device():
        h_s, h_c = C.c_void_p(), C.c_void_p()
        _native._check(lib.visacd_bvh_build(ctx.handle, C.c_void_p(d_v.data_ptr()), n,
                                            C.c_void_p(d_t.data_ptr()), len(t), 1, C.byref(h_s)), "bvh")
        _native._check(lib.visacd_bvh_build(ctx.handle, C.c_void_p(d_cv.data_ptr()), len(cv),
                                            C.c_void_p(d_ct.data_ptr()), len(ct), 1, C.byref(h_c)), "bvh")
        ne = C.c_int64()
        _native._check(lib.visacd_visibility(ctx.handle, C.c_void_p(d_v.data_ptr()), n, None, 1, h_s,
                                             h_c, C.byref(ne), None), "visibility")
        d_e, ne2 = C.c_void_p(), C.c_int64()
        lib.visacd_visibility_edges_device(ctx.handle, C.byref(d_e), C.byref(ne2))
        _native._check(lib.visacd_score_planes(ctx.handle, C.c_void_p(d_planes.data_ptr()), N_PLANES,
                                               C.c_void_p(d_v.data_ptr()), n, d_e, ne2.value, 1,
                                               C.c_void_p(d_scores.data_ptr()), None), "score")
        lib.visacd_bvh_destroy(h_s)
        lib.visacd_bvh_destroy(h_c)
        return ne.value

    # e2e: the C ABI with host buffers (pinned inputs copied in, edges + scores out).
    h_v = torch.from_numpy(v.astype(np.float32)).pin_memory().numpy()
    h_t = torch.from_numpy(t.astype(np.int32)).pin_memory().numpy().view(np.uint32)
    h_cv = torch.from_numpy(cv.astype(np.float32)).pin_memory().numpy()
    h_ct = torch.from_numpy(ct.astype(np.int32)).pin_memory().numpy().view(np.uint32)
    h_planes = torch.from_numpy(planes).pin_memory().numpy()
    cap = len(edges0) + 1024
    h_edges = torch.empty((cap, 2), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    h_scores = torch.empty(N_PLANES, dtype=torch.float64).pin_memory().numpy()
    bytes_in = h_v.nbytes + h_t.nbytes + h_cv.nbytes + h_ct.nbytes + h_planes.nbytes + h_v.nbytes

    def step_e2e():
        ne = C.c_int64()
        _native._check(lib.visacd_compute_intersection_matrix(
            ctx.handle, h_v.ctypes.data, n, h_t.ctypes.data, len(t), None, h_cv.ctypes.data, len(cv),
            h_ct.ctypes.data, len(ct), h_edges.ctypes.data, cap, C.byref(ne), None), "cim")
        _native._check(lib.visacd_score_planes(ctx.handle, h_planes.ctypes.data, N_PLANES,
                                               h_v.ctypes.data, n, h_edges.ctypes.data, ne.value, 0,
                                               h_scores.ctypes.data, None), "score")
        return ne.value

    for _ in range(args.warmup):
        step_device()
        step_e2e()
    torch.cuda.synchronize()
    # An asynchronous scoring call reports lost work as NaN scores.
    assert not torch.isnan(d_scores).any().item(), "scoring reported lost work (NaN scores)"

    # value: device-resident, CUDA events per step on the launching stream,
    # L2 flushed (untimed) before each step; the library's per-kernel event
    # timing is off here and on in a second pass of the same steps below.
    ctx.set_timing(False)
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            ne = step_device()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = sum(a.elapsed_time(b) for a, b in ev)
    launches = ctx.launches - launches0
    # Per-kernel times (CUDA events around every launch) over the same steps.
    ctx.set_timing(True)
    ctx.reset_times()
    for k in range(args.steps):
        flush.zero_()
        step_device()
    torch.cuda.synchronize()
    ktimes = ctx.kernel_times()
    ctx.set_timing(False)
    ms = max_over_ranks(ms, world)
    ms_step = ms / args.steps
    value = world * n_pairs / (ms_step / 1e3)
    assert not torch.isnan(d_scores).any().item(), "scoring reported lost work (NaN scores)"

    # e2e (host buffers, copies inside the timing).
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ne_e = step_e2e()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    e2e = {"value": world * n_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(bytes_in + ne_e * 8),
           "d2h_bytes_per_step": int(ne_e * 8 + N_PLANES * 8), "ms_per_step": e2e_s * 1e3}

    # Rooflines. The hot kernels work out of L1/L2 (the grid, the BVHs and
    # the edge records are L2-resident), so the denominator of their work
    # models is this GPU's measured FP32 FMA rate (MEASURED_PEAKS.json lists
    # HBM copy and bf16 GEMM only); ncu's L1 / L2 throughput and issue
    # activity of each (profiles/) say what binds them.
    walk_ms, walk_n = ktimes.get("vis_walk", (0.0, 0))
    walk_launch_s = walk_ms / max(walk_n, 1) / 1e3
    # Free-space walk per launch: one point-sampled texture fetch of the bound
    # grid per step (grid reads, counted by the kernel), and around it the
    # point (3 FMA), its cell coordinates (3 sub + 3 mul) and the step (sub,
    # mul, add): 15 FLOP. The texture fetch rate binds it (ncu: L1/TEX is its
    # busiest unit); the FP32 figure is kept beside it.
    walk_fetch = walk_reads / walk_launch_s / 1e9 if walk_ms else None
    walk_flop = 15.0 * walk_reads
    walk_achieved = walk_flop / walk_launch_s / 1e12 if walk_ms else None
    vis_ms, vis_n = ktimes.get("visibility", (0.0, 0))
    sc_ms, sc_n = ktimes.get("score_planes", (0.0, 0))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    fp32_peak = ctx.fp32_peak_tflops()
    tex_coherent, tex_divergent = ctx.tex_peak_gfetch()
    vis_launch_s = vis_ms / max(vis_n, 1) / 1e3
    # Traversal arithmetic per launch: each packet node visit runs 2 packed
    # slab tests (12 FLOP each) on 32 lanes; each triangle test ~60 FLOP.
    vis_flop = st0["node_visits"] * 32 * 24 + st0["tri_tests"] * 60
    vis_achieved = vis_flop / vis_launch_s / 1e12 if vis_ms else None
    sc_launch_s = sc_ms / max(sc_n, 1) / 1e3
    sc_flop = 12.0 * N_PLANES * ne
    sc_achieved = sc_flop / sc_launch_s / 1e12 if sc_ms else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64recheck", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD_TEXT if args.workload == "blob_s5" else args.workload,
                   "pairs": n_pairs, "edges": int(ne), "planes": N_PLANES,
                   "name": args.workload, "bvh_depth": bvh_depth,
                   "visibility_counters": st0,
                   "vis_variant": tuned_variant, "vis_variant_ms": [round(x, 3) for x in tuned_ms],
                   "score_planes_per_thread": score_k,
                   "score_k_ms": {str(k): round(x, 4) for k, x in zip((1, 2, 4, 8), score_k_ms)},
                   "l2": "flushed before each timed step (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "kernels_ms_per_step": {k: v[0] / args.steps for k, v in sorted(ktimes.items(), key=lambda kv: -kv[1][0])},
        "kernel_launches": {k: v[1] for k, v in ktimes.items()},
        "roofline": {"kernel": "visibility_walk_kernel", "bound": "texture-fetch",
                     "achieved": walk_fetch, "peak": tex_coherent, "unit": "Gfetch/s",
                     "frac": walk_fetch / tex_coherent if walk_fetch else None,
                     "frac_of_divergent_fetch_rate": walk_fetch / tex_divergent if walk_fetch else None,
                     "peak_divergent": tex_divergent,
                     "fp32_model": {"achieved": walk_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                                    "frac": walk_achieved / fp32_peak if walk_achieved else None,
                                    "work_model": "grid reads x 15 FLOP (point, cell coordinates, step)"},
                     "traffic": measured_traffic(args.workload, "visibility_walk_kernel"),
                     "ncu": measured_throughput(args.workload, "visibility_walk_kernel"),
                     "ms_per_launch": walk_ms / max(walk_n, 1),
                     "segments_cleared": int(walk_cleared), "grid_reads": int(walk_reads),
                     "work_model": "grid reads (one point-sampled tex3D<float> fetch each) per launch",
                     "peak_source": "measured in-process: tex3D<float> point fetches from a cache-resident "
                                    "32^3 texture, coherent 8x4 texel blocks per warp (peak) and one line per "
                                    "lane (peak_divergent); HBM peak of measured "
                                    f"{peaks.get('hbm_gbs')} GB/s not binding (L2-resident grid)"},
        "roofline_traversal": {"kernel": "visibility_kernel", "bound": "fp32-issue",
                               "achieved": vis_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                               "frac": vis_achieved / fp32_peak if vis_achieved else None,
                               "traffic": measured_traffic(args.workload, "visibility_kernel"),
                               "ncu": measured_throughput(args.workload, "visibility_kernel"),
                               "ms_per_launch": vis_ms / max(vis_n, 1),
                               "pairs_per_s": n_pairs / (vis_launch_s + walk_launch_s) if vis_ms else None,
                               "work_model": "packet node visits x 32 lanes x 2 boxes x 12 FLOP + "
                                             "triangle tests x 60 FLOP (the pairs the walk left)"},
        "roofline_scoring": {"kernel": "score_planes_kernel", "bound": "fp32-issue",
                             "achieved": sc_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": sc_achieved / fp32_peak if sc_achieved else None,
                             "ms_per_launch": sc_ms / max(sc_n, 1),
                             "plane_edge_pairs_per_s": N_PLANES * ne / sc_launch_s if sc_ms else None,
                             "work_model": "12 FLOP per (plane, edge) pair"},
        "clocks": clk.summary(),
        "peaks_source": "MEASURED_PEAKS.json" if peaks else "fallback",
    }
    out["_edges"] = edges0
    out["_planes"] = planes
    return out, rank


def cpu_step(v, t, cv, ct, planes, rows):
    """The step on the host cores: the FP64 oracle's visibility over the listed
    pair rows (BVH traversal, all threads) and its exact scoring of the planes
    against the edges found. Returns (pairs, seconds, per-pair result bytes)."""
    import oracle

    t0 = time.perf_counter()
    bits, st = oracle.visibility_rows(v, t, cv, ct, rows)
    edges = oracle.pairs_from_linear(np.nonzero(bits & 1)[0], len(v))
    oracle.score_planes(planes, v.astype(np.float32), edges)
    return st["pairs"], time.perf_counter() - t0, bits


def grazing_check(v, bits, edges_gpu) -> dict:
    """GPU edges against the FP64 oracle's per-pair results on every pair."""
    import oracle

    n = len(v)
    gpu = np.zeros(n * (n - 1) // 2, dtype=bool)
    gpu[oracle.linear_from_pairs(edges_gpu, n)] = True
    diff = gpu != (bits & 1).astype(bool)
    graze = (bits & 2).astype(bool)
    g = int(graze.sum())
    return {"oracle_grazing_pairs": g, "grazing_frac": g / len(bits),
            "differing_pairs": int(diff.sum()),
            "differing_outside_grazing_band": int((diff & ~graze).sum())}


def run_hulls(args) -> dict:
    """Convex hulls of a batch of clipped parts (64 displaced blobs, s3 and
    s4, each cut by two seeded planes with the host clip: planar caps, as the
    decomposition's parts have): visacd_convex_hulls in one call against the
    host QuickHull on one core, wall clock with host buffers, and whether
    every GPU hull equals the host's triangle for triangle."""
    from visacd_gb300 import _native as N, build, meshgen

    build.build_host()
    from visacd_gb300 import visacd as V

    rng = np.random.default_rng(23)
    parts = []

    def plane():
        nrm = rng.normal(size=3)
        return [*(nrm / np.linalg.norm(nrm)), rng.uniform(-0.3, 0.3)]

    for s in range(64):
        v, t = meshgen.displaced_blob(3 + (s % 2), seed=40 + s)
        halves, _, _ = V._clip(v, t, plane())
        for h in halves:
            quarters, _, _ = V._clip(np.asarray(h["vertices"]), np.asarray(h["triangles"]), plane())
            parts += [np.asarray(q["vertices"]) for q in quarters]
    ctx = N.Context(0)
    try:
        ctx.convex_hulls(parts[:4])

        def med(f, r):
            ts = []
            for _ in range(r):
                t0 = time.perf_counter()
                f()
                ts.append(time.perf_counter() - t0)
            return 1e3 * float(np.median(ts))

        gpu = ctx.convex_hulls(parts)
        equal = all(np.array_equal(g, np.asarray(V._convex_hull(p)["triangles"], np.int32).reshape(-1, 3))
                    for p, g in zip(parts, gpu))
        out = {"parts": len(parts), "points": int(sum(len(p) for p in parts)),
               "gpu_ms_one_call": med(lambda: ctx.convex_hulls(parts), 3),
               "host_ms_one_core": med(lambda: [V._convex_hull(p) for p in parts], 3),
               "gpu_ms_two_parts": med(lambda: ctx.convex_hulls(parts[:2]), 5),
               "host_ms_two_parts_one_core": med(lambda: [V._convex_hull(p) for p in parts[:2]], 5),
               "equal_to_host": bool(equal)}
    finally:
        ctx.close()
    return out


def run_decompositions(args) -> dict:
    """End-to-end visacd.process() on the torus (64 x 32, concavity 0.04, 32
    parts) and the s5 blob (concavity 0.02, 64 parts): decompositions/s."""
    from visacd_gb300 import build, meshgen

    build.build_host()
    import visacd
    from visacd_gb300 import visacd as V

    visacd.config.verbose = False
    out = {}
    cases = {"torus_64x32": (meshgen.torus(R=1.0, r=0.35, nu=64, nv=32, perturb=0.02, seed=42), 0.04, 32),
             "blob_s5": (meshgen.displaced_blob(5, seed=2026), 0.02, 64)}
    for name, ((v, t), conc, nparts) in cases.items():
        m = visacd.Mesh()
        m.vertices = visacd.VecArray3d(v.tolist())
        m.triangles = visacd.make_vecarray3i(t.astype(np.int32))
        times = []
        for rep in range(2):
            visacd.set_seed(42)
            t0 = time.perf_counter()
            r = visacd.process(m, conc, nparts)
            times.append(time.perf_counter() - t0)
        st = V._stage_times()
        out[name] = {"decomps_per_s": 1.0 / times[-1], "s_per_decomp": times[-1], "parts": r.num_parts,
                     "concavity": r.concavity,
                     "stages_ms": {k: round(v, 1) for k, v in st.items() if k.endswith("_ms")}}
    return out


def run_learned_batch(args) -> dict:
    """Decompositions/s of the batched + learned method against the plain one on
    held-out blobs (displaced icospheres, subdivision 3-4, seeds 1,000,000+,
    never seen in training), process(concavity 0.02, 64 parts):
      plain    — the reference's loop, one mesh after another, exhaustive split
                 search (set_seed(seed) per mesh);
      batched  — process_batch over all meshes (one worker thread and GPU
                 stream each), exhaustive search: bit-identical results;
      batched + learned — process_batch with the learned proposer (probe of 64
                 reference candidates, fallback to the exhaustive search).
    The concavity gap of learned vs plain is set beside the plain method's own
    seed-to-seed spread (same meshes, seed + 1000), its noise floor."""
    from visacd_gb300 import build, proposer as pp

    build.build_host()
    from visacd_gb300 import visacd as V

    V.config.verbose = False
    seeds = list(range(pp.HELDOUT_SEED0, pp.HELDOUT_SEED0 + args.c5_blobs))
    meshes = V.MeshList()
    for s in seeds:
        _, v, t, _, _ = pp.make_blob(s)
        m = V.Mesh()
        m.vertices = V.VecArray3d(v.tolist())
        m.triangles = V.make_vecarray3i(t.astype(np.int32))
        meshes.append(m)
    conc, nparts = 0.02, 64
    V.set_seed(0)
    V.process(meshes[0], conc, nparts)  # warm-up (context, kernels, allocator)

    def sequential(mode, seed_shift=0):
        V.config.plane_proposer = mode
        V._reset_counters()
        t0 = time.perf_counter()
        res = []
        for m, s in zip(meshes, seeds):
            V.set_seed(s + seed_shift)
            res.append(V.process(m, conc, nparts))
        dt = time.perf_counter() - t0
        return dt, res, V._stage_times()

    def batched(mode, seed_shift=0):
        V.config.plane_proposer = mode
        V._reset_counters()
        t0 = time.perf_counter()
        res = V.process_batch(meshes, conc, nparts, [s + seed_shift for s in seeds], args.c5_threads)
        return time.perf_counter() - t0, res, V._stage_times()

    try:
        t_plain, r_plain, st_plain = sequential("exhaustive")
        t_bx, r_bx, _ = batched("exhaustive")
        t_bl, r_bl, st_bl = batched("learned")
        _, r_alt, _ = sequential("exhaustive", 1000) if args.c5_noise else (None, None, None)
        _, _, st_l = sequential("learned") if args.c5_fallbacks else (None, None, None)
        # Seed spread: the same meshes under other engine seeds, both methods
        # (batched exhaustive results equal plain ones, so the batch runs them).
        spread = []
        for k in range(1, args.c5_seeds):
            _, ra, _ = batched("exhaustive", 1000 * k)
            _, rb, _ = batched("learned", 1000 * k)
            spread.append((np.mean([r.concavity for r in ra]), np.mean([r.concavity for r in rb]),
                           np.mean([r.num_parts for r in ra]), np.mean([r.num_parts for r in rb])))
    finally:
        V.config.plane_proposer = "exhaustive"
    n = len(seeds)
    cp = np.array([r.concavity for r in r_plain])
    cl = np.array([r.concavity for r in r_bl])
    out = {
        "workload": f"{n} held-out displaced-icosphere blobs (subdivision 3-4), process(0.02, 64)",
        "plain_decomps_per_s": n / t_plain,
        "batched_decomps_per_s": n / t_bx,
        "batched_learned_decomps_per_s": n / t_bl,
        "speedup_batched_learned_vs_plain": t_plain / t_bl,
        "speedup_batched_vs_plain": t_plain / t_bx,
        "batched_identical_to_plain": all(a.concavity == b.concavity and a.num_parts == b.num_parts
                                          for a, b in zip(r_bx, r_plain)),
        "threads": args.c5_threads or os.cpu_count(),
        "concavity_plain_mean": float(cp.mean()),
        "concavity_learned_mean": float(cl.mean()),
        "concavity_gap_of_means": float(cl.mean() / cp.mean() - 1.0),
        "parts_plain_mean": float(np.mean([r.num_parts for r in r_plain])),
        "parts_learned_mean": float(np.mean([r.num_parts for r in r_bl])),
        "stages_ms_plain_all_meshes": {k: round(v, 1) for k, v in st_plain.items()
                                       if k.startswith("conc_") or k in ("vis_ms", "score_ms", "lp_ms")},
        "stages_ms_batched_learned_thread_sum": {k: round(v, 1) if isinstance(v, float) else v
                                                 for k, v in st_bl.items()},
    }
    if spread:
        pm = [float(cp.mean())] + [float(x[0]) for x in spread]
        lm = [float(cl.mean())] + [float(x[1]) for x in spread]
        gaps = [b / a - 1.0 for a, b in zip(pm, lm)]
        out["seed_spread"] = {
            "engine_seeds": [f"seed + {1000 * k}" for k in range(args.c5_seeds)],
            "concavity_plain_mean_per_seed": pm,
            "concavity_learned_mean_per_seed": lm,
            "parts_plain_mean_per_seed": [out["parts_plain_mean"]] + [float(x[2]) for x in spread],
            "parts_learned_mean_per_seed": [out["parts_learned_mean"]] + [float(x[3]) for x in spread],
            "gap_per_seed": gaps,
            "gap_of_means_over_seeds": float(np.mean(lm) / np.mean(pm) - 1.0),
            "plain_seed_to_seed_rel_std": float(np.std(pm, ddof=1) / np.mean(pm)),
            "learned_seed_to_seed_rel_std": float(np.std(lm, ddof=1) / np.mean(lm)),
        }
    if r_alt is not None:
        ca = np.array([r.concavity for r in r_alt])
        out["concavity_plain_reseeded_mean"] = float(ca.mean())
        out["concavity_gap_of_means_plain_reseeded"] = float(ca.mean() / cp.mean() - 1.0)
    if st_l is not None:
        out["learned_fallback_rate"] = st_l["lp_fallbacks"] / max(st_l["lp_calls"], 1)
        out["learned_splits"] = st_l["lp_calls"]
    return out


def run_micro(args) -> dict:
    """Each kernel family once per repetition on a small representative case
    (per-call device time by CUDA events on the context stream): the command
    the ncu captures of the kernels other than visibility run.
      visibility  — s4 blob (2562 vertices, all 3,280,641 pairs) vs its 0.03 cage
      scoring     — 2^20 random edges x 4096 planes
      learned     — one training step of the proposer, 64 parts (forward,
                    backward, Adam; forward per-edge layers on tcgen05 and on
                    mma.sync), the forward alone on both paths, one proposal
      sdf_remesh  — the s5 blob's 0.03 cage at scale 40
      hausdorff   — concavity metric of the remeshed s4 blob vs its hull (3000)
      hull_dist   — all 2016 pairs of 64 hulls of 50..700 vertices
      clip        — the s5 blob cut by a plane through its centre"""
    from visacd_gb300 import _native as N, build, meshgen as mg, proposer as pp

    build.build_all()
    from visacd_gb300 import visacd as V

    V.config.verbose = False
    ctx = N.Context(0)
    rng = np.random.default_rng(3)
    out = {}

    def timed(name, fn, reps=3, **extra):
        fn()
        ctx.synchronize()
        ctx.set_timing(True)
        ctx.reset_times()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = fn()
        ctx.synchronize()
        wall = (time.perf_counter() - t0) / reps
        kt = ctx.kernel_times()
        ctx.set_timing(False)
        out[name] = {"wall_ms_per_call": wall * 1e3,
                     "kernels_ms_per_call": {k: round(v[0] / reps, 4) for k, v in kt.items() if v[1]},
                     **extra}
        return r

    v4, t4 = mg.displaced_blob(4, seed=2026)
    cv4, ct4 = mg.offset_cage(v4, t4, 0.03)
    sb, cb = ctx.bvh(v4, t4), ctx.bvh(cv4, ct4)
    timed("visibility", lambda: ctx.visibility(v4, sb, cb), pairs=len(v4) * (len(v4) - 1) // 2)
    E, P = 1 << 20, 4096
    pts = rng.uniform(-1, 1, size=(2 * E, 3)).astype(np.float32)
    edges = np.arange(2 * E, dtype=np.uint32).reshape(E, 2)
    nrm = rng.normal(size=(P, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    planes = np.concatenate([nrm, rng.uniform(-0.8, 0.8, size=(P, 1))], axis=1).astype(np.float32)
    timed("scoring", lambda: ctx.score_planes(planes, pts, edges), plane_edge_pairs=P * E)
    lp = N.PlaneProposer(ctx, seed=1)
    feats = rng.uniform(-1, 1, size=(64, N.LP_POINTS, N.LP_FEATURES)).astype(np.float32)
    labels = np.concatenate([nrm[:64 * 8].reshape(64, 8, 3), rng.uniform(-0.5, 0.5, size=(64, 8, 1))], -1)
    w = np.ones((64, 8), np.float32)
    timed("learned_train_step", lambda: lp.train_step(feats, labels, w, 1e-3),
          flop_per_step=3 * 2 * 64 * N.LP_POINTS * (16 * 64 + 64 * 128 + 128 * 256))
    lp.set_tcgen05(False)
    timed("learned_train_step_mma_sync", lambda: lp.train_step(feats, labels, w, 1e-3),
          flop_per_step=3 * 2 * 64 * N.LP_POINTS * (16 * 64 + 64 * 128 + 128 * 256))
    lp.set_tcgen05(True)
    fwd_flop = 2 * 64 * N.LP_POINTS * (16 * 64 + 64 * 128 + 128 * 256)
    timed("learned_forward_tcgen05", lambda: lp.forward(feats), flop=fwd_flop)
    lp.set_tcgen05(False)
    timed("learned_forward_mma_sync", lambda: lp.forward(feats), flop=fwd_flop)
    lp.set_tcgen05(True)
    e4, _ = ctx.visibility(v4, sb, cb)
    c, h = pp.part_frame(v4)
    timed("learned_propose", lambda: lp.propose(v4, e4, c, h))
    v5, t5 = mg.displaced_blob(5, seed=2026)
    v5 = v5 / np.abs(v5).max()
    timed("sdf_remesh", lambda: ctx.sdf_remesh(v5, t5, 40.0, 0.03))
    r4 = V._manifold_preprocess_gpu(v4 / np.abs(v4).max(), t4, 30.0, 0.55 / 30)
    hv = V._convex_hull(r4["vertices"])
    V.set_seed(1)
    xa, ia = V._sample_points(r4["vertices"], r4["triangles"], 3000)
    xb, ib = V._sample_points(hv["vertices"], hv["triangles"], 3000)
    timed("hausdorff", lambda: ctx.face_hausdorff(r4["vertices"], r4["triangles"], xa, ia, hv["vertices"],
                                                  hv["triangles"], xb, ib), samples=len(xa) + len(xb))
    hulls = [rng.uniform(-1, 1, 3) + rng.normal(scale=0.1, size=(int(rng.integers(50, 700)), 3)) for _ in range(64)]
    pairs = np.array([(a, b) for a in range(64) for b in range(a)], np.int32)
    timed("hull_dist", lambda: ctx.hull_distances(hulls, pairs), pairs=len(pairs))
    timed("clip", lambda: ctx.clip(v5, t5, [0.6, 0.8, 0.0, 0.0]))
    sb.close()
    cb.close()
    return out


class RefScoringKernel:
    """The reference's plane_point_side_and_rate_kernel (lib/cuda/plane_intersections.cu),
    compiled unchanged from its source into a cubin, launched through the CUDA
    driver API with the reference host wrapper's configuration (256 threads,
    one thread per (plane, edge) pair, scores zeroed first)."""

    NAME = b"_Z32plane_point_side_and_rate_kernelPKfS0_PKjPfiiif"

    def __init__(self, path: Path):
        import ctypes as C

        self.C = C
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self.fn = C.c_void_p()
        if self.cu.cuModuleLoad(C.byref(self.mod), str(path).encode()) != 0:
            raise RuntimeError("cuModuleLoad failed")
        if self.cu.cuModuleGetFunction(C.byref(self.fn), self.mod, self.NAME) != 0:
            raise RuntimeError("cuModuleGetFunction failed")

    def launch(self, d_planes, d_points, d_edges, d_scores, P, N, E, stream):
        C = self.C
        total = P * E
        grid = (total + 255) // 256
        if grid > 2**31 - 1:
            raise RuntimeError("grid too large for the reference launch")
        args = [C.c_void_p(d_planes), C.c_void_p(d_points), C.c_void_p(d_edges), C.c_void_p(d_scores),
                C.c_int(P), C.c_int(N), C.c_int(E), C.c_float(1e-6)]
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        rc = self.cu.cuLaunchKernel(self.fn, C.c_uint(grid), 1, 1, 256, 1, 1, 0, C.c_void_p(stream), ptrs, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel failed ({rc})")


def run_precision_sweep(args) -> dict:
    """Scoring at E in {2^20, 2^22, 2^24, 2^26} edges (endpoints U[-1,1]^3),
    P = 4096 planes (normals uniform on S^2, offsets U(-0.8, 0.8)): plane-edge
    pairs/s of this kernel and of the reference's kernel on the same GPU, FP64
    re-decided blocks, and the error against FP64 on a 16-plane slice."""
    import torch

    from visacd_gb300 import _native, build, meshgen

    build.build_gpu()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = _native.Context(0, stream.cuda_stream)
    import ctypes as C

    lib = _native.lib()
    cubin = ROOT / "oracle" / "_ref" / "ref_plane_intersections.cubin"
    ref = RefScoringKernel(cubin) if cubin.exists() else None
    P = 4096
    planes = meshgen.random_planes(P, seed=4096)
    d_pl = torch.from_numpy(planes).cuda()
    rows = []
    fp32_peak = ctx.fp32_peak_tflops()
    for lg in args.sweep_sizes:
        E = 1 << lg
        rng = np.random.default_rng(lg)
        pts = rng.uniform(-1, 1, size=(2 * E, 3)).astype(np.float32)
        edges = np.arange(2 * E, dtype=np.uint32).reshape(E, 2)
        d_pt = torch.from_numpy(pts).cuda()
        d_ed = torch.from_numpy(edges.view(np.int32)).cuda()
        d_sc = torch.empty(P, dtype=torch.float64, device="cuda")
        st = ctx.score_planes_device(d_pl.data_ptr(), P, d_pt.data_ptr(), 2 * E, d_ed.data_ptr(), E,
                                     d_sc.data_ptr(), stats=True)
        # Each planes-per-thread choice (what the scoring autotuner times),
        # best of 3; the row reports the fastest.
        ms_k = {}
        for k in (1, 2, 4, 8):
            ctx.set_score_k(k)
            evs = []
            for _ in range(3):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.score_planes_device(d_pl.data_ptr(), P, d_pt.data_ptr(), 2 * E, d_ed.data_ptr(), E,
                                        d_sc.data_ptr())
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize()
            ms_k[k] = min(a.elapsed_time(b) for a, b in evs)
        ctx.set_score_k(0)
        best_k = min(ms_k, key=ms_k.get)
        ms = ms_k[best_k]
        ctx.set_score_k(best_k)
        ctx.score_planes_device(d_pl.data_ptr(), P, d_pt.data_ptr(), 2 * E, d_ed.data_ptr(), E, d_sc.data_ptr())
        ctx.set_score_k(0)
        row = {"edges": E, "planes": P, "ms": ms, "planes_per_thread": best_k,
               "ms_per_planes_per_thread": {str(k): round(v, 4) for k, v in ms_k.items()},
               "plane_edge_pairs_per_s": P * E / (ms / 1e3),
               "tflops": 12.0 * P * E / (ms / 1e3) / 1e12, "band_blocks": st["band_blocks"]}
        row["frac_of_fp32_peak"] = row["tflops"] / fp32_peak
        if ref is not None:
            d_rs = torch.zeros(P, dtype=torch.float32, device="cuda")
            rtimes = []
            for _ in range(2):
                d_rs.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ref.launch(d_pl.data_ptr(), d_pt.data_ptr(), d_ed.data_ptr(), d_rs.data_ptr(), P, 2 * E, E,
                           stream.cuda_stream)
                b.record(stream)
                torch.cuda.synchronize()
                rtimes.append(a.elapsed_time(b))
            row["reference_kernel_ms"] = min(rtimes)
            row["reference_plane_edge_pairs_per_s"] = P * E / (min(rtimes) / 1e3)
            ours = d_sc.cpu().numpy()
            theirs = d_rs.cpu().numpy().astype(np.float64)
            row["reference_vs_ours_max_rel"] = float(np.max(np.abs(theirs - ours) / np.maximum(ours, 1e-30)))
            row["reference_argmax_equal"] = bool(np.argmax(theirs) == np.argmax(ours))
        if E <= (1 << 22):
            sub = np.arange(0, P, P // 16)
            s64 = _score_fp64_numpy(planes[sub], pts, edges)
            ours = d_sc.cpu().numpy()[sub]
            row["max_rel_err_vs_fp64"] = float(np.max(np.abs(ours - s64) / s64))
        rows.append(row)
        del d_pt, d_ed
        torch.cuda.empty_cache()
    # Segment-triangle decisions: FP32 filter + FP64 re-decision vs FP64 alone.
    S = args.segtri
    seg, tri, built = meshgen.segment_triangle_cases(S, 0.05, seed=11)
    ctx.segment_triangle_tests(seg, tri)
    ctx.set_timing(True)
    ctx.reset_times()
    t0 = time.perf_counter()
    hit, n64 = ctx.segment_triangle_tests(seg, tri)
    wall = time.perf_counter() - t0
    kms = ctx.kernel_times().get("seg_tri", (0.0, 0))[0]
    ctx.set_timing(False)
    ref = _segtri_fp64_numpy(seg, tri)
    segtri = {"tests": S, "built_to_graze": int(built.sum()), "fp64_rechecks": n64,
              "fp64_share": n64 / S, "kernel_ms": kms, "wall_ms_with_copies": wall * 1e3,
              "tests_per_s_kernel": S / (kms / 1e3) if kms else None,
              "decisions_equal_fp64": bool(np.array_equal(hit, ref)),
              "decisions_differing_from_fp64": int(np.sum(hit != ref))}
    return {"precision_sweep": rows, "fp32_peak_tflops": fp32_peak, "segment_triangle": segtri}


def _score_fp64_numpy(planes, pts, edges):
    """FP64 restatement of the score for a few planes: the summed FP64 length
    of the edges whose endpoints lie strictly on opposite sides (|value| >
    1e-6), numpy, independent of the kernels."""
    p = pts.astype(np.float64)
    a, b = p[edges[:, 0]], p[edges[:, 1]]
    ln = np.sqrt(((b - a) ** 2).sum(axis=1))
    out = np.zeros(len(planes))
    for k, pl in enumerate(planes.astype(np.float64)):
        va = a @ pl[:3] + pl[3]
        vb = b @ pl[:3] + pl[3]
        sa = np.where(va > 1e-6, 1, np.where(va < -1e-6, -1, 0))
        sb = np.where(vb > 1e-6, 1, np.where(vb < -1e-6, -1, 0))
        out[k] = ln[sa * sb == -1].sum()
    return out


def _segtri_fp64_numpy(seg, tri):
    """FP64 segment-triangle decision (edge functions relative to the origin,
    tmin 0.001), numpy, in the evaluation order of the kernels' FP64 path."""
    s = seg.astype(np.float64)
    t = tri.astype(np.float64).reshape(-1, 3, 3)
    o = s[:, :3]
    A, B, Cc, D = t[:, 0] - o, t[:, 1] - o, t[:, 2] - o, s[:, 3:] - o

    def cross(u, v):
        return np.stack([u[:, 1] * v[:, 2] - u[:, 2] * v[:, 1], u[:, 2] * v[:, 0] - u[:, 0] * v[:, 2],
                         u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]], axis=1)

    def dot(u, v):
        return (u[:, 0] * v[:, 0] + u[:, 1] * v[:, 1]) + u[:, 2] * v[:, 2]

    BC, CA, AB = cross(B, Cc), cross(Cc, A), cross(A, B)
    Wa, Wb, Wc = dot(D, BC), dot(D, CA), dot(D, AB)
    det = (Wa + Wb) + Wc
    vol = dot(A, BC)
    ln = np.sqrt((D[:, 0] * D[:, 0] + D[:, 1] * D[:, 1]) + D[:, 2] * D[:, 2])
    inside = ((Wa >= 0) & (Wb >= 0) & (Wc >= 0)) | ((Wa <= 0) & (Wb <= 0) & (Wc <= 0))
    tmin = float(np.float32(0.001))
    lhs, rhs = vol * ln, tmin * det
    hit = np.where(det > 0, (lhs >= rhs) & (vol <= det), (lhs <= rhs) & (vol >= det))
    return inside & (det != 0) & hit


def batch_parts(n_parts: int, seed: int = 7):
    """The batching workload: displaced blobs of subdivision drawn uniformly
    from {2, 3, 4, 5} with independent seeds, 0.03 offset cages, and 512
    candidate planes per part (normals uniform on the sphere, offsets uniform
    over the part's projection on the normal)."""
    from visacd_gb300 import meshgen

    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_parts):
        lv = int(rng.integers(2, 6))
        v, t = meshgen.displaced_blob(lv, seed=int(rng.integers(1 << 30)))
        cv, ct = meshgen.offset_cage(v, t, 0.03)
        nrm = rng.normal(size=(512, 3))
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        proj = v @ nrm.T
        d = -rng.uniform(proj.min(0), proj.max(0))
        out.append((v.astype(np.float32), t, cv, ct, np.concatenate([nrm, d[:, None]], 1).astype(np.float32)))
    return out


def run_batching(args) -> dict:
    """One graph-captured launch sequence over all parts vs per-part calls of
    the plain entry points (visibility then scoring, part by part)."""
    import torch

    from visacd_gb300 import _native, build

    build.build_gpu()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = _native.Context(0, stream.cuda_stream)
    parts = batch_parts(args.batch_parts)
    bv = [(v, ctx.bvh(v, t), ctx.bvh(cv, ct), pl) for v, t, cv, ct, pl in parts]
    batch = _native.Batch(ctx, bv)
    pairs, planes = batch.info()
    batch.run(True)  # capture + first replay
    batch.results()
    times = []
    for _ in range(max(args.steps, 2)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        batch.run(True)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ne, scores, am, _ = batch.results()
    t_batch = float(np.median(times)) / 1e3
    # Plain: per-part C-ABI calls (device-resident points, host sync per call).
    t0 = time.perf_counter()
    for v, sb, cb, pl in bv:
        e, _ = ctx.visibility(v, sb, cb)
        if len(e):
            ctx.score_planes(pl, v, e)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    batch.close()
    return {"batching": {"parts": len(parts), "pairs": pairs, "planes": planes, "edges": int(ne.sum()),
                         "graph_run_s": t_batch, "plain_loop_s": t_plain,
                         "batched_pairs_per_s": pairs / t_batch, "plain_pairs_per_s": pairs / t_plain,
                         "parts_per_s_batched": len(parts) / t_batch, "parts_per_s_plain": len(parts) / t_plain,
                         "speedup": t_plain / t_batch}}


def run_batch_decompositions(args) -> dict:
    """Decompositions of the batching workload's meshes (displaced blobs of
    subdivision 2-5, independent seeds), process(0.02, 64): process_batch over
    all of them (exhaustive and learned) against the plain sequential loop on
    the first --c3-plain of them (the loop's rate is per mesh, so a prefix
    measures it; the prefix's results are checked equal to the batch's)."""
    from visacd_gb300 import build

    build.build_host()
    from visacd_gb300 import visacd as V

    V.config.verbose = False
    parts = batch_parts(args.batch_parts)
    meshes = V.MeshList()
    for v, t, _, _, _ in parts:
        m = V.Mesh()
        m.vertices = V.VecArray3d(v.astype(np.float64).tolist())
        m.triangles = V.make_vecarray3i(np.asarray(t, dtype=np.int32))
        meshes.append(m)
    seeds = list(range(7000, 7000 + len(meshes)))
    conc, nparts = 0.02, 64
    V.set_seed(0)
    V.process(meshes[0], conc, nparts)  # warm-up
    out = {"workload": f"{len(meshes)} displaced blobs, subdivision 2-5 (the batching workload's meshes), "
                       "process(0.02, 64)", "meshes": len(meshes)}
    try:
        for mode in ("exhaustive", "learned"):
            V.config.plane_proposer = mode
            t0 = time.perf_counter()
            res = V.process_batch(meshes, conc, nparts, seeds, args.c5_threads)
            out[f"batched_{mode}_decomps_per_s"] = len(meshes) / (time.perf_counter() - t0)
            out[f"batched_{mode}_parts_mean"] = float(np.mean([r.num_parts for r in res]))
            out[f"batched_{mode}_concavity_mean"] = float(np.mean([r.concavity for r in res]))
            if mode == "exhaustive":
                batched = res
        V.config.plane_proposer = "exhaustive"
        k = min(args.c3_plain, len(meshes))
        t0 = time.perf_counter()
        plain = []
        for i in range(k):
            V.set_seed(seeds[i])
            plain.append(V.process(meshes[i], conc, nparts))
        out["plain_decomps_per_s"] = k / (time.perf_counter() - t0)
        out["plain_meshes_timed"] = k
        out["plain_equals_batched"] = all(a.concavity == b.concavity and a.num_parts == b.num_parts
                                          for a, b in zip(plain, batched[:k]))
    finally:
        V.config.plane_proposer = "exhaustive"
    out["speedup_batched_vs_plain"] = out["batched_exhaustive_decomps_per_s"] / out["plain_decomps_per_s"]
    out["speedup_batched_learned_vs_plain"] = out["batched_learned_decomps_per_s"] / out["plain_decomps_per_s"]
    return {"batch_decompositions": out}


WORKLOAD_TEXT = ("displaced icosphere s5 blob: 10242 verts, 20480 tris, all 52,444,161 pairs vs "
                 "part + 0.03 offset cage, then 2500 candidate planes scored")
REF_STRIDE = 4  # the reference arm's step: every 4th pair row (a quarter of the pairs)


def run_reference(args) -> dict:
    """The reference path's CPU restatement (the FP64 oracle: visibility by BVH
    traversal, then exact scoring of the same 2500 planes against the edges
    found), all host threads. Step k covers the pair rows i = k mod 4, so four
    consecutive steps do the whole workload once."""
    import oracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None, rank
    v, t, cv, ct = workload()
    n = len(v)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    # The candidate planes come from the edges, as in the GPU arm (setup).
    bits, _ = oracle.visibility_rows(v, t, cv, ct, np.arange(n))
    planes = bisector_planes(v, oracle.pairs_from_linear(np.nonzero(bits & 1)[0], n), N_PLANES, seed=1)
    times, pairs = [], []
    for k in range(args.warmup + args.steps):
        np_k, dt, _ = cpu_step(v, t, cv, ct, planes, np.arange(k % REF_STRIDE, n, REF_STRIDE))
        if k >= args.warmup:
            times.append(dt)
            pairs.append(np_k)
    value = sum(pairs) / sum(times)
    sample = (f"each step: the pair rows i = k mod {REF_STRIDE} of step k (about a quarter of the "
              f"52,444,161 pairs) plus the 2500 planes scored against that step's edges; "
              f"{REF_STRIDE} consecutive steps cover the whole workload")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "impl": "reference",
           "config": {"workload": WORKLOAD_TEXT, "pairs": n * (n - 1) // 2, "planes": N_PLANES,
                      "name": "blob_s5", "l2": "not applicable (host cores)",
                      "parallelism": "replicas x1"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out, rank


def cpu_baseline_full(v, t, cv, ct, planes, edges_gpu) -> tuple[dict, dict]:
    """The whole step once on the host cores (every pair row), timed, and the
    GPU's edges checked against its per-pair results."""
    import oracle

    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = len(v)
    pairs, dt, bits = cpu_step(v, t, cv, ct, planes, np.arange(n))
    base = {"value": pairs / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the whole workload once: all {pairs} pairs, then the 2500 planes scored "
                      f"(FP64 oracle, BVH traversal), {dt:.1f} s"}
    return base, grazing_check(v, bits, edges_gpu)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-process", action="store_true", help="skip the end-to-end decompositions")
    ap.add_argument("--workload", default="blob_s5", choices=sorted(WORKLOADS))
    ap.add_argument("--sweep", action="store_true", help="scoring precision sweep only")
    ap.add_argument("--batch", action="store_true", help="batching workload only")
    ap.add_argument("--batch-parts", type=int, default=256)
    ap.add_argument("--c3-decomps", action="store_true",
                    help="decompositions of the batching workload's meshes: batched vs plain")
    ap.add_argument("--c3-plain", type=int, default=64, help="meshes the plain loop times in --c3-decomps")
    ap.add_argument("--no-c3", action="store_true", help="skip the 256-mesh decompositions")
    ap.add_argument("--no-hulls", action="store_true", help="skip the batched convex hull timing")
    ap.add_argument("--sweep-sizes", type=int, nargs="+", default=[20, 22, 24, 26])
    ap.add_argument("--segtri", type=int, default=1 << 20, help="segment-triangle tests in the sweep")
    ap.add_argument("--c5", action="store_true", help="batched + learned decompositions only")
    ap.add_argument("--no-c5", action="store_true", help="skip the batched + learned decompositions")
    ap.add_argument("--c5-blobs", type=int, default=64)
    ap.add_argument("--c5-threads", type=int, default=0, help="process_batch workers (0 = all cores)")
    ap.add_argument("--c5-noise", action="store_true", help="also run plain with other seeds (noise floor)")
    ap.add_argument("--c5-fallbacks", action="store_true", help="also run learned sequentially (fallback rate)")
    ap.add_argument("--c5-seeds", type=int, default=4,
                    help="engine seeds for the concavity spread of both methods (batched runs)")
    ap.add_argument("--micro", action="store_true", help="one small case per kernel family (for ncu)")
    args = ap.parse_args()
    if args.micro:
        print(json.dumps(run_micro(args)))
        return
    if args.c5:
        print(json.dumps(run_learned_batch(args)))
        return
    if args.sweep:
        print(json.dumps(run_precision_sweep(args)))
        return
    if args.batch:
        print(json.dumps(run_batching(args)))
        return
    if args.c3_decomps:
        print(json.dumps(run_batch_decompositions(args)))
        return
    if args.impl == "reference":
        out, rank = run_reference(args)
    else:
        out, rank = run_ours(args)
        # The CPU baseline and the single-GPU decomposition workloads run on
        # rank 0 at N = 1 only (replica runs report the visibility step alone).
        single = out is not None and out["n_gpus"] == 1
        edges_gpu = out.pop("_edges", None) if out is not None else None
        planes = out.pop("_planes", None) if out is not None else None
        if rank == 0 and single and not args.no_cpu_baseline:
            v, t, cv, ct = workload(name=args.workload)
            out["cpu_baseline"], out["config"]["grazing"] = cpu_baseline_full(v, t, cv, ct, planes,
                                                                                edges_gpu)
        if rank == 0 and single and not args.no_process:
            out["process"] = run_decompositions(args)
        if rank == 0 and single and not args.no_c5:
            out["decomps"] = run_learned_batch(args)
        if rank == 0 and single and not args.no_c3:
            out["decomps_256"] = run_batch_decompositions(args)["batch_decompositions"]
        if rank == 0 and single and not args.no_hulls:
            out["hulls"] = run_hulls(args)
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
