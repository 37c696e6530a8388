"""Benchmark: signed-distance queries/s against a 1.3M-triangle mesh on GB300.

Workload (one "step"): quest::SignedDistance::computeDistances over 16,777,216
query points uniform in the 1.2x-expanded box of a level-8 displaced icosphere
(1,310,720 triangles, 655,362 vertices), all seeded synthetic data
(axom_gb300.workloads).  The headline ``value`` is the mixed-precision form
(FP32 outward-rounded traversal, FP64 refine and sign); the plain FP64 form is
reported beside it, and the BVH build time over the 1,310,720 triangle boxes
is reported as ``build_ms``.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

With N > 1 (launched by torch.distributed.run) every rank holds a replica of
the mesh and BVH and processes its own 16M points (weak scaling, no
collective on the data path); ``value`` is the total over ranks divided by
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SDF queries/s at 1.3M tris (mixed precision; FP64 path beside it)"
UNIT = "queries/s"
LEVEL = 8
MESH_SEED = 1234
QUERIES = 1 << 24
FALLBACK_HBM_GBS = 6800.0
BATCH_MESHES = 512
# Per point of one k_sdf_mixed launch, from the ncu capture summarised in
# profiles/k_sdf_mixed_level8_uniform_1M.md (1,048,576 uniform points of the
# same mesh): DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) and L2
# bytes (lts__t_sectors.sum x 32); the bench scales them by its point count.
MIXED_DRAM_BYTES_PER_POINT = (2.303622e9 + 0.580745e9) / 1048576
MIXED_L2_BYTES_PER_POINT = 2884381452 * 32 / 1048576
BATCH_SEED = 5
# The 100,000-box workload: boxes from seed 1, query boxes from seed 2.
C1_BOXES = 100_000
# Algorithmic bytes of one build per box: boxes read (48), codes and
# permutation through 4 LSD passes (2 x 8 each), tree links (12), refit (2 x 48).
BUILD_BYTES_PER_BOX = 48 + 4 * 2 * 8 + 12 + 2 * 48


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gsq", choices=["gsq", "reference"])
    ap.add_argument("--queries", type=int, default=QUERIES)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--only-config1", action="store_true",
                    help="run only the 100,000-box build and find leg (for profiling); prints its object")
    ap.add_argument("--no-forms", dest="forms", action="store_false",
                    help="skip the near-surface and adjoint legs")
    ap.add_argument("--batch-meshes", type=int, default=BATCH_MESHES,
                    help="meshes of the batched-form leg (0 skips it)")
    ap.add_argument("--batch-point-scale", type=float, default=1.0,
                    help="scales every mesh's point count in the batched leg")
    return ap.parse_args()


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def mesh():
    from axom_gb300 import workloads as W
    return W.displaced_icosphere(LEVEL, MESH_SEED)


def algorithmic_bytes_per_query(port, v, f, q_sample, threads):
    """B_q = 32 + 104 N_node + 88 N_leaf with N_node = box tests / 2 and N_leaf
    = triangle tests, counted by the instrumented oracle on a sample."""
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    nb, nl = port.sdf_counts(h, q_sample, threads=threads)
    return 32.0 + 104.0 * nb.mean() / 2.0 + 88.0 * nl.mean(), float(nb.mean()), float(nl.mean())


def median_time(fn, reps=3):
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def config1_leg(args, G, torch, port, threads):
    """The 100,000-box workload (BVH::initialize over 100,000 boxes, then
    findBoundingBoxes for 100,000 query boxes): device build and find times
    with their rooflines, the whole call with host buffers, the CSR against
    the oracle, and the oracle port's 1-thread and all-thread times."""
    from axom_gb300 import workloads as W
    boxes = W.random_boxes(C1_BOXES, 1)
    q = W.random_boxes(C1_BOXES, 2)
    bd = torch.from_numpy(boxes).cuda()
    qd = torch.from_numpy(q).cuda()
    bvh = G.BVH()
    build_ms, find_ms, find_call_ms = [], [], []
    for i in range(args.warmup + args.steps):
        bvh.initialize(bd)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = bvh.find_bounding_boxes(qd)
        torch.cuda.synchronize()
        if i >= args.warmup:
            build_ms.append(bvh.last_build_ms())
            find_ms.append(bvh.last_find_ms())
            find_call_ms.append((time.perf_counter() - t0) * 1000.0)
    off, cnt, cand = (r.cpu().numpy() for r in res)
    # end to end: host boxes in, host CSR out, copies inside
    e2e = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        hb = G.BVH(boxes)
        hres = hb.find_bounding_boxes(q)
        if i >= args.warmup:
            e2e.append((time.perf_counter() - t0) * 1000.0)
    hp = port.bvh(boxes)
    want = port.find_boxes(hp, q)
    equal = all(np.array_equal(np.asarray(a), b) for a, b in zip((off, cnt, cand), want)) and \
        all(np.array_equal(np.asarray(a), b) for a, b in zip(hres, want))
    nb = port.find_boxes_counts(hp, q)
    bq = 48.0 + 104.0 * nb.mean() / 2.0 + 4.0 * (cand.size / C1_BOXES + 2.0)
    hbm, kind = peaks()
    bms, fms = statistics.median(build_ms), statistics.median(find_ms)
    build_gbs = BUILD_BYTES_PER_BOX * C1_BOXES / (bms / 1000.0) / 1e9
    find_gbs = bq * C1_BOXES / (fms / 1000.0) / 1e9
    cpu_build_1 = median_time(lambda: port.bvh(boxes))
    cpu_find_1 = median_time(lambda: port.find_boxes(hp, q))
    cpu_find_n = median_time(lambda: port.find_boxes_mt(hp, q, threads))
    return {
        "workload": f"{C1_BOXES} boxes (seed 1) and {C1_BOXES} query boxes (seed 2): centres U[0,1]^3, "
                    "sides log-uniform in [1e-3, 1e-2]; scale 1.000123",
        "build_ms": bms, "find_ms": fms, "find_call_ms": statistics.median(find_call_ms),
        "candidates": int(cand.size), "box_tests_per_query": float(nb.mean()),
        "e2e_ms": statistics.median(e2e), "e2e_note": "host boxes in, host CSR out: build + find calls, copies inside",
        "oracle_equal": bool(equal),
        "roofline_build": {"bound": "hbm", "achieved": build_gbs, "peak": hbm, "unit": "GB/s",
                           "frac": build_gbs / hbm, "peak_kind": kind,
                           "algorithmic_bytes_per_box": BUILD_BYTES_PER_BOX},
        "roofline_find": {"bound": "hbm", "achieved": find_gbs, "peak": hbm, "unit": "GB/s",
                          "frac": find_gbs / hbm, "peak_kind": kind, "algorithmic_bytes_per_query": bq},
        "cpu_baseline": {"kind": "port", "build_ms_1_thread": 1000.0 * cpu_build_1,
                         "find_ms_1_thread": 1000.0 * cpu_find_1, "find_ms_all_threads": 1000.0 * cpu_find_n,
                         "cores": threads,
                         "sample": "the whole workload, median of 3; the build is serial as the reference's SEQ "
                                   "path is; the threaded find splits the queries into contiguous ranges"},
    }


def cpu_baseline(port, v, f, q, seconds, threads):
    """The oracle port on the host cores, on a bounded stratified sample."""
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    probe = q[:: max(1, q.shape[0] // 4000)][:4000]
    t0 = time.perf_counter()
    port.sdf_eval(h, probe, threads=threads)
    rate = probe.shape[0] / max(time.perf_counter() - t0, 1e-6)
    n = int(min(q.shape[0], max(2000, rate * seconds)))
    sample = q[np.linspace(0, q.shape[0] - 1, n).astype(np.int64)]
    t0 = time.perf_counter()
    port.sdf_eval(h, sample, threads=threads)
    dt = time.perf_counter() - t0
    # one core, on a smaller stratified sample (about a fifth of the time above)
    n1 = int(min(q.shape[0], max(500, rate / threads * seconds / 5)))
    s1 = q[np.linspace(0, q.shape[0] - 1, n1).astype(np.int64)]
    t0 = time.perf_counter()
    port.sdf_eval(h, s1, threads=1)
    dt1 = time.perf_counter() - t0
    # the SignedDistance constructor (mesh box, cell boxes, BVH::initialize) and
    # BVH::initialize alone over the triangle boxes, one core
    sdf_ctor = median_time(lambda: port.sdf(v[:, 0], v[:, 1], v[:, 2], f))
    tri = v[f]
    tboxes = np.concatenate([tri.min(1), tri.max(1)], 1)
    bvh_init = median_time(lambda: port.bvh(tboxes))
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} stratified points of the {q.shape[0]} (every {q.shape[0] // n}th), "
                      f"{dt:.1f} s on {threads} host threads",
            "one_core": {"value": n1 / dt1, "unit": UNIT, "sample": f"{n1} stratified points, {dt1:.1f} s"},
            "sdf_ctor_ms_1_thread": 1000.0 * sdf_ctor, "bvh_init_ms_1_thread": 1000.0 * bvh_init,
            "bvh_init_boxes": int(f.shape[0])}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args, world, rank):
    """Reference arm: the CPU implementation of the path (oracle port) on all host cores."""
    if rank != 0:
        return
    import oracle
    from axom_gb300 import workloads as W
    threads = os.cpu_count() or 1
    port = oracle.Port()
    v, f = mesh()
    q = W.uniform_queries(v, args.queries, 3)
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    probe = q[:2000]
    t0 = time.perf_counter()
    port.sdf_eval(h, probe, threads=threads)
    rate = probe.shape[0] / (time.perf_counter() - t0)
    n = int(min(q.shape[0], max(2000, rate * 8.0)))
    times = []
    for s in range(args.warmup + args.steps):
        idx = np.linspace(s, q.shape[0] - 1, n).astype(np.int64)
        sample = q[idx]
        t0 = time.perf_counter()
        port.sdf_eval(h, sample, threads=threads)
        if s >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = n * len(times) / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * args.queries / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, f),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} stratified points of {args.queries} per step, timed on {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_leg(args, G, torch, lib, threads):
    """The batched form: BATCH_MESHES icospheres of levels 2..6 (random rotation,
    scale 0.5..2, translation in [-10, 10]^3), each with a log-uniform 1k..1M
    points uniform in its 1.2x box.  A step rebuilds every tree and evaluates
    every point: one CUDA graph launch."""
    import oracle
    from axom_gb300 import workloads as W
    meshes, pts = W.batch_meshes(args.batch_meshes, BATCH_SEED, point_scale=args.batch_point_scale)
    tris = sum(f.shape[0] for _, f in meshes)
    flat = np.concatenate(pts)
    m = flat.shape[0]
    b = G.Batch(meshes, pts)
    t0 = time.perf_counter()
    tuned = b.tune()
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.run_device()
    torch.cuda.synchronize()
    launches0 = lib.gsq_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    graph_ms = []
    ev0.record()
    for _ in range(args.steps):
        graph_ms.append(b.run_device())
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = lib.gsq_kernel_launches() - launches0
    # the build alone: the same meshes without points
    bb = G.Batch(meshes, [p[:0] for p in pts])
    build_ms = []
    for i in range(args.warmup + args.steps):
        bb.run_device()
        if i >= args.warmup:
            build_ms.append(bb.last_ms())
    del bb
    # end to end: pinned host vertices and points in, pinned host distances out
    allv = np.concatenate([v for v, _ in meshes])
    xyz = tuple(torch.from_numpy(np.ascontiguousarray(allv[:, k])).pin_memory() for k in range(3))
    q_pin = torch.from_numpy(flat).pin_memory()
    out_pin = torch.empty(m, dtype=torch.float64).pin_memory()
    for _ in range(max(1, args.warmup)):
        b.set_vertices(xyz)
        b.set_points(q_pin)
        b.run(out=out_pin)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.set_vertices(xyz)
        b.set_points(q_pin)
        b.run(out=out_pin)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    # parity spot check: a few meshes against a standalone SignedDistance
    d = out_pin.numpy()
    parts = b.split(d)
    exact = True
    for k in np.linspace(0, len(meshes) - 1, 4).astype(int):
        v, f = meshes[k]
        ref = G.SignedDistance(v, f).compute_distances(pts[k][:20000])
        exact &= bool(np.array_equal(ref.view(np.int64), parts[k][:20000].view(np.int64)))
    # CPU baseline, timed on a sample: the port builds 16 of the meshes (evenly
    # spaced, 1 thread, as the reference's SEQ build) and evaluates a stratified
    # sample of each one's points (all host threads); the rate is the sample's
    # points over the sample's build + query time
    port = oracle.Port()
    sample_meshes = np.linspace(0, len(meshes) - 1, 16).astype(int)
    cpu_build_s, cpu_tris, cpu_q_s, cpu_q = 0.0, 0, 0.0, 0
    for k in sample_meshes:
        v, f = meshes[k]
        t0 = time.perf_counter()
        h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
        cpu_build_s += time.perf_counter() - t0
        cpu_tris += f.shape[0]
        pk = pts[k]
        qs = pk[np.linspace(0, pk.shape[0] - 1, min(pk.shape[0], 20000)).astype(np.int64)]
        t0 = time.perf_counter()
        port.sdf_eval(h, qs, threads=threads)
        cpu_q_s += time.perf_counter() - t0
        cpu_q += qs.shape[0]
    return {
        "workload": f"batched form: {len(meshes)} icospheres (levels 2-6, {tris} triangles), {m} points "
                    f"(log-uniform 1k-1M per mesh); a step rebuilds every tree and evaluates every point",
        "value": m / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms, "graph_ms": statistics.mean(graph_ms),
        "build_only_ms": statistics.median(build_ms), "meshes": len(meshes), "triangles": int(tris),
        "points": int(m), "tuned": tuned, "max_tree_depth": b.max_depth(), "tune_s": tune_s,
        "gpu_launches": int(launches), "graph_launches_per_step": 1,
        "e2e": {"value": m / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 24 * m + 24 * int(allv.shape[0]), "d2h_bytes_per_step": 8 * m},
        "spot_check_bit_exact": exact,
        "cpu_baseline": {"value": cpu_q / (cpu_build_s + cpu_q_s), "unit": UNIT, "cores": threads, "kind": "port",
                         "build_s": cpu_build_s, "query_s": cpu_q_s,
                         "sample": f"timed: port build of {len(sample_meshes)} of the meshes ({cpu_tris} triangles, "
                                   f"1 thread) and {cpu_q} stratified points of those meshes ({threads} threads); "
                                   f"rate = sample points / (build + query seconds)"},
    }


def near_surface_leg(args, G, torch, v, f):
    """Sign robustness at scale: 16M points on the level-8 mesh, half uniform in
    the 1.2x box and half at a random surface point offset along the normal by
    10^U[-9,-3] (either side).  The mixed form against the FP64 form on the
    GPU over every point: relative error and sign mismatches."""
    from axom_gb300 import workloads as W
    m = args.queries
    q = torch.from_numpy(W.mixed_queries(v, f, m, 4)).cuda()
    sd = G.SignedDistance(v, f, precision=G.PRECISION_MIXED)
    dm = torch.empty(m, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        sd.compute_distances(q, out=dm)
    kms = []
    for _ in range(args.steps):
        sd.compute_distances(q, out=dm)
        kms.append(sd.last_eval_ms())
    sd.set_precision(G.PRECISION_FP64)
    d64 = sd.compute_distances(q)
    rel = (dm - d64).abs() / d64.abs().clamp_min(1e-300)
    res = {"workload": f"{m} points: half uniform in the 1.2x box, half within 1e-9..1e-3 of the surface",
           "value": m / (statistics.median(kms) / 1000.0), "unit": UNIT, "kernel_ms": statistics.median(kms),
           "fp64_kernel_ms": sd.last_eval_ms(),
           "sign_mismatches": int((torch.signbit(dm) != torch.signbit(d64)).sum().item()),
           "max_rel_err": float(rel.max().item()),
           "rel_err_p50_p99_p999": [float(x) for x in torch.quantile(
               rel[:: max(1, m // (1 << 20))].float(), torch.tensor([0.5, 0.99, 0.999], device="cuda")).tolist()],
           "bit_identical_to_fp64": bool(torch.equal(dm.view(torch.int64), d64.view(torch.int64)))}
    del q, dm, d64
    return res


def adjoint_leg(args, G, torch):
    """Differentiated form: level-6 displaced icosphere (81,920 triangles),
    1,048,576 uniform points, L = sum w d^2 with w ~ U[0,1]: forward (mixed,
    saving each point's closest triangle as an autograd forward would) plus
    the hand-written adjoint (dL/dpoints and the deterministic vertex
    reduction) per step."""
    from axom_gb300 import workloads as W
    v, f = W.displaced_icosphere(6, MESH_SEED)
    m = 1 << 20
    q = torch.from_numpy(W.uniform_queries(v, m, 3)).cuda()
    w = torch.from_numpy(np.random.default_rng(6).uniform(0, 1, m)).cuda()
    sd = G.SignedDistance(v, f, precision=G.PRECISION_MIXED)

    def step():
        d, tri = sd.compute_distances_tri(q)
        return sd.backward(q, 2.0 * w * d, dist=d, triangles=tri)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        gp, gv = step()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    gp2, gv2 = step()
    return {"workload": f"level-6 mesh ({f.shape[0]} triangles, {v.shape[0]} vertices), {m} uniform points, "
                        "forward (distances and closest triangles) + backward per step",
            "value": m / (ms / 1000.0), "unit": "points/s (forward + backward)", "ms_per_step": ms,
            "deterministic": bool(torch.equal(gv.view(torch.int64), gv2.view(torch.int64)))}


def closest_point_leg(args, G, torch, port, v, threads):
    """DistributedClosestPoint's local query: the 655,362 vertices of the
    level-8 mesh as object points, 16M query points uniform in the 1.2x box,
    no threshold; both precisions, and the oracle port on a sample."""
    from axom_gb300 import workloads as W
    m = args.queries
    q = torch.from_numpy(W.uniform_queries(v, m, 8)).cuda()
    cp = G.ClosestPoint(v)
    res = {"workload": f"{v.shape[0]} object points (the level-8 mesh vertices), {m} uniform query points"}
    outs = {}
    for name, prec in (("mixed", G.PRECISION_MIXED), ("fp64", G.PRECISION_FP64)):
        for _ in range(args.warmup):
            cp.compute_closest_points(q, precision=prec)
        ms = []
        for _ in range(args.steps):
            outs[name] = cp.compute_closest_points(q, precision=prec)
            ms.append(cp.last_query_ms())
        res[name] = {"value": m / (statistics.median(ms) / 1000.0), "unit": UNIT, "kernel_ms": statistics.median(ms)}
    res["mixed_equals_fp64"] = bool(all(torch.equal(a.view(torch.int32) if a.dtype == torch.int32 else
                                                    a.view(torch.int64), b.view(torch.int32) if
                                                    b.dtype == torch.int32 else b.view(torch.int64))
                                        for a, b in zip(outs["mixed"], outs["fp64"])))
    sample = q[:: max(1, m // 200_000)].cpu().numpy()
    h = port.cp(v)
    t0 = time.perf_counter()
    want = port.cp_query(h, sample, threads=threads)
    dt = time.perf_counter() - t0
    got = outs["mixed"][0][:: max(1, m // 200_000)].cpu().numpy()
    res["oracle_sample_equal"] = bool(np.array_equal(got, want[0]))
    res["cpu_baseline"] = {"value": sample.shape[0] / dt, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": f"{sample.shape[0]} of the query points"}
    del q
    return res


def workload_config(args, f):
    return {"workload": f"signed distance: displaced icosphere level {LEVEL} ({f.shape[0]} triangles), "
                        f"{args.queries} uniform points in the 1.2x box per GPU",
            "mesh_triangles": int(f.shape[0]), "queries_per_gpu": int(args.queries), "precision": args.precision,
            "l2": "no flush: the 402 MB of query points and outputs per step exceed the 129 MB L2"}


def run_gsq(args, world, rank, local):
    import torch
    import axom_gb300 as G
    import oracle
    from axom_gb300 import workloads as W

    torch.cuda.set_device(local)
    torch.cuda.init()
    if args.only_config1:
        print(json.dumps(config1_leg(args, G, torch, oracle.Port(), os.cpu_count() or 1)), flush=True)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = G.load()
    v, f = mesh()
    m = args.queries
    q_host = W.uniform_queries(v, m, 3 + rank)
    q_dev = torch.from_numpy(q_host).cuda()
    prec = G.PRECISION_MIXED if args.precision == "mixed" else G.PRECISION_FP64
    sd = G.SignedDistance(v, f, precision=prec)
    out = torch.empty(m, dtype=torch.float64, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # BVH build over the 1,310,720 triangle boxes (BVH::initialize).
    tri = v[f]
    boxes = torch.from_numpy(np.concatenate([tri.min(1), tri.max(1)], 1)).cuda()
    bvh = G.BVH()
    build_ms = []
    for i in range(args.warmup + args.steps):
        bvh.initialize(boxes)
        if i >= args.warmup:
            build_ms.append(bvh.last_build_ms())
    # the SignedDistance constructor (host vertices and cells in: the copies,
    # the cell boxes, the BVH build, the FP64 and FP32 records), wall clock
    ctor_ms = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sd_new = G.SignedDistance(v, f, precision=prec)
        torch.cuda.synchronize()
        ctor_ms.append((time.perf_counter() - t0) * 1000.0)
        del sd_new

    def run_steps(precision, steps, warmup):
        sd.set_precision(precision)
        for _ in range(warmup):
            sd.compute_distances(q_dev, out=out)
        barrier()
        launches0 = lib.gsq_kernel_launches()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kms = []
        ev0.record()
        for _ in range(steps):
            sd.compute_distances(q_dev, out=out)
            kms.append(sd.last_eval_ms())
        ev1.record()
        barrier()
        ms = ev0.elapsed_time(ev1) / steps
        return max_over_ranks(ms), statistics.mean(kms), lib.gsq_kernel_launches() - launches0

    clocks = Clocks(local)
    clocks.start()
    ms, kernel_ms, launches = run_steps(prec, args.steps, args.warmup)
    clk = clocks.stop()
    value = world * m / (ms / 1000.0)

    # End to end through the public API with host buffers: pinned host points in,
    # pinned host distances out, copies inside the timed region (measured right
    # after the device-resident steps, before the FP64 leg).
    q_pin = torch.from_numpy(q_host).pin_memory()
    out_pin = torch.empty(m, dtype=torch.float64).pin_memory()
    for _ in range(max(1, args.warmup)):
        sd.compute_distances(q_pin, out=out_pin)
    # the host link's copy rates at this moment (the GPUs of a machine share
    # their hosts' memory, so other jobs can slow these copies)
    link = {}
    for name, dst, src in (("h2d_gbs", q_dev, q_pin), ("d2h_gbs", out_pin, out)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        link[name] = src.numel() * src.element_size() / (time.perf_counter() - t1) / 1e9
    barrier()
    clocks_e2e = Clocks(local)
    clocks_e2e.start()
    t0 = time.perf_counter()
    e2e_steps = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        sd.compute_distances(q_pin, out=out_pin)
        e2e_steps.append((time.perf_counter() - t1) * 1000.0)
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1000.0 / args.steps)
    clk_e2e = clocks_e2e.stop()

    other = G.PRECISION_FP64 if prec == G.PRECISION_MIXED else None
    fp64 = None
    if other is not None:
        out_mixed = out.clone()
        ms64, kms64, _ = run_steps(other, max(1, min(args.steps, 3)), 1)
        fp64 = {"value": world * m / (ms64 / 1000.0), "ms_per_step": ms64, "kernel_ms": kms64,
                "speedup_mixed_over_fp64": ms64 / ms,
                "mixed_bit_identical": bool(torch.equal(out_mixed.view(torch.int64), out.view(torch.int64))),
                "sign_mismatches": int((torch.signbit(out_mixed) != torch.signbit(out)).sum().item())}
        del out_mixed
        sd.set_precision(prec)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    hbm, hbm_kind = peaks()
    threads = os.cpu_count() or 1
    port = oracle.Port()
    sample = q_host[np.linspace(0, m - 1, 20000).astype(np.int64)]
    bq, nb, nl = algorithmic_bytes_per_query(port, v, f, sample, threads)
    achieved = bq * m / (kernel_ms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 traversal + f64 refine" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": workload_config(args, f),
        "fp64": fp64,
        "sdf_ctor_ms": {"value": statistics.median(ctor_ms), "runs": len(ctor_ms),
                        "note": "SignedDistance constructor from host vertices and cells, wall clock"},
        "build_ms": {"value": statistics.median(build_ms), "boxes": int(f.shape[0]), "runs": len(build_ms),
                     "roofline": {"bound": "hbm", "unit": "GB/s", "peak": hbm, "peak_kind": hbm_kind,
                                  "algorithmic_bytes_per_box": BUILD_BYTES_PER_BOX,
                                  "achieved": BUILD_BYTES_PER_BOX * f.shape[0] / (statistics.median(build_ms) / 1e3) / 1e9,
                                  "frac": BUILD_BYTES_PER_BOX * f.shape[0] / (statistics.median(build_ms) / 1e3) / 1e9 / hbm}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": MIXED_DRAM_BYTES_PER_POINT * m if args.precision == "mixed" else None,
                     "traffic_note": "ncu DRAM bytes per point on a 1,048,576-point launch, scaled to this launch "
                                     "(profiles/k_sdf_mixed_level8_uniform_1M.md)",
                     "l2_bytes": MIXED_L2_BYTES_PER_POINT * m if args.precision == "mixed" else None,
                     "l2_gbs": (MIXED_L2_BYTES_PER_POINT * m / (kernel_ms / 1000.0) / 1e9
                                if args.precision == "mixed" else None),
                     "peak_kind": hbm_kind,
                     "kernel": "k_sdf_mixed" if args.precision == "mixed" else "k_sdf_fp64",
                     "kernel_ms": kernel_ms,
                     "algorithmic_bytes_per_query": bq, "box_tests_per_query": nb, "leaf_tests_per_query": nl},
        "e2e": {"value": world * m / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": 24 * m, "d2h_bytes_per_step": 8 * m, "clocks": clk_e2e,
                "step_ms_min_median_max": [min(e2e_steps), statistics.median(e2e_steps), max(e2e_steps)],
                "link": link},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(port, v, f, q_host, args.cpu_seconds, threads)
    if world == 1 and args.forms:
        line["config1"] = config1_leg(args, G, torch, port, threads)
        line["near_surface"] = near_surface_leg(args, G, torch, v, f)
        line["adjoint"] = adjoint_leg(args, G, torch)
        line["closest_point"] = closest_point_leg(args, G, torch, port, v, threads)
    if world == 1 and args.batch_meshes > 0:
        torch.cuda.empty_cache()
        line["batched"] = batched_leg(args, G, torch, lib, threads)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gsq(args, world, rank, local)


if __name__ == "__main__":
    main()
