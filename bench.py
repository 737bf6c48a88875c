"""Benchmark: batched GJK+EPA pairs/s on one GB300, mixed vs plain FP64.

Workload: 1,048,576 collider pairs, types uniform over Sphere, Capsule, Box,
Cylinder, Ellipsoid and ConvexHullVertices (hulls of N ~ logU[8,256] points on
the unit sphere scaled by U[0.05,0.3]), centers in [-w,w]^3 with w calibrated
to ~30% intersecting pairs (w = 1 as literally given yields ~3%; both
fractions are printed).  One step = GJK distance for every pair, then EPA on
the intersecting pairs.  Inputs are seeded synthetic data (2.1 M colliders,
~1.6 GB resident, larger than L2, so no flush is needed between steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is the mixed-precision form, inputs resident in HBM; ``fp64`` the
plain FP64 drop-in on the same data; ``e2e`` the mixed form through the C ABI
from pinned host buffers with every host<->device copy inside the timed
region.  ``--impl reference`` times the CPU reference restatement (oracle,
all host cores) on the same workload.  Under torchrun each rank processes its
own shard of pairs (no data exchange) and rank 0 prints one JSON line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PAIRS = 1 << 20
SEED = 2024
METRIC = "GJK+EPA pairs/s (mixed precision form; plain FP64 form alongside)"
UNIT = "pairs/s"
EPA_KW = dict(max_iter=64, max_loose_edges=128, max_faces=256, epsilon=1e-8)
# DRAM bytes per pair of the mixed kernels from one ncu capture of the
# 131,072-pair workload (k_gjk_mixed_a + k_gjk_mixed_b + k_gjk_mixed_end per
# pair; k_epa_warp + k_epa_refine per EPA pair, 38,814 of them); traffic
# grows in proportion to the pairs
NCU_DRAM_BYTES_PER_PAIR = {"gjk_mixed": (78464256 + 3834112 + 140287744 + 23856896 + 45120768 + 1776384) / 131072,
                           "epa_mixed": (33026304 + 36096 + 37686784 + 27904) / 38814}
# this library's kernels per timed mixed step (one graph replay): k_pair_keys,
# k_gjk_mixed_a, k_gjk_mixed_b, k_gjk_mixed_end, k_gjk_distance_f64
# (fallback list), k_epa_select, k_epa_warp<float>, k_epa_refine,
# k_epa_warp<double> (fallback list), k_epa_exact_warp (second fallback
# list); the CUB sort kernels are the toolkit's
MIXED_STEP_LAUNCHES = 10

# Algorithmic bytes per pair (counted once): two collider records, the hull
# vertices of hull colliders, and the outputs.  FP64 record 120 B (pose 96 +
# params 24) + type; FP32 record 60 B.  Hull vertices 24 B (FP64) / 12 B
# (FP32) each.  Outputs: dist 8 + cp1 24 + cp2 24 + simplex 96 + n_simplex 1 +
# status 1 = 154 B; EPA: mtv 24 + status 1 + face count 4 per intersecting pair.
REC64, REC32, OUT_GJK, OUT_EPA = 124, 64, 154, 29

# Flop model of one GJK iteration (FMA = 2), fixed before any flop rate was
# measured and not tuned since: support function by collider type (sphere,
# capsule, box as an 8-vertex hull, cylinder, ellipsoid; a hull costs 6 per
# vertex) plus an average closest-point solve (line ~20, triangle ~80,
# tetrahedron ~400, weighted by how often each occurs: 150).
SUPPORT_FLOPS = [12, 50, 48, 50, 50]
HULL_FLOPS_PER_VERTEX = 6
SOLVE_FLOPS = 150


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=N_PAIRS)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--serve-seconds", type=float, default=2.0,
                    help="seconds of Poisson arrivals per load level in the serving report (0: skip)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch parameters (profiling runs)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the broad+narrow, robot and MPR sections (profiling runs)")
    ap.add_argument("--mpr-only", action="store_true",
                    help="run only the MPR section on the workload, without its CPU leg (profiling runs)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(n_pairs, rank):
    from distance3d_gb300 import workloads
    cs, i1, i2 = workloads.pairs_mixed_six(n_pairs, seed=SEED + rank,
                                           center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    return cs, i1, i2


def algorithmic_bytes(cs, i1, n_epa, precision):
    hull = cs.types == 5
    nv = cs.hull_count.astype(np.float64)
    per_vertex = 24 if precision == "fp64" else 12
    rec = REC64 if precision == "fp64" else REC32
    n = len(i1)
    inputs = 2 * n * rec + per_vertex * float(nv[hull].sum()) + 8 * n  # + the two int32 indices
    return inputs + OUT_GJK * n + OUT_EPA * n_epa


def measure_pipe_peaks(dev):
    """FP64 and FP32 FMA throughput (FLOP/s) of this GPU, measured by the
    probe library built beside libd3d_gb300 (8 independent FMA chains per
    thread, SMs x 8 blocks of 256 threads)."""
    import ctypes
    import torch
    from distance3d_gb300 import build as b
    lib = ctypes.CDLL(b.PEAK_LIB)
    lib.d3d_peak_fma_flops.restype = ctypes.c_double
    lib.d3d_peak_fma_flops.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    fp64 = max(lib.d3d_peak_fma_flops(1, 4096, st) for _ in range(3))
    fp32 = max(lib.d3d_peak_fma_flops(0, 65536, st) for _ in range(3))
    return fp64, fp32


def gjk_model_flops(cs, i1, i2, iterations):
    """Model FLOPs of the plain GJK over all pairs, from the per-pair
    iteration counts (exact: the FP64 kernel reports them)."""
    cost = np.zeros(len(cs))
    for t, f in enumerate(SUPPORT_FLOPS):
        cost[cs.types == t] = f
    hull = cs.types == 5
    cost[hull] = HULL_FLOPS_PER_VERTEX * cs.hull_count[hull]
    per_iter = cost[i1] + cost[i2] + SOLVE_FLOPS
    return float(np.sum(per_iter * iterations))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def accuracy_report(store, i1, i2, out_mixed, out_fp64, dev):
    """Errors of the mixed form against the FP64 form (= the reference).

    Distances: relative error where the reference is self-consistent; where
    its distance disagrees with its own closest points (rare), the mixed
    result's own duality bracket (exact FP64 supports) is reported instead.
    EPA depths: both forms return h(n) = n . (s1(n) - s2(-n)), an upper bound
    on the true depth; pairs where the reference's depth exceeds h(n_mixed)
    by more than 1e-5 are counted as reference errors, the rest give the
    error statistics, and any pair where the mixed depth is the larger one
    beyond 1e-5 is counted as a mixed error."""
    import torch
    gm, hm, em = out_mixed
    gf, hf, ef = out_fp64
    dm, df = gm["dist"], gf["dist"]
    sep_f = (gf["cp1"] - gf["cp2"]).norm(dim=1)
    incons = ((sep_f - df).abs() > 1e-9 * df.clamp(min=1.0)) & (df > 0)
    ok = ~incons
    rel = ((dm - df).abs() / df.abs().clamp(min=1.0))[ok].cpu().numpy()
    sep = df > 1e-6
    out = {"max_rel_dist_err": float(rel.max()), "p99_rel_dist_err": float(np.percentile(rel, 99)),
           "flags_identical_beyond_1e-6": bool(torch.equal(dm[sep] > 0, df[sep] > 0)),
           "reference_self_inconsistent_pairs": int(incons.sum().item())}
    k = torch.nonzero(incons & (dm > 0)).flatten()
    if k.numel():
        v = gm["cp1"][k] - gm["cp2"][k]
        ub = v.norm(dim=1)
        u = v / ub[:, None]
        w = store.support(i1[k], -u) - store.support(i2[k], u)
        lb = (u * w).sum(dim=1)
        out["mixed_certified_gap_on_those"] = float(((ub - lb) / ub.clamp(min=1.0)).max().item())
    common, ia, ib = np.intersect1d(hm.cpu().numpy(), hf.cpu().numpy(), return_indices=True)
    ia = torch.as_tensor(ia, device=dev)
    ib = torch.as_tensor(ib, device=dev)
    both = (em["status"][ia] == 0) & (ef["status"][ib] == 0)
    a = em["mtv"][ia][both]
    b = ef["mtv"][ib][both]
    da, db = a.norm(dim=1), b.norm(dim=1)
    tol = 1e-5 * db.clamp(min=1.0)
    pairs = torch.as_tensor(common, device=dev)[both]
    n = a / da.clamp(min=1e-300)[:, None]
    h = (n * (store.support(i1[pairs], n) - store.support(i2[pairs], -n))).sum(dim=1)
    ref_wrong = (db > da + tol) & (h < db - tol)
    good = ~ref_wrong
    derr = ((da - db).abs() / db.clamp(min=1.0))[good].cpu().numpy()
    out.update({"epa_pairs_both_converged": int(both.sum().item()),
                "epa_converged_mixed": int((em["status"] == 0).sum().item()),
                "epa_converged_fp64": int((ef["status"] == 0).sum().item()),
                "epa_depth_max_rel_err": float(derr.max()) if derr.size else None,
                "epa_depth_p99_rel_err": float(np.percentile(derr, 99)) if derr.size else None,
                "epa_pairs_reference_depth_not_minimal": int(ref_wrong.sum().item()),
                "epa_pairs_mixed_deeper_than_reference": int((da > db + tol).sum().item())})
    return out


def cpu_oracle_pass(cs, i1, i2, nthreads=0):
    """The reference algorithm on the host (C restatement, OpenMP): GJK
    distance for every pair, EPA on pairs with a full simplex."""
    from oracle import oracle
    r = oracle.gjk_distance(cs, i1, i2, nthreads=nthreads)
    hit = np.flatnonzero((r["dist"] == 0.0) & (r["n_simplex"] == 4))
    oracle.epa(cs, i1[hit], i2[hit], r["simplex"][hit], nthreads=nthreads, **EPA_KW)
    return len(i1)


def time_cpu(cs, i1, i2, seconds):
    """Pairs/s of the oracle on all host cores over at least `seconds` (or
    one full pass), after one warm pass on a slice."""
    from oracle import oracle
    cpu_oracle_pass(cs, i1[:20000], i2[:20000])
    done, t0 = 0, time.perf_counter()
    while True:
        done += cpu_oracle_pass(cs, i1, i2)
        el = time.perf_counter() - t0
        if el >= seconds or done >= 20 * len(i1):
            break
    return done / el, oracle.max_threads(), done, el


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cs, i1, i2 = make_workload(args.pairs, 0)
    from oracle import oracle
    for _ in range(args.warmup):
        cpu_oracle_pass(cs, i1[:50000], i2[:50000])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_oracle_pass(cs, i1, i2)
    el = time.perf_counter() - t0
    value = args.steps * len(i1) / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": f"{len(i1):,} six-type pairs, GJK distance + EPA (256 faces) on intersecting pairs",
                   "pairs": len(i1)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.max_threads(), "kind": "port",
                         "sample": f"{args.steps} full passes over {len(i1)} pairs"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def serve_report(store, i1_np, i2_np, seconds, seed=7, capacity=8192, slots=8, repeats=3):
    """The continuous-batching server (the library's native server) on the
    same resident store: peak pairs/s with a burst of requests all arriving
    at once, then Poisson arrivals at 50/80/100% of that peak; latency from
    each request's arrival to its results in host memory, p50/p99.  Each
    load level runs `repeats` times (fresh arrivals each time); the run with
    the median p99 is reported, with every run's p99 beside it.  Mixed and
    plain FP64 form.  Requests: lognormal pair counts (median 2,000, clipped
    to [1, 50,000]) of pairs drawn from the batched workload."""
    from distance3d_gb300.serve import NativeCollisionServer, request_sizes
    from distance3d_gb300.tune import autotune, get_tuning, set_tuning
    rng = np.random.default_rng(seed)
    mean_size = float(request_sizes(np.random.default_rng(seed + 1), 200000).mean())
    # the launch parameters for the server's saturated regime, every slot's
    # batch in flight: tuned on capacity * slots pairs (restored after)
    before = get_tuning()
    tuned = autotune(store, i1_np[:capacity * slots], i2_np[:capacity * slots], epa_kw=EPA_KW)

    def trace(count):
        sizes = request_sizes(rng, count)
        sel = rng.integers(0, len(i1_np), int(sizes.sum()))
        return sizes, i1_np[sel], i2_np[sel]

    out = {"request_pairs": {"median": 2000, "clip": [1, 50000], "mean": mean_size},
           "latency": "arrival to results in host memory", "server": "native (d3d_server), CUDA graphs",
           "capacity": capacity, "slots": slots, "tuning": tuned}
    for precision in ("mixed", "fp64"):
        srv = NativeCollisionServer(store, capacity=capacity, slots=slots, precision=precision, epa_kw=EPA_KW)
        try:
            sz, a, b = trace(20)
            srv.replay(sz, a, b, np.zeros(len(sz)))
            sz, a, b = trace(600 if precision == "mixed" else 60)
            lat, span = srv.replay(sz, a, b, np.zeros(len(sz)))
            peak = float(sz.sum()) / span
            res = {"peak_pairs_per_s": peak}
            for load in (0.5, 0.8, 1.0):
                rate = load * peak / mean_size
                count = max(20, int(rate * seconds))
                runs = []
                for _ in range(repeats):
                    sz, a, b = trace(count)
                    offsets = np.cumsum(rng.exponential(1.0 / rate, count))
                    lat, span = srv.replay(sz, a, b, offsets)
                    runs.append((float(np.percentile(lat, 50) * 1e3), float(np.percentile(lat, 99) * 1e3),
                                 float(lat.max() * 1e3), float(sz.sum()) / span))
                med = sorted(runs, key=lambda r: r[1])[len(runs) // 2]  # the run with the median p99
                res[f"load_{int(load * 100)}"] = {
                    "offered_pairs_per_s": load * peak, "p50_ms": med[0], "p99_ms": med[1], "max_ms": med[2],
                    "served_pairs_per_s": med[3], "requests": count,
                    "p99_ms_per_run": [r[1] for r in runs]}
        finally:
            srv.close()
        out[precision] = res
    set_tuning(**before)
    return out


def broad_narrow_report(dev, n_colliders=131072, seed=3, reps=3):
    """The broad+narrow workload: n colliders of the six types in
    [-20,20]^3, FP64 AABBs, LBVH build, self-overlap query, then GJK + EPA on
    the overlapping pairs (distance3d_gb300.pipeline.collide_scene).  Device
    milliseconds per stage, best of `reps` after one warm-up, both forms."""
    from distance3d_gb300 import workloads
    from distance3d_gb300.pipeline import collide_scene
    from distance3d_gb300.store import ColliderStore
    cs = workloads.scene_mixed_six(n_colliders, seed=seed)
    st = ColliderStore(cs, device=dev)
    out = {"colliders": n_colliders, "box_half_width": 20.0, "seed": seed}
    for precision in ("mixed", "fp64"):
        collide_scene(st, precision=precision, epa_kw=EPA_KW)
        best = None
        for _ in range(reps):
            pairs, r, t = collide_scene(st, precision=precision, epa_kw=EPA_KW, timings=True)
            if best is None or sum(t.values()) < sum(best.values()):
                best = t
        total = sum(best.values())
        out[precision] = {"ms": total, "stages_ms": best, "pairs": int(pairs.shape[0]),
                          "epa_pairs": int((r["epa_status"] >= 0).sum().item()),
                          "scenes_per_s": 1e3 / total, "narrow_pairs_per_s": pairs.shape[0] / best["gjk_epa"] * 1e3}
    return out


def robot_report(dev, n_configs=16384, seed=0, reps=3):
    """Robot self-collision batch: n_configs joint configurations of a
    synthetic 7-DoF arm (link lengths U[0.1,0.4] m, joint values
    U[-pi,pi]) with 30 bodies (capsules r 0.04-0.08, boxes, cylinders);
    every body pair on non-adjacent links tested per configuration
    (forward kinematics, pose update, GJK + EPA in one CUDA graph).  Device
    time per batch, best of `reps` after a warm-up, both forms; contact flags
    compared between the forms."""
    import torch
    from distance3d_gb300.robot import SelfCollisionBatch, SerialArm
    arm = SerialArm.synthetic(seed=seed)
    q = torch.as_tensor(np.random.default_rng(seed + 1).uniform(-np.pi, np.pi, (n_configs, arm.dof)),
                        dtype=torch.float64, device=dev)
    out = {"configs": n_configs, "dof": arm.dof, "bodies": arm.n_bodies,
           "pairs_per_config": int(len(arm.pair_table())), "seed": seed}
    res = {}
    for precision in ("mixed", "fp64"):
        b = SelfCollisionBatch(arm, n_configs, precision=precision, graph=True, device=dev)
        b.run(q)
        stream = torch.cuda.current_stream(dev)
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = b.run(q, sync=False)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        res[precision] = {k: v.clone() for k, v in r.items()}
        out[precision] = {"ms_per_batch": best, "configs_per_s": n_configs / best * 1e3,
                          "pairs_per_s": b.n_pairs / best * 1e3,
                          "configs_in_collision": float(r["any"].float().mean().item())}
        del b
    df, dm = res["fp64"]["dist"], res["mixed"]["dist"]
    sep = df > 1e-6
    out["contact_flags_identical_beyond_1e-6"] = bool(torch.equal(dm[sep] > 0, df[sep] > 0))
    out["max_rel_dist_err"] = float(((dm - df).abs() / df.clamp(min=1.0)).max().item())
    out["mixed_over_fp64"] = out["fp64"]["ms_per_batch"] / out["mixed"]["ms_per_batch"]
    return out


def mpr_report(store, cs, i1_np, i2_np, dev, reps=3, check_pairs=20000, cpu_pairs=262144, cpu=True):
    """MPR on the batched workload: device time for all pairs (best of `reps`
    after a warm-up), both forms (plain FP64, the reference bit for bit; mixed)
    and both calls (mpr_penetration, mpr_intersection); the oracle (C
    restatement, all host threads) on a sample; a bit-exact check of the FP64
    form against the oracle on a sample; the mixed form's flags and depths
    against the FP64 form on all pairs."""
    import time
    import torch
    from distance3d_gb300.mpr import mpr_batch
    from oracle import oracle
    i1 = torch.as_tensor(i1_np, device=dev)
    i2 = torch.as_tensor(i2_np, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {"pairs": len(i1_np), "tolerance": 1e-4, "max_iterations": 100}
    res = {}
    for precision in ("fp64", "mixed"):
        out[precision] = {}
        for name, pen in (("penetration", True), ("intersection", False)):
            r = mpr_batch(store, i1, i2, penetration=pen, precision=precision)
            best = None
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r = mpr_batch(store, i1, i2, penetration=pen, precision=precision)
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            out[precision][name] = {"ms": best, "pairs_per_s": len(i1_np) / best * 1e3,
                                    "intersecting_fraction": float(r["hit"].float().mean().item())}
            if pen:
                res[precision] = {k: v.cpu().numpy() for k, v in r.items()}
    out["mixed_over_fp64"] = out["fp64"]["penetration"]["ms"] / out["mixed"]["penetration"]["ms"]
    f, m = res["fp64"], res["mixed"]
    both = f["hit"] & m["hit"]
    err = np.abs(m["depth"][both] - f["depth"][both]) / np.maximum(1.0, f["depth"][both])
    # where the flags differ: how far each pair is from touching (FP64 GJK
    # separation, FP64 EPA depth), and which form agrees with GJK there
    from distance3d_gb300.epa import epa_batch
    from distance3d_gb300.gjk import gjk_distance_batch
    diff = np.flatnonzero(f["hit"] != m["hit"]).astype(np.int32)
    mixed_wrong_margin, mixed_right, fp64_right = 0.0, 0, 0
    if len(diff):
        g = {k: v.cpu().numpy() for k, v in gjk_distance_batch(store, i1_np[diff], i2_np[diff]).items()}
        margin = np.where(g["dist"] > 0.0, g["dist"], 0.0)
        full = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
        if len(full):
            e = {k: v.cpu().numpy() for k, v in epa_batch(store, i1_np[diff][full], i2_np[diff][full],
                                                             g["simplex"][full], **EPA_KW).items()}
            ok = e["status"] == 0
            margin[full[ok]] = np.linalg.norm(e["mtv"][ok], axis=1)
        gjk_hit = g["dist"] == 0.0
        mixed_ok = m["hit"][diff] == gjk_hit
        mixed_right, fp64_right = int(mixed_ok.sum()), int((f["hit"][diff] == gjk_hit).sum())
        if (~mixed_ok).any():
            mixed_wrong_margin = float(margin[~mixed_ok].max())
    out["mixed_accuracy"] = {
        "flags_differ": int(len(diff)),
        "flags_differ_mixed_agrees_with_gjk": mixed_right,
        "flags_differ_fp64_agrees_with_gjk": fp64_right,
        "flags_differ_mixed_wrong_max_distance_from_touching": mixed_wrong_margin,
        "depth_rel_err_frac_above_1e-5": float(np.mean(err > 1e-5)),
        "depth_rel_err_p99": float(np.quantile(err, 0.99)),
        "depth_rel_err_p999": float(np.quantile(err, 0.999)),
        "note": "MPR's flag is defined up to its tolerance (1e-4): within it, a pair is a hit if the "
                "portal can still expand by more than the tolerance; MPR's depth depends on the final "
                "portal face: moving every collider by 1e-9 changes the FP64 depth by >1e-5 on ~2% "
                "of pairs (tests/test_mpr_gpu.py)"}
    k = np.arange(check_pairs)
    got = {key: v[:check_pairs].cpu().numpy() for key, v in mpr_batch(store, i1[:check_pairs], i2[:check_pairs]).items()}
    ref = oracle.mpr(cs, i1_np[k], i2_np[k])
    out["fp64_bit_exact_vs_oracle_sample"] = bool(
        np.array_equal(got["hit"], ref["hit"]) and np.array_equal(got["status"], ref["status"])
        and all(np.array_equal(got[key], ref[key], equal_nan=True) for key in ("depth", "dir", "pos")))
    out["check_pairs"] = check_pairs
    if not cpu:
        return out
    t0 = time.perf_counter()
    oracle.mpr(cs, i1_np[:cpu_pairs], i2_np[:cpu_pairs])
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"pairs_per_s": cpu_pairs / cpu_s, "cores": oracle.max_threads(), "kind": "port",
                           "sample": f"{cpu_pairs} pairs, mpr_penetration, C restatement with OpenMP"}
    return out


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from distance3d_gb300 import _lib
    from distance3d_gb300.store import ColliderStore, PinnedColliderSet
    from distance3d_gb300.gjk import gjk_distance_batch
    from distance3d_gb300.epa import epa_batch, epa_scratch_bytes

    _lib.load()
    cs, i1_np, i2_np = make_workload(args.pairs, rank)
    n = len(i1_np)
    store = ColliderStore(cs, device=dev)
    if args.mpr_only:
        if rank == 0:
            print(json.dumps({"mpr": mpr_report(store, cs, i1_np, i2_np, dev, reps=max(1, args.steps),
                                                check_pairs=min(n, 20000), cpu=False)}), flush=True)
        return 0
    i1 = torch.as_tensor(i1_np, device=dev)
    i2 = torch.as_tensor(i2_np, device=dev)
    stream = torch.cuda.current_stream(dev)
    scratch = torch.empty(max(epa_scratch_bytes(n, precision=p, **EPA_KW) for p in ("fp64", "mixed")),
                          dtype=torch.uint8, device=dev)

    def step(precision, ev=None):
        if ev is not None:
            ev[0].record(stream)
        g = gjk_distance_batch(store, i1, i2, precision=precision)
        if ev is not None:
            ev[1].record(stream)
        hit = torch.nonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4)).flatten()
        if ev is not None:
            ev[2].record(stream)
        e = epa_batch(store, i1[hit], i2[hit], g["simplex"][hit], scratch=scratch, precision=precision, **EPA_KW)
        if ev is not None:
            ev[3].record(stream)
        return g, hit, e

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def timed(precision):
        for _ in range(args.warmup):
            step(precision)
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
        barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        out = None
        for k in range(args.steps):
            out = step(precision, evs[k])
        end.record(stream)
        barrier()
        total = start.elapsed_time(end) / 1e3
        gjk = float(np.mean([e[0].elapsed_time(e[1]) for e in evs])) / 1e3
        epa = float(np.mean([e[2].elapsed_time(e[3]) for e in evs])) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        return total, gjk, epa, out

    # the batched form: the autotuner picks the launch parameters on a sample,
    # then one CUDA graph of d3d_collide (GJK, device-side EPA pair selection,
    # EPA) per precision is replayed per step, inputs resident
    from distance3d_gb300.serve import CollisionBatch
    from distance3d_gb300.tune import autotune
    from distance3d_gb300.tune import get_tuning
    # on the workload itself, outside the timed region
    tuned = get_tuning() if args.no_tune else autotune(store, i1, i2, epa_kw=EPA_KW)
    batches = {}
    for precision in ("mixed", "fp64"):
        b = CollisionBatch(store, n, precision=precision, epa_kw=EPA_KW, graphs=False, classes=[n])
        b.i1.copy_(i1)
        b.i2.copy_(i2)
        b.n_dev.fill_(n)
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(b.stream):
            b._launch(n)  # first use, outside the capture
        b.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=b.stream):
            b._launch(n)
        batches[precision] = (b, g)

    def graph_timed(precision):
        b, g = batches[precision]
        for _ in range(args.warmup):
            g.replay()
        barrier()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            g.replay()
        end.record(stream)
        barrier()
        total = start.elapsed_time(end) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total = float(t.item())
        o = b.out
        hit = torch.nonzero(o["epa_status"] >= 0).flatten()
        return total, (o, hit, {"mtv": o["mtv"][hit], "status": o["epa_status"][hit]})

    with ClockSampler(local) as clocks:
        t_mixed, out_mixed = graph_timed("mixed")
    t_fp64, out_fp64 = graph_timed("fp64")
    # per-phase split (GJK / EPA) of each form from the separate-call path, one
    # extra timed pass each (not the headline)
    _, gjk_mixed, epa_mixed, _ = timed("mixed")
    _, gjk_fp64, epa_fp64, _ = timed("fp64")

    # accuracy of the mixed form against the FP64 form (which equals the
    # reference bit for bit); see accuracy_report
    acc = accuracy_report(store, i1, i2, out_mixed, out_fp64, dev)
    gm, hm, em = out_mixed
    n_epa = int(hm.numel())

    # end to end through the public API from pinned host buffers: every step
    # copies its colliders to the device and packs them into a resident store
    # (ColliderStore.update), copies its pairs in, runs GJK and EPA as one
    # CUDA graph of d3d_collide and copies every result back
    # (CollisionBatch.submit).  Consecutive steps alternate between two such
    # lanes (store, batch, stream), so that one step's copies overlap the
    # previous step's kernels, as a pipelined caller would.
    from distance3d_gb300.serve import CollisionBatch
    pinned = PinnedColliderSet(cs)
    lanes = []
    for _ in range(2):
        st_l = ColliderStore(pinned, device=dev)
        lanes.append(CollisionBatch(st_l, n, precision="mixed", epa_kw=EPA_KW, graphs=True))
    torch.cuda.synchronize(dev)

    def e2e_step(k):
        b = lanes[k % 2]
        with torch.cuda.stream(b.stream):
            b.store.update(pinned)
            b.submit(i1_np, i2_np)
        return sum(v[:n].numel() * v.element_size() for v in b.h_out.values())

    for k in range(args.warmup):
        e2e_step(k)
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        d2h = e2e_step(k)
    barrier()
    t_e2e = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([t_e2e], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(t.item())
    h2d = pinned.nbytes() + n * 4 * 2 + 8
    del lanes

    value = world * n * args.steps / t_mixed
    fp64_value = world * n * args.steps / t_fp64
    e2e_value = world * n * args.steps / t_e2e

    # compute roofline of the plain FP64 GJK kernel (one kernel per call):
    # model FLOPs from its exact iteration counts / event-timed duration,
    # against the measured FP64 FMA peak
    peak64, peak32 = measure_pipe_peaks(dev)
    gf = out_fp64[0]
    flops64 = gjk_model_flops(cs, i1_np, i2_np, gf["iterations"].cpu().numpy())
    compute_roofline = {"kernel": "k_gjk_distance_f64", "bound": "fp64 pipe",
                        "model_flops_per_launch": flops64, "achieved_tflops": flops64 / gjk_fp64 / 1e12,
                        "peak_tflops": peak64 / 1e12, "frac": flops64 / gjk_fp64 / peak64,
                        "peak_source": "measured in this run (FMA chains, libd3d_peak)",
                        "fp32_peak_tflops": peak32 / 1e12}

    # roofline: the dominant kernel of the mixed step
    gjk_bytes = algorithmic_bytes(cs, i1_np, 0, "mixed") - OUT_EPA * 0
    epa_bytes = n_epa * (2 * REC64 + OUT_EPA + 96)
    if gjk_mixed >= epa_mixed:
        dom, t_dom, bytes_dom = ("d3d_gjk_distance mixed (k_gjk_mixed_a, k_gjk_mixed_b, k_gjk_mixed_end)", gjk_mixed,
                                 gjk_bytes)
        traffic = NCU_DRAM_BYTES_PER_PAIR["gjk_mixed"] * n
    else:
        dom, t_dom, bytes_dom = "d3d_epa mixed (k_epa_warp, k_epa_refine)", epa_mixed, epa_bytes
        traffic = NCU_DRAM_BYTES_PER_PAIR["epa_mixed"] * n_epa
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bytes_dom / t_dom / 1e9

    line = None
    if rank == 0:
        serve = serve_report(store, i1_np, i2_np, args.serve_seconds) if args.serve_seconds > 0 else None
        broad = None if args.no_extras else broad_narrow_report(dev)
        robot = None if args.no_extras else robot_report(dev)
        mpr = None if args.no_extras else mpr_report(store, cs, i1_np, i2_np, dev)
        cpu_value, cores, cpu_pairs, cpu_s = time_cpu(cs, i1_np, i2_np, args.cpu_seconds)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_mixed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{n:,} six-type pairs, GJK distance + EPA (256 faces) on "
                                   "intersecting pairs, centers in [-0.38,0.38]^3",
                       "pairs_per_gpu": n, "intersecting_fraction": n_epa / n, "epa_pairs": n_epa,
                       "l2": "inputs 1.6 GB > L2, no flush", "parallelism": f"replicas x{world}"},
            "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": 1e3 * t_fp64 / args.steps,
                     "gjk_ms": 1e3 * gjk_fp64, "epa_ms": 1e3 * epa_fp64},
            "mixed_over_fp64": value / fp64_value,
            "kernels_ms": {"gjk_mixed": 1e3 * gjk_mixed, "epa": 1e3 * epa_mixed,
                           "gjk_fp64": 1e3 * gjk_fp64},
            "accuracy": acc,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum at 131,072 pairs, "
                                           "scaled by the pair count",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback"},
            "compute_roofline": compute_roofline,
            "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{cpu_pairs} pairs ({cpu_s:.1f} s) of the same workload, "
                                       "GJK + EPA, C restatement with OpenMP"},
            "serve": serve,
            "broad_narrow": broad,
            "robot_self_collision": robot,
            "mpr": mpr,
            "tuning": tuned,
            "step": "one CUDA-graph replay of d3d_collide (GJK, EPA pair selection, EPA) over all pairs",
            "gpu_launches": MIXED_STEP_LAUNCHES * args.steps,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
