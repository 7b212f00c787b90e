#!/usr/bin/env python3
"""Keyframes/s of the SLOAM keyframe hot path on GB300.

Workload (one step): a batch of 64 synthetic 64x2048 keyframes (16 distinct
scans; float32 XYZI, ~131k points each; 150 trunks with radius U(0.08, 0.6)
m, shrubs, 10% outliers; per-point labels from the generator), each run
through projection, Trellis, ground planes, the cylinder fits, association
against a 400-landmark submap and 10 Gauss-Newton pose iterations (FP32
residuals, FP64 6x6 solve).  `value` is the learned-proposal path (8 network
proposals per tree + 3 LS iterations, RANSAC fallback); `plain` the
256-hypothesis point RANSAC + 3 LS; `reference_algorithm` the reference's own
vertex-line RANSAC (cyl_mode 0) on the GPU.  Inputs are device-resident for
these; `e2e` runs the learned path through the host C ABI
(sloam_keyframes_host) from pinned host buffers.  L2 is flushed (256 MB
write) before every timed step.

`roofline` is the batch projection stage (k_project, k_label_batch,
k_compact_batch over the step's 64 keyframes per launch group), timed with
CUDA events on its streams inside the timed steps: 26 algorithmic bytes per point (16 B XYZI +
1 B label read, 4 B pixel index + 4 B range + 1 B mask written).  `kernels`
holds the kernels that decide keyframes/s, each timed alone with CUDA events
against the roof that binds it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's algorithm (vertex-line RANSAC) in its
CPU implementation (the std-only restatement in oracle/: the reference itself
cannot be built here) on all host cores, one keyframe per thread, over the
same 16 distinct scans.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

# Up to 32 hardware work queues instead of 8, so that the keyframe slots'
# streams do not alias onto shared queues (read when CUDA initialises).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "keyframes/s at 64\u00d72048: learned-proposal vs plain RANSAC, equal cylinder error"
UNIT = "keyframes/s"
WORKLOAD = ("C2: 64x2048 keyframes, 150 trees, 400-landmark submap, 10 GN iterations; value: "
            "learned proposals (8 per tree, tensor-core network, RANSAC fallback below 0.6 "
            "inlier ratio) + 3 LS; plain: 256 RANSAC hypotheses per tree + 3 LS")
# DRAM bytes (read + write) per keyframe of the batch projection stage, summed
# over its three kernels in one ncu capture with the caches left as they are
# (dram__bytes_read.sum + dram__bytes_write.sum of one 64-keyframe launch
# group: 478 MB).
FRONT_TRAFFIC_PER_KF = 7.47e6


def max_over_ranks(x, device=None):
    """The maximum of x over the ranks of the job (the slowest rank's time is
    the job's time); x itself without a process group."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()):
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def job_value(batch, steps, world, total_ms):
    """Whole-job keyframes/s: every rank processed batch * steps keyframes."""
    return batch * steps * world / (total_ms / 1000.0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--distinct", type=int, default=16)
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="end-to-end steps (0: the same as --steps)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--extra", type=int, default=1,
                    help="also measure the C1 and C3 workloads and the kernels alone")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--slots", type=int, default=32,
                    help="keyframes in flight at once (context batch slots)")
    return ap.parse_args()


def workload(seed, distinct):
    from sloam_gb300 import synth
    cfg = synth.C2
    forest, kfs = synth.scene(cfg, seed=seed, n_kf=distinct)
    P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, cyl_hypotheses=256,
                            cyl_ls_iters=3, gn_iters=10)
    return cfg, forest, kfs, P


# ------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU legs
def cpu_run_keyframes(P, forest, kfs, seconds, threads=1, min_kf=2):
    """The oracle (the reference algorithm's std-only restatement) on host
    threads, one independent keyframe at a time per thread; returns kf/s."""
    from oracle import loader
    from sloam_gb300 import capi as A
    L = loader.lib()
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    counts = [0] * threads
    stop = [False]

    def worker(t):
        s = L.oracle_create(C.byref(P))
        kf0 = kfs[0]
        r = A.RunBuffers(P)
        L.oracle_keyframe(s, A.ptr(kf0.xyzi, C.c_float), len(kf0.xyzi),
                          A.ptr(kf0.labels, C.c_uint8), None,
                          C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc, nm, C.byref(r.s))
        k = 0
        while not stop[0] or counts[t] < min_kf:
            kf = kfs[1 + (t + k) % (len(kfs) - 1)]
            r = A.RunBuffers(P)
            L.oracle_keyframe(s, A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                              A.ptr(kf.labels, C.c_uint8), None,
                              C.byref(A.SE3.from_qt(*kf.pose_est_qt())), mapc, nm, C.byref(r.s))
            counts[t] += 1
            k += 1
        L.oracle_destroy(s)

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    time.sleep(seconds)
    stop[0] = True
    for th in ths:
        th.join()
    dt = time.perf_counter() - t0
    return sum(counts) / dt, sum(counts), dt


def glibc_pixel_differences(P, kfs):
    """Per keyframe: points whose pixel differs between the projection
    contract (correctly rounded atan2f/asinf, which the GPU reproduces) and
    the literal host-libm expression the reference compiles to."""
    import numpy as np
    from oracle import loader
    from sloam_gb300 import capi as A
    L = loader.lib()
    n = P.img_w * P.img_h
    out = []
    for kf in kfs:
        res = []
        for variant in (0, 1):
            px = np.zeros(n, np.int32)
            py = np.zeros(n, np.int32)
            rng = np.zeros(n, np.float32)
            msk = np.zeros(n, np.uint8)
            gidx = np.zeros(n, np.int32)
            tree = np.zeros((n, 4), np.float32)
            so = A.ScanOut()
            so.px, so.py = A.ptr(px, C.c_int32), A.ptr(py, C.c_int32)
            so.range_image, so.mask_out = A.ptr(rng, C.c_float), A.ptr(msk, C.c_uint8)
            so.ground_idx, so.tree_cloud = A.ptr(gidx, C.c_int32), A.ptr(tree, C.c_float)
            L.oracle_project_mask(C.byref(P), A.ptr(kf.xyzi, C.c_float), n,
                                  A.ptr(kf.labels, C.c_uint8), None, variant, C.byref(so))
            res.append((px, py))
        (a, b), (c, d) = res
        out.append(int(((a != c) | (b != d)).sum()))
    return out


def run_reference(args):
    """The reference's algorithm on the CPU: the oracle in the reference's
    cylinder mode (vertex-line RANSAC, cylinder.cpp:115-139), every host
    thread running keyframes of the same 16 distinct scans as the GPU arm,
    one keyframe per thread per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg, forest, kfs, P = workload(args.seed, args.distinct)
    P.cyl_mode = 0
    threads = os.cpu_count() or 1
    from oracle import loader
    from sloam_gb300 import capi as A
    L = loader.lib()
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    states = []
    for t in range(threads):
        s = L.oracle_create(C.byref(P))
        kf0 = kfs[0]
        r = A.RunBuffers(P)
        L.oracle_keyframe(s, A.ptr(kf0.xyzi, C.c_float), len(kf0.xyzi),
                          A.ptr(kf0.labels, C.c_uint8), None,
                          C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc, nm, C.byref(r.s))
        states.append(s)

    def one(t, step):
        kf = kfs[(t * args.steps + step) % len(kfs)]
        r = A.RunBuffers(P)
        L.oracle_keyframe(states[t], A.ptr(kf.xyzi, C.c_float), len(kf.xyzi),
                          A.ptr(kf.labels, C.c_uint8), None,
                          C.byref(A.SE3.from_qt(*kf.pose_est_qt())), mapc, nm, C.byref(r.s))

    from concurrent.futures import ThreadPoolExecutor
    ex = ThreadPoolExecutor(threads)

    def step(s):
        list(ex.map(lambda t: one(t, s), range(threads)))

    for s in range(args.warmup):
        step(s)
    t0 = time.perf_counter()
    for s in range(args.steps):
        step(s)
    dt = time.perf_counter() - t0
    for s in states:
        L.oracle_destroy(s)
    v = threads * args.steps / dt
    sample = (f"{threads} keyframes per step (one per host thread) of the 16 distinct 64x2048 "
              "scans, the reference's algorithm (vertex-line cylinder RANSAC, cyl_mode 0) in the "
              "oracle restatement")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": config_block(args, 1), "threads": threads,
        "algorithm": "the reference's vertex-line cylinder RANSAC (cyl_mode 0)",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def config_block(args, world):
    """The workload's description; the same in both arms."""
    return {"workload": WORKLOAD, "batch_keyframes": args.batch,
            "distinct_scans": args.distinct,
            "l2": "flushed (256 MB write) before every timed step",
            "parallelism": f"replicas x{world}"}


# -------------------------------------------------------------- GPU leg
def measure(args, L, A, P, forest, kfs, dev, world, mode, weights, batch=None):
    """One context in cylinder mode `mode` (0 the reference's vertex-line
    RANSAC, 1 plain point RANSAC, 2 learned proposals): the first scan, W
    warm-up and K timed batch steps."""
    import torch
    from sloam_gb300.lib import Context
    Pm = P.copy()
    Pm.cyl_mode = mode
    ctx = Context(Pm, device=dev.index or 0)
    if mode == 2:
        ctx.set_proposal_weights(weights)
    mapc = A.cylinders_from_array(forest.map_cylinders())
    nm = len(forest.radius)
    N = Pm.img_w * Pm.img_h
    B = args.batch if batch is None else batch
    kf0 = kfs[0]
    r = A.RunBuffers(Pm)
    ctx.check(L.sloam_keyframe(ctx.h, A.ptr(kf0.xyzi, C.c_float), N, A.ptr(kf0.labels, C.c_uint8),
                               None, C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc, nm,
                               C.byref(r.s)))
    order = [i % len(kfs) for i in range(B)]
    X = torch.from_numpy(np.stack([kfs[i].xyzi for i in order])).to(dev)
    Lb = torch.from_numpy(np.stack([kfs[i].labels for i in order])).to(dev)
    Mp = torch.from_numpy(np.frombuffer(bytes(mapc), np.uint8).copy()).to(dev)
    poses = (A.SE3 * B)(*[A.SE3.from_qt(*kfs[i].pose_est_qt()) for i in order])
    pose_out = torch.zeros(B * 7, dtype=torch.float64, device=dev)
    succ = torch.zeros(B, dtype=torch.int32, device=dev)
    ncyl = torch.zeros(B, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)

    def step():
        ctx.check(L.sloam_keyframes_device(ctx.h, X.data_ptr(), N, B, Lb.data_ptr(), poses,
                                           Mp.data_ptr(), nm, pose_out.data_ptr(),
                                           succ.data_ptr(), ncyl.data_ptr()))
        return ctx.launches()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
    torch.cuda.synchronize()
    evs, launches = [], 0
    fe_ms, fe_launches, fe_kf = 0.0, 0, 0
    host_s = 0.0  # host time to enqueue a step (the call returns before the GPU is done)
    for s in range(args.steps):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        h0 = time.perf_counter()
        launches += step()
        host_s += time.perf_counter() - h0
        e1.record(ext)
        evs.append((e0, e1))
        # the batch projection launches of this step (events on their stream)
        ms, nch, nkf = C.c_float(), C.c_int32(), C.c_int32()
        ctx.check(L.sloam_frontend_time(ctx.h, C.byref(ms), C.byref(nch), C.byref(nkf)))
        fe_ms += ms.value
        fe_launches += nch.value
        fe_kf += nkf.value
    torch.cuda.synchronize()
    if world > 1:
        tdist.barrier()
    total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), dev)
    return dict(ctx=ctx, P=Pm, X=X, Lb=Lb, poses=poses, mapc=mapc, nm=nm, N=N, B=B,
                value=job_value(B, args.steps, world, total_ms), total_ms=total_ms,
                launches=launches, fe=(fe_ms, fe_launches, fe_kf), host_s=host_s,
                ok=int(succ.sum().item()), ncyl=float(ncyl.float().mean().item()))


def accuracy(L, A, m, forest, kfs):
    """Median axis / radius error of the fitted cylinders against the
    generator's trunks over the distinct keyframes, the trees at each stage
    and the trees that fell back to RANSAC.  Each keyframe runs as in the
    batch: after the first scan (keyframe 0 at its true pose), at its
    perturbed estimate."""
    from sloam_gb300 import synth
    ctx, P = m["ctx"], m["P"]
    angs, rerrs, fb, nl, slow, nlm, nfit = [], [], 0, 0, 0, 0, 0
    stats = (C.c_int32 * 6)()
    kf0 = kfs[0]
    for kf in kfs[1:]:
        ctx.check(L.sloam_reset(ctx.h))
        r0 = A.RunBuffers(P)
        ctx.check(L.sloam_keyframe(ctx.h, A.ptr(kf0.xyzi, C.c_float), m["N"],
                                   A.ptr(kf0.labels, C.c_uint8), None,
                                   C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), m["mapc"], m["nm"],
                                   C.byref(r0.s)))
        r = A.RunBuffers(P)
        st = L.sloam_keyframe(ctx.h, A.ptr(kf.xyzi, C.c_float), m["N"],
                              A.ptr(kf.labels, C.c_uint8), None,
                              C.byref(A.SE3.from_qt(*kf.pose_est_qt())), m["mapc"], m["nm"],
                              C.byref(r.s))
        if st not in (0, A.SLOAM_ERR_NOT_CONVERGED):
            ctx.check(st)
        r.refresh()
        a, e = synth.cylinder_errors(forest, r.m.cyl_array())
        angs.append(a)
        rerrs.append(e)
        L.sloam_keyframe_stats(ctx.h, stats, 6)
        nlm += stats[0]
        nl += stats[1]
        fb += stats[3]
        slow += stats[4]
        nfit += stats[5]
    a, e = np.concatenate(angs), np.concatenate(rerrs)
    k = max(len(kfs) - 1, 1)
    return {"median_axis_deg": float(np.median(a)), "median_radius_cm": float(100 * np.median(e)),
            "cylinders_matched": int(len(a)), "keyframes": len(kfs) - 1,
            "fallback_trees": int(fb), "valid_cylinders": int(nl),
            "trees_per_keyframe": {"trunks_in_scene": 150, "trellis_landmarks": nlm / k,
                                   "point_fit": nfit / k, "valid_cylinders": nl / k},
            "fp64_projection_points_per_keyframe": slow / k}


def time_kernel(L, m, which, reps=20):
    ms = C.c_float()
    m["ctx"].check(L.sloam_time_kernel(m["ctx"].h, which, reps, C.byref(ms)))
    return ms.value


def extra_workload(args, L, A, dev, world, name, weights):
    """keyframes/s of the 16x1024 keyframe (C1: 20 trunks, 64 hypotheses;
    64-keyframe batches of 16 distinct scans) or of the uneven batch (C3: 64
    keyframes of 64x2048 with 20-400 trees each, clusters up to ~20k points),
    plain point RANSAC and learned proposals, device-resident, L2 flushed."""
    from sloam_gb300 import synth
    if name == "c1":
        cfg = synth.C1
        forest, kfs = synth.scene(cfg, seed=args.seed, n_kf=16)
        P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, cyl_hypotheses=64,
                                cyl_ls_iters=3, gn_iters=10)
        P.batch_slots = args.slots
        batch = args.batch
    else:
        forest, kfs, counts = synth.c3_scene(args.seed, n_kf=64)
        P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
        P.batch_slots = args.slots
        batch = len(kfs)
    tuning = None
    if name == "c3":
        import torch
        from sloam_gb300 import autotune
        tuning = autotune.apply(P, torch.cuda.get_device_name(dev), "c3")
    out = {}
    for mode in (1, 2):
        m = measure(args, L, A, P, forest, kfs, dev, world, mode, weights, batch=batch)
        out["plain" if mode == 1 else "learned"] = m["value"]
        m["ctx"].close()
    if tuning is not None:
        out["tuning"] = tuning
    return out


def main():
    args = parse()
    if args.e2e_steps <= 0:
        args.e2e_steps = args.steps
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    from sloam_gb300 import autotune, build, capi as A, proposal
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    if rank == 0:
        build.build()
    if dist:
        tdist.barrier()
    from sloam_gb300.lib import load
    L = load()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    cfg, forest, kfs, P = workload(args.seed + rank, args.distinct)
    P.batch_slots = args.slots
    tuning = autotune.apply(P, torch.cuda.get_device_name(dev), "c2")
    weights = proposal.load_weights()
    clocks = Clocks(local)
    clocks.start()
    learned = measure(args, L, A, P, forest, kfs, dev, world, 2, weights)
    plain = measure(args, L, A, P, forest, kfs, dev, world, 1, weights)
    refalg = measure(args, L, A, P, forest, kfs, dev, world, 0, weights)
    ck = clocks.stop()
    ctx = learned["ctx"]
    N, B, mapc, nm = learned["N"], learned["B"], learned["mapc"], learned["nm"]

    acc_l = accuracy(L, A, learned, forest, kfs)
    acc_p = accuracy(L, A, plain, forest, kfs)
    # per-stage breakdown of one keyframe, and kernels alone, over the last
    # keyframe each context ran
    stages = (C.c_float * 4)()
    L.sloam_profile_stages(ctx.h, stages, 4)
    stats = (C.c_int32 * 6)()
    L.sloam_keyframe_stats(ctx.h, stats, 6)
    net_samples = stats[0] * learned["P"].prop_samples
    k_ms = {"k_prop_infer_tc": time_kernel(L, learned, 2),
            "k_project": time_kernel(L, learned, 0),
            "cylinder_stage_learned": time_kernel(L, learned, 3),
            "cylinder_stage_plain": time_kernel(L, plain, 3),
            "cylinder_stage_reference_algorithm": time_kernel(L, refalg, 3),
            "k_cyl_queue_plain": time_kernel(L, plain, 6),
            "k_vertex": time_kernel(L, plain, 4),
            "k_gn": time_kernel(L, plain, 5)}
    pstats = (C.c_int32 * 9)()
    L.sloam_keyframe_stats(plain["ctx"].h, pstats, 9)

    # ---- e2e: the same keyframes through the host C ABI from pinned host
    # buffers (sloam_keyframes_host): host->device copies of every scan and
    # label array and the device->host read of every result are inside the
    # timed region, over as many steps as `value`.
    hX = learned["X"].cpu().pin_memory()
    hL = learned["Lb"].cpu().pin_memory()
    h_pose = np.zeros(B * 7, np.float64)
    h_succ = np.zeros(B, np.int32)
    h_ncyl = np.zeros(B, np.int32)
    poses = learned["poses"]

    def e2e_step():
        ctx.check(L.sloam_keyframes_host(ctx.h, hX.data_ptr(), N, B, hL.data_ptr(), poses, mapc, nm,
                                         h_pose.ctypes.data, h_succ.ctypes.data,
                                         h_ncyl.ctypes.data))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        e2e_step()
    e2e_dt = time.perf_counter() - t0
    e2e = B * args.e2e_steps * world / max_over_ranks(e2e_dt, dev)
    h2d = B * (N * 16 + N + 7 * 8) + C.sizeof(mapc)
    d2h = B * (7 * 8 + 4 + 4)
    e2e_ok = int(h_succ.sum())

    # ---- roofline: the batch projection stage (HBM-bound), per launch group
    # (64 keyframes per launch with the inputs in device memory);
    # algorithmic bytes = 26 B per point.
    peaks, peak_src = {}, "fallback"
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak_src = "measured"
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    fe_ms, fe_launches, fe_kf = learned["fe"]
    fe_bytes = 26.0 * N * fe_kf
    achieved = fe_bytes / (fe_ms / 1000.0) / 1e9 if fe_ms > 0 else None
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak if achieved else None,
        "traffic": (FRONT_TRAFFIC_PER_KF * fe_kf / fe_launches
                    if fe_launches and FRONT_TRAFFIC_PER_KF else None),
        "peak_source": peak_src,
        "kernel": "batch projection stage: k_project + k_label_batch + k_compact_batch, "
                  f"{fe_kf / max(fe_launches, 1):.0f} keyframes per launch",
        "algorithmic_bytes_per_launch": fe_bytes / fe_launches if fe_launches else None,
        "ms_per_launch": fe_ms / fe_launches if fe_launches else None,
        "launches_timed": fe_launches,
    }
    # ---- kernels that decide keyframes/s, each alone on one keyframe
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s, FMA lanes x max clock
    fp64_peak = 1.25                                  # TFLOP/s, nominal
    net_flops = net_samples * 2.0 * 128 * (64 * 128 + 128 * 256)
    net_tf = net_flops / (k_ms["k_prop_infer_tc"] / 1000.0) / 1e12
    roofline_net = {
        "bound": "tensor", "achieved": net_tf, "peak": bf16_peak, "unit": "TFLOP/s",
        "frac": net_tf / bf16_peak, "traffic": None,
        "kernel": f"k_prop_infer_tc, {net_samples} samples (one keyframe), alone",
        "flops_per_launch": net_flops, "ms_per_launch": k_ms["k_prop_infer_tc"],
    }
    # the cylinder queue (plain): inlier tests (8 FLOP each: two FP32
    # subtractions, two multiplies, an add, two compares) over every fitted
    # tree's points x 256 hypotheses, plus the 3 LS passes (~70 FLOP per
    # inlier point); FP32 issue-bound
    kernels = {
        "k_prop_infer_tc": roofline_net,
        "k_cyl_queue": {"bound": "FP32 issue (SIMT ballot counting)", "ms": k_ms["k_cyl_queue_plain"],
                        "unit": "TFLOP/s", "peak": fp32_peak, "peak_source": "nominal: 152 SMs "
                        "x 128 FP32 lanes x 2 x max SM clock"},
        "k_vertex": {"bound": "latency (warp quickselect / bitonic sort per beam, L2 gathers)",
                     "ms": k_ms["k_vertex"], "unit": "GB/s", "peak": hbm_peak},
        "k_gn": {"bound": "latency + FP64 pipe (one block; FP64 6x6 solve per iteration)",
                 "ms": k_ms["k_gn"], "unit": "TFLOP/s", "peak": fp64_peak,
                 "peak_source": "nominal FP64"},
    }
    # algorithmic work of the last keyframe the plain context ran
    fit_pts, buckets, resid = int(pstats[6]), int(pstats[7]), int(pstats[8])
    q = kernels["k_cyl_queue"]
    q["points"] = fit_pts
    q["flops"] = 8.0 * fit_pts * P.cyl_hypotheses + 70.0 * P.cyl_ls_iters * fit_pts
    q["achieved"] = q["flops"] / (q["ms"] / 1000.0) / 1e12
    q["frac"] = q["achieved"] / fp32_peak
    q["work"] = ("8 FLOP per (point, hypothesis) inlier test + ~70 FLOP per point and LS "
                 "iteration, over the fitted trees' points")
    v = kernels["k_vertex"]
    v["points"] = buckets
    v["bytes"] = 36.0 * buckets
    v["achieved"] = v["bytes"] / (v["ms"] / 1000.0) / 1e9
    v["frac"] = v["achieved"] / hbm_peak
    v["work"] = "36 B per tree pixel: 4 B bucket index + 16 B point read, 16 B kept point written"
    g = kernels["k_gn"]
    g["residuals"] = resid
    g["flops"] = 100.0 * resid * P.gn_iters
    g["achieved"] = g["flops"] / (g["ms"] / 1000.0) / 1e12
    g["frac"] = g["achieved"] / fp64_peak
    g["work"] = "~100 FLOP per residual and iteration (residual, Jacobian row, J^T J, J^T r)"

    # ---- the other configurations (rank 0 of a single-GPU run)
    extra = {}
    if args.extra and world == 1:
        extra["c1_16x1024"] = extra_workload(args, L, A, dev, world, "c1", weights)
        extra["c3_uneven_batch"] = extra_workload(args, L, A, dev, world, "c3", weights)

    # CPU baseline (rank 0, N=1): the oracle, one host thread, bounded
    # samples of the same workload: the reference's algorithm (cyl_mode 0)
    # and the point-level RANSAC the GPU plain path runs (cyl_mode 1)
    cpu = None
    if rank == 0 and world == 1:
        P0 = plain["P"].copy()
        P0.cyl_mode = 0
        v0, n0, dt0 = cpu_run_keyframes(P0, forest, kfs, args.cpu_seconds, threads=1)
        v1, n1, dt1 = cpu_run_keyframes(plain["P"], forest, kfs, args.cpu_seconds / 2, threads=1)
        cpu = {"value": v0, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{n0} keyframes of the same 16 distinct 64x2048 scans in {dt0:.1f} s, "
                         "one host thread, the reference's algorithm (vertex-line cylinder "
                         "RANSAC, cyl_mode 0; the reference path is single-threaded)",
               "point_ransac": {"value": v1, "keyframes": n1, "seconds": dt1,
                                "algorithm": "cyl_mode 1: 256 point hypotheses + 3 LS per tree"}}
        diffs = glibc_pixel_differences(plain["P"], kfs)
        cpu["projection_pixels_differing_from_glibc_per_keyframe"] = {
            "mean": float(np.mean(diffs)), "max": int(max(diffs)), "keyframes": len(diffs)}

    if rank == 0:
        cyl_l, cyl_p = k_ms["cylinder_stage_learned"], k_ms["cylinder_stage_plain"]
        line = {
            "metric": METRIC, "value": learned["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": learned["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(args, world),
            "tuning": tuning,
            "learned": {"value": learned["value"], "accuracy": acc_l,
                        "keyframes_ok": learned["ok"],
                        "cylinders_per_keyframe": learned["ncyl"]},
            "plain": {"value": plain["value"], "ms_per_step": plain["total_ms"] / args.steps,
                      "accuracy": acc_p, "keyframes_ok": plain["ok"],
                      "cylinders_per_keyframe": plain["ncyl"],
                      "gpu_launches": int(plain["launches"])},
            "reference_algorithm": {
                "value": refalg["value"], "ms_per_step": refalg["total_ms"] / args.steps,
                "keyframes_ok": refalg["ok"], "cylinders_per_keyframe": refalg["ncyl"],
                "algorithm": "the reference's vertex-line cylinder RANSAC (cyl_mode 0) on the GPU"},
            "learned_over_plain": learned["value"] / plain["value"],
            "cylinder_stage_ms_per_keyframe": {
                "learned": cyl_l, "plain": cyl_p,
                "reference_algorithm": k_ms["cylinder_stage_reference_algorithm"],
                "plain_over_learned": cyl_p / cyl_l if cyl_l > 0 else None,
                "how": "the whole cylinder stage of one keyframe alone (CUDA events, mean of 20)"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "keyframes_ok": e2e_ok,
                    "steps": args.e2e_steps,
                    "api": "sloam_keyframes_host, pinned host buffers, learned path"},
            "gpu_launches": int(learned["launches"]),
            "stages_ms_per_keyframe": {"project_mask": stages[0], "trellis": stages[1],
                                       "models": stages[2], "assoc_pose": stages[3]},
            "kernels_ms": k_ms,
            "kernels": kernels,
            "host_enqueue_ms_per_step": 1000.0 * learned["host_s"] / args.steps,
            "clocks": ck,
            "roofline": roofline,
            "roofline_proposal_net": roofline_net,
            "cpu_baseline": cpu,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    learned["ctx"].close()
    plain["ctx"].close()
    refalg["ctx"].close()
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
