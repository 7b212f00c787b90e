#!/usr/bin/env python3
"""Keyframes/s of the SLOAM keyframe hot path on GB300.

Workload (one step): a batch of B synthetic 64x2048 keyframes (float32 XYZI,
~131k points each; 150 trunks with radius U(0.08, 0.6) m, shrubs, 10%
outliers; per-point labels from the generator), each run through projection,
Trellis, ground planes, the point-level cylinder RANSAC (256 hypotheses per
tree, 3 cm inlier band, 3 LS iterations), association against a 400-landmark
submap and 10 Gauss-Newton pose iterations (FP32 residuals, FP64 6x6 solve).
Inputs are device-resident for `value`; `e2e` runs the same keyframes through
the host C ABI (sloam_keyframes_host) from pinned host buffers.  L2 is flushed
(256 MB write) before every timed step.

`roofline` is the batch projection stage (k_project, k_resolve, k_mask,
k_label, k_ground_compact over 8 keyframes per launch), timed with CUDA
events on its stream inside the timed steps: 26 algorithmic bytes per point
(16 B XYZI + 1 B label read, 4 B pixel index + 4 B range + 1 B mask
written).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference algorithm's CPU implementation (the
std-only restatement in oracle/, the reference itself cannot be built here)
on all host cores, one keyframe per thread per step.
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
# (dram__bytes_read.sum + dram__bytes_write.sum of two 16-keyframe chunk
# launches: 4.15 and 6.43 MB per keyframe).
FRONT_TRAFFIC_PER_KF = 5.29e6


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
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
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
            kf = kfs[(t + k) % len(kfs)]
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


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg, forest, kfs, P = workload(args.seed, min(args.distinct, 8))
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
        kf = kfs[(t + step) % len(kfs)]
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
    sample = f"{threads} keyframes per step (one per host thread), oracle restatement, 64x2048"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "threads": threads},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# -------------------------------------------------------------- GPU leg
def measure(args, L, A, P, forest, kfs, dev, world, mode, weights, clocks_run=None):
    """One context in cylinder mode `mode` (1 plain RANSAC, 2 learned
    proposals): the first scan, W warm-up and K timed batch steps."""
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
    B = args.batch
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
    generator's trunks over the distinct keyframes, and the trees that fell
    back to RANSAC.  Each keyframe runs as in the batch: after the first
    scan (keyframe 0 at its true pose), at its perturbed estimate."""
    from sloam_gb300 import synth
    ctx, P = m["ctx"], m["P"]
    angs, rerrs, fb, nl, slow = [], [], 0, 0, 0
    stats = (C.c_int32 * 5)()
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
        L.sloam_keyframe_stats(ctx.h, stats, 5)
        fb += stats[3]
        nl += stats[1]
        slow += stats[4]
    a, e = np.concatenate(angs), np.concatenate(rerrs)
    return {"median_axis_deg": float(np.median(a)), "median_radius_cm": float(100 * np.median(e)),
            "cylinders_matched": int(len(a)), "keyframes": len(kfs) - 1,
            "fallback_trees": int(fb), "valid_cylinders": int(nl),
            "fp64_projection_points_per_keyframe": slow / max(len(kfs) - 1, 1)}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    from sloam_gb300 import build, capi as A, proposal
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
    weights = proposal.load_weights()
    clocks = Clocks(local)
    clocks.start()
    learned = measure(args, L, A, P, forest, kfs, dev, world, 2, weights)
    plain = measure(args, L, A, P, forest, kfs, dev, world, 1, weights)
    ck = clocks.stop()
    ctx = learned["ctx"]
    N, B, mapc, nm = learned["N"], learned["B"], learned["mapc"], learned["nm"]

    # per-stage breakdown of one keyframe, and kernels in isolation
    stages = (C.c_float * 4)()
    L.sloam_profile_stages(ctx.h, stages, 4)
    net_ms, proj_ms, cnt_ms = C.c_float(), C.c_float(), C.c_float()
    ctx.check(L.sloam_time_kernel(ctx.h, 2, 20, C.byref(net_ms)))
    stats = (C.c_int32 * 5)()
    L.sloam_keyframe_stats(ctx.h, stats, 5)
    net_samples = stats[0] * learned["P"].prop_samples
    ctx.check(L.sloam_time_kernel(ctx.h, 0, 20, C.byref(proj_ms)))
    plain["ctx"].check(L.sloam_time_kernel(plain["ctx"].h, 1, 20, C.byref(cnt_ms)))
    acc_l = accuracy(L, A, learned, forest, kfs)
    acc_p = accuracy(L, A, plain, forest, kfs)

    # ---- e2e: the same keyframes through the host C ABI from pinned host
    # buffers (sloam_keyframes_host): host->device copies of every scan and
    # label array and the device->host read of every result are inside the
    # timed region.
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

    e2e_step()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        e2e_step()
    e2e_dt = time.perf_counter() - t0
    e2e = B * args.e2e_steps / e2e_dt
    h2d = B * (N * 16 + N + 7 * 8) + C.sizeof(mapc)
    d2h = B * (7 * 8 + 4 + 4)
    e2e_ok = int(h_succ.sum())

    # ---- roofline: the batch projection stage (HBM-bound), per launch group
    # (16 keyframes per launch with the inputs in device memory);
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
        "kernel": "batch projection stage: k_project + k_label + k_ground_compact, "
                  f"{fe_kf / max(fe_launches, 1):.0f} keyframes per launch",
        "algorithmic_bytes_per_launch": fe_bytes / fe_launches if fe_launches else None,
        "ms_per_launch": fe_ms / fe_launches if fe_launches else None,
        "launches_timed": fe_launches,
    }
    # the proposal network (tensor-bound): dense bf16 FLOPs of the two
    # tensor-core layers per 128-point sample over the isolated launch time
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    net_flops = net_samples * 2.0 * 128 * (64 * 128 + 128 * 256)
    net_tf = net_flops / (net_ms.value / 1000.0) / 1e12 if net_ms.value > 0 else None
    roofline_net = {
        "bound": "tensor", "achieved": net_tf, "peak": bf16_peak, "unit": "TFLOP/s",
        "frac": net_tf / bf16_peak if net_tf else None, "traffic": None,
        "kernel": f"k_prop_infer_tc, {net_samples} samples (one keyframe), alone",
        "flops_per_launch": net_flops, "ms_per_launch": net_ms.value,
    }

    # CPU baseline (rank 0, N=1): the oracle, one host thread, bounded sample
    cpu = None
    if rank == 0 and world == 1:
        v, n_kf, dt = cpu_run_keyframes(plain["P"], forest, kfs, args.cpu_seconds, threads=1)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{n_kf} keyframes of the same 64x2048 workload in {dt:.1f} s, "
                         "one host thread, the reference's plain path (the reference path "
                         "is single-threaded)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": learned["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": learned["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "batch_keyframes": B, "distinct_scans": args.distinct,
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{world}"},
            "learned": {"value": learned["value"], "accuracy": acc_l,
                        "keyframes_ok": learned["ok"],
                        "cylinders_per_keyframe": learned["ncyl"]},
            "plain": {"value": plain["value"], "ms_per_step": plain["total_ms"] / args.steps,
                      "accuracy": acc_p, "keyframes_ok": plain["ok"],
                      "cylinders_per_keyframe": plain["ncyl"],
                      "gpu_launches": int(plain["launches"])},
            "learned_over_plain": learned["value"] / plain["value"],
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "keyframes_ok": e2e_ok,
                    "api": "sloam_keyframes_host, pinned host buffers, learned path"},
            "gpu_launches": int(learned["launches"]),
            "stages_ms_per_keyframe": {"project_mask": stages[0], "trellis": stages[1],
                                       "models": stages[2], "assoc_pose": stages[3]},
            "kernels_ms": {"k_prop_infer_tc": net_ms.value, "k_project": proj_ms.value,
                           "k_cyl_count_plain": cnt_ms.value},
            "host_enqueue_ms_per_step": 1000.0 * learned["host_s"] / args.steps,
            "clocks": ck,
            "roofline": roofline,
            "roofline_proposal_net": roofline_net,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    learned["ctx"].close()
    plain["ctx"].close()
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
