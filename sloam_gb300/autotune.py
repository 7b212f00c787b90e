"""Autotuner of the point-level cylinder fit's work queue and of the batch
width, per GPU and workload.

    python -m sloam_gb300.autotune [--workload c2|c3|all] [--out FILE]

The cylinder fit (cylqueue.cu) cuts each tree into work items of
`cyl_chunk_points` points, stages `cyl_hyp_tile` hypotheses in shared memory
per pass and runs `cyl_queue_blocks` persistent blocks; `batch_slots`
keyframes of a batch are in flight at once.  None of these changes a result
(the tests check bit-identity across shapes); they change the speed.  The
tuner measures keyframes/s of the workload's batch (plain RANSAC, the path
the queue serves) with CUDA events for every queue shape at 32 slots, then
the batch width at the best shape, and writes the best settings keyed by the
GPU's name and the workload to `tuning.json` beside this file, which
`bench.py` applies (`apply`).

Workloads: c2 = 64 keyframes of 64x2048 (16 distinct scans), 150 trees,
256 hypotheses; c3 = the uneven batch, 64 keyframes with 20-400 trees each.
"""
import argparse
import ctypes as C
import itertools
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING = os.path.join(HERE, "tuning.json")
CHUNKS = (256, 512, 1024)
TILES = (64, 128, 256, 512, 1024)
BLOCKS = (76, 152, 304, 608)
SLOTS = (16, 24, 32, 48)
KEYS = ("cyl_chunk_points", "cyl_hyp_tile", "cyl_queue_blocks", "batch_slots")


def load(path=TUNING):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(gpu_name, workload, path=TUNING):
    """The tuned settings of (GPU, workload), or None."""
    return load(path).get(gpu_name, {}).get(workload)


def apply(P, gpu_name, workload, path=TUNING):
    """Sets the tuned fields of params P in place; returns the settings used
    (the defaults when the GPU or workload has not been tuned)."""
    t = lookup(gpu_name, workload, path)
    if t:
        for k in KEYS:
            if k in t:
                setattr(P, k, int(t[k]))
    return {k: int(getattr(P, k)) for k in KEYS} | {"tuned": bool(t)}


def workload(name, seed=0):
    """(params, forest, keyframes of the batch, map) of a workload."""
    from . import capi as A
    from . import synth
    if name == "c2":
        cfg = synth.C2
        forest, kfs = synth.scene(cfg, seed=seed, n_kf=16)
        P = synth.preset_params(cfg, two_step_optim=0, cyl_mode=1, cyl_hypotheses=256,
                                cyl_ls_iters=3, gn_iters=10)
        batch = [kfs[i % len(kfs)] for i in range(64)]
    elif name == "c3":
        forest, kfs, _ = synth.c3_scene(seed, n_kf=64)
        P = synth.c3_params(forest, two_step_optim=0, cyl_mode=1)
        batch = kfs
    else:
        raise ValueError(name)
    mapc = A.cylinders_from_array(forest.map_cylinders())
    return P, forest, batch, mapc


class BatchRunner:
    """One context running a device-resident batch; `rate` times steps."""

    def __init__(self, P, batch, mapc, n_map, dev):
        import torch
        from . import capi as A
        from .lib import Context
        self.A, self.torch = A, torch
        self.ctx = Context(P, device=dev.index or 0)
        L = self.L = self.ctx.L
        kf0 = batch[0]
        r = A.RunBuffers(P)
        self.ctx.check(L.sloam_keyframe(self.ctx.h, A.ptr(kf0.xyzi, C.c_float), len(kf0.xyzi),
                                        A.ptr(kf0.labels, C.c_uint8), None,
                                        C.byref(A.SE3.from_qt(*kf0.pose_gt_qt())), mapc, n_map,
                                        C.byref(r.s)))
        self.B, self.N = len(batch), P.img_w * P.img_h
        self.X = torch.from_numpy(np.stack([k.xyzi for k in batch])).to(dev)
        self.Lb = torch.from_numpy(np.stack([k.labels for k in batch])).to(dev)
        self.Mp = torch.from_numpy(np.frombuffer(bytes(mapc), np.uint8).copy()).to(dev)
        self.poses = (A.SE3 * self.B)(*[A.SE3.from_qt(*k.pose_est_qt()) for k in batch])
        self.pose_out = torch.zeros(self.B * 7, dtype=torch.float64, device=dev)
        self.succ = torch.zeros(self.B, dtype=torch.int32, device=dev)
        self.ncyl = torch.zeros(self.B, dtype=torch.int32, device=dev)
        self.n_map = n_map
        self.ext = torch.cuda.ExternalStream(self.ctx.stream(), device=dev)

    def step(self):
        self.ctx.check(self.L.sloam_keyframes_device(
            self.ctx.h, self.X.data_ptr(), self.N, self.B, self.Lb.data_ptr(), self.poses,
            self.Mp.data_ptr(), self.n_map, self.pose_out.data_ptr(), self.succ.data_ptr(),
            self.ncyl.data_ptr()))
        return self.ctx.launches()

    def rate(self, warmup=2, steps=5, flush=None):
        """Keyframes/s over `steps` timed batch steps (CUDA events on the
        context stream), L2 flushed before each when `flush` is given."""
        torch = self.torch
        for _ in range(warmup):
            self.step()
        torch.cuda.synchronize()
        total = 0.0
        for s in range(steps):
            if flush is not None:
                flush.fill_(float(s))
                torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.ext)
            self.step()
            e1.record(self.ext)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        return self.B * steps / (total / 1000.0)

    def close(self):
        self.ctx.close()


def tune(name, dev, log=print):
    import torch
    P0, forest, batch, mapc = workload(name)
    nm = len(forest.radius)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    sweep = []
    t0 = time.time()
    for chunk, tile, blocks in itertools.product(CHUNKS, TILES, BLOCKS):
        P = P0.copy()
        P.cyl_chunk_points, P.cyl_hyp_tile, P.cyl_queue_blocks = chunk, tile, blocks
        P.batch_slots = 32
        r = BatchRunner(P, batch, mapc, nm, dev)
        v = r.rate(flush=flush)
        r.close()
        sweep.append({"cyl_chunk_points": chunk, "cyl_hyp_tile": tile,
                      "cyl_queue_blocks": blocks, "batch_slots": 32, "kf_per_s": v})
        log(f"{name} chunk {chunk:5d} tile {tile:5d} blocks {blocks:4d}: {v:9.1f} kf/s")
    best = max(sweep, key=lambda x: x["kf_per_s"])
    slots = []
    for ns in SLOTS:
        P = P0.copy()
        P.cyl_chunk_points, P.cyl_hyp_tile = best["cyl_chunk_points"], best["cyl_hyp_tile"]
        P.cyl_queue_blocks, P.batch_slots = best["cyl_queue_blocks"], ns
        r = BatchRunner(P, batch, mapc, nm, dev)
        v = r.rate(flush=flush, steps=8)
        r.close()
        slots.append({"batch_slots": ns, "kf_per_s": v})
        log(f"{name} slots {ns:3d}: {v:9.1f} kf/s")
    bs = max(slots, key=lambda x: x["kf_per_s"])
    default = next(x for x in sweep if (x["cyl_chunk_points"], x["cyl_hyp_tile"],
                                        x["cyl_queue_blocks"]) == (256, 256, 152))
    return {"cyl_chunk_points": best["cyl_chunk_points"], "cyl_hyp_tile": best["cyl_hyp_tile"],
            "cyl_queue_blocks": best["cyl_queue_blocks"], "batch_slots": bs["batch_slots"],
            "kf_per_s": bs["kf_per_s"], "default_shape_kf_per_s": default["kf_per_s"],
            "shapes_tried": len(sweep), "seconds": time.time() - t0,
            "top_shapes": sorted(sweep, key=lambda x: -x["kf_per_s"])[:5], "slots": slots}


def main():
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="all", choices=["c2", "c3", "all"])
    ap.add_argument("--out", default=TUNING)
    a = ap.parse_args()
    import torch
    from . import build
    build.build()
    dev = torch.device("cuda", 0)
    gpu = torch.cuda.get_device_name(dev)
    data = load(a.out)
    entry = data.setdefault(gpu, {})
    for name in (("c2", "c3") if a.workload == "all" else (a.workload,)):
        entry[name] = tune(name, dev)
        print(json.dumps({name: {k: entry[name][k] for k in KEYS + ("kf_per_s",)}}))
    with open(a.out, "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")
    print(f"wrote {a.out}")


if __name__ == "__main__":
    main()
