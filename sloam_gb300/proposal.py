"""Host side of the learned cylinder proposal: training driver, weight file,
evaluation on held-out synthetic clusters, and a plain PyTorch FP32 forward
of the same network (used by the tests as the numerics reference).

    python -m sloam_gb300.proposal train --steps 3000 --batch 1024 --out W.f32

The network (see csrc/proposal.cuh): 128 centred, scale-normalised points ->
shared MLP 3-64-128-256 (ReLU) -> max-pool -> 256-128 (ReLU) -> 7:
axis (3), centre xy (2), log(radius / scale), confidence logit.
"""
import argparse
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "proposal_weights.f32")

D1, D2, D3, D4, D5 = 64, 128, 256, 128, 7
SHAPES = [("W1", (3, D1)), ("b1", (D1,)), ("W2", (D1, D2)), ("b2", (D2,)),
          ("W3", (D2, D3)), ("b3", (D3,)), ("W4", (D3, D4)), ("b4", (D4,)),
          ("W5", (D4, D5)), ("b5", (D5,))]
NUM_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)  # 75 399


def _lib():
    from .lib import load
    L = load()
    L.sloam_prop_num_params.restype = C.c_int
    L.sloam_prop_train.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                   C.c_int64, C.c_void_p, C.c_void_p]
    L.sloam_prop_sample.argtypes = [C.c_uint64, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]
    L.sloam_prop_infer.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]
    L.sloam_prop_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                  C.c_void_p]
    return L


def unpack(w):
    """FP32 parameter vector -> dict of arrays (row-major W[in][out])."""
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = w[o:o + n].reshape(shape)
        o += n
    return out


def load_weights(path=WEIGHTS):
    w = np.fromfile(path, dtype=np.float32)
    if w.size != NUM_PARAMS:
        raise ValueError(f"{path}: {w.size} values, expected {NUM_PARAMS}")
    return w


def train(steps, batch=1024, lr=1e-3, seed=1, first_id=0, init=None):
    """Runs the GPU training kernels; returns (weights, per-step mean loss)."""
    L = _lib()
    w = np.zeros(NUM_PARAMS, np.float32)
    loss = np.zeros(max(steps, 1), np.float32)
    ini = None if init is None else np.ascontiguousarray(init, np.float32)
    st = L.sloam_prop_train(None if ini is None else ini.ctypes.data, steps, batch, lr, seed,
                            first_id, w.ctypes.data, loss.ctypes.data)
    if st:
        raise RuntimeError(f"sloam_prop_train failed ({st})")
    return w, loss[:steps]


def grad(w, X, T):
    """The training kernels' mean gradient and per-cluster losses of weights
    w on device samples X [n,128,3], T [n,8] (no update)."""
    L = _lib()
    g = np.zeros(NUM_PARAMS, np.float32)
    loss = np.zeros(X.shape[0], np.float32)
    ww = np.ascontiguousarray(w, np.float32)
    st = L.sloam_prop_grad(ww.ctypes.data, X.data_ptr(), T.data_ptr(), X.shape[0], g.ctypes.data,
                           loss.ctypes.data)
    if st:
        raise RuntimeError(f"sloam_prop_grad failed ({st})")
    return g, loss


def torch_loss(w, X, T):
    """The training loss in plain PyTorch FP32 (per cluster): squared error
    on axis, centre xy and log radius, plus 0.1 x the binary cross-entropy
    of the confidence against exp(-e / 0.01), e the centre and log-radius
    squared error (the target is a constant of the step).  w is a torch
    parameter vector."""
    import torch
    p, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        p[name] = w[o:o + n].reshape(shape)
        o += n
    a1 = torch.relu(X @ p["W1"] + p["b1"])
    a2 = torch.relu(a1 @ p["W2"] + p["b2"])
    h = torch.relu((a2 @ p["W3"] + p["b3"]).max(dim=1).values)
    y1 = torch.relu(h @ p["W4"] + p["b4"])
    out = y1 @ p["W5"] + p["b5"]
    mse = ((out[:, :6] - T[:, :6]) ** 2).sum(1)
    ec = ((out[:, 3:6] - T[:, 3:6]) ** 2).sum(1).detach()
    ct = torch.exp(-ec / 0.01)
    z = out[:, 6]
    bce = ct * torch.nn.functional.softplus(-z) + (1 - ct) * torch.nn.functional.softplus(z)
    return mse + 0.1 * bce


def sample(n, seed=7, first_id=10 ** 9):
    """n synthetic clusters on the GPU: (points [n,128,3], targets [n,8]) as
    torch CUDA tensors.  Targets: axis (3), centre xy (2), log(r/s), s, r."""
    import torch
    L = _lib()
    X = torch.empty((n, 128, 3), dtype=torch.float32, device="cuda")
    T = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    st = L.sloam_prop_sample(seed, first_id, n, X.data_ptr(), T.data_ptr())
    if st:
        raise RuntimeError(f"sloam_prop_sample failed ({st})")
    return X, T


def infer(w, X, mode=0):
    """Network outputs [n, 8] (7 used) for normalised samples X (CUDA);
    mode 0 tensor cores, 1 the SIMT kernel of the same arithmetic."""
    import torch
    L = _lib()
    out = torch.zeros((X.shape[0], 8), dtype=torch.float32, device="cuda")
    ww = np.ascontiguousarray(w, np.float32)
    st = L.sloam_prop_infer(ww.ctypes.data, X.data_ptr(), X.shape[0], out.data_ptr(), mode)
    if st:
        raise RuntimeError(f"sloam_prop_infer failed ({st})")
    return out


def torch_forward(w, X, bf16=True):
    """Plain PyTorch FP32 forward; bf16=True rounds the weights and the
    activations A1, A2 to bf16 where the GPU kernels do."""
    import torch
    p = {k: torch.from_numpy(np.ascontiguousarray(v)).to(X.device) for k, v in unpack(w).items()}

    def r(t):
        return t.to(torch.bfloat16).float() if bf16 else t
    if bf16:
        p = {k: r(v) for k, v in p.items()}
    a1 = r(torch.relu(X @ p["W1"] + p["b1"]))
    a2 = r(torch.relu(a1 @ p["W2"] + p["b2"]))
    a3 = torch.relu(a2 @ p["W3"] + p["b3"])
    h = a3.max(dim=1).values
    y1 = torch.relu(h @ p["W4"] + p["b4"])
    return y1 @ p["W5"] + p["b5"]


def errors(out, T):
    """Per-cluster axis angle (deg), centre error (m) and radius error (m)
    of network outputs against the generator's targets."""
    import torch
    a = out[:, :3] / out[:, :3].norm(dim=1, keepdim=True)
    ang = torch.rad2deg(torch.arccos(torch.clamp((a * T[:, :3]).sum(1).abs(), max=1.0)))
    s = T[:, 6]
    cerr = (out[:, 3:5] - T[:, 3:5]).norm(dim=1) * s
    rerr = (torch.exp(out[:, 5]) - torch.exp(T[:, 5])).abs() * s
    return ang, cerr, rerr


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--steps", type=int, default=3000)
    t.add_argument("--batch", type=int, default=1024)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=1)
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--resume", default=None)
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--n", type=int, default=20000)
    a = ap.parse_args()
    if a.cmd == "train":
        import time
        init = load_weights(a.resume) if a.resume else None
        t0 = time.time()
        w, loss = train(a.steps, a.batch, a.lr, a.seed, init=init)
        dt = time.time() - t0
        w.tofile(a.out)
        k = max(1, len(loss) // 10)
        print(f"trained {a.steps} steps x {a.batch} clusters in {dt:.1f} s; "
              f"loss {loss[:k].mean():.4f} -> {loss[-k:].mean():.4f}; wrote {a.out}")
    else:
        import torch
        w = load_weights(a.weights)
        X, T = sample(a.n)
        ang, cerr, rerr = errors(infer(w, X, 0), T)
        print(f"median axis {ang.median():.3f} deg, centre {100 * cerr.median():.2f} cm, "
              f"radius {100 * rerr.median():.2f} cm over {a.n} held-out clusters")


if __name__ == "__main__":
    main()
