"""The learned cylinder proposal: parameter layout, the tensor-core
inference against the SIMT kernel of the same arithmetic and against a plain
PyTorch FP32 forward, training, and the committed weights' accuracy on
held-out synthetic clusters."""
import os

import numpy as np
import pytest

from sloam_gb300 import proposal as Pn


def test_parameter_layout():
    assert Pn.NUM_PARAMS == 75399
    assert Pn._lib().sloam_prop_num_params() == 75399
    u = Pn.unpack(np.arange(Pn.NUM_PARAMS, dtype=np.float32))
    assert u["W3"].shape == (128, 256) and u["b5"][-1] == Pn.NUM_PARAMS - 1


def test_committed_weights():
    w = Pn.load_weights()
    assert w.shape == (Pn.NUM_PARAMS,) and np.isfinite(w).all()


def _weights():
    if os.path.exists(Pn.WEIGHTS):
        return Pn.load_weights()
    rng = np.random.default_rng(0)
    return (rng.standard_normal(Pn.NUM_PARAMS) * 0.1).astype(np.float32)


@pytest.mark.gpu
def test_tensor_core_inference_matches_simt_and_torch():
    import torch
    w = _weights()
    X, _ = Pn.sample(300)
    o_tc = Pn.infer(w, X, mode=0)[:, :7]
    o_ref = Pn.infer(w, X, mode=1)[:, :7]
    o_t = Pn.torch_forward(w, X)
    # same bf16 operands, FP32 accumulation in a different order: a rare
    # bf16 rounding flip of an activation moves an output by ~1e-3
    scale = o_t.abs().max().item() + 1e-6
    assert (o_tc - o_ref).abs().max().item() < 5e-3 * scale
    assert (o_ref - o_t).abs().max().item() < 5e-3 * scale
    assert torch.isfinite(o_tc).all()


@pytest.mark.gpu
def test_training_reduces_the_loss():
    w, loss = Pn.train(80, batch=256, seed=3, first_id=5 * 10 ** 8)
    assert np.isfinite(loss).all()
    assert loss[-10:].mean() < 0.7 * loss[:10].mean()


@pytest.mark.gpu
def test_committed_weights_accuracy():
    w = Pn.load_weights()
    X, T = Pn.sample(4000)
    ang, cerr, rerr = Pn.errors(Pn.infer(w, X, 0), T)
    # the proposal alone (before LS refinement and inlier scoring)
    assert ang.median().item() < 3.0
    assert rerr.median().item() < 0.03


@pytest.mark.gpu
def test_training_gradient_matches_autograd():
    """One step of the hand-written backward (k_prop_train + k_prop_reduce)
    against torch.autograd of the same loss in FP32, on 64 clusters: every
    gradient entry but a few within 2e-4 of the gradient's largest magnitude
    (the sums run in another order; a max-pool argmax or a ReLU at zero
    within rounding of a tie may route one cluster's gradient differently),
    each layer's gradient within 2e-3 of its norm, the per-cluster losses
    within 1e-4 relative."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    w = _weights()
    X, T = Pn.sample(64, seed=31, first_id=3 * 10 ** 8)
    g, loss = Pn.grad(w, X, T)
    wt = torch.tensor(w, device="cuda", requires_grad=True)
    lt = Pn.torch_loss(wt, X, T)
    lt.mean().backward()
    gt = wt.grad.cpu().numpy()
    np.testing.assert_allclose(loss, lt.detach().cpu().numpy(), rtol=1e-4, atol=1e-6)
    scale = np.abs(gt).max()
    assert (np.abs(g - gt) > 2e-4 * scale).sum() <= 16
    for name, (a, b) in zip([n for n, _ in Pn.SHAPES],
                            zip(Pn.unpack(g).values(), Pn.unpack(gt).values())):
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 2e-3 * nb + 1e-7, name


@pytest.mark.gpu
def test_adam_steps_match_torch_optim():
    """Three training steps (fresh clusters per step, as sloam_prop_train
    draws them) against torch.optim.Adam with the same hyper-parameters on
    the same clusters.  Early Adam steps move each weight by about lr x the
    sign of its gradient, so the weights agree within 1e-6 except where a
    gradient entry is near zero and its sign follows rounding (at most 0.5 %
    of them, each within 2 lr x steps)."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    w0 = _weights()
    steps, batch, lr, seed, first = 3, 64, 1e-3, 9, 7 * 10 ** 8
    w_gpu, _ = Pn.train(steps, batch=batch, lr=lr, seed=seed, first_id=first, init=w0)
    wt = torch.tensor(w0, device="cuda", requires_grad=True)
    opt = torch.optim.Adam([wt], lr=lr, betas=(0.9, 0.999), eps=1e-8)
    for s in range(steps):
        X, T = Pn.sample(batch, seed=seed ^ 0x5a5a5a5a, first_id=first + s * batch)
        opt.zero_grad()
        Pn.torch_loss(wt, X, T).mean().backward()
        opt.step()
    w_t = wt.detach().cpu().numpy()
    d = np.abs(w_gpu - w_t)
    assert d.max() <= 2 * lr * steps + 1e-6
    assert (d > 1e-6).mean() < 5e-3
