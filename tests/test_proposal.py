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
