"""The learned start value's network: the numpy oracle's gradient is checked
against finite differences (CPU); the CUDA forward/backward kernels are
checked against the oracle (GPU)."""
import numpy as np
import pytest

import mlp_oracle as MO
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import solver


def synthetic_records(n, seed=0):
    """Records shaped like the recorder's: features in realistic ranges,
    target = log(p*/p_L) of an acoustic estimate (smooth in the features)."""
    rng = np.random.default_rng(seed)
    rr = np.exp(rng.normal(0, 0.7, n))
    pr = np.exp(rng.normal(0, 1.0, n))
    du = rng.normal(0, 1.0, n)
    cr = np.sqrt(pr / rr)
    gam = np.full(n, 5.0 / 3.0)
    lpl = rng.normal(0, 1.0, n)
    y = np.log(np.maximum((1 + pr) / 2 - 0.25 * du * (1 + cr) * (1 + rr) / 2, 1e-3))
    rec = np.zeros((n, A.AST_RECORD_FLOATS), dtype=np.float32)
    rec[:, :7] = np.stack([rr, pr, du, cr, gam, lpl, y], 1)
    return rec


def init_params(rec, seed=3):
    rng = np.random.default_rng(seed)
    p = np.zeros(MO.NPARAM)
    x = MO.input_map(rec[:, :6])
    p[0:6] = x.mean(0)
    sd = x.std(0)
    p[6:12] = np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-12), 1.0)
    p[12:] = rng.normal(0, 0.3, MO.NPARAM - 12)
    return p


def test_oracle_gradient_matches_finite_differences():
    rec = synthetic_records(64)
    p = init_params(rec)
    g = MO.grad(p, rec[:, :6], rec[:, 6])
    idx = [12, 100, 204, 236, 700, 1259, 1260, 1292, 1323, 1324]
    fd = MO.fd_grad(p, rec[:, :6], rec[:, 6], idx)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-5, atol=1e-9)


def test_mlp_init_statistics():
    rec = synthetic_records(5000)
    p = solver.mlp_init(rec, seed=7)
    x = MO.input_map(rec[:, :6])
    np.testing.assert_allclose(p[0:6], x.mean(0), rtol=1e-4, atol=1e-5)
    assert np.all(p[6:12] > 0)
    assert np.all(p[204:236] == 0) and abs(p[1324] - rec[:, 6].mean()) < 1e-4
    assert np.array_equal(p, solver.mlp_init(rec, seed=7))


@pytest.mark.gpu
def test_cuda_forward_and_gradient_match_oracle():
    rec = synthetic_records(3000, seed=1)
    p = init_params(rec).astype(np.float32)
    y = solver.mlp_forward(p, rec[:, :6])
    y_ref, _ = MO.forward(p, rec[:, :6])
    np.testing.assert_allclose(y, y_ref, rtol=1e-4, atol=1e-4)
    g, loss = solver.mlp_grad(p, rec)
    g_ref = MO.grad(p, rec[:, :6], rec[:, 6])
    assert abs(loss - MO.loss(p, rec[:, :6], rec[:, 6])) < 1e-4 * max(1.0, loss)
    assert np.all(g[:12] == 0)
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(g - g_ref)) < 1e-3 * scale, np.max(np.abs(g - g_ref)) / scale


@pytest.mark.gpu
def test_cuda_training_lowers_the_loss():
    rec = synthetic_records(1 << 15, seed=2)
    p0 = solver.mlp_init(rec, seed=7)
    p, losses = solver.mlp_train(rec, p0, epochs=12, batch=4096, lr=3e-3, seed=7)
    assert losses[-1] < 0.35 * losses[0], losses
    assert MO.loss(p, rec[:, :6], rec[:, 6]) < 0.35 * MO.loss(p0, rec[:, :6], rec[:, 6])


@pytest.mark.gpu
def test_tensor_core_inference_matches_fp32_network():
    """The step kernel evaluates the network on the tensor cores (f16
    operands, f32 accumulation, tanh-form SiLU in f16x2); on the trained
    network and recorded-like inputs it agrees with the FP32 network to the
    precision of f16 (absolute 0.02 in log p*)."""
    import os
    from conftest import ROOT
    path = os.path.join(ROOT, "asteriy_2d_gb300", "data", "guess_blast.npy")
    params = np.load(path) if os.path.exists(path) else init_params(synthetic_records(4000)).astype(np.float32)
    rec = synthetic_records(4000, seed=4)
    y32 = solver.mlp_forward(params, rec[:, :6])
    ytc = solver.mlp_forward_tc(params, rec[:, :6])
    err = np.abs(ytc - y32)
    print("tensor-core vs FP32 network: max", err.max(), "median", np.median(err))
    assert np.median(err) < 5e-3 and np.percentile(err, 99.9) < 0.02 and err.max() < 0.05
