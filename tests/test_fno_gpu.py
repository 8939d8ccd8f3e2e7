"""GPU kernels of the learned warm start against NumPy and the FP64 FNO oracle.

* ``pg_gemm_bf16``: every transpose combination, alpha/beta, batch strides and ragged sizes
  against an FP64 product of the same BF16-rounded operands (FP32 accumulation: 1e-5).
* The network's forward output and every parameter gradient against ``oracle.fno`` with the
  same (BF16-rounded) parameters: BF16 activations bound the difference (1e-2 relative L2 for
  the output and for every gradient).
* Forty Adam steps halve the loss of a small fitting problem.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import fno as ofno
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _bf16_round(a):
    """Round FP32 values to BF16 (nearest even) and back, in NumPy."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("engine", [0, 1])
@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_bf16_matches_numpy(cuda_lib, ta, tb, engine):
    """Both engines: 0 = tcgen05 (accumulators in tensor memory), 1 = mma.sync."""
    import ctypes

    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    _lib.check(lib.pg_gemm_set_engine(engine), "pg_gemm_set_engine")
    rng = np.random.default_rng(ta * 2 + tb)
    for M, N, K, batch in [(70, 45, 33, 3), (128, 64, 256, 1), (5, 130, 7, 2), (300, 200, 96, 1),
                           (136, 72, 40, 2)]:
        a_shape = (batch, K, M) if ta else (batch, M, K)
        b_shape = (batch, N, K) if tb else (batch, K, N)
        a = _bf16_round(rng.standard_normal(a_shape))
        b = _bf16_round(rng.standard_normal(b_shape))
        c0 = rng.standard_normal((batch, M, N)).astype(np.float32)
        A = torch.tensor(a, device="cuda").to(torch.bfloat16)
        B = torch.tensor(b, device="cuda").to(torch.bfloat16)
        Cm = torch.tensor(c0, device="cuda")
        lda = M if ta else K
        ldb = K if tb else N
        _lib.check(lib.pg_gemm_bf16(A.data_ptr(), B.data_ptr(), Cm.data_ptr(), M, N, K, lda, ldb, N, ta, tb,
                                    0.75, -0.5, batch, M * K, N * K, M * N, None), "pg_gemm_bf16")
        am = np.swapaxes(a, 1, 2) if ta else a
        bm = np.swapaxes(b, 1, 2) if tb else b
        expect = 0.75 * np.einsum("bmk,bkn->bmn", am.astype(np.float64), bm.astype(np.float64)) - 0.5 * c0
        assert rel_l2(Cm.cpu().numpy(), expect) < 1e-5, (M, N, K, batch, engine)
    count = ctypes.c_int32()
    _lib.check(lib.pg_gemm_timeouts(ctypes.byref(count), 1), "pg_gemm_timeouts")
    assert count.value == 0
    _lib.check(lib.pg_gemm_set_engine(0), "pg_gemm_set_engine")


def _small():
    return dict(c_in=3, c_out=3, width=8, modes=4, layers=2, hidden=16)


def test_fno_forward_and_gradients_match_oracle(cuda_lib):
    import torch

    from polarism_gb300.fno import FNO2d, init_params

    cfg = _small()
    n, B = 32, 2
    params = init_params(seed=3, **cfg)
    rng = np.random.default_rng(5)
    for k in params:
        if k.endswith("_b") or (k.startswith("b") and k[1:].isdigit()):
            params[k] = 0.1 * rng.standard_normal(params[k].shape)
    # The GPU computes with BF16 copies of the weights: give the oracle the same values.
    p_bf = {k: _bf16_round(v).astype(np.float64) for k, v in params.items()}
    net = FNO2d(n, params=params, **cfg)
    a = rng.standard_normal((B, 3, n, n)).astype(np.float32)
    a = _bf16_round(a)
    target = rng.standard_normal((B, 3, n, n)).astype(np.float32)
    out, cache = net.forward(torch.tensor(a, device="cuda"))
    ref, rcache = ofno.forward(p_bf, a.astype(np.float64), cfg["modes"], cfg["layers"])
    assert rel_l2(out.cpu().numpy(), ref) < 1e-2
    loss, grad = net.mse(out, torch.tensor(target, device="cuda"))
    ref_loss, ref_grad = ofno.mse(ref, target.astype(np.float64))
    assert abs(loss - ref_loss) <= 2e-2 * ref_loss
    grads = net.backward(cache, grad)
    ref_grads = ofno.backward(p_bf, rcache, ref_grad, cfg["modes"], cfg["layers"])
    for k, g in ref_grads.items():
        assert rel_l2(grads[k].cpu().numpy(), g) < 1e-2, k


def test_adam_steps_reduce_the_loss(cuda_lib):
    import torch

    from polarism_gb300.fno import FNO2d

    cfg = _small()
    n, B = 32, 4
    rng = np.random.default_rng(2)
    a = torch.tensor(rng.standard_normal((B, 3, n, n)).astype(np.float32), device="cuda")
    x = np.linspace(-1, 1, n)
    tgt = np.stack([np.exp(-4 * (x[None, :] ** 2 + x[:, None] ** 2))] * 3)[None].repeat(B, 0)
    target = torch.tensor(tgt.astype(np.float32), device="cuda")
    net = FNO2d(n, seed=1, **cfg)
    losses = []
    for _ in range(40):
        out, cache = net.forward(a)
        loss, grad = net.mse(out, target)
        losses.append(loss)
        net.adam_step(net.backward(cache, grad), lr=3e-3)
    assert losses[-1] < 0.5 * losses[0] and losses[-1] < min(losses[:5]), losses[::8]


@pytest.mark.parametrize("engine", [0, 1])
def test_split_k_two_level_batch_and_slice_sum(cuda_lib, engine):
    """dW = sum_b G_b X_b^T with each sample's K split in slices through the inner batch level,
    summed in a fixed order (the weight-gradient path of the network)."""
    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    _lib.check(lib.pg_gemm_set_engine(engine), "pg_gemm_set_engine")
    rng = np.random.default_rng(7)
    B, M, N, P, chunk = 3, 32, 24, 4096 * 2, 4096
    g = _bf16_round(rng.standard_normal((B, M, P)))
    x = _bf16_round(rng.standard_normal((B, N, P)))
    G = torch.tensor(g, device="cuda").to(torch.bfloat16)
    X = torch.tensor(x, device="cuda").to(torch.bfloat16)
    S = P // chunk
    parts = torch.empty((B * S, M, N), device="cuda")
    _lib.check(lib.pg_gemm_bf16_2d(G.data_ptr(), X.data_ptr(), parts.data_ptr(), M, N, chunk, P, P, N, 0, 1,
                                   1.0, 0.0, B, M * P, N * P, S * M * N, S, chunk, chunk, M * N, None),
               "pg_gemm_bf16_2d")
    out = torch.full((M, N), 1.5, device="cuda")
    _lib.check(lib.pg_fno_sum_slices(parts.data_ptr(), out.data_ptr(), M * N, B * S, 1, None), "sum")
    expect = 1.5 + np.einsum("bmp,bnp->mn", g.astype(np.float64), x.astype(np.float64))
    assert rel_l2(out.cpu().numpy(), expect) < 1e-5
    _lib.check(lib.pg_gemm_set_engine(0), "pg_gemm_set_engine")
