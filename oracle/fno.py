"""FP64 NumPy Fourier neural operator: the CPU oracle for the warm-start network.

Test infrastructure only: the tests check the GPU forward and backward passes against it.
Nothing in the product imports this module.

The reference has no learned component; this is the architecture the warm start is built on
(Li et al., "Fourier Neural Operator for Parametric PDEs", 2021): a pointwise lift to ``width``
channels, ``layers`` Fourier layers ``v <- act(K v + W v + b)`` whose spectral convolution keeps
the lowest ``modes`` x-frequencies and the ``modes`` lowest positive and negative y-frequencies
of ``rfft2``, multiplying each kept mode by a complex ``width x width`` matrix, then a pointwise
projection ``width -> hidden -> outputs`` with one activation.  The activation is the tanh form
of GELU.  Channels-first arrays ``(batch, channels, ny, nx)``.
"""
from __future__ import annotations

import numpy as np

GELU_C = np.sqrt(2.0 / np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    u = GELU_C * (x + 0.044715 * x ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3 * 0.044715 * x * x)


def kept_rows(ny, modes):
    """Indices of the kept y-frequencies: 0..modes-1 and ny-modes..ny-1."""
    return np.concatenate([np.arange(modes), np.arange(ny - modes, ny)])


def init_params(c_in, c_out, width=32, modes=16, layers=4, hidden=128, seed=0):
    rng = np.random.default_rng(seed)
    p = {"lift_w": rng.standard_normal((width, c_in)) / np.sqrt(c_in), "lift_b": np.zeros(width)}
    scale = 1.0 / (width * width)
    for l in range(layers):
        p[f"spec{l}_re"] = scale * rng.uniform(-1, 1, (2 * modes, modes, width, width))
        p[f"spec{l}_im"] = scale * rng.uniform(-1, 1, (2 * modes, modes, width, width))
        p[f"w{l}"] = rng.standard_normal((width, width)) / np.sqrt(width)
        p[f"b{l}"] = np.zeros(width)
    p["proj1_w"] = rng.standard_normal((hidden, width)) / np.sqrt(width)
    p["proj1_b"] = np.zeros(hidden)
    p["proj2_w"] = rng.standard_normal((c_out, hidden)) / np.sqrt(hidden)
    p["proj2_b"] = np.zeros(c_out)
    return p


def _pointwise(w, b, v):
    return np.einsum("oi,bi...->bo...", w, v) + b.reshape((1, -1) + (1,) * (v.ndim - 2))


def _spectral(re, im, v, modes):
    """K v: rfft2, per-mode complex matrix on the kept modes, irfft2.  Weight layout
    [kept ky (2 modes)][kx (modes)][in][out]."""
    ny, nx = v.shape[-2:]
    vh = np.fft.rfft2(v, axes=(-2, -1))
    rows = kept_rows(ny, modes)
    sub = vh[:, :, rows, :modes]                            # (B, in, 2m, m)
    w = re + 1j * im                                        # (2m, m, in, out)
    out_sub = np.einsum("biyx,yxio->boyx", sub, w)
    oh = np.zeros((v.shape[0], w.shape[-1], ny, nx // 2 + 1), dtype=complex)
    oh[:, :, rows, :modes] = out_sub
    return np.fft.irfft2(oh, s=(ny, nx), axes=(-2, -1)), sub


def forward(p, a, modes=16, layers=4):
    """Returns the output and the cache the backward pass needs."""
    cache = {"a": a}
    v = _pointwise(p["lift_w"], p["lift_b"], a)
    for l in range(layers):
        cache[f"v{l}"] = v
        ks, sub = _spectral(p[f"spec{l}_re"], p[f"spec{l}_im"], v, modes)
        cache[f"sub{l}"] = sub
        u = ks + _pointwise(p[f"w{l}"], p[f"b{l}"], v)
        cache[f"u{l}"] = u
        v = gelu(u) if l < layers - 1 else u
    cache["v_last"] = v
    h = _pointwise(p["proj1_w"], p["proj1_b"], v)
    cache["h"] = h
    q = gelu(h)
    cache["q"] = q
    out = _pointwise(p["proj2_w"], p["proj2_b"], q)
    return out, cache


def _pointwise_back(w, v, du):
    dw = np.einsum("boyx,biyx->oi", du, v)
    db = du.sum(axis=tuple(i for i in range(du.ndim) if i != 1))
    dv = np.einsum("oi,bo...->bi...", w, du)
    return dw, db, dv


def _spectral_back(re, im, sub, du, modes):
    """Adjoint of _spectral with respect to the input and the weights."""
    ny, nx = du.shape[-2:]
    rows = kept_rows(ny, modes)
    # irfft2 adjoint: d(out_hat) = rfft2-like projection with the Hermitian weights.
    dh = np.fft.rfft2(du, axes=(-2, -1)) / (ny * nx)
    weight = np.full(nx // 2 + 1, 2.0)
    weight[0] = 1.0
    if nx % 2 == 0:
        weight[-1] = 1.0
    dh = dh * weight                                        # gradient w.r.t. re/im of out_hat
    dsub_out = dh[:, :, rows, :modes]                       # (B, out, 2m, m)
    w = re + 1j * im
    dw = np.einsum("biyx,boyx->yxio", np.conj(sub), dsub_out)
    dsub = np.einsum("boyx,yxio->biyx", dsub_out, np.conj(w))
    vh_grad = np.zeros((du.shape[0], re.shape[2], ny, nx // 2 + 1), dtype=complex)
    vh_grad[:, :, rows, :modes] = dsub
    # rfft2 adjoint: real part of the full inverse transform of the one-sided gradient.
    full = np.zeros((du.shape[0], re.shape[2], ny, nx), dtype=complex)
    full[..., : nx // 2 + 1] = vh_grad
    dv = np.real(np.fft.fft2(np.conj(full), axes=(-2, -1)))
    return dw.real, dw.imag, dv


def backward(p, cache, dout, modes=16, layers=4):
    """Gradients of sum(dout * out) with respect to every parameter."""
    g = {}
    g["proj2_w"], g["proj2_b"], dq = _pointwise_back(p["proj2_w"], cache["q"], dout)
    dh = dq * gelu_grad(cache["h"])
    g["proj1_w"], g["proj1_b"], dv = _pointwise_back(p["proj1_w"], cache["v_last"], dh)
    for l in reversed(range(layers)):
        du = dv * gelu_grad(cache[f"u{l}"]) if l < layers - 1 else dv
        g[f"w{l}"], g[f"b{l}"], dv_point = _pointwise_back(p[f"w{l}"], cache[f"v{l}"], du)
        g[f"spec{l}_re"], g[f"spec{l}_im"], dv_spec = _spectral_back(
            p[f"spec{l}_re"], p[f"spec{l}_im"], cache[f"sub{l}"], du, modes)
        dv = dv_point + dv_spec
    g["lift_w"], g["lift_b"], _ = _pointwise_back(p["lift_w"], cache["a"], dv)
    return g


def mse(out, target):
    """Mean squared error and its gradient."""
    diff = out - target
    return float(np.mean(diff * diff)), 2.0 * diff / diff.size
