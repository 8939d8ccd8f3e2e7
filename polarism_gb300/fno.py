"""Fourier neural operator trained and run on the GB300 kernels of ``csrc/fno.cu``.

The learned warm start maps a pump (its profile and strength, plus the coordinates) to a
steady state ``(psi, n_R)``; the plain solver then integrates from it and judges it
(:mod:`polarism_gb300.warmstart`).  Polarism has no learned component, so nothing here
replaces reference code.

Architecture (Li et al. 2021): pointwise lift to ``width`` channels, ``layers`` Fourier layers
``v <- GELU(K v + W v + b)`` (no activation after the last), pointwise projection
``width -> hidden -> outputs`` with one GELU.  The spectral convolution ``K`` keeps the lowest
``modes`` x-frequencies and the ``modes`` lowest positive and negative y-frequencies.  It is
computed without FFTs as truncated DFTs, i.e. GEMMs: along x ``X = v F_x`` (real to ``modes``
complex columns), along y ``Y = G X`` (``2 modes`` complex rows), the per-mode complex
``width x width`` mixing, ``Z = G^H O`` and ``u = Z H_x`` (the one-sided inverse).  The
backward pass runs the transposed GEMMs.  Every GEMM has BF16 operands and FP32 accumulators
(``pg_gemm_bf16``); activations and master weights stay FP32, with BF16 copies for the GEMMs;
Adam updates the FP32 weights and refreshes the BF16 copies.  PyTorch only allocates device
memory and provides the stream; every arithmetic operation is one of this package's kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from polarism_gb300 import _lib


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def kept_rows(n, modes):
    return np.concatenate([np.arange(modes), np.arange(n - modes, n)])


def init_params(c_in, c_out, width=32, modes=16, layers=4, hidden=128, seed=0):
    """FP64 initial parameters (the layout the FNO oracle uses): spectral weights
    [kept ky][kx][in][out] uniform in +-1/width^2, pointwise weights scaled by 1/sqrt(fan-in)."""
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


class FNO2d:
    """The network on one GPU: parameters, Adam state and the forward/backward passes."""

    def __init__(self, n, c_in=3, c_out=3, width=32, modes=16, layers=4, hidden=128, params=None,
                 seed=0):
        import torch

        self.torch = torch
        self.lib = _lib.load()
        self.n, self.c_in, self.c_out = int(n), int(c_in), int(c_out)
        self.width, self.modes, self.layers, self.hidden = int(width), int(modes), int(layers), int(hidden)
        if 2 * self.modes > self.n or self.modes > self.n // 2:
            raise ValueError("modes must be at most n / 2")
        dev = torch.device("cuda")
        self.device = dev
        host = params if params is not None else init_params(c_in, c_out, width, modes, layers, hidden, seed)
        self.names = list(host)
        # torch.tensor keeps NumPy's strides: hand it C-ordered copies, the kernels index linearly.
        self.w = {k: torch.tensor(np.ascontiguousarray(v, dtype=np.float32), device=dev)
                  for k, v in host.items()}
        self.w_bf = {k: torch.empty(v.shape, dtype=torch.bfloat16, device=dev) for k, v in self.w.items()}
        for k in self.names:
            self._bf(self.w[k], self.w_bf[k])
        self.m1 = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.m2 = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.steps = 0
        self._dft_tables()

    # ------------------------------------------------------------------ kernels
    @property
    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _check(self, rc, what):
        _lib.check(rc, what)

    def _bf(self, x, out):
        if not (x.is_contiguous() and out.is_contiguous()):
            raise ValueError("FNO kernels need contiguous tensors")
        self._check(self.lib.pg_fno_to_bf16(_ptr(x), _ptr(out), x.numel(), self.stream), "pg_fno_to_bf16")
        return out

    def _gemm(self, A, B, Cm, M, N, K, lda, ldb, ldc, ta=0, tb=0, alpha=1.0, beta=0.0, batch=1,
              sA=0, sB=0, sC=0, a_off=0, b_off=0, c_off=0):
        a = C.c_void_p(A.data_ptr() + 2 * a_off)
        b = C.c_void_p(B.data_ptr() + 2 * b_off)
        c = C.c_void_p(Cm.data_ptr() + 4 * c_off)
        self._check(self.lib.pg_gemm_bf16(a, b, c, M, N, K, lda, ldb, ldc, ta, tb, float(alpha),
                                          float(beta), batch, sA, sB, sC, self.stream), "pg_gemm_bf16")

    def _dft_tables(self):
        torch = self.torch
        n, m = self.n, self.modes
        x = np.arange(n)
        k = np.arange(m)
        ang = 2 * np.pi * np.outer(x, k) / n                       # (n, m)
        fx = np.concatenate([np.cos(ang), -np.sin(ang)], axis=1)   # X = v Fx: [re | im]
        rows = kept_rows(n, m)
        angy = 2 * np.pi * np.outer(rows, x) / n                   # (2m, n)
        gre, gim = np.cos(angy), -np.sin(angy)                      # G = exp(-i ky y)
        wk = np.where(k == 0, 1.0, 2.0)[:, None]
        hx = np.concatenate([wk * np.cos(ang.T), -wk * np.sin(ang.T)], axis=0) / (n * n)  # (2m, n)
        def bf(a):  # built in FP64 on the host, rounded once to BF16 on the device
            x = torch.tensor(np.ascontiguousarray(a, dtype=np.float32), device=self.device)
            return self._bf(x, torch.empty(x.shape, dtype=torch.bfloat16, device=self.device))

        self.fx, self.gre, self.gim, self.hx = bf(fx), bf(gre), bf(gim), bf(hx)

    # ------------------------------------------------------------------ building blocks
    def _pointwise(self, wname, bname, v_bf, batch, cin, cout, out, gelu, act=None, act_bf=None,
                   accumulate=False):
        P = self.n * self.n
        self._gemm(self.w_bf[wname], v_bf, out, cout, P, cin, cin, P, P, batch=batch,
                   sB=cin * P, sC=cout * P, beta=1.0 if accumulate else 0.0)
        self._check(self.lib.pg_fno_bias_act(_ptr(out), _ptr(self.w[bname]),
                                             _ptr(act) if act is not None else None,
                                             _ptr(act_bf) if act_bf is not None else None, cout, P,
                                             out.numel(), 1 if gelu else 0, self.stream), "pg_fno_bias_act")

    def _cmul_y(self, src_bf, dst, batch, inverse):
        """Complex left products along y for `batch` matrices.  Forward (inverse=False):
        dst (2m x 2m) = G src (n x 2m).  Inverse: dst (n x 2m) = G^H src (2m x 2m).  Columns
        hold [re (m) | im (m)]."""
        n, m = self.n, self.modes
        if not inverse:
            rows, k, sB, sC, ta, lda = 2 * m, n, n * 2 * m, 4 * m * m, 0, n
            sign_im = -1.0  # dst_re = Gre s_re - Gim s_im, dst_im = Gre s_im + Gim s_re
        else:
            rows, k, sB, sC, ta, lda = n, 2 * m, 4 * m * m, n * 2 * m, 1, n
            sign_im = 1.0   # dst_re = Gre^T s_re + Gim^T s_im, dst_im = Gre^T s_im - Gim^T s_re
        common = dict(M=rows, N=m, K=k, lda=lda, ldb=2 * m, ldc=2 * m, ta=ta, batch=batch, sA=0, sB=sB, sC=sC)
        self._gemm(self.gre, src_bf, dst, b_off=0, c_off=0, alpha=1.0, beta=0.0, **common)
        self._gemm(self.gim, src_bf, dst, b_off=m, c_off=0, alpha=sign_im, beta=1.0, **common)
        self._gemm(self.gre, src_bf, dst, b_off=m, c_off=m, alpha=1.0, beta=0.0, **common)
        self._gemm(self.gim, src_bf, dst, b_off=0, c_off=m, alpha=-sign_im, beta=1.0, **common)

    def _empty(self, *shape, bf=False):
        torch = self.torch
        return torch.empty(shape, dtype=torch.bfloat16 if bf else torch.float32, device=self.device)

    # ------------------------------------------------------------------ forward / backward
    def forward(self, a, keep=True):
        """a: float32 device tensor (B, c_in, n, n).  Returns (out, cache)."""
        torch = self.torch
        B = a.shape[0]
        n, m, W = self.n, self.modes, self.width
        P = n * n
        cache = {"B": B}
        a_bf = self._bf(a.contiguous(), self._empty(B, self.c_in, n, n, bf=True))
        cache["a_bf"] = a_bf
        v = self._empty(B, W, n, n)
        v_bf = self._empty(B, W, n, n, bf=True)
        self._pointwise("lift_w", "lift_b", a_bf, B, self.c_in, W, v, False, act_bf=v_bf)
        for l in range(self.layers):
            cache[f"v{l}_bf"] = v_bf
            X = self._empty(B, W, n, 2 * m)
            self._gemm(v_bf, self.fx, X, B * W * n, 2 * m, n, n, 2 * m, 2 * m)
            X_bf = self._bf(X, self._empty(B, W, n, 2 * m, bf=True))
            Y = self._empty(B, W, 2 * m, 2 * m)
            self._cmul_y(X_bf, Y, B * W, inverse=False)
            cache[f"Y{l}"] = Y
            O = self._empty(B, W, 2 * m, 2 * m)
            self._check(self.lib.pg_fno_mode_mix(_ptr(Y), _ptr(self.w_bf[f"spec{l}_re"]),
                                                 _ptr(self.w_bf[f"spec{l}_im"]), _ptr(O), B, W, W, m,
                                                 self.stream), "pg_fno_mode_mix")
            O_bf = self._bf(O, self._empty(B, W, 2 * m, 2 * m, bf=True))
            Z = self._empty(B, W, n, 2 * m)
            self._cmul_y(O_bf, Z, B * W, inverse=True)
            Z_bf = self._bf(Z, self._empty(B, W, n, 2 * m, bf=True))
            u = self._empty(B, W, n, n)
            self._gemm(Z_bf, self.hx, u, B * W * n, n, 2 * m, 2 * m, n, n)
            last = l == self.layers - 1
            v_next = self._empty(B, W, n, n) if last else None
            v_next_bf = self._empty(B, W, n, n, bf=True)
            self._pointwise(f"w{l}", f"b{l}", v_bf, B, W, W, u, not last, act=v_next, act_bf=v_next_bf,
                            accumulate=True)
            cache[f"u{l}"] = u
            v_bf = v_next_bf
        cache["vL_bf"] = v_bf
        H = self.hidden
        h = self._empty(B, H, n, n)
        q_bf = self._empty(B, H, n, n, bf=True)
        self._pointwise("proj1_w", "proj1_b", v_bf, B, W, H, h, True, act_bf=q_bf)
        cache["h"], cache["q_bf"] = h, q_bf
        out = self._empty(B, self.c_out, n, n)
        self._pointwise("proj2_w", "proj2_b", q_bf, B, H, self.c_out, out, False)
        if not keep:
            cache = None
        return out, cache

    def _pointwise_back(self, wname, x_bf, g_bf, g32, batch, cin, cout, grads, dx=None, dx_accumulate=False):
        P = self.n * self.n
        # dW = sum over samples and sites of g x^T: a split-K GEMM (the samples and 4096-site
        # slices of the plane each give one partial product), then a fixed-order sum.
        chunk = 4096 if P % 4096 == 0 else P
        slices = P // chunk
        parts = self._empty(batch * slices, cout, cin)
        self._check(self.lib.pg_gemm_bf16_2d(
            _ptr(g_bf), _ptr(x_bf), _ptr(parts), cout, cin, chunk, P, P, cin, 0, 1, 1.0, 0.0,
            batch, cout * P, cin * P, slices * cout * cin, slices, chunk, chunk, cout * cin,
            self.stream), "pg_gemm_bf16_2d")
        dw = self._empty(cout, cin)
        self._check(self.lib.pg_fno_sum_slices(_ptr(parts), _ptr(dw), cout * cin, batch * slices, 0,
                                               self.stream), "pg_fno_sum_slices")
        grads[wname] = dw
        db = self._empty(cout)
        self._check(self.lib.pg_fno_channel_sum(_ptr(g32), _ptr(db), batch, cout, P, 0, self.stream),
                    "pg_fno_channel_sum")
        grads[wname.replace("_w", "_b") if wname.endswith("_w") else "b" + wname[1:]] = db
        if dx is not None:
            self._gemm(self.w_bf[wname], g_bf, dx, cin, P, cout, cin, P, P, ta=1, batch=batch,
                       sB=cout * P, sC=cin * P, beta=1.0 if dx_accumulate else 0.0)

    def backward(self, cache, dout):
        """Gradients of sum(dout * out); dout: float32 device tensor like the output."""
        B = cache["B"]
        n, m, W, H = self.n, self.modes, self.width, self.hidden
        grads = {}
        dout = dout.contiguous()
        dout_bf = self._bf(dout, self._empty(*dout.shape, bf=True))
        dq = self._empty(B, H, n, n)
        self._pointwise_back("proj2_w", cache["q_bf"], dout_bf, dout, B, H, self.c_out, grads, dx=dq)
        dh = self._empty(B, H, n, n)
        dh_bf = self._empty(B, H, n, n, bf=True)
        self._check(self.lib.pg_fno_gelu_backward(_ptr(cache["h"]), _ptr(dq), _ptr(dh), _ptr(dh_bf),
                                                  dh.numel(), self.stream), "pg_fno_gelu_backward")
        dv = self._empty(B, W, n, n)
        self._pointwise_back("proj1_w", cache["vL_bf"], dh_bf, dh, B, W, H, grads, dx=dv)
        for l in reversed(range(self.layers)):
            du = self._empty(B, W, n, n)
            du_bf = self._empty(B, W, n, n, bf=True)
            if l < self.layers - 1:
                self._check(self.lib.pg_fno_gelu_backward(_ptr(cache[f"u{l}"]), _ptr(dv), _ptr(du),
                                                          _ptr(du_bf), du.numel(), self.stream),
                            "pg_fno_gelu_backward")
            else:
                du = dv
                self._bf(du, du_bf)
            dv_new = self._empty(B, W, n, n)
            self._pointwise_back(f"w{l}", cache[f"v{l}_bf"], du_bf, du, B, W, W, grads, dx=dv_new)
            # Spectral adjoint: dZ = du Hx^T, dO = G dZ, (dY, dR) = mixing adjoint, dX = G^H dY,
            # dv += dX Fx^T.
            dZ = self._empty(B, W, n, 2 * m)
            self._gemm(du_bf, self.hx, dZ, B * W * n, 2 * m, n, n, n, 2 * m, tb=1)
            dZ_bf = self._bf(dZ, self._empty(B, W, n, 2 * m, bf=True))
            dO = self._empty(B, W, 2 * m, 2 * m)
            self._cmul_y(dZ_bf, dO, B * W, inverse=False)
            dY = self._empty(B, W, 2 * m, 2 * m)
            dre = self._empty(2 * m, m, W, W)
            dim = self._empty(2 * m, m, W, W)
            self._check(self.lib.pg_fno_mode_mix_backward(
                _ptr(cache[f"Y{l}"]), _ptr(dO), _ptr(self.w_bf[f"spec{l}_re"]), _ptr(self.w_bf[f"spec{l}_im"]),
                _ptr(dY), _ptr(dre), _ptr(dim), B, W, W, m, self.stream), "pg_fno_mode_mix_backward")
            grads[f"spec{l}_re"], grads[f"spec{l}_im"] = dre, dim
            dY_bf = self._bf(dY, self._empty(B, W, 2 * m, 2 * m, bf=True))
            dX = self._empty(B, W, n, 2 * m)
            self._cmul_y(dY_bf, dX, B * W, inverse=True)
            dX_bf = self._bf(dX, self._empty(B, W, n, 2 * m, bf=True))
            self._gemm(dX_bf, self.fx, dv_new, B * W * n, n, 2 * m, 2 * m, 2 * m, n, tb=1, beta=1.0)
            dv = dv_new
        dv_bf = self._bf(dv, self._empty(B, W, n, n, bf=True))
        self._pointwise_back("lift_w", cache["a_bf"], dv_bf, dv, B, self.c_in, W, grads)
        return grads

    # ------------------------------------------------------------------ training
    def adam_step(self, grads, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, decay=0.0):
        self.steps += 1
        for k in self.names:
            w = self.w[k]
            self._check(self.lib.pg_fno_adam(_ptr(w), _ptr(grads[k]), _ptr(self.m1[k]), _ptr(self.m2[k]),
                                             _ptr(self.w_bf[k]), w.numel(), float(lr), float(betas[0]),
                                             float(betas[1]), float(eps), self.steps, float(decay),
                                             self.stream), "pg_fno_adam")

    def mse(self, out, target, channel_weight=None, want_grad=True):
        """(loss, grad): mean over all values of w_c (out - target)^2 (FP64 reduction)."""
        torch = self.torch
        n_el = out.numel()
        partials = torch.empty(4096, dtype=torch.float64, device=self.device)
        grad = self._empty(*out.shape) if want_grad else None
        used = C.c_int32()
        wptr = _ptr(channel_weight) if channel_weight is not None else None
        self._check(self.lib.pg_fno_mse(_ptr(out), _ptr(target.contiguous()), wptr, self.c_out,
                                        self.n * self.n, _ptr(grad) if grad is not None else None, None,
                                        _ptr(partials), 4096, n_el, 1.0 / n_el, C.byref(used),
                                        self.stream), "pg_fno_mse")
        loss = float(partials[:used.value].sum().item()) / n_el
        return loss, grad

    def state_dict(self):
        return {k: v.detach().cpu().numpy().astype(np.float64) for k, v in self.w.items()}
