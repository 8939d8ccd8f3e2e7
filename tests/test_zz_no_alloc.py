"""The allocation-free norm entry point against the allocating one (GPU).

Callers that must not allocate device memory -- for example code running beside another
framework's pooling allocator that owns the device memory, or a stepping loop that cannot
pay for the synchronisation cudaMalloc/cudaFree imply -- call pg_field_norms_noalloc, whose
per-block partial sums live in a fixed device array instead of per-call allocations.  This
file is collected last so a failure here never hides another test's result; it also passes
when run alone in a fresh process.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _norms(lib, fn, psi, prec, members, sites, cell):
    import torch

    from polarism_gb300 import _lib

    out = torch.full((members,), -1.0, dtype=torch.float64, device="cuda")
    _lib.check(getattr(lib, fn)(psi.data_ptr(), prec, members, sites, cell, out.data_ptr(), None), fn)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_norms_match_allocating_entry_point_twice():
    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    assert lib.pg_device_count() >= 1
    rng = np.random.default_rng(123)
    cases = [(torch.complex64, _lib.PG_SINGLE, 5, (48, 64), 0.39),
             (torch.complex128, _lib.PG_DOUBLE, 3, (1024, 1024), 0.1526)]
    for dtype, prec, members, (ny, nx), cell in cases:   # two calls in a row, different shapes
        host = rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx))
        psi = torch.as_tensor(host, dtype=dtype, device="cuda")
        expect = _norms(lib, "pg_field_norms", psi, prec, members, ny * nx, cell)
        got = _norms(lib, "pg_field_norms_noalloc", psi, prec, members, ny * nx, cell)
        np.testing.assert_allclose(got, expect, rtol=1e-12, atol=0)


def test_noalloc_norms_with_fewer_blocks_than_the_allocating_call_match_fp64_numpy():
    """48 members of 512 x 1024 sites: the allocating call uses 256 blocks a member, the
    fixed array holds only 8192 / 48 = 170, so this case runs the clamped block count.  Both
    calls are checked against FP64 NumPy sums of the same values, twice in a row."""
    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(7)
    members, ny, nx, cell = 48, 512, 1024, 0.25
    host = (rng.standard_normal((members, 1, ny, nx)) +
            1j * rng.standard_normal((members, 1, ny, nx))).astype(np.complex64)
    psi = torch.as_tensor(host, device="cuda")
    h64 = host.astype(np.complex128)
    expect = (np.abs(h64) ** 2).reshape(members, -1).sum(axis=1) * cell
    for _ in range(2):
        got = _norms(lib, "pg_field_norms_noalloc", psi, _lib.PG_SINGLE, members, ny * nx, cell)
        np.testing.assert_allclose(got, expect, rtol=1e-12, atol=0)
    np.testing.assert_allclose(_norms(lib, "pg_field_norms", psi, _lib.PG_SINGLE, members, ny * nx, cell),
                               expect, rtol=1e-12, atol=0)


def test_noalloc_rejects_more_members_than_the_scratch_holds():
    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    psi = torch.zeros(8193, dtype=torch.complex64, device="cuda")
    out = torch.zeros(8193, dtype=torch.float64, device="cuda")
    status = lib.pg_field_norms_noalloc(psi.data_ptr(), _lib.PG_SINGLE, 8193, 1, 1.0, out.data_ptr(), None)
    assert status == _lib.PG_ERR_INVALID
    assert b"8192" in lib.pg_last_error()
