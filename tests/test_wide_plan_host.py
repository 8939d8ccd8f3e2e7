"""Index arithmetic of the full-width RK4 kernel's wide rows, checked on CPU: the shared-memory
row of band b holds grid columns b*1024 - 4 .. b*1024 + 1027 (periodic), fetched by one bulk
copy or two where the band wraps (the plan of ``issue()`` in csrc/rk4_wide.cu, restated here).
Every piece must start and end on 16 bytes for the 8-byte field and the 4-byte reservoir and
pump rows, and the pieces must cover the row exactly once."""
from __future__ import annotations

import pytest

NX_BAND, HALO = 1024, 4
W = NX_BAND + 2 * HALO


def row_copies(gnx, band):
    """(shared-memory column, grid column, columns) of each bulk copy of one row."""
    gc0 = band * NX_BAND - HALO
    first = HALO if gc0 < 0 else (gnx - gc0 if gc0 + W > gnx else W)
    src0 = gnx - HALO if gc0 < 0 else gc0
    pieces = [(0, src0, first)]
    if first < W:
        pieces.append((first, 0, W - first))
    return pieces


@pytest.mark.parametrize("gnx", [1024 * k for k in range(2, 17)])
def test_band_row_copies_cover_the_band_and_stay_aligned(gnx):
    for band in range(gnx // NX_BAND):
        covered = []
        for dst, src, cols in row_copies(gnx, band):
            assert cols > 0 and src + cols <= gnx and dst + cols <= W
            for elem in (8, 4):  # complex64 field, float32 reservoir and pump
                assert (src * elem) % 16 == 0 and (cols * elem) % 16 == 0
                assert (dst * elem) % 16 == 0
            covered += [(src + i) % gnx for i in range(cols)]
        want = [(band * NX_BAND - HALO + c) % gnx for c in range(W)]
        assert covered == want
        # The written columns (shared-memory 4 .. 1027) are exactly the band's own.
        assert covered[HALO:HALO + NX_BAND] == list(range(band * NX_BAND, (band + 1) * NX_BAND))


def test_ring_rows_keep_copies_on_16_bytes():
    # Ring slot s of the field starts at s * W * 8 bytes and the scalar rows at s * W * 4.
    for slot in range(8):
        assert (slot * W * 8) % 16 == 0 and (slot * W * 4) % 16 == 0
