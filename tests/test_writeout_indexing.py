"""CPU emulation of the sweep kernel's host write-out addressing
(sn_gpu_sweep_download): over all blocks of a lattice, the rows a CTA
writes -- 3*Bz floats starting at 3*(((x0+lx)*Y + y0+ly)*Z + z0) -- cover the
caller's 3*N-float buffer exactly once, and every tile slot read lies in the
block interior of the staged tile (halo coordinates H..H+B-1 on each axis)."""
import numpy as np
import pytest

import starrynight_gb300 as sn


@pytest.mark.parametrize("shape,rc", [((32, 32, 32), 3), ((48, 32, 64), 3), ((96, 64, 1), 3), ((24, 24, 24), 2),
                                      ((60, 60, 60), 5), ((16, 16, 16), 1)])
def test_block_rows_cover_the_buffer_once(native_lib, shape, rc):
    X, Y, Z = shape
    for c in sn.plan_candidates(X, Y, Z, rc, False, 4):
        bx, by, bz = c["bx"], c["by"], c["bz"]
        assert (X % bx, Y % by, Z % bz) == (0, 0, 0)
        hits = np.zeros(3 * X * Y * Z, np.int32)
        lx, ly = np.meshgrid(np.arange(bx), np.arange(by), indexing="ij")
        e = np.arange(3 * bz)
        for x0 in range(0, X, bx):
            for y0 in range(0, Y, by):
                for z0 in range(0, Z, bz):
                    o0 = 3 * (((x0 + lx) * Y + (y0 + ly)) * Z + (0 if Z == 1 else z0))
                    idx = (o0[..., None] + e).ravel()
                    assert idx.min() >= 0 and idx.max() < 3 * X * Y * Z
                    np.add.at(hits, idx, 1)
        assert np.all(hits == 1), (shape, rc, (bx, by, bz))
        # tile side: interior coordinates of the staged tile (block + halo)
        H, HZ = rc, (0 if Z == 1 else rc)
        Tx, Ty, Tz = bx + 2 * H, by + 2 * H, (1 if Z == 1 else bz + 2 * HZ)
        assert 0 <= H and H + bx - 1 < Tx and H + by - 1 < Ty and HZ + bz - 1 < Tz
