"""G rows formed in the path kernel in warp mode (items of few paths, FP32
stepping, the 20-nearest Gaussian patch stencil): the warp that ran an item
forms the item's row from its moments in global memory and zeroes them again,
so the next such launch needs no memset.

 - Warp mode against slot mode on the same Philox stream (the same paths,
   hence the same exits; only the order of the FP32 moment sums differs).
   Both count the same stencil windows formed into rows (fk_last_windows).
 - A second warp-mode launch on the same stream gives the same system, also
   after an FP64 assembly (which leaves moments in the buffer) in between:
   nothing of one launch's moments reaches the next.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _assemble(gpu, fk, mesh, b, paths, h, prec, stream):
    gpu.set_stream(stream)
    r = gpu.assemble(mesh, b, paths, h, prec, items=True, item_G=True)
    return r["val"], r["B"], r["item_G"]


@pytest.mark.parametrize("eps_sp", [3.0, 1.0])
def test_warp_mode_rows_match_slot_mode(gpu, fk, eps_sp):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, eps_sp, 20)  # 10,584 items: one chunk each
    b = gpu.register_bvp(fk.ANISO)
    paths, h = 300, 1e-3
    v_w, B_w, G_w = _assemble(gpu, fk, mesh, b, paths, h, fk.FP32, 41)
    win_w = gpu.last_windows()
    gpu.set_launch(256, 1 << 20)  # one chunk per item in the shared slots
    try:
        v_s, B_s, G_s = _assemble(gpu, fk, mesh, b, paths, h, fk.FP32, 41)
        win_s = gpu.last_windows()
    finally:
        gpu.set_launch(0, 0)
    # the same exits choose the same windows (fk_last_windows: windows formed into rows)
    assert win_s > 0 and abs(win_w - win_s) <= 1e-3 * win_s
    scale = np.abs(v_s).max()
    assert np.abs(v_w - v_s).max() <= 2e-6 * scale
    # (B_r sums items' estimates of both signs: compared on its overall scale;
    # the FP32 per-lane sums run over other subsets of the paths)
    assert np.abs(B_w - B_s).max() <= 2e-6 * np.abs(B_s).max()
    assert np.abs(G_w - G_s).max() <= 2e-6 * np.abs(G_s).max()


def test_warp_mode_moments_do_not_leak_into_the_next_launch(gpu, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, 3.0, 20)
    b = gpu.register_bvp(fk.ANISO)
    paths, h = 300, 1e-3
    first = _assemble(gpu, fk, mesh, b, paths, h, fk.FP32, 77)
    again = _assemble(gpu, fk, mesh, b, paths, h, fk.FP32, 77)
    for x, y in zip(first, again):
        assert np.allclose(x, y, rtol=1e-12, atol=1e-15)
    _assemble(gpu, fk, mesh, b, paths, h, fk.FP64, 78)  # moments left in the accumulators
    after = _assemble(gpu, fk, mesh, b, paths, h, fk.FP32, 77)
    for x, y in zip(first, after):
        assert np.allclose(x, y, rtol=1e-12, atol=1e-15)
