"""The path kernel's k-window lookup for exits on a patch boundary and the
fixed range of Gaussian weights it visits, checked on the host
(fk_mesh_window evaluates the kernel's window table and comparison in FP64).

 - For points along every side of every patch of the 8x8 square-patch mesh
   (the config-2 shape, eps x spacing = 3 and 1), the window's k chain nodes
   are the k nodes nearest to the point (brute force over the patch chain, as
   the oracle's knn_select does).
 - Where a patch visits a fixed range around the nearest node (walk mode 2),
   every node within the weight cutoff of the point lies within that range:
   +-2 chain places for FP32 stepping (cutoff exp(-17.3)), +-4 for FP64
   (exp(-69)).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

K = 20
CUT = {0: 17.3, 1: 69.0}      # walk-mode field -> weight cutoff (FP32, FP64)
SPAN = {0: 2, 1: 4}


@pytest.fixture(scope="module")
def host(fk):
    c = fk.Context(device=-1, seed=1)
    yield c
    c.close()


def _side_points(chain, rect, spacing, per_side=48):
    """Points along each rectangle side that carries chain nodes, from one
    spacing before its first node to one after its last (within the side)."""
    pts = []
    for axis, coord in ((1, rect[0]), (0, rect[1]), (1, rect[2]), (0, rect[3])):
        if axis == 0:
            on = np.abs(chain[:, 1] - coord) < 1e-12
            along = chain[on, 0]
        else:
            on = np.abs(chain[:, 0] - coord) < 1e-12
            along = chain[on, 1]
        if along.size == 0:
            continue
        lo_side, hi_side = (rect[0], rect[2]) if axis == 0 else (rect[1], rect[3])
        lo = max(along.min() - spacing, lo_side)
        hi = min(along.max() + spacing, hi_side)
        for v in np.linspace(lo, hi, per_side):
            pts.append((v, coord) if axis == 0 else (coord, v))
    return np.array(pts)


@pytest.mark.parametrize("eps_sp", [3.0, 1.0])
def test_window_is_k_nearest_and_span_holds(host, fk, eps_sp):
    from oracle_py import square_patch_mesh
    ref = square_patch_mesh((0, 0, 1, 1), 8, 31, 0.25)
    spacing = float(ref["spacing"])
    e2 = (eps_sp / spacing) ** 2
    mesh = host.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, eps_sp, K)
    nxy, _ = host.mesh_nodes(mesh)
    checked = span_checked = 0
    for s, patch in enumerate(ref["patches"]):
        gids = host.mesh_stencil_nodes(mesh, s)
        chain = nxy[gids]
        m = len(chain)
        rect = patch["rect"]
        closed = rect[0] > 0 and rect[1] > 0 and rect[2] < 1 and rect[3] < 1
        for x, y in _side_points(chain, rect, spacing):
            L, nearest, walk = host.mesh_window(mesh, s, x, y)
            d2 = (chain[:, 0] - x) ** 2 + (chain[:, 1] - y) ** 2
            order = np.argsort(d2, kind="stable")
            if d2[order[K]] - d2[order[K - 1]] < 1e-12 * max(d2[order[K]], 1e-300):
                continue  # a tie at the k-th distance: either window is the k nearest
            win = {(L + i) % m for i in range(K)} if closed else set(range(L, L + K))
            assert (closed or 0 <= L <= m - K), (s, L, m)
            assert win == set(order[:K].tolist()), (s, x, y, L)
            checked += 1
            for field in (0, 1):
                if (walk >> (2 * field)) & 3 != 2:
                    continue
                near = np.flatnonzero(e2 * d2 < CUT[field])
                off = np.abs(near - nearest)
                if closed:
                    off = np.minimum(off, m - off)
                assert off.max(initial=0) <= SPAN[field], (s, x, y, field, off.max())
                span_checked += 1
    assert checked > 5000
    if eps_sp == 3.0:
        assert span_checked > 5000  # both FP32 and FP64 use the fixed range at this shape
