"""Host-side setup of the product library (no GPU): the circle mesh must equal
the reference's Malla/Interfaz/SistemaLineal construction bit for bit
(golden fixtures from the reference), and the square-patch mesh must satisfy
its structural invariants."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.mark.parametrize("name", ["serial", "unit3"])
def test_circle_mesh_matches_reference(host_ctx, name):
    g = np.load(os.path.join(GOLDEN, f"mesh_{name}.npz"))
    Nl, sup, th0, npc, c2c, c2s = g["cfg"]
    mid = host_ctx.mesh_circles(g["dom"], int(Nl), sup, th0, int(npc), c2c, c2s)
    info = host_ctx.mesh_info(mid)
    xy, flags = host_ctx.mesh_nodes(mid)
    assert info["n_nodes"] == len(g["node_int"])
    order = np.argsort(g["node_int"][:, 0])
    assert np.array_equal(xy, g["node_dbl"][order][:, :2])
    # frontera of arc end points (full-circle nodes are false in both)
    assert np.array_equal(flags, g["node_int"][order][:, 3])
    rp, col, v0 = host_ctx.mesh_csr(mid)
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(col, g["col"]) and np.array_equal(v0, g["val0"])
    # stencils: node ids per circle, and FK items = interior nodes of perimeter circles in reference order
    ii = g["iface_int"]
    off = 0
    exp_rows, exp_st = [], []
    ioff = 0
    for k in range(len(ii)):
        n, n_in = int(ii[k, 2]), int(ii[k, 3])
        assert np.array_equal(host_ctx.mesh_stencil_nodes(mid, k), g["iface_gids"][off:off + n])
        if ii[k, 1]:
            exp_rows += list(g["iface_inner"][ioff:ioff + n_in])
            exp_st += [k] * n_in
        off += n
        ioff += n_in
    row, ixy, st, fr = host_ctx.mesh_items(mid)
    assert list(row) == exp_rows and list(st) == exp_st


def test_square_patch_mesh_structure(host_ctx):
    n_sub, nps, e = 8, 31, 0.25
    mid = host_ctx.mesh_square_patches((0, 0, 1, 1), n_sub, nps, e, 3.0, 20)
    info = host_ctx.mesh_info(mid)
    H = 1.0 / n_sub
    assert abs(info["spacing"] - (1 + 2 * e) * H / (nps + 1)) < 1e-15
    xy, _ = host_ctx.mesh_nodes(mid)
    assert np.all((xy > 0) & (xy < 1))
    row, ixy, st, fr = host_ctx.mesh_items(mid)
    assert np.array_equal(ixy, xy[row])
    rp, col, v0 = host_ctx.mesh_csr(mid)
    # each item's node is strictly inside its patch and on another patch's boundary
    counts = np.bincount(row, minlength=info["n_rows"])
    for s in range(info["n_stencils"]):
        a, b = divmod(s, n_sub)
        r = ((a - e) * H, (b - e) * H, (a + 1 + e) * H, (b + 1 + e) * H)
        sel = st == s
        p = ixy[sel]
        assert np.all((p[:, 0] > r[0]) & (p[:, 0] < r[2]) & (p[:, 1] > r[1]) & (p[:, 1] < r[3]))
        gids = host_ctx.mesh_stencil_nodes(mid, s)
        assert not np.isin(row[sel], gids).any()
    # every node has at least one equation; the diagonal counts the containing patches
    assert counts.min() >= 1
    diag = np.array([v0[rp[i]:rp[i + 1]][col[rp[i]:rp[i + 1]] == i][0] for i in range(info["n_rows"])])
    assert np.array_equal(diag, counts.astype(float))
    # CSR rows sorted, pattern symmetric
    for i in range(info["n_rows"]):
        c = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(c) > 0)
    S = set(zip(np.repeat(np.arange(info["n_rows"]), np.diff(rp)), col))
    assert all((j, i) in S for (i, j) in S)


def test_mesh_argument_errors(host_ctx, fk):
    with pytest.raises(fk.FKError) as e:
        host_ctx.mesh_circles((0, 0, 1, 1), 1, 1.2, 0.1, 20)
    assert e.value.code == fk.FK_ERR_ARG
    with pytest.raises(fk.FKError):
        host_ctx.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.6, 3.0, 20)
    with pytest.raises(fk.FKError):
        host_ctx.mesh_square_patches((0, 0, 1, 1), 2, 5, 0.25, 3.0, 20)  # fewer nodes than the stencil


@pytest.mark.parametrize("n_sub,nps", [(8, 31), (3, 9), (4, 15)])
def test_oracle_square_patch_layout_equals_product(host_ctx, orc, n_sub, nps):
    """The CPU side's numpy restatement of the square-patch layout (used by
    the timed CPU baseline, which must not load the product library) gives the
    product's nodes, patch chains and items exactly."""
    m = orc.square_patch_mesh((0, 0, 1, 1), n_sub, nps, 0.25)
    mid = host_ctx.mesh_square_patches((0, 0, 1, 1), n_sub, nps, 0.25, 3.0, 6)
    info = host_ctx.mesh_info(mid)
    xy, _ = host_ctx.mesh_nodes(mid)
    assert np.array_equal(xy, m["nodes"])
    assert m["spacing"] == info["spacing"]
    row, ixy, st, fr = host_ctx.mesh_items(mid)
    it = np.array(m["items"])
    assert np.array_equal(row, it[:, 0]) and np.array_equal(st, it[:, 1])
    for s, p in enumerate(m["patches"]):
        assert np.array_equal(host_ctx.mesh_stencil_nodes(mid, s), p["gids"])
