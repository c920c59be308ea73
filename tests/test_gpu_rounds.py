"""Adaptive assembly in rounds (fk_assembly_begin / round / end): the path
sums stay on the device between rounds, and the end pass forms each item's
path-weighted G row and B.

On a 4 x 4 square-patch mesh in FP64, against the oracle's node solves on
each round's Philox stream (item i, path p of the round with stream id s uses
the counter (step, p, i, s), as one fk_assemble call does):
 - after one round, G rows and B equal the oracle's for that round's paths;
 - after a second round (other path counts, some items given none), they
   equal the path-weighted combination of the two rounds' oracle solves,
   (N1 G1 + N2 G2) / (N1 + N2), and the CSR values and B are those rows
   scattered as SistemaLineal::Actualiza_GB does;
 - a round whose items mix the plain BVP and the exact-gradient control
   variate equals the oracle item by item with each item's own BVP.
FP32 rounds are paired with FP64 rounds on the same streams."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20251203
N_SUB, NPS, ENL, K = 4, 15, 0.25, 20


def _rect(s):
    H = 1.0 / N_SUB
    a, b = divmod(int(s), N_SUB)
    return ((a - ENL) * H, (b - ENL) * H, (a + 1 + ENL) * H, (b + 1 + ENL) * H)


def _oracle_round(gpu, orc, mesh, stream, paths, cvs, h, eps):
    """Per-item oracle (G row, B) of one round; items given no paths: None."""
    row, ixy, stn, fr = gpu.mesh_items(mesh)
    nxy, _ = gpu.mesh_nodes(mesh)
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=stream)
    out = []
    for i in range(len(row)):
        if paths[i] == 0:
            out.append(None)
            continue
        gids = gpu.mesh_stencil_nodes(mesh, stn[i])
        G, Bv, _, _ = s.node_solve_knn(orc.bvp(2, cv=int(cvs[i])), ixy[i, 0], ixy[i, 1], _rect(stn[i]), nxy[gids], K,
                                       eps, int(paths[i]), h, item=i)
        out.append((G, Bv))
    return out


def _combine(rounds, paths_list, n):
    G, B = [], []
    for i in range(n):
        tot = sum(int(p[i]) for p in paths_list)
        g = sum(int(p[i]) * r[i][0] for r, p in zip(rounds, paths_list) if r[i] is not None)
        b = sum(int(p[i]) * r[i][1] for r, p in zip(rounds, paths_list) if r[i] is not None)
        G.append(g / tot)
        B.append(b / tot)
    return np.concatenate(G), np.array(B)


@pytest.mark.parametrize("eps_sp", [3.0, 1.0])
def test_rounds_fp64_match_oracle(gpu, orc, fk, eps_sp):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, eps_sp, K)
    info = gpu.mesh_info(mesh)
    n = info["n_items"]
    eps = eps_sp / info["spacing"]
    h = 5e-4
    b = gpu.register_bvp(fk.ANISO)
    rng = np.random.default_rng(3)
    p1 = rng.integers(60, 200, n).astype(np.uint32)
    p2 = np.where(rng.random(n) < 0.3, 0, rng.integers(40, 120, n)).astype(np.uint32)
    gpu.assembly_begin(mesh)
    gpu.set_stream(501)
    gpu.assembly_round(mesh, b, p1, h, fk.FP64)
    r1 = gpu.assembly_end(mesh)
    o1 = _oracle_round(gpu, orc, mesh, 501, p1, np.zeros(n), h, eps)
    G1, B1 = _combine([o1], [p1], n)
    assert np.allclose(r1["item_B"], B1, rtol=1e-9, atol=1e-12)
    assert np.allclose(r1["item_G"], G1, rtol=1e-9, atol=1e-9)
    assert np.all(r1["item_stats"]["n_paths"] == p1)
    gpu.set_stream(502)
    var = gpu.assembly_round(mesh, b, p2, h, fk.FP64)
    assert np.all(var[p2 > 0] > 0) and np.all(var[p2 == 0] == 0)
    r2 = gpu.assembly_end(mesh)
    o2 = _oracle_round(gpu, orc, mesh, 502, p2, np.zeros(n), h, eps)
    G12, B12 = _combine([o1, o2], [p1, p2], n)
    assert np.allclose(r2["item_B"], B12, rtol=1e-9, atol=1e-12)
    assert np.allclose(r2["item_G"], G12, rtol=1e-9, atol=1e-9)
    assert np.all(r2["item_stats"]["n_paths"] == p1 + p2)
    # CSR values and B: the combined rows scattered (Actualiza_GB)
    rp, col, v0 = gpu.mesh_csr(mesh)
    row, _, stn, _ = gpu.mesh_items(mesh)
    val, Bs = v0.copy(), np.zeros(info["n_rows"])
    off = 0
    for i in range(n):
        gids = gpu.mesh_stencil_nodes(mesh, stn[i])
        for j, g in enumerate(gids):
            val[rp[row[i]] + np.searchsorted(col[rp[row[i]]:rp[row[i] + 1]], g)] += G12[off + j]
        Bs[row[i]] += B12[i]
        off += len(gids)
    assert np.allclose(r2["val"], val, rtol=1e-9, atol=1e-9)
    assert np.allclose(r2["B"], Bs, rtol=1e-9, atol=1e-12)


def test_round_with_mixed_control_variates_matches_oracle(gpu, orc, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, 3.0, K)
    info = gpu.mesh_info(mesh)
    n = info["n_items"]
    b0 = gpu.register_bvp(fk.ANISO)
    b1 = gpu.register_bvp(fk.ANISO, cv=fk.CV_EXACT)
    cvs = (np.arange(n) % 2).astype(np.int32)
    bv = np.where(cvs == 1, b1, b0).astype(np.int32)
    p = np.full(n, 150, dtype=np.uint32)
    gpu.assembly_begin(mesh)
    gpu.set_stream(601)
    gpu.assembly_round(mesh, b0, p, 5e-4, fk.FP64, bvp_of_item=bv)
    r = gpu.assembly_end(mesh)
    o = _oracle_round(gpu, orc, mesh, 601, p, cvs, 5e-4, 3.0 / info["spacing"])
    G, B = _combine([o], [p], n)
    assert np.allclose(r["item_B"], B, rtol=1e-9, atol=1e-12)
    assert np.allclose(r["item_G"], G, rtol=1e-9, atol=1e-9)


def test_rounds_fp32_paired_with_fp64(gpu, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, 3.0, K)
    n = gpu.mesh_info(mesh)["n_items"]
    b = gpu.register_bvp(fk.ANISO)
    out = {}
    for prec in (fk.FP64, fk.FP32):
        gpu.assembly_begin(mesh)
        for sid, N in ((701, 2000), (702, 3000)):
            gpu.set_stream(sid)
            gpu.assembly_round(mesh, b, np.full(n, N, dtype=np.uint32), 5e-4, prec)
        out[prec] = gpu.assembly_end(mesh)
    r64, r32 = out[fk.FP64], out[fk.FP32]
    se = np.sqrt(np.maximum(r64["item_stats"]["phiphi"] - r64["item_stats"]["phi"] ** 2, 1e-30) / 5000)
    assert np.all(np.abs(r32["item_B"] - r64["item_B"]) < 0.5 * se + 1e-6)
    assert np.allclose(r32["item_G"], r64["item_G"], atol=0.02)
    assert np.allclose(r32["val"], r64["val"], atol=0.05)


def test_round_argument_errors(gpu, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, 3.0, K)
    n = gpu.mesh_info(mesh)["n_items"]
    b = gpu.register_bvp(fk.ANISO)
    bd = gpu.register_bvp(fk.FRANKE)
    gpu.assembly_begin(mesh)
    p = np.full(n, 10, dtype=np.uint32)
    with pytest.raises(fk.FKError) as e:  # one problem functor per round
        gpu.assembly_round(mesh, b, p, 5e-4, fk.FP64, bvp_of_item=np.where(np.arange(n) % 2 == 0, b, bd))
    assert e.value.code == fk.FK_ERR_ARG
    gpu.assembly_round(mesh, b, p, 5e-4, fk.FP64)
    with pytest.raises(fk.FKError) as e:  # one h per assembly
        gpu.assembly_round(mesh, b, p, 1e-3, fk.FP64)
    assert e.value.code == fk.FK_ERR_ARG
    circ = gpu.mesh_circles((0, 0, 1, 1), 3, 1.2, 0.121, 20)
    with pytest.raises(fk.FKError) as e:
        gpu.assembly_begin(circ)
    assert e.value.code == fk.FK_ERR_ARG
