"""The 8x8 square-patch G/B assembly at its full shape (31 nodes per patch
side, the 20 nearest nodes in the Gaussian exit stencil, eps = 3/spacing as
specified and eps = 1/spacing), through the C ABI against the CPU oracle.

 - FP64 stepping on a seeded sample of 64 items (a few hundred paths each,
   the other items given no paths) equals the oracle's node solves on the same
   Philox stream: B to rtol 1e-9, G entries to 1e-9.
 - FP32 stepping on every item is paired with FP64 on the same stream: B
   within half a standard error, G entries within 0.02 (a path whose exit
   decision differs moves an entry by at most |w|/N).
 - The row residual of the assembled system with the exact solution,
   (sum_j val_rj u(x_j) - B_r) / diag_r, measures the exit stencil's
   interpolation error: Gaussian weights at eps * spacing = 3 sum to 0.21
   halfway between two nodes, so the residual is O(0.1); at eps * spacing = 1
   they sum to 0.9998 and the residual is the O(h) bias of the step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20251203
N_SUB, NPS, ENL, K = 8, 31, 0.25, 20


def _u(x, y):
    f = (0.75 * np.exp(-0.25 * ((9 * x - 2) ** 2 + (9 * y - 2) ** 2)) +
         0.75 * np.exp(-((9 * x + 1) ** 2) / 49 - 0.1 * (9 * y + 1)) +
         0.5 * np.exp(-0.25 * ((9 * x - 7) ** 2 + (9 * y - 3) ** 2)) -
         0.2 * np.exp(-((9 * x - 4) ** 2) - (9 * y - 7) ** 2))
    return f * (1 + x * y)


def _rect(s):
    H = 1.0 / N_SUB
    a, b = divmod(int(s), N_SUB)
    return ((a - ENL) * H, (b - ENL) * H, (a + 1 + ENL) * H, (b + 1 + ENL) * H)


@pytest.mark.parametrize("eps_sp", [3.0, 1.0])
def test_config2_fp64_sample_matches_oracle(gpu, orc, fk, eps_sp):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, eps_sp, K)
    info = gpu.mesh_info(mesh)
    row, ixy, stn, fr = gpu.mesh_items(mesh)
    nxy, _ = gpu.mesh_nodes(mesh)
    rng = np.random.default_rng(8)
    pick = np.sort(rng.choice(info["n_items"], 64, replace=False))
    N, h = 300, 5e-4
    ppi = np.zeros(info["n_items"], dtype=np.uint32)
    ppi[pick] = N
    b = gpu.register_bvp(fk.ANISO)
    gpu.set_stream(41)
    r = gpu.assemble(mesh, b, 0, h, fk.FP64, paths_per_item=ppi)
    sizes = np.array([len(gpu.mesh_stencil_nodes(mesh, s)) for s in range(info["n_stencils"])])
    goff = np.concatenate([[0], np.cumsum(sizes[stn])])
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=41)
    ob = orc.bvp(2)
    eps = eps_sp / info["spacing"]
    for i in pick:
        gids = gpu.mesh_stencil_nodes(mesh, stn[i])
        G, Bv, _, _ = s.node_solve_knn(ob, ixy[i, 0], ixy[i, 1], _rect(stn[i]), nxy[gids], K, eps, N, h, item=int(i))
        assert np.isclose(r["item_B"][i], Bv, rtol=1e-9, atol=1e-12), i
        assert np.allclose(r["item_G"][goff[i]:goff[i + 1]], G, rtol=1e-9, atol=1e-9), i
    # items given no paths contribute nothing
    rest = np.setdiff1d(np.arange(info["n_items"]), pick)
    assert np.all(r["item_B"][rest] == 0.0)


@pytest.mark.parametrize("eps_sp", [3.0, 1.0])
def test_config2_fp32_paired_with_fp64(gpu, fk, eps_sp):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, eps_sp, K)
    b = gpu.register_bvp(fk.ANISO)
    N = 2000
    gpu.set_stream(43)
    r64 = gpu.assemble(mesh, b, N, 5e-4, fk.FP64)
    gpu.set_stream(43)
    r32 = gpu.assemble(mesh, b, N, 5e-4, fk.FP32)
    se = np.sqrt(np.maximum(r64["item_stats"]["phiphi"] - r64["item_stats"]["phi"] ** 2, 1e-30) / N)
    assert np.all(np.abs(r32["item_B"] - r64["item_B"]) < 0.5 * se + 1e-6)
    assert np.allclose(r32["item_G"], r64["item_G"], atol=0.02)
    assert np.allclose(r32["val"], r64["val"], atol=0.05)
    assert np.all(r32["item_stats"]["n_paths"] == N)


def test_config2_row_residual_measures_the_stencil(gpu, fk):
    b = gpu.register_bvp(fk.ANISO)
    rms = {}
    for eps_sp in (3.0, 1.0):
        mesh = gpu.mesh_square_patches((0, 0, 1, 1), N_SUB, NPS, ENL, eps_sp, K)
        rp, col, v0 = gpu.mesh_csr(mesh)
        nxy, _ = gpu.mesh_nodes(mesh)
        u = _u(nxy[:, 0], nxy[:, 1])
        n = len(rp) - 1
        diag = np.array([v0[rp[i]:rp[i + 1]][col[rp[i]:rp[i + 1]] == i][0] for i in range(n)])
        r = gpu.assemble(mesh, b, 20000, 5e-4, fk.FP32, items=False)
        e = (np.add.reduceat(r["val"] * u[col], rp[:-1]) - r["B"]) / diag
        rms[eps_sp] = float(np.sqrt(np.mean(e ** 2)))
    # eps * spacing = 1: the O(h) bias of h = 5e-4 (about 6e-3) and the Monte
    # Carlo error; eps * spacing = 3: the weights' missing mass between nodes
    assert rms[1.0] < 1.2e-2, rms
    assert rms[3.0] > 5e-2, rms
