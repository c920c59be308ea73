"""Uneven batched solves of several BVPs in one persistent launch, and the
autotuner: per point the same paths as the oracle (FP64), and results that do
not depend on the launch shape the autotuner picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20251203


def _disks(gpu, fk):
    specs = [(0.3, 0.0, 0.0), (0.8, 3.0, -1.0), (0.55, -2.0, 2.0)]
    ids = [gpu.register_bvp(fk.DISK, dom=(r, cx, cy), prob=(cx, cy, r, 0)) for r, cx, cy in specs]
    rng = np.random.default_rng(8)
    xy, which = [], []
    for k, (r, cx, cy) in enumerate(specs):
        for _ in range(5):
            rr, th = r * np.sqrt(rng.uniform(0, 0.95)), rng.uniform(0, 2 * np.pi)
            xy.append((cx + rr * np.cos(th), cy + rr * np.sin(th)))
            which.append(k)
    return specs, np.array(ids), np.array(xy), np.array(which)


def test_multi_bvp_fp64_matches_oracle(gpu, orc, fk):
    specs, ids, xy, which = _disks(gpu, fk)
    rng = np.random.default_rng(9)
    paths = rng.integers(100, 900, len(xy)).astype(np.uint32)
    h = rng.choice([1e-3, 5e-4], len(xy))
    gpu.set_stream(303)
    st = gpu.solve_points_multi(ids[which], xy, paths, h, fk.FP64)
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=303)
    for i, (x, y) in enumerate(xy):
        r, cx, cy = specs[which[i]]
        b = orc.bvp(3, dom=(r, cx, cy, 0), dom_shape=orc.CIRCLE, prob=(cx, cy, r, 0))
        o = s.point_solve(b, x, y, int(paths[i]), h[i], item=i)
        for k in orc.STAT_NAMES:
            assert np.isclose(st[k][i], o[k], rtol=1e-9, atol=1e-12), (i, k)


def test_multi_bvp_rejects_mixed_functors(gpu, fk):
    a = gpu.register_bvp(fk.FRANKE)
    b = gpu.register_bvp(fk.ANISO)
    with pytest.raises(fk.FKError) as e:
        gpu.solve_points_multi([a, b], np.array([[0.5, 0.5], [0.4, 0.4]]), 10, 1e-3)
    assert e.value.code == fk.FK_ERR_ARG


def test_autotune_keeps_results_and_stream(gpu, fk):
    specs, ids, xy, which = _disks(gpu, fk)
    rng = np.random.default_rng(10)
    paths = np.exp(rng.uniform(np.log(500), np.log(20000), len(xy))).astype(np.uint32)
    h = rng.choice([1e-3, 5e-4], len(xy))
    gpu.set_launch(256, 0)
    gpu.set_stream(404)
    before = gpu.solve_points_multi(ids[which], xy, paths, h, fk.FP64)
    gpu.set_stream(404)
    block, chunk, ms = gpu.autotune_points(ids[which], xy, paths, h, fk.FP64, sample_fraction=0.1)
    assert block in (64, 128, 256) and chunk in (512, 2048, 8192, 32768) and ms > 0
    assert gpu.get_stream() == 404  # tuning does not consume stream ids
    after = gpu.solve_points_multi(ids[which], xy, paths, h, fk.FP64)
    for k in ("phi", "phiphi", "phi_VR", "APL", "RNGC", "n_domain_exits"):
        assert np.allclose(before[k], after[k], rtol=1e-12, atol=1e-14), k
    gpu.set_launch(256, 0)


def test_zero_path_items_contribute_nothing(gpu, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 3, 9, 0.25, 1.0, 6)
    info = gpu.mesh_info(mesh)
    b = gpu.register_bvp(fk.ANISO)
    pp = np.zeros(info["n_items"], dtype=np.uint32)
    pp[::2] = 200
    r = gpu.assemble(mesh, b, 0, 5e-4, fk.FP32, paths_per_item=pp)
    assert np.all(np.isfinite(r["val"])) and np.all(np.isfinite(r["B"]))
    assert np.all(r["item_B"][1::2] == 0.0)
    rp, col, v0 = gpu.mesh_csr(mesh)
    row, _, _, _ = gpu.mesh_items(mesh)
    # rows whose items all got zero paths keep the pattern values
    live_rows = set(row[pp > 0])
    for i in range(info["n_rows"]):
        if i not in live_rows:
            assert np.array_equal(r["val"][rp[i]:rp[i + 1]], v0[rp[i]:rp[i + 1]])
