"""Learned control variate: the tensor-core MLP kernels against the CPU FP64
MLP of the oracle, training, and the control variate on the path kernel.

BF16 operands with FP32 accumulation bound the agreement with FP64 to about
1e-2 relative (gradients compared as whole vectors); the control variate must
keep the estimator unbiased (means within 4 combined standard errors of the
plain estimator) and cut the variance."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mlp(gpu, fk, rects, seed=7):
    rects = np.ascontiguousarray(rects, dtype=np.float64).ravel()
    mid = C.c_int()
    gpu.check(gpu.L.fk_mlp_create(gpu.h, len(rects) // 4, rects.ctypes.data_as(fk._dp), seed, C.byref(mid)))
    n = C.c_int()
    gpu.check(gpu.L.fk_mlp_num_params(gpu.h, mid.value, C.byref(n)))
    return mid.value, n.value


def _params(gpu, fk, mid, n, regions=1):
    p = np.zeros(n * regions, dtype=np.float32)
    gpu.check(gpu.L.fk_mlp_get_params(gpu.h, mid, p.ctypes.data_as(fk._fp)))
    return p


def _cpu(orc, p, rect):
    cx, cy = 0.5 * (rect[0] + rect[2]), 0.5 * (rect[1] + rect[3])
    return orc.MlpParams(p.astype(np.float64), 64, (cx, cy), (2.0 / (rect[2] - rect[0]), 2.0 / (rect[3] - rect[1])))


def _eval(gpu, fk, mid, xy, region=None):
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    out = np.zeros((len(xy), 3))
    rp = None
    if region is not None:
        region = np.ascontiguousarray(region, dtype=np.int32)
        rp = region.ctypes.data_as(fk._ip)
    gpu.check(gpu.L.fk_mlp_eval(gpu.h, mid, len(xy), xy.ctypes.data_as(fk._dp), rp, out.ctypes.data_as(fk._dp)))
    return out


def _train(gpu, fk, mid, xy, tgt, steps, batch=4096, lr=3e-3, region=None, seed=11):
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    tgt = np.ascontiguousarray(tgt, dtype=np.float64)
    hist = np.zeros(max(steps, 1), dtype=np.float32)
    rp = None
    if region is not None:
        region = np.ascontiguousarray(region, dtype=np.int32)
        rp = region.ctypes.data_as(fk._ip)
    gpu.check(gpu.L.fk_mlp_train(gpu.h, mid, len(tgt), xy.ctypes.data_as(fk._dp), tgt.ctypes.data_as(fk._dp), rp,
                                 steps, batch, lr, seed, hist.ctypes.data_as(fk._fp)))
    return hist


def _franke(orc, xy):
    b = orc.bvp(0)
    return np.array([orc.coefficients(b, x, y)[0] for x, y in xy])


def test_mlp_loss_gradient_matches_cpu_fp64(gpu, orc, fk):
    rect = (0.0, 0.0, 1.0, 1.0)
    mid, n = _mlp(gpu, fk, [rect])
    rng = np.random.default_rng(1)
    xy = rng.uniform(0, 1, size=(300, 2))
    tgt = _franke(orc, xy)
    loss = C.c_double()
    g = np.zeros(n, dtype=np.float32)
    xyc = np.ascontiguousarray(xy)
    gpu.check(gpu.L.fk_mlp_loss_grad(gpu.h, mid, len(tgt), xyc.ctypes.data_as(fk._dp),
                                     np.ascontiguousarray(tgt).ctypes.data_as(fk._dp), C.byref(loss),
                                     g.ctypes.data_as(fk._fp)))
    cpu = _cpu(orc, _params(gpu, fk, mid, n), rect)
    lc, gc = cpu.loss_grad(xy, tgt)
    assert abs(loss.value - lc) < 1e-2 * lc
    rel = np.linalg.norm(g - gc) / np.linalg.norm(gc)
    cos = g @ gc / (np.linalg.norm(g) * np.linalg.norm(gc))
    assert rel < 3e-2 and cos > 0.999, (rel, cos)
    # every parameter block carries gradient
    sizes = [128, 64, 4096, 64, 4096, 64, 64, 1]
    off = np.cumsum([0] + sizes)
    for i in range(8):
        blk_g, blk_c = g[off[i]:off[i + 1]], gc[off[i]:off[i + 1]]
        assert np.linalg.norm(blk_g - blk_c) <= 5e-2 * np.linalg.norm(blk_c) + 1e-6, i


def test_mlp_eval_value_and_input_gradient(gpu, orc, fk):
    rects = [(0.0, 0.0, 1.0, 1.0), (-0.5, 0.2, 0.3, 0.9)]
    mid, n = _mlp(gpu, fk, rects, seed=3)
    p = _params(gpu, fk, mid, n, regions=2)
    rng = np.random.default_rng(2)
    xy = rng.uniform(0, 1, size=(257, 2))
    reg = rng.integers(0, 2, size=257)
    out = _eval(gpu, fk, mid, xy, reg)
    for r in (0, 1):
        cpu = _cpu(orc, p[r * n:(r + 1) * n], rects[r])
        sel = reg == r
        ref = cpu.eval(xy[sel])
        scale = np.abs(ref).max(axis=0) + 1e-3
        assert np.all(np.abs(out[sel] - ref) <= 2e-2 * scale), r


def test_mlp_training_converges(gpu, orc, fk):
    rect = (0.0, 0.0, 1.0, 1.0)
    mid, n = _mlp(gpu, fk, [rect], seed=5)
    rng = np.random.default_rng(3)
    xy = rng.uniform(0, 1, size=(4000, 2))
    tgt = _franke(orc, xy)
    hist = _train(gpu, fk, mid, xy, tgt, steps=2000, batch=4096, lr=1e-2)
    assert hist[-50:].mean() < 1e-2 * hist[:10].mean()
    # gradient of the fit against the exact Franke gradient
    test = rng.uniform(0.05, 0.95, size=(500, 2))
    out = _eval(gpu, fk, mid, test)
    b = orc.bvp(0, cv=1)
    F = np.array([orc.coefficients(b, x, y)[10:12] for x, y in test])  # F = -sqrt2 grad u
    grad_exact = -F / 1.41421356237
    err = np.linalg.norm(out[:, 1:] - grad_exact, axis=1)
    assert np.median(err) < 0.15 * np.median(np.linalg.norm(grad_exact, axis=1))


def test_learned_cv_unbiased_and_variance_reduced(gpu, orc, fk):
    """Point solves on the Franke problem: a network trained on exact u gives
    a control variate that keeps the mean and cuts the variance."""
    rect = (0.0, 0.0, 1.0, 1.0)
    mid, n = _mlp(gpu, fk, [rect], seed=9)
    rng = np.random.default_rng(4)
    xy = rng.uniform(0, 1, size=(4000, 2))
    _train(gpu, fk, mid, xy, _franke(orc, xy), steps=2000, batch=4096, lr=1e-2)
    gpu.check(gpu.L.fk_mlp_build_table(gpu.h, mid, 512))
    b_plain = gpu.register_bvp(fk.FRANKE)
    b_cv = gpu.register_bvp(fk.FRANKE, cv=fk.CV_MLP, mlp_id=mid)
    pts = np.array([[0.3, 0.4], [0.7, 0.2], [0.5, 0.8], [0.15, 0.15]])
    N = 40000
    for prec in (fk.FP64, fk.FP32):
        s0 = gpu.solve_points(b_plain, pts, N, 1e-3, prec)
        s1 = gpu.solve_points(b_cv, pts, N, 1e-3, prec)
        v0 = s0["phiphi_VR"] - s0["phi_VR"] ** 2
        v1 = s1["phiphi_VR"] - s1["phi_VR"] ** 2
        assert np.all(v1 < v0 / 3), (v0, v1)
        se = np.sqrt(v0 / N + v1 / N)
        assert np.all(np.abs(s1["phi_VR"] - s0["phi_VR"]) < 4 * se)
        # the score without the control term is the plain estimator on the same paths
        assert np.allclose(s1["phi"], s0["phi"], rtol=0, atol=4 * np.sqrt(v0 / N).max())


def _trainer_run(gpu, fk, orc, trainer, steps, batch, regions=1, seed=5):
    rects = [(0.0, 0.0, 1.0, 1.0)] if regions == 1 else [(0.0, 0.0, 0.5, 1.0), (0.5, 0.0, 1.0, 1.0)]
    mid, n = _mlp(gpu, fk, rects, seed=seed)
    gpu.check(gpu.L.fk_mlp_set_trainer(gpu.h, mid, trainer))
    rng = np.random.default_rng(3)
    xy = rng.uniform(0, 1, size=(3000, 2))
    reg = None if regions == 1 else (xy[:, 0] >= 0.5).astype(np.int32)
    hist = _train(gpu, fk, mid, xy, _franke(orc, xy), steps=steps, batch=batch, lr=1e-2, region=reg)
    return hist, _params(gpu, fk, mid, n, regions), mid


@pytest.mark.parametrize("batch,regions", [(4096, 1), (2048, 1), (8192, 1), (4096, 2)])
def test_grid_trainer_follows_step_trainer(gpu, orc, fk, batch, regions):
    """The persistent grid trainer (one cooperative launch, Adam on each CTA's
    slice between grid barriers) computes the same steps as the per-step
    launches: both sum the same CTA partials, in different fixed orders, so
    losses and parameters agree to that rounding, which Adam's normalised
    steps amplify only where a gradient component is near zero."""
    steps = 200
    h_g, p_g, _ = _trainer_run(gpu, fk, orc, fk.TRAIN_GRID, steps, batch, regions)
    h_s, p_s, _ = _trainer_run(gpu, fk, orc, fk.TRAIN_STEPS, steps, batch, regions)
    assert np.all(np.isfinite(h_g)) and np.all(np.isfinite(p_g))
    assert np.abs(h_g[:5] - h_s[:5]).max() <= 1e-3 * h_s[0]
    assert np.abs(h_g[-20:].mean() - h_s[-20:].mean()) <= 0.05 * h_s[-20:].mean()
    assert h_g[-20:].mean() < 0.2 * h_g[:5].mean()
    scale = np.abs(p_s).max()
    assert np.median(np.abs(p_g - p_s)) <= 1e-3 * scale
    assert np.abs(p_g - p_s).max() <= 5e-2 * scale


def test_grid_trainer_one_step_matches(gpu, orc, fk):
    """One Adam step from the same weights: the first step moves each weight
    by lr g / |g| (bias-corrected Adam), so both trainers give the same update
    except for components whose gradient is ~0."""
    _, p_g, _ = _trainer_run(gpu, fk, orc, fk.TRAIN_GRID, 1, 4096)
    _, p_s, _ = _trainer_run(gpu, fk, orc, fk.TRAIN_STEPS, 1, 4096)
    mid, n = _mlp(gpu, fk, [(0.0, 0.0, 1.0, 1.0)], seed=5)
    p0 = _params(gpu, fk, mid, n)
    d_g, d_s = p_g - p0, p_s - p0
    same = np.abs(d_g - d_s) <= 1e-6 + 1e-3 * np.abs(d_s)
    assert same.mean() > 0.99


def _loss_grad(gpu, fk, mid, n, xy, tgt):
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    tgt = np.ascontiguousarray(tgt, dtype=np.float64)
    loss = C.c_double()
    g = np.zeros(n, dtype=np.float32)
    gpu.check(gpu.L.fk_mlp_loss_grad(gpu.h, mid, len(tgt), xy.ctypes.data_as(fk._dp), tgt.ctypes.data_as(fk._dp),
                                     C.byref(loss), g.ctypes.data_as(fk._fp)))
    return loss.value, g


@pytest.mark.parametrize("regions", [1, 2])
def test_fit_output_layer_is_least_squares(gpu, orc, fk, regions):
    """After fk_mlp_fit_output the output layer is the (ridge 1e-6) least-squares
    fit on the hidden features: the loss does not increase, and the loss
    gradient with respect to W4 and b4 nearly vanishes (what remains is the
    ridge term and the BF16 rounding of the features in the backward pass),
    while the hidden layers are untouched."""
    rects = [(0.0, 0.0, 1.0, 1.0)] if regions == 1 else [(0.0, 0.0, 0.5, 1.0), (0.5, 0.0, 1.0, 1.0)]
    mid, n = _mlp(gpu, fk, rects, seed=9)
    rng = np.random.default_rng(4)
    xy = rng.uniform(0, 1, size=(1500, 2))
    reg = None if regions == 1 else (xy[:, 0] >= 0.5).astype(np.int32)
    tgt = _franke(orc, xy)
    _train(gpu, fk, mid, xy, tgt, steps=200, batch=4096, lr=1e-2, region=reg)
    p_before = _params(gpu, fk, mid, n, regions)
    if regions == 1:
        l0, g0 = _loss_grad(gpu, fk, mid, n, xy, tgt)
    rp = None if reg is None else np.ascontiguousarray(reg).ctypes.data_as(fk._ip)
    xyc, tc = np.ascontiguousarray(xy), np.ascontiguousarray(tgt)
    gpu.check(gpu.L.fk_mlp_fit_output(gpu.h, mid, len(tc), xyc.ctypes.data_as(fk._dp), tc.ctypes.data_as(fk._dp), rp,
                                      1e-6))
    p_after = _params(gpu, fk, mid, n, regions)
    off_w4 = n - 65
    for r in range(regions):
        a, b = p_before[r * n:(r + 1) * n], p_after[r * n:(r + 1) * n]
        assert np.array_equal(a[:off_w4], b[:off_w4])          # hidden layers untouched
        assert not np.array_equal(a[off_w4:], b[off_w4:])      # output layer refitted
    if regions == 1:
        l1, g1 = _loss_grad(gpu, fk, mid, n, xy, tgt)
        assert l1 <= l0 * (1 + 1e-4)
        assert np.abs(g1[off_w4:]).max() <= 2e-2 * np.abs(g0[off_w4:]).max()


@pytest.mark.parametrize("trainer", ["steps", "grid"])
def test_adam_steps_match_cpu_adam(gpu, orc, fk, trainer):
    """Four training calls of one step each against a CPU Adam in FP64
    (beta1 0.9, beta2 0.999, eps 1e-8, bias corrections 1 - beta^t with t
    counted across calls; a one-step call runs at the full rate lr).  The
    batch rows are drawn as the trainer draws them: row r of step t takes
    sample Philox4x32-10((t, r, region, 0x6d6c70), seed).x mod n.  The
    batch-mean gradient comes from fk_mlp_loss_grad on those rows in batch
    order, at the trainer's current weights; with 64-row tiles it sums the
    same tile partials in the same order as the per-step trainer, so there
    the gradients are the trainer's own and only the FP32 Adam arithmetic
    differs from the CPU's.  The grid trainer sums the partials in another
    fixed order: its updates agree except for components whose gradient is
    at rounding level."""
    rect = (0.0, 0.0, 1.0, 1.0)
    mid, n = _mlp(gpu, fk, [rect], seed=13)
    gpu.check(gpu.L.fk_mlp_set_trainer(gpu.h, mid, fk.TRAIN_STEPS if trainer == "steps" else fk.TRAIN_GRID))
    rng = np.random.default_rng(6)
    xy = rng.uniform(0, 1, size=(500, 2))
    tgt = _franke(orc, xy)
    batch, lr, seed = 256, 1e-2, 0x1234567890ab
    b1, b2, eps = 0.9, 0.999, 1e-8
    key = (seed & 0xFFFFFFFF, seed >> 32)
    m = np.zeros(n)
    v = np.zeros(n)
    agree = []
    for t in range(4):
        p0 = _params(gpu, fk, mid, n)
        rows = np.array([orc.philox((t, r, 0, 0x6D6C70), key)[0] % len(xy) for r in range(batch)])
        _, g = _loss_grad(gpu, fk, mid, n, xy[rows], tgt[rows])
        g = g.astype(np.float64)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        upd = lr * (m / (1 - b1 ** (t + 1))) / (np.sqrt(v / (1 - b2 ** (t + 1))) + eps)
        _train(gpu, fk, mid, xy, tgt, steps=1, batch=batch, lr=lr, seed=seed)
        d = (p0.astype(np.float64) - _params(gpu, fk, mid, n).astype(np.float64))
        # one FP32 rounding of the weight, FP32 Adam arithmetic
        tol = 2 * np.spacing(np.abs(p0).astype(np.float32)).astype(np.float64) + 1e-5 * np.abs(upd)
        agree.append((np.abs(d - upd) <= tol).mean())
    if trainer == "steps":
        assert min(agree) == 1.0, agree
    else:
        assert min(agree) > 0.99, agree
