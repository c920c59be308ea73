"""fk_solve_points_noalloc: point solves for callers that cannot allocate
device memory when they solve (embedders that reserve all device memory up
front, real-time hosts that cannot afford an allocation).  Its scratch is a
static device array inside the library; these tests call it through the C ABI
with caller-owned device buffers and check two calls in a row against the
allocating fk_solve_points on the same random stream, the step-cap report in
the per-point counts, the spreading of one point's paths over the grid, and
the argument checks.  Collected last on purpose, so that a failure here comes
after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 4242
RTOL = {0: 1e-9, 1: 1e-6}   # FP64: same paths to rounding; FP32: compensated thread sums


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_allocating_entry_point(fk, prec):
    import torch
    L = fk.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(17)
    n, N, h = 37, 3000, 1e-3
    pts = rng.uniform(0.05, 0.95, size=(n, 2))
    ctx = fk.Context(device=0, seed=SEED)
    try:
        b = ctx.register_bvp(fk.ANISO)
        desc = fk.BvpDesc(fk.ANISO, fk.CV_NONE, fk.RECT, (C.c_double * 4)(0, 0, 1, 1), (C.c_double * 4)(0, 0, 0, 0), -1)
        xy = torch.tensor(pts, dtype=torch.float64, device="cuda")
        paths = torch.full((n,), N, dtype=torch.int32, device="cuda")
        hh = torch.full((n,), h, dtype=torch.float64, device="cuda")
        out = torch.zeros((n, len(fk.STAT_FIELDS)), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for sid in (11, 12):  # two calls in a row share the static scratch array
            ctx.set_stream(sid)
            ref = ctx.solve_points(b, pts, N, h, prec)
            out.fill_(-1.0)
            rc = L.fk_solve_points_noalloc(C.byref(desc), SEED, sid, n, _ptr(xy), _ptr(paths), _ptr(hh), prec, 1 << 24,
                                           C.c_void_p(stream), _ptr(out))
            assert rc == fk.FK_OK
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            for j, name in enumerate(fk.STAT_FIELDS):
                assert np.allclose(got[:, j], ref[name], rtol=RTOL[prec], atol=1e-12), (sid, name)
            assert np.all(got[:, fk.STAT_FIELDS.index("n_paths")] == N)
    finally:
        ctx.close()


def test_noalloc_rejects_sizes_beyond_the_maximum(fk):
    import torch
    L = fk.load()
    n = 16384  # FK_NOALLOC_MAX_POINTS in include/spac_fk.h
    desc = fk.BvpDesc(fk.FRANKE, fk.CV_NONE, fk.RECT, (C.c_double * 4)(0, 0, 1, 1), (C.c_double * 4)(0, 0, 0, 0), -1)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = L.fk_solve_points_noalloc(C.byref(desc), 1, 0, n + 1, _ptr(buf), _ptr(buf), _ptr(buf), 0, 1000, None,
                                   _ptr(buf))
    assert rc == fk.FK_ERR_CAPACITY


def _desc(fk, problem=None, dom=(0, 0, 1, 1)):
    problem = fk.ANISO if problem is None else problem
    return fk.BvpDesc(problem, fk.CV_NONE, fk.RECT, (C.c_double * 4)(*dom), (C.c_double * 4)(0, 0, 0, 0), -1)


def test_noalloc_reports_capped_paths_in_the_counts(fk):
    """max_steps stops paths; the call does not wait for the kernels, so the
    caps show in d_out: n_capped > 0 while every path still completes."""
    import torch
    L = fk.load()
    n, N = 3, 500
    xy = torch.tensor([[0.5, 0.5], [0.3, 0.6], [0.7, 0.2]], dtype=torch.float64, device="cuda")
    paths = torch.full((n,), N, dtype=torch.int32, device="cuda")
    hh = torch.full((n,), 1e-4, dtype=torch.float64, device="cuda")
    out = torch.zeros((n, len(fk.STAT_FIELDS)), dtype=torch.float64, device="cuda")
    desc = _desc(fk)
    rc = L.fk_solve_points_noalloc(C.byref(desc), 5, 0, n, _ptr(xy), _ptr(paths), _ptr(hh), 1, 3, None, _ptr(out))
    assert rc == fk.FK_OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(got[:, fk.STAT_FIELDS.index("n_capped")] > 0)
    assert np.all(got[:, fk.STAT_FIELDS.index("n_paths")] == N)
    assert np.all(got[:, fk.STAT_FIELDS.index("mean_steps")] <= 3.0)


def test_noalloc_spreads_one_point_over_the_grid(fk):
    """One point with many paths is split into chunks over the whole grid, as
    in fk_solve_points: same statistics on the same stream, and comparable
    time (the kernel alone, CUDA events, against the allocating call's)."""
    import torch
    L = fk.load()
    N, h, sid = 4_000_000, 1e-3, 21
    ctx = fk.Context(device=0, seed=SEED)
    try:
        b = ctx.register_bvp(fk.ANISO)
        ctx.set_stream(sid)
        ref = ctx.solve_points(b, np.array([[0.4, 0.55]]), N, h, fk.FP32)
        t_ref = ctx.last_timing()[0]
        xy = torch.tensor([[0.4, 0.55]], dtype=torch.float64, device="cuda")
        paths = torch.full((1,), N, dtype=torch.int32, device="cuda")
        hh = torch.full((1,), h, dtype=torch.float64, device="cuda")
        out = torch.zeros((1, len(fk.STAT_FIELDS)), dtype=torch.float64, device="cuda")
        desc = _desc(fk)
        s = torch.cuda.current_stream()
        best = 1e30
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            rc = L.fk_solve_points_noalloc(C.byref(desc), SEED, sid, 1, _ptr(xy), _ptr(paths), _ptr(hh), 1, 1 << 24,
                                           C.c_void_p(s.cuda_stream), _ptr(out))
            e1.record(s)
            assert rc == fk.FK_OK
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        got = out.cpu().numpy()[0]
        for j, name in enumerate(fk.STAT_FIELDS):
            assert np.isclose(got[j], ref[name][0], rtol=1e-6, atol=1e-12), name
        # the no-alloc time includes its prepare and finalize launches
        assert best < 2.0 * t_ref + 0.5, (best, t_ref)
    finally:
        ctx.close()


def test_noalloc_rejects_empty_domains(fk):
    import torch
    L = fk.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    for dom in ((0, 0, 0, 1), (0, 1, 1, 0.5)):
        desc = _desc(fk, fk.FRANKE, dom)
        rc = L.fk_solve_points_noalloc(C.byref(desc), 1, 0, 1, _ptr(buf), _ptr(buf), _ptr(buf), 0, 1000, None,
                                       _ptr(buf))
        assert rc == fk.FK_ERR_ARG
    desc = fk.BvpDesc(fk.DISK, fk.CV_NONE, fk.CIRCLE, (C.c_double * 4)(0, 0.5, 0.5, 0), (C.c_double * 4)(0.5, 0.5, 1, 0),
                      -1)
    rc = L.fk_solve_points_noalloc(C.byref(desc), 1, 0, 1, _ptr(buf), _ptr(buf), _ptr(buf), 0, 1000, None, _ptr(buf))
    assert rc == fk.FK_ERR_ARG
    desc = fk.BvpDesc(fk.FRANKE, fk.CV_MLP, fk.RECT, (C.c_double * 4)(0, 0, 1, 1), (C.c_double * 4)(0, 0, 0, 0), 0)
    rc = L.fk_solve_points_noalloc(C.byref(desc), 1, 0, 1, _ptr(buf), _ptr(buf), _ptr(buf), 0, 1000, None, _ptr(buf))
    assert rc == fk.FK_ERR_ARG
