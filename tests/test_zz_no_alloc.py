"""fk_solve_points_noalloc: point solves for callers that cannot allocate
device memory while solving (stream capture, pre-reserved memory, real-time
hosts).  Its scratch is a static device array inside the library; this test
calls it through the C ABI with caller-owned device buffers and checks two
calls in a row against the allocating fk_solve_points on the same random
stream.  Collected last on purpose, so that a failure here comes after every
other test has run."""
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
