"""The kernels' bounded waits give up, report an error status and leave the
context usable (fk_set_wait_limits).  Nothing here faults or hangs a GPU:
each test sets a limit of 1 ns, so the first wait that any warp (path
kernel: a chunk slot that another warp of its CTA is still refilling) or CTA
(persistent MLP trainer: the grid barrier) starts runs out at once; the
kernel then ends early, the call returns FK_ERR_CUDA, and the next call with
the default limits succeeds."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_slot_wait_limit_gives_up_and_reports(gpu, fk):
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, 3.0, 20)
    b = gpu.register_bvp(fk.ANISO)
    gpu.set_launch(256, 32768)  # shared chunk slots: warps wait for each other's refills
    gpu.set_wait_limits(1e-9, 0.0)
    try:
        with pytest.raises(fk.FKError) as e:
            gpu.assemble(mesh, b, 2000, 5e-4, fk.FP32, items=False)
        assert e.value.code == fk.FK_ERR_CUDA and "timed out" in str(e.value)
    finally:
        gpu.set_wait_limits(0.0, 0.0)
        gpu.set_launch(0, 0)
    r = gpu.assemble(mesh, b, 2000, 5e-4, fk.FP32)
    assert np.all(r["item_stats"]["n_paths"] == 2000)


def test_trainer_barrier_limit_gives_up_and_reports(gpu, fk):
    rects = np.array([0.0, 0.0, 1.0, 1.0])
    mid = C.c_int()
    gpu.check(gpu.L.fk_mlp_create(gpu.h, 1, rects.ctypes.data_as(fk._dp), 3, C.byref(mid)))
    mid = mid.value
    gpu.check(gpu.L.fk_mlp_set_trainer(gpu.h, mid, fk.TRAIN_GRID))
    rng = np.random.default_rng(2)
    xy = np.ascontiguousarray(rng.uniform(0, 1, (512, 2)))
    tgt = np.ascontiguousarray(np.sin(3 * xy[:, 0]) * xy[:, 1])

    def train(steps):
        return gpu.L.fk_mlp_train(gpu.h, mid, len(tgt), xy.ctypes.data_as(fk._dp), tgt.ctypes.data_as(fk._dp), None,
                                  steps, 4096, 1e-2, 5, None)

    gpu.set_wait_limits(0.0, 1e-9)
    try:
        rc = train(20)
        assert rc == fk.FK_ERR_CUDA
        assert "timed out" in gpu.L.fk_last_error(gpu.h).decode()
    finally:
        gpu.set_wait_limits(0.0, 0.0)
    assert train(20) == fk.FK_OK


def test_wait_limits_reject_bad_values(gpu, fk):
    for bad in ((-1.0, 0.0), (0.0, float("nan")), (2e6, 0.0)):
        with pytest.raises(fk.FKError) as e:
            gpu.set_wait_limits(*bad)
        assert e.value.code == fk.FK_ERR_ARG
