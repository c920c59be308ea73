"""The C-ABI library loads, exports every entry point declared in
include/spac_fk.h, and fails loudly (no CPU fallback) without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(fk_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(fk):
    L = C.CDLL(fk.lib_path()) if hasattr(fk, "lib_path") else fk.load()
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    # the Python binding covers exactly the declared entry points
    assert set(fk.exported_symbols()) == set(names)


def test_no_device_fails_loudly(fk):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fk.FKError) as e:
        fk.Context(device=0)
    assert e.value.code == fk.FK_ERR_NO_DEVICE


def test_host_only_context_rejects_solves(host_ctx, fk):
    b = host_ctx.register_bvp(fk.FRANKE)
    with pytest.raises(fk.FKError) as e:
        host_ctx.solve_points(b, [[0.5, 0.5]], 10, 1e-3)
    assert e.value.code == fk.FK_ERR_NO_DEVICE
    mid = host_ctx.mesh_circles((0, 0, 1, 1), 3, 1.2, 0.121, 20)
    with pytest.raises(fk.FKError) as e:
        host_ctx.assemble(mid, b, 10, 1e-3)
    assert e.value.code == fk.FK_ERR_NO_DEVICE


def test_registry_errors(host_ctx, fk):
    with pytest.raises(fk.FKError) as e:
        host_ctx.register_bvp(7)
    assert e.value.code == fk.FK_ERR_REGISTRY
    with pytest.raises(fk.FKError) as e:
        host_ctx.register_bvp(fk.FRANKE, dom=(0, 0, -1, 1))
    assert e.value.code == fk.FK_ERR_ARG
    with pytest.raises(fk.FKError) as e:
        host_ctx.register_bvp(fk.DISK, dom_shape=fk.RECT)
    assert e.value.code == fk.FK_ERR_ARG
    with pytest.raises(fk.FKError) as e:
        host_ctx.register_bvp(fk.FRANKE, dom=(0, 0, float("nan"), 1))
    assert e.value.code == fk.FK_ERR_ARG
    with pytest.raises(fk.FKError) as e:
        host_ctx.mesh_info(99)
    assert e.value.code == fk.FK_ERR_REGISTRY
