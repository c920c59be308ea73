"""Reflecting (Neumann / Robin) sides: Paso_Reflejante (Solvers/FeynmanKacSolver.cpp:19-67).

The reference's reflecting step reads uninitialised values (Nprop in its loop
test, dist_k on a path's first step), so it has no defined output to match;
the oracle restates the scheme it implements (Lepingle's reflected Euler
step) and pins it against the exact solution of a manufactured Robin problem
(FK_PROBLEM_ROBIN: u = Franke (1 + x y) on [0,1]^2, psi = d_n u - varphi u on
the reflecting sides).  The GPU kernels follow the oracle's paths exactly in
FP64 on the same Philox stream.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

SEED = 977
GPU_SEED = 20251203  # the gpu fixture's context seed


def u_exact(x, y):
    x, y = np.asarray(x, float), np.asarray(y, float)
    F = (0.75 * np.exp(-0.25 * ((9 * x - 2) ** 2 + (9 * y - 2) ** 2)) +
         0.75 * np.exp(-((9 * x + 1) ** 2) / 49 - 0.1 * (9 * y + 1)) +
         0.5 * np.exp(-0.25 * ((9 * x - 7) ** 2 + (9 * y - 3) ** 2)) -
         0.2 * np.exp(-(9 * x - 4) ** 2 - (9 * y - 7) ** 2))
    return F * (1 + x * y)


# side masks: 1 x = 0, 2 y = 0, 4 x = 1, 8 y = 1
CONFIGS = [  # mask, varphi, rho, points
    (1, 0.0, 0.05, [(0.0, 0.5), (0.05, 0.3), (0.4, 0.6)]),   # Neumann on x = 0
    (12, -0.5, 0.05, [(1.0, 0.5), (0.9, 0.95), (0.6, 1.0)]),  # Robin on x = 1 and y = 1
    (3, -1.0, 0.05, [(0.0, 0.0), (0.02, 0.3), (0.3, 0.01)]),  # Robin on a corner's two sides
]


# ------------------------------------------------------------------ oracle ----
def test_oracle_no_reflecting_side_is_the_absorbing_problem(orc):
    """With an empty side mask the reflecting problem follows the ANISO paths
    bit for bit (the restatement adds only zero terms)."""
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=3)
    a, r = orc.bvp(2), orc.bvp(orc.ROBIN, prob=(0, -0.5, 0.1, 0))
    for p in range(40):
        e1 = s.path(a, 0.2, 0.7, 1e-3, 5, p)
        e2 = s.path(r, 0.2, 0.7, 1e-3, 5, p)
        assert (e1.x, e1.y, e1.Y, e1.Z, e1.xi, e1.steps, e1.outcome) == \
               (e2.x, e2.y, e2.Y, e2.Z, e2.xi, e2.steps, e2.outcome)


def test_oracle_paths_never_stop_on_a_reflecting_side(orc):
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=4)
    b = orc.bvp(orc.ROBIN, prob=(1 + 2, 0.0, 0.05, 0))
    n_hit = 0
    for p in range(300):
        e = s.path(b, 0.03, 0.04, 1e-3, 1, p)
        assert e.outcome == orc.OUT_DOMAIN
        # exits lie on the absorbing sides x = 1 or y = 1 only
        assert e.x == 1.0 or e.y == 1.0, (e.x, e.y)
        n_hit += e.steps
    assert n_hit > 300


def test_oracle_reflection_changes_the_paths(orc):
    """Near a reflecting side the paths differ from the absorbing problem's
    (they are pushed back instead of stopping) and live longer."""
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=5)
    a, r = orc.bvp(2), orc.bvp(orc.ROBIN, prob=(1, 0.0, 0.05, 0))
    st_a = s.point_solve(a, 0.01, 0.5, 400, 1e-3, item=2)
    st_r = s.point_solve(r, 0.01, 0.5, 400, 1e-3, item=2)
    assert st_r["APL"] > 5 * st_a["APL"]


@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
def test_oracle_matches_the_exact_robin_solution(orc, cfg):
    """Exact-gradient control variate (near-zero variance), h = 1e-4: the
    estimate is within 4 standard errors plus the scheme's bias allowance
    (O(sqrt h) from the local-time discretisation; measured < 8e-3 at these
    points) of u.  Without the psi term (or with psi at the pre-step point)
    the same paths miss by 2e-2 to 9e-2."""
    mask, varphi, rho, pts = CONFIGS[cfg]
    s = orc.Session(orc.RNG_PHILOX, seed=SEED, stream=10 + cfg)
    b = orc.bvp(orc.ROBIN, cv=1, prob=(mask, varphi, rho, 0))
    N = 600
    for i, (x, y) in enumerate(pts):
        o = s.point_solve(b, x, y, N, 1e-4, item=i)
        se = np.sqrt(max(o["phiphi_VR"] - o["phi_VR"] ** 2, 0.0) / N)
        err = o["phi_VR"] - u_exact(x, y)
        assert abs(err) < 4 * se + 8e-3, (cfg, (x, y), err, se)


# ------------------------------------------------------------ host checks ----
def test_register_rejects_bad_reflecting_parameters(host_ctx, fk):
    for prob in ((16, 0, 0.1, 0), (1.5, 0, 0.1, 0), (-1, 0, 0.1, 0), (1, 0, -0.1, 0)):
        with pytest.raises(fk.FKError) as e:
            host_ctx.register_bvp(fk.ROBIN, prob=prob)
        assert e.value.code == fk.FK_ERR_ARG
    with pytest.raises(fk.FKError):
        host_ctx.register_bvp(fk.ROBIN, dom=(1.0, 0.5, 0.5, 0), dom_shape=fk.CIRCLE, prob=(1, 0, 0.1, 0))
    assert host_ctx.register_bvp(fk.ROBIN, prob=(15, 0.2, 0.0, 0)) >= 0


DESCRIBE_TU = r"""
#include <cmath>
#include <cstdio>
#include "ref_types.hpp"
#include "spac_fk_gpu.hpp"
using namespace ref_like;
static double u_fn(Vector2d) { return 0.0; }
static double other_u(Vector2d) { return 0.0; }
static double rect(std::vector<double>, Vector2d, Vector2d&, Vector2d&) { return 0.0; }
// Stopping_mix of BVPs/Franke_Poisson.hpp:74-77 with its commented-out side:
// reflecting where x = 0 (here) and y = 1
static bool absorbing(Vector2d p) { return !(std::fabs(p[0]) < 1e-8 || std::fabs(p[1] - 1.0) < 1e-8); }
int main() {
  const double prob[4] = {0.0, -0.25, 0.0, 0.0};
  FeynmanKacSolverGPU::Register_Problem(&u_fn, FK_PROBLEM_ROBIN, nullptr, prob);
  FeynmanKacSolverGPU::Register_Problem(&other_u, FK_PROBLEM_ANISO);
  FeynmanKacSolverGPU::Register_Distance(&rect, FK_SHAPE_RECT);
  BVP bvp;
  bvp.u.funcion = &u_fn;
  bvp.frontera_dominio.Distancia = &rect;
  bvp.frontera_dominio.parametros = {0.0, 0.0, 1.0, 1.0};
  bvp.frontera_dominio.Absorbente = &absorbing;
  fk_bvp_desc d = spac_fk_gpu::describe_bvp(bvp, true, 0.3);
  std::printf("%d %g %g %g\n", d.problem, d.prob[0], d.prob[1], d.prob[2]);
  bvp.u.funcion = &other_u;
  try {
    spac_fk_gpu::describe_bvp(bvp, true, 0.3);
    std::printf("no-throw\n");
  } catch (const std::exception&) {
    std::printf("throws\n");
  }
  bvp.frontera_dominio.Absorbente = nullptr;
  d = spac_fk_gpu::describe_bvp(bvp, true, 0.3);
  std::printf("%d %g\n", d.problem, d.prob[0]);
  return 0;
}
"""


def test_drop_in_derives_reflecting_sides_from_frontera():
    """spac_fk_gpu.hpp maps Frontera::Absorbente (false on a side) to the
    side mask and the call's rho into the description; a reflecting side on
    a problem without Robin functors is an error."""
    inc = os.path.join(ROOT, "include")
    cpp = os.path.join(ROOT, "tests", "cpp")
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "d.cpp"), os.path.join(tmp, "d")
        with open(src, "w") as f:
            f.write(DESCRIBE_TU)
        subprocess.run(["g++", "-std=c++17", "-O1", "-I" + inc, "-I" + cpp, src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    assert out[0].split() == ["4", str(1 + 8), "-0.25", "0.3"]
    assert out[1] == "throws"
    assert out[2].split() == ["2", "0"]


# --------------------------------------------------------------------- GPU ----
@pytest.mark.gpu
@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
@pytest.mark.parametrize("cv", [0, 1])
def test_gpu_fp64_follows_the_oracle(gpu, orc, fk, cfg, cv):
    mask, varphi, rho, pts = CONFIGS[cfg]
    b = gpu.register_bvp(fk.ROBIN, cv=cv, prob=(mask, varphi, rho, 0))
    N, h = 300, 1e-3
    gpu.set_stream(300 + cfg)
    st = gpu.solve_points(b, np.array(pts), N, h, fk.FP64)
    s = orc.Session(orc.RNG_PHILOX, seed=GPU_SEED, stream=300 + cfg)
    ob = orc.bvp(orc.ROBIN, cv=cv, prob=(mask, varphi, rho, 0))
    for i, (x, y) in enumerate(pts):
        o = s.point_solve(ob, x, y, N, h, item=i)
        for k in orc.STAT_NAMES:
            assert np.isclose(st[k][i], o[k], rtol=1e-9, atol=1e-12), (k, i, st[k][i], o[k])
        assert st["n_capped"][i] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", range(len(CONFIGS)))
def test_gpu_fp32_matches_the_exact_solution(gpu, fk, cfg):
    mask, varphi, rho, pts = CONFIGS[cfg]
    b = gpu.register_bvp(fk.ROBIN, cv=fk.CV_EXACT, prob=(mask, varphi, rho, 0))
    N = 20000
    gpu.set_stream(320 + cfg)
    st = gpu.solve_points(b, np.array(pts), N, 1e-4, fk.FP32)
    se = np.sqrt(np.maximum(st["phiphi_VR"] - st["phi_VR"] ** 2, 0) / N)
    err = st["phi_VR"] - u_exact(*np.array(pts).T)
    assert np.all(np.abs(err) < 4 * se + 8e-3), (err, se)
    # the plain estimator agrees within its (larger) standard error
    sep = np.sqrt(np.maximum(st["phiphi"] - st["phi"] ** 2, 0) / N)
    assert np.all(np.abs(st["phi"] - u_exact(*np.array(pts).T)) < 4 * sep + 8e-3)


@pytest.mark.gpu
def test_gpu_assembly_with_a_reflecting_side_follows_the_oracle(gpu, orc, fk):
    """G/B assembly on square patches of a domain whose side x = 0 reflects:
    items of the patches next to it match the oracle's node solves (same
    Philox stream, FP64)."""
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 2, 9, 0.25, 1.0, 6)
    b = gpu.register_bvp(fk.ROBIN, prob=(1, -0.3, 0.05, 0))
    gpu.set_stream(340)
    r = gpu.assemble(mesh, b, 128, 1e-3, fk.FP64)
    row, ixy, stn, fr = gpu.mesh_items(mesh)
    nxy, _ = gpu.mesh_nodes(mesh)
    info = gpu.mesh_info(mesh)
    s = orc.Session(orc.RNG_PHILOX, seed=GPU_SEED, stream=340)
    ob = orc.bvp(orc.ROBIN, prob=(1, -0.3, 0.05, 0))
    H = 0.5
    offs = np.concatenate([[0], np.cumsum([len(gpu.mesh_stencil_nodes(mesh, stn[i])) for i in range(info["n_items"])])])
    checked = 0
    for i in range(info["n_items"]):
        a, bb = divmod(int(stn[i]), 2)
        if a != 0 or fr[i]:
            continue  # patches touching x = 0 only
        rect = ((a - 0.25) * H, (bb - 0.25) * H, (a + 1.25) * H, (bb + 1.25) * H)
        gids = gpu.mesh_stencil_nodes(mesh, stn[i])
        G, Bv, _, _ = s.node_solve_knn(ob, ixy[i, 0], ixy[i, 1], rect, nxy[gids], 6, 1.0 / info["spacing"], 128, 1e-3,
                                       item=i)
        assert np.isclose(r["item_B"][i], Bv, rtol=1e-9, atol=1e-12), (i, r["item_B"][i], Bv)
        assert np.allclose(r["item_G"][offs[i]:offs[i + 1]], G, atol=1e-9), i
        checked += 1
    assert checked >= 4


@pytest.mark.gpu
def test_gpu_fp32_assembly_with_reflecting_sides_pairs_with_fp64(gpu, fk):
    """FP32 stepping (slot mode, the patch kernel's 4-CTA build where it fits)
    on a mesh with reflecting sides x = 0 and y = 0, paired with FP64 on the
    same stream: item B within half a standard error, G entries close."""
    mesh = gpu.mesh_square_patches((0, 0, 1, 1), 3, 15, 0.25, 3.0, 20)
    b = gpu.register_bvp(fk.ROBIN, prob=(1 + 2, -0.5, 0.05, 0))
    N = 4000
    gpu.set_stream(360)
    r64 = gpu.assemble(mesh, b, N, 5e-4, fk.FP64)
    gpu.set_stream(360)
    r32 = gpu.assemble(mesh, b, N, 5e-4, fk.FP32)
    se = np.sqrt(np.maximum(r64["item_stats"]["phiphi"] - r64["item_stats"]["phi"] ** 2, 1e-30) / N)
    assert np.all(np.abs(r32["item_B"] - r64["item_B"]) < 0.5 * se + 1e-6)
    assert np.allclose(r32["item_G"], r64["item_G"], atol=0.02)
    assert r64["item_stats"]["n_capped"].sum() == 0
