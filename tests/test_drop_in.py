"""The C++ drop-in FeynmanKacSolverGPU (include/spac_fk_gpu.hpp).

CPU: the header compiles against the reference's own headers (where they
exist) with both Solve_OMP_Analytic signatures instantiated on the
reference's BVP / Nudo / Interfaz types, and a driver built on the test
doubles of tests/cpp links against libspac_fk.
GPU: that driver, run the way the reference's serial driver runs the CPU
solver, gives the same statistics, G rows and B as the C ABI called directly
with the same seed and call sequence.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import oracle_py

INC = os.path.join(ROOT, "include")
CPP = os.path.join(ROOT, "tests", "cpp")
LIBDIR = os.path.join(ROOT, "spac_gb300", "_build")

REF_TU = r"""
#include "BVP/BVP.hpp"
#include "Mesh/Nudo.hpp"
#include "Mesh/Interfaz.hpp"
#include "spac_fk_gpu.hpp"
void drive(FeynmanKacSolverGPU& s, BVP& bvp, Nudo& nudo, Interfaz& interfaz) {
  Eigen::Vector2d X0;
  X0[0] = 0.5; X0[1] = 0.5;
  s.Solve_OMP_Analytic(X0, 1000u, 1e-3, 0.1, bvp);
  s.Solve_OMP_Analytic(nudo, 1000u, 1e-3, 1.0, bvp, interfaz);
  FeynmanKacSolverGPU::Register_Problem(bvp.u.funcion, FK_PROBLEM_FRANKE, bvp.F.funcion);
  FeynmanKacSolverGPU::Register_Distance(bvp.frontera_dominio.Distancia, FK_SHAPE_RECT);
}
// main_test_serial.cpp:67-75 with the GPU class
void drive_ps(PseudoespectralCirculoSolverGPU& ps, BVP& bvp, Interfaz& it) {
  ps.Inicializa(it.centro, it.radio, it.nudos_circunferencia.size(), 43,
                it.nudos_circunferencia[0].posicion_angular, bvp);
  ps.Resuelve(bvp, it.nudos_interior, it.nudos_circunferencia);
}
"""


def _driver(tmp):
    exe = os.path.join(tmp, "drop_in_main")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + INC, "-I" + CPP, os.path.join(CPP, "drop_in_main.cpp"),
                    "-L" + LIBDIR, "-lspac_fk", "-Wl,-rpath," + LIBDIR, "-o", exe], check=True)
    return exe


def test_header_compiles_against_reference_headers():
    if not os.path.isdir(oracle_py.REF_SRC):
        pytest.skip("reference sources not present")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "tu.cpp")
        with open(src, "w") as f:
            f.write(REF_TU)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w", "-I" + os.path.join(ROOT, "oracle", "shim"),
                            "-I" + oracle_py.REF_SRC, "-I" + INC, src], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]


def test_driver_builds_and_links(fk):
    fk.load()
    with tempfile.TemporaryDirectory() as tmp:
        assert os.path.exists(_driver(tmp))


def _arc_file(path):
    """One arc of the golden unit3 mesh (with the reference's iPsi) and its items."""
    m = np.load(os.path.join(GOLDEN, "mesh_unit3.npz"))
    A = np.load(os.path.join(GOLDEN, "assembly_unit3_p0_f0.npz"))
    ii, dd = m["iface_int"], m["iface_dbl"]
    off = np.concatenate([[0], np.cumsum(ii[:, 2])])
    k = int(A["item_int"][0, 1])
    n = int(ii[k, 2])
    gids = m["iface_gids"][off[k]:off[k] + n]
    theta_of = {int(g): t for g, t in zip(m["node_int"][:, 0], m["node_dbl"][:, 2])}
    xy_of = {int(g): (x, y) for g, (x, y) in zip(m["node_int"][:, 0], m["node_dbl"][:, :2])}
    ipsi_k = [i for i in range(len(ii)) if i < k and m["iface_ipsi_off"][i + 1] > m["iface_ipsi_off"][i]]
    P = m["iface_ipsi"][m["iface_ipsi_off"][k]:m["iface_ipsi_off"][k + 1]]
    assert len(P) == n * n
    items = [(xy_of[int(r)][0], xy_of[int(r)][1], int(fr), int(r)) for r, iface, fr, _ in A["item_int"] if iface == k]
    arc = dict(cx=dd[k, 0], cy=dd[k, 1], radius=dd[k, 2], c2=dd[k, 3], interior=int(ii[k, 0]),
               theta=np.array([theta_of[int(g)] for g in gids]), gids=gids, iPsi=P.reshape(n, n, order="F"))
    with open(path, "w") as f:
        f.write("%.17g %.17g %.17g %.17g %d %d\n" % (arc["cx"], arc["cy"], arc["radius"], arc["c2"], arc["interior"], n))
        for t, g in zip(arc["theta"], gids):
            f.write("%.17g %d\n" % (t, g))
        f.write(" ".join("%.17g" % v for v in P) + "\n")
        f.write("%d\n" % len(items))
        for x, y, fr, r in items:
            f.write("%.17g %.17g %d %d\n" % (x, y, fr, r))
    return arc, items


@pytest.mark.gpu
def test_drop_in_matches_c_abi(fk):
    seed = 4242
    with tempfile.TemporaryDirectory() as tmp:
        exe = _driver(tmp)
        arc, items = _arc_file(os.path.join(tmp, "arc.txt"))
        out = subprocess.run([exe, os.path.join(tmp, "arc.txt"), str(seed)], capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")
    ctx = fk.Context(0, seed)
    b = ctx.register_bvp(fk.FRANKE)
    st = ctx.solve_points(b, [(0.31, 0.4)], 2000, 1e-3, fk.FP64)
    v = [float(t) for t in lines[0].split()[1:]]
    for name, got in zip(("phi", "phiphi", "phi_VR", "APL", "RNGC", "xi"), v):
        assert np.isclose(got, st[name][0], rtol=1e-12, atol=1e-14), name
    bcv = ctx.register_bvp(fk.FRANKE, cv=fk.CV_EXACT)
    st = ctx.solve_points(bcv, [(0.31, 0.4)], 2000, 1e-3, fk.FP64)
    v = [float(t) for t in lines[1].split()[1:]]
    for name, got in zip(("phi", "phi_VR", "phiphi_VR"), v):
        assert np.isclose(got, st[name][0], rtol=1e-12, atol=1e-14), name
    a = ctx.register_arc(arc["cx"], arc["cy"], arc["radius"], arc["c2"], arc["interior"], arc["theta"], arc["gids"],
                         iPsi=arc["iPsi"])
    n = len(arc["gids"])
    for k, (x, y, fr, r) in enumerate(items):
        G, B, s = ctx.solve_nodes_arc(b, [(x, y, 1e-3, 500, fr, r, a)], {a: n}, fk.FP64)
        parts = lines[2 + k].split()
        assert parts[0] == "node" and int(parts[1]) == r
        assert np.isclose(float(parts[2]), B[0], rtol=1e-12, atol=1e-14), k
        if not fr:
            assert np.isclose(float(parts[3]), s["phi"][0], rtol=1e-12, atol=1e-14), k
            got = dict((int(p.split(":")[0]), float(p.split(":")[1])) for p in parts[4:])
            assert sorted(got) == sorted(int(g) for g in arc["gids"])
            # the FP64 moment sums are atomics in arbitrary order and iPsi has
            # condition ~1e10: G agrees to ~1e-11 between two runs of one path set
            for g, val in zip(arc["gids"], G):
                assert np.isclose(got[int(g)], val, rtol=1e-9, atol=1e-9), (k, g)


@pytest.mark.gpu
def test_disk_drop_in_matches_c_abi(fk):
    """PseudoespectralCirculoSolverGPU (Inicializa + Resuelve on Nudo vectors)
    gives the G entries (keyed by periphery indice_global) and B of the C ABI."""
    from test_disk_ps import golden_disks
    d = golden_disks()[0]
    assert d["problem"] == 0
    gids = 100 + np.arange(d["nc"])
    with tempfile.TemporaryDirectory() as tmp:
        exe = _driver(tmp)
        path = os.path.join(tmp, "disk.txt")
        with open(path, "w") as f:
            f.write("%.17g %.17g %.17g %d %d %.17g %d\n" % (d["cx"], d["cy"], d["R"], d["nc"], d["nr"], d["th0"], d["nc"]))
            for t, g in zip(d["theta"], gids):
                f.write("%.17g %d\n" % (t, g))
            f.write("%d\n" % len(d["xy"]))
            for k, (x, y) in enumerate(d["xy"]):
                f.write("%.17g %.17g %d\n" % (x, y, k))
        out = subprocess.run([exe, "--disk", path], capture_output=True, text=True, check=True)
    ctx = fk.Context(0, 1)
    b = ctx.register_bvp(fk.FRANKE)
    (G, B), = ctx.solve_disks_ps(b, [dict(cx=d["cx"], cy=d["cy"], radius=d["R"], theta0=d["th0"], n_circle=d["nc"],
                                          n_radial=d["nr"], periph_theta=d["theta"], inner_xy=d["xy"])])
    lines = [l for l in out.stdout.split("\n") if l.startswith("inner")]
    assert len(lines) == len(d["xy"])
    for k, line in enumerate(lines):
        parts = line.split()
        assert int(parts[1]) == k and float(parts[2]) == B[k]
        got = dict((int(p.split(":")[0]), float(p.split(":")[1])) for p in parts[3:])
        assert sorted(got) == [int(g) for g in gids]
        assert [got[int(g)] for g in gids] == list(G[k])


@pytest.mark.gpu
def test_robin_drop_in_matches_c_abi(fk):
    """Frontera::Absorbente false on x = 0 and the call's rho reach the
    device as FK_PROBLEM_ROBIN's side mask and prob[2]: the drop-in's point
    solve equals the C ABI's on the same seed and stream."""
    seed = 5151
    with tempfile.TemporaryDirectory() as tmp:
        exe = _driver(tmp)
        out = subprocess.run([exe, "--robin", str(seed)], capture_output=True, text=True, check=True)
    v = [float(t) for t in out.stdout.split()[1:]]
    ctx = fk.Context(0, seed)
    b = ctx.register_bvp(fk.ROBIN, prob=(1, -0.5, 0.1, 0))
    st = ctx.solve_points(b, [(0.02, 0.4)], 2000, 1e-3, fk.FP64)
    for name, got in zip(("phi", "phiphi", "APL", "RNGC"), v):
        assert np.isclose(got, st[name][0], rtol=1e-12, atol=1e-14), name
    ctx.close()
