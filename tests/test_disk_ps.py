"""Pseudospectral disk rows (PseudoespectralCirculoSolver + Interpolador_PS).

The golden fixtures ps_disks.npz and ps_rows_*.npz come from the reference's
own Solvers/PseudoespectralCirculoSolver.cpp and BVP/Interpolador_PS.cpp,
compiled unmodified against oracle/shim (tests/golden/make_golden.py).  The
solve is deterministic FP64, so parity is a tolerance on the solver noise:
the collocation matrix's condition number grows like (N_c N_r)^2 (8.7e4 at
16 x 11, 4.3e7 at the serial driver's 44 x 43), and two backward-stable FP64
solvers (the reference's QR, the oracle's partial-pivot LU, the GPU's
per-Fourier-mode solves) differ by up to about kappa * 1e-16 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def ps_tol(nc, nr):
    """Relative (to the largest entry) tolerance of a disk solve."""
    return 4e-15 * float(nc * nr) ** 2


def golden_disks():
    z = np.load(os.path.join(GOLDEN, "ps_disks.npz"))
    out, oth, oxy, og = [], 0, 0, 0
    for c in z["cases"]:
        problem, cx, cy, R, nc, nr, th0, npp, nin = c
        nc, nr, npp, nin = int(nc), int(nr), int(npp), int(nin)
        out.append(dict(problem=int(problem), cx=cx, cy=cy, R=R, nc=nc, nr=nr, th0=th0,
                        theta=z["periph_theta"][oth:oth + npp], xy=z["inner_xy"][oxy:oxy + nin],
                        G=z["G"][og:og + nin * npp].reshape(nin, npp), B=z["B"][oxy:oxy + nin]))
        oth += npp
        oxy += nin
        og += nin * npp
    return out


def problem_dom(problem):
    return (-200, -200, 200, 200) if problem == 1 else (0, 0, 1, 1)


def full_circles(mesh_npz):
    """(cx, cy, R, circle gids, interior gids) of every interior (non-perimeter) circle."""
    m = np.load(os.path.join(GOLDEN, mesh_npz))
    out, og, oi = [], 0, 0
    for k, (interior, perimeter, n, n_in) in enumerate(m["iface_int"]):
        gids = m["iface_gids"][og:og + n]
        inner = m["iface_inner"][oi:oi + n_in]
        og += n
        oi += n_in
        if not perimeter:
            cx, cy, R, _ = m["iface_dbl"][k]
            out.append((cx, cy, R, gids, inner))
    return m, out


def test_ps_disk_oracle_matches_reference(orc):
    for d in golden_disks():
        b = orc.bvp(d["problem"], dom=problem_dom(d["problem"]))
        G, B = orc.ps_disk(b, d["cx"], d["cy"], d["R"], d["nc"], d["nr"], d["th0"], d["theta"], d["xy"])
        tol = ps_tol(d["nc"], d["nr"])
        assert np.abs(G - d["G"]).max() <= tol * np.abs(d["G"]).max()
        assert np.abs(B - d["B"]).max() <= tol * np.abs(d["B"]).max()


def test_ps_disk_properties(orc):
    # with c = 0 the interpolated cardinal solutions sum to one (-G rows sum to 1);
    # the disk solve reproduces the exact Franke solution to the discretisation error
    d = golden_disks()[3]
    b = orc.bvp(0)
    G, B = orc.ps_disk(b, d["cx"], d["cy"], d["R"], d["nc"], d["nr"], d["th0"], d["theta"], d["xy"])
    assert np.allclose(-G.sum(1), 1.0, atol=1e-9)
    ring = np.stack([d["cx"] + d["R"] * np.cos(d["theta"]), d["cy"] + d["R"] * np.sin(d["theta"])], 1)
    u_ring = np.array([orc.coefficients(b, x, y)[0] for x, y in ring])
    u_in = np.array([orc.coefficients(b, x, y)[0] for x, y in d["xy"]])
    assert np.abs(B - G @ u_ring - u_in).max() < 1e-6
    with pytest.raises(ValueError):
        orc.ps_disk(b, 0.5, 0.5, 0.2, 15, 11, 0.0, d["theta"][:15], d["xy"])   # N_circunferencia odd
    with pytest.raises(ValueError):
        orc.ps_disk(b, 0.5, 0.5, 0.2, 16, 10, 0.0, d["theta"][:16], d["xy"])   # N_radio even


@pytest.mark.parametrize("name", ["unit3", "serial"])
def test_ps_rows_oracle_matches_reference(orc, name):
    """Interior-circle rows of a reference mesh through Actualiza_GB(Interfaz&)."""
    g = np.load(os.path.join(GOLDEN, f"ps_rows_{name}.npz"))
    problem, nr = (int(v) for v in g["params"])
    m, circles = full_circles(f"mesh_{name}.npz")
    assert circles
    theta0 = float(m["cfg"][2])
    nodes = {int(r[0]): i for i, r in enumerate(m["node_int"])}
    xy_all, th_all = m["node_dbl"][:, :2], m["node_dbl"][:, 2]
    val, B = m["val0"].copy(), np.zeros(len(m["rowptr"]) - 1)
    rp, col = m["rowptr"], m["col"]
    b = orc.bvp(problem, dom=tuple(m["dom"]))
    for cx, cy, R, gids, inner in circles:
        th = th_all[[nodes[g] for g in gids]]
        xy = xy_all[[nodes[g] for g in inner]]
        G, Bd = orc.ps_disk(b, cx, cy, R, len(gids), nr, theta0, th, xy)
        for p, row in enumerate(inner):
            assert orc.actualiza_gb(int(row), gids, G[p], Bd[p], rp, col, val, B) == 0
    tol = ps_tol(len(circles[0][3]), nr)
    assert np.abs(val - g["val"]).max() <= tol * np.abs(g["val"]).max()
    assert np.abs(B - g["B"]).max() <= tol * np.abs(g["B"]).max()


# ---- GPU: the disk kernels against the reference's golden outputs ----------

def _desc(d, nr=None):
    return dict(cx=d["cx"], cy=d["cy"], radius=d["R"], theta0=d["th0"], n_circle=d["nc"],
                n_radial=nr or d["nr"], periph_theta=d["theta"], inner_xy=d["xy"])


@pytest.mark.gpu
def test_gpu_ps_disks_match_reference(gpu, fk):
    disks = golden_disks()
    for problem in sorted({d["problem"] for d in disks}):
        sel = [d for d in disks if d["problem"] == problem]
        b = gpu.register_bvp(problem, dom=problem_dom(problem))
        out = gpu.solve_disks_ps(b, [_desc(d) for d in sel])    # one batched call per problem
        for d, (G, B) in zip(sel, out):
            tol = ps_tol(d["nc"], d["nr"])
            assert np.abs(G - d["G"]).max() <= tol * np.abs(d["G"]).max(), (problem, d["nc"], d["nr"])
            assert np.abs(B - d["B"]).max() <= tol * np.abs(d["B"]).max(), (problem, d["nc"], d["nr"])
        t = gpu.last_timing()
        assert t[0] > 0 and t[1] > 0


@pytest.mark.gpu
def test_gpu_ps_disk_properties(gpu, fk, orc):
    # the serial driver's sizes on a disk with many interior nodes: -G rows sum
    # to 1 (c = 0) and B - G u(ring) reproduces the exact solution
    rng = np.random.default_rng(5)
    cx, cy, R, nc, nr, th0 = 0.55, 0.45, 0.3, 44, 43, 0.1428
    th = th0 + 2 * np.pi * np.arange(nc) / nc
    rr = 0.95 * R * np.sqrt(rng.random(500))
    aa = 2 * np.pi * rng.random(500)
    xy = np.stack([cx + rr * np.cos(aa), cy + rr * np.sin(aa)], 1)
    b = gpu.register_bvp(fk.FRANKE)
    (G, B), = gpu.solve_disks_ps(b, [dict(cx=cx, cy=cy, radius=R, theta0=th0, n_circle=nc, n_radial=nr,
                                          periph_theta=th, inner_xy=xy)])
    assert np.allclose(-G.sum(1), 1.0, atol=1e-9)
    ob = orc.bvp(0)
    u_ring = np.array([orc.coefficients(ob, cx + R * np.cos(t), cy + R * np.sin(t))[0] for t in th])
    u_in = np.array([orc.coefficients(ob, x, y)[0] for x, y in xy])
    assert np.abs(B - G @ u_ring - u_in).max() < 1e-6
    # against the oracle on a subset
    Go, Bo = orc.ps_disk(ob, cx, cy, R, nc, nr, th0, th, xy[:40])
    tol = ps_tol(nc, nr)
    assert np.abs(G[:40] - Go).max() <= tol * np.abs(Go).max()
    assert np.abs(B[:40] - Bo).max() <= tol * np.abs(Bo).max()


@pytest.mark.gpu
def test_gpu_ps_disk_argument_errors(gpu, fk):
    b = gpu.register_bvp(fk.FRANKE)
    th = np.linspace(0, 2 * np.pi, 16, endpoint=False)
    base = dict(cx=0.5, cy=0.5, radius=0.2, theta0=0.0, n_circle=16, n_radial=11, periph_theta=th,
                inner_xy=np.array([[0.5, 0.55]]))
    for bad in (dict(n_circle=15), dict(n_radial=10), dict(n_radial=65), dict(radius=0.0),
                dict(periph_theta=th[:1])):
        with pytest.raises(fk.FKError):
            gpu.solve_disks_ps(b, [dict(base, **bad)])
    # empty interior: nothing to interpolate, no error
    (G, B), = gpu.solve_disks_ps(b, [dict(base, inner_xy=np.zeros((0, 2)))])
    assert G.size == 0 and B.size == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["unit3", "serial"])
def test_gpu_ps_rows_in_assembly(gpu, fk, name):
    """fk_assemble with the disk solver on: the interior-circle rows added to
    val and B equal the reference's (PS rows of main_test_serial.cpp:67-80)."""
    g = np.load(os.path.join(GOLDEN, f"ps_rows_{name}.npz"))
    problem, nr = (int(v) for v in g["params"])
    m, circles = full_circles(f"mesh_{name}.npz")
    Nl, sup, th0, npc, c2c, c2s = m["cfg"]
    mesh = gpu.mesh_circles(tuple(m["dom"]), int(Nl), sup, th0, int(npc), c2c, c2s)
    rp, col, v0 = gpu.mesh_csr(mesh)
    assert np.array_equal(rp, m["rowptr"]) and np.array_equal(col, m["col"])
    b = gpu.register_bvp(problem, dom=tuple(m["dom"]))
    gpu.set_stream(91)
    r0 = gpu.assemble(mesh, b, 8, 1e-3, fk.FP64)
    gpu.mesh_set_disk_solver(mesh, nr)
    gpu.set_stream(91)
    r1 = gpu.assemble(mesh, b, 8, 1e-3, fk.FP64)
    gpu.mesh_set_disk_solver(mesh, 0)
    tol = ps_tol(len(circles[0][3]), nr)
    dval, dB = r1["val"] - r0["val"], r1["B"] - r0["B"]
    ref_val, ref_B = g["val"] - g["val0"], g["B"]
    assert np.abs(dval - ref_val).max() <= tol * np.abs(ref_val).max()
    assert np.abs(dB - ref_B).max() <= tol * np.abs(ref_B).max()


@pytest.mark.gpu
def test_gpu_serial_driver_pipeline_solves_franke(gpu, fk):
    """The reference serial driver end to end (main_test_serial.cpp:38-89): FK
    rows for the interior nodes of perimeter circles, pseudospectral rows for
    interior circles, then the assembled system solved on the host (GMRES):
    the node values approximate the exact Franke solution to the FK error."""
    dom = (0.0, 0.0, 1.25, 1.25)
    mesh = gpu.mesh_circles(dom, 4, 1.0, 0.1428, 44)
    gpu.mesh_set_disk_solver(mesh, 43)
    b = gpu.register_bvp(fk.FRANKE, dom=dom)
    gpu.set_stream(5)
    r = gpu.assemble(mesh, b, 4000, 1e-4, fk.FP64)
    gpu.mesh_set_disk_solver(mesh, 0)
    rp, col, _ = gpu.mesh_csr(mesh)
    x, it, res, rc = fk.gmres(rp, col, r["val"], r["B"], tol=1e-12, max_iter=4000, restart=80)
    assert rc == 0
    from spac_gb300.workloads import franke
    xy, _ = gpu.mesh_nodes(mesh)
    err = x - franke(xy[:, 0], xy[:, 1])
    assert np.sqrt(np.mean(err ** 2)) < 1e-2 and np.abs(err).max() < 5e-2, (np.sqrt(np.mean(err ** 2)), np.abs(err).max())


@pytest.mark.gpu
def test_gpu_ps_disk_periphery_off_grid(gpu, fk, orc):
    """Constant c (spectral path) with periphery nodes that are not the grid
    angles and fewer of them than grid angles (n_periph = 12, N_c = 16): the
    cardinal right-hand sides are general ring data; against the oracle."""
    rng = np.random.default_rng(8)
    cx, cy, R, nc, nr, th0 = 0.45, 0.55, 0.25, 16, 11, 0.3
    th = 0.05 + 2 * np.pi * np.arange(12) / 12 + 0.02 * rng.standard_normal(12)
    rr = 0.9 * R * np.sqrt(rng.random(20))
    aa = 2 * np.pi * rng.random(20)
    xy = np.stack([cx + rr * np.cos(aa), cy + rr * np.sin(aa)], 1)
    for problem, dom in ((fk.FRANKE, (0, 0, 1, 1)), (fk.MONEGROS, (-200, -200, 200, 200))):
        c = (cx, cy, R) if problem == fk.FRANKE else (-72.0, -38.0, 5.0)
        pts = xy if problem == fk.FRANKE else np.stack([c[0] + (xy[:, 0] - cx) * 20, c[1] + (xy[:, 1] - cy) * 20], 1)
        b = gpu.register_bvp(problem, dom=dom)
        (G, B), = gpu.solve_disks_ps(b, [dict(cx=c[0], cy=c[1], radius=c[2], theta0=th0, n_circle=nc, n_radial=nr,
                                              periph_theta=th, inner_xy=pts)])
        Go, Bo = orc.ps_disk(orc.bvp(problem, dom=dom), c[0], c[1], c[2], nc, nr, th0, th, pts)
        tol = ps_tol(nc, nr)
        assert np.abs(G - Go).max() <= tol * np.abs(Go).max(), problem
        assert np.abs(B - Bo).max() <= tol * np.abs(Bo).max(), problem
