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
