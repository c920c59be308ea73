"""Generates the golden fixtures of tests/golden/ by running the reference
implementation itself: SpAc's own hot-path sources compiled unmodified
against oracle/shim (oracle/Makefile target `ref`, library oracle/_ref/).

Run where the reference sources exist:  python tests/golden/make_golden.py
(`python tests/golden/make_golden.py ps` writes only the pseudospectral disk
fixtures ps_disks.npz and ps_rows_*.npz; `... points` only points.npy and
coefs_monegros.npz.)
The random stream is the shim's sequential stream with one OpenMP thread,
which the oracle reproduces in its sequential mode.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libspac_ref.so")
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# reference mesh configurations: (name, dom, Nl, superposicion, theta0, nodes per circle)
MESHES = [
    ("serial", (0.0, 0.0, 1.25, 1.25), 4, 1.0, 0.1428, 44),   # main_test_serial.cpp:38-48
    ("unit3", (0.0, 0.0, 1.0, 1.0), 3, 1.2, 0.121, 20),
]
ASSEMBLIES = [  # (mesh name, problem, use_F, N, h)
    ("unit3", 0, 0, 64, 1e-3),
    ("unit3", 2, 1, 64, 1e-3),
]
# pseudospectral disks (PseudoespectralCirculoSolver): (problem, cx, cy, R, N_circunferencia, N_radio, theta0,
# periphery angle offset from the angular grid, interior nodes)
PS_DISKS = [
    (0, 0.5, 0.5, 0.3, 16, 11, 0.1, 0.0, 12),
    (1, -72.0, -38.0, 5.0, 20, 15, 0.3, 0.0, 9),
    (2, 0.4, 0.6, 0.25, 12, 9, 0.0, 0.2, 7),
    (0, 0.3, 0.7, 0.2, 44, 43, 0.1428, 0.0, 16),   # the serial driver's sizes (main_test_serial.cpp:48,70)
]
PS_ROWS = [("unit3", 0, 11), ("serial", 0, 43)]  # (mesh, problem, N_radio): interior-circle rows only
POINTS = [  # (problem, use_F, dom, (x, y), sub_kind, sub, N, h)
    (0, 0, (0, 0, 1, 1), (0.31, 0.4), 0, None, 200, 1e-3),
    (0, 1, (0, 0, 1, 1), (0.8, 0.85), 0, None, 200, 1e-2),
    (1, 0, (-200, -200, 200, 200), (-72.0, -38.0), 2, (-72.3, -38.2, -71.75, -37.7), 200, 1e-3),
    (1, 1, (-200, -200, 200, 200), (150.0, 40.0), 2, (149.7, 39.8, 150.25, 40.3), 200, 1e-2),
    (2, 0, (0, 0, 1, 1), (0.5, 0.5), 1, (0.2, 0.5, 0.5), 200, 1e-3),
    (2, 1, (0, 0, 1, 1), (0.05, 0.93), 0, None, 200, 1e-3),
    # Monegros_Poisson (c = 0), the problem of main_test_mpi.cpp
    (5, 0, (-200, -200, 200, 200), (-72.0, -38.0), 2, (-72.3, -38.2, -71.75, -37.7), 200, 1e-3),
    (5, 1, (-200, -200, 200, 200), (10.0, -20.0), 1, (0.3, 10.1, -20.05), 200, 1e-2),
]
# coefficient probes of the two Monegros problems (1: c = -1, 5: c = 0) on their domain
MONEGROS_PROBES = 64


def ref():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    L = C.CDLL(REF_LIB)
    L.ref_solver_new.restype = C.c_void_p
    L.ref_solver_new.argtypes = [C.c_int]
    L.ref_point_solve.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, _dp, C.c_double, C.c_double, C.c_uint,
                                  C.c_double, _dp]
    L.ref_assemble_circles.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int,
                                       C.c_double, C.c_double, C.c_uint, C.c_double, C.c_int]
    L.ref_circulo.argtypes = [_dp, C.c_double, C.c_double, _dp]
    L.ref_rectangulo.argtypes = [_dp, C.c_double, C.c_double, _dp]
    L.ref_coefficients.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
    L.ref_calcula_psi.argtypes = [C.c_int, _dp, C.c_double, _dp]
    L.ref_calcula_psi.restype = C.c_double
    return L


def mesh_and_assembly(L, name, problem, use_F, N, h, solve, do_solve=1):
    cfg = {m[0]: m for m in MESHES}[name]
    _, dom, Nl, sup, th0, npc = cfg
    s = L.ref_solver_new(1)
    d = (C.c_double * 4)(*dom)
    L.ref_assemble_circles(s, problem, use_F, d, Nl, sup, th0, npc, 1.5, 1.1, N, h, do_solve if solve else 0)
    nr, nnz, ni, nn, nf = (C.c_int() for _ in range(5))
    L.ref_last_sizes(C.byref(nr), C.byref(nnz), C.byref(ni), C.byref(nn), C.byref(nf))
    rp = np.zeros(nr.value + 1, np.int32)
    col = np.zeros(nnz.value, np.int32)
    v0 = np.zeros(nnz.value)
    val = np.zeros(nnz.value)
    B = np.zeros(nr.value)
    L.ref_last_csr(rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip), v0.ctypes.data_as(_dp), val.ctypes.data_as(_dp),
                   B.ctypes.data_as(_dp))
    out = dict(rowptr=rp, col=col, val0=v0)
    ints = (C.c_int * 4)()
    dbl = (C.c_double * 10)()
    nodes_i, nodes_d = [], []
    for i in range(nn.value):
        L.ref_last_node(i, ints, dbl)
        nodes_i.append(list(ints))
        nodes_d.append(list(dbl)[:3])
    out["node_int"] = np.array(nodes_i, np.int32)        # gid, iface_x, iface_y, frontera
    out["node_dbl"] = np.array(nodes_d)                  # x, y, theta
    if_i, if_d, gids, inner, ipsi, ipsi_off = [], [], [], [], [], [0]
    for i in range(nf.value):
        L.ref_last_iface(i, ints, dbl)
        ii = list(ints)
        if_i.append(ii)
        if_d.append(list(dbl)[:4])
        g = np.zeros(ii[2], np.int32)
        t = np.zeros(ii[2])
        P = np.zeros(ii[2] * ii[2])
        ig = np.zeros(max(ii[3], 1), np.int32)
        has = L.ref_last_iface_arrays(i, g.ctypes.data_as(_ip), t.ctypes.data_as(_dp), P.ctypes.data_as(_dp),
                                      ig.ctypes.data_as(_ip))
        gids.append(g)
        inner.append(ig[:ii[3]])
        if has:
            ipsi.append(P)
            ipsi_off.append(ipsi_off[-1] + len(P))
        else:
            ipsi_off.append(ipsi_off[-1])
    out["iface_int"] = np.array(if_i, np.int32)          # interior, perimeter, n, n_inner
    out["iface_dbl"] = np.array(if_d)                    # cx, cy, radius, c2 (c2 only meaningful on perimeter arcs)
    out["iface_gids"] = np.concatenate(gids)
    out["iface_inner"] = np.concatenate(inner) if inner else np.zeros(0, np.int32)
    out["iface_ipsi"] = np.concatenate(ipsi) if ipsi else np.zeros(0)
    out["iface_ipsi_off"] = np.array(ipsi_off, np.int64)
    if solve:
        it_i, it_d, it_cols, it_G = [], [], [], []
        for i in range(ni.value):
            L.ref_last_item(i, ints, dbl)
            ii = list(ints)
            it_i.append(ii)
            it_d.append(list(dbl))
            cols = np.zeros(max(ii[3], 1), np.int32)
            G = np.zeros(max(ii[3], 1))
            L.ref_last_item_G(i, cols.ctypes.data_as(_ip), G.ctypes.data_as(_dp))
            it_cols.append(cols[:ii[3]])
            it_G.append(G[:ii[3]])
        out["item_int"] = np.array(it_i, np.int32)       # row, iface, frontera, nG
        out["item_dbl"] = np.array(it_d)                 # B, phi, phiphi, phi_VR, phiphi_VR, xi, xixi, xiphi, APL, RNGC
        out["item_cols"] = np.concatenate(it_cols) if it_cols else np.zeros(0, np.int32)
        out["item_G"] = np.concatenate(it_G) if it_G else np.zeros(0)
        out["val"] = val
        out["B"] = B
        out["params"] = np.array([problem, use_F, N, h])
    L.ref_solver_free(C.c_void_p(s))
    return out


def ps_fixtures(L):
    L.ref_ps_disk.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, C.c_int,
                              _dp, C.c_int, _dp, _dp, _dp]
    L.ref_set_ps_radial.argtypes = [C.c_int]
    rng = np.random.default_rng(2027)
    cases, th, xy, G, B = [], [], [], [], []
    for problem, cx, cy, R, nc, nr, th0, off, n_in in PS_DISKS:
        pth = th0 + off + 2 * np.pi * np.arange(nc) / nc
        rr = 0.92 * R * np.sqrt(rng.random(n_in))
        aa = 2 * np.pi * rng.random(n_in)
        pts = np.ascontiguousarray(np.stack([cx + rr * np.cos(aa), cy + rr * np.sin(aa)], 1))
        g = np.zeros((n_in, nc))
        b = np.zeros(n_in)
        L.ref_ps_disk(problem, cx, cy, R, nc, nr, th0, nc, pth.ctypes.data_as(_dp), n_in, pts.ctypes.data_as(_dp),
                      g.ctypes.data_as(_dp), b.ctypes.data_as(_dp))
        cases.append([problem, cx, cy, R, nc, nr, th0, nc, n_in])
        th.append(pth)
        xy.append(pts)
        G.append(g.ravel())
        B.append(b)
    np.savez_compressed(os.path.join(HERE, "ps_disks.npz"), cases=np.array(cases), periph_theta=np.concatenate(th),
                        inner_xy=np.concatenate(xy), G=np.concatenate(G), B=np.concatenate(B))
    for name, problem, nr in PS_ROWS:
        L.ref_set_ps_radial(nr)
        a = mesh_and_assembly(L, name, problem, 0, 1, 1e-3, True, do_solve=2)
        L.ref_set_ps_radial(0)
        np.savez_compressed(os.path.join(HERE, f"ps_rows_{name}.npz"), val=a["val"], B=a["B"], val0=a["val0"],
                            params=np.array([problem, nr]))


def point_fixtures(L):
    """points.npy (reference point solves) and coefs_monegros.npz."""
    # point solves: each on a fresh session (sequential stream from the start)
    pts = []
    for problem, use_F, dom, (x, y), sk, sub, N, h in POINTS:
        s = L.ref_solver_new(1)
        out = (C.c_double * 9)()
        sp = (C.c_double * 4)(*(sub if sub else (0, 0, 0, 0)))
        L.ref_point_solve(s, problem, use_F, (C.c_double * 4)(*dom), sk, sp, x, y, N, h, out)
        L.ref_solver_free(C.c_void_p(s))
        subv = list(sub) if sub else [0, 0, 0, 0]
        subv += [0] * (4 - len(subv))
        pts.append([problem, use_F, *dom, x, y, sk, *subv, N, h, *list(out)])
    np.save(os.path.join(HERE, "points.npy"), np.array(pts))
    rng = np.random.default_rng(11)
    probe = rng.uniform(-200.0, 200.0, size=(MONEGROS_PROBES, 2))
    o12 = (C.c_double * 12)()
    coefs = []
    for x, y in probe:
        row = []
        for p in (1, 5):
            L.ref_coefficients(p, x, y, o12)
            row += list(o12)
        coefs.append(row)
    np.savez_compressed(os.path.join(HERE, "coefs_monegros.npz"), probe=probe, coefs=np.array(coefs))


def main():
    L = ref()
    L.ref_solver_free.argtypes = [C.c_void_p]
    if sys.argv[1:] == ["ps"]:
        ps_fixtures(L)
        print("pseudospectral fixtures written to", HERE)
        return 0
    if sys.argv[1:] == ["points"]:
        point_fixtures(L)
        print("point fixtures written to", HERE)
        return 0
    for name, dom, Nl, sup, th0, npc in MESHES:
        m = mesh_and_assembly(L, name, 0, 0, 1, 1e-3, False)
        np.savez_compressed(os.path.join(HERE, f"mesh_{name}.npz"), dom=np.array(dom),
                            cfg=np.array([Nl, sup, th0, npc, 1.5, 1.1]), **m)
    for name, problem, use_F, N, h in ASSEMBLIES:
        a = mesh_and_assembly(L, name, problem, use_F, N, h, True)
        np.savez_compressed(os.path.join(HERE, f"assembly_{name}_p{problem}_f{use_F}.npz"), **a)
    # the reference's text outputs of the first assembly (Escribe_GB_COO, then
    # Escribe_GB_CSR, which rewrites B.txt with 10 decimals; Escribe_Posiciones)
    import shutil
    import tempfile
    tmp = tempfile.mkdtemp()
    os.makedirs(os.path.join(tmp, "Output"))
    L.ref_set_output_dir.argtypes = [C.c_char_p]
    L.ref_set_output_dir(tmp.encode())
    name, problem, use_F, N, h = ASSEMBLIES[0]
    mesh_and_assembly(L, name, problem, use_F, N, h, True)
    L.ref_set_output_dir(b"")
    out = os.path.join(HERE, "text_unit3")
    os.makedirs(out, exist_ok=True)
    for f in ("G.txt", "B.txt", "G_i.txt", "G_j.txt", "G_ij.txt", "knot_position.txt"):
        shutil.copy(os.path.join(tmp, "Output", f), os.path.join(out, f))
    shutil.rmtree(tmp)
    point_fixtures(L)
    # distance functors and coefficients at probe points, incl. centre lines and corners
    rng = np.random.default_rng(7)
    probe = np.concatenate([rng.uniform(-0.3, 1.3, size=(200, 2)),
                            np.array([[0.5, 0.5], [0.5, 0.9], [0.9, 0.5], [0.5, 1.2], [1.2, 0.5], [-0.1, -0.1],
                                      [1.1, -0.2], [0.0, 0.0], [1.0, 1.0], [0.25, 0.5], [0.5, 0.25]])])
    rect = (0.1, 0.0, 0.9, 1.0)
    circ = (0.4, 0.5, 0.45)
    d_rect, d_circ, coefs = [], [], []
    o5 = (C.c_double * 5)()
    o12 = (C.c_double * 12)()
    for x, y in probe:
        L.ref_rectangulo((C.c_double * 4)(*rect), x, y, o5)
        d_rect.append(list(o5))
        L.ref_circulo((C.c_double * 3)(*circ), x, y, o5)
        d_circ.append(list(o5))
        row = []
        for p in (0, 2):
            L.ref_coefficients(p, x, y, o12)
            row += list(o12)
        coefs.append(row)
    L.ref_circulo((C.c_double * 3)(*circ), 0.5, 0.45, o5)
    np.savez_compressed(os.path.join(HERE, "functors.npz"), probe=probe, rect=np.array(rect), circ=np.array(circ),
                        d_rect=np.array(d_rect), d_circ=np.array(d_circ), coefs=np.array(coefs),
                        circ_center=np.array(list(o5)))
    ps_fixtures(L)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    sys.exit(main())
