"""The CPU oracle against the reference itself.

Golden fixtures in tests/golden/ were produced by the reference's own sources
(tests/golden/make_golden.py); with the sequential random stream the oracle
must reproduce them bit for bit.  Where the reference build is present
(oracle/_ref), extra cases are compared live.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_philox_known_answers(orc):
    # Random123 Philox4x32-10 known-answer vectors (Salmon et al., SC'11 distribution)
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_distance_functors_and_coefficients(orc):
    g = np.load(os.path.join(GOLDEN, "functors.npz"))
    b0, b2 = orc.bvp(0, cv=1), orc.bvp(2, cv=1)
    for i, (x, y) in enumerate(g["probe"]):
        assert orc.rectangulo(g["rect"], x, y) == list(g["d_rect"][i])
        assert orc.circulo(g["circ"], x, y) == list(g["d_circ"][i])
        assert orc.coefficients(b0, x, y) == list(g["coefs"][i][:12])
        assert orc.coefficients(b2, x, y) == list(g["coefs"][i][12:])
    # point at the circle centre: radius clamped at 5e-4 (Circulo.hpp:17)
    assert orc.circulo(g["circ"], 0.5, 0.45) == list(g["circ_center"])


def test_monegros_coefficients(orc):
    """Both Monegros problems (Monegros_Revamped.hpp, c = -1; Monegros_Poisson.hpp, c = 0)."""
    g = np.load(os.path.join(GOLDEN, "coefs_monegros.npz"))
    b1, b5 = orc.bvp(1, cv=1), orc.bvp(orc.MONEGROS_POISSON, cv=1)
    for i, (x, y) in enumerate(g["probe"]):
        assert orc.coefficients(b1, x, y) == list(g["coefs"][i][:12])
        assert orc.coefficients(b5, x, y) == list(g["coefs"][i][12:])


@pytest.mark.parametrize("problem", [0, 2])
def test_cv_table_lookup(orc, problem):
    """The oracle's tabulated grad u_hat (cv = 3, the layout of
    fk_mlp_get_table): F = -sigma grad u_hat with grad u_hat bilinear in the
    lattice, the point clamped into the rectangle; against numpy on a random
    table, at points inside, outside and on the edges of the rectangle."""
    G, rect = 17, (0.2, -0.1, 1.3, 0.7)
    rng = np.random.default_rng(3)
    tab = rng.standard_normal((G, G, 2)).astype(np.float32)  # [j][i][component]
    flat = np.ascontiguousarray(tab.ravel())
    T = orc.CvTable(G, (C.c_double * 4)(*rect), flat.ctypes.data_as(C.POINTER(C.c_float)))
    b = orc.bvp(problem, cv=3, mlp=T)
    pts = np.concatenate([rng.uniform(-0.2, 1.5, size=(200, 2)), [[rect[0], rect[1]], [rect[2], rect[3]]]])
    for x, y in pts:
        c = orc.coefficients(b, x, y)
        s = c[6]  # sigma = s I for both problems
        u = min(max((x - rect[0]) * (G - 1) / (rect[2] - rect[0]), 0.0), G - 1 - 1e-3)
        v = min(max((y - rect[1]) * (G - 1) / (rect[3] - rect[1]), 0.0), G - 1 - 1e-3)
        i, j = int(u), int(v)
        fu, fv = u - i, v - j
        t = tab.astype(np.float64)
        g = (1 - fv) * ((1 - fu) * t[j, i] + fu * t[j, i + 1]) + fv * ((1 - fu) * t[j + 1, i] + fu * t[j + 1, i + 1])
        assert np.allclose(c[10:12], -s * g, rtol=1e-13, atol=1e-14), (x, y)
        assert c[7] == 0.0 and c[8] == 0.0


def test_point_solves_bit_exact(orc):
    pts = np.load(os.path.join(GOLDEN, "points.npy"))
    for row in pts:
        problem, use_F = int(row[0]), int(row[1])
        dom = tuple(row[2:6])
        x, y, sk = row[6], row[7], int(row[8])
        sub = row[9:13]
        N, h = int(row[13]), row[14]
        ref = row[15:24]
        s = orc.Session(orc.RNG_SEQUENTIAL)
        b = orc.bvp(problem, cv=use_F, dom=dom)
        if sk == 0:
            shp = None
        elif sk == 1:
            shp = orc.shape(orc.CIRCLE, sub[:3])
        else:
            shp = orc.shape(orc.RECT, sub)
        out = s.point_solve(b, x, y, N, h, sub=shp)
        assert [out[k] for k in orc.STAT_NAMES] == list(ref), (problem, use_F)


def _mesh(name):
    return np.load(os.path.join(GOLDEN, f"mesh_{name}.npz"))


def _arcs(m):
    ii, dd = m["iface_int"], m["iface_dbl"]
    gids = m["iface_gids"]
    theta_of = {int(g): t for g, t in zip(m["node_int"][:, 0], m["node_dbl"][:, 2])}
    arcs, off, poff = [], 0, 0
    for k in range(len(ii)):
        n = int(ii[k, 2])
        g = gids[off:off + n]
        off += n
        a = dict(interior=int(ii[k, 0]), perimeter=int(ii[k, 1]), n=n, cx=dd[k, 0], cy=dd[k, 1], radius=dd[k, 2],
                 c2=dd[k, 3], gids=g, theta=np.array([theta_of[int(v)] for v in g]))
        lo, hi = m["iface_ipsi_off"][k], m["iface_ipsi_off"][k + 1]
        if hi > lo:
            a["iPsi"] = m["iface_ipsi"][lo:hi].reshape((n, n), order="F")
        arcs.append(a)
    return arcs


@pytest.mark.parametrize("name", ["serial", "unit3"])
def test_calcula_psi_bit_exact(orc, name):
    for a in _arcs(_mesh(name)):
        if "iPsi" in a:
            iP, _ = orc.calcula_psi(a["theta"], a["c2"])
            assert np.array_equal(iP, a["iPsi"])


@pytest.mark.parametrize("fname", ["assembly_unit3_p0_f0.npz", "assembly_unit3_p2_f1.npz"])
def test_node_solves_and_csr_bit_exact(orc, fname):
    A = np.load(os.path.join(GOLDEN, fname))
    problem, use_F, N, h = int(A["params"][0]), int(A["params"][1]), int(A["params"][2]), A["params"][3]
    m = _mesh("unit3")
    arcs = _arcs(m)
    node_xy = {int(g): (x, y) for g, (x, y) in zip(m["node_int"][:, 0], m["node_dbl"][:, :2])}
    s = orc.Session(orc.RNG_SEQUENTIAL)
    b = orc.bvp(problem, cv=use_F)
    val = A["val0"].copy()
    B = np.zeros(len(A["rowptr"]) - 1)
    rp = np.ascontiguousarray(A["rowptr"], dtype=np.int32)
    col = np.ascontiguousarray(A["col"], dtype=np.int32)
    goff = 0
    L = orc.load()
    for k, (row, iface, frontera, nG) in enumerate(A["item_int"]):
        x, y = node_xy[int(row)]
        G, Bv, st = s.node_solve_arc(b, x, y, frontera, arcs[iface], N, h)
        ref_B, ref_st = A["item_dbl"][k, 0], A["item_dbl"][k, 1:]
        assert Bv == ref_B
        if frontera:
            assert nG == 0
        else:
            assert nG == len(G)
            assert np.array_equal(G, A["item_G"][goff:goff + nG])
            assert np.array_equal(A["item_cols"][goff:goff + nG], arcs[iface]["gids"])
            assert [st[q] for q in orc.STAT_NAMES] == list(ref_st)
        cols = np.ascontiguousarray(arcs[iface]["gids"], dtype=np.int32)
        Gc = np.ascontiguousarray(G if not frontera else np.zeros(0))
        rc = L.orc_actualiza_gb(int(row), len(Gc), cols.ctypes.data_as(C.POINTER(C.c_int)),
                                Gc.ctypes.data_as(C.POINTER(C.c_double)), Bv, rp.ctypes.data_as(C.POINTER(C.c_int)),
                                col.ctypes.data_as(C.POINTER(C.c_int)), val.ctypes.data_as(C.POINTER(C.c_double)),
                                B.ctypes.data_as(C.POINTER(C.c_double)))
        assert rc == 0
        goff += nG
    assert np.array_equal(val, A["val"])
    assert np.array_equal(B, A["B"])


def test_full_pivot_inverse_properties(orc):
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 20, 46):
        A = rng.standard_normal((n, n)) + n * np.eye(n)
        inv = orc.full_pivot_inverse(A)
        assert np.allclose(inv @ A, np.eye(n), atol=1e-10)


def test_live_reference_extra_cases(orc):
    """Extra sequential-stream cases run against the compiled reference."""
    if not os.path.exists(orc.REF_LIB):
        if not os.path.isdir(orc.REF_SRC):
            pytest.skip("reference sources not present")
        orc.build(ref=True)
    R = C.CDLL(orc.REF_LIB)
    R.ref_solver_new.restype = C.c_void_p
    R.ref_solver_new.argtypes = [C.c_int]
    R.ref_solver_free.argtypes = [C.c_void_p]
    dp = C.POINTER(C.c_double)
    R.ref_point_solve.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, C.c_int, dp, C.c_double, C.c_double, C.c_uint,
                                  C.c_double, dp]
    rs = R.ref_solver_new(1)
    s = orc.Session(orc.RNG_SEQUENTIAL)
    rng = np.random.default_rng(11)
    # consecutive calls share the stream, as one FeynmanKacSolver object does
    for _ in range(12):
        problem = int(rng.integers(0, 3)) if False else int(rng.choice([0, 2]))
        use_F = int(rng.integers(0, 2))
        x, y = rng.uniform(0.02, 0.98, 2)
        h = float(rng.choice([1e-3, 4e-3, 1e-2]))
        sub = (x - 0.2, y - 0.15, x + 0.1, y + 0.25)
        out = (C.c_double * 9)()
        R.ref_point_solve(rs, problem, use_F, (C.c_double * 4)(0, 0, 1, 1), 2, (C.c_double * 4)(*sub), x, y, 50, h, out)
        o = s.point_solve(orc.bvp(problem, cv=use_F), x, y, 50, h, sub=orc.shape(orc.RECT, sub))
        assert [o[k] for k in orc.STAT_NAMES] == list(out)
    R.ref_solver_free(rs)
