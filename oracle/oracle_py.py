"""ctypes binding of the CPU oracle (oracle/fk_oracle.cpp) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product path never does.  `build()` compiles the oracle with
the recipe in oracle/Makefile.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfk_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libspac_ref.so")
REF_SRC = "/root/reference"

RNG_PHILOX, RNG_SEQUENTIAL = 0, 1
RECT, CIRCLE = 0, 1
OUT_INSIDE, OUT_DOMAIN, OUT_SUBDOMAIN = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Bvp(C.Structure):
    _fields_ = [("problem", C.c_int), ("cv", C.c_int), ("dom_shape", C.c_int), ("dom", C.c_double * 4),
                ("prob", C.c_double * 4), ("mlp", C.c_void_p)]


class Shape(C.Structure):
    _fields_ = [("shape", C.c_int), ("p", C.c_double * 4)]


class Arc(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double), ("c2", C.c_double),
                ("interior", C.c_int), ("n", C.c_int), ("theta", _dp), ("iPsi", _dp)]


class Knn(C.Structure):
    _fields_ = [("m", C.c_int), ("xy", _dp), ("k", C.c_int), ("eps", C.c_double)]


class Exit(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("Y", C.c_double), ("Z", C.c_double), ("xi", C.c_double),
                ("t", C.c_double), ("outcome", C.c_int), ("steps", C.c_int)]


class CvTable(C.Structure):
    """orc_cv_table: a tabulated grad u_hat (bvp cv = 3; the layout of fk_mlp_get_table)."""
    _fields_ = [("grid", C.c_int), ("rect", C.c_double * 4), ("tab", C.POINTER(C.c_float))]


class Mlp(C.Structure):
    _fields_ = [("width", C.c_int), ("in_lo", C.c_double * 2), ("in_scale", C.c_double * 2)] + \
        [(n, _dp) for n in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4")]


def build(ref=None):
    """Build the oracle (and, where the reference sources exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    return LIB


_O = None


def load():
    global _O
    if _O is None:
        if not os.path.exists(LIB):
            build(ref=False)
        L = C.CDLL(LIB)
        L.orc_session_new.restype = C.c_void_p
        L.orc_session_new.argtypes = [C.c_int, C.c_uint64]
        L.orc_session_free.argtypes = [C.c_void_p]
        L.orc_session_set_stream.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_circulo.argtypes = [_dp, C.c_double, C.c_double, _dp]
        L.orc_rectangulo.argtypes = [_dp, C.c_double, C.c_double, _dp]
        L.orc_coefficients.argtypes = [C.POINTER(Bvp), C.c_double, C.c_double, _dp]
        L.orc_path.argtypes = [C.c_void_p, C.POINTER(Bvp), C.POINTER(Shape), C.c_double, C.c_double, C.c_double,
                               C.c_uint32, C.c_uint32, C.c_int, C.POINTER(Exit)]
        L.orc_point_solve.argtypes = [C.c_void_p, C.POINTER(Bvp), C.POINTER(Shape), C.c_double, C.c_double,
                                      C.c_uint, C.c_double, C.c_uint32, _dp]
        L.orc_node_solve_arc.argtypes = [C.c_void_p, C.POINTER(Bvp), C.c_double, C.c_double, C.c_int,
                                         C.POINTER(Arc), C.c_uint, C.c_double, C.c_uint32, _dp, _dp, _dp]
        L.orc_node_solve_knn.argtypes = [C.c_void_p, C.POINTER(Bvp), C.c_double, C.c_double, C.POINTER(Shape),
                                         C.POINTER(Knn), C.c_uint, C.c_double, C.c_uint32, _dp, _dp, _dp, _dp]
        L.orc_full_pivot_inverse.argtypes = [C.c_int, _dp, _dp]
        L.orc_calcula_psi.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.orc_calcula_psi.restype = C.c_double
        L.orc_knn_weights.argtypes = [C.POINTER(Knn), C.c_double, C.c_double, _ip, _dp]
        L.orc_actualiza_gb.argtypes = [C.c_int, C.c_int, _ip, _dp, C.c_double, _ip, _ip, _dp, _dp]
        L.orc_mlp_eval.argtypes = [C.POINTER(Mlp), C.c_double, C.c_double, _dp]
        L.orc_mlp_loss_grad.argtypes = [C.POINTER(Mlp), C.c_int, _dp, _dp, _dp]
        L.orc_mlp_loss_grad.restype = C.c_double
        L.orc_ps_disk.argtypes = [C.POINTER(Bvp), C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double,
                                  C.c_int, _dp, C.c_int, _dp, _dp, _dp]
        _O = L
    return _O


def bvp(problem, cv=0, dom=(0, 0, 1, 1), dom_shape=RECT, prob=(0, 0, 0, 0), mlp=None):
    return Bvp(problem, cv, dom_shape, (C.c_double * 4)(*dom), (C.c_double * 4)(*prob),
               C.cast(C.pointer(mlp), C.c_void_p) if mlp is not None else None)


def shape(kind, p):
    p = list(p) + [0.0] * (4 - len(p))
    return Shape(kind, (C.c_double * 4)(*p))


def philox(ctr, key):
    L = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


ROBIN = 4  # ORC_PROBLEM_ROBIN: prob = (side mask, varphi, rho, 0)
MONEGROS_POISSON = 5  # ORC_PROBLEM_MONEGROS_POISSON: BVPs/Monegros_Poisson.hpp (c = 0)
STAT_NAMES = ("phi", "phiphi", "phi_VR", "phiphi_VR", "xi", "xixi", "xiphi", "APL", "RNGC")


class Session:
    """An RNG stream: Philox counters keyed by `seed`, or the sequential stream
    the compiled reference consumes with one OpenMP thread."""

    def __init__(self, mode=RNG_PHILOX, seed=1234, stream=0):
        self.L = load()
        self.h = self.L.orc_session_new(mode, seed)
        self.L.orc_session_set_stream(self.h, stream)

    def set_stream(self, s):
        self.L.orc_session_set_stream(self.h, s)

    def __del__(self):
        try:
            self.L.orc_session_free(self.h)
        except Exception:
            pass

    def point_solve(self, b, x, y, N, h, item=0, sub=None):
        out = (C.c_double * 9)()
        rc = self.L.orc_point_solve(self.h, C.byref(b), C.byref(sub) if sub is not None else None, x, y, N, h, item,
                                    out)
        assert rc == 0
        return dict(zip(STAT_NAMES, list(out)))

    def path(self, b, x, y, h, item, path, sub=None, max_steps=0):
        e = Exit()
        self.L.orc_path(self.h, C.byref(b), C.byref(sub) if sub is not None else None, x, y, h, item, path,
                        max_steps, C.byref(e))
        return e

    def node_solve_arc(self, b, x, y, frontera, arc, N, h, item=0):
        theta = np.ascontiguousarray(arc["theta"], dtype=np.float64)
        iPsi = np.ascontiguousarray(np.asarray(arc["iPsi"]).ravel(order="F"), dtype=np.float64)
        a = Arc(arc["cx"], arc["cy"], arc["radius"], arc["c2"], arc["interior"], len(theta),
                theta.ctypes.data_as(_dp), iPsi.ctypes.data_as(_dp))
        G = np.zeros(len(theta))
        B = C.c_double()
        st = (C.c_double * 9)()
        rc = self.L.orc_node_solve_arc(self.h, C.byref(b), x, y, int(frontera), C.byref(a), N, h, item,
                                       G.ctypes.data_as(_dp), C.byref(B), st)
        assert rc == 0
        return G, B.value, dict(zip(STAT_NAMES, list(st)))

    def node_solve_knn(self, b, x, y, rect, nodes_xy, k, eps, N, h, item=0):
        xy = np.ascontiguousarray(nodes_xy, dtype=np.float64).ravel()
        kn = Knn(len(xy) // 2, xy.ctypes.data_as(_dp), k, eps)
        G = np.zeros(len(xy) // 2)
        B = C.c_double()
        st = (C.c_double * 9)()
        ex = (C.c_double * 4)()
        sh = shape(RECT, rect)
        rc = self.L.orc_node_solve_knn(self.h, C.byref(b), x, y, C.byref(sh), C.byref(kn), N, h, item,
                                       G.ctypes.data_as(_dp), C.byref(B), st, ex)
        assert rc == 0
        return G, B.value, dict(zip(STAT_NAMES, list(st))), list(ex)


def calcula_psi(theta, c2):
    L = load()
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    n = len(theta)
    out = np.zeros(n * n)
    k = L.orc_calcula_psi(n, theta.ctypes.data_as(_dp), c2, out.ctypes.data_as(_dp))
    return out.reshape((n, n), order="F"), k


def full_pivot_inverse(A):
    L = load()
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    a = np.ascontiguousarray(A.ravel(order="F"))
    out = np.zeros(n * n)
    L.orc_full_pivot_inverse(n, a.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    return out.reshape((n, n), order="F")


def ps_disk(b, cx, cy, radius, n_circle, n_radial, theta0, periph_theta, inner_xy):
    """PseudoespectralCirculoSolver::Inicializa + Resuelve(bvp, interior, periphery):
    returns G (n_inner x n_periph) and B (n_inner)."""
    L = load()
    pth = np.ascontiguousarray(periph_theta, dtype=np.float64)
    xy = np.ascontiguousarray(inner_xy, dtype=np.float64).reshape(-1, 2)
    G = np.zeros((len(xy), len(pth)))
    B = np.zeros(len(xy))
    rc = L.orc_ps_disk(C.byref(b), cx, cy, radius, n_circle, n_radial, theta0, len(pth), pth.ctypes.data_as(_dp),
                       len(xy), xy.ctypes.data_as(_dp), G.ctypes.data_as(_dp), B.ctypes.data_as(_dp))
    if rc != 0:
        raise ValueError("orc_ps_disk: invalid sizes")
    return G, B


def square_patch_mesh(dom, n_sub, nodes_per_side, enlarge):
    """The square-patch layout of configs 2 and 5, restated in numpy for the
    CPU side (the reference has no such geometry; its circle layout is
    Malla::Construye_Cuadrado, Mesh/Malla.cpp:12-83, and its CSR rows come
    from SistemaLineal::Anadir_Lista_Adyacencia, Mesh/SistemaLineal.cpp:8-18).

    n_sub x n_sub subdomains of dom, each enlarged by `enlarge` of its width
    per side; nodes_per_side equispaced nodes per patch side, kept where they
    lie strictly inside dom, numbered patch by patch (x-index outer) along a
    counter-clockwise chain (bottom, right, top, left) that starts after a
    dropped node when the patch is clipped.  An item is (node, patch holding
    the node strictly inside), in node order, then patch order.

    Returns dict(nodes (n, 2), patches [dict(rect, chain (m, 2), gids)],
    items [(gid, patch)], spacing)."""
    dom = [float(v) for v in dom]
    Hx, Hy = (dom[2] - dom[0]) / n_sub, (dom[3] - dom[1]) / n_sub
    sx = (1 + 2 * enlarge) * Hx / (nodes_per_side + 1)
    sy = (1 + 2 * enlarge) * Hy / (nodes_per_side + 1)
    tol = 1e-12 * max(dom[2] - dom[0], dom[3] - dom[1])
    q = np.arange(1, nodes_per_side + 1)
    nodes, patches = [], []
    for a in range(n_sub):
        for b in range(n_sub):
            r = (dom[0] + (a - enlarge) * Hx, dom[1] + (b - enlarge) * Hy,
                 dom[0] + (a + 1 + enlarge) * Hx, dom[1] + (b + 1 + enlarge) * Hy)
            ring = np.concatenate([np.stack([r[0] + q * sx, np.full(len(q), r[1])], 1),
                                   np.stack([np.full(len(q), r[2]), r[1] + q * sy], 1),
                                   np.stack([r[2] - q * sx, np.full(len(q), r[3])], 1),
                                   np.stack([np.full(len(q), r[0]), r[3] - q * sy], 1)])
            keep = ((ring[:, 0] > dom[0] + tol) & (ring[:, 0] < dom[2] - tol) &
                    (ring[:, 1] > dom[1] + tol) & (ring[:, 1] < dom[3] - tol))
            R = len(ring)
            start = 0
            if not keep.all():
                start = next((i + 1) % R for i in range(R) if not keep[i] and keep[(i + 1) % R])
            order = [(start + t) % R for t in range(R) if keep[(start + t) % R]]
            chain = ring[order]
            gids = np.arange(len(nodes), len(nodes) + len(chain))
            nodes.extend(chain.tolist())
            patches.append(dict(rect=r, chain=chain, gids=gids, cell=(a, b)))
    nodes = np.array(nodes)
    owner = np.concatenate([np.full(len(p["gids"]), s) for s, p in enumerate(patches)])
    gs, ss = [], []
    for s, p in enumerate(patches):
        r = p["rect"]
        inside = ((nodes[:, 0] > r[0] + tol) & (nodes[:, 0] < r[2] - tol) &
                  (nodes[:, 1] > r[1] + tol) & (nodes[:, 1] < r[3] - tol) & (owner != s))
        g = np.nonzero(inside)[0]
        gs.append(g)
        ss.append(np.full(len(g), s))
    gs, ss = np.concatenate(gs), np.concatenate(ss)
    order = np.lexsort((ss, gs))  # node order, then patch order
    items = list(zip(gs[order].tolist(), ss[order].tolist()))
    return dict(nodes=nodes, patches=patches, items=items, spacing=sx)


def actualiza_gb(row, cols, G, b, rowptr, col, val, B):
    """SistemaLineal::Actualiza_GB(nudo) on CSR arrays (val and B updated in place);
    cols ascending, as the keys of the node's std::map."""
    L = load()
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    G = np.ascontiguousarray(G, dtype=np.float64)
    assert rowptr.dtype == np.int32 and col.dtype == np.int32 and val.flags.c_contiguous and B.flags.c_contiguous
    return L.orc_actualiza_gb(row, len(cols), cols.ctypes.data_as(_ip), G.ctypes.data_as(_dp), b,
                              rowptr.ctypes.data_as(_ip), col.ctypes.data_as(_ip), val.ctypes.data_as(_dp),
                              B.ctypes.data_as(_dp))


def rectangulo(p, x, y):
    L = load()
    pp = (C.c_double * 4)(*p)
    o = (C.c_double * 5)()
    L.orc_rectangulo(pp, x, y, o)
    return list(o)


def circulo(p, x, y):
    L = load()
    pp = (C.c_double * 3)(*p)
    o = (C.c_double * 5)()
    L.orc_circulo(pp, x, y, o)
    return list(o)


def coefficients(b, x, y):
    L = load()
    o = (C.c_double * 12)()
    L.orc_coefficients(C.byref(b), x, y, o)
    return list(o)


class MlpParams:
    """FP64 MLP parameters in the packing of fk_mlp_get_params."""

    def __init__(self, flat, width, in_lo, in_scale):
        W = width
        self.flat = np.ascontiguousarray(flat, dtype=np.float64)
        sizes = [2 * W, W, W * W, W, W * W, W, W, 1]
        offs = np.cumsum([0] + sizes)
        self.parts = [self.flat[offs[i]:offs[i + 1]] for i in range(8)]
        self.s = Mlp(W, (C.c_double * 2)(*in_lo), (C.c_double * 2)(*in_scale),
                     *[p.ctypes.data_as(_dp) for p in self.parts])

    def eval(self, xy):
        L = load()
        out = np.zeros((len(xy), 3))
        o = (C.c_double * 3)()
        for i, (x, y) in enumerate(np.asarray(xy, dtype=np.float64)):
            L.orc_mlp_eval(C.byref(self.s), x, y, o)
            out[i] = list(o)
        return out

    def loss_grad(self, xy, target):
        L = load()
        xy = np.ascontiguousarray(xy, dtype=np.float64).ravel()
        t = np.ascontiguousarray(target, dtype=np.float64)
        g = np.zeros_like(self.flat)
        loss = L.orc_mlp_loss_grad(C.byref(self.s), len(t), xy.ctypes.data_as(_dp), t.ctypes.data_as(_dp),
                                   g.ctypes.data_as(_dp))
        return loss, g
