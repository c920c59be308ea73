"""ctypes binding of libspac_fk (include/spac_fk.h) with numpy arrays.

`Context` is a 1:1 wrapper of the C ABI; `FeynmanKacSolverGPU` mirrors the
public interface of the reference's FeynmanKacSolver
(Solvers/FeynmanKacSolver.hpp:43-98): the two Solve_OMP_Analytic overloads
and the public statistics members they fill.
"""
import ctypes as C

import numpy as np

from . import lib_path

FK_OK = 0
FK_ERR_ARG, FK_ERR_CUDA, FK_ERR_REGISTRY, FK_ERR_STEP_CAP = -1, -2, -3, -4
FK_ERR_NOT_FOUND, FK_ERR_NO_DEVICE, FK_ERR_CAPACITY = -5, -6, -7
FRANKE, MONEGROS, ANISO, DISK, ROBIN, MONEGROS_POISSON = 0, 1, 2, 3, 4, 5
# reflecting sides of FK_PROBLEM_ROBIN (prob[0] is their sum)
SIDE_X0, SIDE_Y0, SIDE_X1, SIDE_Y1 = 1, 2, 4, 8
RECT, CIRCLE = 0, 1
CV_NONE, CV_EXACT, CV_MLP = 0, 1, 2
FP64, FP32 = 0, 1
TRAIN_AUTO, TRAIN_GRID, TRAIN_STEPS = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint)
_fp = C.POINTER(C.c_float)


class BvpDesc(C.Structure):
    _fields_ = [("problem", C.c_int), ("cv", C.c_int), ("dom_shape", C.c_int), ("dom", C.c_double * 4),
                ("prob", C.c_double * 4), ("mlp_id", C.c_int)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("phi", "phiphi", "phi_VR", "phiphi_VR", "xi", "xixi", "xiphi", "APL",
                                          "RNGC", "B", "n_paths", "n_domain_exits", "n_capped", "xi_mean",
                                          "xi_sq_mean", "mean_steps")]


STAT_FIELDS = [f[0] for f in Stats._fields_]


class ArcDesc(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double), ("c2", C.c_double),
                ("interior", C.c_int), ("n", C.c_int), ("theta", _dp), ("gids", _ip), ("iPsi", _dp)]


class NodeItem(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("h", C.c_double), ("paths", C.c_uint),
                ("frontera", C.c_int), ("row", C.c_int), ("stencil", C.c_int)]


class DiskDesc(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double), ("theta0", C.c_double),
                ("n_circle", C.c_int), ("n_radial", C.c_int), ("n_periph", C.c_int), ("periph_theta", _dp),
                ("n_inner", C.c_int), ("inner_xy", _dp)]


class MeshInfo(C.Structure):
    _fields_ = [("n_rows", C.c_int), ("nnz", C.c_int), ("n_items", C.c_int), ("n_nodes", C.c_int),
                ("n_stencils", C.c_int), ("max_stencil", C.c_int), ("spacing", C.c_double)]


_LIB = None

# name -> (restype, argtypes)
_SIGS = {
    "fk_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_ulonglong]),
    "fk_destroy": (C.c_int, [C.c_void_p]),
    "fk_last_error": (C.c_char_p, [C.c_void_p]),
    "fk_set_stream": (C.c_int, [C.c_void_p, C.c_uint]),
    "fk_get_stream": (C.c_int, [C.c_void_p, _up]),
    "fk_set_max_steps": (C.c_int, [C.c_void_p, C.c_int]),
    "fk_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fk_set_wait_limits": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    "fk_cuda_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "fk_last_timing": (C.c_int, [C.c_void_p, _dp]),
    "fk_last_windows": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "fk_mesh_window": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, _ip, _ip, _ip]),
    "fk_register_bvp": (C.c_int, [C.c_void_p, C.POINTER(BvpDesc), _ip]),
    "fk_solve_points": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _up, _dp, _ip, _dp, C.c_int,
                                  C.POINTER(Stats)]),
    "fk_solve_points_multi": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _up, _dp, C.c_int, C.POINTER(Stats)]),
    "fk_autotune_points": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _up, _dp, C.c_int, C.c_double, _ip, _ip, _dp]),
    "fk_register_arc": (C.c_int, [C.c_void_p, C.POINTER(ArcDesc), _ip]),
    "fk_arc_ipsi": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "fk_solve_nodes_arc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(NodeItem), C.c_int, _dp, _dp,
                                     C.POINTER(Stats)]),
    "fk_mesh_circles": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                  C.c_double, _ip]),
    "fk_mesh_square_patches": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                         _ip]),
    "fk_mesh_get_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(MeshInfo)]),
    "fk_mesh_nodes": (C.c_int, [C.c_void_p, C.c_int, _dp, _ip]),
    "fk_mesh_items": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _ip, _ip]),
    "fk_mesh_stencil_nodes": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _ip]),
    "fk_mesh_csr": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _dp]),
    "fk_assemble": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_uint, _up, C.c_double, C.c_int, _dp, _dp, _dp,
                              _dp, C.POINTER(Stats)]),
    "fk_assembly_begin": (C.c_int, [C.c_void_p, C.c_int]),
    "fk_assembly_round": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip, _up, C.c_double, C.c_int, _dp]),
    "fk_assembly_end": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(Stats)]),
    "fk_solve_disks_ps": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(DiskDesc), _dp, _dp]),
    "fk_mesh_set_disk_solver": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fk_mlp_create": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_ulonglong, _ip]),
    "fk_mlp_num_params": (C.c_int, [C.c_void_p, C.c_int, _ip]),
    "fk_mlp_get_params": (C.c_int, [C.c_void_p, C.c_int, _fp]),
    "fk_mlp_set_params": (C.c_int, [C.c_void_p, C.c_int, _fp]),
    "fk_mlp_train": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip, C.c_int, C.c_int, C.c_double,
                               C.c_ulonglong, _fp]),
    "fk_mlp_eval": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip, _dp]),
    "fk_mlp_set_trainer": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fk_mlp_fit_output": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip, C.c_double]),
    "fk_mlp_build_table": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fk_mlp_get_table": (C.c_int, [C.c_void_p, C.c_int, _ip, _fp]),
    "fk_mlp_loss_grad": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _fp]),
    "fk_gmres_csr": (C.c_int, [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, _ip, _dp]),
    "fk_gmres_csr_pc": (C.c_int, [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int, _ip,
                                  _dp]),
    "fk_write_gb_coo": (C.c_int, [C.c_char_p, C.c_int, _ip, _ip, _dp, _dp]),
    "fk_write_gb_csr": (C.c_int, [C.c_char_p, C.c_int, _ip, _ip, _dp, _dp]),
    "fk_read_gb_coo": (C.c_int, [C.c_char_p, _ip, _ip, _ip, _ip, _dp]),
    "fk_write_positions": (C.c_int, [C.c_char_p, C.c_int, _ip, _dp, _dp]),
    "fk_solve_points_noalloc": (C.c_int, [C.POINTER(BvpDesc), C.c_ulonglong, C.c_uint, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
}


def load():
    """Load libspac_fk.so and bind every declared entry point."""
    global _LIB
    if _LIB is None:
        L = C.CDLL(lib_path())
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _LIB = L
    return _LIB


def exported_symbols():
    return sorted(_SIGS)


class FKError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libspac_fk error {code}: {msg}")
        self.code = code


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def _u(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(_up)


def stats_array(arr):
    """fk_stats array -> dict of per-item numpy columns (a copy of the buffer, no per-item Python work)."""
    n = len(arr)
    flat = np.frombuffer(arr, dtype=np.float64, count=n * len(STAT_FIELDS)).reshape(n, len(STAT_FIELDS)).copy()
    return {k: flat[:, i] for i, k in enumerate(STAT_FIELDS)}


def _stats_out(n):
    """An n x 16 buffer in the fk_stats layout and its pointer (no ctypes struct array)."""
    buf = np.zeros((n, len(STAT_FIELDS)))
    return buf, buf.ctypes.data_as(C.POINTER(Stats))


def _stats_cols(buf):
    return {k: buf[:, i] for i, k in enumerate(STAT_FIELDS)}


def _per_item(a, n, conv):
    """A per-item argument: a scalar filled to n entries, or an array of n."""
    if np.ndim(a) == 0:
        return conv(np.full(n, a))
    return conv(np.broadcast_to(a, (n,)))


class Context:
    """One GPU context (device, Philox seed, stream, registries)."""

    def __init__(self, device=0, seed=1234):
        self.L = load()
        self.h = C.c_void_p()
        rc = self.L.fk_create(C.byref(self.h), device, seed)
        if rc != FK_OK:
            raise FKError(rc, "fk_create failed (no usable CUDA device?)")

    def close(self):
        if self.h:
            self.L.fk_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc, allow=()):
        if rc != FK_OK and rc not in allow:
            raise FKError(rc, self.L.fk_last_error(self.h).decode())
        return rc

    # -- context
    def set_stream(self, s):
        self.check(self.L.fk_set_stream(self.h, s))

    def get_stream(self):
        v = C.c_uint()
        self.check(self.L.fk_get_stream(self.h, C.byref(v)))
        return v.value

    def set_max_steps(self, m):
        self.check(self.L.fk_set_max_steps(self.h, m))

    def set_wait_limits(self, slot_wait_s=0.0, barrier_s=0.0):
        """fk_set_wait_limits (seconds; 0 = the defaults)."""
        self.check(self.L.fk_set_wait_limits(self.h, slot_wait_s, barrier_s))

    def set_launch(self, block=0, chunk=0):
        self.check(self.L.fk_set_launch(self.h, block, chunk))

    def cuda_stream(self):
        v = C.c_void_p()
        self.check(self.L.fk_cuda_stream(self.h, C.byref(v)))
        return v.value

    def mesh_window(self, mesh, s, x, y):
        """(first chain node of the k-window, nearest node, walk modes) the path
        kernel picks for a point on the boundary of patch s (fk_mesh_window)."""
        w, nr, wk = C.c_int(), C.c_int(), C.c_int()
        self.check(self.L.fk_mesh_window(self.h, mesh, s, x, y, C.byref(w), C.byref(nr), C.byref(wk)))
        return w.value, nr.value, wk.value

    def last_windows(self):
        """Stencil windows whose moments the last patch-stencil solve formed into G rows."""
        out = C.c_longlong()
        self.check(self.L.fk_last_windows(self.h, C.byref(out)))
        return int(out.value)

    def last_timing(self):
        out = (C.c_double * 3)()
        self.check(self.L.fk_last_timing(self.h, out))
        return list(out)

    # -- registry
    def register_bvp(self, problem, cv=CV_NONE, dom=(0, 0, 1, 1), dom_shape=None, prob=(0, 0, 0, 0), mlp_id=-1):
        if dom_shape is None:
            dom_shape = CIRCLE if problem == DISK else RECT
        d = BvpDesc(problem, cv, dom_shape, (C.c_double * 4)(*dom), (C.c_double * 4)(*prob), mlp_id)
        i = C.c_int()
        self.check(self.L.fk_register_bvp(self.h, C.byref(d), C.byref(i)))
        if not hasattr(self, "_descs"):
            self._descs = {}
        self._descs[i.value] = dict(problem=problem, cv=cv, dom=tuple(dom), dom_shape=dom_shape, prob=tuple(prob),
                                    mlp_id=mlp_id)
        return i.value

    def bvp_with_rho(self, bvp, rho):
        """The registered BVP with the reflecting-zone width rho (FK_PROBLEM_ROBIN
        keeps it in prob[2]); other problems ignore rho."""
        d = getattr(self, "_descs", {}).get(bvp)
        if d is None or d["problem"] != ROBIN or d["prob"][2] == rho:
            return bvp
        key = ("rho", bvp, float(rho))
        if key not in self._descs:
            prob = (d["prob"][0], d["prob"][1], float(rho), d["prob"][3])
            self._descs[key] = self.register_bvp(d["problem"], d["cv"], d["dom"], d["dom_shape"], prob, d["mlp_id"])
        return self._descs[key]

    # -- point solves
    def solve_points(self, bvp, xy, paths, h, precision=FP64, sub_shape=None, sub_params=None, allow=()):
        xy, pxy = _d(np.reshape(xy, (-1, 2)))
        n = xy.shape[0]
        paths, pp = _per_item(paths, n, _u)
        h, ph = _per_item(h, n, _d)
        ss = ps = None
        if sub_shape is not None:
            ss, ps_ = _i(np.broadcast_to(sub_shape, (n,)))
            sp, psp = _d(np.reshape(sub_params, (n, 4)))
        buf, out = _stats_out(n)
        rc = self.L.fk_solve_points(self.h, bvp, n, pxy, pp, ph, ps_ if ss is not None else None,
                                    psp if ss is not None else None, precision, out)
        self.check(rc, allow)
        return _stats_cols(buf)

    def solve_points_multi(self, bvp_ids, xy, paths, h, precision=FP64, allow=()):
        xy, pxy = _d(np.reshape(xy, (-1, 2)))
        n = xy.shape[0]
        ids, pid = _per_item(bvp_ids, n, _i)
        paths, pp = _per_item(paths, n, _u)
        h, ph = _per_item(h, n, _d)
        buf, out = _stats_out(n)
        self.check(self.L.fk_solve_points_multi(self.h, n, pid, pxy, pp, ph, precision, out), allow)
        return _stats_cols(buf)

    def autotune_points(self, bvp_ids, xy, paths, h, precision=FP64, sample_fraction=0.1):
        xy, pxy = _d(np.reshape(xy, (-1, 2)))
        n = xy.shape[0]
        ids, pid = _i(np.broadcast_to(bvp_ids, (n,)))
        paths, pp = _u(np.broadcast_to(paths, (n,)))
        h, ph = _d(np.broadcast_to(h, (n,)))
        b, c, t = C.c_int(), C.c_int(), C.c_double()
        self.check(self.L.fk_autotune_points(self.h, n, pid, pxy, pp, ph, precision, sample_fraction, C.byref(b),
                                             C.byref(c), C.byref(t)))
        return b.value, c.value, t.value

    # -- arcs / node solves
    def register_arc(self, cx, cy, radius, c2, interior, theta, gids, iPsi=None):
        theta, pt = _d(theta)
        gids, pg = _i(gids)
        ip = None
        if iPsi is not None:
            iPsi, ip = _d(np.asfortranarray(iPsi).ravel(order="F"))
        d = ArcDesc(cx, cy, radius, c2, interior, len(theta), pt, pg, ip)
        i = C.c_int()
        self.check(self.L.fk_register_arc(self.h, C.byref(d), C.byref(i)))
        return i.value

    def arc_ipsi(self, arc_id, n):
        out = np.zeros(n * n)
        self.check(self.L.fk_arc_ipsi(self.h, arc_id, out.ctypes.data_as(_dp)))
        return out.reshape((n, n), order="F")

    def solve_nodes_arc(self, bvp, items, arc_sizes, precision=FP64):
        n = len(items)
        arr = (NodeItem * n)(*[NodeItem(*it) for it in items])
        gt = int(sum(arc_sizes[it[6]] for it in items))
        G = np.zeros(gt)
        B = np.zeros(n)
        st = (Stats * n)()
        self.check(self.L.fk_solve_nodes_arc(self.h, bvp, n, arr, precision, G.ctypes.data_as(_dp),
                                             B.ctypes.data_as(_dp), st))
        return G, B, stats_array(st)

    # -- meshes
    def mesh_circles(self, dom, n_side, superposicion, theta0, nodes_per_circle, c2_corner=1.5, c2_side=1.1):
        dom, pd = _d(dom)
        i = C.c_int()
        self.check(self.L.fk_mesh_circles(self.h, pd, n_side, superposicion, theta0, nodes_per_circle, c2_corner,
                                          c2_side, C.byref(i)))
        return i.value

    def mesh_set_disk_solver(self, mesh, n_radial):
        """fk_mesh_set_disk_solver: interior-circle rows by the pseudospectral disk solve (0 = off)."""
        self.check(self.L.fk_mesh_set_disk_solver(self.h, mesh, n_radial))

    def solve_disks_ps(self, bvp, disks):
        """fk_solve_disks_ps.  disks: dicts with cx, cy, radius, theta0, n_circle,
        n_radial, periph_theta, inner_xy.  Returns [(G (n_inner x n_periph), B)] per disk."""
        keep, descs = [], (DiskDesc * max(len(disks), 1))()
        n_g = n_b = 0
        for i, d in enumerate(disks):
            th = np.ascontiguousarray(d["periph_theta"], dtype=np.float64)
            xy = np.ascontiguousarray(d["inner_xy"], dtype=np.float64).reshape(-1, 2)
            keep += [th, xy]
            descs[i] = DiskDesc(d["cx"], d["cy"], d["radius"], d["theta0"], d["n_circle"], d["n_radial"], len(th),
                                th.ctypes.data_as(_dp), len(xy), xy.ctypes.data_as(_dp))
            n_g += len(th) * len(xy)
            n_b += len(xy)
        G = np.zeros(max(n_g, 1))
        B = np.zeros(max(n_b, 1))
        self.check(self.L.fk_solve_disks_ps(self.h, bvp, len(disks), descs, G.ctypes.data_as(_dp),
                                            B.ctypes.data_as(_dp)))
        out, og, ob = [], 0, 0
        for d, k in zip(disks, range(0, len(keep), 2)):
            npp, ni = len(keep[k]), len(keep[k + 1])
            out.append((G[og:og + ni * npp].reshape(ni, npp).copy(), B[ob:ob + ni].copy()))
            og += ni * npp
            ob += ni
        return out

    def mesh_square_patches(self, dom, n_sub, nodes_per_side, enlarge=0.25, eps_spacing=3.0, knn=20):
        dom, pd = _d(dom)
        i = C.c_int()
        self.check(self.L.fk_mesh_square_patches(self.h, pd, n_sub, nodes_per_side, enlarge, eps_spacing, knn,
                                                 C.byref(i)))
        return i.value

    def mesh_info(self, mesh):
        m = MeshInfo()
        self.check(self.L.fk_mesh_get_info(self.h, mesh, C.byref(m)))
        return {k: getattr(m, k) for k, _ in MeshInfo._fields_}

    def mesh_nodes(self, mesh):
        info = self.mesh_info(mesh)
        xy = np.zeros((info["n_nodes"], 2))
        fl = np.zeros(info["n_nodes"], dtype=np.int32)
        self.check(self.L.fk_mesh_nodes(self.h, mesh, xy.ctypes.data_as(_dp), fl.ctypes.data_as(_ip)))
        return xy, fl

    def mesh_items(self, mesh):
        info = self.mesh_info(mesh)
        n = info["n_items"]
        row = np.zeros(n, dtype=np.int32)
        xy = np.zeros((n, 2))
        st = np.zeros(n, dtype=np.int32)
        fr = np.zeros(n, dtype=np.int32)
        self.check(self.L.fk_mesh_items(self.h, mesh, row.ctypes.data_as(_ip), xy.ctypes.data_as(_dp),
                                        st.ctypes.data_as(_ip), fr.ctypes.data_as(_ip)))
        return row, xy, st, fr

    def mesh_stencil_nodes(self, mesh, s):
        n = C.c_int()
        self.check(self.L.fk_mesh_stencil_nodes(self.h, mesh, s, None, C.byref(n)))
        g = np.zeros(n.value, dtype=np.int32)
        self.check(self.L.fk_mesh_stencil_nodes(self.h, mesh, s, g.ctypes.data_as(_ip), C.byref(n)))
        return g

    def mesh_csr(self, mesh):
        info = self.mesh_info(mesh)
        rp = np.zeros(info["n_rows"] + 1, dtype=np.int32)
        col = np.zeros(info["nnz"], dtype=np.int32)
        v0 = np.zeros(info["nnz"])
        self.check(self.L.fk_mesh_csr(self.h, mesh, rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip),
                                      v0.ctypes.data_as(_dp)))
        return rp, col, v0

    def assemble(self, mesh, bvp, paths, h, precision=FP64, paths_per_item=None, items=True, item_G=True, csr=True,
                 allow=()):
        """fk_assemble into numpy arrays.  items: per-item B and statistics;
        item_G: per-item G rows too; csr: the CSR values and B."""
        info = self.mesh_info(mesh)
        val = np.zeros(info["nnz"]) if csr else None
        B = np.zeros(info["n_rows"]) if csr else None
        pp = None
        if paths_per_item is not None:
            ppi, pp = _u(paths_per_item)
        G = iB = st = None
        if items:
            if item_G:
                sizes = [len(self.mesh_stencil_nodes(mesh, s)) for s in range(info["n_stencils"])]
                _, _, stn, _ = self.mesh_items(mesh)
                G = np.zeros(int(sum(sizes[s] for s in stn)))
            iB = np.zeros(info["n_items"])
            st = (Stats * info["n_items"])()
        rc = self.L.fk_assemble(self.h, mesh, bvp, int(paths), pp, h, precision,
                                val.ctypes.data_as(_dp) if csr else None, B.ctypes.data_as(_dp) if csr else None,
                                G.ctypes.data_as(_dp) if G is not None else None,
                                iB.ctypes.data_as(_dp) if items else None, st if items else None)
        self.check(rc, allow)
        return dict(val=val, B=B, item_G=G, item_B=iB, item_stats=stats_array(st) if items else None)


    # -- adaptive assembly in rounds (device-resident sums)
    def assembly_begin(self, mesh):
        self.check(self.L.fk_assembly_begin(self.h, mesh))

    def assembly_round(self, mesh, bvp, paths_per_item, h, precision=FP64, bvp_of_item=None, want_var=True,
                       allow=()):
        """fk_assembly_round; returns each item's per-path variance of this round (or None)."""
        pp, ppp = _u(paths_per_item)
        pb = None
        if bvp_of_item is not None:
            bo, pb = _i(bvp_of_item)
        var = np.zeros(len(pp)) if want_var else None
        self.check(self.L.fk_assembly_round(self.h, mesh, bvp, pb, ppp, h, precision,
                                            var.ctypes.data_as(_dp) if want_var else None), allow)
        return var

    def assembly_end(self, mesh, csr=True, items=True, item_G=True, allow=(), out=None):
        """fk_assembly_end.  `out` may hold caller-owned output buffers (e.g.
        page-locked): "val", "B", "item_B" (float64 arrays of the right sizes)
        and "item_stats" (a ctypes Stats array of n_items)."""
        info = self.mesh_info(mesh)
        out = out or {}
        val = (out["val"] if "val" in out else np.zeros(info["nnz"])) if csr else None
        B = (out["B"] if "B" in out else np.zeros(info["n_rows"])) if csr else None
        G = iB = st = None
        if items:
            if item_G:
                sizes = [len(self.mesh_stencil_nodes(mesh, s)) for s in range(info["n_stencils"])]
                _, _, stn, _ = self.mesh_items(mesh)
                G = np.zeros(int(sum(sizes[s] for s in stn)))
            iB = out["item_B"] if "item_B" in out else np.zeros(info["n_items"])
            st = out["item_stats"] if "item_stats" in out else (Stats * info["n_items"])()
        self.check(self.L.fk_assembly_end(self.h, mesh, val.ctypes.data_as(_dp) if csr else None,
                                          B.ctypes.data_as(_dp) if csr else None,
                                          G.ctypes.data_as(_dp) if G is not None else None,
                                          iB.ctypes.data_as(_dp) if items else None, st if items else None), allow)
        # (columns over the statistics buffer, which the arrays keep alive)
        cols = _stats_cols(np.frombuffer(st, dtype=np.float64).reshape(-1, len(STAT_FIELDS))) if items else None
        return dict(val=val, B=B, item_G=G, item_B=iB, item_stats=cols)


class FeynmanKacSolverGPU:
    """Mirror of FeynmanKacSolver's public interface on the GPU path.

    Solve_OMP_Analytic(X0, N, h, rho, bvp) fills phi, phiphi, phi_VR,
    phiphi_VR, xi, xixi, xiphi, APL, RNGC (FeynmanKacSolver.cpp:335-342);
    rho is the width of the zone near a reflecting side where the reflecting
    step runs (FK_PROBLEM_ROBIN); absorbing problems ignore it.
    """

    def __init__(self, ctx, precision=FP64):
        self.ctx = ctx
        self.precision = precision
        self.N = 0
        for k in ("phi", "phiphi", "phi_VR", "phiphi_VR", "xi", "xixi", "xiphi", "APL", "RNGC"):
            setattr(self, k, 0.0)

    def Solve_OMP_Analytic(self, X0, N, h, rho, bvp):
        bvp = self.ctx.bvp_with_rho(bvp, rho)
        st = self.ctx.solve_points(bvp, np.asarray(X0, dtype=np.float64).reshape(1, 2), N, h, self.precision)
        self.N = N
        for k in ("phi", "phiphi", "phi_VR", "phiphi_VR", "xi", "xixi", "xiphi", "APL", "RNGC"):
            setattr(self, k, float(st[k][0]))
        return self


# ---- host-side consumers of the assembled system ------------------------------
PC_JACOBI, PC_ILU0 = 0, 1


def gmres(rowptr, col, val, b, x0=None, tol=1e-10, max_iter=2000, restart=50, precond=None):
    """fk_gmres_csr (precond None: Jacobi) or fk_gmres_csr_pc (PC_JACOBI,
    PC_ILU0): returns (x, iterations, relative residual, status)."""
    L = load()
    rp, prp = _i(rowptr)
    cl, pcl = _i(col)
    v, pv = _d(val)
    bb, pb = _d(b)
    x = np.array(np.zeros(len(bb)) if x0 is None else x0, dtype=np.float64)
    it, res = C.c_int(), C.c_double()
    if precond is None:
        rc = L.fk_gmres_csr(len(bb), prp, pcl, pv, pb, x.ctypes.data_as(_dp), tol, max_iter, restart, C.byref(it),
                            C.byref(res))
    else:
        rc = L.fk_gmres_csr_pc(len(bb), prp, pcl, pv, pb, x.ctypes.data_as(_dp), tol, max_iter, restart, precond,
                               C.byref(it), C.byref(res))
    return x, it.value, res.value, rc


def write_gb(dir_, rowptr, col, val, B, fmt="coo"):
    L = load()
    rp, prp = _i(rowptr)
    cl, pcl = _i(col)
    v, pv = _d(val)
    bb, pb = _d(B)
    f = L.fk_write_gb_coo if fmt == "coo" else L.fk_write_gb_csr
    return f(str(dir_).encode(), len(bb), prp, pcl, pv, pb)


def read_gb_coo(path):
    L = load()
    nr, nz = C.c_int(), C.c_int()
    rc = L.fk_read_gb_coo(str(path).encode(), C.byref(nr), C.byref(nz), None, None, None)
    if rc != FK_OK:
        raise FKError(rc, "fk_read_gb_coo: cannot read " + str(path))
    rp = np.zeros(nr.value + 1, dtype=np.int32)
    col = np.zeros(nz.value, dtype=np.int32)
    val = np.zeros(nz.value)
    rc = L.fk_read_gb_coo(str(path).encode(), C.byref(nr), C.byref(nz), rp.ctypes.data_as(_ip),
                          col.ctypes.data_as(_ip), val.ctypes.data_as(_dp))
    if rc != FK_OK:
        raise FKError(rc, "fk_read_gb_coo: malformed " + str(path))
    return rp, col, val


def write_positions(path, gids, xy, u):
    L = load()
    g, pg = _i(gids)
    p, pp = _d(np.reshape(xy, (-1, 2)))
    uu, pu = _d(u)
    return L.fk_write_positions(str(path).encode(), len(g), pg, pp, pu)
