"""Named synthetic workloads of the Feynman-Kac hot path and their runners.

  point_solves  32 x 32 grid nodes (i/33, j/33) of the Franke Poisson problem
                on [0,1]^2, 1e4 paths per node, h = 1e-3 (FP64 and FP32)
  assembly      the plain 8 x 8 FP32 G/B assembly (bench.py's step) at --paths
                per item (20000) and step --h (5e-4), three times
  uneven        16 independent disk BVPs, radius ~ U[0.25, 1], 2^14 nodes
                (1024 per disk, uniform in area), paths log-uniform in
                [1e3, 1e5], h in {1e-3, 5e-4}, one persistent launch with the
                autotuned block/chunk
  large         32 x 32 subdomains, 63 nodes per patch side, h = 2.5e-4,
                paths added per item until its standard error is below 1e-4,
                learned control variate with plain FK as the per-item fallback
  disk_rows     pseudospectral rows of the interior circles of a 32 x 32
                circle layout: 900 disks of the serial driver's size
                (44 grid angles, N_radio 43, 44 periphery and 44 interior
                nodes each, main_test_serial.cpp:48-70), Franke problem

  serial_driver the reference serial driver end to end (main_test_serial.cpp:
                38-89): 4 x 4 circles on [0, 1.25]^2 (44 nodes each,
                superposicion 1), Franke, FK rows (1000 paths, h = 1e-5,
                FP64) for perimeter circles, pseudospectral rows (N_radio 43)
                for interior circles, GMRES on the host, node error

  assembly_cv   the 8 x 8 assembly (eps = 1/spacing) with the learned control
                variate at --paths per item (734), step --h (5e-5): pilot,
                training, refit, table and three assemblies

  python -m spac_gb300.workloads point_solves|uneven|large|disk_rows|serial_driver|robin|assembly|assembly_cv
      [--scale s] [--paths n] [--h h]

All inputs are seeded synthetic data; nothing is read from disk.
"""
import argparse
import json
import time

import numpy as np

from . import fk


def franke(x, y):
    return (0.75 * np.exp(-0.25 * ((9 * x - 2) ** 2 + (9 * y - 2) ** 2)) +
            0.75 * np.exp(-((9 * x + 1) ** 2) / 49 - 0.1 * (9 * y + 1)) +
            0.5 * np.exp(-0.25 * ((9 * x - 7) ** 2 + (9 * y - 3) ** 2)) -
            0.2 * np.exp(-((9 * x - 4) ** 2) - (9 * y - 7) ** 2))


_PINNED = {}


def _pinned(n, what):
    """A page-locked float64 host array of n entries (torch's pinned
    allocator) for the output `what`, one per (output, size), kept for the
    process as a caller keeps its output buffers across calls."""
    import torch
    key = (what, max(int(n), 1))
    if key not in _PINNED:
        _PINNED[key] = torch.empty(key[1], dtype=torch.float64, pin_memory=True)
    return _PINNED[key].numpy()


def _sync_time(fn):
    t0 = time.perf_counter()
    r = fn()
    return r, time.perf_counter() - t0


def point_solves(ctx, paths=10000, h=1e-3, precisions=(fk.FP64, fk.FP32)):
    g = np.arange(1, 33) / 33.0
    xy = np.array([(x, y) for x in g for y in g])
    u = franke(xy[:, 0], xy[:, 1])
    b = ctx.register_bvp(fk.FRANKE)
    out = {"nodes": len(xy), "paths_per_node": paths, "h": h}
    for prec in precisions:
        ctx.solve_points(b, xy[:8], 64, h, prec)  # warm-up
        st, t = _sync_time(lambda: ctx.solve_points(b, xy, paths, h, prec))
        k_ms = ctx.last_timing()[0]
        err = st["phi"] - u
        se = np.sqrt(np.maximum(st["phiphi"] - st["phi"] ** 2, 0) / paths)
        name = "fp64" if prec == fk.FP64 else "fp32"
        out[name] = {"seconds": t, "kernel_ms": k_ms, "paths_per_s": len(xy) * paths / t,
                     "node_solves_per_s": len(xy) / t, "path_steps_per_s": len(xy) * paths * st["mean_steps"].mean() / t,
                     "mean_steps": float(st["mean_steps"].mean()), "rms_error": float(np.sqrt(np.mean(err ** 2))),
                     "mean_se": float(se.mean()), "max_abs_z": float(np.max(np.abs(err) / se)),
                     "bias_rms_est": float(np.sqrt(max(np.mean(err ** 2) - np.mean(se ** 2), 0.0)))}
    return out


def aniso_u(x, y):
    return franke(x, y) * (1 + x * y)


def robin(ctx, paths=4000, h=1e-4, n=24, mask=1 + 8, varphi=-0.5, rho=0.05):
    """Reflecting sides (FK_PROBLEM_ROBIN, Paso_Reflejante): point solves on an
    n x n grid of the unit square whose sides x = 0 and y = 1 reflect (Robin,
    varphi) and whose other sides absorb; FP32 stepping with the exact-gradient
    control variate (error against the exact u) and plain (throughput next to
    the all-absorbing problem on the same points)."""
    g = (np.arange(n) + 0.5) / n
    xy = np.stack(np.meshgrid(g, g, indexing="ij"), axis=-1).reshape(-1, 2)
    u = aniso_u(xy[:, 0], xy[:, 1])
    out = {"points": len(xy), "paths": paths, "h": h, "mask": mask, "varphi": varphi, "rho": rho}
    b_abs = ctx.register_bvp(fk.ANISO)
    b_rob = ctx.register_bvp(fk.ROBIN, prob=(mask, varphi, rho, 0))
    b_cv = ctx.register_bvp(fk.ROBIN, cv=fk.CV_EXACT, prob=(mask, varphi, rho, 0))
    for name, b in (("absorbing", b_abs), ("robin", b_rob), ("robin_exact_cv", b_cv)):
        ctx.solve_points(b, xy[:8], 64, h, fk.FP32)  # warm-up
        st, t = _sync_time(lambda: ctx.solve_points(b, xy, paths, h, fk.FP32))
        key = "phi_VR" if name == "robin_exact_cv" else "phi"
        var = np.maximum(st["phiphi_VR" if key == "phi_VR" else "phiphi"] - st[key] ** 2, 0)
        se = np.sqrt(var / paths)
        err = st[key] - u
        out[name] = {"seconds": t, "kernel_ms": ctx.last_timing()[0], "paths_per_s": len(xy) * paths / t,
                     "mean_steps": float(st["mean_steps"].mean()), "mean_se": float(se.mean())}
        if name != "absorbing":
            out[name].update(rms_error=float(np.sqrt(np.mean(err ** 2))), max_abs_error=float(np.abs(err).max()),
                             bias_rms_est=float(np.sqrt(max(np.mean(err ** 2) - np.mean(se ** 2), 0.0))))
    return out


def uneven_nodes(ctx, seed=2026, n_bvp=16, nodes=1 << 14, scale=1.0):
    """The uneven batch: n_bvp disks of random radius 0.25..1 (FK_PROBLEM_DISK,
    one registered BVP each, centres 2.5 apart on the x axis), nodes//n_bvp
    uniform nodes in each, paths log-uniform in 1e3..1e5 (times scale), h
    1e-3 or 5e-4 at random.  Returns a dict: bvp_ids (per node), xy, paths,
    h, u (the exact solution), disks [(radius, cx, cy)] and disk (per node)."""
    rng = np.random.default_rng(seed)
    R = rng.uniform(0.25, 1.0, n_bvp)
    centers = np.stack([2.5 * np.arange(n_bvp), np.zeros(n_bvp)], axis=1)
    per = nodes // n_bvp
    ids, xy, bvp_of = [], [], []
    for k in range(n_bvp):
        bid = ctx.register_bvp(fk.DISK, dom=(R[k], centers[k, 0], centers[k, 1]),
                               prob=(centers[k, 0], centers[k, 1], R[k], 0.0))
        ids.append(bid)
        r = R[k] * np.sqrt(rng.uniform(0, 1, per))
        th = rng.uniform(0, 2 * np.pi, per)
        xy.append(np.stack([centers[k, 0] + r * np.cos(th), centers[k, 1] + r * np.sin(th)], axis=1))
        bvp_of += [k] * per
    xy = np.ascontiguousarray(np.concatenate(xy))
    bvp_of = np.array(bvp_of)
    bvp_ids = np.array(ids, dtype=np.int32)[bvp_of]
    paths = np.exp(rng.uniform(np.log(1e3), np.log(1e5), len(xy)))
    paths = np.maximum(1, np.round(paths * scale)).astype(np.uint32)
    h = rng.choice([1e-3, 5e-4], len(xy))
    xi = (xy[:, 0] - centers[bvp_of, 0]) / (2 * R[bvp_of]) + 0.5
    eta = (xy[:, 1] - centers[bvp_of, 1]) / (2 * R[bvp_of]) + 0.5
    return {"bvp_ids": bvp_ids, "xy": xy, "paths": paths, "h": h, "u": franke(xi, eta),
            "disks": [(float(R[k]), float(centers[k, 0]), float(centers[k, 1])) for k in range(n_bvp)],
            "disk": bvp_of, "rng": rng}


def uneven(ctx, seed=2026, n_bvp=16, nodes=1 << 14, scale=1.0, autotune=True, fp64_fraction=0.05):
    U = uneven_nodes(ctx, seed, n_bvp, nodes, scale)
    bvp_ids, xy, paths, h, u, rng = U["bvp_ids"], U["xy"], U["paths"], U["h"], U["u"], U["rng"]
    bvp_of = U["disk"]
    R = [d[0] for d in U["disks"]]
    out = {"bvps": n_bvp, "nodes": len(xy), "total_paths": int(paths.sum()), "radius": R}
    if autotune:
        bb, bc, tms = ctx.autotune_points(bvp_ids, xy, paths, h, fk.FP32, sample_fraction=0.05)
        out["autotune"] = {"block": bb, "chunk": bc, "sample_kernel_ms": tms}
    ctx.solve_points_multi(bvp_ids[:64], xy[:64], 100, h[:64], fk.FP32)  # warm-up
    st, t = _sync_time(lambda: ctx.solve_points_multi(bvp_ids, xy, paths, h, fk.FP32))
    steps = float((st["mean_steps"] * paths).sum())
    out["fp32"] = {"seconds": t, "kernel_ms": ctx.last_timing()[0], "paths_per_s": paths.sum() / t,
                   "node_solves_per_s": len(xy) / t, "path_steps_per_s": steps / t, "mean_steps": steps / paths.sum()}
    err32 = st["phi"] - u
    se32 = np.sqrt(np.maximum(st["phiphi"] - st["phi"] ** 2, 0) / paths)
    # FP64 on a subsample of the same nodes (paths scaled) for the precision comparison
    sub = rng.choice(len(xy), size=max(64, int(fp64_fraction * len(xy))), replace=False)
    p64 = np.maximum(1000, paths[sub] // 4).astype(np.uint32)
    stream = ctx.get_stream()  # both precisions on the same Philox stream: paired paths
    s64, t64 = _sync_time(lambda: ctx.solve_points_multi(bvp_ids[sub], xy[sub], p64, h[sub], fk.FP64))
    ctx.set_stream(stream)
    s32 = ctx.solve_points_multi(bvp_ids[sub], xy[sub], p64, h[sub], fk.FP32)
    out["fp64_vs_fp32"] = {"nodes": len(sub), "paths": int(p64.sum()), "fp64_seconds": t64,
                           "fp64_paths_per_s": p64.sum() / t64,
                           "rms_error_fp64": float(np.sqrt(np.mean((s64["phi"] - u[sub]) ** 2))),
                           "rms_error_fp32": float(np.sqrt(np.mean((s32["phi"] - u[sub]) ** 2))),
                           "rms_fp32_minus_fp64": float(np.sqrt(np.mean((s32["phi"] - s64["phi"]) ** 2)))}
    per_bvp = []
    for k in range(n_bvp):
        sel = bvp_of == k
        _, tk = _sync_time(lambda: ctx.solve_points_multi(bvp_ids[sel], xy[sel], paths[sel], h[sel], fk.FP32))
        per_bvp.append({"radius": float(R[k]), "paths": int(paths[sel].sum()),
                        "paths_per_s_alone": float(paths[sel].sum() / tk),
                        "rms_error_fp32": float(np.sqrt(np.mean(err32[sel] ** 2))),
                        "mean_se_fp32": float(se32[sel].mean())})
    out["per_bvp"] = per_bvp
    out["sum_of_separate_seconds"] = float(sum(p["paths"] / p["paths_per_s_alone"] for p in per_bvp))
    return out


def collocation_pilot(ctx, bvp, grid=64, paths=500, h=1e-3, precision=fk.FP32):
    """Whole-domain plain point solves on a grid x grid lattice of the unit
    square: estimates of u that use the boundary data only (the training
    targets of the learned control variate)."""
    g = (np.arange(grid) + 0.5) / grid
    xy = np.ascontiguousarray(np.stack(np.meshgrid(g, g, indexing="ij"), axis=-1).reshape(-1, 2))
    st = ctx.solve_points(bvp, xy, paths, h, precision)
    return xy, np.ascontiguousarray(st["phi"])


def learned_cv(ctx, problem, pxy, target, steps=50, lr=1e-2, table=256, seed=99):
    """A one-region network on [0,1]^2 trained on (pxy, target): Adam steps,
    the output-layer refit and the gradient table; returns the BVP id that
    uses it."""
    rects = np.array([[0.0, 0.0, 1.0, 1.0]])
    mid = fk.C.c_int()
    ctx.check(ctx.L.fk_mlp_create(ctx.h, 1, rects.ctypes.data_as(fk._dp), seed, fk.C.byref(mid)))
    mid = mid.value
    if steps > 0:
        ctx.check(ctx.L.fk_mlp_train(ctx.h, mid, len(target), pxy.ctypes.data_as(fk._dp),
                                     target.ctypes.data_as(fk._dp), None, steps, 4096, lr, 5, None))
    ctx.check(ctx.L.fk_mlp_fit_output(ctx.h, mid, len(target), pxy.ctypes.data_as(fk._dp),
                                      target.ctypes.data_as(fk._dp), None, 1e-6))
    ctx.check(ctx.L.fk_mlp_build_table(ctx.h, mid, table))
    return ctx.register_bvp(problem, cv=fk.CV_MLP, mlp_id=mid)


def assembly_cv(ctx, paths=734, h=5e-5, eps_spacing=1.0, pilot_grid=24, pilot_paths=300, pilot_h=1e-3, steps=10,
                lr=1e-2, table=128, repeats=3):
    """The 8 x 8 assembly with the learned control variate (the metric's CV
    arm at a fixed path count): pilot point solves, training, output refit,
    gradient table, then `repeats` assemblies; path and finalize kernel times."""
    mesh = ctx.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, eps_spacing, 20)
    b_plain = ctx.register_bvp(fk.ANISO)
    pxy, tgt = collocation_pilot(ctx, b_plain, pilot_grid, pilot_paths, pilot_h)
    b_cv = learned_cv(ctx, fk.ANISO, pxy, tgt, steps=steps, lr=lr, table=table)
    out = []
    for _ in range(repeats):
        r, t = _sync_time(lambda: ctx.assemble(mesh, b_cv, paths, h, fk.FP32, items=False))
        out.append({"seconds": t, "kernels_ms": ctx.last_timing()[:2]})
    return {"paths_per_item": paths, "h": h, "runs": out}


def assembly(ctx, paths=20000, h=5e-4, eps_spacing=3.0, repeats=3):
    """The plain 8 x 8 FP32 assembly (ANISO, 20-nearest Gaussian stencil) at
    `paths` per item and step h, `repeats` times: path and statistics kernel
    times and the mean steps per path (the item statistics of the last run)."""
    mesh = ctx.mesh_square_patches((0, 0, 1, 1), 8, 31, 0.25, eps_spacing, 20)
    b = ctx.register_bvp(fk.ANISO)
    out = []
    for i in range(repeats):
        r, t = _sync_time(lambda: ctx.assemble(mesh, b, paths, h, fk.FP32, items=i == repeats - 1, item_G=False))
        out.append({"seconds": t, "kernels_ms": ctx.last_timing()[:2]})
    st = r["item_stats"]
    return {"paths_per_item": paths, "h": h, "mean_steps": float(np.mean(st["mean_steps"])), "runs": out}


def large(ctx, n_sub=32, nodes_per_side=63, h=2.5e-4, se_target=1e-4, pilot_paths=256, max_rounds=6,
          max_paths=4_000_000, eps_spacing=3.0):
    """Adaptive assembly of the full CSR G/B: per item, paths until the
    standard error of its estimate is below se_target, learned control
    variate where it lowers the variance and plain FK as the fallback, with
    the per-item path sums (G rows, B, statistics) kept on the device across
    rounds (fk_assembly_begin/round/end).

    The network learns u from whole-domain point solves at 64 x 64
    collocation points (boundary data only).  The first two rounds run
    pilot_paths per item with each method; each later round runs the paths
    that the chosen method's variance asks for."""
    mesh, t_mesh = _sync_time(lambda: ctx.mesh_square_patches((0, 0, 1, 1), n_sub, nodes_per_side, 0.25,
                                                               eps_spacing, 20))
    info = ctx.mesh_info(mesh)
    n = info["n_items"]
    row, ixy, stn, fr = ctx.mesh_items(mesh)
    b_plain = ctx.register_bvp(fk.FRANKE)
    # the caller's output buffers (page-locked, as a caller keeps them):
    # the CSR values (1.4 GB at 32 x 32), B, per-item B and statistics
    outs = {"val": _pinned(info["nnz"], "val"), "B": _pinned(info["n_rows"], "B"), "item_B": _pinned(n, "item_B")}
    outs["item_stats"] = (fk.Stats * n).from_address(_pinned(n * len(fk.STAT_FIELDS), "item_stats").ctypes.data)
    # the mesh's device side (stencil inverses, window tables) and the rounds'
    # buffers are set up once per mesh: counted with the mesh, not the assembly
    _, t_dev = _sync_time(lambda: ctx.assembly_begin(mesh))
    t_mesh += t_dev
    t0 = time.perf_counter()
    pxy, tgt = collocation_pilot(ctx, b_plain)
    t_pilot = time.perf_counter() - t0
    b_cv = learned_cv(ctx, fk.FRANKE, pxy, tgt)
    t_net = time.perf_counter() - t0 - t_pilot
    ctx.assembly_begin(mesh)
    p0 = np.full(n, pilot_paths, dtype=np.uint32)
    v_cv = np.maximum(ctx.assembly_round(mesh, b_cv, p0, h, fk.FP32), 1e-30)
    v_pl = np.maximum(ctx.assembly_round(mesh, b_plain, p0, h, fk.FP32), 1e-30)
    use_cv = v_cv < v_pl  # plain FK is the fallback where the control variate does not help
    n_cv = np.full(n, pilot_paths, dtype=np.int64)
    n_pl = np.full(n, pilot_paths, dtype=np.int64)
    sv_cv, sv_pl = v_cv * pilot_paths, v_pl * pilot_paths  # path-weighted variance sums per method
    total_paths, rounds, kern_ms = int(2 * pilot_paths * n), 2, []
    bvp_of = np.where(use_cv, b_cv, b_plain).astype(np.int32)

    def se2():
        N = n_cv + n_pl
        return (n_cv * (sv_cv / n_cv) + n_pl * (sv_pl / n_pl)) / N ** 2

    while rounds < max_rounds + 2:
        v = np.where(use_cv, sv_cv / n_cv, sv_pl / n_pl)
        N = n_cv + n_pl
        # extra paths x of the chosen method: (S + x v) / (N + x)^2 <= se^2
        S = n_cv * (sv_cv / n_cv) + n_pl * (sv_pl / n_pl)
        a2 = se_target ** 2
        disc = np.maximum((2 * N * a2 - v) ** 2 - 4 * a2 * (a2 * N * N - S), 0.0)
        x = np.where(se2() > a2, np.ceil(((v - 2 * N * a2) + np.sqrt(disc)) / (2 * a2)), 0)
        need = np.clip(x, 0, max_paths).astype(np.uint32)
        if need.max() == 0:
            break
        vr = np.maximum(ctx.assembly_round(mesh, b_plain, need, h, fk.FP32, bvp_of_item=bvp_of), 1e-30)
        kern_ms.append(ctx.last_timing()[0])
        m = need > 0
        cvm, plm = m & use_cv, m & ~use_cv
        sv_cv[cvm] += vr[cvm] * need[cvm]
        n_cv[cvm] += need[cvm]
        sv_pl[plm] += vr[plm] * need[plm]
        n_pl[plm] += need[plm]
        total_paths += int(need.sum())
        rounds += 1
    r = ctx.assembly_end(mesh, items=True, item_G=False, out=outs)
    t_total = time.perf_counter() - t0
    end_ms = ctx.last_timing()[1]
    # the end pass per G entry: the running row sum (8 B) and its CSR position
    # (4 B) read, the CSR value read and written (16 B); per item its 12
    # statistics read and its 16 written, B read and written
    g_entries = int(sum(len(ctx.mesh_stencil_nodes(mesh, s)) * c for s, c in
                        enumerate(np.bincount(stn, minlength=info["n_stencils"]))))
    end_bytes = g_entries * (8 + 4 + 16) + n * (12 * 8 + 16 * 8 + 16)
    # row residual of the assembled system with the exact solution
    rp, col, v0 = ctx.mesh_csr(mesh)
    nxy, _ = ctx.mesh_nodes(mesh)
    u_nodes = franke(nxy[:, 0], nxy[:, 1])
    diag = v0[rp[:-1] + np.array([np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(len(rp) - 1)])]
    resid = (np.add.reduceat(r["val"] * u_nodes[col], rp[:-1]) - r["B"]) / diag
    se = np.sqrt(se2())
    u = franke(ixy[:, 0], ixy[:, 1])
    phi = r["item_stats"]["phi_VR"]
    return {"items": n, "rows": info["n_rows"], "nnz": info["nnz"], "g_entries": g_entries,
            "mesh_seconds": t_mesh, "pilot_seconds": t_pilot, "network_seconds": t_net,
            "assembly_seconds": t_total, "rounds": rounds, "total_paths": total_paths,
            "paths_per_s": total_paths / t_total, "node_solves_per_s": n / t_total,
            "round_kernel_ms": kern_ms, "cv_items": int(use_cv.sum()),
            "variance_reduction_median": float(np.median(v_pl / v_cv)),
            "se_max": float(se.max()), "se_median": float(np.median(se)),
            "items_below_target": float(np.mean(se <= se_target * 1.001)),
            "rms_row_residual": float(np.sqrt(np.mean(resid ** 2))),
            "rms_node_error_exact_exit": float(np.sqrt(np.mean((phi - u) ** 2))),
            "paths_per_item_median": float(np.median(n_cv + n_pl)),
            "end_pass": {"ms": end_ms, "algorithmic_bytes": end_bytes,
                         "GB_per_s": end_bytes / (end_ms * 1e-3) / 1e9 if end_ms > 0 else None,
                         "what": "rows from the device-resident sums into the CSR values and B"}}


def disk_rows(ctx, n_disks=900, n_circle=44, n_radial=43, n_inner=44, seed=7, repeats=5):
    rng = np.random.default_rng(seed)
    side = int(np.ceil(np.sqrt(n_disks)))
    H = 1.0 / (side + 1)
    R = H / np.sqrt(2.0)
    disks = []
    for d in range(n_disks):
        cx, cy = (d // side + 1) * H, (d % side + 1) * H
        rr = 0.95 * R * np.sqrt(rng.random(n_inner))
        aa = 2 * np.pi * rng.random(n_inner)
        disks.append(dict(cx=cx, cy=cy, radius=R, theta0=0.1428, n_circle=n_circle, n_radial=n_radial,
                          periph_theta=0.1428 + 2 * np.pi * np.arange(n_circle) / n_circle,
                          inner_xy=np.stack([cx + rr * np.cos(aa), cy + rr * np.sin(aa)], 1)))
    b = ctx.register_bvp(fk.FRANKE)
    ctx.solve_disks_ps(b, disks)  # warm-up
    walls, solve_ms, interp_ms = [], [], []
    for _ in range(repeats):
        t = time.perf_counter()
        out = ctx.solve_disks_ps(b, disks)
        walls.append(time.perf_counter() - t)
        tm = ctx.last_timing()
        solve_ms.append(tm[0])
        interp_ms.append(tm[1])
    G0, B0 = out[0]
    return {"disks": n_disks, "n_circle": n_circle, "n_radial": n_radial, "n_inner": n_inner,
            "rows": n_disks * n_inner, "wall_s_median": float(np.median(walls)),
            "solve_kernels_ms_median": float(np.median(solve_ms)),
            "interp_kernel_ms_median": float(np.median(interp_ms)),
            "disks_per_s": n_disks / float(np.median(walls)),
            "row_sum_err": float(np.abs(-G0.sum(1) - 1.0).max())}


def serial_driver(ctx, paths=1000, h=1e-5, n_radial=43, precision=fk.FP64, repeats=3):
    dom = (0.0, 0.0, 1.25, 1.25)
    mesh, t_mesh = _sync_time(lambda: ctx.mesh_circles(dom, 4, 1.0, 0.1428, 44))
    ctx.mesh_set_disk_solver(mesh, n_radial)
    b = ctx.register_bvp(fk.FRANKE, dom=dom)
    rp, col, _ = ctx.mesh_csr(mesh)
    xy, _ = ctx.mesh_nodes(mesh)
    u = franke(xy[:, 0], xy[:, 1])
    ctx.assemble(mesh, b, paths, h, precision)  # warm-up
    t_asm, t_solve = [], []
    for _ in range(repeats):
        r, t = _sync_time(lambda: ctx.assemble(mesh, b, paths, h, precision, items=False, item_G=False))
        t_asm.append(t)
        (x, it, res, rc), t = _sync_time(lambda: fk.gmres(rp, col, r["val"], r["B"], tol=1e-12, max_iter=4000,
                                                            restart=80))
        t_solve.append(t)
    info = ctx.mesh_info(mesh)
    err = x - u
    return {"rows": info["n_rows"], "nnz": info["nnz"], "fk_items": info["n_items"], "paths": paths, "h": h,
            "n_radial": n_radial, "mesh_s": t_mesh, "assembly_s_median": float(np.median(t_asm)),
            "gmres_s_median": float(np.median(t_solve)), "gmres_iters": it, "gmres_rel_resid": res,
            "rms_node_error": float(np.sqrt(np.mean(err ** 2))), "max_node_error": float(np.abs(err).max())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["point_solves", "uneven", "large", "disk_rows", "serial_driver", "robin",
                                         "assembly_cv", "assembly"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--paths", type=int, default=0, help="assembly, assembly_cv: paths per item")
    ap.add_argument("--h", type=float, default=0.0, help="assembly, assembly_cv: step size")
    ap.add_argument("--seed", type=int, default=2026)
    a = ap.parse_args()
    ctx = fk.Context(0, seed=a.seed)
    if a.workload == "point_solves":
        r = point_solves(ctx, paths=max(64, int(10000 * a.scale)))
    elif a.workload == "uneven":
        r = uneven(ctx, scale=a.scale)
    elif a.workload == "disk_rows":
        r = disk_rows(ctx, n_disks=max(1, int(900 * a.scale)))
    elif a.workload == "serial_driver":
        r = serial_driver(ctx, paths=max(16, int(1000 * a.scale)))
    elif a.workload == "assembly_cv":
        r = assembly_cv(ctx, paths=a.paths or max(32, int(734 * a.scale)), h=a.h or 5e-5)
    elif a.workload == "assembly":
        r = assembly(ctx, paths=a.paths or max(32, int(20000 * a.scale)), h=a.h or 5e-4)
    elif a.workload == "robin":
        r = robin(ctx, paths=max(64, int(4000 * a.scale)))
    else:
        r = large(ctx, n_sub=max(2, int(round(32 * a.scale))), nodes_per_side=63 if a.scale >= 1 else 31)
    print(json.dumps({"workload": a.workload, **r}))


if __name__ == "__main__":
    main()
