"""Benchmark of the GB300 Feynman-Kac G/B assembly.

Workload (one step): the PDDSparse G/B assembly on [0,1]^2 with 8x8 square
subdomains, patches = subdomains enlarged by 0.25 of their width, 31 nodes
per patch side, Gaussian RBF exit stencil on the 20 nearest patch-boundary
nodes (eps = 3/spacing), anisotropic advection-reaction problem (sigma
sigma^T = 2(1 + 0.5 sin 2pi x sin 2pi y) I, b = (y-1/2, 1/2-x),
c = -(1+x^2+y^2), u = Franke (1+xy)), 2e4 paths per (node, patch) item,
h = 5e-4, FP32 stepping with FP64 node sums; output: CSR G and B.

  value  paths/s of the whole job with the assembly API writing device
         buffers (CUDA events on the library's stream, L2 flushed between steps)
  e2e    paths/s through fk_assemble into host buffers (device->host copy of G
         and B inside the timed region)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

METRIC = "time to 1e-3 RMS node error, learned-CV vs plain FK, 1 GB300; paths/s"
CFG = dict(workload="pddsparse-gb-assembly-8x8", n_sub=8, nodes_per_side=31, enlarge=0.25, eps_spacing=3.0,
           knn=20, problem="aniso", paths_per_item=20000, h=5e-4, precision="fp32", domain=[0, 0, 1, 1])

# Algorithmic operation counts of one path step of the FP32 anisotropic path
# kernel, counted from the source (FMA = 2 flops): Franke value/gradient/
# Laplacian 86, anisotropic coefficients and source 24, Box-Muller 8, state
# update 14, two rectangle distances 30, sigma at the new point and the
# Gobet test 12.  Transcendentals (4 exp, 2 sinpi, 2 sqrt per step plus half a
# log/sqrt/sincospi) are counted separately and not included.
FLOPS_PER_STEP = 174


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- CPU side ----
def _cpu_worker(args):
    """Oracle node solves for a slice of items (one process per host core)."""
    import oracle_py as orc
    items, nodes_xy, seed, N, h, k, eps = args
    s = orc.Session(orc.RNG_PHILOX, seed=seed, stream=1)
    b = orc.bvp(orc.__dict__.get("PROBLEM_ANISO", 2))
    t0 = time.perf_counter()
    npaths = 0
    for (i, x, y, rect, gidx) in items:
        s.node_solve_knn(b, x, y, rect, nodes_xy[gidx], k, eps, N, h, item=i)
        npaths += N
    return npaths, time.perf_counter() - t0


def cpu_baseline(host_mesh, cores, budget_s=12.0):
    """Times the CPU oracle port on a bounded sample of the same workload."""
    import oracle_py as orc
    orc.build(ref=False)
    ctx, mesh = host_mesh
    info = ctx.mesh_info(mesh)
    row, ixy, st, fr = ctx.mesh_items(mesh)
    nxy, _ = ctx.mesh_nodes(mesh)
    n_sub, e = CFG["n_sub"], CFG["enlarge"]
    H = 1.0 / n_sub
    eps = CFG["eps_spacing"] / info["spacing"]
    gid = {s: ctx.mesh_stencil_nodes(mesh, s) for s in range(info["n_stencils"])}

    def item(i):
        a, b = divmod(int(st[i]), n_sub)
        return (i, ixy[i, 0], ixy[i, 1], ((a - e) * H, (b - e) * H, (a + 1 + e) * H, (b + 1 + e) * H), gid[int(st[i])])

    # calibrate on one item, then size the sample to the time budget
    rng = np.random.default_rng(5)
    N = 2000
    n_cal, t_cal = _cpu_worker(([item(int(rng.integers(info["n_items"])))], nxy, 9, N, CFG["h"], CFG["knn"], eps))
    rate1 = n_cal / max(t_cal, 1e-6)
    per_core = max(1, int(budget_s * rate1 / N / 1.5))
    picks = rng.choice(info["n_items"], size=min(info["n_items"], per_core * cores), replace=False)
    slices = [[item(int(i)) for i in picks[c::cores]] for c in range(cores)]
    args = [(sl, nxy, 9, N, CFG["h"], CFG["knn"], eps) for sl in slices if sl]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(len(args)) as pool:
        res = pool.map(_cpu_worker, args)
    wall = time.perf_counter() - t0
    npaths = sum(r[0] for r in res)
    return {"value": npaths / wall, "unit": "paths/s", "cores": len(args), "kind": "port",
            "sample": f"{len(picks)} of {info['n_items']} items x {N} paths (oracle FP64, one process per core, "
                      f"{wall:.1f} s wall)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from spac_gb300 import fk
    cores = os.cpu_count() or 1
    hctx = fk.Context(device=-1)
    mesh = hctx.mesh_square_patches(CFG["domain"], CFG["n_sub"], CFG["nodes_per_side"], CFG["enlarge"],
                                    CFG["eps_spacing"], CFG["knn"])
    vals = []
    base = None
    for k in range(args.steps):
        base = cpu_baseline((hctx, mesh), cores, budget_s=8.0)
        vals.append(base["value"])
    v = float(np.mean(vals))
    info = hctx.mesh_info(mesh)
    total_paths = info["n_items"] * CFG["paths_per_item"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "paths/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * total_paths / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(CFG, precision="fp64", note="CPU oracle port of the reference FK node solve "
                           "(the reference itself has no square-patch/Gaussian stencil; its sources need Eigen "
                           "and Boost, absent on the GPU host)"),
            "cpu_baseline": dict(base, value=v),
            "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------- replicas ------
# The assembly shards by item with no exchange on the data path: under
# torchrun every rank assembles its own replica of the workload (weak
# scaling), the ranks meet only at barriers, and the job's time is the
# slowest rank's.
def max_over_ranks(x, dist):
    """Max of a float over the ranks (a CUDA tensor under NCCL, CPU under gloo)."""
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, paths_per_rank, ms_per_step):
    """Whole-job paths/s: the paths all ranks processed over the slowest rank's time."""
    return world * paths_per_rank / (ms_per_step / 1000.0)


# --------------------------------------------------------------- GPU side ----
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--paths", type=int, default=CFG["paths_per_item"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-metric", action="store_true", help="skip the time-to-1e-3 comparison")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    CFG["paths_per_item"] = args.paths

    # CPU baseline first (spawned pool, before any GPU call), rank 0 at N=1 only
    from spac_gb300 import fk
    base = None
    if rank == 0 and world == 1 and not args.no_cpu:
        hctx = fk.Context(device=-1)
        hmesh = hctx.mesh_square_patches(CFG["domain"], CFG["n_sub"], CFG["nodes_per_side"], CFG["enlarge"],
                                         CFG["eps_spacing"], CFG["knn"])
        base = cpu_baseline((hctx, hmesh), os.cpu_count() or 1)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ctx = fk.Context(device=local, seed=1000003 + 7919 * rank)
    mesh = ctx.mesh_square_patches(CFG["domain"], CFG["n_sub"], CFG["nodes_per_side"], CFG["enlarge"],
                                   CFG["eps_spacing"], CFG["knn"])
    info = ctx.mesh_info(mesh)
    bvp = ctx.register_bvp(fk.ANISO)
    prec = fk.FP32
    paths = CFG["paths_per_item"]
    total_paths = info["n_items"] * paths
    val = torch.empty(info["nnz"], dtype=torch.float64, device="cuda")
    Bd = torch.empty(info["n_rows"], dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 512 MB > L2
    ext = torch.cuda.ExternalStream(ctx.cuda_stream())
    dptr = lambda t: fk.C.cast(t.data_ptr(), fk._dp)

    def step_device():
        rc = ctx.L.fk_assemble(ctx.h, mesh, bvp, paths, None, CFG["h"], prec, dptr(val), dptr(Bd), None, None, None)
        ctx.check(rc)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    times, kern = [], []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        step_device()
        e1.record(ext)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        kern.append(ctx.last_timing())
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_step = float(np.sum(times)) / args.steps  # ms
    if dist:
        t_step = max_over_ranks(t_step, dist)
        dist.barrier()
    value = job_value(world, total_paths, t_step)

    # end to end: pinned host output buffers (the item table goes host->device
    # and val, B and the kernels' check flags device->host inside the timed region)
    val_h = _pinned(info["nnz"])
    B_h = _pinned(info["n_rows"])
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rc = ctx.L.fk_assemble(ctx.h, mesh, bvp, paths, None, CFG["h"], prec, val_h.ctypes.data_as(fk._dp),
                               B_h.ctypes.data_as(fk._dp), None, None, None)
        ctx.check(rc)
        e2e_t.append(time.perf_counter() - t0)
    e2e_step = float(np.mean(e2e_t))
    if dist:
        e2e_step = max_over_ranks(e2e_step, dist)
    # per call: one 96-byte item record and one 12-byte chunk record per item
    # (an item of <= 32768 paths is one chunk); back: CSR values, B, 4 check words
    item_bytes = info["n_items"] * (96 + 12)
    d2h = 8 * (info["nnz"] + info["n_rows"]) + 16

    # roofline of the dominant kernel (the path kernel): algorithmic flops / its event time
    k_ms = float(np.mean([k[0] for k in kern]))
    f_ms = float(np.mean([k[1] for k in kern]))
    steps_per_assembly = _mean_steps(ctx, mesh, bvp, prec, paths)
    flops = total_paths * steps_per_assembly * FLOPS_PER_STEP
    peaks, src = _peaks()
    smax = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * smax * 1e6 / 1e12  # TFLOP/s, nominal at the maximum SM clock
    achieved = flops / (k_ms / 1000.0) / 1e12
    traffic = _read_traffic()
    ttt = None
    if rank == 0 and not args.no_metric:
        ttt = time_to_target_all(ctx, mesh)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(CFG, items=info["n_items"], rows=info["n_rows"], nnz=info["nnz"],
                               paths_per_step=total_paths, l2="flushed between steps (512 MB write)"),
                "e2e": {"value": world * total_paths / e2e_step, "unit": "paths/s", "h2d_bytes_per_step": item_bytes,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": 2 * args.steps,
                "kernels_ms": {"paths": k_ms, "finalize_scatter": f_ms},
                "mean_steps_per_path": steps_per_assembly,
                "roofline_scatter": _scatter_roofline(info, f_ms, peaks, src),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak, "traffic": traffic,
                             "peak_source": f"nominal FP32: 152 SMs x 128 lanes x 2 flop x {smax:.0f} MHz "
                                            f"(sm_max_mhz of MEASURED_PEAKS.json, {src}); no FP32 figure is measured",
                             "flops_per_step": FLOPS_PER_STEP,
                             # the path kernel is bound by instruction issue: ncu pipe figures of the
                             # committed capture (profiles/paths_kernel_8x8_assembly.md)
                             "ncu_pipes": {k[len("paths_kernel_"):]: v for k, v in _read_profile_figures().items()
                                           if k.startswith("paths_kernel_") and not k.endswith("per_launch")}},
                "clocks": clocks,
                "time_to_1e-3": ttt,
                "cpu_baseline": base}
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def _franke_np(x, y):
    return (0.75 * np.exp(-0.25 * ((9 * x - 2) ** 2 + (9 * y - 2) ** 2)) +
            0.75 * np.exp(-((9 * x + 1) ** 2) / 49 - 0.1 * (9 * y + 1)) +
            0.5 * np.exp(-0.25 * ((9 * x - 7) ** 2 + (9 * y - 3) ** 2)) -
            0.2 * np.exp(-((9 * x - 4) ** 2) - (9 * y - 7) ** 2))


def _u_aniso(xy):
    return _franke_np(xy[:, 0], xy[:, 1]) * (1 + xy[:, 0] * xy[:, 1])


_PINNED = {}


def _pinned(n):
    """Page-locked host array of n doubles (kept for reuse), as a user keeps its
    output buffers."""
    if n not in _PINNED:
        import torch
        _PINNED[n] = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    return _PINNED[n]


def _assemble_stats(ctx, mesh, bvp, paths, prec, h, kernels=None):
    """One fk_assemble call into pinned host buffers (CSR values and B);
    returns (seconds, per-item stats).  `kernels`, if a list, receives the
    path and finalize kernel times (ms)."""
    from spac_gb300 import fk
    info = ctx.mesh_info(mesh)
    st = (fk.Stats * info["n_items"])()
    val = _pinned(info["nnz"])
    B = _pinned(info["n_rows"])
    t0 = time.perf_counter()
    ctx.check(ctx.L.fk_assemble(ctx.h, mesh, bvp, int(paths), None, h, prec, val.ctypes.data_as(fk._dp),
                                B.ctypes.data_as(fk._dp), None, None, st))
    dt = time.perf_counter() - t0
    if kernels is not None:
        kernels.extend(ctx.last_timing()[:2])
    return dt, fk.stats_array(st)


def time_to_target_all(ctx, mesh, target=1e-3, hs=(5e-4, 1e-4, 5e-5)):
    """time_to_target at the configured h and at smaller steps (the bias floor
    of the configured h can exceed the target)."""
    res = {}
    for h in hs:
        res["h=%g" % h] = time_to_target(ctx, mesh, target=target, h=h)
    return res


def time_to_target(ctx, mesh, target=1e-3, h=5e-4, pilot_grid=24, pilot_paths=600, pilot_h=1e-3, train_steps=800,
                   table=128, lr=3e-2, batch=4096, fit_output=True):
    """Time to `target` RMS node error on the assembly, plain FK vs the learned
    control variate (both FP32 stepping, same h).

    Node error of an item = its FK estimate of u at the node (exit value taken
    exactly, so the figure does not depend on the exit stencil) minus the exact
    u.  RMS^2 = bias^2 + mean(var)/N: each method's N comes from an untimed
    calibration run.  The learned-CV time includes its pilot (whole-domain
    point solves at pilot_grid^2 collocation points: boundary data only),
    training (train_steps Adam steps, batch 4096; with fit_output the output
    layer is then refitted by least squares on the hidden features), the
    gradient table and the assembly with the control term."""
    from spac_gb300 import fk
    info = ctx.mesh_info(mesh)
    row, ixy, stn, fr = ctx.mesh_items(mesh)
    u_exact = _u_aniso(ixy)
    prec = fk.FP32
    b_plain = ctx.register_bvp(fk.ANISO)

    def rms_of(st):
        return float(np.sqrt(np.mean((st["phi_VR"] - u_exact) ** 2)))

    # calibration of the plain method
    n_cal = 4000
    _, st = _assemble_stats(ctx, mesh, b_plain, n_cal, prec, h)
    var_p = np.maximum(st["phiphi_VR"] - st["phi_VR"] ** 2, 0)
    bias2 = max(rms_of(st) ** 2 - var_p.mean() / n_cal, 0.0)
    out = {"target": target, "bias_rms_est": float(np.sqrt(bias2)), "plain_var_mean": float(var_p.mean())}
    if bias2 >= 0.8 * target ** 2:
        out["unreachable"] = "bias floor at h=%g is above 0.9 x target" % h
        return out
    budget = target ** 2 - bias2
    n_plain = int(np.ceil(1.05 * var_p.mean() / budget))
    kp = []
    t_plain, st = _assemble_stats(ctx, mesh, b_plain, n_plain, prec, h, kp)
    out["plain"] = {"paths_per_item": n_plain, "seconds": t_plain, "rms": rms_of(st), "kernels_ms": kp}

    # learned control variate: pilot from boundary data only
    t0 = time.perf_counter()
    g = (np.arange(pilot_grid) + 0.5) / pilot_grid
    pxy = np.stack(np.meshgrid(g, g, indexing="ij"), axis=-1).reshape(-1, 2)  # x outer, y inner
    # the pilot only has to approximate u (any u_hat keeps the estimator
    # unbiased), so it runs at the coarse step pilot_h
    pst = ctx.solve_points(b_plain, pxy, pilot_paths, pilot_h, prec)
    t_pilot = time.perf_counter() - t0
    pilot_kernel_ms = ctx.last_timing()[0]
    rects = np.array([[0.0, 0.0, 1.0, 1.0]])
    mid = fk.C.c_int()
    ctx.check(ctx.L.fk_mlp_create(ctx.h, 1, rects.ctypes.data_as(fk._dp), 12345, fk.C.byref(mid)))
    mid = mid.value
    tgt = np.ascontiguousarray(pst["phi"])
    pxy = np.ascontiguousarray(pxy)
    hist = np.zeros(train_steps, dtype=np.float32)
    t1 = time.perf_counter()
    ctx.check(ctx.L.fk_mlp_train(ctx.h, mid, len(tgt), pxy.ctypes.data_as(fk._dp), tgt.ctypes.data_as(fk._dp), None,
                                 train_steps, batch, lr, 777, hist.ctypes.data_as(fk._fp)))
    t_train = time.perf_counter() - t1
    t_fit = 0.0
    if fit_output:
        # output layer refitted by least squares on the trained hidden layers
        t3 = time.perf_counter()
        ctx.check(ctx.L.fk_mlp_fit_output(ctx.h, mid, len(tgt), pxy.ctypes.data_as(fk._dp),
                                          tgt.ctypes.data_as(fk._dp), None, 1e-6))
        t_fit = time.perf_counter() - t3
    t2 = time.perf_counter()
    ctx.check(ctx.L.fk_mlp_build_table(ctx.h, mid, table))
    t_table = time.perf_counter() - t2
    b_cv = ctx.register_bvp(fk.ANISO, cv=fk.CV_MLP, mlp_id=mid)
    # calibration of the control-variate run (untimed, as for plain)
    _, stc = _assemble_stats(ctx, mesh, b_cv, n_cal, prec, h)
    var_c = np.maximum(stc["phiphi_VR"] - stc["phi_VR"] ** 2, 0)
    n_cv = max(32, int(np.ceil(1.05 * var_c.mean() / budget)))
    kc = []
    t_run, stc = _assemble_stats(ctx, mesh, b_cv, n_cv, prec, h, kc)
    t_cv = t_pilot + t_train + t_fit + t_table + t_run
    out["learned_cv"] = {"paths_per_item": n_cv, "seconds": t_cv, "rms": rms_of(stc), "pilot_s": t_pilot,
                         "train_s": t_train, "train_steps": train_steps, "fit_output_s": t_fit, "table_s": t_table,
                         "run_s": t_run, "run_kernels_ms": kc,
                         "pilot_kernel_ms": pilot_kernel_ms,
                         "pilot": f"{len(pxy)} collocation points x {pilot_paths} whole-domain paths, h={pilot_h:g}",
                         "train_loss_first_last": [float(hist[0]), float(hist[-1])]}
    out["variance_reduction"] = float(var_p.mean() / max(var_c.mean(), 1e-300))
    out["speedup_cv_over_plain"] = t_plain / t_cv
    out["speedup_cv_run_only"] = t_plain / t_run
    return out


def _mean_steps(ctx, mesh, bvp, prec, paths):
    """Mean Euler steps per path of the workload (from the kernel's own counters)."""
    from spac_gb300 import fk
    st = (fk.Stats * ctx.mesh_info(mesh)["n_items"])()
    rc = ctx.L.fk_assemble(ctx.h, mesh, bvp, min(paths, 2000), None, CFG["h"], prec, None, None, None, None, st)
    ctx.check(rc)
    ms = np.array([s.mean_steps for s in st])
    return float(ms.mean())


def _scatter_roofline(info, f_ms, peaks, src):
    """HBM roofline of the finalize/scatter kernel.  Algorithmic bytes per
    launch: per item its FP64 stencil moments (nwin x k words of the patch's
    windows), its 12 FP64 statistics, a read-modify-write of its G entries in
    the CSR values (16 B each) and of its B (16 B); per patch the FP32 window
    corrections E_W (nwin x k^2) read once."""
    k = CFG["knn"]
    m = info["max_stencil"]            # patch-boundary nodes = windows of a closed chain
    per_item = m * k * 8 + 12 * 8 + m * 16 + 16
    per_patch = m * k * k * 4
    bytes_ = info["n_items"] * per_item + info["n_stencils"] * per_patch
    achieved = bytes_ / (f_ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": _read_profile_figures().get("finalize_dram_bytes_per_launch"), "algorithmic_bytes": bytes_,
            "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({src})",
            "note": "latency-bound: CTA-wide phases per item (moments staged, window products, CSR scatter); profiles/"}


def _read_profile_figures():
    """Figures of the committed ncu summary (profiles/traffic.txt): name -> value."""
    out = {}
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and not parts[0].startswith("#"):
                    try:
                        out[parts[0]] = float(parts[1])
                    except ValueError:
                        pass
    return out


def _read_traffic():
    """DRAM bytes per path-kernel launch from the committed ncu summary, if present."""
    return _read_profile_figures().get("paths_kernel_dram_bytes_per_launch")


if __name__ == "__main__":
    sys.exit(main())
