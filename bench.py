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

    def start(self, interval_ms=50, wait_s=5.0):
        """Starts sampling every interval_ms and returns once the first sample
        has arrived (nvidia-smi takes a while to start), so that the samples
        cover the region timed after this call."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", str(interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < wait_s:
            time.sleep(0.005)

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
# The CPU legs (cpu_baseline, --impl reference) never load the product
# library: the layout comes from the oracle's numpy restatement of the mesh.
def _cpu_items(eps_spacing=None):
    """Items of the workload for the oracle: (item, x, y, patch rect, patch
    chain coordinates), the Gaussian shape eps, and the item count."""
    import oracle_py as orc
    m = orc.square_patch_mesh(CFG["domain"], CFG["n_sub"], CFG["nodes_per_side"], CFG["enlarge"])
    eps = (CFG["eps_spacing"] if eps_spacing is None else eps_spacing) / m["spacing"]
    items = [(i, float(m["nodes"][g, 0]), float(m["nodes"][g, 1]), m["patches"][s]["rect"],
              np.ascontiguousarray(m["patches"][s]["chain"])) for i, (g, s) in enumerate(m["items"])]
    return items, eps


def _cpu_worker(args):
    """Oracle node solves (Gaussian k-nearest stencil) of a slice of items; one
    process per host core."""
    import oracle_py as orc
    items, seed, stream, N, h, k, eps = args
    s = orc.Session(orc.RNG_PHILOX, seed=seed, stream=stream)
    b = orc.bvp(2)  # ORC_PROBLEM_ANISO
    t0 = time.perf_counter()
    npaths = 0
    for (i, x, y, rect, chain) in items:
        s.node_solve_knn(b, x, y, rect, chain, k, eps, N, h, item=i)
        npaths += N
    return npaths, time.perf_counter() - t0


class CpuSample:
    """A fixed, seeded sample of the workload's items, solved by the oracle
    (FP64, 2,000 paths per item) on a pool of spawned processes, one per host
    core; `run()` times one pass over the sample (wall clock)."""

    N = 2000

    def __init__(self, cores, budget_s):
        self.items, self.eps = _cpu_items()
        rng = np.random.default_rng(5)
        # calibrate on one item (in this process), then size the sample so that
        # one pass takes about budget_s on `cores` processes
        n_cal, t_cal = _cpu_worker(([self.items[int(rng.integers(len(self.items)))]], 9, 1, self.N, CFG["h"],
                                    CFG["knn"], self.eps))
        per_core = max(1, int(budget_s * n_cal / max(t_cal, 1e-6) / self.N))
        picks = rng.choice(len(self.items), size=min(len(self.items), per_core * cores), replace=False)
        self.picks = picks
        self.slices = [[self.items[int(i)] for i in picks[c::cores]] for c in range(cores)]
        self.slices = [sl for sl in self.slices if sl]
        self.pool = mp.get_context("spawn").Pool(len(self.slices))
        self.pool.map(_cpu_worker, [(sl[:1], 9, 1, 16, CFG["h"], CFG["knn"], self.eps) for sl in self.slices])

    @property
    def cores(self):
        return len(self.slices)

    def describe(self, wall):
        return (f"{len(self.picks)} of {len(self.items)} items x {self.N} paths per step (oracle FP64, "
                f"one process per core, {wall:.2f} s wall per step)")

    def run(self, stream=1):
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_worker, [(sl, 9, stream, self.N, CFG["h"], CFG["knn"], self.eps)
                                          for sl in self.slices])
        wall = time.perf_counter() - t0
        return sum(r[0] for r in res), wall

    def close(self):
        self.pool.close()
        self.pool.join()


# The other configs' workloads, restated with numpy from their descriptions
# (the GPU side builds them in spac_gb300.workloads with the same seeds).
def _config1_points():
    g = np.arange(1, 33) / 33.0
    return np.array([(x, y) for x in g for y in g])


def _config3_points(seed=2026, n_bvp=16, nodes=1 << 14):
    """The 16 uneven disks: radius, centre, paths and h per node (the same
    draws, in the same order, as spac_gb300.workloads.uneven)."""
    rng = np.random.default_rng(seed)
    R = rng.uniform(0.25, 1.0, n_bvp)
    centers = np.stack([2.5 * np.arange(n_bvp), np.zeros(n_bvp)], axis=1)
    per = nodes // n_bvp
    xy, disk = [], []
    for k in range(n_bvp):
        r = R[k] * np.sqrt(rng.uniform(0, 1, per))
        th = rng.uniform(0, 2 * np.pi, per)
        xy.append(np.stack([centers[k, 0] + r * np.cos(th), centers[k, 1] + r * np.sin(th)], axis=1))
        disk += [k] * per
    xy = np.concatenate(xy)
    disk = np.array(disk)
    paths = np.maximum(1, np.round(np.exp(rng.uniform(np.log(1e3), np.log(1e5), len(xy))))).astype(np.int64)
    h = rng.choice([1e-3, 5e-4], len(xy))
    return xy, disk, R, centers, paths, h


def _cpu_job(args):
    """Oracle solves of one slice of a config's sample: point solves (configs 1
    and 3) or Gaussian-stencil node solves (config 5).  Returns (paths, nodes,
    seconds)."""
    import oracle_py as orc
    kind, jobs = args
    s = orc.Session(orc.RNG_PHILOX, seed=9, stream=1)
    t0 = time.perf_counter()
    npaths = 0
    for j in jobs:
        if kind == "points":
            i, problem, dom, dshape, prob, x, y, N, h = j
            s.point_solve(orc.bvp(problem, dom=dom, dom_shape=dshape, prob=prob), x, y, N, h, item=i)
        else:
            i, x, y, rect, chain, k, eps, N, h = j
            s.node_solve_knn(orc.bvp(0), x, y, rect, chain, k, eps, N, h, item=i)
        npaths += N
    return npaths, len(jobs), time.perf_counter() - t0


def cpu_configs(cores, budget_s=4.0):
    """The CPU oracle (FP64, the reference's arithmetic, pinned to its own
    sources) on bounded seeded samples of configs 1, 3 and 5, one spawned
    process per host core: paths/s and node solves/s beside the GPU's."""
    import oracle_py as orc
    orc.build(ref=False)
    rng = np.random.default_rng(11)
    samples = {}
    p1 = _config1_points()
    samples["config1"] = ("points", [(i, 0, (0, 0, 1, 1), orc.RECT, (0, 0, 0, 0), x, y, 10000, 1e-3)
                                     for i, (x, y) in enumerate(p1)], "32x32 nodes x 1e4 paths, h=1e-3, Franke")
    xy, disk, R, cen, paths, h = _config3_points()
    jobs = [(i, 3, (R[disk[i]], cen[disk[i], 0], cen[disk[i], 1], 0), orc.CIRCLE,
             (cen[disk[i], 0], cen[disk[i], 1], R[disk[i]], 0), xy[i, 0], xy[i, 1], int(paths[i]), h[i])
            for i in range(len(xy))]
    samples["config3"] = ("points", jobs, "16 uneven disks, 2^14 nodes, paths log-uniform 1e3..1e5, h in {1e-3, 5e-4}")
    m = orc.square_patch_mesh((0, 0, 1, 1), 32, 63, 0.25)
    eps = 3.0 / m["spacing"]

    class Items5:  # the config-5 items as jobs, built on access (409k chain copies would not fit)
        def __len__(self):
            return len(m["items"])

        def __getitem__(self, i):
            g, st = m["items"][i]
            return (i, float(m["nodes"][g, 0]), float(m["nodes"][g, 1]), m["patches"][st]["rect"],
                    np.ascontiguousarray(m["patches"][st]["chain"]), 20, eps, 1000, 2.5e-4)

    samples["config5"] = ("knn", Items5(), "32x32 square-patch items x 1000 paths, h=2.5e-4, Gaussian 20-NN stencil")
    out = {}
    with mp.get_context("spawn").Pool(cores) as pool:
        for name, (kind, jobs, desc) in samples.items():
            # calibrate on a few jobs, then take a seeded sample worth budget_s on `cores` processes
            probe = [jobs[int(i)] for i in rng.choice(len(jobs), size=min(4, len(jobs)), replace=False)]
            n_cal, k_cal, t_cal = _cpu_job((kind, probe))
            per_job = t_cal / max(k_cal, 1)
            n_take = int(min(len(jobs), max(cores, budget_s * cores / max(per_job, 1e-6))))
            pick = rng.choice(len(jobs), size=n_take, replace=False)
            sl = [(kind, [jobs[int(i)] for i in pick[c::cores]]) for c in range(cores)]
            t0 = time.perf_counter()
            res = pool.map(_cpu_job, [x for x in sl if x[1]])
            wall = time.perf_counter() - t0
            npaths, nodes = sum(r[0] for r in res), sum(r[1] for r in res)
            out[name] = {"paths_per_s": npaths / wall, "node_solves_per_s": nodes / wall, "cores": cores,
                         "kind": "port", "sample": f"{nodes} of {len(jobs)} nodes ({desc}); oracle FP64, "
                                                   f"{wall:.2f} s wall"}
    return out


def cpu_baseline(cores, budget_s=12.0):
    """The CPU oracle port timed on a bounded sample of the same workload."""
    import oracle_py as orc
    orc.build(ref=False)
    cs = CpuSample(cores, budget_s)
    try:
        npaths, wall = cs.run()
    finally:
        cs.close()
    return {"value": npaths / wall, "unit": "paths/s", "cores": cs.cores, "kind": "port",
            "sample": cs.describe(wall)}


def run_reference(args):
    """The reference arm: the oracle port of the reference's FK node solve
    (pinned bit for bit to the reference's own sources) on all host cores.
    Each step is one pass over a fixed sample of the workload's items; W
    untimed passes, then K timed ones."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle_py as orc
    orc.build(ref=False)
    cores = os.cpu_count() or 1
    cs = CpuSample(cores, budget_s=2.0)
    try:
        for w in range(args.warmup):
            cs.run(stream=100 + w)
        walls, paths = [], 0
        for k in range(args.steps):
            n, wall = cs.run(stream=1 + k)
            walls.append(wall)
            paths += n
    finally:
        cs.close()
    t_step = float(np.mean(walls))
    v = paths / float(np.sum(walls))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "paths/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(CFG, precision="fp64", paths_per_item=cs.N, items_per_step=len(cs.picks),
                           sample=cs.describe(t_step),
                           note="CPU oracle port of the reference FK node solve (the reference itself has no "
                                "square-patch/Gaussian stencil; its sources need Eigen and Boost, absent on the GPU "
                                "host); mesh from the oracle's own layout code"),
            "cpu_baseline": {"value": v, "unit": "paths/s", "cores": cs.cores, "kind": "port",
                             "sample": cs.describe(t_step)},
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
    ap.add_argument("--no-configs", action="store_true", help="skip configs 1, 3 and 5 (GPU and CPU)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    CFG["paths_per_item"] = args.paths

    # CPU baseline first (spawned pool, before any GPU call), rank 0 at N=1 only
    base = cpu_cfg = None
    if rank == 0 and world == 1 and not args.no_cpu:
        base = cpu_baseline(os.cpu_count() or 1)
        if not args.no_configs:
            cpu_cfg = cpu_configs(os.cpu_count() or 1)

    from spac_gb300 import fk
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

    def step_device(precision=prec):
        rc = ctx.L.fk_assemble(ctx.h, mesh, bvp, paths, None, CFG["h"], precision, dptr(val), dptr(Bd), None, None,
                               None)
        ctx.check(rc)

    def timed_device(n, precision=prec):
        times, kern = [], []
        for _ in range(n):
            with torch.cuda.stream(ext):
                flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            step_device(precision)
            e1.record(ext)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            kern.append(ctx.last_timing())
        return times, kern

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    times, kern = timed_device(args.steps)
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
    windows = ctx.last_windows()  # stencil windows whose moments became G rows in the last assembly
    if dist:
        e2e_step = max_over_ranks(e2e_step, dist)
    # per call: one 96-byte item record and one 12-byte chunk record per item
    # (an item of <= 32768 paths is one chunk); back: CSR values, B, 4 check words
    item_bytes = info["n_items"] * (96 + 12)
    d2h = 8 * (info["nnz"] + info["n_rows"]) + 16

    # the same assembly with FP64 stepping (the reference's arithmetic): the
    # precision-matched GPU figure beside the CPU oracle's FP64 one
    step_device(fk.FP64)
    t64, _ = timed_device(2, fk.FP64)
    fp64 = {"value": total_paths / (float(np.mean(t64)) / 1000.0), "unit": "paths/s", "ms_per_step": float(np.mean(t64)),
            "note": "same assembly, FP64 stepping and FP64 stencil products, device buffers"}

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
    ttt = cfgs = None
    if rank == 0 and not args.no_metric:
        ttt = _guarded(lambda: time_to_target_all(ctx), ctx)
    if rank == 0 and not args.no_configs:
        cfgs = _guarded(lambda: other_configs(ctx, cpu_cfg), ctx)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(CFG, items=info["n_items"], rows=info["n_rows"], nnz=info["nnz"],
                               paths_per_step=total_paths, l2="flushed between steps (512 MB write)"),
                "e2e": {"value": world * total_paths / e2e_step, "unit": "paths/s", "h2d_bytes_per_step": item_bytes,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": 2 * args.steps,
                "node_solves_per_s": world * info["n_items"] / (t_step / 1000.0),
                "fp64_stepping": fp64,
                "kernels_ms": {"paths": k_ms, "finalize_scatter": f_ms},
                "mean_steps_per_path": steps_per_assembly,
                "roofline_scatter": _scatter_roofline(info, f_ms, peaks, src, windows),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak, "traffic": traffic,
                             "peak_source": f"nominal FP32: 152 SMs x 128 lanes x 2 flop x {smax:.0f} MHz "
                                            f"(sm_max_mhz of MEASURED_PEAKS.json, {src}); no FP32 figure is measured",
                             "flops_per_step": FLOPS_PER_STEP,
                             "traffic_source": "ncu dram bytes of one launch, committed capture",
                             # the path kernel is bound by instruction issue: ncu pipe figures of the
                             # committed capture of this kernel on this workload
                             "ncu_pipes": {k[len("paths_kernel_"):]: v for k, v in _read_profile_figures().items()
                                           if k.startswith("paths_kernel_") and
                                           (k.endswith("_pipe") or k.endswith("issue_active"))},
                             "issue": _issue_roofline(total_paths, steps_per_assembly, k_ms, smax)},
                "clocks": clocks,
                "time_to_1e-3": ttt,
                "configs": cfgs,
                "cpu_baseline": base}
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def _guarded(fn, ctx):
    """Runs a secondary leg of the bench (the metric, the other configs); a
    library error there (for instance the kernels' own completed-path check)
    is recorded in the line instead of ending the run before the headline
    figures are printed."""
    from spac_gb300 import fk
    try:
        return fn()
    except fk.FKError as e:
        return {"error": str(e)}


def other_configs(ctx, cpu=None):
    """Configs 1, 3 and 5 on the GPU (spac_gb300.workloads), each beside the
    CPU oracle's figure on a sample of the same workload when it was timed."""
    from spac_gb300 import workloads as wl
    out = {}
    c1 = wl.point_solves(ctx)
    out["config1"] = {"gpu": c1}
    c3 = wl.uneven(ctx)
    ctx.set_launch(0, 0)  # (the autotuner keeps its launch shape in the context)
    out["config3"] = {"gpu": c3}
    c5 = wl.large(ctx)
    out["config5"] = {"gpu": c5}
    # the same adaptive assembly with the stencil shape whose rows interpolate
    # the exit value accurately (eps = 1/spacing; the specified 3/spacing
    # leaves an O(0.1) row residual)
    out["config5_eps_spacing_1"] = {"gpu": wl.large(ctx, eps_spacing=1.0)}
    if cpu:
        for k in out:
            out[k]["cpu"] = cpu.get(k)
        out["config1"]["gpu_over_cpu_paths_per_s_fp64"] = c1["fp64"]["paths_per_s"] / cpu["config1"]["paths_per_s"]
        out["config3"]["gpu_over_cpu_paths_per_s"] = c3["fp32"]["paths_per_s"] / cpu["config3"]["paths_per_s"]
        out["config5"]["gpu_over_cpu_paths_per_s"] = c5["paths_per_s"] / cpu["config5"]["paths_per_s"]
    return out


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


def _assemble_host(ctx, mesh, bvp, paths, prec, h, kernels=None, stats=False):
    """One fk_assemble call into pinned host buffers (CSR values and B, as a
    caller of the C ABI keeps them); returns (seconds, val, B, per-item
    stats or None).  `kernels`, if a list, receives the path and finalize
    kernel times (ms)."""
    from spac_gb300 import fk
    info = ctx.mesh_info(mesh)
    st = (fk.Stats * info["n_items"])() if stats else None
    val = _pinned(info["nnz"])
    B = _pinned(info["n_rows"])
    t0 = time.perf_counter()
    ctx.check(ctx.L.fk_assemble(ctx.h, mesh, bvp, int(paths), None, h, prec, val.ctypes.data_as(fk._dp),
                                B.ctypes.data_as(fk._dp), None, None, st))
    dt = time.perf_counter() - t0
    if kernels is not None:
        kernels.extend(ctx.last_timing()[:2])
    return dt, val.copy(), B.copy(), fk.stats_array(st) if stats else None


class AssembledSystem:
    """The assembled 8x8 system G u = B of one mesh and the exact solution at
    its nodes: the error measures of the time-to-1e-3 metric.

    row residual  e_r = (sum_j val_rj u(x_j) - B_r) / diag_r, with u the exact
                  solution: the average, over the row's items, of the item's
                  FK estimate of u(x_r) given the exact values at its stencil
                  nodes, minus u(x_r) (the reference's own check G u_exact ~ B,
                  Mesh/Interfaz.cpp:252-262, divided by the diagonal).  It
                  includes the exit stencil's interpolation error.
    GMRES error   the host GMRES solution of the assembled system minus u at
                  the nodes (the system the reference solves,
                  Solvers/SistemaLinealSolverGMRES.hpp:157-597)."""

    def __init__(self, ctx, mesh):
        self.ctx, self.mesh = ctx, mesh
        self.rp, self.col, v0 = ctx.mesh_csr(mesh)
        xy, _ = ctx.mesh_nodes(mesh)
        self.u = _u_aniso(xy)
        n = len(self.rp) - 1
        self.diag = v0[self.rp[:-1] + np.array([np.searchsorted(self.col[self.rp[i]:self.rp[i + 1]], i)
                                                 for i in range(n)])]
        self.row, ixy, _, _ = ctx.mesh_items(mesh)
        self.u_items = _u_aniso(ixy)

    def residual(self, val, B):
        Au = np.add.reduceat(val * self.u[self.col], self.rp[:-1])
        return (Au - B) / self.diag

    def gmres_rms(self, val, B):
        from spac_gb300 import fk
        x, it, res, rc = fk.gmres(self.rp, self.col, val, B, tol=1e-10, max_iter=3000, restart=60)
        return {"rms": float(np.sqrt(np.mean((x - self.u) ** 2))), "max": float(np.abs(x - self.u).max()),
                "iterations": it, "rel_resid": res, "converged": rc == 0}

    def calibrate(self, bvp, h, n_cal, streams=(9001, 9002)):
        """Two independent assemblies at n_cal paths per item: their residual
        difference gives the per-path variance of the row residual (bias
        cancels), their mean the bias.  Returns (bias^2, variance per path,
        the exact-exit item variance of the first run)."""
        from spac_gb300 import fk
        es, st0 = [], None
        saved = self.ctx.get_stream()
        for s in streams:
            self.ctx.set_stream(s)
            _, val, B, st = _assemble_host(self.ctx, self.mesh, bvp, n_cal, fk.FP32, h, stats=st0 is None)
            es.append(self.residual(val, B))
            st0 = st if st0 is None else st0
        self.ctx.set_stream(saved)
        var_path = float(np.mean((es[0] - es[1]) ** 2) / 2.0 * n_cal)
        bias2 = max(float(np.mean(((es[0] + es[1]) / 2) ** 2)) - var_path / (2 * n_cal), 0.0)
        return bias2, var_path, st0


def _rms(e):
    return float(np.sqrt(np.mean(e ** 2)))


def weight_sum_defect(eps_spacing, k=20):
    """Sum of the Gaussian k-nearest weights w = A^-1 phi(x) at points of a
    straight chain of equispaced nodes (the inside of a patch side): 1 at a
    node, less in between (Gaussian RBF interpolation does not reproduce
    constants).  The probe points sit at fractions 0, 1/4 and 1/2 of a spacing
    from a node in the middle of the window."""
    x = np.arange(k, dtype=np.float64)
    A = np.exp(-(eps_spacing * (x[:, None] - x[None, :])) ** 2)
    out = {}
    for name, f in (("at_node", 0.0), ("quarter", 0.25), ("midpoint", 0.5)):
        t = k // 2 - 1 + f
        phi = np.exp(-(eps_spacing * (t - x)) ** 2)
        out[name] = float(np.linalg.solve(A, phi).sum())
    return out


def time_to_target_all(ctx, target=1e-3):
    """The metric on the assembled system at the configured stencil shape
    (eps = 3/spacing) and at eps = 1/spacing, at the configured h and at
    smaller steps (the O(h) bias floor of h = 5e-4 exceeds the target)."""
    res = {"error_measure": "RMS over rows of the row residual (sum_j val_rj u(x_j) - B_r) / diag_r with the exact u",
           "weight_sum": {"eps_spacing=3": weight_sum_defect(3.0), "eps_spacing=1": weight_sum_defect(1.0)}}
    for eps_sp in (3.0, 1.0):
        mesh = ctx.mesh_square_patches(CFG["domain"], CFG["n_sub"], CFG["nodes_per_side"], CFG["enlarge"], eps_sp,
                                       CFG["knn"])
        sysm = AssembledSystem(ctx, mesh)
        hs = (5e-4,) if eps_sp == 3.0 else (5e-4, 1e-4, 5e-5, 2.5e-5, 1e-5)
        r = {}
        for h in hs:
            r["h=%g" % h] = _guarded(lambda: time_to_target(ctx, sysm, target=target, h=h), ctx)
        res["eps_spacing=%g" % eps_sp] = r
    return res


def time_to_target(ctx, sysm, target=1e-3, h=5e-4, pilot_grid=24, pilot_paths=300, pilot_h=1e-3, train_steps=10,
                   table=128, lr=1e-2, batch=4096, fit_output=True, n_cal=4000, only=None, gmres=True,
                   rep_streams=(7101, 7102), pilot_max_steps=0):
    """Time to `target` RMS row residual of the assembled system, plain FK vs
    the learned control variate (both FP32 stepping, same h, same paths for
    every item).

    RMS^2 = bias^2 + var/N per method, from two untimed calibration
    assemblies; the timed assembly runs at the N that this predicts for the
    target (x 1.05), and again at a larger N if its measured RMS is above the
    target.  The learned-CV time includes its pilot (whole-domain point solves
    at pilot_grid^2 collocation points: boundary data only), training
    (train_steps Adam steps; with fit_output the output layer is then refitted
    by least squares on the hidden features), the gradient table and the
    assembly with the control term.  Each timed assembly's system is also
    solved by the host GMRES and its node error reported.  Each method is
    then timed again on the replicate streams at the same paths per item
    (the CV's whole pipeline included) and the median time is reported."""
    from spac_gb300 import fk
    prec = fk.FP32
    b_plain = ctx.register_bvp(fk.ANISO)
    out = {"target": target}

    def run_to_target(bvp, bias2, var_path, floor_paths=32):
        budget = target ** 2 - bias2
        n = max(floor_paths, int(np.ceil(1.05 * var_path / budget)))
        attempts = []
        for _ in range(3):
            kern = []
            t, val, B, st = _assemble_host(ctx, sysm.mesh, bvp, n, prec, h, kern)
            e = sysm.residual(val, B)
            attempts.append({"paths_per_item": n, "seconds": t, "rms": _rms(e), "kernels_ms": kern})
            if _rms(e) <= target:
                break
            n = int(np.ceil(n * 1.05 * max(_rms(e) ** 2 - bias2, 1e-30) / budget))
        last = dict(attempts[-1])
        if gmres:
            last["gmres_node_error"] = sysm.gmres_rms(val, B)
        if len(attempts) > 1:
            last["earlier_attempts"] = attempts[:-1]
        return last

    def replicate(bvp, n, before):
        """Timed assemblies at n paths per item on the replicate streams;
        `before()` runs first on each stream (its result is returned beside
        the assembly time).  Returns ([(seconds, before()), ...], [rms, ...])."""
        saved = ctx.get_stream()
        ts, rs = [], []
        for s in rep_streams:
            ctx.set_stream(s)
            f = before()
            t, val, B, _ = _assemble_host(ctx, sysm.mesh, bvp, n, prec, h)
            ts.append((t, f))
            rs.append(_rms(sysm.residual(val, B)))
        ctx.set_stream(saved)
        return ts, rs

    # the pilot's collocation lattice: a fixed input, laid out once (as the mesh is)
    g = (np.arange(pilot_grid) + 0.5) / pilot_grid
    pilot_xy = np.ascontiguousarray(np.stack(np.meshgrid(g, g, indexing="ij"), axis=-1).reshape(-1, 2))  # x outer

    def cv_pipeline(drop=False):
        """Pilot, training, output refit and gradient table of the learned
        control variate (the network's weights reset to their initial values
        first, untimed, as creating the network is); returns the stage times."""
        t0 = time.perf_counter()
        pxy = pilot_xy
        # the pilot only has to approximate u (any u_hat keeps the estimator
        # unbiased), so it runs at the coarse step pilot_h
        if pilot_max_steps:
            # the pilot's paths stop after pilot_max_steps (a stopped path is
            # scored at its nearest boundary point): the pilot only shapes u_hat
            ctx.set_max_steps(pilot_max_steps)
        pst = ctx.solve_points(b_plain, pxy, pilot_paths, pilot_h, prec, allow=(fk.FK_ERR_STEP_CAP,))
        if pilot_max_steps:
            ctx.set_max_steps(1 << 24)
        t_pilot = time.perf_counter() - t0
        pilot_kernel_ms = ctx.last_timing()[0]
        tgt = np.ascontiguousarray(pst["phi"])
        pxy = np.ascontiguousarray(pxy)
        # one network per context; its device buffers persist
        mid = _cv_network(ctx, pxy, tgt, table)
        t_reset0 = time.perf_counter()
        ctx.check(ctx.L.fk_mlp_set_params(ctx.h, mid, _CV_NET[ctx.h.value][1].ctypes.data_as(fk._fp)))
        t_reset = time.perf_counter() - t_reset0
        hist = np.zeros(max(train_steps, 1), dtype=np.float32)
        t1 = time.perf_counter()
        if train_steps > 0:
            ctx.check(ctx.L.fk_mlp_train(ctx.h, mid, len(tgt), pxy.ctypes.data_as(fk._dp),
                                         tgt.ctypes.data_as(fk._dp), None, train_steps, batch, lr, 777,
                                         hist.ctypes.data_as(fk._fp)))
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
        r = {"pilot_s": t_pilot, "train_s": t_train, "fit_output_s": t_fit, "table_s": t_table,
             "fixed_s": t_pilot + t_train + t_fit + t_table, "untimed_weight_reset_s": t_reset,
             "pilot_kernel_ms": pilot_kernel_ms}
        if not drop:
            r["mlp_id"] = mid
            r["hist"] = hist
        return r

    bias2, var_p, st_cal = sysm.calibrate(b_plain, h, n_cal)
    out["bias_rms_est"] = float(np.sqrt(bias2))
    # diagnostic: the same items scored with the exact exit value instead of the stencil
    out["diagnostic_exact_exit_rms_at_calibration"] = _rms(st_cal["phi_VR"] - sysm.u_items)
    out["plain_var_per_path"] = var_p
    if bias2 >= 0.8 * target ** 2:
        out["unreachable"] = "bias floor %.2e of the row residual at h=%g is above 0.9 x target" % (np.sqrt(bias2), h)
        return out
    if only != "cv":
        out["plain"] = plain = run_to_target(b_plain, bias2, var_p)
        ts, rs = replicate(b_plain, plain["paths_per_item"], lambda: {})
        plain["seconds_first"] = plain["seconds"]
        plain["seconds_each"] = [plain["seconds"]] + [t for t, _ in ts]
        plain["rms_each"] = [plain["rms"]] + rs
        plain["seconds"] = float(np.median(plain["seconds_each"]))

    # learned control variate: pilot from boundary data only
    fixed0 = cv_pipeline()
    mid = fixed0.pop("mlp_id")
    b_cv = ctx.register_bvp(fk.ANISO, cv=fk.CV_MLP, mlp_id=mid)
    bias2_c, var_c, _ = sysm.calibrate(b_cv, h, n_cal)
    cv = run_to_target(b_cv, bias2_c, var_c)
    hist = fixed0.pop("hist")
    cv.update(fixed0)
    first_total = fixed0["fixed_s"] + cv["seconds"]
    cv.update({"seconds_run": cv["seconds"], "seconds_first": first_total,
               "train_steps": train_steps, "batch": batch, "lr": lr,
               "bias_rms_est": float(np.sqrt(bias2_c)), "var_per_path": var_c,
               "pilot": f"{pilot_grid ** 2} collocation points x {pilot_paths} whole-domain paths, h={pilot_h:g}",
               "train_loss_first_last": [float(hist[0]), float(hist[max(train_steps, 1) - 1])]})
    # the whole pipeline again (weights reset, new pilot, training, refit,
    # table, assembly) on other random streams
    ts, rs = replicate(b_cv, cv["paths_per_item"], lambda: cv_pipeline(drop=True))
    cv["seconds_each"] = [first_total] + [t + f["fixed_s"] for t, f in ts]
    cv["seconds_run_each"] = [cv["seconds_run"]] + [t for t, _ in ts]
    cv["fixed_s_each"] = [fixed0["fixed_s"]] + [f["fixed_s"] for _, f in ts]
    cv["rms_each"] = [cv["rms"]] + rs
    cv["seconds"] = float(np.median(cv["seconds_each"]))
    cv["seconds_run"] = float(np.median(cv["seconds_run_each"]))
    out["learned_cv"] = cv
    out["variance_reduction"] = float(var_p / max(var_c, 1e-300))
    if "plain" in out:
        out["speedup_cv_over_plain"] = out["plain"]["seconds"] / cv["seconds"]
        out["speedup_cv_run_only"] = out["plain"]["seconds"] / cv["seconds_run"]
        out["timing"] = (f"median of {1 + len(rep_streams)} timed runs per method: the run that met the target "
                         f"and {len(rep_streams)} replicates at its paths per item on other random streams "
                         "(each CV replicate redoes the pilot, training, refit and table)")
    return out


_CV_NET = {}


def _cv_network(ctx, pxy, tgt, table):
    """The learned control variate's network of a context: created once, its
    buffers warmed by one untimed pass of training, refit and table build;
    returns its id (the initial weights are kept for resets)."""
    from spac_gb300 import fk
    key = ctx.h.value
    if key not in _CV_NET:
        rects = np.array([[0.0, 0.0, 1.0, 1.0]])
        mid = fk.C.c_int()
        ctx.check(ctx.L.fk_mlp_create(ctx.h, 1, rects.ctypes.data_as(fk._dp), 12345, fk.C.byref(mid)))
        mid = mid.value
        n = fk.C.c_int()
        ctx.check(ctx.L.fk_mlp_num_params(ctx.h, mid, fk.C.byref(n)))
        p0 = np.zeros(n.value, dtype=np.float32)
        ctx.check(ctx.L.fk_mlp_get_params(ctx.h, mid, p0.ctypes.data_as(fk._fp)))
        # (the per-step history and schedule buffers grow with the step count: warm them for up to 256 steps)
        ctx.check(ctx.L.fk_mlp_train(ctx.h, mid, len(tgt), pxy.ctypes.data_as(fk._dp), tgt.ctypes.data_as(fk._dp),
                                     None, 256, 4096, 1e-3, 1, None))
        ctx.check(ctx.L.fk_mlp_fit_output(ctx.h, mid, len(tgt), pxy.ctypes.data_as(fk._dp),
                                          tgt.ctypes.data_as(fk._dp), None, 1e-6))
        ctx.check(ctx.L.fk_mlp_build_table(ctx.h, mid, table))
        _CV_NET[key] = (mid, p0)
    return _CV_NET[key][0]


def _mean_steps(ctx, mesh, bvp, prec, paths):
    """Mean Euler steps per path of the workload (from the kernel's own
    counters, on a 2,000-path run of the same assembly)."""
    from spac_gb300 import fk
    st = (fk.Stats * ctx.mesh_info(mesh)["n_items"])()
    rc = ctx.L.fk_assemble(ctx.h, mesh, bvp, min(paths, 2000), None, CFG["h"], prec, None, None, None, None, st)
    ctx.check(rc)
    ms = np.array([s.mean_steps for s in st])
    return float(ms.mean())


def _scatter_roofline(info, f_ms, peaks, src, windows):
    """The G/B scatter of the 8x8 assembly.  It is fused into the path kernel:
    the last warp out of an item forms the item's G row from its moments in
    shared memory and adds it to the CSR values, so the window moments never
    reach DRAM and the scatter's time cannot be separated from the path
    kernel's.  Algorithmic DRAM bytes: per row its CSR entries written, 12 B
    each with their column, and B, 12 B; the per-row figure that also counts
    20 FP64 moments (160 B) per window the exits chose is given beside it,
    with the window count the kernel reports (fk_last_windows).  Both against
    the path kernel's DRAM traffic per launch in the committed capture; the
    finalize launch that remains writes only statistics and B.  The standalone
    HBM-bound scatter is config 5's end pass (configs.config5.gpu.end_pass)."""
    bytes_ = info["nnz"] * 12 + info["n_rows"] * 12
    with_windows = bytes_ + 160 * windows
    traffic = _read_profile_figures().get("paths_kernel_dram_bytes_per_launch")
    return {"bound": "hbm", "fused_into": "paths_kernel", "algorithmic_bytes": bytes_, "traffic": traffic,
            "traffic_over_algorithmic": traffic / bytes_ if traffic else None,
            "visited_windows": windows, "bytes_with_window_moments": with_windows,
            "traffic_over_bytes_with_window_moments": traffic / with_windows if traffic else None,
            "finalize_head_ms": f_ms, "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
            "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({src})",
            "note": "traffic: ncu dram bytes of one path-kernel launch (committed capture, slot mode, whole items)"}


def _issue_roofline(total_paths, steps_per_path, k_ms, smax):
    """The path kernel against its issue bound: its warp instructions (the
    committed ncu fit, per path-step and per path, times this run's paths and
    mean steps) over its event time, against one warp instruction per cycle
    on each of the 4 x 152 schedulers at the maximum SM clock."""
    figs = _read_profile_figures()
    ips, ipp = figs.get("paths_kernel_warp_inst_per_step"), figs.get("paths_kernel_warp_inst_per_path")
    if not (ips and ipp):
        return None
    inst = total_paths * (ipp + ips * steps_per_path)
    achieved = inst / (k_ms / 1000.0) / 1e12
    peak = 152 * 4 * smax * 1e6 / 1e12
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "T warp instructions/s", "frac": achieved / peak,
            "warp_inst_per_step": ips, "warp_inst_per_path": ipp,
            "source": "instruction counts: committed ncu fit over two step sizes (profiles/traffic.txt); time: this run"}


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
