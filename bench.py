"""Benchmark of the KDTree hot path on GB300.

Default workload (the FOF configuration): 2^20 particles, 70% in 500 Plummer spheres
+ 30% uniform background, periodic box L=100, linking length 0.2 x mean spacing,
minnum 20. One step = GPU tree build (bucket 16) + FOF, i.e. the reference's
KDTree(...) + FOF(ll, ngroup, 20). The line also carries the other parts of the metric
under "metric_parts": kNN-density rates (32768 uniform particles in the periodic unit box
with k=32 FindNearest + CalcDensity, 2^20 clustered particles with CalcDensity(32), 256^3
clustered particles with CalcDensity(64) + CalcVelDensity(64, 64)), the batched path on
20,000 power-law groups against the per-tree loop, and the adjoint's cost. Every
component's full record (phases, CPU figures) goes to the file named by
"components_file" (NBKDT_BENCH_DETAIL, default bench_components.json in the temp dir).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value  = particles per second with inputs already in HBM (device pointers);
e2e    = the same through the C ABI with host buffers (H2D of positions and masses and
         D2H of the group array inside each step);
impl reference = the CPU restatement of the reference (oracle/) on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "kNN-density queries/s & FOF particles/s, batched vs per-tree, 1 GB300"
N_FOF = 1 << 20
BOX = 100.0
MINNUM = 20
BUCKET = 16
# DRAM bytes of one k_link launch at 2^20 particles: 240.4 MB measured by ncu on the same
# recipe at 2^22 particles (the bench's --profile fof case), divided by 4
K_LINK_DRAM_BYTES_PER_LAUNCH = 240.435e6 / 4


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        # raw samples go to NBKDT_CLOCKS_DIR (default: the system temp directory); the
        # summary goes into the JSON line
        out_dir = os.environ.get("NBKDT_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            # the timed region starts once sampling is live (nvidia-smi takes a moment to
            # start), so a short region still falls between samples 20 ms apart
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        # replicas only: the process group carries the barrier and the max over ranks
        backend = os.environ.get("NBKDT_DIST_BACKEND") or (
            "nccl" if torch.cuda.is_available() else "gloo")
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- workloads
def fof_inputs():
    from nbodylib_gb300 import synthetic as syn
    pos, mass = syn.clustered_box(N_FOF, BOX, seed=2)
    return pos, mass, syn.linking_length(N_FOF, BOX)


def fof_config(ll, groups, world):
    """The workload description both arms print (identical keys and values)."""
    return {"workload": "FOF, 2^20 clustered particles, periodic L=100, ll=0.2 mean "
                        "spacing, minnum 20; step = tree build (b=16) + FOF",
            "n": N_FOF, "bucket": BUCKET, "minnum": MINNUM, "linking_length": ll,
            "groups": int(groups), "l2": "flushed (512 MB write) before every timed step",
            "parallelism": f"replicas x{world}"}


def write_components(comps):
    """Write the full per-workload record to a JSON file and return its path; the stdout
    line keeps only the summary (metric_parts). NBKDT_BENCH_DETAIL names the file; the
    default is bench_components.json in the system temp directory."""
    path = os.environ.get("NBKDT_BENCH_DETAIL") or os.path.join(tempfile.gettempdir(),
                                                                "bench_components.json")
    try:
        d = os.path.dirname(path)
        if d:
            os.makedirs(d, exist_ok=True)
        with open(path, "w") as f:
            json.dump(comps, f, indent=1)
    except OSError as e:
        log(f"bench: could not write {path}: {e}")
        return None
    return path


def metric_parts(fof_value, comps):
    """The three parts of the metric, short enough for one stdout line: FOF particles/s
    (the headline value), kNN-density queries/s with the FP64 roofline fraction of the
    density kernel, the batched path against the per-tree loop, and the adjoint cost."""
    def g(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r(x, nd=4):
        return None if x is None else float(f"{x:.{nd}g}")

    knn = {}
    for name in ("uniform_32768_periodic_k32", "clustered_2pow20_k32"):
        c = comps.get(name, {})
        knn[name] = {"density_kernel_queries_per_s": r(c.get("density_queries_per_s")),
                     "step_queries_per_s": r(c.get("queries_per_s_step")),
                     "fp64_frac": r(g(c, "roofline_fp64", "frac"), 3),
                     "cpu_findnearest_queries_per_s": r(g(c, "cpu", "findnearest_queries_per_s"))}
    c3 = comps.get("clustered_256cubed_k64_density_veldensity", {})
    n3 = c3.get("n", 1 << 24)
    knn["clustered_256cubed_k64"] = {
        "density_kernel_queries_per_s": r(n3 / (c3["density_kernel_ms"] / 1e3))
        if c3.get("density_kernel_ms") else None,
        "veldensity_kernel_queries_per_s": r(n3 / (c3["veldensity_kernel_ms"] / 1e3))
        if c3.get("veldensity_kernel_ms") else None,
        "fp64_frac": r(g(c3, "roofline_fp64_density", "frac"), 3),
        "cpu_density_queries_per_s": r(g(c3, "cpu", "density_queries_per_s"))}
    b = comps.get("batched_20000_groups_k32", {})
    at = b.get("autotuned", {})
    batched = {"particles": b.get("particles"),
               "build_plus_search_speedup": r(g(b, "build_plus_search", "speedup"), 4),
               "search_only_speedup": r(g(b, "search_only", "speedup"), 4),
               "batched_graph_ms": r(g(b, "search_only", "batched_graph_ms")),
               "pertree_loop_ms": r(g(b, "build_plus_search", "pertree_loop_ms")),
               "autotuned": {k: at.get(k) for k in ("bucket", "query_bucket",
                                                   "warp_per_query", "batched_graph_ms")},
               "queries_per_s": r(b.get("batched_queries_per_s"))}
    a = comps.get("adjoint_clustered_2pow20_k32", {})
    return {"fof_particles_per_s": r(fof_value),
            "knn_density": knn,
            "batched_vs_pertree": batched,
            "adjoint_backward_over_forward": r(a.get("backward_over_forward"), 3),
            "fp64_peak_gflops_measured": r(comps.get("fp64_peak_gflops_measured"))}


def run_gpu(args, world, rank, local):
    import torch

    from nbodylib_gb300 import KDTree, _build, _capi
    _build.build()
    lib = _capi.load()
    torch.cuda.set_device(local)
    pos, mass, ll = fof_inputs()
    per = [BOX] * 3
    dpos = torch.from_numpy(pos).cuda()
    dmass = torch.from_numpy(mass).cuda()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def step_device():
        t = KDTree(dpos, None, dmass, BUCKET, kerntype=0, period=per, device=True)
        g, ng = t.FOF(ll, MINNUM)
        t.close()
        return ng

    for _ in range(args.warmup):
        ng = step_device()
    torch.cuda.synchronize()
    lib.nbk_trace_reset()
    lib.nbk_trace_enable(1)
    l0 = lib.nbk_launch_count()
    times = []
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            ng = step_device()
            e.record()
            times.append((s, e))
        torch.cuda.synchronize()
    barrier(world)
    launches = (lib.nbk_launch_count() - l0) // max(args.steps, 1)
    lib.nbk_trace_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    lib.nbk_trace_json(buf, len(buf))
    trace = json.loads(buf.value.decode())
    ms = [s.elapsed_time(e) for s, e in times]
    tot_s = max_over_ranks(sum(ms) / 1e3, world)
    value = world * N_FOF * args.steps / tot_s
    clocks = clk.summary()

    # end to end through the C ABI with host (pinned) buffers
    hpos = torch.from_numpy(pos).pin_memory().numpy()
    hmass = torch.from_numpy(mass).pin_memory().numpy()

    def step_host():
        t = KDTree(hpos, None, hmass, BUCKET, kerntype=0, period=per)
        g, ng = t.FOF(ll, MINNUM)
        t.close()
        return g

    for _ in range(max(3, args.warmup)):
        step_host()
    torch.cuda.synchronize()
    barrier(world)
    e2e_steps = max(args.steps, 20)  # a host-timed step is short; 20 keep the mean stable
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g = step_host()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = world * N_FOF * e2e_steps / e2e_s

    # roofline of the dominant kernel (FOF link): algorithmic bytes = 24 (position) +
    # 4 (group id) per particle
    link = trace.get("fof_link", {"count": 0, "ms": 0.0})
    hbm, which = peaks()
    achieved = None
    if link["count"]:
        per_launch_s = link["ms"] / link["count"] / 1e3
        achieved = 28.0 * N_FOF / per_launch_s / 1e9
    phases = {k: round(v["ms"] / max(v["count"], 1), 4) for k, v in trace.items()}
    comps = components(args, lib)
    detail_path = write_components(comps)
    result = {
        "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded clustered Plummer spheres + background)",
        "config": fof_config(ll, ng, world),
        "e2e": {"value": e2e, "unit": "particles/s", "steps": e2e_steps,
                "h2d_bytes_per_step": int(pos.nbytes + mass.nbytes),
                "d2h_bytes_per_step": int(g.nbytes + 4)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     "traffic": K_LINK_DRAM_BYTES_PER_LAUNCH,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                       "one k_link launch on 2^22 clustered particles at the "
                                       "same density, scaled by particles to 2^20",
                     "kernel": "fof_link (k_link)", "peak_source": which,
                     "algorithmic_bytes_per_launch": 28 * N_FOF},
        "phase_ms_per_step": phases,
        "clocks": clocks,
        "metric_parts": metric_parts(value, comps),
        "components_file": detail_path,
    }
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline_fof(pos, mass, ll)
    return result


def _timed(fn, reps, flush=None, stream=None):
    """Mean CUDA-event milliseconds of fn() over reps calls (L2 flushed before each), the
    events recorded on the stream the work is launched on."""
    import torch
    ms = []
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        torch.cuda.synchronize()
        ms.append(s.elapsed_time(e))
    return float(np.mean(ms))


def _trace(lib, fn):
    """Run fn() with the library's phase trace on; return {phase: ms per call}."""
    lib.nbk_trace_reset()
    lib.nbk_trace_enable(1)
    fn()
    lib.nbk_trace_enable(0)
    buf = ctypes.create_string_buffer(1 << 16)
    lib.nbk_trace_json(buf, len(buf))
    tr = json.loads(buf.value.decode())
    return {k: v["ms"] / max(v["count"], 1) for k, v in tr.items()}


def components(args, lib):
    """The other workloads of the metric: kNN-density on the 32768-particle uniform box and
    on 2^20 clustered particles, kNN density + velocity density on 256^3 clustered
    particles (k=64), the batched persistent density on the power-law group batch against
    the per-tree loop, and the density adjoint against its forward."""
    import torch

    from nbodylib_gb300 import BatchedDensity, KDTree
    from nbodylib_gb300 import synthetic as syn
    fp64 = ctypes.c_double()
    lib.nbk_probe_fp64(ctypes.byref(fp64))
    out = {"fp64_peak_gflops_measured": fp64.value}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    reps = max(3, args.steps)

    def fp64_roofline(flop_per_query, n, ms):
        g = flop_per_query * n / (ms / 1e3) / 1e9
        return {"achieved_gflops": g, "peak_gflops": fp64.value, "frac": g / fp64.value}

    cases = [("uniform_32768_periodic_k32", syn.uniform_box(32768, 1.0, seed=1), [1.0] * 3, 32),
             ("clustered_2pow20_k32", syn.clustered_box(N_FOF, BOX, seed=2), None, 32)]
    for name, (pos, mass), per, k in cases:
        dpos = torch.from_numpy(pos).cuda()
        dmass = torch.from_numpy(mass).cuda()
        n = len(mass)

        def step():
            t = KDTree(dpos, None, dmass, BUCKET, kerntype=0, period=per, device=True)
            t.FindNearest(k)
            rho = t.CalcDensity(k)
            t.sync()
            t.close()
            return rho

        _timed(step, 3)
        step_ms = _timed(step, reps, flush)
        ph = _trace(lib, lambda: [(flush.zero_(), step()) for _ in range(reps)])
        kd_ms = ph.get("knn_density", float("nan"))
        out[name] = {
            "n": n, "k": k, "step_ms": step_ms,
            "queries_per_s_step": n / (step_ms / 1e3),
            "density_kernel_ms": kd_ms,
            "density_queries_per_s": n / (kd_ms / 1e3),
            "fp64_flop_per_query": 20 * k,
            "algorithmic_bytes_per_query": 40,
            # FP64 roofline of the density kernel: 20k algorithmic flop per query over the
            # measured FMA rate of this GPU
            "roofline_fp64": fp64_roofline(20 * k, n, kd_ms),
            "phase_ms": {kk: round(v, 4) for kk, v in ph.items()},
        }
        if not args.no_cpu:
            out[name]["cpu"] = cpu_knn_density(pos, mass, per, k, full_density=n <= 65536)
        del dpos, dmass

    # 256^3 clustered particles in L=250 with velocities: CalcDensity(64), then
    # CalcVelDensity(64, 64) on the same tree
    n3 = 1 << 24
    pos, mass, vel = syn.clustered_box(n3, 250.0, seed=3, velocities=True)
    dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
    del pos, mass, vel

    def step3():
        t = KDTree(dpos, dvel, dmass, BUCKET, kerntype=0, device=True)
        t.CalcDensity(64)
        t.CalcVelDensity(64, 64)
        t.sync()
        t.close()

    _timed(step3, 1)
    ms3 = _timed(step3, 2, flush)
    ph3 = _trace(lib, step3)
    out["clustered_256cubed_k64_density_veldensity"] = {
        "n": n3, "k": 64, "step_ms": ms3, "particles_per_s_step": n3 / (ms3 / 1e3),
        "density_kernel_ms": ph3.get("knn_density"),
        "veldensity_kernel_ms": ph3.get("knn_veldensity"),
        # 20k flop for the physical density; the velocity density adds 8 per neighbour
        # for |dv| and 12 for the kernel
        "roofline_fp64_density": fp64_roofline(20 * 64, n3, ph3.get("knn_density", float("nan"))),
        "phase_ms": {kk: round(v, 4) for kk, v in ph3.items()},
    }
    if not args.no_cpu:
        # the reference's CalcDensity / CalcVelDensity are serial loops over particles: the
        # CPU figure is their per-particle forms on 2000 sampled particles of the full tree
        import oracle
        oracle.build(ref=False)
        threads = os.cpu_count() or 1
        pos, mass, vel = syn.clustered_box(n3, 250.0, seed=3, velocities=True)
        t0 = time.perf_counter()
        o = oracle.OracleTree(pos, vel, mass, BUCKET, 0, 0, 1000, None, backend="port",
                              nthreads=threads)
        tb = time.perf_counter() - t0
        ids = np.random.default_rng(3).choice(n3, 2000, replace=False)
        t0 = time.perf_counter()
        for i in ids:
            o.density_particle(int(i), 64)
        td = time.perf_counter() - t0
        t0 = time.perf_counter()
        for i in ids:
            o.veldensity_particle(int(i), 64, 64)
        tv = time.perf_counter() - t0
        o.close()
        del pos, mass, vel
        out["clustered_256cubed_k64_density_veldensity"]["cpu"] = {
            "kind": "port", "cores": threads, "build_s": tb,
            "density_queries_per_s": len(ids) / td, "veldensity_queries_per_s": len(ids) / tv,
            "sample": "tree build with all OpenMP threads; CalcDensityParticle(64) and "
                      "CalcVelDensityParticle(64, 64) at 2000 random particles, serial"}
    del dpos, dmass, dvel
    torch.cuda.empty_cache()

    # batched persistent density against the plain per-tree loop on the power-law group
    # batch: build + search (a new batch of groups each time, as a halo finder sees them)
    # and search alone (graph replay against one launch per group over the same forest)
    sizes = syn.group_sizes(20000, 20, 200000, seed=4)
    gp, gv, gm, off = syn.plummer_groups(sizes, seed=4)
    dgp, dgm, doff = (torch.from_numpy(a).cuda() for a in (gp, gm, off))
    st = torch.cuda.Stream()
    rho = torch.empty(len(gm), dtype=torch.float64, device="cuda")

    def batched_build_search():
        B = BatchedDensity(dgp, dgm, doff, bucket_size=BUCKET, device=True)
        B.set_stream(st)
        B.density(32, use_graph=False, out=rho)
        B.close()

    batched_build_search()
    bbs_ms = _timed(batched_build_search, reps, flush, st)
    B = BatchedDensity(dgp, dgm, doff, bucket_size=BUCKET, device=True)
    B.set_stream(st)
    B.density(32, use_graph=True, out=rho)
    B.density_pertree_search(32, out=rho)
    graph_ms = _timed(lambda: B.density(32, use_graph=True, out=rho), reps, flush, st)
    loop_search_ms = _timed(lambda: B.density_pertree_search(32, out=rho), 2, flush, st)
    pertree_ms = _timed(lambda: B.density_pertree(32, out=rho), 1, flush, st)
    B.close()
    Bt = BatchedDensity(dgp, dgm, doff, bucket_size=0, device=True)  # autotuned b, qb, mapping
    bt, qbt, tune = Bt.params()
    wpqt = Bt.query_mapping()
    Bt.set_stream(st)
    Bt.density(32, use_graph=True, out=rho)
    graph_tuned_ms = _timed(lambda: Bt.density(32, use_graph=True, out=rho), reps, flush, st)
    Bt.close()
    out["batched_20000_groups_k32"] = {
        "groups": len(sizes), "particles": int(len(gm)), "k": "min(32, n-1)", "bucket": BUCKET,
        "build_plus_search": {"batched_ms": bbs_ms, "pertree_loop_ms": pertree_ms,
                              "speedup": pertree_ms / bbs_ms},
        "search_only": {"batched_graph_ms": graph_ms, "pertree_loop_ms": loop_search_ms,
                        "speedup": loop_search_ms / graph_ms},
        "autotuned": {"bucket": bt, "query_bucket": qbt, "warp_per_query": wpqt,
                      "batched_graph_ms": graph_tuned_ms,
                      "table": json.loads(tune) if tune else None},
        "batched_queries_per_s": len(gm) / (graph_ms / 1e3),
        "target": "batched >= 5x the per-tree loop",
    }
    if not args.no_cpu:
        out["batched_20000_groups_k32"]["cpu"] = cpu_batched(gp, gm, off)
    del B, Bt, rho, dgp, dgm, doff

    # adjoint: d(sum w log rho)/d(x, m) with frozen neighbour lists against the forward
    pos, mass = syn.clustered_box(N_FOF, BOX, seed=2)
    dpos, dmass = torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda()
    w = torch.from_numpy(np.random.default_rng(5).standard_normal(N_FOF)).cuda()
    t = KDTree(dpos, None, dmass, BUCKET, kerntype=0, device=True)
    t.DensityAdjoint(32, w)
    t.CalcDensity(32)
    t.sync()
    fwd_ms = _timed(lambda: (t.CalcDensity(32), t.sync()), reps, flush)
    adj_ms = _timed(lambda: (t.DensityAdjoint(32, w), t.sync()), reps, flush)
    pha = _trace(lib, lambda: t.DensityAdjoint(32, w))
    t.close()
    bwd = pha.get("adjoint_backward", float("nan"))
    out["adjoint_clustered_2pow20_k32"] = {
        "n": N_FOF, "k": 32, "forward_density_ms": fwd_ms,
        "forward_with_saved_lists_plus_backward_ms": adj_ms,
        "backward_kernel_ms": bwd,
        "backward_over_forward": bwd / fwd_ms,
        "phase_ms": {kk: round(v, 4) for kk, v in pha.items()},
        "target": "backward <= 2x forward",
    }
    del dpos, dmass, w

    # FOFCriterion with the FOF6d comparator on the physical tree of the same particles
    # with velocities: linking length ll in position (search region the same, so every
    # link is found from both ends), 0.2 in velocity
    pos, mass, vel = syn.clustered_box(N_FOF, BOX, seed=2, velocities=True)
    dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
    ll = syn.linking_length(N_FOF, BOX)
    crit = [0, ll * ll, 0, 0, 0, 0, ll * ll, 0.04]

    def crit_step():
        t = KDTree(dpos, dvel, dmass, BUCKET, kerntype=0, period=[BOX] * 3, device=True)
        g, ng = t.FOFCriterion(2, crit, MINNUM)
        t.sync()
        t.close()
        return ng

    ngc = crit_step()
    crit_ms = _timed(crit_step, reps, flush)
    phc = _trace(lib, crit_step)
    out["fof_criterion_fof6d_clustered_2pow20"] = {
        "n": N_FOF, "params": crit, "minnum": MINNUM, "groups": int(ngc),
        "step_build_plus_fofcriterion_ms": crit_ms,
        "particles_per_s_step": N_FOF / (crit_ms / 1e3),
        "phase_ms": {kk: round(v, 4) for kk, v in phc.items()}}
    if not args.no_cpu:
        # the reference's breadth-first FOFCriterion tests every particle within ll of each
        # member (no whole-node shortcut), so the CPU sample is the same recipe at 2^15
        # particles and the same number density
        import oracle
        oracle.build(ref=False)
        threads = os.cpu_count() or 1
        ns = 1 << 15
        bs = BOX * (ns / N_FOF) ** (1.0 / 3.0)
        ps, ms, vs = syn.clustered_box(ns, bs, seed=2, velocities=True)
        lls = syn.linking_length(ns, bs)
        t0 = time.perf_counter()
        o = oracle.OracleTree(ps, vs, ms, BUCKET, 0, 0, 1000, [bs] * 3, backend="port",
                              nthreads=threads)
        o.fof_criterion(2, [0, lls * lls, 0, 0, 0, 0, lls * lls, 0.04], MINNUM, 0)
        dt = time.perf_counter() - t0
        o.close()
        out["fof_criterion_fof6d_clustered_2pow20"]["cpu"] = {
            "particles_per_s": ns / dt, "cores": threads, "kind": "port",
            "sample": "the same recipe at 2^15 particles and the same number density: build "
                      "with all OpenMP threads + serial FOFCriterion"}
    del dpos, dmass, dvel

    # phase-space tree (TreeType TPHS) on the 2^20 clustered particles with velocities:
    # build + CalcDensity(32) with the local metric (the reference's default), and
    # FindNearest(32) with the local metric and with the plain phase distance; every query
    # walks the tree in the reference's order (the local-metric result depends on it)
    pos, mass, vel = syn.clustered_box(N_FOF, BOX, seed=2, velocities=True)
    dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
    from nbodylib_gb300.kdtree import TPHS

    def phase_step():
        t = KDTree(dpos, dvel, dmass, BUCKET, treetype=TPHS, kerntype=0, device=True)
        t.CalcDensity(32)
        t.sync()
        t.close()

    phase_step()
    ph_ms = _timed(phase_step, reps, flush)
    php = _trace(lib, phase_step)
    res = {"n": N_FOF, "k": 32, "step_build_plus_density_ms": ph_ms,
           "particles_per_s_step": N_FOF / (ph_ms / 1e3),
           "phase_ms": {kk: round(v, 4) for kk, v in php.items()}}
    for aniso, tag in ((0, "local_metric"), (-1, "plain")):
        t = KDTree(dpos, dvel, dmass, BUCKET, treetype=TPHS, kerntype=0, aniso=aniso,
                   device=True)
        t.FindNearest(32)
        t.sync()
        knn_ms = _timed(lambda: (t.FindNearest(32), t.sync()), reps, flush)
        res[f"findnearest_{tag}_ms"] = knn_ms
        res[f"findnearest_{tag}_queries_per_s"] = N_FOF / (knn_ms / 1e3)
        t.close()
    if not args.no_cpu:
        import oracle
        oracle.build(ref=False)
        threads = os.cpu_count() or 1
        sub = np.arange(0, N_FOF, 64)
        o = oracle.OracleTree(pos, vel, mass, BUCKET, 3, 0, 1000, None, backend="port",
                              nthreads=threads)
        x = np.concatenate([pos[sub], vel[sub]], 1)
        t0 = time.perf_counter()
        o.knn_coord(x, 32)
        dt = time.perf_counter() - t0
        o.close()
        res["cpu_findnearest_local_metric"] = {
            "queries_per_s": len(sub) / dt, "cores": threads, "kind": "port",
            "sample": f"FindNearest(x) at {len(sub)} particles' own phase-space coordinates "
                      "(every 64th), local metric, OpenMP over queries"}
    out["phase_space_clustered_2pow20_k32"] = res
    del dpos, dmass, dvel
    out.update(components_ball_smooth_fofnn(args, lib, flush, reps))
    return out


def components_ball_smooth_fofnn(args, lib, flush, reps):
    """Ball search, the SPH smoothing family and FOF over neighbour lists, each with the
    C restatement timed beside it:

    * SearchBallPosTagged(i, r^2) for every particle of a 2^20 uniform periodic unit box,
      r such that a ball holds 32 particles on average (CSR output of tree indices);
    * CalcSmoothVel(32) + CalcSmoothVelDisp(32) with the density from CalcDensity(32), on
      the 2^20 clustered particles with velocities;
    * FOFNNCriterion (FOF3d, ll = 0.2 mean spacing, minnum 20) over the same tree's
      FindNearest(16) lists."""
    import torch

    from nbodylib_gb300 import KDTree
    from nbodylib_gb300 import synthetic as syn
    out = {}
    threads = os.cpu_count() or 1
    if not args.no_cpu:
        import oracle
        oracle.build(ref=False)

    nb = N_FOF
    pos, mass = syn.uniform_box(nb, 1.0, seed=7)
    r2 = (3.0 * 32 / (4.0 * np.pi * nb)) ** (2.0 / 3.0)
    dpos, dmass = torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda()
    t = KDTree(dpos, None, dmass, BUCKET, kerntype=0, period=[1.0] * 3, device=True)
    tgt = torch.arange(nb, dtype=torch.int32, device="cuda")
    offs, _ = t.SearchBallPosTagged(tgt, r2)
    t.sync()
    pairs = int(offs[-1].item())
    ball_ms = _timed(lambda: (t.SearchBallPosTagged(tgt, r2), t.sync()), reps, flush)
    t.close()
    res = {"n": nb, "fdist2": r2, "found": pairs, "mean_per_ball": pairs / nb,
           "ms": ball_ms, "queries_per_s": nb / (ball_ms / 1e3),
           "found_per_s": pairs / (ball_ms / 1e3),
           "note": "count pass + fill pass through the public call, output allocated per call"}
    if not args.no_cpu:
        o = oracle.OracleTree(pos, None, mass, BUCKET, 0, 0, 1000, [1.0] * 3, backend="port",
                              nthreads=threads)
        sub = range(0, nb, 64)
        t0 = time.perf_counter()
        for i in sub:
            o.ball_tagged(i, r2)
        dt = time.perf_counter() - t0
        o.close()
        res["cpu"] = {"kind": "port", "cores": 1, "queries_per_s": len(sub) / dt,
                      "sample": f"SearchBallPosTagged at every 64th particle ({len(sub)}), "
                                "serial calls"}
    out["ball_uniform_2pow20_periodic_32_per_ball"] = res
    del dpos, dmass, tgt

    pos, mass, vel = syn.clustered_box(N_FOF, BOX, seed=2, velocities=True)
    dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
    t = KDTree(dpos, dvel, dmass, BUCKET, kerntype=0, device=True)
    rho = t.CalcDensity(32)

    def smooth():
        sv = t.CalcSmoothVel(32, rho)
        t.CalcSmoothVelDisp(sv, 32, rho)
        t.sync()

    smooth()
    sm_ms = _timed(smooth, reps, flush)
    phs = _trace(lib, smooth)
    res = {"n": N_FOF, "k": 32, "smoothvel_plus_disp_ms": sm_ms,
           "particles_per_s": N_FOF / (sm_ms / 1e3),
           "phase_ms": {kk: round(v, 4) for kk, v in phs.items()}}
    ll = syn.linking_length(N_FOF, BOX)
    params = [0, 0, 0, 0, 0, 0, ll * ll, 0]
    nn16, _ = t.FindNearest(16)
    _, ngn = t.FOFNNCriterion(0, params, nn16, MINNUM)
    t.sync()
    fnn_ms = _timed(lambda: (t.FOFNNCriterion(0, params, nn16, MINNUM), t.sync()), reps, flush)
    resf = {"n": N_FOF, "numnn": 16, "params": params, "minnum": MINNUM, "groups": int(ngn),
            "fofnn_ms": fnn_ms, "particles_per_s": N_FOF / (fnn_ms / 1e3),
            "note": "the lists come from FindNearest(16) on the same tree, outside the timing"}
    rho_h = rho.cpu().numpy()
    t.close()
    if not args.no_cpu:
        o = oracle.OracleTree(pos, vel, mass, BUCKET, 0, 0, 1000, None, backend="port",
                              nthreads=threads)
        t0 = time.perf_counter()
        sv = o.smooth_vel_moments(0, 32, rho=rho_h)
        o.smooth_vel_moments(1, 32, rho=rho_h, smvel=sv)
        dt = time.perf_counter() - t0
        res["cpu"] = {"kind": "port", "cores": 1, "particles_per_s": N_FOF / dt,
                      "sample": "the full CalcSmoothVel(32) + CalcSmoothVelDisp(32) with the "
                                "given density, serial as the reference ships them"}
        pn, _ = o.tree_knn(16)
        t0 = time.perf_counter()
        o.fof_nn(0, params, pn, MINNUM)
        dt = time.perf_counter() - t0
        o.close()
        resf["cpu"] = {"kind": "port", "cores": 1, "particles_per_s": N_FOF / dt,
                       "sample": "the full FOFNNCriterion over the same lists, serial as shipped"}
    out["smoothvel_veldisp_clustered_2pow20_k32"] = res
    out["fofnn_fof3d_clustered_2pow20_k16"] = resf
    del dpos, dmass, dvel, rho
    torch.cuda.empty_cache()
    return out


def cpu_knn_density(pos, mass, per, k, full_density):
    """The C restatement on the host cores for a kNN-density component: tree build and
    FindNearest(k) for every particle with all OpenMP threads (as the reference's test
    loops them), and CalcDensity(k), serial as the reference ships it, where the set is
    small enough to finish in a second or two."""
    import oracle
    oracle.build(ref=False)
    threads = os.cpu_count() or 1
    n = len(mass)
    t0 = time.perf_counter()
    o = oracle.OracleTree(pos, None, mass, BUCKET, 0, 0, 1000, per, backend="port",
                          nthreads=threads)
    t1 = time.perf_counter()
    o.knn(k)
    t2 = time.perf_counter()
    res = {"kind": "port", "cores": threads, "build_s": t1 - t0,
           "findnearest_queries_per_s": n / (t2 - t1)}
    if full_density:
        o.density(k)
        t3 = time.perf_counter()
        res["density_serial_queries_per_s"] = n / (t3 - t2)
        res["step_queries_per_s"] = n / (t3 - t0 - (t2 - t1))
    o.close()
    return res


def cpu_batched(gp, gm, off, sample=2000):
    """The per-group loop of the reference's pattern (one KDTree + CalcDensity(min(32,
    n-1)) per group) on the C restatement, serial, over every 10th of the first
    10*sample groups."""
    import oracle
    oracle.build(ref=False)
    t0 = time.perf_counter()
    parts = 0
    for g in range(0, min(10 * sample, len(off) - 1), 10):
        a, b = int(off[g]), int(off[g + 1])
        if b - a < 2:
            continue
        o = oracle.OracleTree(gp[a:b], None, gm[a:b], BUCKET, 0, 0, 1000, None, backend="port",
                              nthreads=1)
        o.density(min(32, b - a - 1))
        o.close()
        parts += b - a
    dt = time.perf_counter() - t0
    return {"kind": "port", "cores": 1, "particles_per_s": parts / dt,
            "sample": f"every 10th of the first {10 * sample} groups ({parts} particles), "
                      "build + density per group, one core"}


def cpu_baseline_fof(pos, mass, ll):
    import oracle
    oracle.build(ref=False)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    reps = 0
    while reps < 2:
        o = oracle.OracleTree(pos, None, mass, BUCKET, 0, 0, 1000, [BOX] * 3, backend="port",
                              nthreads=threads)
        o.fof(ll, MINNUM)
        o.close()
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return {"value": N_FOF / dt, "unit": "particles/s", "cores": threads, "kind": "port",
            "sample": f"{reps} full steps (tree build with {threads} OpenMP threads + serial "
                      "FOF, as the reference ships them) on the 2^20 FOF workload"}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    import oracle
    oracle.build(ref=False)
    pos, mass, ll = fof_inputs()
    threads = os.cpu_count() or 1
    # the host caches are flushed before every timed step, as the GPU arm flushes L2
    flush = np.zeros(512 << 20, dtype=np.uint8)

    def step():
        o = oracle.OracleTree(pos, None, mass, BUCKET, 0, 0, 1000, [BOX] * 3, backend="port",
                              nthreads=threads)
        _, ng = o.fof(ll, MINNUM)
        o.close()
        return ng

    ng = 0
    for _ in range(args.warmup):
        ng = step()
    steps = max(1, args.steps)
    dt = 0.0
    for _ in range(steps):
        flush[::64] += 1
        t0 = time.perf_counter()
        ng = step()
        dt += time.perf_counter() - t0
    dt /= steps
    v = N_FOF / dt
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "particles/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded clustered Plummer spheres + background)",
            "config": fof_config(ll, ng, world),
            "cpu_baseline": {"value": v, "unit": "particles/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} full steps on the host cores (build with "
                                       f"{threads} OpenMP threads, FOF serial as shipped)"},
            "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def profile_case(args):
    """A small case of one kernel family, device-resident, for ncu captures: the FOF step
    (build + FOF), the kNN-density step, the phase-space density step (build + CalcDensity
    with the local metric), the FOFCriterion FOF6d step or CalcSmoothVel +
    CalcSmoothVelDisp on args.n clustered particles, SearchBallPosTagged for every particle
    of args.n uniform ones, or the batched density on a power-law group batch of about
    args.n particles."""
    import torch

    from nbodylib_gb300 import BatchedDensity, KDTree, _build
    from nbodylib_gb300 import synthetic as syn
    _build.build()
    torch.cuda.set_device(0)
    n = args.n
    box = BOX * (n / N_FOF) ** (1.0 / 3.0)  # keep the FOF workload's number density
    pos, mass = syn.clustered_box(n, box, seed=2)
    dpos, dmass = torch.from_numpy(pos).cuda(), torch.from_numpy(mass).cuda()
    if args.profile == "batch":
        sizes = syn.group_sizes(20000, 20, 200000, seed=4)
        sizes = sizes[np.cumsum(sizes) <= n]
        gp, gv, gm, off = syn.plummer_groups(sizes, seed=4)
        B = BatchedDensity(torch.from_numpy(gp).cuda(), torch.from_numpy(gm).cuda(),
                           torch.from_numpy(off).cuda(), bucket_size=16, device=True)
        out = torch.empty(len(gm), dtype=torch.float64, device="cuda")
        for _ in range(args.steps):
            B.density(32, use_graph=True, out=out)
        torch.cuda.synchronize()
        return
    if args.profile == "phase":
        from nbodylib_gb300.kdtree import TPHS
        pos, mass, vel = syn.clustered_box(n, box, seed=2, velocities=True)
        dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
        for _ in range(args.steps):
            t = KDTree(dpos, dvel, dmass, BUCKET, treetype=TPHS, kerntype=0, device=True)
            t.CalcDensity(32)
            t.sync()
            t.close()
        torch.cuda.synchronize()
        return
    if args.profile == "smooth":
        pos, mass, vel = syn.clustered_box(n, box, seed=2, velocities=True)
        dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
        t = KDTree(dpos, dvel, dmass, BUCKET, kerntype=0, device=True)
        rho = t.CalcDensity(32)
        for _ in range(args.steps):
            sv = t.CalcSmoothVel(32, rho)
            t.CalcSmoothVelDisp(sv, 32, rho)
        t.sync()
        t.close()
        torch.cuda.synchronize()
        return
    if args.profile == "ball":
        # uniform periodic unit box, 32 particles per ball on average
        upos, umass = syn.uniform_box(n, 1.0, seed=7)
        r2 = (3.0 * 32 / (4.0 * np.pi * n)) ** (2.0 / 3.0)
        t = KDTree(torch.from_numpy(upos).cuda(), None, torch.from_numpy(umass).cuda(), BUCKET,
                   kerntype=0, period=[1.0] * 3, device=True)
        tgt = torch.arange(n, dtype=torch.int32, device="cuda")
        for _ in range(args.steps):
            t.SearchBallPosTagged(tgt, r2)
        t.sync()
        t.close()
        torch.cuda.synchronize()
        return
    if args.profile == "crit6":
        pos, mass, vel = syn.clustered_box(n, box, seed=2, velocities=True)
        dpos, dmass, dvel = (torch.from_numpy(a).cuda() for a in (pos, mass, vel))
        ll = syn.linking_length(n, box)
        crit = [0, ll * ll, 0, 0, 0, 0, ll * ll, 0.04]
        for _ in range(args.steps):
            t = KDTree(dpos, dvel, dmass, BUCKET, kerntype=0, period=[box] * 3, device=True)
            t.FOFCriterion(2, crit, MINNUM)
            t.sync()
            t.close()
        torch.cuda.synchronize()
        return
    for _ in range(args.steps):
        per = [box] * 3 if args.profile == "fof" else None
        t = KDTree(dpos, None, dmass, BUCKET, kerntype=0, period=per, device=True)
        if args.profile == "fof":
            t.FOF(syn.linking_length(n, box), MINNUM)
        elif args.profile == "knn":
            t.CalcDensity(32)
        elif args.profile == "adjoint":
            w = torch.ones(n, dtype=torch.float64, device="cuda")
            t.DensityAdjoint(32, w)
        t.sync()
        t.close()
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", choices=["fof", "knn", "build", "batch", "adjoint", "phase",
                                          "crit6", "smooth", "ball"],
                    help="run only `steps` steps of one small case (for ncu), print nothing")
    ap.add_argument("--n", type=int, default=1 << 18, help="particles for --profile")
    args = ap.parse_args()
    if args.profile:
        profile_case(args)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        # only rank 0 times the CPU path; no process group is needed
        world = int(os.environ.get("WORLD_SIZE", "1"))
        res = run_reference(args, world, int(os.environ.get("RANK", "0")))
        if res is not None:
            print(json.dumps(res), flush=True)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        res = run_reference(args, world, rank)
    else:
        res = run_gpu(args, world, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
