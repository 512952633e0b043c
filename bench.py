"""Benchmark of the GB300 Morton location-code tree.

Headline workload (one step = one OctreePoint Create): 16,000,000 FP64 points (70% uniform in
[0,1]^3, 30% on a noisy sphere shell r=0.4, sd 0.005, seeded), max depth 10, max 20 entities per
node, space = the points' bounding box. value = M entities/s over the timed steps, device-resident
input, CUDA events on the build stream; e2e = the same Create through the C-ABI from pinned host
memory (H2D copy, build, status read-back inside the timed region).

Secondary lines (under "queries"): the 1M-point / 10k range / 10k kNN(k=8) workload, batched kNN
with k in 1..64 on the 16M tree, and 4M-box self collision; each query kernel variant is timed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--no-queries]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_POINTS = 16_000_000
MAX_DEPTH = 10
MAX_ELEM = 20
METRIC = "M entities/s build (OctreePoint Create, 16M FP64 points, depth 10, max 20 per node)"
# single-thread Create time of the oracle port over that of the reference itself on the same 1M
# and 2M shell points (x86 container, both built with g++ -O2): the port is this much slower, so a
# CPU figure of kind "port" understates the reference's speed by about this factor
PORT_VS_REFERENCE = {"1M": 1.39, "2M": 1.27}
# mean dram__bytes_read.sum + dram__bytes_write.sum of the four radix passes of this build (one ncu capture)
SORT_PASS_DRAM_BYTES = 191.7e6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def shell_points(n, seed):
    """70% uniform in [0,1]^3, 30% on a sphere shell r=0.4 (radius N(0.4, 0.005)) around the centre."""
    rng = np.random.default_rng(seed)
    n_shell = int(n * 0.3)
    pts = np.empty((n, 3), np.float64)
    pts[: n - n_shell] = rng.random((n - n_shell, 3))
    d = rng.normal(size=(n_shell, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.normal(0.4, 0.005, (n_shell, 1))
    pts[n - n_shell :] = 0.5 + d * r
    return pts[rng.permutation(n)]


def c1_workload(n_ranges=10_000, n_knn=10_000):
    """The 1M-point query workload: 1,000,000 FP64 points uniform in [0,100)^3 (seed 101); range
    boxes with centres uniform in the domain (seed 102) and edge lengths uniform in [0.5, 5] per
    axis drawn from their own stream (seed 105), so size and position are independent; kNN query
    points uniform in the domain (seed 103). Returns (points, ranges (n, 6), knn points (n, 3))."""
    pts = np.random.default_rng(101).random((1_000_000, 3)) * 100
    c = np.random.default_rng(102).random((10_000, 3)) * 100
    e = np.random.default_rng(105).uniform(0.5, 5, (10_000, 3))
    ranges = np.concatenate([c - e / 2, c + e / 2], 1)[:n_ranges]
    q = (np.random.default_rng(103).random((10_000, 3)) * 100)[:n_knn]
    return pts, ranges, q


class ClockSampler:
    """SM clock and clock-event reasons of this process's GPU, polled every millisecond through NVML
    (the driver's libnvidia-ml, read-only queries) while running; nvidia-smi every 200 ms if NVML
    cannot be loaded."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.samples = []  # (sm MHz, max sm MHz, reason bits)
        self.stop = threading.Event()
        self.nvml = None

    def _nvml_handle(self):
        import ctypes

        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        uuid = None
        try:
            import torch

            u = getattr(torch.cuda.get_device_properties(self.index), "uuid", None)
            uuid = ("GPU-" + str(u)) if u is not None else None
        except Exception:
            uuid = None
        if not (uuid and lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h)) == 0):
            if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
                return None
        self.nvml = lib
        return h

    def _poll(self, h):
        import ctypes

        lib = self.nvml
        reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        sm, bits = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0 and reasons_fn(h, ctypes.byref(bits)) == 0:
                self.samples.append((sm.value, mx.value, bits.value))
            self.stop.wait(0.001)

    def __enter__(self):
        try:
            h = self._nvml_handle()
        except Exception:
            h = None
        if h is not None:
            self.t = threading.Thread(target=self._poll, args=(h,), daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self.stop.set()
        if self.nvml is not None:
            self.t.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.samples:
            reasons = sorted({nm for _, _, b in self.samples for bit, nm in self.REASONS.items() if b & bit})
            return {
                "sm_mhz": statistics.median(s for s, _, _ in self.samples),
                "sm_max_mhz": max(m for _, m, _ in self.samples),
                "reasons": reasons,
                "samples": len(self.samples),
                "source": "nvml 1 ms",
            }
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi 200 ms"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(values, world):
    """Element-wise maximum over the ranks (replicas: the slowest rank sets the time)."""
    if world == 1:
        return values
    import torch
    import torch.distributed as dist

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_throughput(units_per_rank, ms_max, world):
    """Whole-job throughput of independent replicas: all ranks' units over the slowest rank's time."""
    return world * units_per_rank / (ms_max / 1e3)


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------- CPU baselines
def oracle_lib():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _oracle_lib import OracleLib, ORACLE_SO, REF_SO

    if os.path.exists(REF_SO):
        return OracleLib(REF_SO), "reference"
    return OracleLib(ORACLE_SO), "port"


def cpu_threads(lib):
    """Host threads of the timed CPU Create: every core for the oracle port, whose location transform
    and sort run on workers as the reference's ParExec steps do; 1 for the reference harness built
    here (its std::execution::par runs sequentially without a parallel backend)."""
    if not hasattr(lib.lib, "oro_time_create_points_par"):
        return 1
    return os.cpu_count() or 1


def time_cpu_create(lib, pts, reps, threads):
    """Seconds of `reps` CPU Creates of `pts` on `threads` workers."""
    import ctypes

    p = np.ascontiguousarray(pts)
    ptr = p.ctypes.data_as(ctypes.c_void_p)
    if threads > 1:
        return lib.lib.oro_time_create_points_par(ptr, p.shape[0], MAX_DEPTH, MAX_ELEM, reps, threads)
    return lib.lib.oro_time_create_points(ptr, p.shape[0], MAX_DEPTH, MAX_ELEM, reps)


def cpu_build_rate(pts, reps):
    """(M entities/s, kind, threads) of the CPU Create on `pts` (oracle port, or the reference where it
    was built), on every host thread it can use."""
    lib, kind = oracle_lib()
    threads = cpu_threads(lib)
    secs = time_cpu_create(lib, pts, reps, threads)
    return len(pts) * reps / secs / 1e6, kind, threads


def headline_config(nodes, world):
    """The `config` object of the headline line, the same for the GPU and the reference arm."""
    return {
        "workload": "OctreePoint Create, 16M FP64 points (70% uniform, 30% noisy shell r=0.4), bounding box of the data",
        "max_depth": MAX_DEPTH,
        "max_elements": MAX_ELEM,
        "nodes": nodes,
        "l2": "inputs (384 MB of points) larger than L2 (129 MB); no flush",
        "parallelism": f"replicas x{world}",
    }


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    # the whole 16M-point workload every step, as the GPU arm builds it
    pts = shell_points(N_POINTS, 301)
    lib, kind = oracle_lib()
    threads = cpu_threads(lib)
    # the first warm-up Create also gives the node count of the workload's tree
    nodes = int(lib.create(pts, 0, MAX_DEPTH, None, MAX_ELEM, threads=threads).node_count)
    for _ in range(max(0, args.warmup - 1)):
        time_cpu_create(lib, pts, 1, threads)
    times = []
    for _ in range(args.steps):
        times.append(time_cpu_create(lib, pts, 1, threads))
    ms = statistics.mean(times) * 1e3
    value = N_POINTS / (ms / 1e3) / 1e6
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "M entities/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": headline_config(nodes, world),
        "cpu_baseline": {
            "value": value,
            "unit": "M entities/s",
            "cores": threads,
            "kind": kind,
            "sample": f"all {N_POINTS} points every step (the GPU arm's workload), Create with the location transform and sort "
            f"on {threads} threads, BuildSubtree sequential as in the reference",
            "port_vs_reference_time": PORT_VS_REFERENCE if kind == "port" else None,
        },
        "e2e": {"value": value, "unit": "M entities/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------- GPU arm
def phase_bytes(n, key_bytes, passes):
    """Algorithmic HBM bytes per build phase (points, FP64: 24 B per point)."""
    w = 24
    sort = n * key_bytes + n * (key_bytes + 4) + (passes - 1) * 2 * n * (key_bytes + 4)
    return {
        "bbox": n * w,
        "codegen": n * w + n * key_bytes,
        "sort": sort,
        "gather": n * (4 + w + w),
    }


def run_gpu(args):
    import torch

    import octree_gb300 as otg

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()

    pts_h = shell_points(N_POINTS, 301 + rank)
    pts_d = torch.as_tensor(pts_h, device="cuda")
    tree = otg.Tree("points")
    otg.profile_enable(True)

    for _ in range(args.warmup):
        tree.create(pts_d, max_depth=MAX_DEPTH, max_elements=MAX_ELEM, stream=stream)
    tree.sync(stream)
    torch.cuda.synchronize()
    barrier(world)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    phases = {}
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(world)
        for i in range(args.steps):
            ev[i][0].record(stream)
            tree.create(pts_d, max_depth=MAX_DEPTH, max_elements=MAX_ELEM, stream=stream)
            ev[i][1].record(stream)
            ev[i][1].synchronize()
            for name, ms in otg.profile_phases():
                phases.setdefault(name, []).append(ms)
        torch.cuda.synchronize()
        barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tree.sync(stream)
    info = tree.info()
    ms = reduce_max([statistics.mean(step_ms)], world)[0]
    value = replica_throughput(N_POINTS, ms, world) / 1e6

    # e2e through the C-ABI: pinned host input, copies inside the timed region
    pinned = torch.from_numpy(pts_h).pin_memory()
    host_tree = otg.Tree("points")
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_tree.create(pinned.numpy(), max_depth=MAX_DEPTH, max_elements=MAX_ELEM, stream=stream)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_ms_v = reduce_max([statistics.mean(e2e_ms)], world)[0]
    e2e_value = replica_throughput(N_POINTS, e2e_ms_v, world) / 1e6
    otg.profile_enable(False)

    # roofline of the dominant phase
    key_bytes = 4 if 3 * MAX_DEPTH + 1 <= 32 else 8
    passes = (3 * MAX_DEPTH + 1 + 7) // 8
    pb = phase_bytes(N_POINTS, key_bytes, passes)
    mean_phase = {k: statistics.mean(v) for k, v in phases.items()}
    dom = max((k for k in mean_phase if k in pb), key=lambda k: mean_phase[k])
    launches = passes if dom == "sort" else 1
    per_launch_ms = mean_phase[dom] / launches
    per_launch_bytes = pb[dom] / launches
    hbm, peak_kind = peaks()
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
    roofline = {
        "bound": "hbm",
        "kernel": dom,
        "achieved": achieved,
        "peak": hbm,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": achieved / hbm,
        # DRAM bytes per sort pass of this workload from one ncu capture
        # (profiles/onesweep_pass_kernel_16m_traffic.md); not measurable inside a timed run
        "traffic": SORT_PASS_DRAM_BYTES if dom == "sort" else None,
        "traffic_source": "profiles/onesweep_pass_kernel_16m_traffic.md" if dom == "sort" else None,
        "algorithmic_bytes_per_launch": per_launch_bytes,
        "launches_per_step": launches,
    }
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "M entities/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": headline_config(int(info.node_count), world),
        "phases_ms": mean_phase,
        "roofline": roofline,
        "e2e": {"value": e2e_value, "unit": "M entities/s", "h2d_bytes_per_step": N_POINTS * 24, "d2h_bytes_per_step": 4 + 32 * 4},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    # kernel launches per build of this workload (as in the ncu launch list of
    # profiles/build16m_launch_list.md): bbox init, bbox, space setup, raster tables, MinPoint table,
    # codegen, the digit bases, the radix passes, gather, root init, the root's classify launch and a
    # split launch per depth 0..D-1
    line["gpu_launches"] = args.steps * (6 + 1 + passes + 1 + 1 + 1 + MAX_DEPTH)
    if rank == 0 and not args.no_cpu_baseline:
        rate, kind, threads = cpu_build_rate(pts_h, 2)
        line["cpu_baseline"] = {
            "value": rate,
            "unit": "M entities/s",
            "cores": threads,
            "kind": kind,
            "sample": f"all 16M points, 2 Creates, location transform and sort on {threads} threads",
            "port_vs_reference_time": PORT_VS_REFERENCE if kind == "port" else None,
        }
    if not args.no_queries:
        line["static_layout"] = run_static_export(tree, pts_h)
        cpu_results = None
        if rank == 0 and not args.no_cpu_baseline:
            line["cpu_configs"], cpu_results = run_cpu_configs()
        line["queries"] = run_queries(tree, pts_d, stream, cpu_results, pts_h)
        line["many_trees"] = run_many_trees()
        line["two_trees"] = run_two_trees()
        line["insert"] = run_insert(cpu=rank == 0 and not args.no_cpu_baseline)
        line["autotune"] = otg.autotune_entries()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_static_export(tree16, pts16_h, reps=5):
    """Export of the 16M-point tree to the static linear layout (StaticLinearOrthoTreeCore's
    arrays): device time of the export, then with the copy of every array to host memory; for
    scale, the CPU side (the oracle port, or the reference where it was built) building the
    dynamic tree and then the static layout of a 1M sample on one thread. The GPU export of that
    sample is checked against the CPU layout."""
    import ctypes

    import torch

    import octree_gb300 as otg

    lib = otg.library()
    lay = otg.StaticLayout()

    def export():
        otg._check(lib.otg_tree_export_static(tree16.h, ctypes.byref(lay), None))

    s_dev = time_query(export, reps)
    s_host = time_query(lambda: tree16.export_static(), reps)
    out = {
        "tree": "the 16M-point Create above (depth 10, max 20)",
        "dynamic_nodes": int(tree16.node_count),
        "static_nodes": int(lay.node_count),
        "export_ms": s_dev * 1e3,
        "export_plus_host_copy_ms": s_host * 1e3,
        "launches_per_export": 3 * (MAX_DEPTH + 1) + 2,
        "bound": "launch latency: three launches per static level and one readback",
    }
    sample = np.ascontiguousarray(pts16_h[:1_000_000])
    lib_o, kind = oracle_lib()
    t0 = time.perf_counter()
    ref = lib_o.create(sample, 0, MAX_DEPTH, None, MAX_ELEM).static_layout()
    out["cpu_dynamic_then_static_1M_s"] = time.perf_counter() - t0
    out["cpu_kind"] = kind
    ts = otg.Tree("points").create(sample, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
    got = ts.export_static()
    same = all(np.array_equal(got[k], ref[k]) for k in ("child_begins", "segments", "depth", "geometry"))
    if kind == "port":
        same = same and np.array_equal(got["entity_storage"], ref["entity_storage"])
    out["sample_layout_equal_to_cpu"] = bool(same)
    # the reference's binary archive of the sample's Managed static tree, and a tree resumed from it
    t0 = time.perf_counter()
    data = ts.save_static(True)
    out["archive_1M_managed_bytes"] = len(data)
    out["archive_1M_save_ms"] = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    resumed = otg.Tree("points").load_static(data)
    out["archive_1M_resume_ms"] = (time.perf_counter() - t0) * 1e3
    out["archive_1M_round_trip_equal"] = resumed.save_static(True) == data
    torch.cuda.synchronize()
    return out


def run_cpu_configs():
    """The CPU side of each query config, beside the GPU figures: the oracle port (or the reference
    where it was built here) on bounded samples of the same inputs. Trees are built with the
    port's threaded location transform and sort where it has them; queries are split over every
    host core (the ctypes calls run in parallel), as the reference's std::for_each(par) would run
    them. Each entry names its sample."""
    from concurrent.futures import ThreadPoolExecutor

    lib, kind = oracle_lib()
    threads = os.cpu_count() or 1
    build_threads = threads if hasattr(lib.lib, "oro_create_threads") else 1
    pool = ThreadPoolExecutor(threads)

    results = {}

    def par_queries(fn, arrays, keep=None):
        # fn(slice arrays...) for `threads` contiguous slices, concurrently; returns seconds. keep:
        # the name under which the CSR result of all slices, in query order, is kept for the
        # comparison with the GPU lines
        n = len(arrays[0])
        cuts = [n * i // threads for i in range(threads + 1)]
        t0 = time.perf_counter()
        parts = list(pool.map(lambda i: fn(*[a[cuts[i] : cuts[i + 1]] for a in arrays]), range(threads)))
        s = time.perf_counter() - t0
        if keep:
            results[keep] = concat_csr(parts)
        return s

    out = {"kind": kind, "query_threads": threads, "build_threads": build_threads}
    # C1: 1M uniform points (depth 10, max 20); 2000 of the 10k range boxes and 2000 kNN(k=8) queries
    p1, ranges, q = c1_workload(2000, 2000)
    t0 = time.perf_counter()
    t1 = lib.create(p1, 0, 10, None, 20, threads=build_threads)
    out["c1_create_1M_s"] = time.perf_counter() - t0
    s = par_queries(lambda r: t1.range_search(r), [ranges], keep="c1_range")
    out["c1_range_Mq_per_s"] = 2000 / s / 1e6
    s = par_queries(lambda x: t1.knn(x, 8), [q], keep="c1_knn8")
    out["c1_knn8_Mq_per_s"] = 2000 / s / 1e6
    out["c1_sample"] = "2000 of the 10k range boxes, 2000 kNN(k=8) queries"
    del t1
    # C3: the 16M shell points; 2000 of the 1M uneven kNN queries (k in 1..64)
    pts = shell_points(N_POINTS, 301)
    t0 = time.perf_counter()
    t3 = lib.create(pts, 0, MAX_DEPTH, None, MAX_ELEM, threads=build_threads)
    out["c3_create_16M_s"] = time.perf_counter() - t0
    qk = shell_points(1_000_000, 302)[:2000]
    ks = np.random.default_rng(303).integers(1, 65, 1_000_000).astype(np.uint32)[:2000]
    s = par_queries(lambda x, k: t3.knn(x, k), [qk, ks], keep="c3_knn_uneven")
    out["c3_knn_uneven_Mq_per_s"] = 2000 / s / 1e6
    out["c3_sample"] = "2000 of the 1M queries, k in 1..64"
    del t3, pts
    # C2: self-collision of every 8th of the 4M clustered boxes (one sequential call: the
    # reference's parallel CollisionDetection is a different traversal order, same pairs)
    boxes = np.ascontiguousarray(cluster_boxes(4_000_000, 201)[::8])
    tb = lib.create(boxes, 1, 12, None, 32, threads=build_threads)
    t0 = time.perf_counter()
    pairs = tb.collide_self()
    s = time.perf_counter() - t0
    results["c2_collide_self_500k"] = pairs
    out["c2_collide_self_500k_ms"] = s * 1e3
    out["c2_collide_self_500k_Mpairs_per_s"] = len(pairs) / s / 1e6
    out["c2_sample"] = "every 8th of the 4M boxes (500k, one eighth of the density), one thread"
    del tb
    # C4: 16 FP32 box trees drawn as the 4096 are: Create, 256 ranges, 256 rays and one frustum each
    ent, off, qr, rays, planes = many_trees(16, 401)
    t0 = time.perf_counter()
    for t in range(16):
        tt = lib.create(ent[off[t] : off[t + 1]], 1, 0, None, 16, threads=build_threads)
        tt.range_search(qr[256 * t : 256 * (t + 1)], 1)
        tt.ray(rays[256 * t : 256 * (t + 1)])
        tt.frustum(planes[t : t + 1])
    s = time.perf_counter() - t0
    out["c4_trees_per_s"] = 16 / s
    out["c4_sample"] = "16 trees of the same distribution, one after another"
    pool.shutdown()
    return out, results


def concat_csr(parts):
    """One CSR result (offsets, ids[, distances]) from the results of consecutive query slices."""
    offs, ids, dists = [np.zeros(1, np.uint64)], [], []
    base = 0
    for p in parts:
        o = np.asarray(p[0], np.uint64)
        offs.append(o[1:] + np.uint64(base))
        base += int(o[-1])
        ids.append(p[1])
        if len(p) > 2 and p[2] is not None:
            dists.append(p[2])
    out = (np.concatenate(offs), np.concatenate(ids) if ids else np.zeros(0, np.uint32))
    return out + (np.concatenate(dists),) if dists else out


def csr_mismatches(a, b):
    """Queries whose id lists (and distances, where both carry them) differ between two CSR results."""
    oa, ob = np.asarray(a[0], np.int64), np.asarray(b[0], np.int64)
    if len(oa) != len(ob):
        return max(len(oa), len(ob)) - 1
    dist = len(a) > 2 and len(b) > 2 and a[2] is not None and b[2] is not None
    bad = 0
    for qi in range(len(oa) - 1):
        x, y = slice(oa[qi], oa[qi + 1]), slice(ob[qi], ob[qi + 1])
        if not np.array_equal(a[1][x], b[1][y]) or (dist and not np.array_equal(a[2][x], b[2][y])):
            bad += 1
    return bad


def pair_mismatches(a, b):
    """Pairs in one canonically sorted (i < j) pair list and not in the other."""
    ka = np.asarray(a, np.uint64).reshape(-1, 2)
    kb = np.asarray(b, np.uint64).reshape(-1, 2)
    ka = ka[:, 0] << np.uint64(32) | ka[:, 1]
    kb = kb[:, 0] << np.uint64(32) | kb[:, 1]
    return int(len(np.setxor1d(ka, kb)))


def time_query(fn, reps=3):
    import torch

    fn()
    torch.cuda.synchronize()
    t = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        t.append(time.perf_counter() - t0)
    return statistics.median(t)


def cluster_boxes(n, seed):
    """Self-collision workload: centres 50% uniform in [0,1000)^3 and 50% from 64 isotropic Gaussian
    clusters (sigma 10, centres uniform), half-extents lognormal(ln 0.5, 0.6) per axis."""
    rng = np.random.default_rng(seed)
    half = n // 2
    centres = np.empty((n, 3))
    centres[:half] = rng.random((half, 3)) * 1000
    cc = np.random.default_rng(seed + 1).random((64, 3)) * 1000
    pick = rng.integers(0, 64, n - half)
    centres[half:] = cc[pick] + rng.normal(0, 10, (n - half, 3))
    ext = rng.lognormal(np.log(0.5), 0.6, (n, 3))
    return np.concatenate([centres - ext, centres + ext], 1)


def mismatched_queries(a, b):
    """Number of queries whose (id, distance) lists differ between two CSR results."""
    oa, ob = a[0].astype(np.int64), b[0].astype(np.int64)
    if np.array_equal(oa, ob) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]):
        return 0
    bad = 0
    for qi in range(len(oa) - 1):
        x = slice(oa[qi], oa[qi + 1])
        y = slice(ob[qi], ob[qi + 1])
        if not (np.array_equal(a[1][x], b[1][y]) and np.array_equal(a[2][x], b[2][y])):
            bad += 1
    return bad


# bytes the query kernels read per unit of the reference's traversal work (FP64 point trees): a node
# record is its link (uint4) and its box (6 doubles), an entity record one point, an id 4 bytes
NODE_RECORD_BYTES, POINT_RECORD_BYTES, ID_BYTES = 16 + 48, 24, 4


def l2_copy_gbs(reps=50):
    """Read + write GB/s of a device copy whose 2 x 32 MB stay in L2 (the roof of L2-resident query
    working sets; the HBM roof is MEASURED_PEAKS.json's)."""
    import torch

    x = torch.ones(8 << 20, device="cuda")
    y = torch.empty_like(x)
    for _ in range(5):
        y.copy_(x)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(reps):
        y.copy_(x)
    b.record()
    b.synchronize()
    return 2 * x.numel() * 4 * reps / (a.elapsed_time(b) / 1e3) / 1e9


def query_work(p1, ranges, q8, pts16, q16, k16):
    """Per-query work of the reference's traversal on the measured inputs, counted by the oracle
    restatement (node records read, entity records read, ids returned): C1 range and kNN(k=8) on
    the 1M tree (all 10k queries), C3 uneven kNN on the 16M tree (the first 20k of the 1M
    queries). Returns {name: (nodes, entities, ids) per query}."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _oracle_lib import oracle

    threads = os.cpu_count() or 1
    o1 = oracle().create(p1, 0, 10, None, 20, threads=threads)
    out = {}
    for name, fn, nq in (("c1_range", lambda t: t.range_search(ranges), len(ranges)), ("c1_knn8", lambda t: t.knn(q8, 8), len(q8))):
        out[name] = tuple(v / nq for v in o1.work(fn))
    del o1
    o3 = oracle().create(pts16, 0, 10, None, 20, threads=threads)
    out["c3_knn_uneven"] = tuple(v / len(q16) for v in o3.work(lambda t: t.knn(q16, k16)))
    return out


def query_roofline(work, mq_per_s, peak_gbs, bound):
    """roofline object of a query line: algorithmic bytes per query (the reference traversal's
    work x record sizes) x queries/s against the roof of its working set."""
    nodes, ents, ids = work
    per_query = nodes * NODE_RECORD_BYTES + ents * POINT_RECORD_BYTES + ids * ID_BYTES
    achieved = per_query * mq_per_s * 1e6 / 1e9
    return {
        "bound": bound,
        "achieved": achieved,
        "peak": peak_gbs,
        "unit": "GB/s",
        "frac": achieved / peak_gbs,
        "bytes_per_query": per_query,
        "work_per_query": {"node_records": nodes, "entity_records": ents, "ids": ids},
    }


def run_queries(tree16, pts16_d, stream, cpu=None, pts16_h=None):
    """cpu: the CPU results of run_cpu_configs on its samples; each is compared with the GPU's
    result on the same sample (mismatched_ids_vs_cpu: queries, or pairs, that differ).
    pts16_h: the host copy of the 16M points, for the traversal work counts of the rooflines."""
    import torch

    import octree_gb300 as otg

    out = {}
    algos = ((otg.ALGO_PLAIN_FP64, "plain_fp64"), (otg.ALGO_FILTERED, "filtered_fp32"))
    rng = np.random.default_rng(104)
    # 1M uniform points in [0,100]^3, 10k range boxes (edges U[0.5,5]), 10k kNN k=8
    p1, ranges_h, q_h = c1_workload()
    t1 = otg.Tree("points").create(p1, max_depth=10, max_elements=20)
    ranges = torch.as_tensor(ranges_h, device="cuda")
    q = torch.as_tensor(q_h, device="cuda")
    mism = {}
    if cpu:
        mism["c1_range_2000"] = csr_mismatches(t1.range_search(ranges_h[:2000])[:2], cpu["c1_range"])
        mism["c1_knn8_2000"] = csr_mismatches(t1.knn(q_h[:2000], 8), cpu["c1_knn8"])
    s = time_query(lambda: t1.range_search(ranges, algo=otg.ALGO_PLAIN_FP64, raw=True))
    out["range_1M_10k_plain_fp64_Mq_per_s"] = 10_000 / s / 1e6
    s = time_query(lambda: t1.range_search(ranges, raw=True))
    out["range_1M_10k_batched_Mq_per_s"] = 10_000 / s / 1e6
    # 10k PickSearch at points of the tree (each finds its point)
    picks = torch.as_tensor(p1[rng.integers(0, len(p1), 10_000)], device="cuda")
    for algo, name in ((otg.ALGO_PLAIN_FP64, "plain_fp64"), (otg.ALGO_DEFAULT, "batched")):
        s = time_query(lambda: t1.pick_search(picks, algo=algo, raw=True))
        out[f"pick_1M_10k_{name}_Mq_per_s"] = 10_000 / s / 1e6
    for algo, name in algos:
        s = time_query(lambda: t1.knn(q, 8, algo=algo, raw=True))
        out[f"knn8_1M_10k_{name}_Mq_per_s"] = 10_000 / s / 1e6
    # plane queries on the same tree: 10k PlaneSearch at a 0.1 tolerance (about 2k ids each) and 256
    # PlanePositiveSegmentation (about half the points each); planes with uniform normals through the data
    nrm = rng.normal(size=(10_000, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    through = rng.random((10_000, 3)) * 100
    planes = torch.as_tensor(np.concatenate([(nrm * through).sum(1, keepdims=True), nrm], 1), device="cuda")
    plane_sets = {}
    for algo, name in ((otg.ALGO_PLAIN_FP64, "plain_fp64"), (otg.ALGO_DEFAULT, "batched")):
        s = time_query(lambda: t1.plane_search(planes, 0.1, algo=algo, raw=True))
        out[f"plane_search_1M_10k_{name}_Mq_per_s"] = 10_000 / s / 1e6
        s = time_query(lambda: t1.plane_positive_segmentation(planes[:256], algo=algo, raw=True))
        r = t1.plane_positive_segmentation(planes[:256], algo=algo, raw=True)
        out[f"plane_positive_1M_256_{name}_ms"] = s * 1e3
        out[f"plane_positive_1M_256_{name}_Mids_per_s"] = r.sizes()[1] / s / 1e6
        plane_sets[name] = (t1.plane_search(planes, 0.1, algo=algo)[:2], r.to_host()[:2])
    out["plane_results_equal_batched_vs_plain"] = bool(
        all(np.array_equal(a, b) for x, y in zip(plane_sets["plain_fp64"], plane_sets["batched"]) for a, b in zip(x, y))
    )
    # batched uneven kNN on the 16M tree: 1M queries from the same mixture, k in 1..64
    qk = torch.as_tensor(shell_points(1_000_000, 302), device="cuda")
    ks = torch.as_tensor(np.random.default_rng(303).integers(1, 65, 1_000_000).astype(np.int32), device="cuda")
    res = {}
    for algo, name in algos:
        s = time_query(lambda: tree16.knn(qk, ks, algo=algo, raw=True), reps=1 if algo == otg.ALGO_PLAIN_FP64 else 3)
        out[f"knn_uneven_16M_1Mq_{name}_Mq_per_s"] = 1_000_000 / s / 1e6
        res[name] = tree16.knn(qk, ks, algo=algo)
    tests, rechecks = tree16.knn(qk, ks, algo=otg.ALGO_FILTERED, raw=True).stats()
    out["knn_uneven_recheck_fraction"] = rechecks / max(tests, 1)
    out["knn_uneven_mismatched_queries_filtered_vs_plain"] = mismatched_queries(res["plain_fp64"], res["filtered_fp32"])
    if cpu:
        mism["c3_knn_uneven_2000"] = csr_mismatches(tree16.knn(qk[:2000], ks[:2000]), cpu["c3_knn_uneven"])
    out["knn_uneven_speedup_filtered_vs_plain"] = out["knn_uneven_16M_1Mq_filtered_fp32_Mq_per_s"] / out["knn_uneven_16M_1Mq_plain_fp64_Mq_per_s"]
    if pts16_h is not None:
        # rooflines of the query lines: the 1M tree and its points (42 MB) stay in L2; the 16M tree
        # (384 MB of points) does not
        work = query_work(p1, ranges_h, q_h, pts16_h, qk.cpu().numpy()[:20_000], ks.cpu().numpy().astype(np.uint32)[:20_000])
        l2 = l2_copy_gbs()
        hbm, hbm_kind = peaks()
        rl = {}
        for key, wname, peak, bound in (
            ("range_1M_10k_batched", "c1_range", l2, "l2"),
            ("range_1M_10k_plain_fp64", "c1_range", l2, "l2"),
            ("knn8_1M_10k_filtered_fp32", "c1_knn8", l2, "l2"),
            ("knn8_1M_10k_plain_fp64", "c1_knn8", l2, "l2"),
            ("knn_uneven_16M_1Mq_filtered_fp32", "c3_knn_uneven", hbm, "hbm"),
            ("knn_uneven_16M_1Mq_plain_fp64", "c3_knn_uneven", hbm, "hbm"),
        ):
            rl[key] = query_roofline(work[wname], out[key + "_Mq_per_s"], peak, bound)
        out["roofline"] = rl
        out["roofline_peaks"] = {"l2_copy_gbs": l2, "hbm_gbs": hbm, "hbm_kind": hbm_kind, "l2_how": "device copy of 2 x 32 MB kept in L2, 50 reps, CUDA events"}
        out["roofline_work_source"] = "oracle restatement counters of the reference's traversal on the measured queries (C3: the first 20k queries)"
    # self-collision of 4M clustered FP64 boxes, depth 12, max 32 per node
    boxes = torch.as_tensor(cluster_boxes(4_000_000, 201), device="cuda")
    tb = otg.Tree("boxes").create(boxes, max_depth=12, max_elements=32)
    tb.sync()
    pair_lists = {}
    for algo, name in algos:
        s = time_query(lambda: tb.collision_self(algo=algo, raw=True), reps=1 if algo == otg.ALGO_PLAIN_FP64 else 3)
        r = tb.collision_self(algo=algo, raw=True)
        pairs = r.sizes()[1] // 2
        pair_lists[name] = r.to_host()[1]
        out[f"collide_self_4M_{name}_ms"] = s * 1e3
        out[f"collide_self_4M_{name}_Mpairs_per_s"] = pairs / s / 1e6
        if algo == otg.ALGO_FILTERED:
            tests, rechecks = r.stats()
            out["collide_self_4M_recheck_fraction"] = rechecks / max(tests, 1)
    out["collide_self_4M_pairs"] = int(pairs)
    out["collide_self_4M_pair_lists_equal"] = bool(np.array_equal(pair_lists["plain_fp64"], pair_lists["filtered_fp32"]))
    out["collide_self_4M_speedup_filtered_vs_plain"] = out["collide_self_4M_plain_fp64_ms"] / out["collide_self_4M_filtered_fp32_ms"]
    if cpu:
        sub = otg.Tree("boxes").create(np.ascontiguousarray(cluster_boxes(4_000_000, 201)[::8]), max_depth=12, max_elements=32)
        mism["c2_collide_self_500k_pairs"] = pair_mismatches(sub.collision_self(), cpu["c2_collide_self_500k"])
        out["mismatched_ids_vs_cpu"] = mism
        out["mismatched_ids_vs_cpu_samples"] = "the CPU samples of cpu_configs (C1: 2000 ranges, 2000 kNN k=8; C3: 2000 uneven kNN; C2: self-collision of every 8th box), run again on the GPU with the default kernels"
    return out


def many_trees(trees, seed):
    """Many small box trees: sizes lognormal(ln 8000, 1.2) clipped to [1000, 200000]; boxes with
    centres uniform in [0,100)^3 and half-extents uniform in [0.05, 1], drawn in FP64 and stored as
    FP32. Per tree 256 range boxes (centres uniform, edges uniform in [0.5, 5]), 256 rays (origins
    uniform, directions uniform on the sphere, unbounded) and one frustum of 6 axis-aligned planes."""
    rng = np.random.default_rng(seed)
    sizes = np.clip(rng.lognormal(np.log(8000), 1.2, trees), 1000, 200000).astype(np.int64)
    n = int(sizes.sum())
    c = rng.random((n, 3)) * 100
    e = rng.uniform(0.05, 1.0, (n, 3))
    boxes = np.empty((n, 6), np.float32)
    boxes[:, :3] = c - e
    boxes[:, 3:] = c + e
    del c, e
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    qrng = np.random.default_rng(seed + 1)
    nq = trees * 256
    qc = qrng.random((nq, 3)) * 100
    qe = qrng.uniform(0.5, 5, (nq, 3))
    ranges = np.concatenate([qc - qe / 2, qc + qe / 2], 1).astype(np.float32)
    d = qrng.normal(size=(nq, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([qrng.random((nq, 3)) * 100, d], 1).astype(np.float32)
    planes = np.zeros((trees, 6, 4), np.float32)
    lo, hi = qrng.random((trees, 3)) * 40, 60 + qrng.random((trees, 3)) * 40
    for a in range(3):
        planes[:, 2 * a, 0], planes[:, 2 * a, 1 + a] = lo[:, a], 1.0
        planes[:, 2 * a + 1, 0], planes[:, 2 * a + 1, 1 + a] = -hi[:, a], -1.0
    return boxes, off, ranges, rays, planes


def run_many_trees(trees=4096, sample=48):
    """The many-small-trees workload: one forest (one build + three batched query launches for all
    trees) against per-tree Create + queries, on a sample of trees, with the one-query-per-thread
    kernels and with the batched (warp-per-query) kernels."""
    import torch

    import octree_gb300 as otg

    boxes, off, ranges, rays, planes = many_trees(trees, 401)
    qoff = np.arange(trees + 1, dtype=np.uint64) * 256
    foff = np.arange(trees + 1, dtype=np.uint64)
    d_boxes = torch.as_tensor(boxes, device="cuda")
    d_ranges = torch.as_tensor(ranges, device="cuda")
    d_rays = torch.as_tensor(rays, device="cuda")
    d_planes = torch.as_tensor(planes, device="cuda")
    f = otg.Forest("boxes", np.float32)

    def forest_step():
        f.create(d_boxes, off, max_elements=16)
        a = f.range_search(d_ranges, qoff, raw=True)
        b = f.ray_all(d_rays, qoff, raw=True)
        c = f.frustum_culling(d_planes, foff, raw=True)
        return a, b, c

    forest_step()
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        res = forest_step()
    torch.cuda.synchronize()
    step_s = (time.perf_counter() - t0) / reps
    # phases of one step
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f.create(d_boxes, off, max_elements=16)
    f.sync()
    t1 = time.perf_counter()
    f.range_search(d_ranges, qoff, raw=True)
    t2 = time.perf_counter()
    f.ray_all(d_rays, qoff, raw=True)
    t3 = time.perf_counter()
    f.frustum_culling(d_planes, foff, raw=True)
    t4 = time.perf_counter()
    n_ids = [r.sizes()[1] for r in res]
    # the same step recorded as a CUDA graph and replayed
    plan = otg.ForestPlan(otg.Forest("boxes", np.float32), d_boxes, off, max_elements=16, ranges=d_ranges, range_offsets=qoff, rays=d_rays,
                          ray_offsets=qoff, planes=d_planes, frustum_offsets=foff, capacity_factor=1.25)
    plan.run()
    torch.cuda.synchronize()
    g0 = time.perf_counter()
    for _ in range(reps):
        plan.run()
    torch.cuda.synchronize()
    graph_step_s = (time.perf_counter() - g0) / reps
    graph_same = all(
        np.array_equal(plan.result(k)[0], r.to_host()[0]) and np.array_equal(plan.result(k)[1], r.to_host()[1]) for k, r in enumerate(res)
    )
    # per-tree plain launches on a sample of trees
    host = [r.to_host() for r in res]
    idx = np.random.default_rng(7).choice(trees, sample, replace=False)
    mism = 0
    t_plain = 0.0
    for t in idx:
        a, b = int(off[t]), int(off[t + 1])
        q = slice(t * 256, (t + 1) * 256)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        tr = otg.Tree("boxes", np.float32).create(d_boxes[a:b], max_elements=16)
        ra = tr.range_search(d_ranges[q], algo=otg.ALGO_PLAIN_FP64)
        rb = tr.ray_all(d_rays[q], algo=otg.ALGO_PLAIN_FP64)
        rc = tr.frustum_culling(d_planes[t : t + 1], algo=otg.ALGO_PLAIN_FP64)
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - s0
        for got, (fo, fi, fd), nper, qi in ((ra, host[0], 256, t * 256), (rb, host[1], 256, t * 256), (rc, host[2], 1, t)):
            o0, o1 = int(fo[qi]), int(fo[qi + nper])
            same = np.array_equal(got[1], fi[o0:o1]) and np.array_equal(np.diff(got[0].astype(np.int64)), np.diff(fo[qi : qi + nper + 1].astype(np.int64)))
            mism += 0 if same else 1
    per_tree_s = t_plain / sample
    # the same per-tree calls with the batched (warp-per-query) kernels, after one untimed pass that
    # lets the autotuner settle the size classes of the sample
    def per_tree_batched(t):
        a, b = int(off[t]), int(off[t + 1])
        q = slice(t * 256, (t + 1) * 256)
        tr = otg.Tree("boxes", np.float32).create(d_boxes[a:b], max_elements=16)
        tr.range_search(d_ranges[q], raw=True)
        tr.ray_all(d_rays[q], raw=True)
        tr.frustum_culling(d_planes[t : t + 1], raw=True)

    for t in idx:
        per_tree_batched(t)
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    for t in idx:
        per_tree_batched(t)
    torch.cuda.synchronize()
    per_tree_batched_s = (time.perf_counter() - s0) / sample
    return {
        "trees": trees,
        "entities": int(off[-1]),
        "queries_per_step": int(2 * trees * 256 + trees),
        "forest_step_ms": step_s * 1e3,
        "forest_trees_per_s": trees / step_s,
        "forest_queries_per_s_M": (2 * trees * 256 + trees) / step_s / 1e6,
        "graph_step_ms": graph_step_s * 1e3,
        "graph_trees_per_s": trees / graph_step_s,
        "graph_results_equal_to_calls": bool(graph_same),
        "forest_build_ms": (t1 - t0) * 1e3,
        "forest_range_ms": (t2 - t1) * 1e3,
        "forest_ray_all_ms": (t3 - t2) * 1e3,
        "forest_frustum_ms": (t4 - t3) * 1e3,
        "result_ids": {"range": int(n_ids[0]), "ray_all": int(n_ids[1]), "frustum": int(n_ids[2])},
        "per_tree_plain_trees_per_s": 1.0 / per_tree_s,
        "per_tree_plain_sample_trees": int(sample),
        "speedup_forest_vs_per_tree": (1.0 / per_tree_s) and (trees / step_s) / (1.0 / per_tree_s),
        "per_tree_batched_trees_per_s": 1.0 / per_tree_batched_s,
        "speedup_forest_vs_per_tree_batched": (trees / step_s) * per_tree_batched_s,
        "speedup_graph_vs_per_tree_batched": (trees / graph_step_s) * per_tree_batched_s,
        "mismatched_query_groups_in_sample": int(mism),
    }


def two_tree_boxes(n, seed, span=4096.0):
    """Boxes with centres uniform in [0, span)^3 and half-extents lognormal(ln 1, 0.8) per axis."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)) * span
    e = rng.lognormal(0.0, 0.8, (n, 3))
    return np.concatenate([c - e, c + e], 1)


def run_two_trees(steps=10):
    """Two-tree collision at scale: a static tree A of 16M boxes against a tree B of 8M boxes that
    moves by a per-box velocity N(0, 0.5) per axis and per step and is rebuilt every step."""
    import torch

    import octree_gb300 as otg

    a = torch.as_tensor(two_tree_boxes(16_000_000, 501), device="cuda")
    b0 = torch.as_tensor(two_tree_boxes(8_000_000, 502), device="cuda")
    v = torch.as_tensor(np.random.default_rng(503).normal(0.0, 0.5, (8_000_000, 3)), device="cuda")
    shift = torch.cat([v, v], 1)
    ta = otg.Tree("boxes")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ta.create(a)
    ta.sync()
    build_a_ms = (time.perf_counter() - t0) * 1e3
    tb = otg.Tree("boxes")
    rebuild, collide, pairs = [], [], []
    plain_ms = None
    equal_step0 = None
    for s in range(steps + 1):
        b = b0 + shift * float(s)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tb.create(b)
        tb.sync()
        t1 = time.perf_counter()
        r = ta.collision_pair(tb, raw=True)
        t2 = time.perf_counter()
        if s == 0:
            # warm-up step; also the plain kernel for comparison
            t3 = time.perf_counter()
            rp = ta.collision_pair(tb, algo=otg.ALGO_PLAIN_FP64, raw=True)
            plain_ms = (time.perf_counter() - t3) * 1e3
            equal_step0 = bool(np.array_equal(r.to_host()[1], rp.to_host()[1]))
            continue
        rebuild.append((t1 - t0) * 1e3)
        collide.append((t2 - t1) * 1e3)
        pairs.append(r.sizes()[1] // 2)
    info = tb.info()
    passes = (3 * info.max_depth + 5 + 7) // 8
    rebuild_bytes = 8_000_000 * (48 + 12 + 8 + 24 * passes + 12)
    tests, rechecks = r.stats()
    return {
        "tree_a_boxes": 16_000_000,
        "tree_b_boxes": 8_000_000,
        "steps": steps,
        "tree_a_build_ms": build_a_ms,
        "rebuild_b_ms_mean": statistics.mean(rebuild),
        "rebuild_b_GBps_algorithmic": rebuild_bytes / (statistics.mean(rebuild) / 1e3) / 1e9,
        "collide_ms_mean": statistics.mean(collide),
        "pairs_per_step_mean": statistics.mean(pairs),
        "pairs_per_s_M": statistics.mean(pairs) / (statistics.mean(collide) / 1e3) / 1e6,
        "step_ms_mean": statistics.mean(rebuild) + statistics.mean(collide),
        "collide_plain_fp64_ms_step0": plain_ms,
        "pair_lists_equal_step0": equal_step0,
        "recheck_fraction": rechecks / max(tests, 1),
    }


def inside(pts, ref):
    """The rows of pts inside the bounding box of ref (new points that a tree of ref can take)."""
    lo, hi = ref.min(0), ref.max(0)
    return pts[np.all((pts >= lo) & (pts <= hi), 1)]


def run_insert(reps=3, cpu=True):
    """Bulk Insert (DynamicHashOrthoTreeCore::Insert) of 1M new shell points into the 16M shell tree
    (depth 10, max 20): each repetition inserts into a fresh Create (untimed); the synchronous insert
    call is timed by the host clock, from device and from host memory; a full Create of all 17M points
    is timed beside it. On the CPU, the oracle's Insert (one thread, as the reference's SeqExec) of
    62.5k points into a 1M-point tree is timed against the GPU on the same case, and the two trees'
    node sets and parent links are compared."""
    import torch

    import octree_gb300 as otg

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _insert_cases import parent_keys
    from _oracle_lib import KIND_POINTS, oracle

    pts = shell_points(16_000_000, 301)
    add = inside(shell_points(1_050_000, 311), pts)[:1_000_000]
    pts_d = torch.as_tensor(pts, device="cuda")
    add_d = torch.as_tensor(add, device="cuda")
    add_pinned = torch.as_tensor(add).pin_memory()
    out = {"insert_points": len(add), "into_tree_points": len(pts)}
    dev_ms, host_ms, nodes, phases = [], [], 0, []
    otg.profile_enable(True)
    for r in range(reps + 1):
        for src, acc in ((add_d, dev_ms), (add_pinned.numpy(), host_ms)):
            t = otg.Tree("points").create(pts_d, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
            t.sync()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            t.insert(src)
            ms = (time.perf_counter() - t0) * 1e3
            if r:
                acc.append(ms)
                if src is add_d:
                    phases.append(dict(otg.profile_phases()))
            nodes = t.node_count
            del t
    otg.profile_enable(False)
    allp = torch.cat([pts_d, add_d])
    rebuild = []
    for r in range(reps + 1):
        t = otg.Tree("points")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t.create(allp, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        if r:
            rebuild.append((time.perf_counter() - t0) * 1e3)
        del t
    out["insert_1M_into_16M_device_ms"] = statistics.median(dev_ms)
    out["insert_1M_into_16M_host_input_ms"] = statistics.median(host_ms)
    out["insert_Mpts_per_s"] = len(add) / statistics.median(dev_ms) / 1e3
    out["nodes_after_insert"] = int(nodes)
    if phases and phases[0]:
        out["insert_phases_ms"] = {k: statistics.median(p[k] for p in phases) for k in phases[0]}
    out["create_17M_ms"] = statistics.median(rebuild)
    # the same small case on the GPU and in the oracle
    small, small_add = pts[::16], add[::16]
    g = []
    for r in range(reps + 1):
        t = otg.Tree("points").create(small, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        t0 = time.perf_counter()
        t.insert(small_add)
        if r:
            g.append((time.perf_counter() - t0) * 1e3)
    out["insert_62k_into_1M_gpu_ms"] = statistics.median(g)
    if cpu:
        o = oracle().create(small, KIND_POINTS, MAX_DEPTH, None, MAX_ELEM, threads=os.cpu_count() or 1)
        t0 = time.perf_counter()
        ok = o.insert(small_add)
        out["insert_62k_into_1M_cpu_ms"] = (time.perf_counter() - t0) * 1e3
        out["insert_cpu_kind"] = "port"
        out["insert_cpu_threads"] = 1
        out["insert_speedup_gpu_vs_cpu_same_case"] = out["insert_62k_into_1M_cpu_ms"] / out["insert_62k_into_1M_gpu_ms"]
        gn, on = t.nodes(), o.nodes()
        same = ok and np.array_equal(np.sort(gn["keys"]), on["keys"]) and np.array_equal(parent_keys(gn), o.parents())
        out["insert_sample_nodes_and_links_equal_to_cpu"] = bool(same)
    return out


PROFILE_CASES = ("knn_4m_200k", "collide_1m", "build_4m", "build_16m", "build_4m_clustered", "forest_frustum_1024", "insert_16m_1m", "insert_4m_250k", "range_1m_10k")


def run_profile_case(name):
    """Small cases for ncu captures (a few hundred MB on the device): each runs its kernels twice."""
    import torch

    import octree_gb300 as otg

    if name == "knn_4m_200k":
        pts = torch.as_tensor(shell_points(4_000_000, 301), device="cuda")
        t = otg.Tree("points").create(pts, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        q = torch.as_tensor(shell_points(200_000, 302), device="cuda")
        k = torch.as_tensor(np.random.default_rng(303).integers(1, 65, 200_000).astype(np.int32), device="cuda")
        for _ in range(2):
            r = t.knn(q, k, algo=otg.ALGO_FILTERED, raw=True)
        print(json.dumps({"case": name, "results": r.sizes()[1], "stats": r.stats()}))
    elif name == "collide_1m":
        boxes = torch.as_tensor(cluster_boxes(1_000_000, 201), device="cuda")
        t = otg.Tree("boxes").create(boxes, max_depth=12, max_elements=32)
        t.sync()
        for _ in range(2):
            r = t.collision_self(algo=otg.ALGO_FILTERED, raw=True)
        print(json.dumps({"case": name, "pairs": r.sizes()[1] // 2, "stats": r.stats()}))
    elif name == "forest_frustum_1024":
        boxes, off, _, _, planes = many_trees(1024, 401)
        d_boxes = torch.as_tensor(boxes, device="cuda")
        d_planes = torch.as_tensor(planes, device="cuda")
        foff = np.arange(1025, dtype=np.uint64)
        f = otg.Forest("boxes", np.float32)
        f.create(d_boxes, off, max_elements=16)
        for _ in range(2):
            r = f.frustum_culling(d_planes, foff, raw=True)
        f.sync()
        print(json.dumps({"case": name, "boxes": int(off[-1]), "frustum_ids": int(r.sizes()[1])}))
    elif name == "build_4m_clustered":
        # half the points in 64 tight clusters: buckets above the shared-memory capacity of one block
        rng = np.random.default_rng(311)
        pts = rng.random((4_000_000, 3))
        centres = rng.random((64, 3))
        pts[:2_000_000] = centres[rng.integers(0, 64, 2_000_000)] + rng.normal(0.0, 0.01, (2_000_000, 3))
        pts = torch.as_tensor(pts, device="cuda")
        t = otg.Tree("points")
        for _ in range(2):
            t.create(pts, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        print(json.dumps({"case": name, "nodes": int(t.node_count)}))
    elif name == "range_1m_10k":
        # C1 RangeSearch (Inside) through the batched kernel at its default shape (autotuning off)
        pts, ranges, _ = c1_workload()
        t = otg.Tree("points").create(torch.as_tensor(pts, device="cuda"), max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        otg.autotune_enable(False)
        rd = torch.as_tensor(ranges, device="cuda")
        for _ in range(2):
            r = t.range_search(rd, otg.RANGE_INSIDE, raw=True)
        print(json.dumps({"case": name, "ids": r.sizes()[1]}))
    elif name in ("insert_16m_1m", "insert_4m_250k"):
        # Insert of new shell points into a fresh shell tree, twice (the launch list covers both)
        n, m = (16_000_000, 1_000_000) if name == "insert_16m_1m" else (4_000_000, 250_000)
        pts = shell_points(n, 301)
        add = torch.as_tensor(inside(shell_points(m + m // 20, 311), pts)[:m], device="cuda")
        pts = torch.as_tensor(pts, device="cuda")
        for _ in range(2):
            t = otg.Tree("points").create(pts, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
            t.insert(add)
        print(json.dumps({"case": name, "nodes": int(t.node_count)}))
    elif name in ("build_4m", "build_16m"):
        # build_16m: the measured workload (384 MB of points, above the L2), about 2 GB on the device
        n = 4_000_000 if name == "build_4m" else N_POINTS
        pts = torch.as_tensor(shell_points(n, 301), device="cuda")
        t = otg.Tree("points")
        for _ in range(2):
            t.create(pts, max_depth=MAX_DEPTH, max_elements=MAX_ELEM)
        t.sync()
        print(json.dumps({"case": name, "nodes": int(t.node_count)}))
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-queries", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", choices=PROFILE_CASES, help="run one small case for an ncu capture and exit")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args.profile_case)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
