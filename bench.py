"""Benchmark of the spatial-query hot path on GB300.

Headline workload (one step = one pass of the path over one batch): first ray hit of 4,194,304 cosine-distributed rays
against a 1024 x 1024-vertex fBm heightfield (2,093,058 triangles), the configuration the metric is quoted on. Inputs
are seeded synthetic data with the benchmark's shapes and distributions (no dataset exists for this path).

  value      Mqueries/s with rays and mesh resident in HBM (device pointers), CUDA events on the launching stream,
             L2 flushed (256 MB write) before every timed step.
  e2e        the same metric through the C ABI with host (pinned) buffers, inside the timed region: the rays go to the
             GPU and (time, index) come back (the library reads and writes pinned arrays in place over NVLink-C2C).
  roofline   algorithmic bytes per launch / mean ray-kernel duration (CUDA events recorded around each launch).
  cpu_baseline  the oracle's restatement of the reference's CPU traversal (reference kd-tree, reference tie order) on a
             bounded sample, all host threads (and one thread on a smaller sample).
  extra      the other workloads measured the same way, device-resident: the FP64 ray re-test and occlusion queries
             on config 1, closest point (config 0), the k-NN graph (config 2), Visibility, the sample graph and
             ShapeDiameter on the config-0 mesh, the batched forest (config 3) and the serving loop (config 4).

--impl reference times the reference's algorithm on the host cores instead: the oracle's restatement, pinned bit for bit
to the reference's own code (which builds only where its sources are, against an Eigen subset; Eigen itself is absent).

Multi-GPU: one process per GPU (torchrun); each rank runs an independent replica on its own batch (weak scaling);
the only exchange is the max-over-ranks of the timed region.
"""

import argparse
import gc
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

from thea_gb300 import workloads as W  # noqa: E402

RAYS = 4194304
HF_GRID = 1024
MESH_BYTES_CFG1 = 12 * (HF_GRID * HF_GRID) + 12 * 2093058        # vertices + faces
ALGO_BYTES_CFG1 = 32 * RAYS + MESH_BYTES_CFG1                    # 24 B in + 8 B out per ray, mesh once
CP_QUERIES = 262144
ALGO_BYTES_CFG0 = 32 * CP_QUERIES + 12 * 40962 + 12 * 81920
KNN_POINTS = 1048576
ALGO_BYTES_CFG2 = 140 * KNN_POINTS


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--case", choices=sorted(CASES), help="run one small profiling case (warm-up calls, then the "
                    "launch to capture) and exit; used by the ncu commands recorded under profiles/")
    return ap.parse_args()


def case_ray():
    """Config 1: three plain calls, then one call with the FP64 watertight re-test."""
    import torch
    import thea_gb300 as T
    V, F, o, d = W.config1()
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=2)
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    for _ in range(3):
        bvh.ray_structure_intersection(od, dd)
    bvh.ray_structure_intersection_ex(od, dd, precision="fp64")
    torch.cuda.synchronize()


def _case_ray_grid(grid):
    import torch
    import thea_gb300 as T
    V, F, o, d = W.config1(grid=grid)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=2)
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    for _ in range(3):
        bvh.ray_structure_intersection(od, dd)
    torch.cuda.synchronize()


def case_ray_hf512():
    """The config-1 rays on a 512 x 512-vertex heightfield (522,242 triangles; nodes + ray records about 42 MB, a
    third of L2): three plain calls."""
    _case_ray_grid(512)


def case_ray_hf2048():
    """The config-1 rays on a 2048 x 2048-vertex heightfield (8,380,418 triangles; nodes + ray records about 670 MB):
    three plain calls."""
    _case_ray_grid(2048)


def case_cfg0_32k():
    """Closest point of the first 32,768 config-0 queries (one query per thread, oriented slabs): three calls."""
    import torch
    import thea_gb300 as T
    V, F, Q = W.config0()
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=1, max_leaf_size=1)
    q = torch.from_numpy(Q[:32768]).cuda()
    for _ in range(3):
        bvh.closest_element(q)
    torch.cuda.synchronize()


def case_sample_graph():
    """Sample proximity graph of 262,144 area samples of the config-0 mesh with face normals, max degree 8,
    reachability against the mesh (the bench's row): three calls."""
    import torch
    import thea_gb300 as T
    V, F, _ = W.config0()
    Vd, Fd = torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda()
    pos, nrm, _ = T.sample_evenly_by_area(Vd, Fd, KNN_POINTS, 2)
    mesh = T.MeshBvh(Vd, Fd, layouts=2)
    g_pts, g_nrm = pos[:262144].contiguous(), nrm[:262144].contiguous()
    for _ in range(3):
        T.sample_graph(g_pts, g_nrm, max_degree=8, seed=1, surface=mesh)
    torch.cuda.synchronize()


def case_cfg3_fp64_64():
    """Batched closest point with FP64 re-check over 64 meshes of the config-3 distribution: two calls."""
    import torch
    import thea_gb300 as T
    V, F, foff, Q, qoff, _ = W.config3_torch(64)
    forest = T.MeshForest(V, F, foff, width=4, max_leaf_size=1, layouts=1)
    for _ in range(2):
        forest.batch_closest_element(Q, qoff, precision="fp64", hard_query_budget=-1, queries_per_warp=64)
    torch.cuda.synchronize()


def case_gram_knn():
    """k-NN graph (k = 16) of 1,048,576 area samples of the config-0 mesh with tensor-core candidates: two calls."""
    import torch
    import thea_gb300 as T
    V, F, _ = W.config0()
    pos, _, _ = T.sample_evenly_by_area(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), 1 << 20, 2)
    pb = T.PointBvh(pos)
    for _ in range(2):
        pb.k_closest_self(16, device=True, candidates="gram")
    torch.cuda.synchronize()


def case_knn():
    """k-NN graph (k = 16) of 1,048,576 area samples of the config-0 mesh by the traversal: three calls."""
    import torch
    import thea_gb300 as T
    V, F, _ = W.config0()
    pos, _, _ = T.sample_evenly_by_area(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), 1 << 20, 2)
    pb = T.PointBvh(pos)
    for _ in range(3):
        pb.k_closest_self(16, device=True)
    torch.cuda.synchronize()


def case_cfg0():
    """Config 0: closest point of 262,144 queries on the noisy icosphere, three calls."""
    import torch
    import thea_gb300 as T
    V, F, Q = W.config0()
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=1)
    Qd = torch.from_numpy(Q).cuda()
    for _ in range(3):
        bvh.closest_element(Qd)
    torch.cuda.synchronize()


def case_cfg3_fp32_64():
    """Batched closest point (FP32, one thread per query throughout) over 64 meshes of the config-3 distribution."""
    import torch
    import thea_gb300 as T
    V, F, foff, Q, qoff, _ = W.config3_torch(64)
    forest = T.MeshForest(V, F, foff, width=4, max_leaf_size=1, layouts=1)
    for _ in range(2):
        forest.batch_closest_element(Q, qoff, hard_query_budget=-1, queries_per_warp=64)
    torch.cuda.synchronize()


def case_ray_host():
    """Config 1 through the C ABI with rays and results in pinned host memory (the in-place e2e kernel): three calls."""
    import ctypes
    import torch
    import thea_gb300 as T
    from thea_gb300 import _native as N
    V, F, o, d = W.config1()
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=2, max_leaf_size=2)
    ho, hd = torch.from_numpy(o).pin_memory(), torch.from_numpy(d).pin_memory()
    ht, hi = torch.empty(len(o)).pin_memory(), torch.empty(len(o), dtype=torch.int32).pin_memory()
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    for _ in range(3):
        N.check(N.lib().thea_ray_intersection(bvh.handle, p(ho), p(hd), len(o), -1.0, p(ht), p(hi), None,
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))


def case_cfg0_host():
    """Config 0 through the C ABI with queries and results in pinned host memory (the in-place kernels): three calls."""
    import ctypes
    import torch
    import thea_gb300 as T
    from thea_gb300 import _native as N
    V, F, Q = W.config0()
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=1, max_leaf_size=1)
    n = len(Q)
    hq = torch.from_numpy(Q).pin_memory()
    hi, hd = torch.empty(n, dtype=torch.int32).pin_memory(), torch.empty(n).pin_memory()
    hc = torch.empty((n, 3)).pin_memory()
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    for _ in range(3):
        N.check(N.lib().thea_closest_element(bvh.handle, p(hq), n, -1.0, p(hi), p(hd), p(hc),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))


CASES = {"ray": case_ray, "ray_host": case_ray_host, "ray_hf512": case_ray_hf512, "ray_hf2048": case_ray_hf2048,
         "cfg0_32k": case_cfg0_32k, "cfg0": case_cfg0, "cfg0_host": case_cfg0_host, "knn": case_knn,
         "cfg3_fp64_64": case_cfg3_fp64_64, "cfg3_fp32_64": case_cfg3_fp32_64, "gram_knn": case_gram_knn,
         "sample_graph": case_sample_graph}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary (profiles/ncu_traffic.txt), or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and not line.startswith("#") and parts[0] == kernel:
            return float(parts[1])
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------------------------------------------
# CPU baseline: the reference's algorithm on the host cores. The oracle restates the reference's kd-tree and traversals
# (reference tie order); the timed build is compiled with the reference's release flags (-std=c++17 -O2 -DNDEBUG
# -fno-strict-aliasing) and nothing else. One routine times every configuration, for the reference arm and for the
# cpu_baseline legs alike: the whole workload in its own order, all host threads with a static partition of the queries
# (a pass before the timed ones faults the tree and the inputs in), and one thread on an evenly strided sample.
# Test infrastructure used here only as the measured baseline; the GPU path never calls it.
# ---------------------------------------------------------------------------------------------------------------------

def host_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def _oracle():
    from oracle import oracle as O
    O.build()
    return O


def _passes(run, passes, warmup):
    for _ in range(warmup):
        run()
    out = []
    for _ in range(passes):
        t0 = time.perf_counter()
        run()
        out.append(time.perf_counter() - t0)
    return out


def cpu_workload(name, data):
    """(count, run(threads), one-core count, run_one_core(), description) of one configuration's reference workload.
    data: config 1 (V, F, o, d); config 0 (V, F, Q); config 2 (P,); config 3 a list of (V, F, Q) meshes."""
    O = _oracle()
    if name == "cfg1":
        V, F, o, d = data
        m = O.MeshIndex(V, F, timed=True)
        o1, d1 = np.ascontiguousarray(o[::16]), np.ascontiguousarray(d[::16])
        return (len(o), lambda th: m.ray_ref(o, d, threads=th), len(o1), lambda: m.ray_ref(o1, d1, threads=1),
                "rayStructureIntersection over the reference kd-tree (leaf size 5), all %d rays in order" % len(o))
    if name == "cfg0":
        V, F, Q = data
        m = O.MeshIndex(V, F, timed=True)
        q1 = np.ascontiguousarray(Q[::16])
        return (len(Q), lambda th: m.closest_ref(Q, threads=th), len(q1), lambda: m.closest_ref(q1, threads=1),
                "closestElement over the reference kd-tree (leaf size 5), all %d queries in order" % len(Q))
    if name == "cfg2":
        (P,) = data
        pi = O.PointIndex(P, timed=True)
        ex = np.arange(len(P), dtype=np.int32)
        p1, e1 = np.ascontiguousarray(P[::16]), np.ascontiguousarray(ex[::16])
        return (len(P), lambda th: pi.knn_ref(P, 16, exclude=ex, threads=th), len(p1),
                lambda: pi.knn_ref(p1, 16, exclude=e1, threads=1),
                "kClosestPairs (k = 16, FilterSelf) over the reference kd-tree of the %d samples, every sample "
                "queried" % len(P))
    if name == "cfg3":
        from concurrent.futures import ThreadPoolExecutor
        idx = [O.MeshIndex(v, f, timed=True) for v, f, _ in data]
        qs = [q for _, _, q in data]
        n = sum(len(q) for q in qs)

        def run(th):
            # meshes handed out to the threads one at a time (each query batch single-threaded)
            with ThreadPoolExecutor(th) as ex:
                list(ex.map(lambda j: idx[j].closest_ref(qs[j], threads=1), range(len(idx))))

        one = list(range(0, len(idx), 16))
        n1 = sum(len(qs[j]) for j in one)
        return (n, run, n1, lambda: [idx[j].closest_ref(qs[j], threads=1) for j in one],
                "per mesh: the reference kd-tree and closestElement, %d meshes (%d queries) sampled evenly from the "
                "batch" % (len(idx), n))
    raise ValueError(name)


def cpu_time(name, data, passes=1, warmup=1, threads=None, one_core=True):
    """Times one configuration's reference workload: mean seconds of `passes` all-thread passes after `warmup`."""
    threads = threads or host_threads()
    n, run, n1, run1, what = cpu_workload(name, data)
    ts = _passes(lambda: run(threads), passes, warmup)
    res = {"value": n / statistics.mean(ts) / 1e6, "unit": "Mqueries/s", "cores": threads, "kind": "port",
           "sample": what + "; %d thread(s), static partition; mean of %d pass(es) after %d untimed" %
                     (threads, passes, warmup),
           "seconds_per_pass": statistics.mean(ts), "build": "oracle/_build/liboracle_timed.so, reference flags"}
    if one_core:
        t1 = _passes(run1, 1, 0)[0]
        res.update({"one_core_value": n1 / t1 / 1e6, "one_core_sample": "%d queries (every 16th) on one thread" % n1})
    return res


def reference_arm(args, rank, world):
    if rank != 0:
        return
    V, F, o, d = W.config1()
    threads = host_threads()
    n, run, _, _, what = cpu_workload("cfg1", (V, F, o, d))
    ts = _passes(lambda: run(threads), args.steps, args.warmup)
    ms = 1000.0 * statistics.mean(ts)
    value = n / (ms / 1000.0) / 1e6
    line = {"impl": "reference", "metric": HEADLINE_METRIC,
            "value": value, "unit": "Mqueries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm heightfield and cosine rays)",
            "config": headline_config(),
            "cpu_baseline": {"value": value, "unit": "Mqueries/s", "cores": threads, "kind": "port",
                             "sample": what + "; every step the whole workload, %d threads, static partition; the "
                                              "reference's algorithm restated in C++ and pinned bit for bit to the "
                                              "reference's own code, compiled with its release flags" % threads},
            "e2e": {"value": value, "unit": "Mqueries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


HEADLINE_METRIC = "Mqueries/s ray first-hit (config 1: 1024^2 heightfield, 4,194,304 rays)"


def headline_config():
    """The workload both arms run (identical in the two JSON lines)."""
    return {"workload": "ray_first_hit_heightfield_1024", "triangles": 2093058, "vertices": 1048576, "rays": RAYS,
            "l2": "GPU arm: flushed by a 256 MB write before every timed step (host arm: no flush)"}


# ---------------------------------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------------------------------

def max_over_ranks(x, dist, device):
    """The largest value of x over all ranks (x itself without a process group): the whole job's time is its slowest
    rank's."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def timed_steps(fn, steps, warmup, flush, stream):
    """Runs warmup steps, then `steps` timed steps each preceded by an L2 flush; returns per-step ms (CUDA events)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def gpu_arm(args, rank, world, local_rank):
    import torch
    import thea_gb300 as T
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    V, F, o, d = W.config1()
    Vd, Fd = torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda()
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bvh = T.MeshBvh(Vd, Fd, layouts=2)
    torch.cuda.synchronize()
    build_ms = 1000 * (time.perf_counter() - t0)
    info = bvh.info()
    out_t = torch.empty(RAYS, dtype=torch.float32, device="cuda")
    out_i = torch.empty(RAYS, dtype=torch.int32, device="cuda")
    from thea_gb300 import _native as N
    L = N.lib()
    import ctypes

    def step():
        N.check(L.thea_ray_intersection(bvh.handle, ctypes.c_void_p(od.data_ptr()), ctypes.c_void_p(dd.data_ptr()),
                                        RAYS, -1.0, ctypes.c_void_p(out_t.data_ptr()),
                                        ctypes.c_void_p(out_i.data_ptr()), None,
                                        ctypes.c_void_p(stream.cuda_stream)))

    # warm-up, then the timed region bracketed by barrier + synchronize, with clocks sampled during it
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    T.profiling_reset()
    T.profiling(True)
    launches0 = T.launch_count()
    with ClockSampler(local_rank) as clk:
        t_wall0 = time.perf_counter()
        ms = timed_steps(step, args.steps, 0, flush, stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    launches = T.launch_count() - launches0
    T.profiling(False)
    k_ms, k_cnt = T.profiling_read("ray_kernel")
    T.profiling_reset()
    step_ms = max_over_ranks(sum(ms) / len(ms), dist, "cuda")
    value = world * RAYS / (step_ms / 1000.0) / 1e6
    kernel_ms = k_ms / max(1, k_cnt)
    peak, peak_kind = peaks()
    achieved = ALGO_BYTES_CFG1 / (kernel_ms / 1000.0) / 1e9

    # end to end through the C ABI with pinned host buffers
    ho = torch.from_numpy(o).pin_memory()
    hd = torch.from_numpy(d).pin_memory()
    ht = torch.empty(RAYS, dtype=torch.float32).pin_memory()
    hi = torch.empty(RAYS, dtype=torch.int32).pin_memory()

    def e2e_step():
        N.check(L.thea_ray_intersection(bvh.handle, ctypes.c_void_p(ho.data_ptr()), ctypes.c_void_p(hd.data_ptr()),
                                        RAYS, -1.0, ctypes.c_void_p(ht.data_ptr()), ctypes.c_void_p(hi.data_ptr()),
                                        None, ctypes.c_void_p(stream.cuda_stream)))

    for _ in range(args.warmup):
        e2e_step()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()  # synchronous: returns once results are in host memory
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e_times), dist, "cuda")
    assert np.array_equal(hi.numpy(), out_i.cpu().numpy()), "host and device paths disagree"
    hits = int((hi.numpy() >= 0).sum())
    # parity of the timed results (the end-to-end call's) with the oracle, every ray: lowest index among equal times
    parity = None
    if rank == 0 and not args.no_cpu:
        ot, oi = _oracle().MeshIndex(V, F).ray_contract(o, d)
        parity = {"checked": RAYS, "indices_equal": bool(np.array_equal(hi.numpy(), oi)),
                  "times_equal": bool(np.array_equal(ht.numpy(), ot.astype(np.float32))),
                  "oracle": "reference kd-tree traversal restated, ties to the lowest index, FP32 arithmetic"}

    extra = {}
    if not args.no_extra:
        # the same rays with the FP64 watertight re-test beside the reference's FP32 verdict (config 1 as specified)
        T.profiling_reset()
        T.profiling(True)
        ms64 = timed_steps(lambda: bvh.ray_structure_intersection_ex(od, dd, precision="fp64"), args.steps,
                           args.warmup, flush, stream)
        T.profiling(False)
        r_ms, r_cnt = T.profiling_read("ray_recheck_kernel")
        T.profiling_reset()
        _, i32, _, i64, flags = bvh.ray_structure_intersection_ex(od, dd, precision="fp64")
        flags = flags.cpu().numpy()
        extra["ray_fp64_recheck_cfg1"] = {
            "value": RAYS / (statistics.mean(ms64) / 1e3) / 1e6, "unit": "Mqueries/s",
            "ms_per_step": statistics.mean(ms64), "kernel_ms": r_ms / max(1, r_cnt),
            "fp32_verdict_equals_plain": bool(torch.equal(i32, out_i)),
            "rays_hit_differs": int((flags & 1).sum()), "rays_element_differs": int(((flags & 2) >> 1).sum())}
        # the same rays as occlusion queries (rayIntersects: any-hit search)
        ms_any = timed_steps(lambda: bvh.ray_intersects(od, dd), args.steps, args.warmup, flush, stream)
        extra["ray_intersects_cfg1"] = {
            "value": RAYS / (statistics.mean(ms_any) / 1e3) / 1e6, "unit": "Mqueries/s",
            "ms_per_step": statistics.mean(ms_any),
            "equals_first_hit": bool(torch.equal(bvh.ray_intersects(od, dd), out_t >= 0))}
        extra.update(extra_workloads(T, torch, stream, flush, args))

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu and world == 1:
            cpu = cpu_time("cfg1", (V, F, o, d))
        traffic = ncu_traffic("ray_persistent_kernel")
        line = {
            "metric": HEADLINE_METRIC,
            "value": value, "unit": "Mqueries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded fBm heightfield and cosine rays)",
            "config": headline_config(),
            "details": {"bvh_width": info["width"], "leaf_size": info["max_leaf_size"], "bvh_nodes": info["num_nodes"],
                        "bvh_depth": info["depth"], "build_ms": build_ms, "hit_fraction": hits / RAYS,
                        "parallelism": "replica per GPU" if world > 1 else "single GPU"},
            "parity": parity,
            "e2e": {"value": world * RAYS / e2e_s / 1e6, "unit": "Mqueries/s", "h2d_bytes_per_step": RAYS * 24,
                    "d2h_bytes_per_step": RAYS * 8},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "ray_persistent_kernel", "kernel_ms": kernel_ms,
                         "algorithmic_bytes_per_launch": ALGO_BYTES_CFG1},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "wall_s_timed_region": t_wall,
            "extra": extra,
        }
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    bvh.close()
    if line is not None:
        print(json.dumps(line), flush=True)


def extra_workloads(T, torch, stream, flush, args):
    """Closest point (config 0) and the k-NN graph of area samples (config 2), device-resident."""
    out = {}
    steps = max(3, min(args.steps, 5))
    # config 0: closest point on the noisy icosphere
    V, F, Q = W.config0()
    # leaf size 1: the autotuner's choice for closest point on these meshes (config 3)
    bvh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=1, max_leaf_size=1)
    Qd = torch.from_numpy(Q).cuda()
    T.profiling_reset()
    T.profiling(True)
    ms = timed_steps(lambda: bvh.closest_element(Qd), steps, 2, flush, stream)
    T.profiling(False)
    # large batches run as two kernels (persistent lanes with a step budget, then one warp per query over budget)
    k_ms, k_cnt = T.profiling_read("batch_closest_phase")
    kms = k_ms / max(1, k_cnt // 2) if k_cnt else 0.0
    out["closest_point_cfg0"] = {"value": CP_QUERIES / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mqueries/s",
                                 "ms_per_step": statistics.mean(ms), "kernel_ms": kms,
                                 "roofline_frac": ALGO_BYTES_CFG0 / (max(kms, 1e-9) / 1e3) / 1e9 / peaks()[0]}
    # end to end through the C ABI with the queries and all three outputs in pinned host memory
    import ctypes
    from thea_gb300 import _native as N
    hq = torch.from_numpy(Q).pin_memory()
    hi = torch.empty(CP_QUERIES, dtype=torch.int32).pin_memory()
    hd, hc = torch.empty(CP_QUERIES).pin_memory(), torch.empty((CP_QUERIES, 3)).pin_memory()
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731

    def cp_e2e():
        N.check(N.lib().thea_closest_element(bvh.handle, p(hq), CP_QUERIES, -1.0, p(hi), p(hd), p(hc),
                                             ctypes.c_void_p(stream.cuda_stream)))

    for _ in range(2):
        cp_e2e()
    e2e_t = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cp_e2e()
        e2e_t.append(time.perf_counter() - t0)
    out["closest_point_cfg0"]["e2e"] = {"value": CP_QUERIES / statistics.mean(e2e_t) / 1e6, "unit": "Mqueries/s",
                                        "ms": 1e3 * statistics.mean(e2e_t), "h2d_bytes": 12 * CP_QUERIES,
                                        "d2h_bytes": 20 * CP_QUERIES, "same_as_device":
                                        bool(torch.equal(hi, bvh.closest_element(Qd)[0].cpu()))}
    # a small call: the two-kernel path with a short step budget, so nearly every query runs as one warp
    Qs = Qd[:32768].contiguous()
    ms_s = timed_steps(lambda: bvh.closest_element(Qs), steps, 2, flush, stream)
    out["closest_point_cfg0"]["first_32768_queries"] = {
        "value": 32768 / (statistics.mean(ms_s) / 1e3) / 1e6, "unit": "Mqueries/s", "ms_per_step": statistics.mean(ms_s),
        "same_as_full_batch": bool(torch.equal(bvh.closest_element(Qs)[0], bvh.closest_element(Qd)[0][:32768]))}
    bvh.close()
    if not args.no_cpu:
        out["closest_point_cfg0"]["cpu_baseline"] = cpu_time("cfg0", (V, F, Q))
        oi, od2, ocp = _oracle().MeshIndex(V, F).closest_contract(Q)
        out["closest_point_cfg0"]["parity"] = {
            "checked": CP_QUERIES, "indices_equal": bool(np.array_equal(hi.numpy(), oi)),
            "distances_equal": bool(np.array_equal(hd.numpy(), np.sqrt(od2.astype(np.float32)))),
            "closest_points_equal": bool(np.array_equal(hc.numpy(), ocp.astype(np.float32)))}
    # config 2: 1,048,576 area samples of the config-0 mesh (reference Random stream), k = 16 graph excluding self;
    # the first draw on the device also computes the generator's jump-ahead table, so the second is the one timed
    Vd, Fd = torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    T.sample_evenly_by_area(Vd, Fd, KNN_POINTS, 2)
    torch.cuda.synchronize()
    first_sample_ms = 1000 * (time.perf_counter() - t0)
    t0 = time.perf_counter()
    pos, _, _ = T.sample_evenly_by_area(Vd, Fd, KNN_POINTS, 2)
    torch.cuda.synchronize()
    sample_ms = 1000 * (time.perf_counter() - t0)
    t0 = time.perf_counter()
    pb = T.PointBvh(pos)
    torch.cuda.synchronize()
    pbuild_ms = 1000 * (time.perf_counter() - t0)
    T.profiling_reset()
    T.profiling(True)
    ms = timed_steps(lambda: pb.k_closest_self(16, device=True), steps, 2, flush, stream)
    T.profiling(False)
    k_ms, k_cnt = T.profiling_read("knn_kernel")
    kms = k_ms / max(1, k_cnt)
    out["knn_graph_cfg2"] = {"value": KNN_POINTS / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mqueries/s",
                             "ms_per_step": statistics.mean(ms), "kernel_ms": kms, "k": 16,
                             "sampling_ms": sample_ms, "first_sampling_ms": first_sample_ms, "point_bvh_build_ms": pbuild_ms,
                             "roofline_frac": ALGO_BYTES_CFG2 / (kms / 1e3) / 1e9 / peaks()[0]}
    # the same graph with tensor-core Gram candidates seeding the exact search (identical results)
    T.profiling_reset()
    T.profiling(True)
    ms = timed_steps(lambda: pb.k_closest_self(16, device=True, candidates="gram"), steps, 2, flush, stream)
    T.profiling(False)
    g_ms, g_cnt = T.profiling_read("gram_bound_kernel")
    k_ms, k_cnt = T.profiling_read("knn_kernel")
    i0, d0 = pb.k_closest_self(16, device=True)
    i1, d1 = pb.k_closest_self(16, device=True, candidates="gram")
    out["knn_graph_cfg2"]["gram_candidates"] = {
        "value": KNN_POINTS / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mqueries/s",
        "ms_per_step": statistics.mean(ms), "gram_kernel_ms": g_ms / max(1, g_cnt),
        "bounded_search_ms": k_ms / max(1, k_cnt), "tensor_flop_per_step": 2 * 16 * 512 * KNN_POINTS,
        "identical_to_traversal": bool(torch.equal(i0, i1) and torch.equal(d0, d1))}
    if not args.no_cpu:
        P = pos.cpu().numpy()
        out["knn_graph_cfg2"]["cpu_baseline"] = cpu_time("cfg2", (P,))
        ri, rd = _oracle().PointIndex(P).knn_contract(P, 16, exclude=np.arange(len(P), dtype=np.int32))
        out["knn_graph_cfg2"]["parity"] = {"checked": KNN_POINTS, "k": 16,
                                           "indices_equal": bool(np.array_equal(i0.cpu().numpy(), ri)),
                                           "sq_distances_equal": bool(np.array_equal(d0.cpu().numpy(),
                                                                                     rd.astype(np.float32)))}
    # closest pair and the 32 closest pairs between these samples and a second 1,048,576-sample set of the same mesh
    pos2, _, _ = T.sample_evenly_by_area(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), KNN_POINTS, 5)
    pb2 = T.PointBvh(pos2)
    ms = timed_steps(lambda: pb.closest_pair(pb2), steps, 2, flush, stream)
    ms_k = timed_steps(lambda: pb.k_closest_pairs(pb2, 32), steps, 2, flush, stream)
    cp_pair = pb.closest_pair(pb2)
    out["bvh_pairs_cfg2"] = {
        "value": KNN_POINTS / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mquery elements/s",
        "closest_pair_ms": statistics.mean(ms), "k32_closest_pairs_ms": statistics.mean(ms_k),
        "points_per_set": KNN_POINTS, "closest_sq_distance": cp_pair[2] if cp_pair else None}
    pb2.close()
    pb.close()
    # Visibility of 65,536 of the surface samples, 100 rays each (directions of Random(seed).sphere())
    mesh = T.MeshBvh(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), layouts=2)
    vis_pts = pos[:65536].contiguous()
    T.profiling_reset()
    T.profiling(True)
    ms = timed_steps(lambda: mesh.visibility(vis_pts, num_rays=100, seed=3), steps, 2, flush, stream)
    T.profiling(False)
    a_ms, a_cnt = T.profiling_read("any_hit_kernel")
    # the Random(seed) stream: one block, or chunks from jump-ahead start states (seed, jumps, chunk kernels) per call
    m_ms = sum(T.profiling_read(k)[0] for k in ("thea_mt_stream_kernel", "mt_seed_kernel", "mt_jump_apply_kernel",
                                                 "mt_chunk_kernel"))
    m_cnt = T.profiling_read("thea_mt_stream_kernel")[1] + T.profiling_read("mt_chunk_kernel")[1]
    vis = mesh.visibility(vis_pts, num_rays=100, seed=3)
    out["visibility_cfg0_mesh"] = {
        "value": 65536 * 100 / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mrays/s", "points": 65536,
        "rays_per_point": 100, "ms_per_step": statistics.mean(ms), "any_hit_kernel_ms": a_ms / max(1, a_cnt),
        "direction_stream_ms": m_ms / max(1, m_cnt), "mean_visibility": float(vis.mean().item())}
    # sample proximity graph of 262,144 of the surface samples with face normals, reachability against the mesh
    g_pts = pos[:262144].contiguous()
    _, g_nrm, _ = T.sample_evenly_by_area(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda(), KNN_POINTS, 2)
    g_nrm = g_nrm[:262144].contiguous()
    ms = timed_steps(lambda: T.sample_graph(g_pts, g_nrm, max_degree=8, seed=1, surface=mesh), 3, 1, flush, stream)
    _, _, g_deg, g_avg = T.sample_graph(g_pts, g_nrm, max_degree=8, seed=1, surface=mesh)
    out["sample_graph_cfg0_mesh"] = {
        "value": 262144 / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Msamples/s", "samples": 262144,
        "max_degree": 8, "ms_per_step": statistics.mean(ms), "mean_degree": float(g_deg.float().mean().item()),
        "separation_estimate": g_avg[0], "mean_separation": g_avg[1], "reachability": "against the mesh"}
    # ShapeDiameter of 65,536 of the surface samples with their face normals (30 cone rays each)
    sd_pts, sd_nrm = g_pts[:65536].contiguous(), g_nrm[:65536].contiguous()
    T.profiling_reset()
    T.profiling(True)
    ms = timed_steps(lambda: mesh.shape_diameter(sd_pts, sd_nrm), steps, 2, flush, stream)
    T.profiling(False)
    r_ms, r_cnt = T.profiling_read("ray_kernel")
    sdf = mesh.shape_diameter(sd_pts, sd_nrm)
    out["shape_diameter_cfg0_mesh"] = {
        "value": 65536 * 30 / (statistics.mean(ms) / 1e3) / 1e6, "unit": "Mrays/s", "points": 65536,
        "rays_per_point": 30, "ms_per_step": statistics.mean(ms), "ray_kernel_ms": r_ms / max(1, r_cnt),
        "points_with_value": int((sdf >= 0).sum().item()), "mean_sdf": float(sdf[sdf >= 0].mean().item())}
    mesh.close()
    T.profiling_reset()
    T.profiling_reset()
    out["batched_closest_cfg3"] = batched_config3(T, torch, stream, flush, args)
    out["serving_cfg4"] = serving_config4(T, torch, args)
    return out


def serving_config4(T, torch, args, num_meshes=256, rate=2000.0, seconds=3.0, seed=W.CONFIG_SEEDS[4]):
    """Config 4: a server with 256 resident meshes drawn as in config 3 and an 8 GB admission budget. Requests arrive
    Poisson at 2,000/s for `seconds`: 60% closest point, 25% first ray hit, 15% k-NN (k = 8) over the mesh's vertices,
    each with a log-uniform 1..1,048,576 queries uniform in its mesh's box grown by 50% (rays: origins there, uniform
    directions). Query and result arrays are pinned host memory; latency runs from submit to results written back."""
    res = {}
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    V, F, foff, _, _, levels = W.config3_torch(num_meshes, seed=seed, min_q=1, max_q=2)
    srv = T.Server(memory_budget_bytes=8 << 30)
    t0 = time.perf_counter()
    ids, boxes = [], []
    for m in range(num_meshes):
        Fm = F[foff[m]:foff[m + 1]]
        lo, hi = int(Fm.min()), int(Fm.max()) + 1
        Vm = V[lo:hi]
        ids.append(srv.add_mesh(Vm, Fm - lo))
        boxes.append((Vm.min(0).values.cpu().numpy(), Vm.max(0).values.cpu().numpy()))
    st = srv.stats()
    res["meshes"] = num_meshes
    res["resident_bytes"] = st["resident_bytes"]
    res["build_s"] = time.perf_counter() - t0
    del V, F
    # the request stream
    rng = np.random.default_rng(seed)
    n_req = int(rate * seconds)
    arrive = np.cumsum(rng.exponential(1.0 / rate, n_req))
    kind = rng.choice(3, size=n_req, p=[0.60, 0.25, 0.15])
    mesh = rng.integers(0, num_meshes, n_req)
    nq = np.exp(rng.uniform(0.0, np.log(1 << 20), n_req)).astype(np.int64).clip(1, 1 << 20)
    # per mesh, one pinned array of points uniform in its grown box, as long as its largest request; shared directions
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    pts = {}
    for m in np.unique(mesh):
        n = int(nq[mesh == m].max())
        lo, hi = boxes[m]
        c, e = 0.5 * (lo + hi), 1.5 * (hi - lo)
        u = torch.rand((n, 3), generator=g, device="cuda")
        pts[m] = (u * torch.as_tensor(e, device="cuda") + torch.as_tensor(c - 0.5 * e, device="cuda")).cpu().pin_memory()
    dirs = torch.nn.functional.normalize(torch.randn((1 << 20, 3), generator=g, device="cuda"), dim=1).cpu().pin_memory()
    # results: a pinned ring far larger than what can be in flight
    ring_idx = torch.empty(64 << 20, dtype=torch.int32).pin_memory()
    ring_val = torch.empty(64 << 20, dtype=torch.float32).pin_memory()
    pos = [0]

    def outputs(rows):
        if pos[0] + rows > ring_idx.numel():
            pos[0] = 0
        a, b = ring_idx[pos[0]:pos[0] + rows], ring_val[pos[0]:pos[0] + rows]
        pos[0] += rows
        return a, b

    names = ("closest", "ray", "knn")
    # warm-up, untimed: every query kind at a small and a multi-piece size on the mesh with the most points, so that
    # first launches and the scratch pool's growth happen before the stream
    mw = max(pts, key=lambda m: pts[m].shape[0])
    warm = []
    for n in (1000, min(200000, pts[mw].shape[0])):
        for kd in names:
            k = 8 if kd == "knn" else 1
            oi, ov = outputs(n * k)
            warm.append(srv.submit(kd, ids[mw], pts[mw][:n], directions=dirs[:n] if kd == "ray" else None, k=k,
                                   out=(oi, ov)))
    for t in warm:
        t.wait()
    tickets = [None] * n_req
    srv.reset_stats()
    torch.cuda.synchronize()
    # the client is this Python loop: keep the garbage collector from pausing it in the middle of the arrival stream
    gc.collect()
    gc.disable()
    late = np.zeros(n_req)
    submit_call = np.zeros(n_req)
    with ClockSampler(torch.cuda.current_device()) as clk:
        start = time.perf_counter()
        for r in range(n_req):
            now = time.perf_counter() - start
            if arrive[r] > now:
                time.sleep(arrive[r] - now)
            late[r] = time.perf_counter() - start - arrive[r]
            n, m, kd = int(nq[r]), int(mesh[r]), names[kind[r]]
            k = 8 if kd == "knn" else 1
            oi, ov = outputs(n * k)
            q = pts[m][:n]
            d = dirs[:n] if kd == "ray" else None
            t_call = time.perf_counter()
            tickets[r] = srv.submit(kd, ids[m], q, directions=d, k=k, out=(oi, ov))
            submit_call[r] = time.perf_counter() - t_call
        submit_s = time.perf_counter() - start
        lat = np.zeros(n_req)
        for r, t in enumerate(tickets):
            t.wait()
            lat[r] = t.latency_ms
            assert t.status == 0
        total_s = time.perf_counter() - start
    gc.enable()
    st = srv.stats()
    srv.close()
    small = nq <= 65536
    slow = small & (lat > 20.0)
    # algorithmic bytes of the queries (12 B per point or 24 B per ray in; 20 B closest, 8 B ray, 8 x 8 B k-NN out)
    qbytes = np.where(kind == 0, 32, np.where(kind == 1, 32, 12 + 8 * 8)) * nq
    per_kind = {}
    for kd_i, kd in enumerate(names):
        sel = kind == kd_i
        sm = sel & small
        per_kind[kd] = {"requests": int(sel.sum()), "p50_ms": float(np.percentile(lat[sel], 50)),
                        "p99_ms": float(np.percentile(lat[sel], 99)),
                        "small_p50_ms": float(np.percentile(lat[sm], 50)) if sm.any() else None,
                        "small_p99_ms": float(np.percentile(lat[sm], 99)) if sm.any() else None}
    res.update({
        "per_kind": per_kind,
        "hbm": {"query_bytes": int(qbytes.sum()), "achieved_gbs": float(qbytes.sum() / st["busy_seconds"] / 1e9),
                "frac": float(qbytes.sum() / st["busy_seconds"] / 1e9 / peaks()[0]),
                "basis": "query input and output bytes over the server's busy time; the resident meshes are read "
                         "from L2/HBM by every batch and not counted"},
        "client_lateness_ms": {"p50": float(1e3 * np.percentile(late, 50)), "p99": float(1e3 * np.percentile(late, 99)),
                               "max": float(1e3 * late.max()),
                               "meaning": "submit time minus scheduled arrival (the Python client); latency itself is "
                                          "measured by the server from submit to results written"},
        "submit_call_ms": {"p99": float(1e3 * np.percentile(submit_call, 99)), "max": float(1e3 * submit_call.max()),
                           "meaning": "duration of the submit call itself (the C-ABI call, its pointer-kind queries "
                                      "and the queue lock)"},
        "slow_small_requests": {"over_ms": 20.0, "count": int(slow.sum()),
                                "arrival_window_s": [float(arrive[slow].min()), float(arrive[slow].max())]
                                if slow.any() else None,
                                "meaning": "when the requests of <= 65,536 queries slower than 20 ms arrived, in seconds "
                                           "from the stream's start: one window in which the client was late too is a "
                                           "pause of the whole process or driver, not queueing"},
        "requests": n_req, "offered_rate_per_s": n_req / arrive[-1], "submit_span_s": submit_s, "drain_s": total_s,
        "queries": int(nq.sum()), "mix": {"closest": int((kind == 0).sum()), "ray": int((kind == 1).sum()),
                                           "knn": int((kind == 2).sum())},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
        "small_requests": int(small.sum()), "small_p50_ms": float(np.percentile(lat[small], 50)),
        "small_p99_ms": float(np.percentile(lat[small], 99)),
        "sustained_queries_per_s": float(nq.sum() / total_s), "server_queries_per_s": st["queries_per_second"],
        "batches": st["batches"], "clocks": clk.summary(),
        "io": "pinned host arrays, staged by the server", "precision": "fp32 reference arithmetic",
    })
    return res


def batched_config3(T, torch, stream, flush, args, num_meshes=4096):
    """Config 3: 4,096 noisy stretched icospheres (320..327,680 triangles each), 1k..100k queries each. The batched
    path is one persistent launch over a forest, autotuned on a sample and replayed from a CUDA graph; the plain path is
    the drop-in loop (one BVH build and one closest-point call per mesh). Both report queries/s over query time."""
    res = {}
    t0 = time.perf_counter()
    V, F, foff, Q, qoff, levels = W.config3_torch(num_meshes)
    torch.cuda.synchronize()
    res["meshes"] = num_meshes
    res["triangles"] = int(foff[-1])
    res["queries"] = int(Q.shape[0])
    res["generate_s"] = time.perf_counter() - t0
    nq = Q.shape[0]
    qoff_h = qoff.cpu().numpy()
    # algorithmic bytes: 32 B per query (12 in, 20 out) + every mesh once (12 B per vertex and per face)
    algo = 32 * nq + 12 * V.shape[0] + 12 * F.shape[0]
    res["algorithmic_bytes"] = int(algo)
    # autotune on every 16th mesh
    samp = np.arange(0, num_meshes, 16)
    sv, sf, sq, sfo, sqo, vb = [], [], [], [0], [0], 0
    for m in samp:
        Fm = F[foff[m]:foff[m + 1]]
        lo = int(Fm.min())
        hi = int(Fm.max()) + 1
        sv.append(V[lo:hi])
        sf.append(Fm - lo + vb)
        vb += hi - lo
        sq.append(Q[qoff_h[m]:qoff_h[m + 1]])
        sfo.append(sfo[-1] + Fm.shape[0])
        sqo.append(sqo[-1] + sq[-1].shape[0])
    t0 = time.perf_counter()
    # tuned for the mixed-precision mode (FP32 traversal, FP64 re-check), the configuration the target is quoted on
    tune = T.autotune_batch_closest(torch.cat(sv), torch.cat(sf), np.array(sfo, np.int64), torch.cat(sq),
                                    torch.as_tensor(np.array(sqo, np.int64), device="cuda"), precision="fp64")
    res["autotune"] = dict(tune, seconds=time.perf_counter() - t0)
    t0 = time.perf_counter()
    forest = T.MeshForest(V, F, foff, width=tune["width"], max_leaf_size=tune["max_leaf_size"], layouts=1)
    torch.cuda.synchronize()
    res["forest_build_s"] = time.perf_counter() - t0
    results = {}
    for prec in ("fp32", "fp64"):
        out = (torch.empty(nq, dtype=torch.int32, device="cuda"), torch.empty(nq, dtype=torch.float32, device="cuda"),
               torch.empty((nq, 3), dtype=torch.float32, device="cuda"), None)
        s = torch.cuda.Stream()
        torch.cuda.synchronize()
        kw = dict(precision=prec, queries_per_warp=tune["queries_per_warp"],
                  hard_query_budget=tune["hard_query_budget"])
        with torch.cuda.stream(s):
            with T.Graph() as g:
                forest.batch_closest_element(Q, qoff, closest_points=True, out=out, **kw)
            ms = timed_steps(g.launch, max(3, min(args.steps, 5)), 2, flush, s)
        g.close()
        # accuracy, untimed: |distance - FP64 distance of the returned element| relative to the distance, floored at
        # 1e-6 of the scene scale (distances near zero)
        _, d, _, e = forest.batch_closest_element(Q, qoff, errors=True, **kw)
        rel = (e / torch.clamp(d, min=1e-6 * float(Q.abs().max()))).max().item()
        res["batched_" + prec] = {"value": nq / (statistics.median(ms) / 1e3) / 1e6, "unit": "Mqueries/s",
                                  "ms": statistics.median(ms), "max_rel_error_vs_fp64": rel,
                                  "roofline_frac": algo / (statistics.median(ms) / 1e3) / 1e9 / peaks()[0]}
        results[prec] = (out[0].cpu().numpy(), out[1].cpu().numpy(), out[2].cpu().numpy())
    forest.close()
    if not args.no_cpu:
        # the reference's per-mesh CPU path on every 64th mesh, and parity of the batched results on those meshes
        # (FP32 bit-exact against the oracle's lowest-index mode; FP64 re-check against the FP64 oracle)
        O = _oracle()
        meshes = []
        for m in range(0, num_meshes, 64):
            Fm = F[foff[m]:foff[m + 1]]
            lo, hi = int(Fm.min()), int(Fm.max()) + 1
            meshes.append((V[lo:hi].cpu().numpy(), (Fm - lo).cpu().numpy(), Q[qoff_h[m]:qoff_h[m + 1]].cpu().numpy()))
        res["cpu_baseline"] = cpu_time("cfg3", meshes)
        eq32 = eq64 = True
        checked = 0
        worst = worst32 = 0.0
        differ32 = 0
        for j, (v, f, q) in enumerate(meshes):
            s = slice(qoff_h[64 * j], qoff_h[64 * j + 1])
            ri, rd2, rcp = O.MeshIndex(v, f).closest_contract(q)
            oi, od2, _ = O.MeshIndex(v, f, fp64=True).closest_contract(q)
            i32, d32, c32 = (x[s] for x in results["fp32"])
            i64, d64 = results["fp64"][0][s], results["fp64"][1][s]
            eq32 = eq32 and np.array_equal(i32, ri) and np.array_equal(d32, np.sqrt(rd2.astype(np.float32))) \
                and np.array_equal(c32, rcp.astype(np.float32))
            eq64 = eq64 and np.array_equal(i64, oi)
            od = np.sqrt(od2)
            worst = max(worst, float(np.max(np.abs(d64 - od) / np.maximum(od, 1e-30))))
            # the reference's FP32 answer against the FP64 nearest element (the FP64 oracle)
            worst32 = max(worst32, float(np.max(np.abs(d32.astype(np.float64) - od) / np.maximum(od, 1e-30))))
            differ32 += int(np.count_nonzero(i32 != oi))
            checked += len(q)
        res["parity"] = {"meshes_checked": len(meshes), "queries_checked": checked,
                         "fp32_bit_exact": bool(eq32), "fp64_indices_equal_fp64_oracle": bool(eq64),
                         "fp64_max_rel_distance_error_vs_fp64_oracle": worst,
                         "fp32_max_rel_distance_error_vs_fp64_oracle": worst32,
                         "fp32_elements_differing_from_fp64_oracle": differ32}
    # the plain drop-in loop: per mesh, build its BVH and run one closest-element call (query time only is timed)
    t_build = 0.0
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(num_meshes)]
    for m in range(num_meshes):
        Fm = F[foff[m]:foff[m + 1]]
        lo = int(Fm.min())
        hi = int(Fm.max()) + 1
        t0 = time.perf_counter()
        bvh = T.MeshBvh(V[lo:hi], Fm - lo, layouts=1)
        t_build += time.perf_counter() - t0
        Qm = Q[qoff_h[m]:qoff_h[m + 1]]
        ev[m][0].record()
        idx, _, _ = bvh.closest_element(Qm, closest_points=False)
        ev[m][1].record()
        bvh.close()
    torch.cuda.synchronize()
    q_ms = sum(a.elapsed_time(b) for a, b in ev)
    res["plain_loop"] = {"value": nq / (q_ms / 1e3) / 1e6, "unit": "Mqueries/s", "query_ms": q_ms,
                         "build_s": t_build, "meshes": num_meshes,
                         "roofline_frac": algo / (q_ms / 1e3) / 1e9 / peaks()[0]}
    res["batched_vs_plain_fp32"] = res["batched_fp32"]["value"] / res["plain_loop"]["value"]
    res["batched_vs_plain_fp64"] = res["batched_fp64"]["value"] / res["plain_loop"]["value"]
    return res


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if "RANK" in os.environ else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.case:
        CASES[args.case]()
        return
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
