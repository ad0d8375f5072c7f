"""Benchmark: BVH ray casting (Accel::Intersect) on the synthetic ray-cast scene.

Workload (one "step"): closest-hit queries of 16,777,216 rays (origins uniform
in [-0.1,1.1]^3, directions uniform on the sphere, tmin 1e-4) against
1,524,288 triangles (1,000,000 seeded random triangles with lognormal edge
lengths in the unit cube plus a 512x512-quad sinusoid heightfield), on a BVH
built once on the GPU.  Metric: Mrays/s.

  value  rays already resident in HBM, K back-to-back traversal launches timed
         with CUDA events on the launching stream;
  e2e    the same query through the host-pointer C-ABI call (lmgpu_trace) with
         pinned host buffers: host->device rays, traversal, device->host hits
         inside the timed region.

`--impl reference` times the reference's fastest native accel, accel::qbvh,
on all host cores over the same rays: the oracle's C restatement of it
(bit-identical hits), or with --use-ref-binary on an x86-64 host the
reference's own sources compiled by oracle/build_ref.sh.

Under torchrun each rank traces its own 16.8M rays against a replicated BVH
(weak scaling); rank 0 prints the JSON line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "lightmetrica-v2_gb300"))

from lmgpu.dist import aggregate_rate, dist_env, max_over_ranks, ray_stream  # noqa: E402

METRIC = "Mrays/s (BVH)"
UNIT = "Mrays/s"
N_RANDOM, HF_RES, N_RAYS = 1_000_000, 512, 1 << 24
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES = 80, 48, 32, 16


def workload_config(extra: dict | None = None) -> dict:
    c = {"workload": "bvh_raycast_closest_hit", "triangles": N_RANDOM + 2 * HF_RES * HF_RES, "rays_per_step": N_RAYS,
         "scene": "1M random tris (lognormal edges, mu=ln 0.005, sigma=0.5) + 512x512 heightfield, seed 0x5EED",
         "tmin": 1e-4, "query": "closest-hit", "l2": "inputs larger than L2 (512 MiB of rays per step), no flush"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak(key: str = "hbm_gbs") -> tuple[float, str]:
    """A measured peak of the GB300s (hbm_gbs: copy GB/s; bf16_tflops:
    cuBLAS bf16 burst TFLOP/s), else the stated fallback."""
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))[key]), f"measured (MEASURED_PEAKS.json {key}, burst)"
    return (6800.0 if key == "hbm_gbs" else 1900.0), "fallback"


def traffic_per_launch() -> float | None:
    """DRAM bytes per full launch from the committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", "trace_closest_traffic.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["dram_bytes_per_full_launch"])
        except Exception:
            return None
    return None


def l2_figures() -> dict | None:
    """L2 throughput of the traversal from the committed ncu summary: the
    level the node and triangle fetches actually hit."""
    p = os.path.join(REPO, "profiles", "trace_closest_traffic.json")
    try:
        return dict(json.load(open(p))["l2"])
    except Exception:
        return None


class CpuReference:
    """The reference's fastest native accel, accel::qbvh, on the host cores.

    kind "port": the oracle's C restatement of accel::qbvh (oracle/, pinned
    bit for bit to the reference's own qbvh: hit ids and points), which runs
    on any host; kind "reference": the reference's own accel::qbvh compiled
    from its sources by oracle/build_ref.sh (x86-64 only: the reference forces
    SSE), used when --use-ref-binary is given and the binary exists.
    """

    def __init__(self, tris: np.ndarray, threads: int, use_ref_binary: bool = False):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import lmoracle

        self.lo = lmoracle
        self.tris = tris
        self.threads = threads
        self.kind = "port"
        self.build_s = None
        if use_ref_binary and os.path.exists(lmoracle.REF_ACCEL) and os.access(lmoracle.REF_ACCEL, os.X_OK):
            self.kind = "reference"
            self.acc = None
        else:
            t0 = time.perf_counter()
            self.acc = lmoracle.OracleAccel(lmoracle.QBVH, tris)
            self.build_s = time.perf_counter() - t0

    def describe(self) -> str:
        if self.kind == "reference":
            return f"reference accel::qbvh compiled from its sources, {self.threads} threads, build excluded"
        return (f"oracle restatement of accel::qbvh (accel_qbvh.cpp:152-497; bit-identical hits to the "
                f"reference's), {self.threads} threads, build excluded")

    def trace(self, rays: np.ndarray) -> float:
        """Traces every ray; returns the seconds spent tracing."""
        if self.kind == "reference":
            with tempfile.TemporaryDirectory() as tmp:
                ps, pr, po = (os.path.join(tmp, x) for x in ("s.bin", "r.bin", "o.bin"))
                self.lo.write_ref_inputs(ps, pr, [self.tris], rays)
                out = subprocess.run([self.lo.REF_ACCEL, "accel::qbvh", ps, pr, po, str(self.threads)],
                                     capture_output=True, text=True, check=True).stdout
            return float(json.loads(out.strip().splitlines()[-1])["trace_s"])
        t0 = time.perf_counter()
        self.acc.trace(rays, threads=self.threads)
        return time.perf_counter() - t0

    def time_sample(self, rays: np.ndarray, budget_s: float) -> dict:
        """Traces a prefix of `rays` sized to about budget_s seconds."""
        n = min(len(rays), 1 << 14)
        est = n / max(self.trace(rays[:n]), 1e-9)
        m = int(min(len(rays), max(n, est * budget_s)))
        dt = self.trace(rays[:m])
        return {"rays_per_s": m / dt, "n": m, "s": dt,
                "sample": f"{m} rays of the step, {self.describe()}, {dt:.1f} s"}


def run_reference(args) -> None:
    """The reference arm: accel::qbvh on all host cores over the same scene
    and rays.  Warm-up steps trace 2^16 rays each; every timed step traces
    all 16,777,216 rays of the step when the whole run fits in about four
    minutes, else the same prefix of each step's rays (marked sampled)."""
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    from lmgpu import scenes

    tris = scenes.raycast_scene(N_RANDOM, HF_RES)
    rays = scenes.raycast_rays(N_RAYS)
    threads = os.cpu_count() or 1
    ref = CpuReference(tris, threads, use_ref_binary=args.use_ref_binary)
    for k in range(args.warmup):
        ref.trace(rays[k << 16:(k + 1) << 16])
    probe = 1 << 18
    est = probe / ref.trace(rays[:probe])
    per_step = int(min(N_RAYS, max(probe, est * 240.0 / max(1, args.steps))))
    per_step = N_RAYS if per_step >= N_RAYS else per_step
    secs = [ref.trace(rays[:per_step]) for _ in range(args.steps)]
    total = float(sum(secs))
    v = per_step * args.steps / total / 1e6
    sample = (f"per step: {'all' if per_step == N_RAYS else 'the first'} {per_step} rays of the step, "
              f"{ref.describe()}")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(), "impl": "reference",
            "sampled": per_step < N_RAYS, "rays_traced_per_step": per_step,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": ref.kind, "sample": sample,
                             "accel": "accel::qbvh", "build_s": ref.build_s},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import lmgpu
    from lmgpu import scenes

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    tris = scenes.raycast_scene(N_RANDOM, HF_RES)
    nr = args.rays
    rays = scenes.raycast_rays(nr, stream=ray_stream(rank))
    stream = torch.cuda.Stream()
    s = stream.cuda_stream
    acc = lmgpu.Accel()
    with torch.cuda.stream(stream):
        d_tris = torch.from_numpy(tris).cuda()
        acc.build_device(d_tris.data_ptr(), tris.shape[0], s)
        d_rays = torch.from_numpy(rays).cuda()
        d_hits = torch.empty((nr, 4), dtype=torch.float32, device="cuda")
    info = acc.info()
    ah = bool(args.anyhit)

    # fetch counts of the same query (instrumented kernel, outside the timed region)
    st = acc.trace_stats_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, ah, s)
    bytes_per_ray = RAY_BYTES + HIT_BYTES + (st["node_fetches"] * NODE_BYTES + st["triangle_fetches"] * TRI_BYTES) / nr

    for _ in range(args.warmup):
        acc.trace_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, ah, s)
    acc.check(s)
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        acc.trace_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, ah, s)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    acc.check(s)
    ms = ev0.elapsed_time(ev1)

    # e2e: host buffers through the C ABI, copies inside the timed region
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((nr, 4), dtype=torch.float32).pin_memory()
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(2):
        acc.trace_ptr(h_rays.data_ptr(), h_hits.data_ptr(), nr, ah)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        acc.trace_ptr(h_rays.data_ptr(), h_hits.data_ptr(), nr, ah)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    single = single_ray_latency(acc, rays, ah) if rank == 0 else None

    # the slowest rank's times; the rate covers all ranks' rays
    ms, e2e_s = max_over_ranks([ms, e2e_s], device="cuda")

    if rank == 0:
        per_launch_s = ms / 1e3 / args.steps
        value = aggregate_rate(nr, ws, per_launch_s) / 1e6
        e2e_value = aggregate_rate(nr * e2e_steps, ws, e2e_s) / 1e6
        peak, peak_src = measured_peak()
        achieved = nr * bytes_per_ray / per_launch_s / 1e9
        # the committed capture is of the closest-hit kernel; its DRAM bytes
        # grow with the rays a launch processes
        traffic = traffic_per_launch()
        traffic = None if (ah or traffic is None) else traffic * nr / N_RAYS
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": workload_config({"parallelism": f"replicated BVH, rays sharded x{ws}" if ws > 1 else "1 GPU",
                                           "rays_per_step": nr, "query": "any-hit" if ah else "closest-hit"}),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nr * RAY_BYTES,
                        "d2h_bytes_per_step": nr * HIT_BYTES, "steps": e2e_steps,
                        "api": "lmgpu_trace (host pointers, pinned)"},
                "gpu_launches": args.steps,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                             "kernel": "k_trace<anyhit>" if ah else "k_trace<closest>",
                             "bytes_per_ray": bytes_per_ray,
                             "nodes_per_ray": st["node_fetches"] / nr,
                             "tris_per_ray": st["triangle_fetches"] / nr,
                             "note": "algorithmic bytes = 32 B ray + 16 B hit + 80 B per node fetch + 48 B per "
                                     "triangle test; node/triangle fetches are mostly L2 hits",
                             "l2": None if ah else l2_figures()},
                "clocks": clk,
                "accel": {"build_ms": info["build_ms"], "wide_nodes": info["num_wide_nodes"],
                          "binary_depth": info["binary_depth"], "wide_depth": info["wide_depth"],
                          "hit_fraction": st["hits"] / nr},
                "single_ray": single}
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            cb = CpuReference(tris, threads).time_sample(rays, 15.0)
            line["cpu_baseline"] = {"value": cb["rays_per_s"] / 1e6, "unit": UNIT, "cores": threads,
                                    "kind": "port", "accel": "accel::qbvh", "sample": cb["sample"]}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_surface(args) -> None:
    """Surface geometry at hits (lmgpu_surface_device, the batched
    IntersectionUtils::CreateTriangleIntersection): closest hits of the
    ray-cast configuration's rays on its scene, every triangle with vertex
    normals and texcoords.  Metric Mhits/s (rays per second through the
    kernel, misses included); value = device-resident hits and planes, e2e =
    the host-pointer lmgpu_surface (rays and hits in, 23 planes out)."""
    import torch

    import lmgpu
    from lmgpu import scenes

    tris = scenes.raycast_scene(N_RANDOM, HF_RES)
    nt = tris.shape[0]
    g = np.random.default_rng(0x5EED)
    gn = np.cross(tris[:, 3:6] - tris[:, 0:3], tris[:, 6:9] - tris[:, 0:3])
    gn /= np.maximum(np.linalg.norm(gn, axis=1, keepdims=True), 1e-30)
    nrm = (np.repeat(gn, 3, axis=0).reshape(-1, 9) + g.normal(scale=0.1, size=(nt, 9))).astype(np.float32)
    tc = g.uniform(size=(nt, 6)).astype(np.float32)
    nr = args.rays
    rays = scenes.raycast_rays(nr, stream=3)
    stream = torch.cuda.Stream()
    s = stream.cuda_stream
    acc = lmgpu.Accel()
    acc.build(tris)
    acc.set_attributes(nrm, tc)
    with torch.cuda.stream(stream):
        d_rays = torch.from_numpy(rays).cuda()
        d_hits = torch.empty((nr, 4), dtype=torch.float32, device="cuda")
        d_out = torch.empty((23, nr), dtype=torch.float32, device="cuda")
    acc.trace_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, False, s)
    acc.check(s)
    hits = d_hits.cpu().numpy().view(np.int32)[:, 1]
    n_hit = int((hits >= 0).sum())
    for _ in range(args.warmup):
        acc.surface_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, d_out.data_ptr(), s)
    acc.check(s)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)  # 256 MiB write: L2 holds none of the inputs when the step starts
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        acc.surface_device(d_rays.data_ptr(), d_hits.data_ptr(), nr, d_out.data_ptr(), s)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
    clk = clocks.stop()
    acc.check(s)
    per_s = total_ms / 1e3 / args.steps
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = d_hits.cpu().pin_memory()
    h_out = torch.empty((23, nr), dtype=torch.float32).pin_memory()
    lib = lmgpu.lib()
    e2e_steps = 3
    lib.lmgpu_surface(acc.handle, h_rays.data_ptr(), h_hits.data_ptr(), nr, h_out.data_ptr())
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        if lib.lmgpu_surface(acc.handle, h_rays.data_ptr(), h_hits.data_ptr(), nr, h_out.data_ptr()) != 0:
            raise RuntimeError(lib.lmgpu_last_error().decode())
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # algorithmic bytes, whatever the layout: a hit reads its hit record (16 B), ray (32 B), the
    # triangle's vertices (36 B), vertex normals (36 B), texcoords (24 B) and flags (1 B); a miss its
    # hit record; every ray writes 23 floats (92 B)
    hit_b, miss_b = 16 + 32 + 36 + 36 + 24 + 1 + 92, 16 + 92
    alg = n_hit * hit_b + (nr - n_hit) * miss_b
    peak, peak_src = measured_peak()
    achieved = alg / per_s / 1e9
    line = {"metric": "Mhits/s (surface geometry at hits)", "value": nr / per_s / 1e6, "unit": "Mhits/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded): the ray-cast scene with random vertex normals and texcoords",
            "config": {"workload": "surface_geometry_raycast_hits", "triangles": nt, "rays_per_step": nr,
                       "hit_fraction": n_hit / nr, "l2": "flushed before every timed step (256 MiB write)"},
            "e2e": {"value": nr / e2e_s / 1e6, "unit": "Mhits/s", "h2d_bytes_per_step": nr * (32 + 16),
                    "d2h_bytes_per_step": nr * 92, "steps": e2e_steps, "api": "lmgpu_surface (host pointers)"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src, "kernel": "k_surface",
                         "bytes_per_ray": alg / nr,
                         "note": "algorithmic bytes: hit 237 B (hit record, ray, vertices, normals, texcoords, "
                                 "flags, 92 B out), miss 108 B; the kernel reads one 128-byte surface record "
                                 "per hit"},
            "clocks": clk}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import lmoracle

        m = min(nr, 1 << 21)
        hh = d_hits[:m].cpu().numpy()
        hin = np.stack([hh[:, 0], hh.view(np.int32)[:, 1].astype(np.float64), hh[:, 2], hh[:, 3]], 1)
        t0 = time.perf_counter()
        lmoracle.surface(tris, nrm, tc, None, rays[:m], hin)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": m / dt / 1e6, "unit": "Mhits/s", "cores": 1, "kind": "port",
                                "sample": f"{m} hits of the step, oracle restatement of CreateTriangleIntersection "
                                          f"(FP64, 1 thread), {dt:.1f} s"}
    print(json.dumps(line), flush=True)
    acc.close()


RENDER_WORKLOADS = {
    # renderer::pt on the Cornell-style box: 256 x 256, 64 spp, max_num_vertices 9 (8 segments)
    "pt": {"renderer": "pt", "workload": "pt_cornell_256x256_64spp", "width": 256, "height": 256, "spp": 64,
           "max_num_vertices": 9, "data": "synthetic (procedural Cornell box)", "cpu_spp": 8},
    # renderer::bdpt on the caustic room: 1280 x 720, 32 spp, path length 10 (10 segments, so
    # max_num_vertices 11), all (s, t) strategies
    "bdpt": {"renderer": "bdpt", "workload": "bdpt_caustic_room_1280x720_32spp", "width": 1280, "height": 720,
             "spp": 32, "max_num_vertices": 11,
             "data": "synthetic (procedural room, level-5 glass icosphere, sphere light behind a panel)",
             "cpu_spp": 1},
    # renderer::ptmis / renderer::ptdirect (next-event estimation) on the Cornell-style box:
    # 256 x 256, 64 spp, max_num_vertices 9
    "ptmis": {"renderer": "ptmis", "workload": "ptmis_cornell_256x256_64spp", "width": 256, "height": 256,
              "spp": 64, "max_num_vertices": 9, "data": "synthetic (procedural Cornell box)", "cpu_spp": 4},
    "ptdirect": {"renderer": "ptdirect", "workload": "ptdirect_cornell_256x256_64spp", "width": 256, "height": 256,
                 "spp": 64, "max_num_vertices": 9, "data": "synthetic (procedural Cornell box)", "cpu_spp": 4},
    # renderer::ltdirect (light tracing, a sensor connection per vertex) on the Cornell-style box:
    # 256 x 256 x 64 light paths, max_num_vertices 9
    "ltdirect": {"renderer": "ltdirect", "workload": "ltdirect_cornell_256x256_64spp", "width": 256, "height": 256,
                 "spp": 64, "max_num_vertices": 9, "data": "synthetic (procedural Cornell box)", "cpu_spp": 8},
}


def single_ray_latency(acc, rays, anyhit: bool, calls: int = 2000) -> dict:
    """Latency of the single-ray path a stock CPU renderer takes through
    accel::cuda's Accel3::Intersect: lmgpu_trace with n = 1 from pageable host
    memory, a new ray per call (wall clock around each call from Python, so
    about a microsecond of ctypes overhead is included)."""
    warm = 50
    r = np.ascontiguousarray(rays[:calls + warm])
    hit = np.empty(4, np.float32)
    for i in range(warm):
        acc.trace_ptr(r[i].ctypes.data, hit.ctypes.data, 1, anyhit)
    ts = np.empty(calls)
    for i in range(calls):
        t0 = time.perf_counter()
        acc.trace_ptr(r[warm + i].ctypes.data, hit.ctypes.data, 1, anyhit)
        ts[i] = time.perf_counter() - t0
    return {"us_median": float(np.median(ts) * 1e6), "us_mean": float(ts.mean() * 1e6),
            "Mrays_s_one_caller": float(1.0 / ts.mean() / 1e6), "calls": calls,
            "api": "lmgpu_trace with n = 1, pageable host buffers (accel::cuda's Accel3::Intersect)"}


def render_trace_roofline(sc, render, step_ms: float, flush) -> dict:
    """Roofline of a render's dominant kernel, its traversal launches (sc: the
    Scene or Batch whose trace profile is read): one
    render (seed of the first timed step) with the counting traversal for
    rays, node and triangle fetches, then the same render with CUDA events
    around each production traversal launch (the library's trace profile),
    L2 flushed before each.  achieved = algorithmic bytes of those launches
    (32 B ray + 16 B hit + 80 B per node fetch + 48 B per triangle test) /
    their summed device time."""
    import lmgpu

    sc.set_trace_profile(lmgpu.TRACE_PROFILE_COUNT)
    flush.fill_(1.0)
    render(1000)
    cnt = sc.read_trace_profile()
    sc.set_trace_profile(lmgpu.TRACE_PROFILE_TIME)
    flush.fill_(2.0)
    render(1000)
    tim = sc.read_trace_profile()
    sc.set_trace_profile(lmgpu.TRACE_PROFILE_OFF)
    if cnt["rays"] == 0 or tim["timed_launches"] == 0 or tim["timed_launches"] != tim["launches"]:
        return None
    nbytes = (cnt["rays"] * (RAY_BYTES + HIT_BYTES) + cnt["node_fetches"] * NODE_BYTES
              + cnt["triangle_fetches"] * TRI_BYTES)
    achieved = nbytes / (tim["device_ms"] * 1e-3) / 1e9
    peak, peak_src = measured_peak()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_src, "kernel": "k_trace (the render's traversal launches)",
            "launches_per_step": tim["launches"], "rays_per_step": cnt["rays"],
            "bytes_per_ray": nbytes / cnt["rays"], "nodes_per_ray": cnt["node_fetches"] / cnt["rays"],
            "tris_per_ray": cnt["triangle_fetches"] / cnt["rays"], "trace_ms_per_step": tim["device_ms"],
            "share_of_step": tim["device_ms"] / step_ms,
            "note": "algorithmic bytes = 32 B ray + 16 B hit + 80 B per node fetch + 48 B per triangle test over "
                    "the summed device time of the render's traversal launches (CUDA events); a BVH that fits "
                    "in L1 serves most node and triangle fetches from L1"}


def run_render(args) -> None:
    """Rendering configurations (renderer::pt, renderer::bdpt, renderer::ltdirect).  Metric
    Msamples/s; value = film left on the device (lmgpu_render_*_device),
    e2e = the host-pointer lmgpu_render_* (film and variance copied back
    every step).  Under torchrun every rank renders its own sample set of the
    view (seeds from rank_seed, weak scaling); the e2e step ends with the film
    sum of all ranks (reduce_film), and the rate covers all ranks' samples
    over the slowest rank's time."""
    import torch

    import lmgpu
    from lmgpu import scenes
    from lmgpu.dist import rank_seed, reduce_film

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    cfg = RENDER_WORKLOADS[args.workload]
    W, H, spp, max_nv = cfg["width"], cfg["height"], cfg["spp"], cfg["max_num_vertices"]
    if args.spp:
        spp = args.spp
    scene = scenes.caustic_room(W, H) if cfg["renderer"] == "bdpt" else scenes.cornell_box(W, H)
    stream = torch.cuda.Stream()
    sc = lmgpu.Scene(scene)
    render_dev = getattr(sc, f"render_{cfg['renderer']}_device")
    render_host = getattr(sc, f"render_{cfg['renderer']}")
    di = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    samples = W * H * spp
    for k in range(args.warmup):
        render_dev(di.data_ptr(), dv.data_ptr(), spp, max_nv, rank_seed(k, rank), stream.cuda_stream)
    torch.cuda.synchronize()
    # each step timed alone with events on the render stream; L2 flushed
    # (a 256 MiB write, untimed) before every step
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = sc.launch_count()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            render_dev(di.data_ptr(), dv.data_ptr(), spp, max_nv, rank_seed(1000 + k, rank), stream.cuda_stream)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = sc.launch_count() - l0
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    roofline = None
    if rank == 0:
        with torch.cuda.stream(stream):
            roofline = render_trace_roofline(
                sc, lambda seed: render_dev(di.data_ptr(), dv.data_ptr(), spp, max_nv, seed, stream.cuda_stream),
                ms, flush)
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        img, var = render_host(spp, max_nv, rank_seed(2000 + k, rank))
        reduce_film(img, var, spp, device="cuda")
    e2e_s = (time.perf_counter() - t0) / args.steps
    barrier()
    ms, e2e_s = max_over_ranks([ms, e2e_s], device="cuda")
    if rank != 0:
        sc.close()
        return
    ntri = int(sum(p["tris"].shape[0] for p in scene["prims"]))
    line = {"metric": f"Msamples/s (renderer::{cfg['renderer']})",
            "value": aggregate_rate(samples, ws, ms * 1e-3) / 1e6,
            "unit": "Msamples/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": cfg["data"],
            "config": {"workload": cfg["workload"] if spp == cfg["spp"] else f"{cfg['workload']} at {spp} spp",
                       "width": W, "height": H, "spp": spp,
                       "max_num_vertices": max_nv, "triangles": ntri,
                       "l2": "flushed before every timed step (256 MiB write, untimed)",
                       "parallelism": f"replicated scene, samples sharded x{ws}, films summed" if ws > 1
                       else "1 GPU"},
            "e2e": {"value": aggregate_rate(samples, ws, e2e_s) / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 3 * 4 * 2,
                    "api": f"lmgpu_render_{cfg['renderer']} (host film)" + (", reduce_film over ranks" if ws > 1
                                                                            else "")},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import lmoracle

        threads = os.cpu_count() or 1
        n_cpu = W * H * cfg["cpu_spp"]
        fn = getattr(lmoracle, f"render_{cfg['renderer']}")
        t0 = time.perf_counter()
        fn(scene, n_cpu, max_nv, 5, threads)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": n_cpu / cpu_s / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{n_cpu} samples ({cfg['cpu_spp']} spp) of the same scene, oracle restatement of "
                      f"renderer::{cfg['renderer']} (renderer_{cfg['renderer']}.cpp), {threads} threads"}
    print(json.dumps(line), flush=True)
    sc.close()


# renderer::vcm on the Cornell-style box: 256 x 256, 4 passes of 262,144 eye samples (4 per pixel) and
# 262,144 photon subpaths, max_num_vertices 8, initial radius 0.02 (the box is 1 unit wide), alpha 0.7
VCM_WORKLOAD = {"workload": "vcm_cornell_256x256_4x4spp", "width": 256, "height": 256, "max_num_vertices": 8,
                "passes": 4, "eye_spp": 4, "photons": 262144, "initial_radius": 0.02, "alpha": 0.7,
                "data": "synthetic (procedural Cornell box)"}


# Algorithmic bytes of renderer::vcm's photon merges: a query's sort slot,
# each eye-subpath vertex record it reads (32 B), each photon entry scanned in
# its grid cells (16 B), and per photon within the radius the entry again and
# its 80-byte prefix record.
MERGE_QUERY_BYTES, EYE_VERTEX_BYTES, ENTRY_BYTES, MERGE_BYTES = 4, 32, 16, 96


def vcm_merge_roofline(sc, render, step_ms: float, flush) -> dict:
    """Roofline of renderer::vcm's dominant kernel, the photon merge: the
    render of the first timed step's seed once with the counting merge
    (queries, eye-vertex reads, scanned entries, merges) and once with CUDA
    events around each production merge launch (the scene's trace
    profile), L2 flushed before each."""
    import lmgpu

    sc.set_trace_profile(lmgpu.TRACE_PROFILE_COUNT)
    flush.fill_(1.0)
    render(1000)
    cnt = sc.read_trace_profile()
    sc.set_trace_profile(lmgpu.TRACE_PROFILE_TIME)
    flush.fill_(2.0)
    render(1000)
    tim = sc.read_trace_profile()
    sc.set_trace_profile(lmgpu.TRACE_PROFILE_OFF)
    if (cnt["merge_queries"] == 0 or tim["merge_timed_launches"] == 0
            or tim["merge_timed_launches"] != tim["merge_launches"]):
        return None
    nbytes = (cnt["merge_queries"] * MERGE_QUERY_BYTES + cnt["merge_eye_vertices"] * EYE_VERTEX_BYTES
              + cnt["merge_entries"] * ENTRY_BYTES + cnt["merges"] * MERGE_BYTES)
    achieved = nbytes / (tim["merge_ms"] * 1e-3) / 1e9
    peak, peak_src = measured_peak()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_src, "kernel": "k_vc_merge (the render's photon-merge launches)",
            "launches_per_step": tim["merge_launches"], "queries_per_step": cnt["merge_queries"],
            "eye_vertices_per_query": cnt["merge_eye_vertices"] / cnt["merge_queries"],
            "entries_per_query": cnt["merge_entries"] / cnt["merge_queries"],
            "merges_per_query": cnt["merges"] / cnt["merge_queries"], "bytes_per_query": nbytes / cnt["merge_queries"],
            "merge_ms_per_step": tim["merge_ms"], "share_of_step": tim["merge_ms"] / step_ms,
            "traversal_ms_per_step": tim["device_ms"],
            "note": "algorithmic bytes = 4 B per query + 32 B per eye-vertex record + 16 B per scanned photon entry "
                    "+ 96 B per photon within the radius (entry and prefix record), over the summed device time of "
                    "the merge launches (CUDA events); the photon grid and records stay in L2, so the kernel is "
                    "bound by latency, not by these bytes"}


def run_vcm(args) -> None:
    """renderer::vcm (vertex connection and merging).  Metric Msamples/s: eye
    samples of all passes per second, photon subpaths and the grid build
    included; value = film left on the device (lmgpu_render_vcm_device), e2e =
    lmgpu_render_vcm with the film and variance copied back every step."""
    import torch

    import lmgpu
    from lmgpu import scenes

    cfg = VCM_WORKLOAD
    W, H = cfg["width"], cfg["height"]
    eye_spp = args.spp or cfg["eye_spp"]
    prm = dict(max_num_vertices=cfg["max_num_vertices"], num_iteration_pass=cfg["passes"],
               num_photon_trace_samples=cfg["photons"], num_eye_trace_samples=W * H * eye_spp,
               initial_radius=cfg["initial_radius"], alpha=cfg["alpha"], mode="vcm")
    samples = prm["num_iteration_pass"] * prm["num_eye_trace_samples"]
    scene = scenes.cornell_box(W, H)
    stream = torch.cuda.Stream()
    sc = lmgpu.Scene(scene)
    di = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    for k in range(args.warmup):
        sc.render_vcm_device(di.data_ptr(), dv.data_ptr(), stream.cuda_stream, seed=k, **prm)
    torch.cuda.synchronize()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = sc.launch_count()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            sc.render_vcm_device(di.data_ptr(), dv.data_ptr(), stream.cuda_stream, seed=1000 + k, **prm)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = sc.launch_count() - l0
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    with torch.cuda.stream(stream):
        roofline = vcm_merge_roofline(
            sc, lambda seed: sc.render_vcm_device(di.data_ptr(), dv.data_ptr(), stream.cuda_stream, seed=seed, **prm),
            ms, flush)
    t0 = time.perf_counter()
    for k in range(args.steps):
        sc.render_vcm(seed=2000 + k, **prm)
    e2e_s = (time.perf_counter() - t0) / args.steps
    line = {"metric": "Msamples/s (renderer::vcm)", "value": samples / ms / 1e3, "unit": "Msamples/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": cfg["data"],
            "config": {"workload": cfg["workload"] if eye_spp == cfg["eye_spp"] else f"{cfg['workload']} at "
                                                                                     f"{eye_spp} spp per pass",
                       "width": W, "height": H, **{k: v for k, v in prm.items()},
                       "l2": "flushed before every timed step (256 MiB write, untimed)"},
            "e2e": {"value": samples / e2e_s / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 3 * 4 * 2, "api": "lmgpu_render_vcm (host film)"},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import lmoracle

        # one pass with 1/32 of the eye samples and of the photons, the radius
        # scaled by sqrt(32): the same expected merges per eye vertex
        threads = os.cpu_count() or 1
        f = 32
        cprm = dict(prm, num_iteration_pass=1, num_photon_trace_samples=prm["num_photon_trace_samples"] // f,
                    num_eye_trace_samples=prm["num_eye_trace_samples"] // f,
                    initial_radius=prm["initial_radius"] * f ** 0.5)
        t0 = time.perf_counter()
        lmoracle.render_vcm(scene, 5, threads, **cprm)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": cprm["num_eye_trace_samples"] / cpu_s / 1e6, "unit": "Msamples/s", "cores": threads,
            "kind": "port",
            "sample": f"one pass of {cprm['num_eye_trace_samples']} eye samples and "
                      f"{cprm['num_photon_trace_samples']} photon subpaths at radius "
                      f"{cprm['initial_radius']:.4f} (the same merges per eye vertex as the workload), oracle "
                      f"restatement of renderer::vcm (renderer_vcm.cpp), {threads} threads"}
    print(json.dumps(line), flush=True)
    sc.close()


def run_batch(args) -> None:
    """Batched configuration: 12 seeded sphere-grid scenes (~1.31M triangles
    each, mixed 640x360 / 1280x720 / 1920x1080), 64 spp, max depth 16
    (max_num_vertices 17), roulette after depth 3, all views in one wavefront
    with graph-replayed bounces and autotuned traversal / wave parameters.
    Metric Msamples/s over all views; value = films left on the device, e2e =
    lmgpu_batch_render_pt with host films."""
    import torch

    import lmgpu
    from lmgpu import scenes

    spp = args.spp or 64
    max_nv, rr_depth = 17, 3
    t0 = time.perf_counter()
    scene_dicts = scenes.batch_scenes(0x5EED, 12)
    scs = [lmgpu.Scene(d) for d in scene_dicts]
    b = lmgpu.Batch(scs)
    setup_s = time.perf_counter() - t0
    npix = sum(s.width * s.height for s in scs)
    samples = npix * spp
    tuning = b.tuning() if args.no_autotune else b.autotune(1, max_nv, 99, rr_depth)
    d_img = torch.empty(3 * npix, dtype=torch.float32, device="cuda")
    d_var = torch.empty(3 * npix, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    for k in range(args.warmup):
        b.render_pt_device(d_img.data_ptr(), d_var.data_ptr(), spp, max_nv, k, rr_depth, stream.cuda_stream)
    torch.cuda.synchronize()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    l0 = b.launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            b.render_pt_device(d_img.data_ptr(), d_var.data_ptr(), spp, max_nv, 1000 + k, rr_depth,
                               stream.cuda_stream)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = b.launch_count() - l0
    ms = sum(a.elapsed_time(c) for a, c in evs) / args.steps
    # the traversal launches of the first timed step's render, counted and
    # then timed (bounces launched one by one while the profile is on)
    with torch.cuda.stream(stream):
        roofline = render_trace_roofline(
            b, lambda seed: b.render_pt_device(d_img.data_ptr(), d_var.data_ptr(), spp, max_nv, seed, rr_depth,
                                               stream.cuda_stream), ms, flush)
    if roofline is not None:
        roofline["kernel"] = "k_trace<MULTI> (the batch's multi-scene traversal launches)"
    t1 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for k in range(e2e_steps):
        b.render_pt(spp, max_nv, 2000 + k, rr_depth)
    e2e_s = (time.perf_counter() - t1) / e2e_steps
    ntri = int(sum(sum(p["tris"].shape[0] for p in d["prims"]) for d in scene_dicts))
    line = {"metric": "Msamples/s (batched renderer::pt, 12 views)", "value": samples / ms / 1e3,
            "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (12 seeded sphere-grid scenes)",
            "config": {"workload": "batch_pt_12_scenes_64spp" if spp == 64 else f"batch_pt_12_scenes_{spp}spp",
                       "views": len(scs), "resolutions": [[s.width, s.height] for s in scs], "pixels": npix,
                       "spp": spp, "max_num_vertices": max_nv, "rr_depth": rr_depth, "triangles": ntri,
                       "tuning": tuning, "scene_setup_s": setup_s,
                       "l2": "flushed before every timed step (256 MiB write, untimed)"},
            "e2e": {"value": samples / e2e_s / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": npix * 3 * 4 * 2, "api": "lmgpu_batch_render_pt (host films)"},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import lmoracle

        threads = os.cpu_count() or 1
        d = dict(scene_dicts[0])
        d["camera"] = dict(d["camera"], width=160, height=90)
        n_cpu = 160 * 90 * 4
        t1 = time.perf_counter()
        lmoracle.render_pt(d, n_cpu, max_nv, 5, threads)
        cpu_s = time.perf_counter() - t1
        line["cpu_baseline"] = {
            "value": n_cpu / cpu_s / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{n_cpu} samples of scene 0 at 160x90 (4 spp), oracle restatement of renderer::pt "
                      f"(roulette at every hit), {threads} threads, BVH build included"}
    print(json.dumps(line), flush=True)
    b.close()
    for sc in scs:
        sc.close()


def mlp_timing(g, box) -> dict:
    """Tensor-core MLP kernels: forward on 2^20 queries and one training step
    (forward, backward, Adam) on 2^18 samples, CUDA events, after warm-up."""
    import torch

    nq, nt = 1 << 20, 1 << 18
    gen = np.random.default_rng(3)
    q = np.zeros((nq, 9), np.float32)
    lo, hi = np.array(box[:3]), np.array(box[3:])
    q[:, :3] = gen.uniform(lo, hi, size=(nq, 3))
    for c in (3, 6):
        v = gen.normal(size=(nq, 3))
        q[:, c:c + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    d_q = torch.from_numpy(q).cuda()
    d_raw = torch.empty((nq, 40), dtype=torch.float32, device="cuda")
    d_dir = torch.from_numpy(q[:nt, 6:9].copy()).cuda()
    d_w = torch.ones(nt, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    for _ in range(3):
        g.forward_device(d_q.data_ptr(), nq, d_raw.data_ptr(), st.cuda_stream)
        g.train_step_device(d_q.data_ptr(), d_dir.data_ptr(), d_w.data_ptr(), nt, 1e-6, st.cuda_stream)
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    reps = 10
    e0.record(st)
    for _ in range(reps):
        g.forward_device(d_q.data_ptr(), nq, d_raw.data_ptr(), st.cuda_stream)
    e1.record(st)
    for _ in range(reps):
        g.train_step_device(d_q.data_ptr(), d_dir.data_ptr(), d_w.data_ptr(), nt, 1e-6, st.cuda_stream)
    e2.record(st)
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / reps
    train_ms = e1.elapsed_time(e2) / reps
    flop_fwd = 2 * (128 * 64 + 3 * 64 * 64 + 64 * 48)  # per query, padded shapes as issued
    peak, peak_src = measured_peak(key="bf16_tflops")
    fwd_tflops = nq * flop_fwd / (fwd_ms * 1e-3) / 1e12

    return {"forward_queries": nq, "forward_ms": fwd_ms, "forward_Mqueries_per_s": nq / fwd_ms / 1e3,
            "train_step_samples": nt, "train_step_ms": train_ms,
            "roofline": {"bound": "tensor", "achieved": fwd_tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": fwd_tflops / peak, "peak_source": peak_src,
                         "note": "forward FLOPs as issued (128-wide input, 48-wide output)"}}


def relmse_image(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    """relMSE of a film against the reference: mean over pixels and channels
    of (img - ref)^2 / (ref^2 + eps)."""
    return float((((img.astype(np.float64) - ref) ** 2) / (ref * ref + eps)).mean())


class Progressive:
    """FP64 accumulation of a renderer's films over calls of growing sample
    counts: the mean image, the variance of that mean, the render wall time
    (the render calls only, film read-back included) and a curve of relMSE
    against time."""

    def __init__(self, shape):
        self.sum = np.zeros(shape, np.float64)
        self.var_sum = np.zeros(shape, np.float64)
        self.spp = 0
        self.seconds = 0.0
        self.curve = []

    def add(self, img, var, spp, seconds):
        self.sum += img.astype(np.float64) * spp
        self.var_sum += var.astype(np.float64) * float(spp) * float(spp)
        self.spp += spp
        self.seconds += seconds

    def mean(self):
        return self.sum / self.spp

    def variance(self):
        return self.var_sum / float(self.spp) ** 2


def time_to_target(curve, target):
    """Wall time at which relMSE (reference noise removed) first reaches
    target: interpolated in log-log between the checkpoints that bracket it,
    else extrapolated from the last checkpoints with relMSE proportional to
    1 / time (the Monte Carlo rate).  Returns (seconds, extrapolated)."""
    for (t0, _, _, e0), (t1, _, _, e1) in zip(curve, curve[1:]):
        if e1 <= target < e0 and e0 > 0 and e1 > 0:
            f = (np.log(e0) - np.log(target)) / (np.log(e0) - np.log(e1))
            return float(np.exp(np.log(t0) + f * (np.log(t1) - np.log(t0)))), False
    if curve and curve[0][3] <= target:
        return float(curve[0][0]), False
    tail = [c for c in curve[len(curve) // 2:] if c[3] > 0]
    if not tail:
        return None, True
    c = float(np.median([t * e for t, _, _, e in tail]))
    return c / target, True


def guided_trace_roofline(sc, guide, W: int, H: int, spp: int = 256) -> dict:
    """Roofline of the guided renderer's traversal launches: renders of spp
    samples per pixel with the trained network and no training, so that the
    counted and the timed render trace the same rays.  The render's own
    device time (CUDA events, L2 flushed) gives the traversal's share."""
    import torch

    d_img = torch.empty(H * W * 3, dtype=torch.float32, device="cuda")
    d_var = torch.empty_like(d_img)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()

    def render(seed):
        sc.render_pt_guided_device(guide, d_img.data_ptr(), d_var.data_ptr(), spp, -1, seed, train=False,
                                   stream=st.cuda_stream)

    with torch.cuda.stream(st):
        for k in range(3):
            render(500 + k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(0.0)
        e0.record(st)
        render(1000)
        e1.record(st)
        torch.cuda.synchronize()
        step_ms = e0.elapsed_time(e1)
        roofline = render_trace_roofline(sc, render, step_ms, flush)
    if roofline is not None:
        roofline["kernel"] = "k_trace (the guided render's traversal launches)"
        roofline["render"] = {"spp": spp, "ms": step_ms, "Msamples_per_s": W * H * spp / step_ms / 1e3,
                              "training": False}
    return roofline


def run_guiding(args) -> None:
    """Learned path guiding vs plain PT on the narrow-gap room: the wall time
    each method needs to reach relMSE 1e-2 against a converged FP64 image.

    Reference: the unguided BSDF-sampling path tracer with throughput-based
    roulette (unbiased, the integrand of renderer::pt) accumulated in FP64;
    its own remaining noise (the mean of var / (ref^2 + eps)) is subtracted
    from every measured relMSE.  Arms, each accumulated in FP64 over render
    calls of doubling sample counts, timed around the render calls:
      plain      renderer::pt as the drop-in (lmgpu_render_pt, roulette 0.5);
      unguided   the guided tracer's code with no network (alpha 1) and the
                 guided arm's throughput roulette;
      guided     the guided tracer trained online from a fresh network
                 (alpha 0.5, Adam lr 1e-3, batch 2^18).
    An arm that does not reach the target within its time cap is
    extrapolated at relMSE ~ 1 / time from its last checkpoints (marked).
    value = time(guided) / time(plain); the target is <= 0.5."""
    import torch  # noqa: F401  (CUDA context for the MLP timing)

    import lmgpu
    from lmgpu import scenes

    W, H = (int(x) for x in os.environ.get("LMGPU_GUIDING_RES", "480x270").split("x"))
    target = 1e-2
    cap = float(os.environ.get("LMGPU_GUIDING_CAP_SECONDS", "120"))
    ref_spp = int(os.environ.get("LMGPU_GUIDING_REF_SPP", "65536"))
    s = scenes.narrow_gap_room(W, H)
    box = scenes.scene_box(s)
    if args.mlp_only:
        g = lmgpu.Guide(box, 3)
        print(json.dumps({"workload": "guiding MLP kernels only", "mlp": mlp_timing(g, box)}), flush=True)
        g.close()
        return
    sc = lmgpu.Scene(s)
    shape = (H, W, 3)
    eps = 1e-2

    # reference: FP64 accumulation in chunks of 4,096 spp
    g0 = lmgpu.Guide(box, 1)
    ref = Progressive(shape)
    chunk, seed = 4096, 1000
    while ref.spp < ref_spp:
        n = min(chunk, ref_spp - ref.spp)
        t0 = time.perf_counter()
        img, var, _ = sc.render_pt_guided(g0, n, -1, seed, alpha=1.0, train=False, rr_mode=1)
        ref.add(img, var, n, time.perf_counter() - t0)
        seed += 1
    R = ref.mean()
    floor = float((ref.variance() / (R * R + eps)).mean())

    def progressive(render, first_spp, max_chunk, seed0):
        acc = Progressive(shape)
        spp, seed = first_spp, seed0
        while True:
            t0 = time.perf_counter()
            img, var = render(spp, seed)
            acc.add(img, var, spp, time.perf_counter() - t0)
            raw = relmse_image(acc.mean(), R, eps)
            acc.curve.append((acc.seconds, acc.spp, raw, raw - floor))
            if raw - floor <= target or acc.seconds >= cap:
                break
            spp, seed = min(2 * spp, max_chunk), seed + 1
        t, extrap = time_to_target(acc.curve, target)
        return {"time_to_target_s": t, "extrapolated": extrap, "seconds_run": acc.seconds, "spp": acc.spp,
                "final_relmse": acc.curve[-1][3], "final_relmse_raw": acc.curve[-1][2],
                "curve": [[round(a, 4), b, round(c, 6), round(d, 6)] for a, b, c, d in acc.curve]}

    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    l0 = sc.launch_count()
    guide = lmgpu.Guide(box, 3)
    guided = progressive(lambda n, sd: sc.render_pt_guided(guide, n, -1, sd, train=True)[:2], 8, 1024, 20000)
    unguided = progressive(lambda n, sd: sc.render_pt_guided(g0, n, -1, sd, alpha=1.0, train=False, rr_mode=1)[:2],
                           8, 2048, 30000)
    plain = progressive(lambda n, sd: sc.render_pt(n, -1, sd), 8, 4096, 40000)
    launches = sc.launch_count() - l0
    clk = clocks.stop()
    mlp = mlp_timing(guide, box)
    roofline = guided_trace_roofline(sc, guide, W, H)

    tg, tu, tp = guided["time_to_target_s"], unguided["time_to_target_s"], plain["time_to_target_s"]
    ratio = tg / tp
    line = {"metric": "time to relMSE 1e-2, guided PT / plain renderer::pt (narrow-gap room)",
            "value": ratio, "unit": "x", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": tg * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 path arithmetic; bf16 MLP with f32 accumulation; f64 film accumulation",
            "data": "synthetic (narrow-gap room: 14-triangle room with a 0.2-wide slit, 2x2 exterior light Le 50, "
                    "100 tessellated furniture boxes, ~203k triangles)",
            "config": {"workload": "guiding_narrow_gap_room", "width": W, "height": H, "target_relmse": target,
                       "relmse": "mean over pixels and channels of (img - ref)^2 / (ref^2 + 1e-2), minus the "
                                 "reference's own noise",
                       "alpha": 0.5, "learning_rate": 1e-3, "batch": 1 << 18, "time_cap_s": cap,
                       "reference": {"spp": ref.spp, "seconds": ref.seconds, "noise_relmse": floor,
                                     "tracer": "unguided BSDF-sampling path tracing, throughput roulette, FP64 "
                                               "accumulation"},
                       "target_met": bool(ratio <= 0.5),
                       "guided_over_unguided_same_roulette": tg / tu,
                       "unguided_over_plain": tu / tp},
            "arms": {"guided": guided, "unguided_same_roulette": unguided, "plain_renderer_pt": plain},
            "e2e": {"value": ratio, "unit": "x", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 3 * 4 * 2,
                    "api": "lmgpu_render_pt / lmgpu_render_pt_guided (host films)"},
            "gpu_launches": launches, "clocks": clk, "mlp": mlp, "roofline": roofline}
    print(json.dumps(line), flush=True)
    for x in (guide, g0):
        x.close()
    sc.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="rays per step (profiling of smaller cases)")
    ap.add_argument("--anyhit", action="store_true", help="time any-hit queries instead of closest hit")
    ap.add_argument("--spp", type=int, default=0, help="samples per pixel of the render workloads (profiling of "
                                                        "smaller cases; default: the workload's own)")
    ap.add_argument("--workload", choices=["raycast", "pt", "ptmis", "ptdirect", "bdpt", "ltdirect", "vcm", "batch",
                                           "guiding", "surface"],
                    default="raycast",
                    help="raycast: the BVH ray-cast configuration (default); pt: renderer::pt on the Cornell "
                         "box; ptmis / ptdirect: next-event estimation on the Cornell box; bdpt: renderer::bdpt on the caustic room; ltdirect: light tracing on the Cornell "
                         "box; vcm: vertex connection and merging on the Cornell box; batch: 12 scenes in one "
                         "wavefront; "
                         "guiding: time to relMSE 1e-2 of guided, unguided and plain PT; surface: surface geometry "
                         "at the ray-cast hits")
    ap.add_argument("--mlp-only", action="store_true", help="guiding: time the MLP kernels only")
    ap.add_argument("--no-autotune", action="store_true", help="batch: keep the default tuning (profiling runs)")
    ap.add_argument("--use-ref-binary", action="store_true",
                    help="reference arm: time the reference's own qbvh (x86-64 harness) if built")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in RENDER_WORKLOADS:
        run_render(args)
    elif args.workload == "vcm":
        run_vcm(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "guiding":
        run_guiding(args)
    elif args.workload == "surface":
        run_surface(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
