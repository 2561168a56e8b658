"""Traversal benchmark: Mrays/s of the MTBVH closest-hit and any-hit kernels.

Workload (one step): for each triangle-soup scene of N = 1M, 4M, 16M
triangles (centroids uniform in the unit cube, equilateral triangles with
edge U(0.001, 0.01), random orientation; seeds 101/104/116), trace 2^24
coherent primary rays (pinhole at (0.5, -1, 0.5) looking along +y, 45 degree
fov, 4096x4096) and 2^24 incoherent rays (cosine-distributed from the primary
hit points), each as a closest-hit query and as an any-hit query with
tmax ~ U(0, 1): 12 launches and 12 * 2^24 rays per step.  Inputs are seeded
synthetic data (the reference publishes no benchmark scenes).

``value`` is device-resident throughput (rays / summed CUDA-event time of the
steps); ``e2e`` is the same metric through the C ABI with pinned host arrays
(host->device copy of rays, kernel, device->host copy of results per call).

``--impl reference`` times the reference algorithm on the host cores: the
reference's traversal is GLSL that needs OpenGL (unavailable on this machine), so
its CPU stand-in is the oracle restatement, run with every host thread on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SIZES = {"1M": 1 << 20, "4M": 1 << 22, "16M": 1 << 24}
SEEDS = {1 << 20: 101, 1 << 22: 104, 1 << 24: 116}
METRIC = "Mrays/s traversal"
UNIT = "Mrays/s"


# kernel of each trace schedule (ZGL_TRACE_* of include/zgl.h); auto resolves
# as the library does
KERNELS = {"thread_per_ray": {"closest": "trace_closest_kernel (no lane budget)",
                              "any": "trace_any_kernel (no lane budget)"},
           "persistent": {"closest": "trace_persistent_kernel<false>", "any": "trace_persistent_kernel<true>"},
           "prefetch": {"closest": "trace_prefetch_kernel<false>", "any": "trace_prefetch_kernel<true>"},
           "auto": {"closest": "trace_closest_kernel (long rays finished by their warps)",
                    "any": "trace_any_kernel (long rays finished by their warps)"}}


def resolved_schedule(schedule: str) -> str:
    return schedule


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sizes", default="1M,4M,16M")
    ap.add_argument("--side", type=int, default=4096, help="primary rays = side^2")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline work")
    ap.add_argument("--ref-rays", type=int, default=1 << 20, help="rays per launch traced by --impl reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--schedule", default="auto", choices=["auto", "thread_per_ray", "persistent", "prefetch"])
    ap.add_argument("--only", default="", help="comma list of launch-name substrings to keep (profiling)")
    ap.add_argument("--render", default="cornell,city,batch,diff", help="render workloads to time ('' for none)")
    ap.add_argument("--render-passes", type=int, default=4, help="timed passes per render workload")
    ap.add_argument("--no-traversal", action="store_true", help="skip the traversal workload (profiling)")
    ap.add_argument("--no-host-build", action="store_true", help="skip timing the host MTBVH builder")
    ap.add_argument("--diff-size", type=int, default=512, help="film side of the differentiable workload")
    ap.add_argument("--diff-spp", type=int, default=32, help="samples per pixel of the differentiable workload")
    ap.add_argument("--batch-requests", type=int, default=64, help="requests of the batched workload")
    ap.add_argument("--batch-no-autotune", action="store_true", help="batched workload with the default schedule")
    ap.add_argument("--batch-schedule", default="", choices=["", "flat", "persistent", "queue"],
                    help="batched workload with this schedule instead of the autotuned one")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device=None) -> float:
    """The largest of every rank's x (the job's time is its slowest rank's);
    x itself outside a process group or with one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 8:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# --------------------------------------------------------------------------
# workload construction
# --------------------------------------------------------------------------
def build_scene(N: int):
    from zillumgl_gb300.synthetic import triangle_soup

    return triangle_soup(N, SEEDS.get(N, 7))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "trace_closest_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


def l2_peak(stream):
    """L2 read bandwidth (GB/s) by the library's own L2-resident read kernel:
    best of 16/32/64 MiB buffers, 200 passes each."""
    import ctypes as C

    from zillumgl_gb300._lib import call

    best, per = 0.0, {}
    for mib in (16, 32, 64):
        v = C.c_double()
        call("zgl_measure_l2_read", mib << 20, 200, C.byref(v), stream.cuda_stream)
        per[f"{mib}MiB"] = round(v.value, 1)
        best = max(best, v.value)
    return best, per


def run_ours(args):
    import torch

    from zillumgl_gb300 import BVH
    from zillumgl_gb300.synthetic import incoherent_rays, primary_rays, shadow_tmax

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.Stream(device=dev)
    if args.no_traversal:  # render workloads only (profiling)
        print(json.dumps({"render": run_render(args, stream, dev)}), flush=True)
        return
    sizes = [SIZES[s] for s in args.sizes.split(",")]
    side = args.side
    nray = side * side

    o_p, d_p = primary_rays(side, side)
    specs = []  # (name, acc, o, d, tmax, query)
    scenes = []
    t_setup = time.time()
    bvh_build = {}
    for N in sizes:
        v, idx = build_scene(N)
        acc, bvh_build[f"{N >> 20}M"] = time_bvh_build(v, idx, dev, stream, host=not args.no_host_build)
        acc.set_trace_schedule(args.schedule)
        log(f"[bench] N={N}: {bvh_build[f'{N >> 20}M']}")
        to = torch.from_numpy(o_p).to(dev)
        td = torch.from_numpy(d_p).to(dev)
        hid, ht = acc.trace_closest(to, td, stream=stream)
        stream.synchronize()
        o_i, d_i = incoherent_rays(v, idx, o_p, d_p, hid.cpu().numpy(), ht.cpu().numpy(), seed=SEEDS.get(N, 7) + 1)
        # the camera sits 1 unit in front of the cube: primary shadow distances are 1 + U(0, 1)
        tm_p = torch.from_numpy(1.0 + shadow_tmax(nray, SEEDS.get(N, 7) + 2)).to(dev)
        tm_i = torch.from_numpy(shadow_tmax(nray, SEEDS.get(N, 7) + 3)).to(dev)
        fam = {"primary": (to, td, tm_p, o_p, d_p), "incoherent": (torch.from_numpy(o_i).to(dev),
                                                                   torch.from_numpy(d_i).to(dev), tm_i, o_i, d_i)}
        for fname, (o, d, tm, oh, dh) in fam.items():
            for q in ("closest", "any"):
                specs.append({"name": f"{N >> 20}M/{fname}/{q}", "N": N, "acc": acc, "o": o, "d": d, "tmax": tm,
                              "o_host": oh, "d_host": dh, "query": q})
        scenes.append((N, v, idx, acc))
        del v, idx
    if args.only:
        keep = [k for k in args.only.split(",") if k]
        specs = [sp for sp in specs if any(k in sp["name"] for k in keep)]
    log(f"[bench] setup {time.time() - t_setup:.1f}s, {len(specs)} launches/step")

    # outputs (device)
    out_id = torch.empty(nray, dtype=torch.int32, device=dev)
    out_t = torch.empty(nray, dtype=torch.float32, device=dev)
    out_occ = torch.empty(nray, dtype=torch.uint8, device=dev)

    # algorithmic bytes: 32 B per table entry visited, 36 B per triangle test,
    # 24 B ray in, 8 B hit out (closest) / 4 B tmax in + 1 B flag out (any)
    for sp in specs:
        vis, tst = sp["acc"].trace_count(sp["o"], sp["d"], sp["tmax"], any_hit=sp["query"] == "any", stream=stream)
        stream.synchronize()
        V = int(vis.sum(dtype=torch.int64).item())
        T = int(tst.sum(dtype=torch.int64).item())
        io = (24 + 8) if sp["query"] == "closest" else (24 + 4 + 1)
        sp["V"], sp["T"] = V, T
        sp["bytes"] = 32 * V + 36 * T + io * nray

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def launch(sp):
        if sp["query"] == "closest":
            sp["acc"].trace_closest(sp["o"], sp["d"], out_id, out_t, stream=stream)
        else:
            sp["acc"].trace_any(sp["o"], sp["d"], sp["tmax"], out_occ, stream=stream)

    def one_step(record):
        evs = []
        for sp in specs:
            if record:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                launch(sp)
                e1.record(stream)
                evs.append((sp, e0, e1))
            else:
                launch(sp)
        return evs

    for _ in range(args.warmup):
        one_step(False)
    stream.synchronize()

    per_launch = {sp["name"]: [] for sp in specs}
    step_ms = []
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush (256 MiB write) outside the timed events
            evs = one_step(True)
            stream.synchronize()
            tot = 0.0
            for sp, e0, e1 in evs:
                ms = e0.elapsed_time(e1)
                per_launch[sp["name"]].append(ms)
                tot += ms
            step_ms.append(tot)
    torch.cuda.synchronize(dev)
    total_ms = max_over_ranks(sum(step_ms), dev)
    rays_per_step = len(specs) * nray
    value = rays_per_step * args.steps * world / (total_ms * 1e-3) / 1e6

    # roofline of the dominant kernel (closest-hit trace)
    closest = [sp for sp in specs if sp["query"] == "closest"]
    anyq = [sp for sp in specs if sp["query"] == "any"]
    t_closest = sum(statistics.mean(per_launch[sp["name"]]) for sp in closest)
    t_any = sum(statistics.mean(per_launch[sp["name"]]) for sp in anyq)
    dom = closest if t_closest >= t_any else anyq
    dom_ms = sum(statistics.mean(per_launch[sp["name"]]) for sp in dom) / len(dom)
    dom_bytes = sum(sp["bytes"] for sp in dom) / len(dom)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = profiled_traffic()
    l2, l2_sweep = l2_peak(stream)
    kname = KERNELS[resolved_schedule(args.schedule)]["closest" if dom is closest else "any"]
    roofline = {"bound": "latency",
                "bound_note": "node and triangle bytes against the L2 / HBM roofline; the measured limiter is "
                              "dependent-load latency and SIMD divergence (warp lanes active per instruction, "
                              "long-scoreboard stalls), not DRAM bandwidth: DRAM traffic is a few percent of the "
                              "algorithmic bytes, which L1 and L2 serve",
                "kernel": kname, "l2_frac": round(achieved / l2, 4), "l2_peak": round(l2, 1),
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": f"{peak_kind} hbm_gbs (copy bandwidth)",
                "l2_peak_source": "zgl_measure_l2_read: L2-resident buffer read by all SMs with 16-byte ld.global.cg, "
                                  f"best of {l2_sweep} GB/s",
                "traffic": traffic.get("dram_bytes_per_launch") if traffic else None,
                "traffic_note": traffic.get("note") if traffic else "no ncu capture committed yet",
                "lanes_active_per_inst": traffic.get("lanes_active_per_inst") if traffic else None,
                "lanes_note": traffic.get("lanes_note") if traffic else None,
                "algorithmic_bytes_per_launch": int(dom_bytes),
                "avg_launch_ms": round(dom_ms, 4)}

    workloads = []
    for sp in specs:
        ms = statistics.mean(per_launch[sp["name"]])
        workloads.append({"name": sp["name"], "ms": round(ms, 4), "mrays_s": round(nray / (ms * 1e-3) / 1e6, 1),
                          "visits_per_ray": round(sp["V"] / nray, 2), "tests_per_ray": round(sp["T"] / nray, 3),
                          "gbs": round(sp["bytes"] / (ms * 1e-3) / 1e9, 1),
                          "l2_frac": round(sp["bytes"] / (ms * 1e-3) / 1e9 / l2, 4)})

    # end to end through the C ABI with pinned host arrays
    e2e = None
    if not args.no_e2e:
        host = {}
        for sp in specs:
            key = (sp["N"], sp["name"].split("/")[1])
            if key not in host:
                host[key] = (torch.from_numpy(sp["o_host"]).pin_memory(), torch.from_numpy(sp["d_host"]).pin_memory(),
                             sp["tmax"].cpu().pin_memory())
            sp["host"] = host[key]
        h_id = torch.empty(nray, dtype=torch.int32).pin_memory()
        h_t = torch.empty(nray, dtype=torch.float32).pin_memory()
        h_occ = torch.empty(nray, dtype=torch.uint8).pin_memory()
        h2d = d2h = 0
        for sp in specs:
            h2d += 24 * nray + (4 * nray if sp["query"] == "any" else 0)
            d2h += (8 if sp["query"] == "closest" else 1) * nray

        def e2e_step():
            for sp in specs:
                o, d, tm = sp["host"]
                if sp["query"] == "closest":
                    sp["acc"].trace_closest(o, d, h_id, h_t, stream=stream)
                else:
                    sp["acc"].trace_any(o, d, tm, h_occ, stream=stream)

        e2e_step()
        stream.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        stream.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
        e2e = {"value": round(rays_per_step * args.steps * world / e2e_s / 1e6, 1), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "note": "C-ABI calls on pinned host arrays: the trace kernels read the rays from and write the hits "
                       "to page-locked host memory over the host link (NVLink-C2C), each call synchronises; "
                       "h2d/d2h bytes are the bytes that cross it"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(scenes, specs, args.ref_rays)
    for N, v, idx, acc in scenes:
        acc.close()
    render = run_render(args, stream, dev) if args.render else None

    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "MTBVH traversal microbench (triangle soups, 2^24 coherent primary + 2^24 "
                                   "incoherent rays, closest-hit and any-hit)",
                       "triangles": sizes, "rays_per_launch": nray, "launches_per_step": len(specs),
                       "parallelism": f"replicas{world}", "l2": "flushed between steps (256 MiB write); inputs > L2"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": len(specs) * args.steps,
            "clocks": clk.summary(), "workloads": workloads, "bvh_build": bvh_build, "render": render}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


# --------------------------------------------------------------------------
# render workloads (secondary metrics): samples/s of the integrators
# --------------------------------------------------------------------------
def time_bvh_build(v, idx, dev, stream, host=True):
    """MTBVH construction of one traversal mesh: the CUDA builder from
    device-resident arrays (best of 3 after a warm-up build), from pageable
    host arrays (copies included), and the host builder on every core.  The
    accelerator returned for tracing is a device-built one (bit-identical)."""
    import torch

    from zillumgl_gb300 import BVH

    tv = torch.from_numpy(v).to(dev)
    ti = torch.from_numpy(idx.view(np.int32)).to(dev)
    torch.cuda.synchronize(dev)
    BVH(tv, ti).build_device(stream=stream).close()
    dev_ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        a = BVH(tv, ti).build_device(stream=stream)
        dev_ms.append((time.perf_counter() - t0) * 1e3)
        a.close()
    del tv, ti
    t0 = time.perf_counter()
    acc = BVH(v, idx).build_device(stream=stream)
    from_host = (time.perf_counter() - t0) * 1e3
    out = {"triangles": int(idx.size // 3), "device_ms": round(min(dev_ms), 2),
           "device_from_host_arrays_ms": round(from_host, 2)}
    if host:
        t0 = time.perf_counter()
        BVH(v, idx).build_host()
        out["host_ms"] = round((time.perf_counter() - t0) * 1e3, 1)
        out["host_threads"] = os.cpu_count()
        out["device_speedup"] = round(out["host_ms"] / out["device_ms"], 1)
    return acc, out


def run_render(args, stream, dev):
    """samples/s of one progressive pass of each integrator (CUDA events over
    `--render-passes` passes after one warm-up pass)."""
    import torch

    from zillumgl_gb300.scene import LightIntegrator, PathIntegrator, Scene, TripleIntegrator
    from zillumgl_gb300.synthetic import city_scene, cornell_scene

    out = {}
    names = [n for n in args.render.split(",") if n]
    for name in names:
        t0 = time.time()
        if name == "batch":
            out[name] = run_batch(args, stream, dev)
            continue
        if name == "diff":
            out[name] = run_diff(args, stream, dev)
            continue
        if name == "cornell":
            data = cornell_scene(seed=1, width=256, height=256)
            runs = [("path", PathIntegrator, dict(max_depth=5))]
        elif name == "city":
            data = city_scene(seed=2)
            runs = [("path", PathIntegrator, dict(max_depth=8, russian_roulette=1, rr_start_depth=3)),
                    ("light", LightIntegrator, dict(max_depth=8, russian_roulette=1, rr_start_depth=3)),
                    ("triple", TripleIntegrator, dict(max_depth=8, russian_roulette=1, rr_start_depth=3))]
        else:
            raise ValueError(name)
        scene = Scene(data)
        W, H = data.film
        log(f"[bench] render scene {name}: {data.obj_indices.size // 3 + data.light_indices.size // 3} tris, "
            f"setup {time.time() - t0:.1f}s")
        res = {"film": [W, H], "triangles": int(data.obj_indices.size // 3 + data.light_indices.size // 3)}
        for kind, cls, params in runs:
            integ = cls(scene, **params)
            integ.render_one_pass(stream)  # warm-up
            stream.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.render_passes):
                integ.render_one_pass(stream)
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / args.render_passes
            if kind == "light":
                paths = 32 * 1536
                res[kind] = {"ms_per_pass": round(ms, 3), "light_paths_per_s": round(paths / (ms * 1e-3), 1),
                             "blocks_per_pass": 32}
            else:
                res[kind] = {"ms_per_pass": round(ms, 3), "samples_per_s": round(W * H / (ms * 1e-3), 1)}
                if kind == "triple":
                    res[kind]["light_paths_per_pass"] = 64 * 1536
            res[kind]["params"] = params
            integ.close()
        if name == "cornell":
            # the configuration's 16 samples per pixel as one multi-pass launch
            integ = PathIntegrator(scene, **runs[0][2])
            integ.render_passes(16, stream)  # warm-up (allocates the pass buffer)
            integ.reset()
            stream.synchronize()
            e0.record(stream)
            for _ in range(args.render_passes):
                integ.reset()
                integ.render_passes(16, stream)
            e1.record(stream)
            stream.synchronize()
            ms16 = e0.elapsed_time(e1) / args.render_passes
            res["path_16spp"] = {"ms_per_render": round(ms16, 3), "samples_per_s": round(W * H * 16 / (ms16 * 1e-3), 1),
                                 "note": "16 passes in one launch (zgl_integrator_render_passes), frame identical "
                                         "to 16 single passes"}
            integ.close()
        if name == "city":
            # the light tracer at a block count that fills the GPU (the reference's
            # default of 32 blocks of 1536 paths holds 49,152 threads)
            nsm = torch.cuda.get_device_properties(dev).multi_processor_count
            full = -(-nsm * 2048 // 1536)
            integ = LightIntegrator(scene, **dict(runs[1][2], blocks_per_pass=full))
            integ.render_one_pass(stream)
            stream.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.render_passes):
                integ.render_one_pass(stream)
            e1.record(stream)
            stream.synchronize()
            lms = e0.elapsed_time(e1) / args.render_passes
            res["light_full_gpu"] = {"ms_per_pass": round(lms, 3), "blocks_per_pass": full,
                                     "light_paths_per_s": round(full * 1536 / (lms * 1e-3), 1),
                                     "note": f"{nsm} SMs x 2048 resident threads / 1536 paths per block"}
            integ.close()
            # the display pass (tone map + gamma) on the 1080p frame: 16 B in, 16 B out per pixel
            from zillumgl_gb300.image import TONE_FILMIC, postprocess

            integ = PathIntegrator(scene, **runs[0][2])
            integ.render_one_pass(stream)
            dframe = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
            integ.get_frame(dframe, stream)
            img = torch.empty_like(dframe)
            postprocess(dframe, W, H, 1.0, TONE_FILMIC, out=img, stream=stream)
            stream.synchronize()
            reps = 20
            e0.record(stream)
            for _ in range(reps):
                postprocess(dframe, W, H, 1.0, TONE_FILMIC, out=img, stream=stream)
            e1.record(stream)
            stream.synchronize()
            pms = e0.elapsed_time(e1) / reps
            peak, _ = measured_peaks()
            # the same pass on an 8192 x 4096 film (1 GiB moved per pass, beyond L2): the HBM roofline
            BW, BH = 8192, 4096
            big = torch.rand((BH, BW, 4), dtype=torch.float32, device=dev)
            bimg = torch.empty_like(big)
            postprocess(big, BW, BH, 1.0, TONE_FILMIC, out=bimg, stream=stream)
            stream.synchronize()
            e0.record(stream)
            for _ in range(reps):
                postprocess(big, BW, BH, 1.0, TONE_FILMIC, out=bimg, stream=stream)
            e1.record(stream)
            stream.synchronize()
            bms = e0.elapsed_time(e1) / reps
            bgbs = BW * BH * 32 / (bms * 1e-3) / 1e9
            res["postprocess"] = {"ms_1080p": round(pms, 4), "ms_8192x4096": round(bms, 3),
                                  "gbs_8192x4096": round(bgbs, 1), "hbm_frac": round(bgbs / peak, 3),
                                  "note": "filmic tone map + pow(1/2.2), 16 B in + 16 B out per pixel; the 1080p "
                                          "frame stays in L2, the 8192x4096 film (1 GiB per pass) does not"}
            del big, bimg
            integ.close()
        # end to end through the C ABI: one pass + the frame read back to pinned host memory
        integ = PathIntegrator(scene, **runs[0][2])
        host = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
        integ.render_one_pass(stream)
        integ.get_frame(host, stream)
        t1 = time.perf_counter()
        for _ in range(args.render_passes):
            integ.render_one_pass(stream)
            integ.get_frame(host, stream)
        e2e_s = (time.perf_counter() - t1) / args.render_passes
        res["path"]["e2e_samples_per_s"] = round(W * H / e2e_s, 1)
        res["path"]["e2e_d2h_bytes_per_pass"] = W * H * 16
        integ.close()
        if not args.no_cpu_baseline:
            res["path"]["cpu_baseline"] = render_cpu_baseline(data, scene, runs[0][2], args.cpu_seconds / 3)
            if name == "city":
                for kind, _, params in runs[1:]:
                    res[kind]["cpu_baseline"] = render_cpu_baseline_splat(data, kind, params, args.cpu_seconds / 3)
        scene.close()
        out[name] = res
    return out


def run_batch(args, stream, dev):
    """Batched serving: 64 seeded requests (1k-500k triangles, 128^2-1024^2,
    4-64 spp, depth 4-8).  Plain = one path-tracer launch per request per
    pass, and one multi-pass launch per request (the stronger baseline);
    batched = the batched renderer (autotuned, graph).  All produce the same
    frames bit for bit.  `speedup` is the median of three timings of one
    multi-pass launch per request over the median of three batched renders."""
    import torch

    from zillumgl_gb300.scene import BatchRenderer, PathIntegrator, Scene
    from zillumgl_gb300.synthetic import batch_requests

    t0 = time.time()
    reqs = batch_requests(seed=3, n=args.batch_requests)
    scenes, frames, total = [], [], 0
    for data, spp, params in reqs:
        scenes.append(Scene(data))
        W, H = data.film
        frames.append(torch.zeros((H, W, 4), dtype=torch.float32, device=dev))
        total += W * H * spp
    log(f"[bench] batch: {len(reqs)} requests, {total / 1e6:.1f}M samples, setup {time.time() - t0:.1f}s")
    # plain: one integrator per request, one launch per pass
    integs = [PathIntegrator(sc, **params) for sc, (_, _, params) in zip(scenes, reqs)]
    integs[0].render_one_pass(stream)
    stream.synchronize()
    for it in integs:
        it.close()
    integs = [PathIntegrator(sc, **params) for sc, (_, _, params) in zip(scenes, reqs)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for it, (_, spp, _) in zip(integs, reqs):
        for _ in range(spp):
            it.render_one_pass(stream)
    e1.record(stream)
    stream.synchronize()
    plain_ms = e0.elapsed_time(e1)
    launches_plain = sum(spp for _, spp, _ in reqs)
    # plain, one multi-pass launch per request (zgl_integrator_render_passes)
    multi = [PathIntegrator(sc, **params) for sc, (_, _, params) in zip(scenes, reqs)]
    for it, (_, spp, _) in zip(multi, reqs):
        it.render_passes(spp, stream)  # warm-up: allocates each pass buffer
        it.reset()
    stream.synchronize()
    multi_runs = []
    for _ in range(3):
        for it in multi:
            it.reset()
        stream.synchronize()
        e0.record(stream)
        for it, (_, spp, _) in zip(multi, reqs):
            it.render_passes(spp, stream)
        e1.record(stream)
        stream.synchronize()
        multi_runs.append(e0.elapsed_time(e1))
    multi_ms = statistics.median(multi_runs)
    for it in multi:
        it.close()
    del multi
    # batched
    sched = {"": {}, "flat": {"schedule": 1}, "persistent": {"schedule": 2}, "queue": {"schedule": 3}}[
        args.batch_schedule]
    batch = BatchRenderer([(sc, spp, params, fr) for sc, (_, spp, params), fr in zip(scenes, reqs, frames)],
                          **sched)
    t1 = time.time()
    tuned = batch.config() if (args.batch_no_autotune or sched) else batch.autotune(stream)
    tune_s = time.time() - t1
    batch.render(stream)  # captures the graph
    stream.synchronize()
    batch_runs = []
    for _ in range(3):
        e0.record(stream)
        batch.render(stream)
        e1.record(stream)
        stream.synchronize()
        batch_runs.append(e0.elapsed_time(e1))
    batch_ms = statistics.median(batch_runs)
    # the other schedules of the batched renderer, for the record
    others = {}
    for nm, sv in (("flat", 1), ("persistent", 2), ("queue", 3)):
        if sv == tuned.get("schedule"):
            continue
        cfg = {"schedule": sv} if sv == 1 else {"schedule": sv, "block_size": 256 if sv == 3 else 128,
                                                 "queue_capacity": 32, "regen_threshold": 16}
        batch.set_config(**cfg)
        batch.render(stream)
        stream.synchronize()
        e0.record(stream)
        batch.render(stream)
        e1.record(stream)
        stream.synchronize()
        others[nm] = {"ms": round(e0.elapsed_time(e1), 2), "config": cfg}
    batch.set_config(**tuned)
    # spot check: the batched frames equal the plain ones
    same = 0
    for it, fr in zip(integs[:4], frames[:4]):
        f, _ = it.get_frame()
        same += int(np.array_equal(f.view(np.uint32), fr.cpu().numpy().view(np.uint32)))
    for it in integs:
        it.close()
    batch.close()
    cpu = None if args.no_cpu_baseline else batch_cpu_baseline(reqs, scenes, args.cpu_seconds / 3)
    for sc in scenes:
        sc.close()
    return {"requests": len(reqs), "samples": total, "cpu_baseline": cpu,
            "plain": {"ms": round(plain_ms, 2), "samples_per_s": round(total / (plain_ms * 1e-3), 1),
                      "launches": launches_plain},
            "plain_one_launch_per_request": {"ms": round(multi_ms, 2), "runs_ms": [round(x, 2) for x in multi_runs],
                                             "samples_per_s": round(total / (multi_ms * 1e-3), 1),
                                             "launches": 2 * len(reqs)},
            "batched": {"ms": round(batch_ms, 2), "runs_ms": [round(x, 2) for x in batch_runs],
                        "samples_per_s": round(total / (batch_ms * 1e-3), 1),
                        "config": tuned, "autotune_s": round(tune_s, 2)},
            "other_schedules": others,
            "speedup": round(multi_ms / batch_ms, 3),
            "speedup_note": "median of 3 one-multi-pass-launch-per-request timings over the median of 3 batched renders",
            "speedup_vs_per_pass_launches": round(plain_ms / batch_ms, 3),
            "frames_bit_identical_checked": f"{same}/4"}


def run_diff(args, stream, dev):
    """Differentiable rendering: the 8-material principled box at 512^2,
    32 spp, depth 6.  The target is rendered at the seed parameters; the
    optimised parameters start perturbed by U(-0.3, 0.3).  One iteration =
    parameter upload, forward (per-sample radiance + mean image), L2 loss
    adjoint, path-replay backward, Adam step; timed with CUDA events over
    `--render-passes` iterations after two warm-up iterations."""
    import torch

    from zillumgl_gb300.scene import DiffRenderer, Scene
    from zillumgl_gb300.synthetic import diff_scene, perturbed_params

    data = diff_scene(seed=11, width=args.diff_size, height=args.diff_size)
    W, H = data.film
    spp, params = args.diff_spp, dict(max_depth=6)
    scene = Scene(data)
    dr = DiffRenderer(scene, spp, **params)
    p_true = dr.params()
    target = dr.forward(stream=stream)
    stream.synchronize()
    p = torch.tensor(perturbed_params(p_true, 8, seed=12), device=dev, requires_grad=True)
    opt = torch.optim.Adam([p], lr=0.01)
    img = torch.empty((H, W, 3), dtype=torch.float32, device=dev)
    losses = []

    def iteration(ev=None):
        dr.set_params(p.detach())
        if ev:
            ev[0].record(stream)
        dr.forward(out=img, stream=stream)
        with torch.cuda.stream(stream):
            diff = img - target
            loss = (diff * diff).mean()
            dimg = diff * (2.0 / diff.numel())
        g = dr.backward(dimg, stream=stream)
        if ev:
            ev[1].record(stream)
        with torch.cuda.stream(stream):
            p.grad = g
            opt.step()
            with torch.no_grad():
                p.clamp_(0.01, 100.0)
        losses.append(loss)

    for _ in range(2):
        iteration()
    stream.synchronize()
    n = max(args.render_passes, 3)
    fb = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(n):
        iteration(fb[k])
    e1.record(stream)
    stream.synchronize()
    it_ms = e0.elapsed_time(e1) / n
    fb_ms = sorted(a.elapsed_time(b) for a, b in fb)[n // 2]
    # kernel split of one forward + backward
    ef = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with torch.cuda.stream(stream):
        dimg = torch.full_like(img, 1e-3)
    ef[0].record(stream)
    dr.forward(out=img, stream=stream)
    ef[1].record(stream)
    dr.backward(dimg, stream=stream)
    ef[2].record(stream)
    stream.synchronize()
    loss_first, loss_last = float(losses[0]), float(losses[-1])
    # the loss step (zgl_diff_step_l2): forward, L2 loss and adjoint queued in one call
    gimg = torch.empty_like(img)
    gbuf = torch.empty(p.numel(), dtype=torch.float32, device=dev)
    lbuf = torch.empty(1, dtype=torch.float32, device=dev)
    for _ in range(2):
        dr.step_l2(target, image=gimg, grad=gbuf, loss=lbuf, stream=stream)
    fe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    for k in range(n):
        fe[k][0].record(stream)
        dr.step_l2(target, image=gimg, grad=gbuf, loss=lbuf, stream=stream)
        fe[k][1].record(stream)
    stream.synchronize()
    fused_ms = sorted(a.elapsed_time(b) for a, b in fe)[n // 2]
    # a full Adam iteration on the fused step
    losses_f = []

    def fused_iteration():
        dr.set_params(p.detach())
        dr.step_l2(target, image=gimg, grad=gbuf, loss=lbuf, stream=stream)
        with torch.cuda.stream(stream):
            p.grad = gbuf
            opt.step()
            with torch.no_grad():
                p.clamp_(0.01, 100.0)
        losses_f.append(lbuf.clone())

    fused_iteration()
    stream.synchronize()
    e0.record(stream)
    for _ in range(n):
        fused_iteration()
    e1.record(stream)
    stream.synchronize()
    fused_it_ms = e0.elapsed_time(e1) / n
    dr.close()
    scene.close()
    res = {"film": [W, H], "spp": spp, "params": params, "n_params": int(p.numel()),
           "fwd_bwd_ms": round(fb_ms, 2), "iteration_ms": round(it_ms, 2),
           "forward_ms": round(ef[0].elapsed_time(ef[1]), 2), "backward_ms": round(ef[1].elapsed_time(ef[2]), 2),
           "samples_per_s_fwd_bwd": round(W * H * spp / (fb_ms * 1e-3), 1),
           "fused_step_ms": round(fused_ms, 2), "fused_iteration_ms": round(fused_it_ms, 2),
           "fused_samples_per_s": round(W * H * spp / (fused_ms * 1e-3), 1),
           "fused_note": "zgl_diff_step_l2: forward (each path's ray casts kept in HBM), L2 loss and adjoint "
                         "(replayed from the kept casts) queued in one call; iteration = parameter upload + step + "
                         "Adam",
           "loss_first": loss_first, "loss_last": loss_last, "iterations": len(losses)}
    res["grad_check"] = diff_grad_check()
    if not args.no_cpu_baseline:
        hs = Scene(data, host_only=True)
        res["cpu_baseline"] = diff_cpu_baseline(data, hs, spp, params, args.cpu_seconds / 3)
        hs.close()
    return res


def diff_grad_check():
    """Gradient error of the adjoint against the FP64 oracle adjoint on a
    reduced case of the same scene (48x48, 2 spp, depth 6): max abs error
    over parameters divided by the largest oracle gradient."""
    import torch

    import oracle
    from zillumgl_gb300.scene import DiffRenderer, Scene
    from zillumgl_gb300.synthetic import diff_scene

    data = diff_scene(seed=11, width=48, height=48)
    params = dict(max_depth=6)
    scene = Scene(data)
    dr = DiffRenderer(scene, 2, **params)
    rng = np.random.default_rng(5)
    dimage = rng.uniform(-1.0, 1.0, (48, 48, 3)).astype(np.float32)
    dr.forward()
    g = dr.backward(torch.from_numpy(dimage).cuda()).cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    ref = oracle.OracleScene(data, scene.export("sobol"), params).diff_grad(data, 2, dimage)
    dt = time.perf_counter() - t0
    dr.close()
    scene.close()
    scale = float(np.abs(ref).max())
    return {"case": "48x48, 2 spp, depth 6, random image adjoint", "max_abs_err_over_max_grad":
            float(np.abs(g - ref).max() / scale), "oracle_s": round(dt, 2)}


def render_cpu_baseline(data, scene, params, target_s: float = 4.0):
    """The oracle path tracer on every host thread, one pass over an evenly
    strided pixel sample sized to about `target_s` seconds."""
    import oracle

    nthreads = os.cpu_count() or 1
    orc = oracle.OracleScene(data, scene.export("sobol"), params)
    W, H = data.film
    npix = W * H
    probe = np.arange(0, npix, max(1, npix // 2048), dtype=np.int32)
    t0 = time.perf_counter()
    orc.render_pt(probe, 1)
    dt = time.perf_counter() - t0
    stride = max(1, int(np.ceil(npix / max(probe.size * target_s / max(dt, 1e-3), 1.0))))
    pix = np.arange(0, npix, stride, dtype=np.int32)
    t0 = time.perf_counter()
    orc.render_pt(pix, 1)
    dt = time.perf_counter() - t0
    return {"samples_per_s": round(pix.size / dt, 1), "cores": nthreads, "kind": "port",
            "sample": f"one pass of the oracle path tracer over every {stride}th pixel of the {W}x{H} film "
                      f"({pix.size} samples, {dt:.2f}s)"}


def render_cpu_baseline_splat(data, kind, params, target_s: float = 4.0):
    """The oracle light tracer or triple integrator on every host thread (per-
    thread films).  The light tracer runs one pass of as many 1536-path blocks
    as fit in about `target_s` seconds on the configuration's film; the triple
    integrator runs one pass on a quarter-size film of the same scene (its
    camera pass covers every pixel)."""
    import oracle
    from zillumgl_gb300.scene import Scene

    nthreads = os.cpu_count() or 1
    W, H = data.film
    if kind == "triple":
        from zillumgl_gb300.synthetic import city_scene

        data = city_scene(seed=2, width=W // 4, height=H // 4)
    sc = Scene(data, host_only=True)
    orc = oracle.OracleScene(data, sc.export("sobol"), params)
    sc.close()
    w, h = data.film
    if kind == "light":
        t0 = time.perf_counter()
        orc.render_threaded(kind, 1, 8, nthreads=nthreads)
        dt8 = time.perf_counter() - t0
        blocks = int(max(8, min(512, 8 * target_s / max(dt8, 1e-3))))
        t0 = time.perf_counter()
        orc.render_threaded(kind, 1, blocks, nthreads=nthreads)
        dt = time.perf_counter() - t0
        return {"light_paths_per_s": round(1536 * blocks / dt, 1), "cores": nthreads, "kind": "port",
                "sample": f"one pass of {blocks} x 1536 light paths on the {w}x{h} film ({dt:.2f}s)"}
    t0 = time.perf_counter()
    orc.render_threaded(kind, 1, 64, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return {"samples_per_s": round(w * h / dt, 1), "cores": nthreads, "kind": "port",
            "sample": f"one triple pass (camera path per pixel + 64 x 1536 light paths) on a {w}x{h} film of the "
                      f"same scene ({dt:.2f}s)"}


def batch_cpu_baseline(reqs, scenes, target_s: float = 4.0):
    """The oracle path tracer on every host thread over an evenly strided
    pixel sample of every request (one pass each): aggregate samples/s."""
    import oracle

    nthreads = os.cpu_count() or 1
    orcs = [oracle.OracleScene(d, sc.export("sobol"), params) for (d, _, params), sc in zip(reqs, scenes)]

    def run(per_req):
        n = 0
        t0 = time.perf_counter()
        for (d, _, _), orc in zip(reqs, orcs):
            W, H = d.film
            pix = np.linspace(0, W * H - 1, per_req).astype(np.int32)
            orc.render_pt(pix, 1)
            n += pix.size
        return n, time.perf_counter() - t0

    n, dt = run(16)
    per = int(max(16, 16 * target_s / max(dt, 1e-3)))
    n, dt = run(per)
    return {"samples_per_s": round(n / dt, 1), "cores": nthreads, "kind": "port",
            "sample": f"one pass of the oracle path tracer over {per} evenly spaced pixels of each of the "
                      f"{len(reqs)} requests ({n} samples, {dt:.2f}s)"}


def diff_cpu_baseline(data, scene, spp, params, target_s: float = 4.0):
    """The FP64 oracle adjoint (forward replay + gradient) on every host thread
    over an evenly spaced pixel sample at the configuration's spp; ms per
    forward+backward iteration extrapolated to the whole film."""
    import oracle

    nthreads = os.cpu_count() or 1
    orc = oracle.OracleScene(data, scene.export("sobol"), params)
    W, H = data.film

    def run(k):
        dimg = np.zeros((W * H, 3), np.float32)
        pix = np.linspace(0, W * H - 1, k).astype(np.int64)
        dimg[pix] = 1e-3
        t0 = time.perf_counter()
        orc.diff_grad(data, spp, dimg.reshape(H, W, 3))
        return time.perf_counter() - t0

    dt = run(64)
    k = int(min(W * H, max(64, 64 * target_s / max(dt, 1e-3))))
    dt = run(k)
    ms_iter = dt / k * W * H * 1e3
    return {"ms_per_iteration": round(ms_iter, 1), "samples_per_s": round(k * spp / dt, 1), "cores": nthreads,
            "kind": "port", "sample": f"FP64 oracle adjoint over {k} evenly spaced pixels x {spp} spp ({dt:.2f}s), "
                                      f"extrapolated to the {W}x{H} film"}


def cpu_baseline(scenes, specs, sample: int):
    """The oracle traversal on every host thread over the first `sample` rays
    of each launch (the rays the reference arm traces)."""
    import oracle

    nthreads = os.cpu_count() or 1
    packed = {}
    for N, v, idx, acc in scenes:
        p = acc.export()
        packed[N] = (p.bounds, p.hitTable, v, idx)

    def run(n):
        rays = 0
        t0 = time.perf_counter()
        for sp in specs:
            b, h, v, idx = packed[sp["N"]]
            o = sp["o_host"][:n]
            d = sp["d_host"][:n]
            if sp["query"] == "closest":
                oracle.trace(b, h, v, idx, o, d, nthreads=nthreads)
            else:
                tm = sp["tmax"][:n].cpu().numpy()
                oracle.trace(b, h, v, idx, o, d, tmax=tm, any_hit=True, nthreads=nthreads)
            rays += o.shape[0]
        return rays, time.perf_counter() - t0

    run(256)  # warm: loads the oracle library
    sample = min(sample, specs[0]["o_host"].shape[0])
    r, s = run(sample)
    return {"value": round(r / s / 1e6, 3), "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"first {sample} rays of each of the {len(specs)} launches ({r} rays, {s:.1f}s) on the "
                      f"oracle restatement with {nthreads} threads; the reference arm traces the same rays"}


def run_reference(args):
    """CPU reference arm: the oracle restatement (the reference's own traversal
    is GLSL behind OpenGL, unavailable on this machine) on the host cores, over the
    same twelve ray sets as the GPU arm: the same soups, the 2^24 coherent
    primary rays and the incoherent rays made from their closest hits, the same
    any-hit distances.  Each step traces the first --ref-rays rays (contiguous
    rows of the primary image) of each of the twelve launches, with every host
    thread; the rays are the ones the GPU arm's cpu_baseline leg samples."""
    import oracle
    from zillumgl_gb300.synthetic import incoherent_rays, primary_rays, shadow_tmax

    rank, world, local = dist_env()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    sizes = [SIZES[s] for s in args.sizes.split(",")]
    side = args.side
    nray = side * side
    S = min(args.ref_rays, nray)
    o_p, d_p = primary_rays(side, side)
    work = []
    t_setup = time.time()
    for N in sizes:
        seed = SEEDS.get(N, 7)
        v, idx = build_scene(N)
        b, h, _ = oracle.bvh_build(v, idx)
        hid, ht, _, _ = oracle.trace(b, h, v, idx, o_p, d_p, nthreads=nthreads)
        o_i, d_i = incoherent_rays(v, idx, o_p, d_p, hid, ht, seed=seed + 1)
        tm_p = 1.0 + shadow_tmax(nray, seed + 2)
        tm_i = shadow_tmax(nray, seed + 3)
        for oo, dd, tm in ((o_p, d_p, tm_p), (o_i, d_i, tm_i)):
            work.append((b, h, v, idx, oo[:S].copy(), dd[:S].copy(), tm[:S].copy()))
        del hid, ht, o_i, d_i
    log(f"[bench] reference arm setup {time.time() - t_setup:.1f}s")

    def step():
        rays = 0
        for b, h, v, idx, oo, dd, tm in work:
            oracle.trace(b, h, v, idx, oo, dd, nthreads=nthreads)
            oracle.trace(b, h, v, idx, oo, dd, tmax=tm, any_hit=True, nthreads=nthreads)
            rays += 2 * oo.shape[0]
        return rays

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    rays = sum(step() for _ in range(args.steps))
    dt = time.perf_counter() - t0
    value = rays / dt / 1e6
    sample = (f"first {S} rays (the top {S // side} rows of the primary image, and their incoherent rays) of each "
              f"of the {2 * len(work)} launches per step, oracle restatement on {nthreads} threads (the reference "
              f"traversal is GLSL/OpenGL, unavailable on this box)")
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": "MTBVH traversal microbench (triangle soups, 2^24 coherent primary + 2^24 "
                                   "incoherent rays, closest-hit and any-hit)",
                       "triangles": sizes, "rays_per_launch": nray, "launches_per_step": 2 * len(work),
                       "rays_traced_per_launch": S, "parallelism": "host threads"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
