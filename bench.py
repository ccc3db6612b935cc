#!/usr/bin/env python3
"""Benchmark: secondary-ray Mrays/s of the per-frame ray-space-hierarchy path on the 1M-triangle scene.

Workload (default): the procedural-architecture scene (40x40 tessellated pillars + slabs + arches,
1,010,240 triangles), 1920x1080, 4 point lights, depth 2 (shadow + cosine-lobe-perturbed reflection per
bounce), FP32, seeded synthetic input. One step = one frame through rsh_render_frame.

  value       secondary rays traced (after trimming) / GPU time from the first secondary ray generation to
              the last secondary intersection of each frame (CUDA events on the frame's stream), through
              rsh_render_frame in its batched form (RSH_FLAG_FUSED: per bounce one segmented hash/sort and
              one persistent fused traversal + intersection launch)
  plain       the same frames through the plain per-frame path (separate traversal -> candidates ->
              intersection kernels, as the reference's wrappers); identical results
  e2e         the same metric through the C ABI with host buffers: camera + lights from host structs in,
              the RGBA8 frame copied to pinned host memory, both inside the timed region
  roofline    the dominant kernel's achieved rate against its roofline (per-stage CUDA events)
  cpu_baseline the oracle's C++/OpenMP restatement of the same algorithm (per-ray descent of the single-ray
               box tree) on the same frame (the same secondary rays), repeated for about --cpu-seconds;
               cpu_baseline.packet: the reference's stage order (packet traversal) restated, one pass

`--impl reference` times the CPU restatement alone (the reference ships no CPU path and cannot be built
here) on the same workload and metric, and prints its own line.
Multi-GPU: replicas only (each rank renders its own frames; max time over ranks).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT), str(ROOT / "ray-tracer_gb300")]

import numpy as np  # noqa: E402

METRIC = "secondary-ray Mrays/s at 1M tris"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
# algorithmic work per unit (bytes or FP32 flops), used for every roofline fraction
ALGO = {
    "raygen": ("hbm", 64.0),       # bytes / ray slot: surface pos+normal read, ray + key written
    "compress": ("hbm", None),     # 4N + 12C bytes (computed from counts)
    "sort": ("hbm", None),         # C * (4 + 16 P) bytes
    "decompress": ("hbm", None),   # 12C + 4R bytes
    "build": ("hbm", 32.0),        # bytes / ray
    "traverse": ("fp32", 24.0),    # flops / packet-node x sphere test
    "intersect": ("fp32", 46.0),   # flops / ray x triangle test
}


def batch_sort_passes(hash_bits: int, n_segments: int, no_compress: bool = False) -> tuple[int, int]:
    """(key bits, 8-bit digit passes) of a batched call's sort, as the batch plans it: segment tag above
    the hash, the hash's lowest bits dropped to fit 31 bits, and 1 or 2 leftover bits of a last pass
    dropped too (no_compress sorts one more bit, empty slots last)."""
    tag_bits = max(0, (n_segments - 1).bit_length())
    drop = max(0, hash_bits + tag_bits - 31)
    extra = 1 if no_compress else 0
    kb = hash_bits + tag_bits - drop + extra
    tail = kb % 8
    if kb > 8 and tail and tail <= 2 and hash_bits - drop > tail:
        kb -= tail
    return kb, (kb + 7) // 8


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "0x1", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def load_peaks() -> dict:
    if PEAKS_FILE.exists():
        d = json.loads(PEAKS_FILE.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured", "sm_max_mhz": float(d.get("sm_max_mhz", 2070))}
    return {"hbm_gbs": 6800.0, "source": "fallback", "sm_max_mhz": 2070.0}


# ---------------------------------------------------------------- distributed (replicas)
def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as td

        backend = "nccl"
        try:
            import torch

            torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        td.init_process_group(backend=backend)
        return rank, world, td
    return rank, world, None


def reduce_max(td, value: float) -> float:
    if td is None:
        return value
    import torch

    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(td, value: float) -> float:
    if td is None:
        return value
    import torch

    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


def barrier(td):
    if td is not None:
        td.barrier()


# ---------------------------------------------------------------- workload
def make_workload(name: str):
    from rsh import scenes

    return scenes.by_name(name)


def cpu_baseline(s, crop=None, threads=None, steps=1, min_seconds=0.0, max_passes=64, algo="box"):
    """The oracle (C++/OpenMP on the host cores) on the frame (crop=None: the whole frame, the GPU metric's
    own rays) or a centred crop of it: primary hits, then `depth` bounces of shadow + reflection rays.
      algo "box":    the headline's own algorithm, the batched form's rays-only traversal restated: every
                     ray descends the scene's single-ray box tree (PLOC, 8-wide) from the root, one ray per
                     host thread at a time (oracle ObjH.trace_box; with RSH_FLAG_SEQUENTIAL_RAYS the GPU's counters
                     equal its counts);
      algo "packet": the reference's stage order, compress -> sort -> decompress -> ray hierarchy -> packet
                     traversal + intersection (oracle ObjH.trace_keyed).
    Times the secondary part only (the GPU metric's window: ray generation to the last intersection of
    the last bounce). One result per pass; passes repeat the same bounces until there are `steps` of them
    and they took `min_seconds` in all (at most `max_passes`)."""
    import oracle

    lib = oracle.lib()
    if threads:
        lib.orc_set_threads(int(threads))
    nthreads = oracle.threads()
    W, H = s.width, s.height
    cw, chh = crop if crop else (W, H)
    x0, y0 = (W - cw) // 2, (H - chh) // 2
    # the camera and the GPU path's default configuration come from the oracle too, so that this leg maps
    # no product code (grid bits, direction bits, packet, cluster, ray level)
    cam = oracle.camera_look_at(s.eye, s.target, s.up, s.fov, W, H)
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    dc = oracle.DEFAULTS
    g, b, P, K, rl = dc["grid_bits"], dc["dir_log2"], dc["packet_size"], dc["cluster_size"], dc["plain_ray_level"]
    t0 = time.perf_counter()
    oh = oracle.ObjH(s.positions, K, lo, hi)
    build_s = time.perf_counter() - t0
    prays, pix = oracle.raygen_primary(cam, W, H)
    px, py = pix % W, pix // W
    sel = (pix != 0xFFFFFFFF) & (px >= x0) & (px < x0 + cw) & (py >= y0) & (py < y0 + chh)
    crays = prays[sel]
    cpix = ((py[sel] - y0) * cw + (px[sel] - x0)).astype(np.uint32)
    scale = oracle.hash_scale(lo, hi, g)
    if algo == "box":
        hits, _ = oh.trace_box(crays, False)
    else:
        keys = oracle.hash_rays(crays, lo, scale, g, b)
        hits, _, _, _ = oh.trace_keyed(crays, keys, 3 * g + 2 * b, P, False, rl)
    spos0, snrm0 = oracle.resolve(s.positions, s.normals, s.material_ids, crays, hits, cpix, cw * chh)
    lp = np.array([l["position"] for l in s.lights], np.float32)
    L = len(lp)
    lbits = max(0, int(np.ceil(np.log2(L)))) if L > 1 else 0

    def trace(rays, keys, key_bits, any_hit):
        if algo == "box":
            v = keys != oracle.KEY_NONE
            out = np.zeros(len(rays), np.uint32) if any_hit else np.full(len(rays), oracle.HIT_NONE, np.uint64)
            out[v], _ = oh.trace_box(rays[v], any_hit)
            return out, int(v.sum())
        res, R, _, _ = oh.trace_keyed(rays, keys, key_bits, P, any_hit, rl)
        return res, R

    results = []
    while len(results) < max_passes and (len(results) < steps or sum(t for _, t in results) < min_seconds):
        spos, snrm, prev = spos0, snrm0, None
        rays_total = 0
        t_sec = 0.0
        for bnc in range(s.depth):
            t1 = time.perf_counter()
            srays, skeys = oracle.raygen_shadow(spos, snrm, cw, chh, lp, 0.01, lo, scale, g, b)
            flags, R1 = trace(srays, skeys, lbits + 3 * g + 2 * b, True)
            rrays, rkeys = oracle.raygen_reflect(spos, snrm, prev, cam[:3] if prev is None else None, cw, chh, 0.01,
                                                 s.jitter, s.seed, bnc, lo, scale, g, b)
            rh, R2 = trace(rrays, rkeys, 3 * g + 2 * b, False)
            spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, rrays, rh, None, cw * chh)
            t_sec += time.perf_counter() - t1
            rays_total += R1 + R2
            prev = rrays
        results.append((rays_total, t_sec))
    return {"results": results, "threads": nthreads, "crop": (cw, chh), "objh_build_s": build_s, "algo": algo}


CPU_ALGO = {"box": "the headline's algorithm restated in C++/OpenMP (every ray descends the single-ray box tree "
                   "from the root, oracle ObjH.trace_box)",
            "packet": "the reference's stage order restated in C++/OpenMP (compress, sort, decompress, ray "
                      "hierarchy, packet traversal + intersection, oracle ObjH.trace_keyed)"}


def cpu_sample_text(s, cb):
    cw, chh = cb["crop"]
    where = f"the whole {cw}x{chh} frame" if (cw, chh) == (s.width, s.height) else f"a centred {cw}x{chh} crop of the frame"
    rays = sum(r for r, _ in cb["results"])
    secs = sum(t for _, t in cb["results"])
    return (f"{CPU_ALGO[cb['algo']]}; {where}, all bounces, {len(cb['results'])} pass(es): {rays} secondary rays "
            f"in {secs:.2f} s (secondary part only, like the GPU metric)")


def gpu_arm(args, s, rank, world, td):
    import ctypes as C

    import rsh

    lib = rsh.load()
    if lib.rsh_device_count() < 1:
        raise RuntimeError("bench needs a CUDA device")
    peaks = load_peaks()
    W, H, depth = s.width, s.height, s.depth
    npix = W * H
    cfg = rsh.default_config(reflect_jitter=float(s.jitter), seed=s.seed)
    ctx = rsh.Context(cfg)
    t0 = time.perf_counter()
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    upload_s = time.perf_counter() - t0
    cam = rsh.camera_look_at(s.eye, s.target, s.up, s.fov, W, H)
    ctx.set_camera(cam)
    ctx.set_lights(s.lights)
    stream = C.c_void_p()
    rsh.check(lib.rsh_stream_create(C.byref(stream)), "stream")
    st = stream.value
    rgba = rsh.DeviceArray(npix, np.uint32)
    host_img = C.c_void_p()
    rsh.check(lib.rsh_malloc_host(C.byref(host_img), npix * 4), "pinned")
    ev0, ev1 = C.c_void_p(), C.c_void_p()
    lib.rsh_event_create(C.byref(ev0))
    lib.rsh_event_create(C.byref(ev1))
    L0 = lib.rsh_kernel_launches()

    def frame(flags):
        cfg.flags = flags
        lib.rsh_set_config(ctx.handle, C.byref(cfg))
        rsh.check(lib.rsh_render_frame(ctx.handle, sc.handle, W, H, depth, rgba.ptr, st), "render")

    def timed(flags, k, e2e=False):
        stats = []
        lights_arr = rsh.make_lights(s.lights)
        barrier(td)
        lib.rsh_stream_synchronize(st)
        lib.rsh_event_record(ev0, st)
        for _ in range(k):
            if e2e:  # host inputs -> device (camera, lights), frame, result -> pinned host
                lib.rsh_camera_set(ctx.handle, C.byref(cam))
                lib.rsh_lights_set(ctx.handle, lights_arr, len(s.lights))
            frame(flags)
            if e2e:
                rsh.check(lib.rsh_memcpy_d2h(host_img, rgba.ptr, npix * 4, st), "d2h")
            fs = rsh.FrameStats()
            rsh.check(lib.rsh_frame_stats_get(ctx.handle, C.byref(fs)), "stats")
            stats.append(fs.as_dict())
        lib.rsh_event_record(ev1, st)
        lib.rsh_stream_synchronize(st)
        ms = C.c_float()
        lib.rsh_event_elapsed(ev0, ev1, C.byref(ms))
        barrier(td)
        return ms.value, stats

    def rays_of(stats):
        return sum(x["shadow_rays"] + x["reflection_rays"] for x in stats)

    def rate(stats):
        ms = reduce_max(td, sum(x["secondary_ms"] for x in stats))
        return reduce_sum(td, rays_of(stats)) / (ms * 1e3) if ms > 0 else 0.0

    passes = {}
    clocks = ClockSampler()
    clocks.start()
    for name, flags in (("plain", 0), ("fused", 2)):
        if args.mode not in ("all", name):
            continue
        for _ in range(args.warmup):  # warm-up (also sizes every buffer)
            frame(flags)
        lib.rsh_stream_synchronize(st)
        l0 = lib.rsh_kernel_launches()
        wall, stats = timed(flags, args.steps)
        passes[name] = {"flags": flags, "wall_ms": reduce_max(td, wall), "stats": stats, "value": rate(stats),
                        "launches": lib.rsh_kernel_launches() - l0}
    clk = clocks.stop()
    head = passes["fused"] if "fused" in passes else passes["plain"]
    value = head["value"]
    ms_per_step = head["wall_ms"] / args.steps
    sec_rays = rays_of(head["stats"])
    sec_ms = sum(x["secondary_ms"] for x in head["stats"])
    launches = head["launches"]

    def pass_summary(p):
        last = p["stats"][-1]
        return {"value": round(p["value"], 3), "unit": "Mrays/s", "ms_per_step": round(p["wall_ms"] / args.steps, 3),
                "secondary_ms_per_step": round(sum(x["secondary_ms"] for x in p["stats"]) / args.steps, 3),
                "node_tests_per_frame": last["node_tests"], "tri_tests_per_frame": last["tri_tests"],
                "candidates_per_frame": last["candidates"], "gpu_launches": p["launches"]}

    e2e = None
    per_stage, roof, last = {}, None, head["stats"][-1]
    if args.mode in ("all", "fused"):
        # e2e through the C ABI with host buffers, headline form
        e_ms, e_stats = timed(head["flags"], args.steps, e2e=True)
        e2e = {"value": round(reduce_sum(td, rays_of(e_stats)) / (reduce_max(td, e_ms) * 1e3), 3), "unit": "Mrays/s",
               "h2d_bytes_per_step": 48 + 32 * len(s.lights), "d2h_bytes_per_step": npix * 4,
               "ms_per_step": round(e_ms / args.steps, 3)}
        # per-stage timers (separate frames: events between stages), headline form
        t_ms, t_stats = timed(head["flags"] | 1, max(1, min(args.steps, 3)))
        stage_names = ["primary", "raygen", "compress", "sort", "decompress", "build", "traverse", "intersect",
                       "shade"]
        nst = len(t_stats)
        stage_ms = {nm: sum(x["stage_ms"][i] for x in t_stats) / nst for i, nm in enumerate(stage_names)}
        last = t_stats[-1]
        chunks = last["chunks"]
        R = last["shadow_rays"] + last["reflection_rays"]
        slots = npix * (len(s.lights) + 1) * depth
        # the batched form sorts both segments of a bounce together (the plain path: per batch, light tag)
        key_bits, passes_sort = batch_sort_passes(3 * cfg.grid_bits + 2 * cfg.dir_log2, 2)
        bytes_stage = {
            "raygen": 64.0 * slots,
            "compress": 4.0 * slots + 12.0 * chunks + 4.0 * R,
            "sort": chunks * (4.0 + 16.0 * passes_sort),
            "decompress": 12.0 * chunks + 4.0 * R,
            "build": 32.0 * R,
        }
        fused_head = head["flags"] == 2
        if fused_head:  # traversal and intersection run in one kernel: charge both to it
            flops_stage = {"traverse": 24.0 * last["node_tests"] + 46.0 * last["tri_tests"], "intersect": 0.0}
        else:
            flops_stage = {"traverse": 24.0 * last["node_tests"], "intersect": 46.0 * last["tri_tests"]}
        for nm in ("raygen", "compress", "sort", "decompress", "build"):
            ms = stage_ms[nm]
            gbs = bytes_stage[nm] / (ms * 1e6) if ms > 0 else 0.0
            per_stage[nm] = {"ms": round(ms, 4), "GB/s": round(gbs, 1), "frac_hbm": round(gbs / peaks["hbm_gbs"], 4)}
        sm_clock = clk.get("sm_mhz") or peaks["sm_max_mhz"]
        n_sm = lib.rsh_sm_count()
        fp32_peak = n_sm * 128 * 2 * sm_clock * 1e6 / 1e12   # TFLOP/s at the observed SM clock
        for nm in ("traverse", "intersect"):
            ms = stage_ms[nm]
            tf = flops_stage[nm] / (ms * 1e9) if ms > 0 else 0.0
            per_stage[nm] = {"ms": round(ms, 4), "TFLOP/s": round(tf, 3), "frac_fp32": round(tf / fp32_peak, 4)}
        # the batched form's kernel: rays alone from the root when the switch level reaches the tree's depth
        fused_kernel = "k_fused_rays" if cfg.ray_level >= lib.rsh_scene_levels(sc.handle) else "k_fused"
        if fused_head:
            per_stage["traverse"]["kernel"] = f"{fused_kernel} (traversal + intersection)"
        dom = max(("raygen", "compress", "sort", "decompress", "build", "traverse", "intersect"),
                  key=lambda k: stage_ms[k])
        if dom in flops_stage:
            ach = per_stage[dom]["TFLOP/s"]
            roof = {"bound": "fp32", "kernel": fused_kernel if (fused_head and dom == "traverse") else f"k_{dom}",
                    "achieved": ach, "peak": round(fp32_peak, 2), "unit": "TFLOP/s", "frac": round(ach / fp32_peak, 4),
                    "traffic": None,
                    "peak_note": f"FP32 issue: {n_sm} SMs x 128 lanes x 2 flops x {sm_clock:.0f} MHz (no measured FP32 peak)"}
        else:
            ach = per_stage[dom]["GB/s"]
            roof = {"bound": "hbm", "kernel": f"k_{dom}", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": round(ach / peaks["hbm_gbs"], 4), "traffic": None,
                    "peak_note": f"{peaks['source']} HBM copy bandwidth"}
        prof = ROOT / "profiles" / "traffic.json"
        if prof.exists():
            try:
                tr = json.loads(prof.read_text())
                if roof["kernel"] in tr:
                    ent = tr[roof["kernel"]]
                    roof["traffic"] = ent["bytes_per_launch"]
                    roof["traffic_note"] = f"ncu dram read+write bytes of one launch, {ent['workload']}"
            except Exception:
                pass
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "Mrays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded procedural architecture scene)",
        "config": {"workload": f"procedural architecture {s.tri_count} tris, {W}x{H}, {len(s.lights)} point lights, "
                               f"depth {depth}, cosine-lobe reflections",
                   "path": "rsh_render_frame " + ("batched form (RSH_FLAG_FUSED)" if head["flags"] == 2 else "plain"),
                   "triangles": s.tri_count, "width": W, "height": H, "lights": len(s.lights), "depth": depth,
                   "grid_bits": cfg.grid_bits, "dir_log2": cfg.dir_log2, "packet_size": cfg.packet_size,
                   "cluster_size": cfg.cluster_size, "ray_level": cfg.ray_level, "plain_ray_level": cfg.plain_ray_level,
                   "l2": "inputs larger than L2 (scene + per-frame rays > 129 MB)", "parallelism": f"replicas x{world}"},
        "secondary_rays_per_step": round(sec_rays / args.steps),
        "secondary_ms_per_step": round(sec_ms / args.steps, 3),
        "e2e": e2e,
        "roofline": roof,
        "stages": per_stage,
        "counters_per_frame": {"chunks": last["chunks"], "candidates": last["candidates"],
                               "node_tests": last["node_tests"], "tri_tests": last["tri_tests"],
                               "overflow_passes": last["overflow_passes"]},
        "gpu_launches": int(launches),
        "clocks": clk,
        "scene_upload_s": round(upload_s, 3),
    }
    for name, p in passes.items():
        out[name] = pass_summary(p)
    if "plain" in passes and "fused" in passes and passes["plain"]["value"] > 0:
        out["fused"]["ratio_vs_plain"] = round(passes["fused"]["value"] / passes["plain"]["value"], 3)
    out["device_errors"] = int(lib.rsh_check_device_errors(ctx.handle, st))
    lib.rsh_free_host(host_img)
    sc.destroy()
    ctx.destroy()
    return out


# ---------------------------------------------------------------- serving (continuous batching)
def fcfs_latency_ms(gaps, service) -> list:
    """Latencies (ms) of requests arriving after the given gaps (s) at one server that takes them first
    come, first served, each for its own service time (s)."""
    free_at, out = 0.0, []
    for a, sv in zip(np.cumsum(gaps), service):
        free_at = max(free_at, a) + sv
        out.append((free_at - a) * 1e3)
    return out


def serving_bench(args):
    """Poisson request arrivals over resident scenes through rsh_server_* at each rate of --serve-rates:
    p50/p99 latency and Mrays/s (clocks sampled while the server runs), next to the same requests rendered
    one at a time through rsh_render_frame, back to back: by the batched form (RSH_FLAG_FUSED) for every
    request, and by the plain per-frame path for the first --serve-plain ones (it is ~50x slower). Each
    serial loop's latency is that of a single renderer taking the same arrivals first come, first served,
    with every request's own measured frame time."""
    import ctypes as C

    import rsh
    from rsh import scenes

    lib = rsh.load()
    rng = np.random.default_rng([scenes.SEED_BASE + 4, 0])
    n_scenes = args.serve_scenes
    tris = np.exp(rng.uniform(np.log(50_000), np.log(1_000_000), n_scenes)).astype(int)
    sd = [scenes.random_soup(int(t), np.random.default_rng([scenes.SEED_BASE + 4, 100 + i])) for i, t in enumerate(tris)]
    ctx = rsh.Context(rsh.default_config(reflect_jitter=1.0))
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    res_choices = [(256, 256), (512, 512), (1920, 1080)][: args.serve_max_res]
    reqs = []
    for k in range(args.serve_requests):
        si = int(rng.integers(0, n_scenes))
        W, H = res_choices[int(rng.integers(0, len(res_choices)))]
        ang = rng.uniform(0, 2 * np.pi)
        eye = (60.0 * np.cos(ang), rng.uniform(-10, 30), 60.0 * np.sin(ang))
        cam = rsh.camera_look_at(eye, (0, 0, 0), (0, 1, 0), 60.0, W, H)
        nl = int(rng.integers(1, 5))
        lights = [{"position": tuple(rng.uniform(-30, 30, 3))} for _ in range(nl)]
        r = rsh.Request()
        r.scene_index, r.camera, r.width, r.height = si, cam, W, H
        r.depth, r.light_count = int(rng.integers(1, 4)), nl
        arr = rsh.make_lights(lights)
        for i in range(nl):
            r.lights[i] = arr[i]
        reqs.append(r)

    def serial(flags, subset):
        """Renders the requests one at a time (synchronised each), returns (service times s, rays)."""
        ctx.set_config(flags=flags)
        for r in reqs[:2]:  # warm-up: buffers sized
            ctx.set_camera(r.camera)
            lib.rsh_lights_set(ctx.handle, r.lights, r.light_count)
            rsh.check(lib.rsh_render_frame(ctx.handle, scs[r.scene_index].handle, r.width, r.height, r.depth, None,
                                           None), "render")
            ctx.stats()
        service, rays = [], 0
        for r in subset:
            t1 = time.perf_counter()
            ctx.set_camera(r.camera)
            lib.rsh_lights_set(ctx.handle, r.lights, r.light_count)
            rsh.check(lib.rsh_render_frame(ctx.handle, scs[r.scene_index].handle, r.width, r.height, r.depth, None,
                                           None), "render")
            fs = ctx.stats()  # synchronises
            rays += fs["shadow_rays"] + fs["reflection_rays"]
            service.append(time.perf_counter() - t1)
        return service, rays

    fused_service, fused_rays = serial(rsh.FLAG_FUSED, reqs)
    plain_subset = reqs[: args.serve_plain]
    plain_service, plain_rays = serial(0, plain_subset)
    ctx.set_config(flags=0)
    arrs = (C.c_void_p * n_scenes)(*[s.handle for s in scs])
    out_rates = []
    for rate in [float(x) for x in args.serve_rates.split(",")]:
        gaps = np.random.default_rng([scenes.SEED_BASE + 4, int(rate)]).exponential(1.0 / rate, len(reqs))
        srv = C.c_void_p()
        rsh.check(lib.rsh_server_create(ctx.handle, arrs, n_scenes, args.serve_budget_gb << 30, 64, C.byref(srv)),
                  "srv")
        if args.serve_step_rays >= 0:
            rsh.check(lib.rsh_server_set_step_rays(srv, args.serve_step_rays), "step rays")
        clocks = ClockSampler()
        clocks.start()
        # a client thread collects results in submission order while requests keep arriving (a finished
        # request holds its device memory until it is collected)
        import queue as _queue

        pending, lat, tally = _queue.Queue(), [], {"rays": 0}

        def collect():
            while True:
                i = pending.get()
                if i is None:
                    return
                rr = rsh.RequestResult()
                if lib.rsh_server_wait(srv, i, 600_000, C.byref(rr), None, None) == rsh.RSH_OK:
                    lat.append(rr.finish_ms - rr.submit_ms)
                    tally["rays"] += rr.rays

        th = threading.Thread(target=collect)
        th.start()
        t0 = time.perf_counter()
        due = t0
        for r, g in zip(reqs, gaps):
            due += g
            delay = due - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            i = C.c_uint64()
            rsh.check(lib.rsh_server_submit(srv, C.byref(r), C.byref(i)), "submit")
            pending.put(i.value)
        pending.put(None)
        th.join()
        rays = tally["rays"]
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        stats = [C.c_uint64() for _ in range(4)]
        lib.rsh_server_stats(srv, *[C.byref(x) for x in stats])
        lib.rsh_server_destroy(srv)
        lat = np.array(lat)
        fl = fcfs_latency_ms(gaps, fused_service)
        pl_ = fcfs_latency_ms(gaps[: len(plain_service)], plain_service)
        # the serial batched loop under the same arrivals: rays over its makespan (first arrival to last finish)
        fused_makespan = float(np.cumsum(gaps)[-1] + fl[-1] / 1e3)
        out_rates.append({
            "arrival_rate_req_s": rate, "requests": len(reqs), "completed": int(len(lat)),
            "arrival_window_s": round(float(np.sum(gaps)), 3),
            "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
            "server_wall_s": round(wall, 3), "server_mrays_s": round(rays / wall / 1e6, 3),
            "serial_fused_mrays_s": round(fused_rays / fused_makespan / 1e6, 3),
            "serial_fused_p50_ms": round(float(np.percentile(fl, 50)), 2),
            "serial_fused_p99_ms": round(float(np.percentile(fl, 99)), 2),
            "serial_plain_p50_ms": round(float(np.percentile(pl_, 50)), 2),
            "serial_plain_p99_ms": round(float(np.percentile(pl_, 99)), 2),
            "steps": stats[1].value, "peak_inflight": stats[2].value, "peak_bytes": stats[3].value, "clocks": clk})
    for s in scs:
        s.destroy()
    ctx.destroy()
    return {"metric": "serving p50/p99 latency and Mrays/s vs serial per-frame loops",
            "scenes_tris": [int(t) for t in tris], "requests": len(reqs),
            "resolutions": [f"{w}x{h}" for w, h in res_choices],
            "serial_fused": {"mrays_s": round(fused_rays / sum(fused_service) / 1e6, 3),
                             "wall_s": round(sum(fused_service), 3), "requests": len(reqs),
                             "form": "rsh_render_frame, RSH_FLAG_FUSED, one request at a time"},
            "serial_plain": {"mrays_s": round(plain_rays / sum(plain_service) / 1e6, 3),
                             "wall_s": round(sum(plain_service), 3), "requests": len(plain_subset),
                             "form": "rsh_render_frame, plain per-frame path, one request at a time"},
            "rates": out_rates, "data": "synthetic (seeded random soups, seeded requests)"}


def batching_bench(args):
    """The batching workload: 256 independent ray batches (sizes log-uniform in [4k, 2M]) over 16 resident
    random soups (10k-1M triangles, log-uniform); rays leave triangle surfaces with uniform-sphere or mirror
    directions (50/50); half the batches closest hit, half any hit. The autotuner picks grid bits, direction
    bins and packet size on this batch; then one CUDA-graph launch traces the whole batch per step.
    Mrays/s = rays per step / device time per step (CUDA events on the graph's stream)."""
    import ctypes as C

    import rsh
    from rsh import scenes

    lib = rsh.load()
    sd, sizes, which, any_hit = scenes.batch_config(n_batches=args.batch_count, max_rays=args.batch_max_rays)
    ctx = rsh.Context(rsh.default_config())
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    rng = np.random.default_rng([scenes.SEED_BASE + 3, 7])
    segs = (rsh.BatchSegment * len(sizes))()
    keep = []
    total = 0
    for i, (n, w, a) in enumerate(zip(sizes, which, any_hit)):
        n = int(n)
        r = scenes.surface_rays(sd[w], n, rng)
        dr = rsh.DeviceArray.from_numpy(r)
        out = rsh.DeviceArray(n, np.uint32 if a else np.uint64)
        keep.append((dr, out))
        segs[i].scene = scs[w].handle
        segs[i].rays = dr.ptr
        segs[i].n = n
        segs[i].any_hit = int(a)
        segs[i].hits = None if a else out.ptr
        segs[i].flags = out.ptr if a else None
        total += n
    st = C.c_void_p()
    rsh.check(lib.rsh_stream_create(C.byref(st)), "stream")
    # per-scene autotuner over origin-grid bits 4..10, direction bins 16..4096 (dir_log2 2..6), switch levels
    # 3..7 and 15 (rays alone from the root), packet sizes 8/16/32 and 4/6/8 CTAs per SM of the traversal
    # launch (coordinate descent; points whose hash exceeds the key's room are skipped)
    t0 = time.perf_counter()
    tuned_ms, untuned_ms = ctx.autotune_scenes(segs, len(sizes), grid_bits=range(4, 11), dir_log2=range(2, 7),
                                               ray_levels=(3, 4, 5, 6, 7, 15), packet_sizes=(8, 16, 32), stream=st,
                                               fused_blocks=(4, 6, 8))
    tune_s = time.perf_counter() - t0
    best = ctx.config
    scene_tuning = [sc.tuning() for sc in scs]
    g = C.c_void_p()
    rsh.check(lib.rsh_batch_graph_create(ctx.handle, segs, len(sizes), st, C.byref(g)), "graph")
    for _ in range(args.warmup):
        rsh.check(lib.rsh_batch_graph_launch(g, st), "launch")
    rsh.check(lib.rsh_stream_synchronize(st), "sync")
    e0, e1 = C.c_void_p(), C.c_void_p()
    lib.rsh_event_create(C.byref(e0))
    lib.rsh_event_create(C.byref(e1))
    l0 = lib.rsh_kernel_launches()
    clocks = ClockSampler()
    clocks.start()
    lib.rsh_event_record(e0, st)
    for _ in range(args.steps):
        rsh.check(lib.rsh_batch_graph_launch(g, st), "launch")
    lib.rsh_event_record(e1, st)
    rsh.check(lib.rsh_stream_synchronize(st), "sync")
    clk = clocks.stop()
    ms = C.c_float()
    lib.rsh_event_elapsed(e0, e1, C.byref(ms))
    ctx.check_device_errors(st)
    lib.rsh_batch_graph_destroy(g)
    # per-stage CUDA events of the same batch (separate untimed-by-graph passes; mean of 3 after 1 warm-up)
    cfg = rsh.Config()
    lib.rsh_get_config(ctx.handle, C.byref(cfg))
    cfg.flags |= rsh.FLAG_STAGE_TIMERS
    rsh.check(lib.rsh_set_config(ctx.handle, C.byref(cfg)), "config")
    stage_runs = []
    for i in range(4):
        rsh.check(lib.rsh_batch_trace(ctx.handle, segs, len(sizes), st), "batch")
        fs = rsh.FrameStats()
        rsh.check(lib.rsh_batch_stats_get(ctx.handle, C.byref(fs)), "stats")
        if i:
            stage_runs.append(fs.as_dict())
    lib.rsh_stream_destroy(st)
    for s in scs:
        s.destroy()
    peaks = load_peaks()
    last = stage_runs[-1]
    n_rays, n_chunks = last["reflection_rays"], last["chunks"]
    def eff(t, k):  # a scene's value, or the context's where the scene keeps it
        return getattr(best, k) if t[k] == rsh.TUNE_DEFAULT else t[k]

    hash_bits = max(3 * eff(t, "grid_bits") + 2 * eff(t, "dir_log2") for t in scene_tuning)
    key_bits, passes = batch_sort_passes(hash_bits, len(sizes), bool(best.flags & rsh.FLAG_NO_COMPRESS))
    stage_bytes = {"hash": 32.0 * n_rays, "compress": 4.0 * n_rays + 12.0 * n_chunks,
                   "sort": n_chunks * (4.0 + 16.0 * passes), "decompress": 12.0 * n_chunks + 4.0 * n_rays,
                   "build": 32.0 * n_rays}
    stage_idx = {"hash": 1, "compress": 2, "sort": 3, "decompress": 4, "build": 5}
    stages = {}
    for nm, b in stage_bytes.items():
        t = sum(r["stage_ms"][stage_idx[nm]] for r in stage_runs) / len(stage_runs)
        gbs = b / (t * 1e6) if t > 0 else 0.0
        stages[nm] = {"ms": round(t, 4), "GB/s": round(gbs, 1), "frac_hbm": round(gbs / peaks["hbm_gbs"], 4)}
    t_fused = sum(r["stage_ms"][6] for r in stage_runs) / len(stage_runs)
    stages["fused"] = {"ms": round(t_fused, 3), "node_tests": int(last["node_tests"]), "tri_tests": int(last["tri_tests"])}
    step_ms = ms.value / args.steps
    out = {"metric": "batched secondary-ray Mrays/s (graph launch per step)", "value": round(total / step_ms / 1e3, 3),
           "unit": "Mrays/s", "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 3),
           "rays_per_step": int(total), "batches": int(len(sizes)), "scenes": len(sd),
           "scenes_tris": [int(s.tri_count) for s in sd],
           "autotuned": {"packet_size": best.packet_size, "fused_blocks_per_sm": best.fused_blocks,
                         "run_compression": not (best.flags & rsh.FLAG_NO_COMPRESS),
                         "shared_launch_ends": not (best.flags & rsh.FLAG_SEQUENTIAL_RAYS),
                         "per_scene": scene_tuning, "tuning_s": round(tune_s, 2),
                         "batch_ms_untuned": round(untuned_ms, 3), "batch_ms_tuned": round(tuned_ms, 3),
                         "context_defaults": {"grid_bits": best.grid_bits, "dir_log2": best.dir_log2,
                                              "ray_level": best.ray_level}},
           "kernels_per_step_launched_by_graph": "compress, sort, decompress, build, fused (one persistent launch)",
           "stages": stages, "stage_sizes": {"rays": int(n_rays), "chunks": int(n_chunks), "key_bits": key_bits,
                                             "sort_passes": passes},
           "stage_peak_note": f"{peaks['source']} HBM copy bandwidth {peaks['hbm_gbs']} GB/s; algorithmic bytes "
                              "(hash 32 B/ray, compress 4N+12C, sort C(4+16P), decompress 12C+4N, build 32 B/ray)",
           "clocks": clk, "data": "synthetic (seeded random soups, surface rays)"}
    ctx.destroy()
    return out


def sort_bench(args):
    """The onesweep sort alone: rsh_sort_pairs on N seeded random 31-bit keys (values = index), 4 digit
    passes; algorithmic bytes C (4 + 16 P) per the stage table. CUDA events around `steps` sorts."""
    import ctypes as C

    import rsh

    lib = rsh.load()
    ctx = rsh.Context(rsh.default_config())
    n = int(args.sort)
    k = np.random.default_rng(scenes_seed(1)).integers(0, 1 << 31, n, dtype=np.uint32)
    ki, ko, vo = rsh.DeviceArray.from_numpy(k), rsh.DeviceArray(n, np.uint32), rsh.DeviceArray(n, np.uint32)

    def one():
        rsh.check(lib.rsh_sort_pairs(ctx.handle, ki.ptr, None, ko.ptr, vo.ptr, n, None, 31, None), "sort")

    for _ in range(args.warmup):
        one()
    e0, e1 = C.c_void_p(), C.c_void_p()
    lib.rsh_event_create(C.byref(e0))
    lib.rsh_event_create(C.byref(e1))
    lib.rsh_stream_synchronize(None)
    lib.rsh_event_record(e0, None)
    for _ in range(args.steps):
        one()
    lib.rsh_event_record(e1, None)
    lib.rsh_stream_synchronize(None)
    ms = C.c_float()
    lib.rsh_event_elapsed(e0, e1, C.byref(ms))
    t = ms.value / args.steps
    alg = n * (4 + 16 * 4)
    peaks = load_peaks()
    ctx.destroy()
    return {"metric": "onesweep sort GB/s (algorithmic)", "value": round(alg / t / 1e6, 1), "unit": "GB/s",
            "ms_per_step": round(t, 4), "pairs": n, "passes": 4, "steps": args.steps, "warmup": args.warmup,
            "frac_hbm": round(alg / t / 1e6 / peaks["hbm_gbs"], 4), "data": "synthetic (seeded random 31-bit keys)"}


def scenes_seed(k: int) -> int:
    from rsh import scenes

    return scenes.SEED_BASE + k


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="rsh", choices=["rsh", "reference"])
    ap.add_argument("--config", default="P", choices=["S", "O", "P"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-crop", default="full", help="CPU sample: 'full' (the whole frame) or WxH, centred")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline: repeat passes for this long")
    ap.add_argument("--width", type=int, default=0, help="override the frame width (profiling runs)")
    ap.add_argument("--height", type=int, default=0, help="override the frame height (profiling runs)")
    ap.add_argument("--mode", default="all", choices=["all", "plain", "fused"],
                    help="all: plain + fused + e2e + stage timers; plain/fused: only that timed pass")
    ap.add_argument("--serving", action="store_true", help="run the serving benchmark instead")
    ap.add_argument("--batching", action="store_true", help="run the batching benchmark (256 batches, 16 scenes)")
    ap.add_argument("--sort", type=int, default=0, help="time rsh_sort_pairs alone on this many pairs")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-max-rays", type=int, default=2_000_000)
    ap.add_argument("--serve-requests", type=int, default=500)
    ap.add_argument("--serve-rates", default="50,500,2000", help="arrival rates (req/s), comma separated")
    ap.add_argument("--serve-plain", type=int, default=64, help="requests the plain serial loop renders")
    ap.add_argument("--serve-step-rays", type=int, default=-1, help="server ray budget per step (-1: default)")
    ap.add_argument("--serve-scenes", type=int, default=8)
    ap.add_argument("--serve-max-res", type=int, default=3)
    ap.add_argument("--serve-budget-gb", type=int, default=32)
    args = ap.parse_args()
    if args.serving:
        print(json.dumps(serving_bench(args)))
        return 0
    if args.batching:
        print(json.dumps(batching_bench(args)))
        return 0
    if args.sort:
        print(json.dumps(sort_bench(args)))
        return 0
    rank, world, td = dist_setup(args.gpus)
    s = make_workload(args.config)
    if args.width:
        s.width = args.width
    if args.height:
        s.height = args.height
    crop = None if args.cpu_crop == "full" else tuple(int(x) for x in args.cpu_crop.split("x"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        cb = cpu_baseline(s, crop=crop, steps=args.warmup + args.steps, max_passes=args.warmup + args.steps,
                          algo="box")
        res = cb["results"][args.warmup:]
        rays = sum(r for r, _ in res)
        secs = sum(t for _, t in res)
        val = rays / secs / 1e6
        line = {"impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "Mrays/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * secs / len(res), 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded procedural architecture scene)",
                "config": {"workload": f"procedural architecture {s.tri_count} tris, {s.width}x{s.height}, "
                                       f"{len(s.lights)} point lights, depth {s.depth}, cosine-lobe reflections"},
                "cpu_baseline": {"value": round(val, 4), "unit": "Mrays/s", "cores": cb["threads"], "kind": "port",
                                 "sample": "one pass per step (warm-up passes untimed); " + cpu_sample_text(s, cb)},
                "e2e": {"value": round(val, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    out = gpu_arm(args, s, rank, world, td)
    if rank == 0:
        if not args.no_cpu_baseline:
            cb = cpu_baseline(s, crop=crop, steps=1, min_seconds=args.cpu_seconds, algo="box")
            rays = sum(r for r, _ in cb["results"])
            secs = sum(t for _, t in cb["results"])
            out["cpu_baseline"] = {"value": round(rays / secs / 1e6, 4), "unit": "Mrays/s", "cores": cb["threads"],
                                   "kind": "port", "sample": cpu_sample_text(s, cb)}
            # second figure: the reference's stage order (packets over the ray-space hierarchy) on the host
            cp = cpu_baseline(s, crop=crop, steps=1, min_seconds=0.0, algo="packet")
            rp = sum(r for r, _ in cp["results"])
            sp_ = sum(t for _, t in cp["results"])
            out["cpu_baseline"]["packet"] = {"value": round(rp / sp_ / 1e6, 4), "unit": "Mrays/s",
                                             "sample": cpu_sample_text(s, cp)}
        print(json.dumps(out))
    if td is not None:
        td.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
