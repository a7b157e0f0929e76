#!/usr/bin/env python
"""Benchmark of the GB300 triangle pipeline: shaded Mpix/s.

Workload (default): the 1920x1080 heightmap terrain of 1,048,576 triangles,
16 point lights (light 0 with a 6x1024^2 shadow cubemap), 16 RGBA8 512^2
textures.  One step = one frame of the reference's frame loop:
generate_realtime_shadowing + render_tris (prearrange, kernel1, kernel2,
kernel3), i.e. gbr_shadow_pass + gbr_render_view.

  value  Mpix/s, device-timed (CUDA events on the launching stream), scene resident
  e2e    Mpix/s through gbr_render_view_host: camera/view in from host memory,
         depth + id + RGBA8 copied back to pinned host buffers every step

--impl reference times the reference's CPU implementation of the same frame on
the host cores, all threads: the reference's own cl2.cl kernels compiled as C++
(oracle/_ref), or the C++ restatement of them where those cannot be built.
Multi-GPU (torchrun): every rank renders its own frames (replicas); value is
the whole job's pixels / max-over-ranks time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from openclrenderer_gb300 import scenes  # noqa: E402
from openclrenderer_gb300 import structs as S  # noqa: E402

METRIC = "shaded Mpix/s @1080p 1M tris, batched/served vs plain on GB300; p50/p99 latency"
WORKLOAD = "terrain_1080p_1M"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbr", choices=["gbr", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the binning-stress, mixed-batch and serving sections")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=150)
    ap.add_argument("--batch-views", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-pass", action="store_true",
                    help="one launch of every kernel inside cudaProfilerStart/Stop (for ncu --profile-from-start off), "
                         "then exit: scene build, a 1080p terrain frame, the four post passes, an 8-view sphere batch "
                         "in each raster / kernel3 mode")
    ap.add_argument("--profile-batch", action="store_true",
                    help="the 64-view sphere batch (the mixed-resolution batched workload) rendered once inside "
                         "cudaProfilerStart/Stop after a warm-up batch, with the tuning its captured graph uses "
                         "(128-thread rasters), then exit")
    ap.add_argument("--tile-stats", action="store_true",
                    help="CPU only: the 1080p terrain frame's records and bins for fine tiles of 8, 16 and 32 "
                         "pixels, from a numpy model of the view setup's culls, bounding boxes and footprints, then "
                         "exit (at 16 pixels it reproduces the GPU's record and bin-entry counts)")
    return ap.parse_args()


def tile_stats():
    """Records per fine tile and bin entries of the 1080p terrain frame for
    8x8, 16x16 and 32x32 tiles.  The view setup modelled in float64: the
    camera rotation, the near clip (whole triangles), projection, rounded
    bounding boxes (min - 1 .. max, clamped, empty boxes dropped), back-face
    cull, then footprints with records over 16 fine tiles in 128-pixel coarse
    bins, as the fill does."""
    sc = scenes.terrain()
    view = sc.views[0]
    W, H, fov = int(view["width"]), int(view["height"]), 960.0
    rot = np.array(sc.cameras[0]["rot"][:3], np.float64)
    c, s = np.cos(rot), np.sin(rot)
    rel = sc.tris["vertices"]["pos"][:, :, :3].astype(np.float64)  # identity descriptors: world = object space
    a = s[2] * rel[..., 1] + c[2] * rel[..., 0]
    b = c[1] * rel[..., 2] + s[1] * a
    d = c[2] * rel[..., 1] - s[2] * rel[..., 0]
    X, Y, Z = c[1] * a - s[1] * rel[..., 2], s[0] * b + c[0] * d, c[0] * b - s[0] * d
    x, y = X / Z * fov + W / 2, Y / Z * fov + H / 2
    cross = (x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (y[:, 1] - y[:, 0]) * (x[:, 2] - x[:, 0])
    xr, yr = np.round(x), np.round(y)
    x0, x1 = np.clip(xr.min(1) - 1, 0, W - 1), np.clip(xr.max(1), 0, W - 1)
    y0, y1 = np.clip(yr.min(1) - 1, 0, H - 1), np.clip(yr.max(1), 0, H - 1)
    keep = np.all(Z > 20, axis=1) & (x1 > x0) & (y1 > y0) & (cross <= 0)
    X0, X1, Y0, Y1 = (v[keep].astype(np.int64) for v in (x0, x1, y0, y1))
    out = {"workload": "terrain_1080p_1M", "records": int(keep.sum()), "tiles": {}}
    for T in (8, 16, 32):
        tx0, tx1, ty0, ty1 = X0 // T, (X1 - 1) // T, Y0 // T, (Y1 - 1) // T
        n = (tx1 - tx0 + 1) * (ty1 - ty0 + 1)
        coarse = n > 16
        cn = ((X1 - 1) // 128 - X0 // 128 + 1) * ((Y1 - 1) // 128 - Y0 // 128 + 1)
        cnt = np.zeros(((H + T - 1) // T, (W + T - 1) // T), np.int64)
        for i in np.nonzero(~coarse)[0]:
            cnt[ty0[i]:ty1[i] + 1, tx0[i]:tx1[i] + 1] += 1
        nz = cnt[cnt > 0]
        out["tiles"][f"{T}x{T}"] = {
            "tiles": int(cnt.size), "bin_entries": int(np.where(coarse, cn, n).sum()),
            "records_per_tile_mean": round(float(nz.mean()), 1), "records_per_tile_p99": round(float(np.percentile(nz, 99))),
            "records_per_tile_max": int(nz.max()), "tiles_over_128_records": round(float(np.mean(cnt > 128)), 4),
            "tiles_over_512_records": round(float(np.mean(cnt > 512)), 4)}
    print(json.dumps(out))


def profile_pass():
    """Every kernel of the pipeline once, between cudaProfilerStart and
    cudaProfilerStop, after an untimed warm-up frame."""
    import torch
    from openclrenderer_gb300.pipeline import GpuScene
    sc = scenes.terrain()
    mb = scenes.spheres_batch(n_spheres=500, n_views=8)
    warm = GpuScene(sc)
    warm.shadow_pass()
    warm.render(sc.cameras[0], sc.views[0])
    warm.close()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    gs = GpuScene(sc)
    gs.shadow_pass()
    cam, view = sc.cameras[0], sc.views[0]
    out = gs.render(cam, view, normals=True)
    glights = sc.lights.copy()
    glights["godray_intensity"][:2] = 1.0
    gs.set_lights(glights)
    gs.post_godrays(cam, view, out)
    gs.set_lights(sc.lights)
    gs.post_pseudo_aa(view, out)
    prev = np.array(cam, S.CAMERA)
    prev["pos"][:3] += np.float32([4.0, 1.0, -6.0])
    gs.post_motion_blur(cam, prev, view, out, 2, 1.0, 0.5)
    rdescs = sc.descs.copy()
    rdescs["feature_flag"] |= 1
    gs.set_descriptors(rdescs)
    gs.post_reflections(cam, view, out)
    g2 = GpuScene(mb)
    for mode in (S.RS_SEQUENTIAL, S.RS_FUSED, S.RS_PIPELINED):
        g2.set_tuning(S.PASS_VIEW, raster_shade=mode)
        g2.render_batch(mb.cameras, mb.views)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print("profile pass done")


def profile_batch():
    """The batched workload's pass once, between cudaProfilerStart and
    cudaProfilerStop, after an untimed warm-up batch."""
    import torch
    from openclrenderer_gb300.pipeline import GpuScene
    mb = scenes.spheres_batch()
    g = GpuScene(mb)
    g.set_tuning(S.PASS_VIEW, raster_threads=128)
    outs = g.render_batch(mb.cameras, mb.views)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    g.render_batch(mb.cameras, mb.views, outs=outs)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print("profile batch done")


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms, world, device=None):
    """The slowest rank's step time, on every rank (all-reduce MAX; the
    process group is NCCL on GPUs, gloo in the CPU tests)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mpix_per_s(pixels_per_step, world, ms):
    """Whole-job throughput: every rank renders pixels_per_step per step
    (replicas, weak scaling), the job takes the slowest rank's time."""
    return world * pixels_per_step / (ms * 1e-3) / 1e6


def scene_config(sc):
    v = sc.views[0]
    return {"workload": WORKLOAD, "width": int(v["width"]), "height": int(v["height"]),
            "triangles": int(len(sc.tris)), "lights": int(len(sc.lights)),
            "shadow_cubemaps": int(sum(1 for l in sc.lights if l["shadow"] == 1)),
            "textures": f"{len(sc.tex_sizes)}x{sc.tex_sizes[0]}^2 RGBA8",
            "l2": "inputs larger than L2 (151 MB of triangles + 80 MB atlas + 25 MB cubemap per step)",
            "parallelism": "replicas"}


# ---- clocks ----------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---- roofline ------------------------------------------------------------------
def algorithmic_bytes(stage, T, T_vis, P, P_cov, n_cubes):
    """Compulsory DRAM bytes of one launch of a stage (intermediates such as
    records, bins and the per-pixel record map excluded):
      shadow_setup / view_setup: 40 B per scene triangle (3 positions + object id)
      shadow_raster: 6*1024^2*4 B per cubemap written
      view_raster: depth + id written, 8 B per pixel
      view_shade: depth + record map read and RGBA8 written (12 B/px), 96 B of
                  vertex data (positions, normals, uv) per visible triangle,
                  16 B of texels per covered pixel
    """
    if stage in ("shadow_setup", "view_setup"):
        return 40 * T
    if stage == "shadow_raster":
        return 6 * 1024 * 1024 * 4 * n_cubes
    if stage == "view_raster":
        return 8 * P
    if stage == "view_shade":
        return 12 * P + 96 * T_vis + 16 * P_cov
    return None


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_profile():
    """Per-launch figures of the committed ncu capture of this workload:
    DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) and warp
    instructions (smsp__inst_executed.sum) per stage."""
    p = os.path.join(ROOT, "profiles", "traffic_terrain_1080p.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def load_traffic(stage):
    return load_profile().get(stage)


def issue_roofline(stage, launch_ms, sm_mhz):
    """The issue-rate bound of an instruction-bound kernel: its warp
    instructions per launch (ncu) over the live launch time, against one warp
    instruction per clock on each of the 4 schedulers of every SM."""
    inst = load_profile().get("warp_inst", {}).get(stage)
    if not inst or not launch_ms or not sm_mhz:
        return None
    try:
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    except Exception:
        sms = 152
    achieved = inst / (launch_ms * 1e-3)
    peak = sms * 4 * sm_mhz * 1e6
    return {"achieved_warp_inst_per_s": round(achieved, 0), "peak_warp_inst_per_s": round(peak, 0),
            "frac": round(achieved / peak, 4), "warp_inst_per_launch": inst, "sms": sms, "sm_mhz": sm_mhz,
            "source": "smsp__inst_executed.sum of the committed ncu capture / live launch time"}


# ---- CPU baseline --------------------------------------------------------------
def cpu_impl():
    """The reference's own cl2.cl kernels compiled as C++ (oracle/_ref, kind
    "reference") when they build here, else the C++ restatement (kind "port")."""
    try:
        from oracle.clref import ref as R
        if R.available():
            R.lib()
            return "reference", R
    except Exception:
        pass
    return "port", None


def cpu_frames(sc, seconds, max_frames, threads):
    """Time full frames (shadow cubemaps + prearrange + kernel1 + kernel2 +
    kernel3) on the host cores; returns (kind, pixels per frame, seconds per frame)."""
    from oracle import oracle as O
    kind, R = cpu_impl()
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    cam, view = sc.cameras[0], sc.views[0]
    W = int(view["width"])
    P = W * int(view["height"])
    fov = O.fov_const(float(view["hfov_deg"]), W)
    atlas = R.textures(sc.tex_sizes, sc.tex_pixels, tex.nums, tex.sizes, tex.mipmap_start) if R else None
    times = []
    t_end = time.perf_counter() + seconds
    while len(times) < max_frames and (not times or time.perf_counter() < t_end):
        t0 = time.perf_counter()
        if R:
            dyn, sta = R.shadow(sc, nthreads=threads, ordered=False)
            R.render(sc, atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov, dyn, sta,
                     nthreads=threads, ordered=False)
        else:
            dyn, sta = O.shadow(sc, nthreads=threads)
            O.render(sc, tex, cam, view, dyn, sta, nthreads=threads)
        times.append(time.perf_counter() - t0)
    return kind, P, times


def host_cpu():
    """nproc and the CPU model of this host (for the CPU baseline record)."""
    model = None
    try:
        for line in open("/proc/cpuinfo"):
            k, _, v = line.partition(":")
            if k.strip() in ("model name", "Model", "CPU part") and v.strip():
                model = v.strip()
                if k.strip() == "model name":
                    break
    except OSError:
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model or "unknown", "machine": os.uname().machine}


def cpu_sample_text(kind, n, threads):
    what = ("the reference's cl2.cl kernels compiled as C++ (prearrange work items in parallel)" if kind == "reference"
            else "cl2.cl restated in C++")
    return (f"{n} full frames of the 1080p terrain (shadow cubemap + prearrange + kernel1 + kernel2 + kernel3), "
            f"{threads} threads, {what}")


def run_reference(args, world, rank):
    if rank != 0:
        return
    sc = scenes.terrain()
    threads = os.cpu_count() or 1
    kind, P, times = cpu_frames(sc, 1e9, args.warmup + args.steps, threads)
    t = times[args.warmup:] or times
    mpix = P * len(t) / sum(t) / 1e6
    line = {"metric": METRIC, "value": round(mpix, 4), "unit": "Mpix/s", "n_gpus": args.gpus,
            "steps": len(t), "warmup": args.warmup, "ms_per_step": round(1e3 * sum(t) / len(t), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded terrain generator)", "impl": "reference",
            "config": scene_config(sc),
            "cpu_baseline": {"value": round(mpix, 4), "unit": "Mpix/s", "cores": threads, "kind": kind,
                             "sample": cpu_sample_text(kind, len(t), threads)},
            "e2e": {"value": round(mpix, 4), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- serving -----------------------------------------------------------------------
def run_serving(args, stream):
    """4 resident scenes (100k / 500k / 1M / 2M triangles); Poisson arrivals at
    a sweep of offered loads; each request a random scene, camera pose and
    resolution from {640x480, 1280x720, 1920x1080, 3840x2160}; results copied
    to host memory.  Reports throughput and p50/p99 latency per load, and the
    reference kernels' per-request CPU latency at each resolution."""
    import torch
    from openclrenderer_gb300.pipeline import GpuScene, Server
    sizes = (100_000, 500_000, 1_000_000, 2_000_000)
    scs = [scenes.serving_scene(n, seed=9 + i) for i, n in enumerate(sizes)]
    gss = [GpuScene(sc) for sc in scs]
    for g in gss:
        g.shadow_pass(stream)
    torch.cuda.synchronize()
    rng = np.random.default_rng(9)
    res = scenes.RESOLUTIONS_SERVE
    maxp = max(w * h for w, h in res)
    pinned = torch.empty(64 * maxp * 4, dtype=torch.uint8, pin_memory=True).numpy()
    pool = [pinned[i * maxp * 4:(i + 1) * maxp * 4] for i in range(64)]
    budget = 6 << 30
    loads = []
    # the default server (one batch per scene on the GPU at once, launched as
    # soon as its scene has requests), then one GPU slot over all scenes with
    # a 2 ms batching window
    batching = {"max_inflight": 1, "batch_window_us": 2000}
    for rate, cfg in ((100.0, {}), (400.0, {}), (1600.0, {}), (float("inf"), {}), (1600.0, batching),
                      (float("inf"), batching)):
        reqs = []
        for k in range(args.serve_requests):
            w, h = res[int(rng.integers(0, len(res)))]
            reqs.append((int(rng.integers(0, len(sizes))), scenes.random_pose(rng), S.make_view(int(w), int(h))))
        srv = Server(gss, hbm_budget_bytes=budget, **cfg)
        # warm-up (untimed): a burst of the same scenes and resolutions from
        # other camera poses, so that the scenes' scratch and the workers'
        # output pools are sized for the batches this mix forms (a batch that
        # outgrows its scratch is re-run at the larger size)
        wrng = np.random.default_rng(10)
        for k, (s_i, cam, view) in enumerate(reqs):
            srv.submit(s_i, scenes.random_pose(wrng), view,
                       rgba=pool[k % len(pool)][:int(view["width"]) * int(view["height"]) * 4], tag=0)
        srv.drain()
        srv.poll(cap=4096)
        t0 = time.perf_counter()
        t_next = t0
        for k, (s_i, cam, view) in enumerate(reqs):
            if rate != float("inf"):
                t_next += float(rng.exponential(1.0 / rate))
                while time.perf_counter() < t_next:
                    pass
            P = int(view["width"]) * int(view["height"])
            srv.submit(s_i, cam, view, rgba=pool[k % len(pool)][:P * 4], tag=1 + k)
        srv.drain()
        wall = time.perf_counter() - t0
        done = srv.poll(cap=4096)
        st = srv.stats()
        srv.close()
        lat = done["latency_ms"]
        pix = sum(int(reqs[int(t) - 1][2]["width"]) * int(reqs[int(t) - 1][2]["height"]) for t in done["user_tag"])
        scene_of = np.array([reqs[int(t) - 1][0] for t in done["user_tag"]])
        per_scene = {}
        for si, n in enumerate(sizes):
            ls = lat[scene_of == si]
            if len(ls):
                per_scene[f"{n // 1000}k"] = {"requests": int(len(ls)), "p50_ms": round(float(np.percentile(ls, 50)), 3),
                                              "p99_ms": round(float(np.percentile(ls, 99)), 3)}
        loads.append({"offered_req_per_s": None if rate == float("inf") else rate, "server": cfg or "default",
                      "per_scene": per_scene,
                      "completed": int(len(done)), "ok": int(np.count_nonzero(done["status"] == 0)),
                      "wall_s": round(wall, 3),
                      "throughput_mpix_s": round(pix / wall / 1e6, 1),
                      "throughput_req_s": round(len(done) / wall, 1),
                      "p50_ms": round(float(np.percentile(lat, 50)), 3),
                      "p99_ms": round(float(np.percentile(lat, 99)), 3),
                      "mean_batch_views": round(float(np.mean(done["batch_views"])), 2),
                      "peak_admitted_mb": round(st["peak_admitted_bytes"] / 2 ** 20, 1)})
    # the plain single-view pipeline on the same requests (the burst list), one
    # call at a time with the same host outputs: the served-vs-plain ratio
    for s_i, cam, view in reqs[:4]:
        P = int(view["width"]) * int(view["height"])
        gss[s_i].render_host(cam, view, False, False,
                             pool[0][:P * 4].reshape(int(view["height"]), int(view["width"]), 4), stream=stream)
    t0 = time.perf_counter()
    pix = 0
    plain_lat = []
    for k, (s_i, cam, view) in enumerate(reqs):
        P = int(view["width"]) * int(view["height"])
        s0 = time.perf_counter()
        gss[s_i].render_host(cam, view, False, False,
                             pool[k % len(pool)][:P * 4].reshape(int(view["height"]), int(view["width"]), 4),
                             stream=stream)
        plain_lat.append(1e3 * (time.perf_counter() - s0))
        pix += P
    plain_wall = time.perf_counter() - t0
    plain = {"form": "gbr_render_view_host per request, sequential", "throughput_mpix_s": round(pix / plain_wall / 1e6, 1),
             "p50_ms": round(float(np.percentile(plain_lat, 50)), 3),
             "p99_ms": round(float(np.percentile(plain_lat, 99)), 3)}
    plain["served_burst_vs_plain"] = round(loads[3]["throughput_mpix_s"] / plain["throughput_mpix_s"], 3)
    plain["served_burst_batching_vs_plain"] = round(loads[5]["throughput_mpix_s"] / plain["throughput_mpix_s"], 3)
    for g in gss:
        g.close()
    # reference kernels on the host cores: one request of every scene at each
    # resolution (the scene's shadow cubemap rendered once, as the server does)
    cpu_lat = {}
    kind, R = cpu_impl()
    if R is not None:
        from oracle import oracle as O
        cam = scenes.random_pose(np.random.default_rng(1))
        for si, sc in enumerate(scs):
            tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
            atlas = R.textures(sc.tex_sizes, sc.tex_pixels, tex.nums, tex.sizes, tex.mipmap_start)
            dyn, sta = R.shadow(sc, ordered=False)
            row = {}
            for w, h in res:
                view = S.make_view(w, h)
                t0 = time.perf_counter()
                R.render(sc, atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, O.fov_const(90.0, w), dyn, sta,
                         ordered=False)
                row[f"{w}x{h}"] = round(1e3 * (time.perf_counter() - t0), 1)
            cpu_lat[f"{sizes[si] // 1000}k"] = row
    return {"workload": "4 resident scenes (100k/500k/1M/2M triangles), Poisson arrivals, resolutions "
                        "640x480/1280x720/1920x1080/3840x2160", "hbm_budget_gb": budget / 2 ** 30,
            "requests_per_load": args.serve_requests, "loads": loads, "plain_sequential": plain,
            "cpu_reference_latency_ms_per_scene": cpu_lat, "cpu_kind": kind,
            "cpu_threads": os.cpu_count()}


# ---- GPU ------------------------------------------------------------------------
def main():
    args = parse()
    world, rank, local = dist_env()
    if args.profile_pass:
        profile_pass()
        return
    if args.profile_batch:
        profile_batch()
        return
    if args.tile_stats:
        tile_stats()
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    import torch
    import torch.distributed as dist
    from openclrenderer_gb300.pipeline import Batch, GpuScene

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    sc = scenes.terrain()
    cam, view = sc.cameras[0], sc.views[0]
    W, H = int(view["width"]), int(view["height"])
    P = W * H
    gs = GpuScene(sc)
    out = None
    stream = torch.cuda.current_stream()

    def step():
        gs.shadow_pass(stream)
        return gs.render(cam, view, out=out, stream=stream)

    out = step()
    for _ in range(max(args.warmup, 3) - 1):
        step()
    torch.cuda.synchronize()
    depth = out.depth.cpu().numpy().view(np.uint32)
    P_cov = int(np.count_nonzero(depth != 0xFFFFFFFF))
    launches0 = gs.stats()["launches"]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = gs.stats()["launches"] - launches0
    ms = max_over_ranks(ms, world, "cuda")
    if world > 1:
        dist.barrier()
    value = job_mpix_per_s(P, world, ms)
    # stage times: the same frames again, after the timed region, with the
    # scene's per-stage CUDA events on (they add event records of their own)
    gs.profile(True)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    st = gs.stats()
    gs.profile(False)

    # per-stage device time and the roofline of the dominant kernel
    per_call = {k: st["stage_ms"][k] / max(st["stage_calls"][k], 1) for k in S.STAGES}
    dom = max(per_call, key=per_call.get)
    T = len(sc.tris)
    T_vis = st["view_records"]
    n_cubes = int(sum(1 for l in sc.lights if l["shadow"] == 1))
    peak, peak_kind = load_peaks()
    alg = algorithmic_bytes(dom, T, T_vis, P, P_cov, n_cubes)
    achieved = alg / (per_call[dom] * 1e-3) / 1e9 if alg else None
    roof = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 2) if achieved else None,
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": round(achieved / peak, 5) if achieved else None,
            "algorithmic_bytes_per_launch": alg, "launch_ms": round(per_call[dom], 4),
            "traffic": load_traffic(dom),
            "issue": issue_roofline(dom, per_call[dom], clk.get("sm_mhz") if clk else None)}

    # end to end through the host-buffer C ABI call
    pin = torch.empty(P * 12, dtype=torch.uint8, pin_memory=True).numpy()
    hd, hi, hr = pin[:4 * P].view(np.uint32), pin[4 * P:8 * P].view(np.uint32), pin[8 * P:]
    for _ in range(2):
        gs.shadow_pass(stream)
        gs.render_host(cam, view, hd, hi, hr, stream=stream)
    lat = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s0 = time.perf_counter()
        gs.shadow_pass(stream)
        gs.render_host(cam, view, hd, hi, hr, stream=stream)
        lat.append(time.perf_counter() - s0)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": round(world * P * args.steps / e2e_s / 1e6, 3), "unit": "Mpix/s",
           "h2d_bytes_per_step": S.CAMERA.itemsize + S.VIEW.itemsize, "d2h_bytes_per_step": 12 * P,
           "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
           "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3)}

    # batched form: many views of the same scene per launch
    batched = None
    if not args.no_batch:
        rng = np.random.default_rng(17)
        cams = [S.make_camera((rng.uniform(-400, 400), rng.uniform(-60, 60), rng.uniform(-100, 200)),
                              (scenes.TERRAIN_CAMERA_PITCH + rng.uniform(-0.1, 0.1), rng.uniform(-0.4, 0.4), 0))
                for _ in range(args.batch_views)]
        views = [view] * args.batch_views
        outs = gs.render_batch(cams, views, stream=stream)
        for _ in range(2):
            gs.shadow_pass(stream)
            gs.render_batch(cams, views, outs=outs, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nb = max(3, args.steps // 4)
        e0.record(stream)
        for _ in range(nb):
            gs.shadow_pass(stream)
            gs.render_batch(cams, views, outs=outs, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        bms_plain = e0.elapsed_time(e1) / nb
        # the same frame as one captured graph (shadow cubemap + 16 views), autotuned
        gb = Batch(gs, views, outs=outs, with_shadow=True)
        pick = gb.autotune(cams, reps=3, stream=stream)
        gb.render(cams, stream=stream)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(nb):
            gb.launch(cams, stream=stream)
        gb.wait()
        e1.record(stream)
        torch.cuda.synchronize()
        bms = e0.elapsed_time(e1) / nb
        info = gb.info()
        gb.close()
        batched = {"views_per_launch": args.batch_views, "ms_per_batch": round(bms, 3),
                   "value": round(world * P * args.batch_views / (bms * 1e-3) / 1e6, 2), "unit": "Mpix/s",
                   "vs_plain": round((P * args.batch_views / bms) / (P / ms), 3),
                   "form": "captured graph (shadow cubemap + views), autotuned",
                   "ms_per_batch_uncaptured": round(bms_plain, 3), "tuning": pick,
                   "graph_nodes": info["graph_nodes"]}

    # binning stress (2,000,000 sub-pixel + 1,000 screen-covering triangles, 2560x1440)
    stress = None
    if not args.no_extra:
        st_sc = scenes.binning_stress()
        sgs = GpuScene(st_sc)
        scam, sview = st_sc.cameras[0], st_sc.views[0]
        so = sgs.render(scam, sview, stream=stream)
        sgs.render(scam, sview, out=so, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            sgs.render(scam, sview, out=so, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        sms = e0.elapsed_time(e1) / 3
        sst = sgs.stats()
        stress = {"workload": "binning_stress_2560x1440_2M_subpixel_1k_fullscreen", "ms_per_frame": round(sms, 3),
                  "value": round(2560 * 1440 / (sms * 1e-3) / 1e6, 2), "unit": "Mpix/s",
                  "reference_fragments": sst["fragments_ref"], "records": sst["view_records"],
                  "bin_entries": sst["view_bin_entries"]}
        sgs.close()
        del st_sc

    # batched mixed resolutions: 64 views of 500 spheres (500k triangles) in one
    # launch per stage, against the same 64 views rendered one call at a time
    mixed = None
    if not args.no_extra:
        mb = scenes.spheres_batch()
        mgs = GpuScene(mb)
        mpix = sum(int(v["width"]) * int(v["height"]) for v in mb.views)
        outs = mgs.render_batch(mb.cameras, mb.views, stream=stream)
        mgs.render_batch(mb.cameras, mb.views, outs=outs, stream=stream)
        singles = [mgs.render(c, v, stream=stream) for c, v in zip(mb.cameras, mb.views)]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            mgs.render_batch(mb.cameras, mb.views, outs=outs, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        bms_uncaptured = e0.elapsed_time(e1) / 3
        # stage times of one uncaptured batch
        mgs.profile(True)
        mgs.render_batch(mb.cameras, mb.views, outs=outs, stream=stream)
        mst = mgs.stats()
        mgs.profile(False)
        batch_stages = {k: round(v, 4) for k, v in mst["stage_ms"].items() if k.startswith("view")}
        # captured graph, autotuned
        gb = Batch(mgs, mb.views, outs=outs)
        pick = gb.autotune(mb.cameras, reps=3, stream=stream)
        gb.render(mb.cameras, stream=stream)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(3):
            gb.launch(mb.cameras, stream=stream)
        gb.wait()
        e1.record(stream)
        torch.cuda.synchronize()
        bms = e0.elapsed_time(e1) / 3
        gb.close()
        e0.record(stream)
        for _ in range(2):
            for c, v, o in zip(mb.cameras, mb.views, singles):
                mgs.render(c, v, out=o, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1) / 2
        mixed = {"workload": "spheres_500x1000tris_64views_mixed_res", "views": len(mb.views), "pixels": mpix,
                 "batched_ms": round(bms, 3), "plain_ms": round(pms, 3),
                 "form": "captured graph, autotuned", "batched_uncaptured_ms": round(bms_uncaptured, 3),
                 "tuning": pick["view"], "batch_stage_ms": batch_stages,
                 "batched_mpix_s": round(mpix / (bms * 1e-3) / 1e6, 1),
                 "plain_mpix_s": round(mpix / (pms * 1e-3) / 1e6, 1), "batched_vs_plain": round(pms / bms, 3)}
        mgs.close()

    serving = None
    if not args.no_extra and not args.no_serve:
        serving = run_serving(args, stream)

    # post passes over the measured 1080p frame (godrays with two shaft lights)
    post = None
    if not args.no_extra:
        glights = sc.lights.copy()
        glights["godray_intensity"][:2] = 1.0
        gs.set_lights(glights)
        gout = torch.empty_like(out.rgba)
        for _ in range(3):
            gs.post_godrays(cam, view, out, rgba_out=gout, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            gs.post_godrays(cam, view, out, rgba_out=gout, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        gms = e0.elapsed_time(e1) / 10
        post = {"godrays": {"lights": 2, "ms": round(gms, 4), "value": round(P / (gms * 1e-3) / 1e6, 1),
                            "unit": "Mpix/s"},
                "note": "each pass out of place over the measured frame's buffers (L2-resident between launches)"}
        gs.set_lights(sc.lights)

        def time_pass(fn, reps=10):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / reps
            return {"ms": round(t, 4), "value": round(P / (t * 1e-3) / 1e6, 1), "unit": "Mpix/s"}

        nout = gs.render(cam, view, normals=True, stream=stream)
        post["pseudo_aa"] = time_pass(lambda: gs.post_pseudo_aa(view, nout, rgba_out=gout, stream=stream))
        prev = np.array(cam, S.CAMERA)
        prev["pos"][:3] += np.float32([4.0, 1.0, -6.0])
        prev["rot"][:2] += np.float32([0.004, -0.006])
        post["motion_blur"] = time_pass(lambda: gs.post_motion_blur(cam, prev, view, out, 2, 1.0, 0.5,
                                                                    rgba_out=gout, stream=stream))
        rdescs = sc.descs.copy()
        rdescs["feature_flag"] |= 1
        gs.set_descriptors(rdescs)
        post["reflections"] = time_pass(lambda: gs.post_reflections(cam, view, out, rgba_out=gout, stream=stream))
        post["reflections"]["note"] = "every object reflective"
        gs.set_descriptors(sc.descs)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        kind, Pc, times = cpu_frames(sc, args.cpu_seconds, 8, threads)
        t = times[1:] if len(times) > 1 else times
        cpu = {"value": round(Pc * len(t) / sum(t) / 1e6, 4), "unit": "Mpix/s", "cores": threads, "kind": kind,
               "sample": cpu_sample_text(kind, len(t), threads) + ", after 1 warm-up frame",
               "host": host_cpu()}
        # one frame on one core, for the single-thread figure
        _, _, t1 = cpu_frames(sc, 0.0, 1, 1)
        cpu["single_thread"] = {"value": round(Pc / t1[0] / 1e6, 4), "unit": "Mpix/s", "cores": 1,
                                "sample": cpu_sample_text(kind, 1, 1)}

    # covered pixel-samples per second against the device's measured atomicMin
    # rates: views resolve them in shared memory (k_raster), cube faces mostly
    # with global atomics from the setup (small triangles) and the rest in
    # shared memory
    rates = {}
    for mode, name in ((1, "shared"), (0, "global")):
        r = ctypes.c_double(0.0)
        if gs.L.gbr_atomic_rate(mode, ctypes.byref(r)) == 0:
            rates[name] = r.value
    v_rate = st["view_samples"] / (per_call["view_raster"] * 1e-3)
    s_rate = st["shadow_samples"] / ((per_call["shadow_setup"] + per_call["shadow_raster"]) * 1e-3)
    raster_samples = {
        "view": st["view_samples"], "shadow": st["shadow_samples"],
        "view_gsamples_per_s": round(v_rate / 1e9, 3), "shadow_gsamples_per_s": round(s_rate / 1e9, 3),
        "atomic_peak_gops": {k: round(v / 1e9, 1) for k, v in rates.items()},
        "view_frac_of_shared_atomic_peak": round(v_rate / rates["shared"], 5) if "shared" in rates else None,
        "shadow_frac_of_global_atomic_peak": round(s_rate / rates["global"], 5) if "global" in rates else None,
        "note": "one depth atomicMin per covered sample, per second of the pass's raster (views) or setup + raster "
                "(cube faces), against the measured 32-bit atomicMin rate of this GPU (gbr_atomic_rate): "
                "the rasters are not atomic-bound"}

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded value-noise terrain, random textures)",
                "config": scene_config(sc), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": int(launches), "clocks": clk,
                "stages_ms": {k: round(v, 4) for k, v in per_call.items()},
                "covered_mpix_s": round(job_mpix_per_s(P_cov, world, ms), 3),
                "raster_samples": raster_samples,
                "batched": batched, "binning_stress": stress, "batched_mixed": mixed, "serving": serving,
                "post_passes": post,
                "impl": "gbr",
                "counts": {"visible_records": T_vis, "covered_px": P_cov, "reference_fragments": st["fragments_ref"],
                           "view_bin_entries": st["view_bin_entries"], "shadow_records": st["shadow_records"]}}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
