"""Benchmark: progressive path tracing throughput (Mrays/s) on GB300.

One step = one pass of the wavefront path tracer over one frame: 1 sample per
pixel of the material-sweep workload (8x8 icosphere grid, 327,684 triangles,
1920x1080, max depth 12, point light + quad emitter), i.e. one call of the
reference's per-frame launch. Ray count = extension rays + shadow rays
actually traced. That is the headline (`value`, `e2e`, `roofline`,
`cpu_baseline`); the same line also carries, under "workloads":

  cornell   512x512 Cornell box, 64 spp, depth 8: GPU throughput, and the CPU
            baseline timed on the whole frame at 64 spp
  terrain   the 9,996,610-triangle textured, alpha-masked terrain, 1920x1080,
            depth 16, measured like the headline (own roofline, e2e, CPU sample)
  guided    learned guiding vs plain at equal wall time on the doorway-lit
            interior, 1280x720, depth 12, 5 seeds, against a 65,536-spp plain
            FP64-accumulated reference of the same frame
  batch     96 views of the terrain and the sweep (sides log-uniform
            128..1024, spp U{16..256}, depth 12, guiding on): aggregate
            throughput, per-view relMSE against FP64 references, HBM fraction

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sweep|terrain|batch] [--quick]

--impl reference times the reference algorithm's CPU restatement (the oracle
integrator, FP32, all host threads) on the headline workload, because the
reference's own OptiX path does not build here; that process loads only the
oracle (the scene comes from a file the library writes in a child process).
Multi-GPU (torchrun): every rank renders its own replica of the frame (the
work is independent per pixel and sample, so there is no data-path
collective); value = rays of all ranks / slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "sweep": {"workload": "material sweep: 8x8 icospheres (subdiv 4) + ground, 327,684 tris, point light + quad emitter",
              "scene": "spheres", "width": 1920, "height": 1080, "max_depth": 12, "spp_per_step": 1},
    "terrain": {"workload": "terrain: 2048x2048-quad fBm height field + 20,000 rocks (30% glass) + 4,000 alpha-masked "
                            "textured foliage cards, normal-mapped ground, 9,996,610 tris, sun quad emitter",
                "scene": "terrain", "width": 1920, "height": 1080, "max_depth": 16, "spp_per_step": 1},
}
CORNELL = {"workload": "Cornell box: 36 tris, quad light (17,12,4), Oren-Nayar walls and boxes",
           "scene": "cornell", "width": 512, "height": 512, "max_depth": 8, "spp": 64}
CPU_SPP = {"sweep": 36, "terrain": 32}  # CPU-baseline sample: about 10-30 s of host work
# Learned guiding vs plain at equal wall time (the headline's second half):
# the indirect-lit interior (1,947,146 tris) at its full 1280x720, against a
# 65,536-spp plain FP64-accumulated reference of the same frame.
GUIDED = {"workload": "indirect-lit interior (doorway only), 1,947,146 tris, depth 12",
          "scene": "interior", "width": 1280, "height": 720, "reference_spp": 65536, "budget_s": 10.0,
          "seeds": [11, 12, 13, 14, 15],
          # guided: online training for the first 1,024 samples per pixel
          # (one path in two records; 512 passes of 2 spp, each with 4 Adam
          # steps), then the network is frozen; mixture selection probability
          # capped at 0.6; the first 6 bounces guided, the path-completion
          # kernel from bounce 7 on (from bounce 8 while the network trains;
          # plain: from bounce 5, the default)
          "guiding_options": {"trainSpp": 1024, "trainStride": 2, "alphaMax": 0.6, "maxDepth": 6},
          "guided_tail_bounce": 7}
BATCH = {"workload": "batched multi-view: 96 views (48 of the terrain, 48 of the material sweep), sides "
                     "log-uniform 128..1024, spp U{16..256}, depth 12, guiding on; both scenes in one multi-scene "
                     "batch, each scene's renderer autotuned with guiding on (BVH tree, block size, compaction)",
         "views_per_scene": 48, "seed": 5,
         "reference_spp_factor": 4}
WORKLOAD = dict(WORKLOADS["sweep"])
METRIC = "Mrays/s (extension + shadow rays traced), progressive path tracing, 1 spp per step"
NODE_BYTES = {8: 80, 2: 64}  # compressed BVH8 node, BVH2 node
TRI_BYTES = 48       # one leaf-ordered triangle record (3 x float4)
RAY_IO_BYTES = 48    # ray in (origin, dir, tmax, path id) + hit out (t, u, v, id)
SHADE_BYTES = 256    # per hit: geometry 112 + compact material 64 + path state 80
ACCUM_BYTES = 64     # per pixel-sample: FP64 sum + sum of squares R/W amortised + output
GEN_BYTES = 64       # per path: ray out 32 + path state init 32
SMS = 152            # GB300 streaming multiprocessors
ISSUE_PER_SM_CLK = 4  # warp instructions issued per SM per clock (four schedulers)


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples go to $OPTPT_CLOCKS_CSV if set, else to a temporary file
        self.path = os.environ.get("OPTPT_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(), "optpt_clocks.csv")

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _camera_basis(eye, target, up, fov, aspect):
    """Camera::setupUvwCoordinatSystem (src/camera.cpp:19-40)."""
    e, t, u = (np.array(v, np.float64) for v in (eye, target, up))
    W = t - e
    W /= np.linalg.norm(W)
    u /= np.linalg.norm(u)
    U = np.cross(u, -W)
    U /= np.linalg.norm(U)
    V = np.cross(-W, U)
    V /= np.linalg.norm(V)
    vl = np.tan(0.5 * np.radians(fov))
    return list((U * vl * aspect).astype(np.float32)), list((V * vl).astype(np.float32)), list(W.astype(np.float32))


def cpu_render(scene, wl, rows, threads, spp=1, sample_base=1000):
    """Times the oracle integrator (FP32, `threads` host threads) on a band of
    `rows` rows (centred) of the workload frame. Returns (seconds, rays,
    pixel samples)."""
    from oracle import oracle as orc
    a = scene.arrays()
    w, h = wl["width"], wl["height"]
    U, V, W = _camera_basis(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"], w / h)
    cam = list(a["camEye"]) + U + V + W + list(a["bgColour"])
    view = orc.SceneView(scene.struct, 4)
    y0 = (h - rows) // 2
    t0 = time.perf_counter()
    _, _, cnt = view.render(cam, w, h, 1, sample_base, spp, wl["max_depth"], y0=y0, y1=y0 + rows,
                            precision=32, threads=threads)
    dt = time.perf_counter() - t0
    return dt, int(cnt[0] + cnt[1]), rows * w * spp


def _scene_for_oracle(name):
    """The workload scene for the CPU-only arm: the library generates it in a
    child process (untimed) and writes it to a file, which the oracle reads,
    so this process never loads the CUDA library."""
    from oracle import scene_file
    path = os.path.join(tempfile.gettempdir(), "optpt_scene_%s_%d.npz" % (name, os.getpid()))
    code = ("import sys; sys.path.insert(0, %r); import __graft_entry__ as g; g.build(); "
            "import optix_pt_gb300 as opt; opt.Scene.procedural(%r).save(%r)" % (ROOT, name, path))
    subprocess.run([sys.executable, "-c", code], check=True)
    try:
        return scene_file.load(path)
    finally:
        os.remove(path)


def reduce_over_ranks(values, n_max, world):
    """The job's aggregate of per-rank measurements (a float64 tensor, the
    same layout on every rank): the first n_max entries by their maximum over
    ranks (times: the job is as slow as its slowest replica), the rest by
    their sum (work: rays, samples). One rank: the values as they are."""
    if world > 1:
        import torch.distributed as dist
        head, tail = values[:n_max].clone(), values[n_max:].clone()
        dist.all_reduce(head, op=dist.ReduceOp.MAX)
        dist.all_reduce(tail, op=dist.ReduceOp.SUM)
        return head.tolist() + tail.tolist()
    return values.tolist()


def _config(world):
    """The headline workload, as both arms report it (identical dicts)."""
    return dict(WORKLOAD, l2="flushed between timed steps (256 MB write, outside the events)")


def run_reference(args, rank, world):
    """The reference arm: the oracle integrator on the host cores."""
    if rank != 0:
        return
    scene = _scene_for_oracle(WORKLOAD["scene"])
    threads = os.cpu_count()
    rows = WORKLOAD["height"]
    for _ in range(args.warmup):
        cpu_render(scene, WORKLOAD, 64, threads)
    tot_t, tot_rays, tot_samples = 0.0, 0, 0
    for k in range(args.steps):
        dt, rays, samples = cpu_render(scene, WORKLOAD, rows, threads, sample_base=2000 + k)
        tot_t += dt
        tot_rays += rays
        tot_samples += samples
    value = tot_rays / tot_t / 1e6
    sample = "one step = the full %dx%d frame at 1 spp, depth %d, FP32 oracle integrator" % (
        WORKLOAD["width"], WORKLOAD["height"], WORKLOAD["max_depth"])
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)", "config": _config(world),
            "parallelism": "%d host threads" % threads,
            "samples_per_s": tot_samples / tot_t,
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _ncu_record(workload, kernel):
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tp):
        return None
    return json.load(open(tp)).get(workload, {}).get(kernel)


def roofline_of(name, r, prof, cnt, w, h, bvh_width, sm_mhz):
    """HBM roofline of the dominant kernel of a profiled pass (algorithmic
    bytes per launch / CUDA-event time per launch), DRAM traffic per launch
    from the committed ncu capture, and the issue-rate bound of the
    traversal kernels (warp instructions per ray from the same capture).
    Rays are split between the per-bounce kernels and the path-completion
    kernel by the pass's per-bounce queue counts."""
    kms = prof["ms"]
    dominant = max(kms, key=kms.get)
    ext_rays = max(1, cnt["extensionRays"])
    sh_rays = max(1, cnt["shadowRays"])
    nodes_ext, tris_ext = cnt["extensionNodes"] / ext_rays, cnt["extensionTris"] / ext_rays
    nodes_sh, tris_sh = cnt["shadowNodes"] / sh_rays, cnt["shadowTris"] / sh_rays
    nb = NODE_BYTES[bvh_width]
    bytes_ext = RAY_IO_BYTES + nodes_ext * nb + tris_ext * TRI_BYTES
    bytes_sh = RAY_IO_BYTES + 4 + nodes_sh * nb + tris_sh * TRI_BYTES
    e, p, m = (x.astype(np.float64) for x in r.queue_counts())   # the profiled render's last pass
    tail = r.stats()["tailBounce"] or len(e) + 1
    scale = prof["extensionRays"] / max(1.0, e.sum())             # passes in the profiled render
    ext_w, ext_t = e[:tail - 1].sum() * scale, e[tail - 1:].sum() * scale
    sh_w, sh_t = (p + m)[:tail - 1].sum() * scale, (p + m)[tail - 1:].sum() * scale
    per_kernel_bytes = {
        "extend": bytes_ext * ext_w,
        "shadow": bytes_sh * sh_w,
        "shade": float(SHADE_BYTES) * ext_w,
        "finish": (bytes_ext + SHADE_BYTES) * ext_t + bytes_sh * sh_t,
        "accumulate": float(ACCUM_BYTES) * 2 * w * h,
        "generate": float(GEN_BYTES) * 2 * w * h,
    }
    rays_of = {"extend": ext_w, "shadow": sh_w, "shade": ext_w, "finish": ext_t + sh_t}
    peak, peak_kind = _peaks()
    nl = max(1, prof["launches"][dominant])
    achieved = (per_kernel_bytes[dominant] / nl) / (kms[dominant] / nl / 1e3) / 1e9
    kname = {"extend": "kExtend", "shadow": "kShadow", "shade": "kShade", "finish": "kFinish"}.get(dominant)
    traffic = None
    rec = _ncu_record(name, kname) if kname else None
    if rec and rec.get("rays_per_launch"):
        traffic = rec["dram_bytes_per_launch"] / rec["rays_per_launch"] * (rays_of[dominant] / nl)
    # Issue-rate bound: the traversal kernels are limited by instruction
    # issue, not by DRAM (their nodes come from L2). peak = SMs x 4 warp
    # instructions per clock at the SM clock sampled during the timed steps.
    issue = {}
    clk = (sm_mhz or 2070.0) * 1e6
    for k, kn in (("extend", "kExtend"), ("shadow", "kShadow"), ("finish", "kFinish")):
        rec = _ncu_record(name, kn)
        if not rec or not rec.get("warp_inst_per_launch") or kms.get(k, 0) <= 0:
            continue
        ipr = rec["warp_inst_per_launch"] / rec["rays_per_launch"]
        achieved_i = ipr * rays_of[k] / (kms[k] / 1e3)
        peak_i = SMS * ISSUE_PER_SM_CLK * clk
        issue[kn] = {"warp_inst_per_ray": ipr, "achieved_ginst_s": achieved_i / 1e9, "peak_ginst_s": peak_i / 1e9,
                     "frac": achieved_i / peak_i, "sm_mhz": clk / 1e6,
                     "simd_efficiency": rec.get("simd_efficiency")}
    return {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "bytes_per_ray": {"extension": bytes_ext, "shadow": bytes_sh},
            "bvh_work_per_ray": {"ext_nodes": nodes_ext, "ext_tris": tris_ext, "sh_nodes": nodes_sh,
                                 "sh_tris": tris_sh},
            "rays_per_pass": {k: v / 2 for k, v in rays_of.items()}, "tail_bounce": r.stats()["tailBounce"],
            "kernel_ms_per_pass": {k: v / 2 for k, v in kms.items()},
            "kernel_share": {k: v / sum(kms.values()) for k, v in kms.items()},
            "issue_bound": issue}


def _launches_per_pass(max_depth, tail):
    return 3 + (4 * (tail - 1) + 1 if tail else 4 * max_depth)


def measure_frames(name, args, rank, world, dev, stream, with_cpu):
    """One workload of 1-spp passes: device-timed throughput (L2 flushed
    between steps), end-to-end throughput through the public API with host
    buffers, the roofline of the dominant kernel and (rank 0, N=1) a CPU
    baseline sample. Returns (line fields, renderer, scene, clocks)."""
    import torch
    import torch.distributed as dist

    import optix_pt_gb300 as opt
    wl = WORKLOADS[name]
    scene = opt.Scene.procedural(wl["scene"])
    r = opt.Renderer(scene, bvh_width=args.bvh_width, leaf_size=args.leaf_size, block_size=args.block_size,
                     tail_bounce=args.tail_bounce)
    w, h = wl["width"], wl["height"]
    r.setupOutputBuffer(w, h)
    a = scene.arrays()
    r.setupCamera(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"])
    r.set_max_depth(wl["max_depth"])
    lp = r.launch_params()
    lp.seed = 1 + rank
    r.updateLaunchParams(lp)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def barrier():
        if world > 1:
            dist.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            r.render(1, stream)
        torch.cuda.synchronize()
        st0 = r.stats()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        barrier()
        torch.cuda.synchronize()
        with ClockSampler(dev.index or 0) as clk:
            for k in range(args.steps):
                flush.zero_()                       # L2 flushed between timed steps (not timed)
                starts[k].record(stream)
                r.render(1, stream)
                ends[k].record(stream)
            torch.cuda.synchronize()
        barrier()
        ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
        st1 = r.stats()
    del flush
    rays = (st1["extensionRays"] - st0["extensionRays"]) + (st1["shadowRays"] - st0["shadowRays"])
    samples = st1["pathSamples"] - st0["pathSamples"]
    ms_all, rays_all, samples_all = reduce_over_ranks(
        torch.tensor([ms, float(rays), float(samples)], dtype=torch.float64, device=dev), 1, world)
    value = rays_all / (ms_all / 1e3) / 1e6

    # End to end through the public API with host buffers: per step the frame
    # constants go host -> device (80 B) and the tone-mapped frame buffer
    # (float4 per pixel) comes back into pinned host memory. The headline
    # uses the pipelined frame loop (optpt_launch_pipelined: frame k's
    # download overlaps frame k + 1's render; every frame reaches the host
    # inside the timed region, the last one by optpt_launch_flush); the
    # synchronous loop (render, then download and wait, as the reference's
    # Renderer::launch) is reported beside it.
    host_fb = torch.empty((h, w, 4), dtype=torch.float32, pin_memory=True)

    def e2e_run(pipelined):
        if pipelined:
            # untimed warm-up: the first pipelined call allocates the two
            # pinned host frames and device snapshots
            for k in range(args.warmup):
                r.launch_pipelined(copy=False)
            r.launch_flush(copy=False)
        barrier()
        torch.cuda.synchronize()
        st0 = r.stats()
        t0 = time.perf_counter()
        if pipelined:
            for k in range(args.steps):
                r.launch_pipelined(copy=False)
            r.launch_flush(copy=False)
        else:
            for k in range(args.steps):
                lp = r.launch_params()
                r.updateLaunchParams(lp)
                r.render(1, stream)
                opt.check(opt.lib.optpt_read_frame_buffer(r._h, host_fb.data_ptr(), stream.cuda_stream))
        e2e_s = time.perf_counter() - t0
        st1 = r.stats()
        e2e_rays = (st1["extensionRays"] - st0["extensionRays"]) + (st1["shadowRays"] - st0["shadowRays"])
        e_s, e_rays = reduce_over_ranks(torch.tensor([e2e_s, float(e2e_rays)], dtype=torch.float64, device=dev),
                                        1, world)
        return e_rays / e_s / 1e6

    e2e_sync = e2e_run(False)
    e2e_value = e2e_run(True)
    clocks = clk.summary()
    out = {"value": value, "ms_per_step": ms_all / args.steps, "samples_per_s": samples_all / (ms_all / 1e3),
           "rays_per_step": rays_all / args.steps / world,
           "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": 80, "d2h_bytes_per_step": w * h * 16,
                   "api": "optpt_launch_pipelined (each frame's download overlaps the next frame's render)",
                   "synchronous": {"value": e2e_sync, "api": "optpt_render + optpt_read_frame_buffer per frame "
                                                            "(render, then download and wait)"}},
           # per pass: generate, accumulate, advance, 4 per bounce (extend,
           # shade, 2 shadow) up to the path-completion bounce, then 1
           "gpu_launches": _launches_per_pass(wl["max_depth"], r.stats()["tailBounce"]) * args.steps}
    if rank == 0:
        prof = r.profile(2, stream)
        cnt = r.traversal_counts(1, stream)
        out["roofline"] = roofline_of(name, r, prof, cnt, w, h, args.bvh_width,
                                      clocks["sm_mhz"] if clocks else None)
        st = r.stats()
        out["traversal_faults"] = {k: st[k] for k in ("traversalStackOverflows", "traversalBudgetExhausted")}
        cpu = None
        if with_cpu and world == 1 and not args.no_cpu:
            threads = os.cpu_count()
            spp = args.cpu_spp or CPU_SPP[name]
            dt, crays, csamples = cpu_render(scene, wl, h, threads, spp=spp)
            cpu = {"value": crays / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                   "sample": "the full %dx%d frame at %d spp, FP32 oracle integrator, %.1f s" % (w, h, spp, dt)}
        out["cpu_baseline"] = cpu
    return out, r, scene, clocks


def measure_cornell(stream, with_cpu):
    """Config 1 at its stated size: the 512x512 Cornell box, 64 spp, depth 8,
    rendered on the GPU (one 64-spp render call, CUDA events; best of 3) and
    by the CPU baseline on the whole frame at 64 spp."""
    import torch

    import optix_pt_gb300 as opt
    c = CORNELL
    scene = opt.Scene.procedural(c["scene"])
    r = opt.Renderer(scene)
    r.setupOutputBuffer(c["width"], c["height"])
    r.set_max_depth(c["max_depth"])
    r.render(c["spp"], stream)                 # warm-up (graph capture)
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        r.resetSampleCount()
        st0 = r.stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.render(c["spp"], stream)
        e1.record(stream)
        torch.cuda.synchronize()
        st1 = r.stats()
        times.append((e0.elapsed_time(e1) / 1e3, (st1["extensionRays"] - st0["extensionRays"]) +
                      (st1["shadowRays"] - st0["shadowRays"])))
    dt, rays = min(times)
    out = {"config": dict(c), "gpu_mrays_per_s": rays / dt / 1e6,
           "gpu_msamples_per_s": c["width"] * c["height"] * c["spp"] / dt / 1e6, "gpu_ms_per_frame": dt * 1e3}
    r.close()
    if with_cpu:
        threads = os.cpu_count()
        cdt, crays, csamples = cpu_render(scene, c, c["height"], threads, spp=c["spp"])
        out["cpu_baseline"] = {"value": crays / cdt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                               "samples_per_s": csamples / cdt, "seconds": cdt,
                               "sample": "the whole 512x512 frame at 64 spp, depth 8 (all of config 1), FP32 "
                                         "oracle integrator"}
    return out


def guided_equal_time(stream, budget_s=None, reference_spp=None):
    """relMSE (mean over pixels of sum_c (I - R)^2 / (R^2 + 1e-2)) of plain and
    guided renders given the same wall-clock budget, online training included
    in the guided budget; per seed a fresh renderer (and network)."""
    import torch

    import optix_pt_gb300 as opt
    g = dict(GUIDED)
    if budget_s:
        g["budget_s"] = budget_s
    if reference_spp:
        g["reference_spp"] = reference_spp
    scene = opt.Scene.procedural(g["scene"])
    w, h = g["width"], g["height"]

    def make(seed, mode):
        r = opt.Renderer(scene, tail_bounce=g["guided_tail_bounce"] if mode else 0)
        r.setupOutputBuffer(w, h)
        r.set_seed(seed)
        if mode:
            r.set_guiding(mode)
            r.guiding_options(**g["guiding_options"])
        return r

    t0 = time.perf_counter()
    ref = make(1000, 0)
    ref.render(g["reference_spp"], stream)
    torch.cuda.synchronize()
    s, q, n = ref.accum()
    R = s.reshape(-1, 3) / n
    # variance of the reference's per-pixel mean (FP64 sum of squares): the
    # reference's own noise, which adds to every render's measured error
    var_ref = np.maximum(q.reshape(-1, 3) / n - R * R, 0.0) / (n - 1)
    den = R ** 2 + 1e-2
    ref_seconds = time.perf_counter() - t0
    ref.close()
    out = {}
    for mode, name in ((0, "plain"), (1, "guided")):
        errs, errs_c, spps, mrays = [], [], [], []
        for seed in g["seeds"]:
            r = make(seed, mode)
            batch = r.stats()["sppBatch"]
            st0 = r.stats()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            spp = 0
            while time.perf_counter() - t0 < g["budget_s"]:
                r.render(batch, stream)
                torch.cuda.synchronize()
                spp += batch
            dt = time.perf_counter() - t0
            st1 = r.stats()
            s, _, n = r.accum()
            I = s.reshape(-1, 3) / n
            errs.append(float(np.mean(((I - R) ** 2 / den).sum(1))))
            errs_c.append(float(np.mean((((I - R) ** 2 - var_ref) / den).sum(1))))
            spps.append(spp)
            mrays.append((st1["extensionRays"] - st0["extensionRays"] + st1["shadowRays"] - st0["shadowRays"]) / dt / 1e6)
            r.close()
        out[name] = {"relmse": float(np.mean(errs)), "relmse_per_seed": errs, "spp_in_budget": spps,
                     "mrays_per_s": float(np.mean(mrays)),
                     "relmse_reference_noise_removed": float(np.mean(errs_c))}
    out["relmse_ratio_plain_over_guided"] = out["plain"]["relmse"] / out["guided"]["relmse"]
    out["relmse_ratio_per_seed"] = [p / q for p, q in zip(out["plain"]["relmse_per_seed"],
                                                           out["guided"]["relmse_per_seed"])]
    # The same ratio with the reference's own variance (estimated per pixel
    # from its sum of squares) subtracted from each render's squared error.
    # The renders and the reference draw independent samples, so this
    # estimates each render's error against the noise-free image (the
    # denominators still use the reference). Reported beside the protocol's
    # ratio, which stays the headline.
    out["relmse_ratio_reference_noise_removed"] = (out["plain"]["relmse_reference_noise_removed"] /
                                                   out["guided"]["relmse_reference_noise_removed"])
    out["config"] = dict(g, reference_seconds=ref_seconds,
                         protocol="equal wall time per seed (budget_s of rendering each, online training inside "
                                  "the guided budget); relMSE is the mean over seeds of each render's relMSE")
    return out


def _batch_views(scene, n, rng):
    a = scene.arrays()
    eye0, tgt0 = np.array(a["camEye"]), np.array(a["camTarget"])
    span = np.linalg.norm(tgt0 - eye0)
    views = []
    for _ in range(n):
        side = 128.0 * 8.0 ** rng.uniform()                 # log-uniform 128 .. 1024
        aspect = rng.uniform(0.6, 1.8)
        w = int(max(16, round(side * np.sqrt(aspect))))
        h = int(max(16, round(side / np.sqrt(aspect))))
        eye = eye0 + rng.normal(scale=0.15 * span, size=3)
        tgt = tgt0 + rng.normal(scale=0.1 * span, size=3)
        views.append((list(eye), list(tgt), [0.0, 1.0, 0.0], float(a["camFovYDeg"]), w, h, int(rng.integers(16, 257))))
    return views


def run_batch(stream, peak):
    """Batched multi-view workload: the 96 views of both scenes in one
    multi-scene batch (every pass one graph launch over both scenes; each
    scene's renderer autotuned), aggregate throughput, per-view relMSE of
    every view against a plain FP64-accumulated render of that view at
    reference_spp_factor x its spp, and the HBM fraction of the whole batch
    (algorithmic bytes of all kernels / time)."""
    import torch

    import optix_pt_gb300 as opt
    rng = np.random.default_rng(BATCH["seed"])
    k_ref = BATCH["reference_spp_factor"]
    names = ("terrain", "spheres")
    scenes, rends, bests, views = [], [], [], []
    for k, name in enumerate(names):
        scene = opt.Scene.procedural(name)
        best, trials = opt.autotune(scene, 320, 180, 16, guiding=1)   # timed as it renders: guided
        builder = "ploc" if best["bvhBuilder"] == 1 else "lbvh"
        r = opt.Renderer(scene, leaf_size=best["leafSize"], block_size=best["blockSize"],
                         compaction=best["compaction"], bvh_builder=builder)
        r.set_max_depth(12)
        r.set_guiding(1)
        scenes.append(scene)
        rends.append(r)
        bests.append(best)
        views += [(k, v) for v in _batch_views(scene, BATCH["views_per_scene"], rng)]
    # warm-up with the same pixel layout at 1 spp: graph capture, network allocation
    opt.render_batch_scenes(rends, [(k, v[:6] + (1,)) for k, v in views], stream)
    torch.cuda.synchronize()
    st0 = [r.stats() for r in rends]
    t0 = time.perf_counter()
    where = opt.render_batch_scenes(rends, views, stream)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    st1 = [r.stats() for r in rends]
    per_scene, rays_all, samples_all, bytes_all = [], 0, 0, 0.0
    rel_all, plain_all = [], []
    for k, name in enumerate(names):
        r, scene, best = rends[k], scenes[k], bests[k]
        mine = [v for kk, v in views if kk == k]
        rays = (st1[k]["extensionRays"] - st0[k]["extensionRays"]) + (st1[k]["shadowRays"] - st0[k]["shadowRays"])
        ext = st1[k]["extensionRays"] - st0[k]["extensionRays"]
        samples = st1[k]["pathSamples"] - st0[k]["pathSamples"]
        # One plain renderer per scene draws the references and, first, a
        # counting pass over the scene's first view for its BVH work per ray.
        ref = opt.Renderer(scene, leaf_size=best["leafSize"], bvh_builder=builder)
        ref.set_max_depth(12)
        eye, tgt, up, fov, w0, h0, _ = mine[0]
        ref.setupOutputBuffer(w0, h0)
        ref.setupCamera(eye, tgt, up, fov)
        cnt = ref.traversal_counts(1, stream)
        bpe = RAY_IO_BYTES + (cnt["extensionNodes"] * 80 + cnt["extensionTris"] * TRI_BYTES) / max(
            1, cnt["extensionRays"])
        bps = RAY_IO_BYTES + 4 + (cnt["shadowNodes"] * 80 + cnt["shadowTris"] * TRI_BYTES) / max(1, cnt["shadowRays"])
        alg = ext * (bpe + SHADE_BYTES) + (rays - ext) * bps + samples * (ACCUM_BYTES + GEN_BYTES)
        rel, rel_plain = {}, {}
        for j, (eye, tgt, up, fov, w, h, spp) in enumerate(mine):
            s, _, n = r.batch_view(j)
            ref.setupOutputBuffer(w, h)
            ref.setupCamera(eye, tgt, up, fov)
            # a plain single-view render at the view's own spp, for scale
            ref.set_seed(104729 + j)
            ref.render(spp, stream)
            torch.cuda.synchronize()
            ps, _, pn = ref.accum()
            ref.resetSampleCount()
            ref.set_seed(7919 + j)
            ref.render(k_ref * spp, stream)
            torch.cuda.synchronize()
            rs, _, rn = ref.accum()
            R = rs.reshape(-1, 3) / rn
            den = R ** 2 + 1e-2
            key = "view%d_%dx%d_%dspp" % (j, w, h, spp)
            rel[key] = float(np.mean(((s / n - R) ** 2 / den).sum(1)))
            rel_plain[key] = float(np.mean(((ps.reshape(-1, 3) / pn - R) ** 2 / den).sum(1)))
        ref.close()
        rel_all += list(rel.values())
        plain_all += list(rel_plain.values())
        per_scene.append({"scene": name, "views": len(mine), "pixels": int(sum(v[4] * v[5] for v in mine)),
                          "samples": int(samples), "rays": int(rays), "autotuned": best,
                          "algorithmic_bytes": alg, "relmse_per_view": rel,
                          "relmse_per_view_plain_single_view": rel_plain, "guide_status": r.guide().status()})
        rays_all += rays
        samples_all += samples
        bytes_all += alg
        r.close()
    ach = bytes_all / dt / 1e9
    return {"config": dict(BATCH), "seconds": dt, "mrays_per_s": rays_all / dt / 1e6,
            "msamples_per_s": samples_all / dt / 1e6, "launch": "one multi-scene batch "
            "(optpt_render_batch_scenes): every pass one CUDA graph launch whose child graphs are both scenes' "
            "passes, run side by side",
            "relmse_per_view_summary": {"views": len(rel_all), "median": float(np.median(rel_all)),
                                        "max": float(np.max(rel_all)), "mean": float(np.mean(rel_all)),
                                        "plain_single_view_median": float(np.median(plain_all)),
                                        "plain_single_view_mean": float(np.mean(plain_all)),
                                        "views_better_than_plain": int(sum(a < b for a, b in zip(rel_all,
                                                                                                 plain_all)))},
            "relmse_reference": "plain render of each view at %dx its spp, FP64 accumulation, independent "
                                "seed (its own noise adds about 1/%d to the measured relMSE); for scale, a "
                                "plain single-view render at the view's own spp against the same reference; "
                                "the sweep's mirror-like spheres and the terrain's glass make the per-view "
                                "relMSE heavy-tailed (caustic fireflies) at these spp" % (k_ref, k_ref),
            "hbm": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "model": "whole batch: extension rays x (ray I/O + BVH nodes + triangles + shade 256 B) + "
                             "shadow rays x (ray I/O + BVH) + samples x (accumulate 64 B + generate 64 B), BVH work "
                             "per ray from a counting pass over each scene's first view"},
            "per_scene": per_scene}


def image_output_measure(r, peak, reps=20):
    """The fused frame-output kernel (RGBA8 + RGBE + HALF payloads in one
    pass) on this frame: CUDA-event time per launch with L2 flushed before
    each, against 48 algorithmic bytes per pixel (two float4 reads, 16 B of
    payload writes); plus wall time of each file dump through the public API
    (GPU payload, copy, host encoding, write)."""
    lp = r.launch_params()
    n = lp.w * lp.h
    ms = r.image_out_profile(reps)  # events recorded by the library around each launch
    achieved = 48.0 * n / (ms / 1e3) / 1e9
    dumps = {}
    with tempfile.TemporaryDirectory() as d:
        for name, fn in (("png", r.dumpFramebuffer), ("hdr", r.dumpAccumFramebufferRgbe),
                         ("exr_zip", r.dumpAccumFramebufferExr)):
            path = os.path.join(d, "out." + name)
            fn(path)  # warm
            t0 = time.perf_counter()
            fn(path)
            dumps[name] = {"ms": (time.perf_counter() - t0) * 1e3, "bytes": os.path.getsize(path)}
    return {"kernel": "kImageOut", "pixels": n, "bytes_per_pixel": 48, "ms_per_launch": ms,
            "achieved_gbs": achieved, "peak_gbs": peak, "frac": achieved / peak,
            "l2": "flushed before each launch", "dump_wall": dumps}


def run_ours(args, rank, world, local_rank):
    import torch

    import optix_pt_gb300 as opt
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    name = args.workload
    head, r, scene, clocks = measure_frames(name, args, rank, world, dev, stream, with_cpu=True)
    if rank != 0:
        r.close()
        return
    peak, _ = _peaks()
    extra = {}
    if world == 1:
        extra["image_output"] = image_output_measure(r, peak)
        # Animation: BVH8 refit of this scene (the reference's per-frame
        # buildAccel(false)), kernel time, against a rebuild measured on the
        # host clock around the whole LBVH build + collapse.
        refit_ms = r.refit_profile(20)
        t0 = time.perf_counter()
        r2 = opt.Renderer(scene)
        rebuild_s = time.perf_counter() - t0
        r2.close()
        extra["animation"] = {"refit_ms": refit_ms, "triangles": scene.num_triangles,
                              "renderer_create_with_bvh_build_ms": rebuild_s * 1e3,
                              "refit_mtris_per_s": scene.num_triangles / (refit_ms / 1e3) / 1e6}
    r.close()
    del r, scene
    workloads = {}
    if world == 1 and not args.quick and name == "sweep":
        # the other configurations, each measured its own way (module docstring)
        workloads["cornell"] = measure_cornell(stream, with_cpu=not args.no_cpu)
        t, tr, _, tclk = measure_frames("terrain", args, rank, world, dev, stream, with_cpu=True)
        tr.close()
        workloads["terrain"] = dict(t, config=dict(WORKLOADS["terrain"]), clocks=tclk)
        if not args.no_guided:
            workloads["guided"] = guided_equal_time(stream, args.guided_budget, args.guided_ref_spp)
        if not args.no_batch:
            workloads["batch"] = run_batch(stream, peak)
    line = {"metric": METRIC, "value": head["value"], "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene, no glTF assets)",
            "config": _config(world), "parallelism": "replicas" if world > 1 else "single GPU",
            "samples_per_s": head["samples_per_s"], "rays_per_step": head["rays_per_step"],
            "e2e": head["e2e"], "gpu_launches": head["gpu_launches"],
            "roofline": head["roofline"], "cpu_baseline": head["cpu_baseline"], "clocks": clocks,
            "traversal_faults": head["traversal_faults"]}
    line.update(extra)
    if workloads:
        line["workloads"] = workloads
        if "guided" in workloads:   # the headline's second half, also at the top level
            line["guided_vs_plain_equal_time"] = workloads["guided"]
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sweep", choices=sorted(WORKLOADS) + ["batch"])
    ap.add_argument("--quick", action="store_true", help="the headline workload only")
    ap.add_argument("--cpu-spp", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-guided", action="store_true", help="skip the guided-vs-plain equal-time comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched multi-view workload")
    ap.add_argument("--guided-only", action="store_true", help="run only the guided-vs-plain comparison")
    ap.add_argument("--guided-budget", type=float, default=0.0, help="seconds per render (default 10)")
    ap.add_argument("--guided-ref-spp", type=int, default=0, help="reference spp (default 65536)")
    ap.add_argument("--bvh-width", type=int, default=8, choices=[2, 8])
    ap.add_argument("--leaf-size", type=int, default=0)
    ap.add_argument("--block-size", type=int, default=0)
    ap.add_argument("--tail-bounce", type=int, default=0,
                    help="first bounce finished by the path-completion kernel (0 = library default, -1 = none)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload in WORKLOADS:
        WORKLOAD.clear()
        WORKLOAD.update(WORKLOADS[args.workload])
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)   # builds in a child process; loads only the oracle
        return
    import __graft_entry__
    __graft_entry__.build()
    import torch
    if args.workload == "batch":
        torch.cuda.set_device(local_rank)
        print(json.dumps(run_batch(torch.cuda.Stream(), _peaks()[0])))
        return
    if args.guided_only:
        torch.cuda.set_device(local_rank)
        print(json.dumps({"guided_vs_plain_equal_time": guided_equal_time(
            torch.cuda.Stream(), args.guided_budget, args.guided_ref_spp)}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
