"""Benchmark: wavefront path samples/s on the 1,024,000-triangle icosphere
field (1920x1080, 64 spp, depth 12, NEE + MIS, Lambert / GGX conductor /
GGX dielectric, 8 quad lights) on one GB300, next to the FP32 megakernel
on the same GPU and the oracle CPU path on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one full 64-spp render of the frame (132.7 M path samples)
through the C ABI, scene resident in HBM.  Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "path samples/s at equal relMSE (wavefront vs megakernel, 1 GB300)"
UNIT = "samples/s"
WORKLOAD = "icosphere-field-1M-tris-1920x1080-64spp-depth12"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--quick", action="store_true", help="small frame for a fast check (not a bench number)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--bvh", default="auto", choices=["auto", "host", "gpu", "gpu-sah"],
                    help="BVH builder of the uploads: host SAH, GPU PLOC (gpu), GPU SAH; auto picks by size")
    ap.add_argument("--profile-spp", type=int, default=8, help="samples per pixel per --profile-case render")
    ap.add_argument("--tuning", default=None,
                    help="--profile-case: this cgpu_tuning (JSON, as the bench line prints it) instead of autotuning")
    ap.add_argument("--profile-case", action="store_true",
                    help="for ncu: the frame with the bench tuning, --steps renders of --profile-spp in a profiler range")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2: the headline line (default); c1 Cornell box, c3 64 batched scenes, "
                         "c4 differentiable scene forward, c5 20.48 M-triangle stress frame: one JSON line each")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene(args):
    from cadise_gb300 import scenes
    if args.quick:
        return scenes.icosphere_field(n_spheres=40, subdivision=3, width=640, height=360, spp=args.spp)
    return scenes.icosphere_field(spp=args.spp)


def frame_config(args, spec):
    """The workload keys of the JSON line, the same in both arms."""
    return {"workload": WORKLOAD if not args.quick else "quick-640x360", "width": spec.width,
            "height": spec.height, "spp": spec.spp, "max_depth": spec.max_depth,
            "triangles": spec.num_triangles(), "l2": "256 MB buffer written between steps"}


def traversal_profile():
    """Counters of the closest-hit pass from the committed small-case ncu
    captures (profiles/traversal_counters.json): L2 hit rate and throughput,
    lanes per warp instruction, per configuration."""
    try:
        with open(os.path.join(ROOT, "profiles", "traversal_counters.json")) as f:
            return json.load(f)
    except Exception:
        return None


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region (read only)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # wait (up to 3 s) until the sampler is live, so a short timed region still gets samples
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0:
            self.file.flush()
            if os.path.getsize(self.file.name) > 0:
                break
            time.sleep(0.02)

    def sample_once(self):
        """One more sample at the end of a timed region shorter than the sampling period."""
        try:
            out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                  "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
            with open(self.file.name, "a") as f:
                f.write(out.stdout)
        except Exception:
            pass

    def stop(self):
        if not self.proc:
            return None
        self.sample_once()
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------- CPU oracle --
def cpu_rate(flat, seconds: float = 12.0, threads: int = 0):
    """The oracle's CPU path tracer (a restatement of the reference's, run on
    all host cores) on a bounded sample of the same frame: whole rows at
    1 spp from the middle of the image until ~`seconds` of CPU work."""
    import oracle
    threads = threads or os.cpu_count() or 1
    ps = oracle.PortScene(flat)
    h, w = flat.desc.height, flat.desc.width
    mid = h // 2
    t0 = time.perf_counter()
    ps.render(seed=1, first=0, count=1, rows=(mid, mid + 1), threads=threads)
    one = max(time.perf_counter() - t0, 1e-3)
    rows = int(max(1, min(h - mid, seconds / one)))
    t0 = time.perf_counter()
    ps.render(seed=1, first=0, count=1, rows=(mid - rows // 2, mid - rows // 2 + rows), threads=threads)
    dt = time.perf_counter() - t0
    samples = rows * w
    return samples / dt, threads, "%d rows x %d px x 1 spp (%d path samples) of the same frame" % (rows, w, samples)


# ---------------------------------------------------------------- GPU arm --
def run_gpu(args, rank, world, local):
    import numpy as np
    import torch

    import cadise_gb300 as cg
    from cadise_gb300 import abi

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    ctx = cg.Context(device=local, stream=stream.cuda_stream)
    ctx.set_bvh_builder(BVH_BUILDERS[args.bvh])
    spec = make_scene(args)
    flat = abi.flatten(spec)
    sid = ctx.upload(flat)
    info = ctx.info(sid)
    npix = spec.width * spec.height
    spp = spec.spp
    # weak scaling: every rank renders its own disjoint sample range of the frame
    first = rank * spp
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def render(mode, graph=True):
        ctx.render([sid], first, spp, seed=2024, mode=mode, graph=graph, sync=False)

    tuning = ctx.tuning()
    if not args.no_autotune:
        cache = os.path.join(tempfile.gettempdir(), "cadise_gb300_tune.jsonl")
        tuning = ctx.autotune([sid], samples=8, cache_path=cache)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1)
            render(cg.CGPU_MODE_WAVEFRONT)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        clocks = ClockSampler(local)
        clocks.start()
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        launches = 0
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(1)
            starts[i].record(stream)
            render(cg.CGPU_MODE_WAVEFRONT)
            ends[i].record(stream)
            launches += ctx.stats().kernel_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        if world > 1:
            torch.distributed.barrier()
        clk = clocks.stop()
        step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        total_ms = sum(step_ms)
        if world > 1:
            t = torch.tensor([total_ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total_ms = float(t.item())
        samples_all = float(npix) * spp * args.steps * world
        value = samples_all / (total_ms / 1e3)

        # megakernel on the same frame and samples (equal estimator => equal relMSE)
        mk_steps = max(1, min(2, args.steps))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(1)
        e0.record(stream)
        for _ in range(mk_steps):
            render(cg.CGPU_MODE_MEGAKERNEL)
        e1.record(stream)
        torch.cuda.synchronize()
        mk_value = float(npix) * spp * mk_steps / (e0.elapsed_time(e1) / 1e3)

        # counting replay (same seeds, counters on) and per-kernel event timing
        ctx.set_counting(True)
        ctx.render([sid], first, 1, seed=2024, mode=cg.CGPU_MODE_WAVEFRONT, graph=False, sync=True)
        st = ctx.stats()
        ctx.set_counting(False)
        ctx.set_profiling(True)
        ctx.render([sid], first, 1, seed=2024, mode=cg.CGPU_MODE_WAVEFRONT, graph=False, sync=True)
        kt = ctx.kernel_times()
        ctx.set_profiling(False)

        # end to end through the public API: render + film read-back into pinned host memory
        film = torch.empty(npix * 7, dtype=torch.float64, pin_memory=True)
        fs = film.numpy()
        e2e_t = []
        h2d = 0
        for i in range(max(1, min(3, args.steps))):
            t0 = time.perf_counter()
            ctx.film_clear(sid)
            ctx.render([sid], first, spp, seed=2024 + i, mode=cg.CGPU_MODE_WAVEFRONT, sync=False)
            h2d = ctx.stats().h2d_bytes
            ctx.film_read_into(sid, fs[:3 * npix], fs[3 * npix:6 * npix], fs[6 * npix:])
            e2e_t.append(time.perf_counter() - t0)
        e2e_value = float(npix) * spp * world / statistics.mean(e2e_t)

    # roofline of the dominant kernel (closest-hit traversal), algorithmic bytes:
    # 64 B per quantized 4-wide node + 48 B per triangle record + 64 B ray/hit queue I/O
    ext_bytes = 64.0 * st.node_visits + 48.0 * st.triangle_tests + 64.0 * st.closest_rays
    ext_ms, ext_launches = kt["extend"]
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = ext_bytes / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else None
    rays_per_sample = (st.closest_rays + st.any_rays) / float(npix)
    prof = traversal_profile()
    traffic = None
    if prof and "c2" in prof:
        # the DRAM bytes per closest-hit ray of the small-case capture, scaled to one launch of this frame
        traffic = prof["c2"]["dram_bytes_per_closest_ray"] * st.closest_rays / max(1, ext_launches)

    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_rate(ctx, args)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, cores, sample = cpu_rate(flat)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(args, spec),
        "gpu_setup": {"bvh_nodes": info.num_bvh_nodes,
                      "bvh": {"builder": {1: "host-sah", 2: "gpu-ploc", 3: "gpu-sah"}[info.bvh_builder],
                              "build_ms": info.bvh_ms},
                      "schedule": "wavefront, CUDA graph per batch",
                      "parallelism": "replicas" if world > 1 else "single", "tuning": tuning},
        "megakernel": {"value": mk_value, "unit": UNIT, "speedup_wavefront": value / world / mk_value,
                       "rays": "the wavefront's: zero-contribution shadow rays skipped, MIS rays resolved "
                               "against their light at the vertex with a bounded any-hit query"},
        "rays": {"closest_per_sample": st.closest_rays / float(npix), "any_per_sample": st.any_rays / float(npix),
                 "mrays_per_s": value * rays_per_sample / 1e6,
                 "nodes_per_closest_ray": st.node_visits / max(1, st.closest_rays),
                 "triangles_per_closest_ray": st.triangle_tests / max(1, st.closest_rays),
                 "nodes_per_any_ray": st.any_node_visits / max(1, st.any_rays),
                 "triangles_per_any_ray": st.any_triangle_tests / max(1, st.any_rays),
                 "tie_rule_fraction_of_closest": st.tie_rays / max(1, st.closest_rays)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": "k_wf_extend_pww (closest-hit traversal)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                     "limiter": "not HBM: the BVH and triangles sit in the 129 MB L2; issue slots and "
                                "L1/L2 latency under divergence (lanes per warp instruction below)",
                     "counters": prof.get("c2") if prof else None},
        "kernel_ms_per_pass": {k: v[0] for k, v in kt.items()},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": npix * 7 * 8,
                "path": "cgpu_film_clear + cgpu_render + cgpu_film_read into pinned host buffers"},
        "adjoint": adjoint,
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cpu,
        "wall_s_timed": wall,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def adjoint_rate(ctx, args):
    """Differentiable-rendering iteration on the 102,400-triangle scene:
    512x512, 32 spp forward pass + path-replay adjoint of the L2 loss against
    a target rendered from perturbed parameters."""
    import numpy as np
    import torch

    from cadise_gb300 import scenes
    if args.quick:
        spec = scenes.diff_scene(width=128, height=128, spp=8, n_spheres=8, subdivision=3)
    else:
        spec = scenes.diff_scene()
    sid = ctx.upload(spec)
    tex, rough, rad = ctx.get_params(sid)
    rng = np.random.default_rng(0)
    # target from perturbed parameters (albedo +-0.2, roughness +-0.15)
    ctx.set_params(sid, texels=np.clip(tex + rng.uniform(-0.2, 0.2, tex.shape), 0.02, 0.98).astype(np.float32),
                   roughness=np.clip(rough + rng.uniform(-0.15, 0.15, rough.shape), 0.05, 1.0).astype(np.float32))
    target = ctx.adjoint_forward(sid, 256 if args.quick else 1024, 77)
    ctx.set_params(sid, texels=tex, roughness=rough)
    npix = spec.width * spec.height
    times_f, times_b = [], []
    for it in range(3):
        t0 = time.perf_counter()
        img = ctx.adjoint_forward(sid, spec.spp, 1000 + it)
        t1 = time.perf_counter()
        grad_img = (2.0 * (img - target) / img.size).astype(np.float32)
        gt, gr, gl = ctx.adjoint_backward(sid, spec.spp, 1000 + it, grad_img)
        t2 = time.perf_counter()
        if it > 0:
            times_f.append(t1 - t0)
            times_b.append(t2 - t1)
    nparams = gt.size + gr.size + gl.size
    # the same backward on the one-thread-per-path schedule, for comparison
    from cadise_gb300 import CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT
    ctx.set_adjoint_mode(CGPU_MODE_MEGAKERNEL)
    ctx.adjoint_backward(sid, spec.spp, 1000, grad_img)
    t0 = time.perf_counter()
    ctx.adjoint_backward(sid, spec.spp, 1000, grad_img)
    bwd_mk = time.perf_counter() - t0
    ctx.set_adjoint_mode(CGPU_MODE_WAVEFRONT)
    ctx.release(sid)
    fwd, bwd = statistics.mean(times_f), statistics.mean(times_b)
    return {"workload": "diff-scene-102k-tris-%dx%d-%dspp" % (spec.width, spec.height, spec.spp),
            "iterations_per_s": 1.0 / (fwd + bwd), "grads_per_s": nparams / (fwd + bwd),
            "unit": "gradient evaluations/s (forward + adjoint)", "parameters": int(nparams),
            "forward_ms": fwd * 1e3, "backward_ms": bwd * 1e3, "backward_ms_megakernel_schedule": bwd_mk * 1e3,
            "backward_path_samples_per_s": npix * spec.spp / bwd}


# ---------------------------------------------------------- reference arm --
def run_reference(args, rank, world, local):
    """The reference's CPU path (its algorithm restated by the oracle, run
    with every host thread) on bounded samples of the same frame."""
    if rank != 0:
        return
    from cadise_gb300 import abi
    import oracle
    spec = make_scene(args)
    flat = abi.flatten(spec)
    threads = os.cpu_count() or 1
    ps = oracle.PortScene(flat)
    w, h = spec.width, spec.height
    # whole rows are the unit of the port's thread pool: a step of 3 rows per
    # thread keeps every host thread busy (~0.1 s of work per step)
    rows = min(h, 3 * threads)
    mid = h // 2
    for i in range(args.warmup):
        ps.render(seed=i, first=0, count=1, rows=(mid, mid + 1), threads=threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        r0 = (mid + i * rows) % max(1, h - rows)
        ps.render(seed=100 + i, first=i, count=1, rows=(r0, r0 + rows), threads=threads)
    dt = time.perf_counter() - t0
    samples = rows * w * args.steps
    value = samples / dt
    sample = "%d steps x %d rows x %d px x 1 spp of the frame" % (args.steps, rows, w)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(args, spec),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------ other configurations --
CONFIGS = {
    "c1": "cornell-box-256x256-16spp-depth6",
    "c3": "64-batched-icosphere-fields-10k-2M-tris-128..1024px-4..256spp-depth4..16",
    "c4": "diff-scene-102k-tris-512x512-32spp-depth6-forward",
    "c5": "env-field-20.48M-tris-3840x2160-depth32-64-lights-hdr-sky-64-ggx-palette (4 spp per step of the 1024)",
}


BVH_BUILDERS = {"auto": 0, "host": 1, "gpu": 2, "gpu-sah": 3}


def run_config(args):
    """The other configurations, one JSON line each: wavefront and
    megakernel path samples/s on the GPU, the oracle's CPU rate on a bounded
    slice, and the set-up times (scene generation, upload with BVH build)."""
    import torch

    import cadise_gb300 as cg
    from cadise_gb300 import abi, scenes

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    ctx = cg.Context(device=0, stream=stream.cuda_stream)
    ctx.set_bvh_builder(BVH_BUILDERS[args.bvh])
    t0 = time.perf_counter()
    if args.config == "c1":
        specs = [scenes.cornell_box()]
    elif args.config == "c3":
        specs = scenes.batch_scenes()
    elif args.config == "c4":
        specs = [scenes.diff_scene()]
    else:
        specs = [scenes.env_field()]
    gen_s = time.perf_counter() - t0
    flats = [abi.flatten(s) for s in specs]
    t0 = time.perf_counter()
    sids = [ctx.upload(f) for f in flats]
    upload_s = time.perf_counter() - t0
    infos = [ctx.info(s) for s in sids]
    npix = [s.width * s.height for s in specs]
    # samples per step: the whole job (c1, c3, c4) or 4 of the 1024 spp (c5)
    counts = [4 if args.config == "c5" else s.spp for s in specs]
    mk_counts = [max(1, c // 8) for c in counts] if args.config in ("c3", "c5") else counts
    steps, warmup = (1, 1) if args.config == "c3" else (args.steps, args.warmup)
    tuning = ctx.autotune(sids, samples=1 if args.config in ("c3", "c5") else 8)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(mode, cnt, k):
        ms = 0.0
        with torch.cuda.stream(stream):
            for i in range(k):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                ctx.render(sids, 0, cnt, seed=11 + i, mode=mode, sync=False)
                e1.record(stream)
                torch.cuda.synchronize()
                ms += e0.elapsed_time(e1)
        return sum(n * c for n, c in zip(npix, cnt)) * k / (ms / 1e3), ms / k

    timed(cg.CGPU_MODE_WAVEFRONT, counts, warmup)
    clocks = ClockSampler(0)
    clocks.start()
    wf, wf_ms = timed(cg.CGPU_MODE_WAVEFRONT, counts, steps)
    clk = clocks.stop()
    timed(cg.CGPU_MODE_MEGAKERNEL, mk_counts, 1)
    mk, _ = timed(cg.CGPU_MODE_MEGAKERNEL, mk_counts, 1)
    # CPU: the oracle on a bounded slice of (a spread of) the scenes
    cpu = None
    if not args.no_cpu_baseline:
        order = sorted(range(len(specs)), key=lambda i: infos[i].num_triangles)
        pick = order if len(order) <= 1 else [order[int(round(j * (len(order) - 1) / 7))] for j in range(8)]
        rates = []
        for i in sorted(set(pick)):
            rate, cores, _ = cpu_rate(flats[i], seconds=12.0 / len(set(pick)))
            rates.append(rate)
        cpu = {"value": statistics.mean(rates), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d scene(s), 1-spp row slices of ~%.1f s each" % (len(rates), 12.0 / len(rates))}
    out = {
        "metric": METRIC, "value": wf, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": wf_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": CONFIGS[args.config], "scenes": len(specs),
                   "triangles": int(sum(i.num_triangles for i in infos)),
                   "samples_per_step": int(sum(n * c for n, c in zip(npix, counts))), "tuning": tuning,
                   "l2": "256 MB buffer written between steps"},
        "megakernel": {"value": mk, "unit": UNIT, "speedup_wavefront": wf / mk,
                       "samples_per_step": int(sum(n * c for n, c in zip(npix, mk_counts)))},
        "setup_s": {"scene_generation": gen_s, "upload_with_bvh_build": upload_s,
                    "bvh_build": sum(i.bvh_ms for i in infos) / 1e3,
                    "bvh_builders": sorted({{1: "host-sah", 2: "gpu-ploc", 3: "gpu-sah"}[i.bvh_builder] for i in infos})},
        "clocks": clk,
        "cpu_baseline": cpu,
        "counters": (traversal_profile() or {}).get(args.config),
    }
    if args.config == "c5" and not args.no_adjoint:
        out["adjoint"] = stress_adjoint_rate(ctx, sids[0], specs[0])
    print(json.dumps(out), flush=True)
    ctx.close()


def stress_adjoint_rate(ctx, sid, spec, spp=4, iters=2):
    """The stress configuration's differentiation: per iteration a forward
    pass of `spp` of the 1024 samples per pixel of the 3840 x 2160 frame and
    the path-replay adjoint of a fixed random d loss / d image over the same
    paths, with FP64 reductions; the parameters asked for are the 64 GGX
    palette roughnesses and the 64 quad lights' radiances (the adjoint also
    returns the roughness entries of the Lambert materials, which are zero)."""
    import numpy as np
    import torch

    from cadise_gb300 import scenes
    ggx = [i for i, m in enumerate(spec.materials) if m.type in (scenes.CONDUCTOR, scenes.ROUGH_DIELECTRIC)]
    W = np.random.default_rng(5).normal(size=(spec.height, spec.width, 3)).astype(np.float32)
    fwd, bwd = [], []
    for it in range(iters + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.adjoint_forward(sid, spp, 700 + it)
        t1 = time.perf_counter()
        gt, gr, gl = ctx.adjoint_backward(sid, spp, 700 + it, W)
        t2 = time.perf_counter()
        if it > 0:  # the first iteration allocates the adjoint buffers
            fwd.append(t1 - t0)
            bwd.append(t2 - t1)
    nparams = len(ggx) + gl.size
    f, b = statistics.mean(fwd), statistics.mean(bwd)
    return {"workload": "env-field-20.48M-tris-3840x2160-depth32, %d spp forward + adjoint per iteration" % spp,
            "parameters": int(nparams), "roughness_parameters": len(ggx), "radiance_parameters": int(gl.size),
            "iterations_per_s": 1.0 / (f + b), "grads_per_s": nparams / (f + b),
            "unit": "gradient evaluations/s (forward + adjoint)", "forward_ms": f * 1e3, "backward_ms": b * 1e3,
            "backward_path_samples_per_s": spec.width * spec.height * spp / b,
            "nonzero_roughness_gradients": int(np.count_nonzero(gr[ggx])),
            "finite": bool(np.all(np.isfinite(gr)) and np.all(np.isfinite(gl)))}


def run_profile_case(args):
    """The bench frame's wavefront passes for ncu, with the tuning the bench
    uses (autotuned the same way first) and direct launches instead of the
    graph; the profiled range (cudaProfilerStart / Stop, for ncu
    --profile-from-start off) holds only the `--steps` renders of
    `--profile-spp` samples per pixel.  --config c1 / c4: the Cornell box or
    the differentiable scene instead of the bench frame."""
    import torch

    import cadise_gb300 as cg
    from cadise_gb300 import abi, scenes
    torch.cuda.set_device(0)
    ctx = cg.Context()
    ctx.set_bvh_builder(BVH_BUILDERS[args.bvh])
    spec = {"c1": scenes.cornell_box, "c4": scenes.diff_scene}.get(args.config, lambda: make_scene(args))()
    sid = ctx.upload(abi.flatten(spec))
    if args.tuning:
        t = json.loads(args.tuning)
        ctx.set_tuning_dict(t)
        tuning = ctx.tuning()
    else:
        tuning = ctx.tuning() if args.no_autotune else ctx.autotune([sid], samples=8)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for i in range(args.steps):
        ctx.render([sid], i * args.profile_spp, args.profile_spp, seed=2024, mode=cg.CGPU_MODE_WAVEFRONT, graph=False)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_case": args.config if args.config != "c2" else WORKLOAD if not args.quick else "quick",
                      "renders": args.steps,
                      "spp_per_render": args.profile_spp, "tuning": tuning,
                      "kernel_launches_last_render": ctx.stats().kernel_launches}))
    ctx.close()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.config != "c2":
        if rank == 0:
            run_config(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
