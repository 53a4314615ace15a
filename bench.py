"""Benchmark: Mpath-samples/s of the GPU MIS volumetric path tracer on the 1080p many-light terrain.

Workload (one step = one frame): 1920x1080, 64 spp, max depth 6, 2,093,058-triangle heightfield with
10,000 emissive triangles sampled through the light tree and a sky environment light; seeded
synthetic scene (no external assets exist).  Scene data (~250 MB) is larger than the 129 MB L2 and L2
is additionally flushed between timed steps.

  value   device-resident throughput: K frames launched back to back on one stream, CUDA events
  e2e     the same metric through lgpu_render with a host film (H2D + D2H film copies inside)
  roofline  for the kernel with the largest share of the frame: its algorithmic bytes (resume: path
          state in and out per resumed path; trace: BVH node and triangle records fetched, counted
          in-kernel by a separate counting render of the same frame, plus ray and hit records) over
          its own time, taken from CUDA events the library records around every launch on the render
          stream; all kernels are listed under roofline.kernels
  cpu_baseline  the reference renderer's own CPU integrator and tile renderer (built from its sources
          with Embree replaced, oracle/build_ref.py) on this host's cores over a bounded sample of
          tiles of the same frame -- or the CPU oracle where the reference cannot be built -- plus
          the per-path agreement of the GPU with it on 20,000 seeded paths of the frame (parity)

--impl reference runs that CPU path alone with all host threads on the same config and metric.
Multi-GPU (torchrun, N > 1): replicas -- every rank renders its own frame (seed = rank); no
collective on the data path; value = all ranks' paths / max time.
"""
import argparse
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpath-samples/s at 1080p, equal relMSE: batched vs plain GPU vs CPU; bwd/fwd ratio"
UNIT = "Mpath-samples/s"
WORKLOAD = dict(workload="many-light terrain (2.1M tris, 10k emitters, sky env), MIS volumetric path tracing",
                width=1920, height=1080, spp=64, max_depth=6, triangles=2093058 + 10000, emitters=10000,
                spectral="RGB3", light_sampler="light tree")
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per unit of work (resumed path, traced
# ray) of the wavefront kernels, from one ncu capture of a 480x270x16 frame of the same scene,
# multiplied by the units of an average launch of the timed run.
NCU_DRAM_BYTES_PER_UNIT = {"k_wave_resume": 858.0, "k_wave_trace": 79.5}
# Algorithmic bytes per unit: a resumed path reads and writes its path state (96 B each way: ray,
# throughput, radiance, pdfs, medium, depth, ids); a traced ray fetches its BVH nodes and triangle
# records (counted in-kernel) plus 32 B of ray and 20 B of hit record.
STATE_BYTES_PER_RESUME = 192
RAY_IO_BYTES = 52


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--width", type=int, default=0, help="0 = the workload's own size")
    p.add_argument("--height", type=int, default=0)
    p.add_argument("--spp", type=int, default=0)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the batched, adjoint and relMSE records of the default line")
    p.add_argument("--mode", default="auto", choices=["auto", "megakernel", "wavefront", "graph"])
    p.add_argument("--pool", type=int, default=0, help="wavefront path-slot pool size (0 = default)")
    p.add_argument("--block", type=int, default=0, help="trace-kernel block size (0 = default)")
    p.add_argument("--workload", default="terrain", choices=["terrain", "volume", "cornell", "batched", "inverse"],
                   help="terrain: the 1080p many-light frame (default); volume, cornell: the other two single-frame "
                        "scenes; batched: 64 uneven views of the terrain and "
                        "volume scenes in one batched render against the same views one at a time")
    return p.parse_args()


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        res = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        sm = []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                res["sm_max_mhz"] = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                pass
        if sm:
            res["sm_mhz"] = float(np.median(sm))
        res["reasons"] = sorted(reasons)
        res["samples"] = len(sm)
        return res


def _tile_sample(W, H, n):
    """n of the frame's 16 x 16 tiles (row-major tile index), evenly strided over the frame."""
    total = ((W + 15) // 16) * ((H + 15) // 16)
    n = max(1, min(total, n))
    return (np.arange(n) * (total / n)).astype(np.int64).astype(np.int32), total


def cpu_baseline(sb, cam, opts, seconds, threads=0, gpu=None, parity_paths=20000):
    """CPU throughput on a bounded sample of the same frame (about `seconds` of work) and, when `gpu`
    (a Renderer of the same scene) is given, per-path agreement of the GPU with the CPU path.

    kind "reference": the reference renderer's own code (RenderMosaic + TileRenderers::UniformSpp +
    MISVolumetricPathIntegrator::Li, built from its sources by oracle/build_ref.py, Embree replaced by
    oracle/ref_shim) over an evenly strided sample of 16 x 16 tiles at full spp, on `threads` host
    threads.  kind "port": the CPU oracle (the restatement) over a stratified pixel sample, where the
    reference cannot be built."""
    from oracle import reference
    W, H, spp = opts.width, opts.height, opts.spp
    threads = threads or os.cpu_count()
    ids_par = None
    if gpu is not None:
        rng = np.random.RandomState(99)
        ids_par = np.sort(rng.choice(W * H * spp, min(parity_paths, W * H * spp), replace=False)).astype(np.uint64)
    if reference.available():
        ref = reference.Reference(sb)
        calib, total = _tile_sample(W, H, 2 * threads)
        t0 = time.perf_counter()
        ref.render_tiles(cam, opts, calib, threads=threads)
        rate = len(calib) / max(time.perf_counter() - t0, 1e-6)   # tiles per second
        tiles, total = _tile_sample(W, H, int(max(4, rate * seconds)))
        t0 = time.perf_counter()
        film = ref.render_tiles(cam, opts, tiles, threads=threads)
        dt = time.perf_counter() - t0
        n_paths = float(film[..., 3].sum())
        res = {"value": n_paths / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "reference",
               "sample": "%d of %d 16x16 tiles (every %.1fth, full %d spp) = %d path samples in %.1f s, by the "
                         "reference's TileRenderers::UniformSpp + MISVolumetricPathIntegrator::Li"
                         % (len(tiles), total, total / len(tiles), spp, n_paths, dt)}
        cpu_paths = ref.render_paths(cam, opts, ids_par, threads=threads) if ids_par is not None else None
        ref.close()
    else:
        from oracle.oracle import Oracle
        o = Oracle(sb)

        def ids_for(npix, offset=0):
            step = max(1, (W * H) // npix)
            px = (np.arange(npix, dtype=np.uint64) * step + offset) % (W * H)
            return (px[:, None] * spp + np.arange(spp, dtype=np.uint64)[None, :]).reshape(-1)

        calib = ids_for(max(1, 2048 // spp * 8), 7)
        t0 = time.perf_counter()
        o.render_paths(cam, opts, calib, threads=threads)
        rate = len(calib) / max(time.perf_counter() - t0, 1e-6)
        npix = int(max(16, min(W * H, rate * seconds / spp)))
        ids = ids_for(npix, 13)
        t0 = time.perf_counter()
        o.render_paths(cam, opts, ids, threads=threads)
        dt = time.perf_counter() - t0
        res = {"value": len(ids) / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
               "why_not_reference": reference.unavailable_reason(),
               "sample": "%d of %d pixels (stratified, every %dth) x %d spp = %d path samples in %.1f s"
                         % (npix, W * H, max(1, (W * H) // npix), spp, len(ids), dt)}
        cpu_paths = o.render_paths(cam, opts, ids_par, threads=threads) if ids_par is not None else None
        o.close()
    if ids_par is not None:
        got = gpu.render_paths(cam, opts, ids_par)
        a, b = got[:, :3].astype(np.float64), cpu_paths[:, :3].astype(np.float64)
        err = np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-6)
        ok = np.all((err <= 1e-4) | (np.abs(a - b) <= 1e-6), axis=1)
        same = ok & (got[:, 3] == cpu_paths[:, 3])
        res["parity"] = {"paths": int(len(ids_par)), "agree": float(same.mean()),
                         "criterion": "rgb within 1e-4 relative (1e-6 floor) and equal random numbers drawn",
                         "against": res["kind"], "differing_ids": [int(i) for i in ids_par[~same][:10]]}
    return res


def replica_seed(rank):
    """Replicas: every rank renders its own frame of the same scene with its own seed."""
    return 1 + rank


def max_over_ranks(values, dist, device):
    """Element-wise max over ranks of per-rank timings (the job takes as long as its slowest rank)."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def job_throughput(paths_per_rank, steps, world, ms):
    """Whole-job Mpath-samples/s: the paths all ranks rendered over the slowest rank's time."""
    return paths_per_rank * steps * world / (ms / 1e3) / 1e6


def kernel_table(per_step, stats, paths, kernel_ms, megakernel):
    """Per-kernel time, work units and algorithmic bytes of one frame (mean over timed frames)."""
    trav_bytes = stats["nodes_visited"] * stats["node_bytes"] + stats["tris_tested"] * stats["tri_record_bytes"] \
        + stats["rays"] * RAY_IO_BYTES
    mean = lambda f: float(np.mean([f(s_) for s_ in per_step]))
    k = {}
    if megakernel:
        k["k_render"] = {"ms": float(np.mean(kernel_ms)), "launches": 1.0, "units": float(paths),
                         "alg_bytes": float(trav_bytes + paths * 16)}
    elif mean(lambda s_: s_["trace_ms"]) == 0.0:
        # graph-replayed bounce loop: no per-launch events; the whole frame against its traversal bytes
        k["wavefront_graph"] = {"ms": float(np.mean(kernel_ms)), "launches": mean(lambda s_: s_["launches"]),
                                "units": float(stats["rays"]), "alg_bytes": float(trav_bytes)}
    else:
        iters = mean(lambda s_: s_["iterations"])
        resumed = mean(lambda s_: sum(s_["resumed"]))
        # launches per frame: first spawn 2, per iteration trace 1 + spawn 2 + one resume per
        # non-empty stage, film reduction 1
        k["k_wave_resume"] = {"ms": mean(lambda s_: s_["shade_ms"]),
                              "launches": mean(lambda s_: s_["launches"]) - 3 * iters - 3, "units": resumed,
                              "alg_bytes": resumed * STATE_BYTES_PER_RESUME,
                              "stage_ms": [mean(lambda s_: s_["stage_ms"][j]) for j in range(6)],
                              "stage_paths": [mean(lambda s_: s_["resumed"][j]) for j in range(6)]}
        k["k_wave_trace"] = {"ms": mean(lambda s_: s_["trace_ms"]), "launches": iters,
                             "units": mean(lambda s_: s_["traced"]), "alg_bytes": float(trav_bytes)}
        k["k_wave_spawn"] = {"ms": mean(lambda s_: s_["spawn_ms"]), "launches": iters + 1, "units": float(paths),
                             "alg_bytes": float(paths * (STATE_BYTES_PER_RESUME // 2 + 32))}
    for k_ in k.values():
        k_["achieved_gbs"] = k_["alg_bytes"] / (k_["ms"] / 1e3) / 1e9 if k_["ms"] > 0 else None
    return k


def batched_views(seed=6, n=64):
    """64 seeded views over the terrain (scene 0) and volume (scene 1) scenes: resolution in
    {128, 256, 512, 1024}^2, spp uniform in 1..64, depth uniform in 4..12, cameras orbiting each
    scene's default viewpoint."""
    from lambda_gb300.scene import Camera
    rng = np.random.RandomState(seed)
    out = []
    for i in range(n):
        scene = int(rng.randint(0, 2))
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = int(rng.randint(1, 65))
        depth = int(rng.randint(4, 13))
        if scene == 0:
            o = np.array([-30.0, 22.0, -38.0]) + rng.uniform(-12, 12, 3) * np.array([1, 0.3, 1])
            cam = Camera(tuple(o), (5.0, -2.0, 5.0), fov=1.1)
        else:
            a = rng.uniform(-0.6, 0.6)
            o = (60.0 * np.sin(a), 10.0 + rng.uniform(-4, 4), -60.0 * np.cos(a))
            cam = Camera(o, (0.0, 2.0, 0.0), fov=0.9)
        out.append((scene, cam, res, res, spp, depth, 100 + i))
    return out


# single-frame workloads: builder, default width, height, spp, depth and the config record
SINGLE = {
    "terrain": (lambda w, h, s: configs_mod().terrain(w, h, s, 6), 1920, 1080, 64, WORKLOAD),
    "volume": (lambda w, h, s: configs_mod().volume(w, h, s, 12), 1280, 720, 128,
               dict(workload="volumetric + instancing: homogeneous medium box (sigma_a 0.05, sigma_s 0.5, g 0.3), "
                             "16 point + 4 spot lights, 1000 instances of a 100k-triangle displaced sphere, "
                             "half dielectric, half Oren-Nayar/GGX mix", max_depth=12, triangles=100352,
                    instances=1000, spectral="RGB3", light_sampler="light tree")),
    "cornell": (lambda w, h, s: configs_mod().cornell(w, h, s, 8), 256, 256, 16,
                dict(workload="Cornell box: 5 walls, icosphere (1280 tris, GGX 0.2), 6500 K quad light", max_depth=8,
                     triangles=1292, spectral="RGB3", light_sampler="light tree")),
}


def configs_mod():
    from lambda_gb300 import configs
    return configs


def workload_scene(args):
    build, w0, h0, s0, rec = SINGLE[args.workload]
    w, h, spp = args.width or w0, args.height or h0, args.spp or s0
    sb, cam, opts = build(w, h, spp)
    cfg = dict(rec)
    cfg["width"], cfg["height"], cfg["spp"] = w, h, spp
    return sb, cam, opts, cfg


def batched_record(steps, warmup):
    """Batched uneven workload: every view of each scene in one lgpu_render_batch call (after
    lgpu_autotune on a 1-spp probe) against the same views rendered one at a time."""
    import torch
    import lambda_gb300 as lg
    from lambda_gb300 import abi, configs
    views = batched_views()
    sbs = [configs.terrain(64, 64, 1, 6)[0], configs.volume(64, 64, 1, 12)[0]]
    rs = [lg.Renderer(sb, device=0) for sb in sbs]
    films = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for (_, _, w, h, _, _, _) in views]
    paths = sum(w * h * spp for (_, _, w, h, spp, _, _) in views)
    opts = abi.render_opts(64, 64, 1, 6)
    per_scene = [[(c, w, h, spp, d, seed, f.data_ptr()) for (sc, c, w, h, spp, d, seed), f in zip(views, films) if sc == k]
                 for k in range(2)]
    tuning = [r.autotune(v, opts, probe_spp=1) for r, v in zip(rs, per_scene)]
    opts.kernel_mode = abi.KERNEL_AUTO

    def batched():
        for r, v in zip(rs, per_scene):
            r.render_batch(v, opts)

    def plain():
        o = abi.render_opts(64, 64, 1, 6)
        o.kernel_mode = abi.KERNEL_WAVEFRONT
        for (sc, c, w, h, spp, d, seed), f in zip(views, films):
            o.width, o.height, o.spp, o.max_bounces, o.seed = w, h, spp, d, seed
            rs[sc].render_device(c, o, f.data_ptr())

    def timed(fn):
        for _ in range(max(1, warmup)):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / steps

    for f in films:
        f.zero_()
    clocks = ClockSampler(0)
    clocks.start()
    tb = timed(batched)
    clk = clocks.stop()
    counts_ok = all(bool(torch.all(f[..., 3] == float(spp * (max(1, warmup) + steps))))
                    for f, (_, _, _, _, spp, _, _) in zip(films, views))
    if not counts_ok:
        raise SystemExit("work check failed: a view's film sample counts do not match its spp")
    tp = timed(plain)
    host = [torch.empty_like(f, device="cpu").pin_memory() for f in films]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        batched()
        for h_, f in zip(host, films):
            h_.copy_(f, non_blocking=True)
        torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / steps
    for r in rs:
        r.close()
    return {"value": paths / tb / 1e6, "unit": UNIT, "ms_per_step": tb * 1e3,
            "plain": {"value": paths / tp / 1e6, "ms_per_step": tp * 1e3,
                      "scheme": "the same views one at a time through lgpu_render_device (wavefront)"},
            "batched_over_plain": tp / tb,
            "e2e": {"value": paths / te / 1e6, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(sum(f.numel() * 4 for f in films))},
            "config": {"workload": "batched uneven views: 64 views of the 1080p terrain and the volume/instancing "
                                   "scene, resolution in {128,256,512,1024}^2, spp 1-64, depth 4-12 (seed 6); one "
                                   "lgpu_render_batch call per scene", "views": len(views), "path_samples": paths,
                       "tuning": tuning},
            "clocks": clk}


def main_batched(args):
    import torch
    import lambda_gb300 as lg
    lg.build()
    torch.cuda.set_device(0)
    rec = batched_record(args.steps, args.warmup)
    line = {"metric": METRIC, "value": rec["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes and views)",
            "config": dict(rec["config"], l2="scene data and per-view films exceed L2"),
            "plain": rec["plain"], "batched_over_plain": rec["batched_over_plain"], "e2e": rec["e2e"],
            "clocks": rec["clocks"]}
    print(json.dumps(line))


def _adam(state, key, x, g, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update of parameter x (numpy) with gradient g; state holds the moments."""
    m, v, t = state.get(key, (np.zeros_like(g), np.zeros_like(g), 0))
    t += 1
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    state[key] = (m, v, t)
    mh, vh = m / (1 - b1 ** t), v / (1 - b2 ** t)
    return x - lr * mh / (np.sqrt(vh) + eps)


def inverse_record(steps, warmup):
    """Inverse rendering on the Cornell box at 512^2 with 8 cameras: each step is a 4-spp forward
    render of every camera, the L2 image loss against a seeded ground truth, and the path-replay
    adjoint of every camera (on paths of an independent seed, so the gradient of the loss is
    unbiased); Adam updates the albedo texture, the GGX roughness and sigma_s.  Reports forward and
    backward times (bwd/fwd), the loss and the parameter errors over the steps, and the adjoint
    against common-random-number central differences on a 64^2 frame (texture direction without
    Russian roulette, and roughness)."""
    import torch
    import lambda_gb300 as lg
    from lambda_gb300 import configs
    Wd = Ht = 512
    spp = 4
    rng = np.random.RandomState(5)
    gt = dict(albedo=rng.uniform(0.1, 0.9, (64, 64, 3)).astype(np.float32), roughness=0.3, sigma_a=0.1, sigma_s=0.8)
    cur = dict(albedo=np.full((64, 64, 3), 0.5, np.float32), roughness=0.6, sigma_a=0.1, sigma_s=0.2)

    def scene(params, seed, w=Wd, h=Ht, s=spp):
        sb, cams, opts = configs.cornell_inverse(w, h, s, **params)
        opts.seed = seed
        return lg.Renderer(sb), cams, opts

    films = [torch.zeros((Ht, Wd, 4), dtype=torch.float32, device="cuda") for _ in range(8)]

    def forward(r, cams, opts):
        for f, cam in zip(films, cams):
            f.zero_()
            r.render_device(cam, opts, f.data_ptr())
        return [f[..., :3] / f[..., 3:4] for f in films]

    r, cams, opts = scene(gt, 1000)
    target = [img.clone() for img in forward(r, cams, opts)]
    r.close()
    gtex = torch.zeros((64, 64, 4), dtype=torch.float32, device="cuda")
    gsc = torch.zeros(3, dtype=torch.float32, device="cuda")
    dloss = [torch.zeros((Ht, Wd, 4), dtype=torch.float32, device="cuda") for _ in range(8)]
    fwd_t, bwd_t, losses, err = [], [], [], []
    adam = {}
    n_steps = max(16, steps)
    for it in range(warmup + n_steps):
        r, cams, opts = scene(cur, 1 + it)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        imgs = forward(r, cams, opts)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss = 0.0
        npx = 8 * Wd * Ht * 3
        for d, img, tg in zip(dloss, imgs, target):
            diff = img - tg
            loss += float((diff.double() ** 2).sum()) / npx
            d[..., :3] = 2.0 * diff / npx
        gtex.zero_()
        gsc.zero_()
        # the adjoint replays paths of an independent seed: with the forward's own paths, the
        # residual and the derivative would be correlated and d(loss) biased
        opts.seed = 1_000_003 + it
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        for d, cam in zip(dloss, cams):
            r.adjoint(cam, opts, (0, 0, 4, 0), d.data_ptr(), gtex.data_ptr(), gsc.data_ptr())
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        r.close()
        if it >= warmup:
            fwd_t.append(t1 - t0)
            bwd_t.append(t3 - t2)
        losses.append(loss)
        err.append({"albedo_mae": float(np.mean(np.abs(cur["albedo"] - gt["albedo"]))),
                    "roughness": cur["roughness"], "sigma_s": cur["sigma_s"]})
        g = gtex.cpu().numpy()[..., :3].astype(np.float64)
        s_ = gsc.cpu().numpy().astype(np.float64)
        cur["albedo"] = np.clip(_adam(adam, "albedo", cur["albedo"], g, 0.03), 0.02, 0.98).astype(np.float32)
        cur["roughness"] = float(np.clip(_adam(adam, "roughness", np.array(cur["roughness"]), s_[0], 0.03), 0.05, 1.0))
        cur["sigma_s"] = float(np.clip(_adam(adam, "sigma_s", np.array(cur["sigma_s"]), s_[2], 0.06), 0.01, 4.0))
    err.append({"albedo_mae": float(np.mean(np.abs(cur["albedo"] - gt["albedo"]))),
                "roughness": cur["roughness"], "sigma_s": cur["sigma_s"]})
    fwd, bwd = float(np.median(fwd_t)), float(np.median(bwd_t))

    # gradient check: adjoint against CRN central differences on one 64^2 camera
    w64 = np.random.RandomState(11).uniform(0.0, 1.0, (64, 64, 3))
    base = dict(albedo=np.random.RandomState(12).uniform(0.1, 0.9, (8, 8, 3)).astype(np.float32),
                roughness=0.3, sigma_a=0.1, sigma_s=0.8)

    def render64(params, no_rr, s):
        sb, cams_, o = configs.cornell_inverse(64, 64, s, tex_res=8, **params)
        if no_rr:
            o.min_bounces = o.max_bounces
        rr = lg.Renderer(sb)
        f = torch.zeros((64, 64, 4), dtype=torch.float32, device="cuda")
        o.kernel_mode = 2
        rr.render_device(cams_[3], o, f.data_ptr())
        torch.cuda.synchronize()
        fn = f.double().cpu().numpy()
        val = float(np.sum(fn[..., :3] / fn[..., 3:4] * w64))
        dl = torch.zeros((64, 64, 4), dtype=torch.float32, device="cuda")
        dl[..., :3] = torch.from_numpy(w64.astype(np.float32)).cuda()
        gt_ = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
        gs_ = torch.zeros(3, dtype=torch.float32, device="cuda")
        o.kernel_mode = 1
        rr.adjoint(cams_[3], o, (0, 0, 4, 0), dl.data_ptr(), gt_.data_ptr(), gs_.data_ptr())
        torch.cuda.synchronize()
        rr.close()
        return val, gt_.cpu().numpy()[..., :3].astype(np.float64), gs_.cpu().numpy().astype(np.float64)

    v = np.random.RandomState(3).uniform(-1, 1, (8, 8, 3)).astype(np.float32)
    _, gtx, _ = render64(base, True, 512)
    e = 1e-3
    fp = render64(dict(base, albedo=base["albedo"] + e * v), True, 512)[0]
    fm = render64(dict(base, albedo=base["albedo"] - e * v), True, 512)[0]
    fd_tex, adj_tex = (fp - fm) / (2 * e), float(np.sum(gtx * v))
    _, _, gsr = render64(base, False, 2048)
    e = 1e-2
    fp = render64(dict(base, roughness=base["roughness"] + e), False, 2048)[0]
    fm = render64(dict(base, roughness=base["roughness"] - e), False, 2048)[0]
    fd_r = (fp - fm) / (2 * e)
    return {"bwd_fwd_ratio": bwd / fwd, "forward_ms": fwd * 1e3, "backward_ms": bwd * 1e3,
            "forward_mpath_s": 8 * Wd * Ht * spp / fwd / 1e6,
            "gradient_check": {"texture_direction": {"adjoint": adj_tex, "finite_difference": fd_tex,
                                                     "rel_error": abs(adj_tex - fd_tex) / abs(fd_tex),
                                                     "setup": "64^2, 512 spp, no roulette, eps 1e-3, CRN"},
                               "roughness": {"adjoint": float(gsr[0]), "finite_difference": fd_r,
                                             "rel_error": abs(gsr[0] - fd_r) / abs(fd_r),
                                             "setup": "64^2, 2048 spp, eps 1e-2, CRN"}},
            "optimisation": {"optimizer": "Adam (lr 0.03 albedo and roughness, 0.06 sigma_s)", "steps": len(losses),
                             "loss": losses, "params": err,
                             "truth": {"roughness": gt["roughness"], "sigma_s": gt["sigma_s"]}},
            "config": {"workload": "inverse rendering: Cornell box 512^2, 8 cameras, 4 spp forward + path-replay "
                                   "adjoint, L2 image loss; unknowns 64x64 albedo texture, GGX roughness, medium sigma_s",
                       "width": Wd, "height": Ht, "spp": spp, "cameras": 8}}


def main_inverse(args):
    import torch
    import lambda_gb300 as lg
    lg.build()
    torch.cuda.set_device(0)
    rec = inverse_record(args.steps, args.warmup)
    line = {"metric": METRIC, "value": rec["forward_mpath_s"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["forward_ms"] + rec["backward_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ground-truth texture and parameters)", "config": rec["config"],
            "adjoint": {k: rec[k] for k in ("bwd_fwd_ratio", "forward_ms", "backward_ms", "gradient_check",
                                             "optimisation")}}
    print(json.dumps(line))


def device_bvh_record(sb, cam, opts, steps=2):
    """The same frame on a BVH built on the device (lgpu_set_bvh_builder, LBVH): its build time for
    the scene's triangles, its node count beside the host SAH tree's, and the frame's throughput."""
    import torch
    import lambda_gb300 as lg
    from lambda_gb300 import abi
    W, H, spp = opts.width, opts.height, opts.spp
    r = lg.Renderer(sb, bvh_builder=abi.BVH_BUILD_DEVICE)
    try:
        st = r.stats()
        film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        r.render_device(cam, opts, film.data_ptr())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            r.render_device(cam, opts, film.data_ptr())
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / steps
        if float(film[..., 3].min()) != spp * (steps + 1):
            raise SystemExit("work check failed: device-BVH frame sample counts")
        d = sb.desc()
        return {"build_ms": st["bvh_build_ms"], "bvh_nodes": st["bvh_nodes"],
                "triangles": sum(d.meshes[k].num_triangles for k in range(d.num_meshes)),
                "frame_ms": t * 1e3, "value": W * H * spp / t / 1e6,
                "builder": "device LBVH: 30-bit Morton codes, radix sort, radix tree, bottom-up boxes, one "
                           "triangle per leaf (the default is the host's binned-SAH build)"}
    finally:
        r.close()


def batched_frame_rate(r, cam, opts, parts=8, steps=2):
    """Mpath-samples/s of this frame rendered through lgpu_render_batch as `parts` views of the same
    camera, each with spp / parts samples at successive sample offsets (together the frame's
    samples), device films; timed with the device synchronised on both sides."""
    import torch
    W, H, spp = opts.width, opts.height, opts.spp
    per = max(1, spp // parts)
    films = [torch.zeros((H, W, 4), dtype=torch.float32, device="cuda") for _ in range(parts)]
    views = [(cam, W, H, per, opts.max_bounces, opts.seed, f.data_ptr(), k * per) for k, f in enumerate(films)]
    r.render_batch(views, opts)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        r.render_batch(views, opts)
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / steps
    if any(float(f[..., 3].min()) != per * (steps + 1) for f in films):
        raise SystemExit("work check failed: batched frame sample counts")
    del films
    return W * H * per * parts / t / 1e6


def relmse_record(r, cam, opts, stream, rates, threshold=1e-3, ref_spp=4096, ref_seed=777,
                  levels=(4, 8, 16, 32, 64, 128, 256, 512, 1024)):
    """Samples per pixel and wall time each renderer needs to reach relMSE <= threshold on this frame.

    Reference image: the GPU render of the same frame at ref_spp with an independent seed.  Test
    images: the frame at growing spp (progressive passes, seed of opts).  relMSE = mean over pixels and
    channels of (I - R)^2 / (R^2 + 1e-2).  The GPU and the reference CPU integrator compute the same
    estimate per path (per-path parity), so they reach the threshold at the same spp and their times
    to it are spp * pixels / throughput (rates: name -> Mpath-samples/s of this frame, the batched
    one from batched_frame_rate; the batched record compares batched and plain on its own uneven
    views at equal spp)."""
    import torch
    W, H = opts.width, opts.height
    o = type(opts).from_buffer_copy(opts)
    ref = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    o.seed, o.spp = ref_seed, 256
    t0 = time.perf_counter()
    for k in range(ref_spp // 256):
        o.sample_offset = k * 256
        r.render_device(cam, o, ref.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    t_ref = time.perf_counter() - t0
    R = (ref[..., :3] / ref[..., 3:4]).double()
    den = R * R + 1e-2
    film = torch.zeros_like(ref)
    o.seed = opts.seed
    done, curve, hit = 0, [], None
    for lv in levels:
        o.spp, o.sample_offset = lv - done, done
        r.render_device(cam, o, film.data_ptr(), stream=stream)
        done = lv
        torch.cuda.synchronize()
        I = (film[..., :3] / film[..., 3:4]).double()
        err = float(torch.mean((I - R) ** 2 / den))
        curve.append([lv, err])
        if err <= threshold:
            hit = lv
            break
    rec = {"threshold": threshold, "definition": "mean((I - R)^2 / (R^2 + 1e-2)) over pixels and RGB",
           "reference": "GPU render of the same frame, %d spp, seed %d (%.1f s)" % (ref_spp, ref_seed, t_ref),
           "curve": curve, "spp_at_threshold": hit}
    if hit is not None:
        rec["seconds_to_threshold"] = {k: hit * W * H / (v * 1e6) for k, v in rates.items() if v}
    return rec


def main():
    args = parse()
    if args.workload == "batched" and args.impl == "ours":
        return main_batched(args)
    if args.workload == "inverse" and args.impl == "ours":
        return main_inverse(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    from lambda_gb300 import abi, configs

    if args.impl == "reference":
        if rank != 0:
            return
        sb, cam, opts, cfg = workload_scene(args)
        K, W_ = args.steps, args.warmup
        vals = []
        for i in range(W_ + K):
            cb = cpu_baseline(sb, cam, opts, max(2.0, min(args.cpu_seconds, 150.0 / (K + W_))))
            if i >= W_:
                vals.append(cb["value"])
        v = float(np.median(vals))
        cb["value"] = v
        cfg["l2"] = "n/a (CPU)"
        print(json.dumps({"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": K, "warmup": W_,
                          "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f32", "data": "synthetic (seeded procedural scene)", "config": cfg,
                          "impl": "reference", "cpu_baseline": cb,
                          "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    import lambda_gb300 as lg
    lg.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    sb, cam, opts, cfg = workload_scene(args)
    opts.seed = replica_seed(rank)
    opts.kernel_mode = {"auto": abi.KERNEL_AUTO, "megakernel": abi.KERNEL_MEGAKERNEL, "wavefront": abi.KERNEL_WAVEFRONT,
                        "graph": abi.KERNEL_WAVEFRONT_GRAPH}[args.mode]
    opts.pool_slots = args.pool
    opts.block_size = args.block
    r = lg.Renderer(sb, device=dev)
    W, H, spp = opts.width, opts.height, opts.spp
    paths = W * H * spp
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # counting launch (outside the timed region): nodes / triangles / rays of one frame
    stats = r.render_count(cam, opts)
    for _ in range(args.warmup):
        r.render_device(cam, opts, film.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    per_step = []
    t_start.record()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record()
        r.render_device(cam, opts, film.data_ptr(), stream=stream)
        ev[k][1].record()
        per_step.append(r.stats())   # host-side copy of the library's per-launch event timings
    t_end.record()
    torch.cuda.synchronize()
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    # every path of every rendered frame must have reached the film (no work skipped)
    rendered = args.warmup + args.steps
    counts = film[..., 3]
    if not bool(torch.all(counts == float(spp * rendered))):
        raise SystemExit("work check failed: film sample counts %s, expected %d per pixel"
                         % (torch.unique(counts)[:8].tolist(), spp * rendered))
    # end to end through the host-buffer API (film copies inside the timed region)
    host_film = np.zeros((H, W, 4), np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        r.render(cam, opts, host_film)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clk = clocks.stop()
    total_ms, e2e_ms = max_over_ranks([total_ms, e2e_s * 1e3], dist, "cuda")
    if dist:
        dist.barrier()
    value = job_throughput(paths, args.steps, world, total_ms)
    launches = int(sum(s_["launches"] for s_ in per_step))
    e2e = job_throughput(paths, args.steps, world, e2e_ms)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    pk = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    mean_kernel_s = float(np.mean(kernel_ms)) / 1e3
    kernels = kernel_table(per_step, stats, paths, kernel_ms, opts.kernel_mode == abi.KERNEL_MEGAKERNEL)
    dom = max(kernels, key=lambda n_: kernels[n_]["ms"])
    kd = kernels[dom]
    per_unit = NCU_DRAM_BYTES_PER_UNIT.get(dom)
    traffic = per_unit * kd["units"] / max(1.0, kd["launches"]) if per_unit else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": kd["achieved_gbs"], "peak": hbm, "unit": "GB/s",
            "frac": kd["achieved_gbs"] / hbm, "traffic": traffic,
            "peak_source": "measured (hbm_gbs)" if "hbm_gbs" in pk else "fallback",
            "algorithmic_bytes_per_launch": kd["alg_bytes"] / max(1.0, kd["launches"]),
            "avg_launch_ms": kd["ms"] / max(1.0, kd["launches"]),
            "kernels": kernels, "nodes_visited": stats["nodes_visited"], "tris_tested": stats["tris_tested"],
            "rays": stats["rays"], "mrays_per_s": stats["rays"] / mean_kernel_s / 1e6,
            "step_ms": float(np.mean(kernel_ms))}
    # the traversal's node and triangle records are served from L2: its roofline is the L2 read
    # peak, measured here (after the timed region) by the module's own read kernel on a 32 MiB
    # buffer; a 4 GiB read beside it checks the probe against the HBM copy peak
    l2 = r.probe_bandwidth(32 << 20, 400)
    hbm_read = r.probe_bandwidth(4 << 30, 5)
    tk = kernels.get("k_wave_trace")
    roof["l2"] = {"peak_gbs": l2, "hbm_read_gbs": hbm_read, "probe": "lgpu_probe_bandwidth: ld.global.cg float4 reads, "
                  "32 MiB x 400 passes (L2) and 4 GiB x 5 (HBM), one launch each",
                  "trace_achieved_gbs": tk["achieved_gbs"] if tk else None,
                  "trace_frac": tk["achieved_gbs"] / l2 if (tk and l2 > 0) else None}
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(sb, cam, opts, args.cpu_seconds, gpu=r)
    extras = {}
    if not args.no_extras and world == 1 and args.workload == "terrain":
        # the rest of the metric: batched vs plain, equal-relMSE times, and the adjoint's cost
        extras["batched"] = batched_record(2, 1)
        rates = {"gpu_plain": value, "gpu_batched": batched_frame_rate(r, cam, opts)}
        if cpu:
            rates["cpu_" + cpu["kind"]] = cpu["value"]
        extras["relmse"] = relmse_record(r, cam, opts, stream, rates)
        extras["adjoint"] = inverse_record(4, 1)
        extras["device_bvh"] = device_bvh_record(sb, cam, opts)
    cfg["l2"] = "scene data > L2 and a 256 MiB buffer is written between timed steps"
    cfg["width"], cfg["height"], cfg["spp"] = W, H, spp
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": cfg, "parallelism": "replicas" if world > 1 else "single GPU",
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": W * H * 16, "d2h_bytes_per_step": W * H * 16},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk}
    line.update(extras)
    print(json.dumps(line))
    r.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
