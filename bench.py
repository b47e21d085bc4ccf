"""Benchmark: photons/s of progressive vertex-merging iterations on the water-pool
workload (512x512-vertex water heightfield, GGX dielectric roughness 0.02 IOR 1.33,
diffuse floor 1.5 below, 2x2 area light, 1920x1080, 16M photons per iteration, max
path depth 8), one JSON line on stdout.

A step is one progressive iteration: light pass (16M light paths, photon store), GPU
KD-tree build over the stored photons, camera pass (one path per pixel, merge
queries), radius gather with FP64 accumulation.

  value   photons/s with the scene already resident in HBM (device-timed with CUDA
          events recorded by the library on its stream around the K steps)
  e2e     photons/s through the public C ABI with host buffers: init() from the
          Blender-layout host arrays (laid out before the timed region, as Blender
          holds them before it calls init), ingest, BVH build, upload, and per step
          one iteration plus the image read back to host memory
  roofline  the gather kernel (HBM-bound): algorithmic bytes per launch / its mean
          event-timed duration, against MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the reference's own estimator on the host cores (oracle port of the
          reference, bit-identical to it on the reference-renderable variant)
  learned_vs_plain  per-pixel RMSE against a reference image versus device time for
          learned-guided and plain vertex merging (same workload, 16 iterations each)

--impl reference times that CPU implementation alone.  --gpus N > 1 runs N
independent replicas (the path is not sharded; torchrun launches one rank per GPU).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "water_pool"
PHOTONS_PER_ITER = 16 << 20
MAX_PATH = 8
METRIC = "photons/s"
# bytes per unit of the gather (algorithmic): each stored photon's 40-byte record read
# once, each merge query's 64-byte record read once, each pixel's FP64 RGB sum read and
# written once (40 P + 64 Q + 48 X); the "touched" variant reads one photon record per
# accepted photon-query pair (40 sum k)
PHOTON_BYTES, QUERY_BYTES, PIXEL_BYTES = 40, 64, 48
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) over algorithmic bytes of one
# k_gather launch on the 960x540 / 4M-path water pool (profiles/k_gather_water_pool_960x540.md)
GATHER_TRAFFIC_OVER_ALGORITHMIC = 1.161
# SM issue efficiency of the persistent light pass from the same kind of capture
# (profiles/k_light_pass_water_pool_960x540.md): issue-active cycles and thread
# instructions per warp instruction
LIGHT_ISSUE_ACTIVE_PCT, LIGHT_LANES_ACTIVE = 62.2, 10.3


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def visible_device(local: int) -> str:
    """CUDA_VISIBLE_DEVICES value that gives a rank its own GPU: the local-th entry of a
    device list the launcher set (its only entry when it set one per rank), else the
    local rank itself."""
    ids = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    if not ids:
        return str(local)
    if len(ids) == 1:
        return ids[0]
    if local < len(ids):
        return ids[local]
    raise SystemExit(f"local rank {local} has no GPU in CUDA_VISIBLE_DEVICES={','.join(ids)}")


class Ranks:
    """Coordination of the ranks of a multi-process run (one process per GPU, launched by
    torch.distributed.run): a gloo group for the barriers around the timed regions and
    the maximum of the timings over ranks.  The ranks are independent replicas, so no
    data moves between them.  With one rank every call is a no-op."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, *values: float) -> list[float]:
        if self.dist is None:
            return [float(v) for v in values]
        import torch
        t = torch.tensor(values, dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return t.tolist()

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def nvsmi_id(lib) -> str:
    """nvidia-smi's name for the GPU this process runs on: the PCI bus id of the current
    CUDA device (nvidia-smi numbers GPUs physically and ignores CUDA_VISIBLE_DEVICES, so
    a CUDA index would name another GPU whenever the visible list does not start at 0),
    with the domain widened to the 8 hex digits nvidia-smi prints."""
    buf = C.create_string_buffer(64)
    if lib.rc_device_bus_id(buf, 64) != 0:
        raise RuntimeError("rc_device_bus_id failed")
    dom, rest = buf.value.decode().split(":", 1)
    return f"{int(dom, 16):08X}:{rest.upper()}"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region (read-only
    queries of the GPU named by `gpu`, a PCI bus id)."""

    def __init__(self, gpu: str):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkdtemp()) / "clocks.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path.exists():
            for line in self.path.read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 7:
                    try:
                        rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[3:7]))
                    except ValueError:
                        pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(seconds: float = 12.0, cores: int | None = None):
    """The reference's own estimator (oracle port, reference mode: its RNG stream, its
    hybrid Metropolis light sampler, its KD-tree) on the water scene's nearest
    reference-renderable variant (smooth glass instead of the rough dielectric, depth
    6, photons per iteration = pixels), one process per core, each rendering one
    iteration of a reduced-resolution frame; photons/s summed over processes."""
    cores = cores or os.cpu_count() or 1
    W, H = 960, 540
    code = f"""
import sys, time, numpy as np, ctypes as C
sys.path.insert(0, {str(ROOT)!r})
import oracle
from realcausticsengine_gb300 import scenes
from realcausticsengine_gb300.scene import InitArgs
sc = scenes.water_pool({W}, {H}, grid=512, samples=1)
sc.materials[0].kind = 'G'
o = oracle.oracle()
a = InitArgs(sc); a.call(o.oracle_init); o.oracle_prepare(None)
img = np.zeros(3*{W}*{H}, np.float32)
t = time.perf_counter(); o.oracle_render_reference(img.ctypes.data, 1); dt = time.perf_counter() - t
print(dt)
"""
    import oracle
    oracle.build()
    procs = [subprocess.Popen([sys.executable, "-c", code], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL)
             for _ in range(cores)]
    times = []
    for p in procs:
        out, _ = p.communicate()
        try:
            times.append(float(out.decode().strip().splitlines()[-1]))
        except (ValueError, IndexError):
            pass
    if not times:
        return None
    photons_each = W * H
    value = sum(photons_each / t for t in times)
    return {"value": value, "unit": METRIC, "cores": len(times), "kind": "port",
            "sample": f"water_pool variant (smooth glass, depth 6) {W}x{H}, {photons_each} light paths + "
                      f"{photons_each} camera paths per process, 1 iteration, {len(times)} processes; "
                      f"mean {np.mean(times):.2f} s per process"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(cores=args.cpu_cores)
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(cores=args.cpu_cores)
        vals.append(last["value"])
    dt = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dt / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD + " (reference-renderable variant)", "parallelism": "processes"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": last["cores"], "kind": last["kind"],
                             "sample": last["sample"]},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    from realcausticsengine_gb300 import _native, scenes
    from realcausticsengine_gb300.scene import InitArgs
    from realcausticsengine_gb300.session import Renderer
    from realcausticsengine_gb300 import abi

    ranks = Ranks()
    rank, world, local = ranks.rank, ranks.world, ranks.local
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = visible_device(local)
    lib = _native.lib()
    sc = scenes.water_pool(args.width, args.height, grid=args.grid, samples=args.steps)
    paths = args.photons

    # ---- device-resident throughput
    r = Renderer(sc, max_path_length=MAX_PATH, photons_per_iter=paths, seed=rank,
                 graph_replay=not args.no_graph_replay)
    r.prepare()
    r.render(args.warmup)
    dev = np.zeros(4, np.float64)
    ranks.barrier()
    with ClockSampler(nvsmi_id(lib)) as clk:
        t0 = time.perf_counter()
        # synchronises the library's stream before its first event and after its last
        _native.check(lib.rc_render_timed(args.steps, dev.ctypes.data), "rc_render_timed")
        wall = time.perf_counter() - t0
    ranks.barrier()
    st = r.stats()
    device_ms = dev[0]
    gather_ms_mean, gather_bytes, nq, nph = dev[1], dev[2], st["queries"], st["photons"]
    r.release()

    # ---- end to end through the C ABI with host buffers
    cfg = abi.RcConfig()
    lib.rc_default_config(C.byref(cfg))
    cfg.max_path_length = MAX_PATH
    cfg.photons_per_iter = paths
    cfg.seed = rank
    cfg.write_exr = 0
    cfg.graph_replay = 0 if args.no_graph_replay else 1
    lib.rc_set_config(C.byref(cfg))
    img = np.zeros((args.height, args.width, 3), np.float32)
    ia = InitArgs(sc)            # the Blender-side structures init() reads
    ranks.barrier()
    t0 = time.perf_counter()
    ia.call(lib.init)
    _native.check(lib.rc_prepare(), "rc_prepare")
    for _ in range(args.steps):
        _native.check(lib.rc_render(1), "rc_render")
        # a synchronous read: the step's image is on the host when it returns
        _native.check(lib.rc_read_image(img.ctypes.data, args.width, args.height), "rc_read_image")
    e2e_s = time.perf_counter() - t0
    ranks.barrier()
    lib.rc_release()
    h2d = sum(m.verts.nbytes + m.normals.nbytes + m.tris.nbytes for m in sc.meshes)
    d2h = img.nbytes            # the FP32 mean image read back each step

    # the slowest rank's times; every rank processed `paths * steps` light paths
    device_ms, e2e_s = ranks.max(device_ms, e2e_s)
    ranks.close()
    if rank != 0:
        return
    value = paths * args.steps * world / (device_ms / 1000.0)
    e2e_value = paths * args.steps * world / e2e_s
    peak, peak_kind = measured_peaks()
    achieved = gather_bytes / (gather_ms_mean / 1000.0) / 1e9 if gather_ms_mean > 0 else 0.0
    # DRAM bytes of one gather: the ncu capture on the 960x540 / 4M-path case moved
    # 1.161x its algorithmic bytes; scaled to this workload's launch by its algorithmic
    # bytes (photon, query and pixel records all scale with their counts)
    traffic = GATHER_TRAFFIC_OVER_ALGORITHMIC * gather_bytes
    touched = PHOTON_BYTES * st["merged"]
    line = {
        "metric": METRIC, "value": float(value), "unit": METRIC,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": device_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{WORKLOAD} {args.width}x{args.height}, {args.grid}x{args.grid}-vertex heightfield "
                               f"({sc.num_tris()} tris), {paths} photons/iter, max depth {MAX_PATH}",
                   "photons_per_iter": paths, "stored_photons_per_iter": nph, "merge_queries_per_iter": nq,
                   "l2": "inputs larger than L2 (photon map and query buffers > 129 MB)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": float(e2e_value), "unit": METRIC, "h2d_bytes_per_step": int(h2d // max(args.steps, 1)),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"kernel": "k_gather (fused photon gather: traversal, merge evaluation, FP64 pixel sums)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": gather_bytes,
                     "bytes_formula": "40 B x stored photons + 64 B x merge queries + 48 B x pixels",
                     "touched_bytes": touched,
                     "touched_frac": (touched / (gather_ms_mean / 1000.0) / 1e9) / peak if gather_ms_mean > 0 else 0.0},
        "kd_roofline": kd_roofline(nph, st["kd_ms"], peak, peak_kind),
        "gpu_launches": int(dev[3]),
        "clocks": clk.summary(),
        "phase_ms_per_step": {k: st[k] for k in ("light_ms", "kd_ms", "camera_ms", "gather_ms")},
        "light_pass": {
            "paths_per_s": paths / (st["light_ms"] / 1000.0) if st["light_ms"] > 0 else None,
            "rays_per_s": st["light_rays"] / (st["light_ms"] / 1000.0) if st["light_ms"] > 0 and st["light_rays"] else None,
            "rays_per_path": st["light_rays"] / paths if st["light_rays"] else None,
            # ncu on the 960x540 / 4M-path case (profiles/k_light_pass_water_pool_960x540.md)
            "issue_active_pct_ncu": LIGHT_ISSUE_ACTIVE_PCT, "lanes_active_per_warp_instruction_ncu": LIGHT_LANES_ACTIVE,
            "note": "window of the last iteration's light pass (the coherent path order included)"},
        "phase_note": "event windows of the last iteration; the camera pass runs on a second stream "
                      "beside the light pass's last launch and the KD build, its window opening there",
        "wall_s": wall,
    }
    if not args.no_learned:
        line["learned_vs_plain"] = learned_equal_time(args)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cores=args.cpu_cores)
        line["same_config"] = same_config_anchor(line["cpu_baseline"])
    print(json.dumps(line), flush=True)


def kd_roofline(nph: float, kd_ms: float, peak: float, peak_kind: str) -> dict:
    """The KD build against the HBM roofline with the algorithmic bytes of a median-split
    build over P photons: 12 P (positions read once) + 2 x 16 P per level over ceil(log2 P)
    levels (x, y, z, id read and written) + 8 B per node of the 2^(floor(log2 P) + 1)-node
    array.  kd_ms is the event window of the build, its boxes and the tree-order records,
    with the camera pass running beside them on the other stream (so a lower bound on
    the build's own rate)."""
    import math
    P = float(nph)
    if P < 2 or kd_ms <= 0:
        return None
    b = 12.0 * P + 32.0 * P * math.ceil(math.log2(P)) + 8.0 * 2 ** (math.floor(math.log2(P)) + 1)
    achieved = b / (kd_ms / 1000.0) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind, "algorithmic_bytes": b, "window_ms": kd_ms,
            "bytes_formula": "12 P + 32 P ceil(log2 P) + 8 x 2^(floor(log2 P) + 1)"}


def same_config_anchor(cpu: dict | None, width: int = 960, height: int = 540, steps: int = 8, warmup: int = 2):
    """The GPU on the workload the CPU baseline runs: the water pool's reference-renderable
    variant (smooth glass), 960x540, the reference's own settings (rc_default_config:
    hybrid Metropolis light sampler, max path depth 6, light paths per iteration =
    pixels).  Device-timed light paths per second next to the CPU's, for a like-for-like
    ratio beside the headline (which runs the rough-glass, depth-8, 16.7M-path workload)."""
    from realcausticsengine_gb300 import _native, abi, scenes
    from realcausticsengine_gb300.session import Renderer
    sc = scenes.water_pool(width, height, grid=512, samples=steps)
    sc.materials[0].kind = "G"
    r = Renderer(sc, max_path_length=6, photons_per_iter=0, sampler=abi.SAMPLER_HYBRID, seed=0)
    r.prepare()
    r.render(warmup)
    out = np.zeros(4, np.float64)
    _native.check(_native.lib().rc_render_timed(steps, out.ctypes.data), "rc_render_timed")
    r.release()
    paths = width * height
    value = paths * steps / (out[0] / 1000.0)
    res = {"workload": f"water_pool variant (smooth glass) {width}x{height}, hybrid Metropolis sampler (65,536 "
                       f"chains), max depth 6, {paths} light paths/iter (= pixels)",
           "value": value, "unit": METRIC, "ms_per_step": out[0] / steps}
    if cpu:
        res["cpu_value"] = cpu["value"]
        res["gpu_over_cpu"] = value / cpu["value"]
    return res


def learned_equal_time(args, iters: int = 16, ref_iters: int = 512, ref_scale: int = 8):
    """Learned-guided vs plain vertex merging on the same workload: per-pixel RMSE of the
    FP64-accumulated image against two reference images, as a function of device time.

      full         reference: plain, `ref_iters` iterations, independent light and camera
                   seeds (its variance ~1/32 of a 16-iteration render's): the whole
                   image error, camera-side noise (pixel jitter, camera paths through the
                   rough water) included.
      photon_side  reference: plain with the same camera seed and iterations as the
                   compared renders (the same camera paths and merge queries) and
                   `ref_scale` x the light paths per iteration: the error of the photon
                   side of the estimator alone, the part an emission proposal can change.

    Plain and learned share their camera seed.  The learned render trains on
    iterations 0..7 (32 Adam steps each, lr 1e-3) and guides from iteration 1, with the
    workload's light paths per iteration and with half of them (the same number of
    stored photons as plain, since guided paths store about twice as many).  Reports the
    end points, and the device-time ratio at which each learned curve reaches plain's
    final error (None when it does not within `iters` iterations)."""
    from realcausticsengine_gb300 import scenes
    from realcausticsengine_gb300.session import Renderer

    sc = scenes.water_pool(args.width, args.height, grid=args.grid, samples=ref_iters)

    def run(n, seed, camera_seed, learned, refs=(), paths=None):
        r = Renderer(sc, max_path_length=MAX_PATH, photons_per_iter=paths or args.photons, seed=seed,
                     camera_seed=camera_seed, learned_proposal=learned, train_iterations=8, train_steps=32,
                     learning_rate=1e-3)
        r.prepare()
        if not refs:
            r.render(n)
            img = r.image().astype(np.float64)
            r.release()
            return img, None
        t, curves = 0.0, [[] for _ in refs]
        for _ in range(n):
            r.render(1)
            t += r.stats()["device_ms"]
            img = r.image().astype(np.float64)
            for c, ref in zip(curves, refs):
                c.append((t, float(np.sqrt(((img - ref) ** 2).mean()))))
        r.release()
        return img, curves

    ref_full, _ = run(ref_iters, 1001, 1002, False)
    ref_cam, _ = run(iters, 1001, 8, False, paths=ref_scale * args.photons)
    _, (plain_full, plain_cam) = run(iters, 7, 8, False, (ref_full, ref_cam))

    def reach(curve, target):
        return next((t for t, e in curve if e <= target), None)

    out = {"workload": "same as the line's config", "iterations": iters,
           "references": {"full": f"plain, {ref_iters} iterations, independent light and camera seeds",
                          "photon_side": f"plain, same camera seed and iterations, {ref_scale}x light paths"},
           "plain": {"device_ms": plain_full[-1][0], "rmse_full": plain_full[-1][1], "rmse_photon_side": plain_cam[-1][1]}}
    for label, paths in (("learned", args.photons), ("learned_half_paths", args.photons // 2)):
        _, (lf, lc) = run(iters, 7, 8, True, (ref_full, ref_cam), paths)
        rf, rc = reach(lf, plain_full[-1][1]), reach(lc, plain_cam[-1][1])
        out[label] = {"light_paths_per_iter": paths, "device_ms": lf[-1][0], "rmse_full": lf[-1][1],
                      "rmse_photon_side": lc[-1][1],
                      "time_ratio_full": rf / plain_full[-1][0] if rf is not None else None,
                      "time_ratio_photon_side": rc / plain_cam[-1][0] if rc is not None else None,
                      "curve_full": [(round(a, 2), round(b, 6)) for a, b in lf]}
    out["plain"]["curve_full"] = [(round(a, 2), round(b, 6)) for a, b in plain_full]
    ratios = [out[k]["time_ratio_full"] for k in ("learned", "learned_half_paths") if out[k]["time_ratio_full"]]
    out["time_ratio_to_plain_rmse"] = min(ratios) if ratios else None
    return out


def run_batch(args):
    """The 64-scene batch.  Every scene gets its own library context (scene, settings,
    device buffers); --batch-threads host threads load the scenes through init() and
    prepare them (BVH build, upload).  Then rc_batch_render renders all of them as one
    launch set per iteration (one light pass and one camera pass over every scene, the
    per-scene KD builds and gathers as branches of one CUDA graph): --warmup iterations
    (each scene's first iteration alone, the batch passes' shape tuning, the graph's
    instantiation), then --steps timed iterations.  value = photons of all scenes over
    the device time of the timed iterations (CUDA events on the batch stream, all scenes
    resident in HBM); e2e = the same photons per iteration over the wall time of load +
    all iterations + readback of every image (the scenes' host arrays and the
    Blender-layout structures init() reads are built before).  per_context: the same
    scenes rendered --steps more iterations each by rc_render_timed from the host
    threads, one scene per context call (the design without the batch launch set)."""
    from concurrent.futures import ThreadPoolExecutor
    from realcausticsengine_gb300 import _native, scenes
    from realcausticsengine_gb300.scene import InitArgs
    from realcausticsengine_gb300 import abi
    lib = _native.lib()
    batch = [scenes.batch_scene(seed) for seed in range(args.batch)]   # host arrays, outside the timing
    blender = [InitArgs(sc) for sc, _ in batch]                        # Blender-side structures, likewise
    ctxs = [lib.rc_context_create() for _ in batch]
    if not all(ctxs):
        raise MemoryError("rc_context_create failed")
    handles = (C.c_void_p * len(ctxs))(*ctxs)
    order = sorted(range(len(batch)), key=lambda k: -batch[k][1] * batch[k][0].num_tris() ** 0.25)
    W, K = max(args.warmup, 1), args.steps

    def load(k):
        sc, paths = batch[k]
        lib.rc_context_bind(ctxs[k])
        try:
            cfg = abi.RcConfig()
            lib.rc_default_config(C.byref(cfg))
            cfg.max_path_length, cfg.photons_per_iter, cfg.seed, cfg.write_exr = MAX_PATH, paths, k, 0
            _native.check(lib.rc_set_config(C.byref(cfg)), "rc_set_config")
            blender[k].call(lib.init)
            _native.check(lib.rc_prepare(), "rc_prepare")
        finally:
            lib.rc_context_bind(None)

    def read(k):
        sc, _ = batch[k]
        lib.rc_context_bind(ctxs[k])
        try:
            img = np.zeros((sc.camera.height, sc.camera.width, 3), np.float32)
            _native.check(lib.rc_read_image(img.ctypes.data, sc.camera.width, sc.camera.height), "rc_read_image")
        finally:
            lib.rc_context_bind(None)

    per_scene = [None] * len(batch)

    def render_alone(k):
        lib.rc_context_bind(ctxs[k])
        try:
            out = np.zeros(4, np.float64)
            _native.check(lib.rc_render_timed(K, out.ctypes.data), "rc_render_timed")
            sc, paths = batch[k]
            per_scene[k] = (k, sc.num_tris(), paths, round(out[0] / K, 3))
        finally:
            lib.rc_context_bind(None)

    T = max(1, args.batch_threads)
    warm = np.zeros(6, np.float64)
    timed = np.zeros(6, np.float64)
    with ThreadPoolExecutor(T) as ex, ClockSampler(nvsmi_id(lib)) as clk:
        t0 = time.perf_counter()
        list(ex.map(load, order))
        t1 = time.perf_counter()
        _native.check(lib.rc_batch_render(handles, len(ctxs), W, warm.ctypes.data), "rc_batch_render (warm-up)")
        t2 = time.perf_counter()
        _native.check(lib.rc_batch_render(handles, len(ctxs), K, timed.ctypes.data), "rc_batch_render")
        t3 = time.perf_counter()
        list(ex.map(read, order))
        t4 = time.perf_counter()
        # the design without the batch launch set, on the same resident scenes
        list(ex.map(render_alone, order))
        t5 = time.perf_counter()
    clocks = clk.summary()
    for c in ctxs:
        lib.rc_context_bind(c)
        lib.rc_release()
        lib.rc_context_bind(None)
        lib.rc_context_destroy(c)
    paths_per_iter = sum(paths for _, paths in batch)
    tris = sum(sc.num_tris() for sc, _ in batch)
    device_ms = float(timed[0])
    line = {"metric": METRIC, "value": paths_per_iter * K / (device_ms / 1000.0), "unit": METRIC, "n_gpus": 1,
            "steps": K, "warmup": W, "ms_per_step": device_ms / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batch of {args.batch} scenes: displaced glass spheres (vertex noise amplitude "
                                   "U(0,0.2)) of log-uniform [1k, 2M] triangles, IOR U(1.3,1.8), roughness U(0,0.1), "
                                   "over a diffuse plane, 1-4 point/area lights, log-uniform [256k, 8M] photons/iter, "
                                   "512x512", "total_triangles": tris, "photons_per_iter": paths_per_iter,
                       "host_threads": T, "contexts": len(batch),
                       "l2": "inputs larger than L2 (64 scenes' photon maps, queries and BVHs)"},
            "e2e": {"value": paths_per_iter * (W + K) / (t4 - t0), "unit": METRIC, "wall_s": t4 - t0,
                    "load_s": t1 - t0, "warmup_s": t2 - t1, "render_s": t3 - t2, "read_s": t4 - t3,
                    "iterations": W + K, "d2h_bytes_per_run": 12 * 512 * 512 * len(batch),
                    "note": "scenes uploaded once by init/rc_prepare, images read back once after the last iteration"},
            "gpu_launches": int(timed[2]),
            "batch": {"graph_iterations": int(timed[1]), "kernels_per_iteration": timed[2] / max(timed[1], 1),
                      "redone_iterations": int(timed[3] + warm[3]), "light_ms_last": timed[4],
                      "camera_ms_last": timed[5], "render_wall_s": t3 - t2},
            "per_context": {"value": paths_per_iter * K / (t5 - t4), "unit": METRIC, "wall_s": t5 - t4,
                            "note": "the same resident scenes, --steps iterations each through rc_render_timed from "
                                    "the host threads (per-scene launches and graphs), wall time",
                            "per_scene": per_scene},
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--photons", type=int, default=PHOTONS_PER_ITER)
    ap.add_argument("--cpu-cores", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-graph-replay", action="store_true",
                    help="every iteration reads its counts back (no asynchronous CUDA-graph replay)")
    ap.add_argument("--workload", default="water_pool", choices=["water_pool", "batch"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--batch-threads", type=int, default=2,
                    help="host threads driving the batch's scenes (one library context per scene)")
    return ap.parse_args(argv)


def main():
    args = parse_args()
    if args.workload == "batch" and args.impl != "reference":
        run_batch(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
