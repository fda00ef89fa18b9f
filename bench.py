"""Benchmark of the DDGI probe-update path (trace + blend) on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--workload NAME]

A frame is one probe update of the whole volume: ray generation, SDF march,
hit shading, irradiance + distance blend with the border copy.  A step is
the workload's 16-frame update sequence.  The metric is probe-rays/s =
probes x rays x frames / time.

  value        device-resident inputs, CUDA events around each frame on the
               launching stream; a 256 MB L2 flush runs between frames
               (outside the events)
  e2e          the same frames through the C ABI with host buffers: each
               frame uploads its direct-light atlas from pinned host memory,
               updates, and reads both probe atlases back
  roofline     the march kernel: algorithmic SDF bytes (mip + full-res
               trilinear taps actually taken + normal taps, counted per ray
               in an untimed debug pass of the same frames) per launch over
               its event time, against the measured HBM copy bandwidth
  cpu_baseline the CPU oracle (FP32, OpenMP, all host threads) on a bounded
               sample of the same workload
  atlas_rel_err_vs_fp64
               per atlas (irradiance, distance), frames 0-2: the GPU's
               atlases against the FP64 oracle's trace + blend of a seeded
               probe sample, fed the GPU's previous atlases
  batched_served
               the batched (48 uneven volumes, one launch per stage, graph,
               autotuned) and served (Poisson arrivals, memory-budget
               admission) forms on the same GPU, and the batched form's
               probe-rays/s over the plain form's `value`

--impl reference times that CPU restatement of the reference shaders alone
(the reference itself is a Windows Vulkan renderer with no CPU path and no
graphics stack on this machine).  Under torchrun every rank updates its own
replica of the volume (replicas only: the volumes are independent).
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

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "probe-rays/s (trace+blend) at ≤2e-3 rel irradiance err vs FP64; served p99 ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="production_32x16x32_r256_sdf256")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline time budget")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--march-variant", type=int, default=None, help="override the volume's march variant (0-5, 10, 11)")
    ap.add_argument("--shade-variant", type=int, default=None, help="override the volume's shade variant (1,2,4,8)")
    ap.add_argument("--ray-order", type=int, default=None, help="override the volume's ray order (0, 1)")
    ap.add_argument("--march-budget", type=int, default=None, help="override the volume's march budget (-1 one pass)")
    ap.add_argument("--shade-order", type=int, default=None, help="override the volume's shading order (0, 1)")
    ap.add_argument("--shade-split", type=int, default=None, help="override the volume's split shading (-1, 0, 1)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serve200: length of the timed Poisson run")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="serve200: requests per second, all sessions")
    ap.add_argument("--serve-budget-gb", type=float, default=120.0, help="serve200: device-memory budget")
    ap.add_argument("--frames-per-step", type=int, default=16, help="frames of the volume in one step")
    ap.add_argument("--no-batched-served", action="store_true", help="skip the batched and served forms")
    ap.add_argument("--batch-tuning", default=None,
                    help="batch48: a fixed tuning (JSON object of luxgi_ddgi_batch_tuning fields) instead of the autotuner")
    ap.add_argument("--no-sequential", action="store_true",
                    help="batch48: skip the one-volume-at-a-time comparison")
    ap.add_argument("--ns-serve-seconds", type=float, default=8.0,
                    help="batched/served leg: length of the timed serving run")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path("/tmp") / f"luxgi_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def traffic_from_profile(workload: str, kernel: str, work_items: int):
    """DRAM bytes of one launch of `kernel` on `workload`, from the committed
    ncu capture summary (profiles/traffic.json): bytes per work item of the
    captured case times this launch's work items (the capture runs a smaller
    case of the same scene; traffic grows with the rays marched)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        e = d.get(workload, {}).get(kernel)
        if not e:
            return None
        return int(e["dram_bytes_per_item"] * work_items)
    except Exception:
        return None


# ------------------------------------------------------------- CPU oracle leg
def cpu_baseline(w, host, rot, seconds: float):
    """FP32 oracle trace + blend on a bounded sample of probes, all threads."""
    import oracle

    vd = w.volume.desc()
    inp = oracle.HostInputs(host, w.volume.light_mode)
    R = w.volume.rays_per_probe
    P = w.volume.probes
    threads = oracle.num_threads()
    n = min(P, 32)
    elapsed = 0.0
    while True:
        t0 = time.perf_counter()
        rays, _ = oracle.trace(vd, inp, rot, 0, precision=0, probes=(0, n), want_info=False)
        dirs = oracle.ray_dirs(rot, R, 0)
        oracle.blend(vd, dirs, rays, first=True, precision=0, border=False, probes=(0, n))
        elapsed = time.perf_counter() - t0
        if elapsed * 4 > seconds or n >= P:
            break
        n = min(P, max(n * 2, int(n * seconds / 2 / max(elapsed, 1e-3))))
    return {"value": n * R / elapsed, "unit": "probe-rays/s", "cores": threads, "kind": "port",
            "sample": f"{n} probes x {R} rays x 1 frame of {w.name} (oracle FP32 trace + blend, {elapsed:.2f} s)"}


def atlas_error_vs_fp64(w, host, snaps, ranges=8, length=128):
    """Relative error (|gpu - fp64| / max(|fp64|, 1e-3)) of each atlas, over
    the cells (interior + border texels) of a seeded sample of probes, for
    every frame in `snaps` = [(rot, frame, prev (irr, dist) or None, cur
    (irr, dist))].  The FP64 oracle traces and blends the sample itself,
    fed the GPU's previous atlases (the bounce source and the hysteresis
    history), so each frame is checked on its own inputs."""
    import numpy as np

    import oracle

    vd = w.volume.desc()
    inp = oracle.HostInputs(host, w.volume.light_mode)
    u = vd.uniform
    R = u.rays_per_probe
    P = w.volume.probes
    length = min(length, P)
    rng = np.random.default_rng(0xE44)
    slots = P // length
    picks = sorted(rng.choice(slots, size=min(ranges, slots), replace=False))
    spans = [(int(k) * length, int(k) * length + length) for k in picks]
    XY = u.probe_counts[0] * u.probe_counts[1]
    errs = {"irradiance": [], "distance": []}
    for rot, f, prev, cur in snaps:
        pi, pd = (None, None) if prev is None else prev
        for p0, p1 in spans:
            r64, _ = oracle.trace(vd, inp, rot, f, pi, pd, precision=1, probes=(p0, p1), want_info=False)
            i64, d64 = oracle.blend(vd, oracle.ray_dirs(rot, R, 1), r64, pi, pd, first=(f == 0), precision=1,
                                    probes=(p0, p1))
            for key, got, ref, n in (("irradiance", cur[0], i64, u.irradiance_probe_side),
                                     ("distance", cur[1], d64, u.depth_probe_side)):
                for p in range(p0, p1):
                    cx, cy = p % XY, p // XY
                    ys = slice(1 + cy * (n + 2), 1 + (cy + 1) * (n + 2))
                    xs = slice(1 + cx * (n + 2), 1 + (cx + 1) * (n + 2))
                    a = got[ys, xs].astype(np.float64)
                    b = ref[ys, xs].astype(np.float64)
                    errs[key].append((np.abs(a - b) / np.maximum(np.abs(b), 1e-3)).ravel())
    out = {}
    for key, parts in errs.items():
        e = np.concatenate(parts)
        out[key] = {"max": float(e.max()), "p99": float(np.quantile(e, 0.99)), "median": float(np.median(e))}
    out["probes"] = len(spans) * length
    out["frames"] = [f for _, f, _, _ in snaps]
    out["bound"] = 2e-3
    out["within_bound"] = bool(max(out["irradiance"]["max"], out["distance"]["max"]) <= 2e-3)
    return out


def workload_config(w, world: int, frames_per_step: int) -> dict:
    """The `config` of a single-volume workload's line (both arms)."""
    v, sc = w.volume, w.scene
    return {"workload": w.name, "probes": v.probes, "rays_per_probe": v.rays_per_probe,
            "probe_counts": list(v.probe_counts), "frames_per_step": frames_per_step,
            "sdf": f"{sc.sdf_resolution}^3 {'fp16' if sc.sdf_format else 'fp32'}", "primitives": sc.num_primitives,
            "atlas": sc.atlas_resolution, "octahedral_sides": [v.irradiance_side, v.depth_side],
            "max_steps": v.max_steps, "light_mode": "per-hit bounce" if v.light_mode else "light cache",
            "blend": "tensor" if v.blend else "fp32 simt", "storage": "fp16" if v.storage else "fp32",
            "parallelism": f"replicas{world}", "l2": "256 MB flush between frames (outside the events)"}


# ------------------------------------------------------------------- ours
def run_ours(args, rank: int, world: int):
    import numpy as np
    import torch

    from luxgi_gb300 import DDGIVolume, DeviceScene, HostScene, WORKLOADS, frame_rotation, _native as N
    from dataclasses import replace

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev_t = torch.device("cuda", local)
    w = WORKLOADS[args.workload]
    for key in ("march_variant", "shade_variant", "ray_order", "march_budget", "shade_order", "shade_split"):
        val = getattr(args, key)
        if val is not None:
            w = replace(w, volume=replace(w.volume, **{key: val}))
    v = w.volume
    P, R = v.probes, v.rays_per_probe
    F = max(1, args.frames_per_step)
    host = HostScene(w.scene)
    dev = DeviceScene(host, v.light_mode, device=f"cuda:{local}")
    vol = DDGIVolume(v)
    vol.bind_scene(dev)
    seed = 0x5EED + rank
    K, W = args.steps, args.warmup
    nf = (W + K) * F
    rots = [frame_rotation(seed, f) for f in range(nf)]
    stream = torch.cuda.current_stream()

    # warm-up frames; the first three are kept (previous and new atlases) for
    # the per-atlas error against the FP64 oracle
    snaps = []
    prev = None
    for f in range(W * F):
        vol.update(rots[f])
        if f < 3:
            torch.cuda.synchronize()
            cur = tuple(a.float().cpu().numpy() for a in vol.atlases())
            snaps.append((rots[f], f, prev, cur))
            prev = cur
    torch.cuda.synchronize()

    # exact algorithmic bytes of the timed traces (untimed debug pass; the
    # march does not depend on the atlases, so counts equal the timed ones)
    vol.set_debug_rays(True)
    esz = 2 if host.sdf_format == N.STORAGE_FP16 else 4
    march_bytes = []
    steps_total = 0
    fine_total = 0
    for f in range(W * F, nf):
        vol.trace(rots[f])
        info = vol.rays()[2]
        st = info[..., 0].to(torch.int64).sum().item()
        fine = info[..., 2].to(torch.int64).sum().item()
        hits = (info[..., 1] >= 0).sum().item()
        steps_total += st
        fine_total += fine
        # SDFCommon.glsl reads per step 8 mip taps, per full-resolution sample
        # 8 taps, per hit 6 x 8 normal taps; the march writes a 20-byte record
        march_bytes.append((st * 8 + fine * 8 + hits * 48) * esz + P * R * 20)
    vol.set_debug_rays(False)
    torch.cuda.synchronize()

    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev_t)
    n_t = K * F
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(n_t)]
    vol.set_stage_timing(True)          # CUDA events between the stages, on the launching stream
    stages = []
    clocks = Clocks(local)
    launches0 = N.ddgi().luxgi_launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    for k in range(n_t):
        flush.zero_()
        ev[k][0].record(stream)
        vol.trace(rots[W * F + k], stream)
        ev[k][1].record(stream)
        vol.probe_update(stream)
        ev[k][2].record(stream)
        vol.end_frame()
        stages.append(vol.stage_times())   # waits for this frame (outside its events)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    vol.set_stage_timing(False)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = N.ddgi().luxgi_launch_count() - launches0
    t_trace = [ev[k][0].elapsed_time(ev[k][1]) for k in range(n_t)]
    t_blend = [ev[k][1].elapsed_time(ev[k][2]) for k in range(n_t)]
    t_all = sum(t_trace) + sum(t_blend)          # ms, flush excluded
    if world > 1:
        t = torch.tensor([t_all], device=dev_t)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_all = float(t.item())
    value = world * P * R * n_t / (t_all / 1e3)

    # e2e through the C ABI with host buffers: every frame uploads its
    # direct-light atlas from pinned memory and reads both probe atlases
    # back.  Uploads and readbacks run on two more streams, overlapped with
    # the neighbouring frames' compute: frame k's upload lands in a device staging buffer
    # (two, alternating) and is moved into the bound atlas on the compute
    # stream; frame k's readback runs while frame k + 1 computes, and frame
    # k + 2 (which overwrites that ping-pong atlas) waits for it.
    e2e = None
    if not args.no_e2e:
        direct_h = [torch.from_numpy(host.direct.view(np.int16)).pin_memory() for _ in range(2)]
        stage = [torch.empty_like(dev.direct) for _ in range(2)]
        irr, dist = vol.atlases()
        irr_h = [torch.empty(irr.shape, dtype=irr.dtype).pin_memory() for _ in range(2)]
        dist_h = [torch.empty(dist.shape, dtype=dist.dtype).pin_memory() for _ in range(2)]
        erots = [frame_rotation(seed + 1000, f) for f in range(n_t + 2)]
        up = torch.cuda.Stream(device=dev_t)
        down = torch.cuda.Stream(device=dev_t)

        def e2e_run(frames):
            up_done = [None, None]        # staging k % 2 filled
            stage_free = [None, None]     # staging k % 2 consumed by its frame
            back_done = [None, None]      # readback of the atlas slot k % 2 finished
            for k in frames:
                b = k % 2
                with torch.cuda.stream(up):
                    if stage_free[b] is not None:
                        up.wait_event(stage_free[b])
                    stage[b].copy_(direct_h[b], non_blocking=True)
                    up_done[b] = torch.cuda.Event()
                    up_done[b].record(up)
                stream.wait_event(up_done[b])
                if back_done[b] is not None:
                    stream.wait_event(back_done[b])
                with torch.cuda.stream(stream):
                    dev.direct.copy_(stage[b], non_blocking=True)
                stage_free[b] = torch.cuda.Event()
                stage_free[b].record(stream)
                vol.update(erots[k], stream)
                done = torch.cuda.Event()
                done.record(stream)
                irr, dist = vol.atlases()
                with torch.cuda.stream(down):
                    down.wait_event(done)
                    irr_h[b].copy_(irr, non_blocking=True)
                    dist_h[b].copy_(dist, non_blocking=True)
                    back_done[b] = torch.cuda.Event()
                    back_done[b].record(down)
            torch.cuda.synchronize()

        e2e_run(range(2))
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        e2e_run(range(2, n_t + 2))
        te = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([te], device=dev_t)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            te = float(t.item())
        e2e = {"value": world * P * R * n_t / te, "unit": "probe-rays/s",
               "h2d_bytes_per_step": F * int(direct_h[0].numel() * 2 + 36),
               "d2h_bytes_per_step": F * int(irr_h[0].numel() * irr_h[0].element_size() +
                                             dist_h[0].numel() * dist_h[0].element_size()),
               "overlap": "uploads and readbacks on two more streams, overlapped with the neighbouring frames"}

    pk = peaks()
    avg_trace_ms = sum(t_trace) / n_t
    stage_avg = {k: sum(s[k] for s in stages) / n_t for k in ("setup", "march", "shade", "blend")}
    avg_bytes = sum(march_bytes) / n_t
    achieved = avg_bytes / (stage_avg["march"] / 1e3) / 1e9
    traffic = traffic_from_profile(w.name, "march_kernel", P * R)
    roofline = {"kernel": "march_kernel (global-SDF sphere tracing)", "bound": "hbm",
                "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / pk["hbm_gbs"], 4), "peak_source": pk["source"],
                "traffic": traffic, "algorithmic_bytes_per_launch": int(avg_bytes),
                "avg_launch_ms": round(stage_avg["march"], 4),
                "avg_march_steps_per_ray": round(steps_total / (n_t * P * R), 2),
                "avg_fine_samples_per_ray": round(fine_total / (n_t * P * R), 2)}
    ns = None
    if not args.no_batched_served and world == 1:
        # the batched and served forms on the same GPU (one process: the
        # scaling run's ranks time the plain form only)
        del vol, dev, flush
        torch.cuda.empty_cache()
        ns = batched_served_leg(args, value)
    if rank != 0:
        return
    cpu, err = (None, None)
    if not args.no_cpu and world == 1:
        # the CPU baseline and the FP64 error check: rank 0 at N = 1 only
        cpu = cpu_baseline(w, host, rots[0], args.cpu_seconds)
        if snaps:
            err = atlas_error_vs_fp64(w, host, snaps)
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "probe-rays/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": round(t_all / K, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16 sdf, fp32 march" if host.sdf_format else "fp32",
        "data": "synthetic (seeded analytic scene)",
        "config": workload_config(w, world, F),
        "ms_per_frame": round(t_all / n_t, 4),
        "stage_ms": {"trace": round(avg_trace_ms, 4), "blend": round(sum(t_blend) / n_t, 4),
                     **{k: round(x, 4) for k, x in stage_avg.items()}},
        "wall_s": round(wall, 4),
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu,
        "atlas_rel_err_vs_fp64": err, "batched_served": ns, "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- batch
def measure_batch(ws, hosts, K: int, W: int, world: int, e2e_on: bool = True, seed: int = 0x5EED,
                  tuning: dict | None = None, sequential: bool = True) -> dict:
    """The batching form over workloads `ws` (scenes `hosts`): `value` is
    the batched, graph-replayed form, autotuned unless `tuning` is given;
    `sequential` the same volumes as plain luxgi_ddgi_update calls per frame
    on the same GPU (skipped when `sequential` is false)."""
    import numpy as np
    import torch

    from luxgi_gb300 import DDGIBatch, DDGIVolume, DeviceScene, frame_rotation, _native as N

    dev_t = torch.device("cuda", torch.cuda.current_device())
    vols, scenes = [], []
    for w, host in zip(ws, hosts):
        dev = DeviceScene(host, w.volume.light_mode, device=str(dev_t))
        v = DDGIVolume(w.volume)
        v.bind_scene(dev)
        scenes.append(dev)
        vols.append(v)
    n = len(vols)
    pr = sum(w.volume.probes * w.volume.rays_per_probe for w in ws)
    rots = [np.stack([frame_rotation(seed + i, f) for i in range(n)]) for f in range(W + K)]
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev_t)

    def timed(step, frames):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in frames]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for (e0, e1), f in zip(ev, frames):
            flush.zero_()
            e0.record(stream)
            step(f)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
        if world > 1:
            t = torch.tensor([ms], device=dev_t)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    def seq_step(f):
        for v, r in zip(vols, rots[f]):
            v.update(r, stream)

    seq_ms = None
    if sequential:
        for f in range(W):
            seq_step(f)
        seq_ms = timed(seq_step, range(W, W + K))

    t0 = time.perf_counter()
    if tuning is None:
        batch = DDGIBatch(vols)
        tuning = batch.autotune(frames=3)
    else:
        batch = DDGIBatch(vols, tuning)
    tune_s = time.perf_counter() - t0

    def batch_step(f):
        batch.update(rots[f], stream)

    for f in range(W):
        batch_step(f)
    dev_index = torch.cuda.current_device()
    clocks = Clocks(dev_index)
    launches0 = N.ddgi().luxgi_launch_count()
    clocks.start()
    b_ms = timed(batch_step, range(W, W + K))
    clk = clocks.stop()
    launches = N.ddgi().luxgi_launch_count() - launches0
    value = world * pr * K / (b_ms / 1e3)
    seq_value = world * pr * K / (seq_ms / 1e3) if seq_ms is not None else None

    # e2e: rotations from the host, every volume's atlases read back to
    # pinned host memory each frame; the readback of frame k runs on a
    # second stream while frame k + 1 computes, and frame k + 2 (which
    # overwrites those ping-pong atlases) waits for it
    e2e = None
    if e2e_on:
        views = [v.atlases() for v in vols]
        hb = [[(torch.empty(i.shape, dtype=i.dtype).pin_memory(), torch.empty(d.shape, dtype=d.dtype).pin_memory())
               for i, d in views] for _ in range(2)]
        copy = torch.cuda.Stream(device=dev_t)

        def e2e_run(frames):
            back_done = [None, None]
            for f in frames:
                b = f % 2
                if back_done[b] is not None:
                    stream.wait_event(back_done[b])
                batch.update(rots[f], stream)
                done = torch.cuda.Event()
                done.record(stream)
                cur = [v.atlases() for v in vols]
                with torch.cuda.stream(copy):
                    copy.wait_event(done)
                    for (i, d), (ih, dh) in zip(cur, hb[b]):
                        ih.copy_(i, non_blocking=True)
                        dh.copy_(d, non_blocking=True)
                    back_done[b] = torch.cuda.Event()
                    back_done[b].record(copy)
            torch.cuda.synchronize()

        e2e_run(range(2))
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        e2e_run(range(W, W + K))
        te = time.perf_counter() - t0
        d2h = sum(ih.numel() * ih.element_size() + dh.numel() * dh.element_size() for ih, dh in hb[0])
        e2e = {"value": world * pr * K / te, "unit": "probe-rays/s", "h2d_bytes_per_step": 36 * n,
               "d2h_bytes_per_step": int(d2h)}
    out = {"value": value, "ms_per_step": b_ms / K, "probe_rays_per_frame": pr, "volumes": n,
           "sequential": None if seq_value is None else {
               "value": round(seq_value, 1), "ms_per_step": round(seq_ms / K, 4),
               "what": f"{n} luxgi_ddgi_update calls per frame, same volumes and GPU"},
           "speedup_vs_sequential": None if seq_value is None else round(value / seq_value, 3), "autotune": tuning,
           "autotune_s": round(tune_s, 2), "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    batch.close()
    for v in vols:
        v.close()
    del scenes, flush
    torch.cuda.empty_cache()
    return out


def batch_config(ws, world: int) -> dict:
    return {"workload": f"batch{len(ws)}_uneven_fp16sdf_tensorblend", "volumes": len(ws),
            "probe_rays_per_frame": sum(w.volume.probes * w.volume.rays_per_probe for w in ws),
            "probes": sum(w.volume.probes for w in ws),
            "rays_per_probe": sorted({w.volume.rays_per_probe for w in ws}),
            "sdf": sorted({w.scene.sdf_resolution for w in ws}),
            "atlas": sorted({w.scene.atlas_resolution for w in ws}), "parallelism": f"replicas{world}",
            "l2": "256 MB flush between frames (outside the events)"}


def run_batch(args, rank: int, world: int):
    """Batching form: 48 uneven volumes, each with its own FP16 SDF scene,
    tensor-core blend."""
    import torch

    from luxgi_gb300 import HostScene
    from luxgi_gb300.scene import batch_workloads

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    count = int(args.workload[len("batch"):] or 48)
    t0 = time.perf_counter()
    ws = batch_workloads(count)
    hosts = [HostScene(w.scene) for w in ws]
    setup_s = time.perf_counter() - t0
    tuning = json.loads(args.batch_tuning) if args.batch_tuning else None
    b = measure_batch(ws, hosts, args.steps, args.warmup, world, not args.no_e2e, seed=0x5EED + rank, tuning=tuning,
                      sequential=not args.no_sequential)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(b["value"], 1), "unit": "probe-rays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(b["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 march, fp16 tensor-core blend operands, fp32 accumulate",
        "data": "synthetic (seeded analytic scenes, one per volume)", "config": batch_config(ws, world),
        **{k: b[k] for k in ("sequential", "speedup_vs_sequential", "autotune", "autotune_s", "e2e",
                             "gpu_launches", "clocks")},
        "setup_s": round(setup_s, 2),
    }
    print(json.dumps(line), flush=True)


def batched_served_leg(args, plain_value: float) -> dict:
    """The batched and served forms, compared with the plain FP32
    single-volume form (`plain_value`): the batched form of 48 uneven
    volumes (FP16 SDFs, tensor-core blend) and a served run of 200 sessions
    over the same 48 workloads (session i runs workload i mod 48, with its
    own resident copy of the scene and atlases), Poisson arrivals at
    --serve-rate under a --serve-budget-gb budget."""
    from luxgi_gb300 import HostScene
    from luxgi_gb300.scene import batch_workloads

    t0 = time.perf_counter()
    ws = batch_workloads(48)
    hosts = [HostScene(w.scene) for w in ws]
    setup_s = time.perf_counter() - t0
    b = measure_batch(ws, hosts, max(args.steps, 10), 3, 1, e2e_on=True)
    sw = [ws[i % len(ws)] for i in range(200)]
    sh = [hosts[i % len(ws)] for i in range(200)]
    s = measure_serve(sw, sh, args.serve_rate, args.ns_serve_seconds, args.serve_budget_gb, warm_seconds=2.0)
    return {
        "batched": {"value": round(b["value"], 1), "unit": "probe-rays/s", "config": batch_config(ws, 1),
                    "ms_per_frame": round(b["ms_per_step"], 4), "frames": max(args.steps, 10),
                    **{k: b[k] for k in ("sequential", "speedup_vs_sequential", "autotune", "e2e", "gpu_launches",
                                         "clocks")}},
        "served": {**s, "config": {"sessions": 200, "workloads": f"the {len(ws)} batched workloads, session i runs "
                                   f"workload i mod {len(ws)} with its own resident scene and atlases",
                                   "rate_per_s": args.serve_rate, "seconds": args.ns_serve_seconds,
                                   "budget_gb": args.serve_budget_gb}},
        "ratio_batched_vs_plain": round(b["value"] / plain_value, 4),
        "target_ratio": 3.0,
        "setup_s": round(setup_s, 2),
    }


# ------------------------------------------------------- surface lighting
def run_surface(args, rank: int, world: int):
    """Surface-cache lighting form: the production scene (2048^2 atlas, 612
    tiles of 80^2 texels), the sun plus seeded point and spot lights, every
    object redrawn (the GI refresh frame of the reference's schedule).  A
    step is one luxgi_surface_light pass: emissive copy, then per light the
    SDF shadow march and the BRDF for every footprint texel the light's
    tile selection covers.  The metric is texel-light evaluations/s."""
    import ctypes

    import numpy as np
    import torch

    import oracle
    from luxgi_gb300 import DeviceScene, HostScene, _native as N
    from luxgi_gb300.scene import PRODUCTION
    from luxgi_gb300.surface import SurfaceLighting, light_array, scene_lights, select_tiles

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev_t = torch.device("cuda", local)
    nl = int(args.workload.rsplit("_l", 1)[1]) if "_l" in args.workload else 4
    w = PRODUCTION
    host = HostScene(w.scene)
    dev = DeviceScene(host, w.volume.light_mode, device=f"cuda:{local}")
    lights = scene_lights(host, nl, seed=7)
    tiles, masks = select_tiles(host, range(host.num_objects), lights)
    tl = (N.SurfaceTile * host.num_tiles).from_buffer_copy(host.tiles.tobytes())
    res = host.atlas
    sizes = np.array([(round(tl[int(t)].extends[2] * res) + 1) * (round(tl[int(t)].extends[3] * res) + 1)
                      for t in tiles], dtype=np.int64)
    texels = int(sizes.sum())
    evals = int(sum(int(sz) * bin(int(m)).count("1") for sz, m in zip(sizes, masks)))
    cam = tuple(host.surface_data.camera_pos)
    pass_ = SurfaceLighting(dev)
    K, W = args.steps, args.warmup
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev_t)
    t_dev = torch.as_tensor(tiles.view(np.int32)).to(dev_t)
    m_dev = torch.as_tensor(masks.view(np.int32)).to(dev_t)
    arr = light_array(lights)
    d = N.SurfaceLighting()
    d.lights = ctypes.cast(arr, ctypes.c_void_p)
    d.num_lights = len(lights)
    d.num_tiles = int(tiles.size)
    d.tiles = t_dev.data_ptr()
    d.light_masks = m_dev.data_ptr()
    d.camera_pos[:] = list(cam)
    d.shadow_bias = pass_.shadow_bias
    d.copy_emissive = 1
    d.max_steps = pass_.max_steps
    lib = N.ddgi()

    def step():
        N.check(lib.luxgi_surface_light(ctypes.byref(dev.sdf_desc), ctypes.byref(dev.surface_desc), ctypes.byref(d),
                                        dev.direct.data_ptr(), stream.cuda_stream), "surface_light")

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = Clocks(local)
    launches0 = lib.luxgi_launch_count()
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    torch.cuda.synchronize()
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        step()
        e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = lib.luxgi_launch_count() - launches0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    if world > 1:
        t = torch.tensor([ms], device=dev_t)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * evals * K / (ms / 1e3)

    # e2e: the light records and tile lists from host memory each step (the
    # reference uploads them as uniforms and vertex buffers per draw), the
    # lit atlas read back to pinned host memory
    e2e = None
    if not args.no_e2e:
        out_h = torch.empty(dev.direct.shape, dtype=dev.direct.dtype).pin_memory()
        t_h = torch.from_numpy(tiles.view(np.int32).copy()).pin_memory()
        m_h = torch.from_numpy(masks.view(np.int32).copy()).pin_memory()

        def e2e_step():
            t_dev.copy_(t_h, non_blocking=True)
            m_dev.copy_(m_h, non_blocking=True)
            step()
            out_h.copy_(dev.direct, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(K):
            e2e_step()
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        e2e = {"value": world * evals * K / te, "unit": "texel-light evaluations/s",
               "h2d_bytes_per_step": int(tiles.nbytes + masks.nbytes + 64 * len(lights)),
               "d2h_bytes_per_step": int(out_h.numel() * out_h.element_size())}
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu and world == 1:
        inp = oracle.HostInputs(host, w.volume.light_mode, mip=dev.mip.cpu().numpy(),
                                chunks=dev.chunks.cpu().numpy().view(np.uint32),
                                culled=dev.culled.cpu().numpy().view(np.uint32))
        n = 4
        while True:
            t0 = time.perf_counter()
            oracle.surface_light(inp, lights, tiles[:n], masks[:n], cam)
            el = time.perf_counter() - t0
            if el * 4 > args.cpu_seconds or n >= tiles.size:
                break
            n = min(int(tiles.size), max(n * 2, int(n * args.cpu_seconds / 2 / max(el, 1e-3))))
        ev_n = int(sum(int(sz) * bin(int(m)).count("1") for sz, m in zip(sizes[:n], masks[:n])))
        cpu = {"value": ev_n / el, "unit": "texel-light evaluations/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"{n} of {tiles.size} tiles, {ev_n} texel-light evaluations (oracle FP32, {el:.2f} s)"}
    line = {
        "metric": "surface-cache texel-light evaluations/s (emissive copy + SDF-shadowed BRDF per light)",
        "value": round(value, 1), "unit": "texel-light evaluations/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": round(ms / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 shading and march, fp16 atlas", "data": "synthetic (seeded analytic scene)",
        "config": {"workload": f"surface_light_production_atlas{res}_l{len(lights)}", "tiles": int(tiles.size),
                   "texels": texels, "texel_light_evaluations": evals, "lights": [int(L.type) for L in lights],
                   "shadow_max_steps": pass_.max_steps, "parallelism": f"replicas{world}",
                   "l2": "256 MB flush between passes (outside the events)"},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------ global SDF build
def sdf_build_scene(count: int = 96, seed: int = 5):
    """Baked mesh SDFs (box, sphere, pillar, slab; 32-64 texels a side as
    SDFBaker's 3-per-texel rule gives for metre-scale meshes, 3 mips) and
    `count` placed objects (rotated, scaled) spread over cascade 0 of the
    reference's default layout (giDistance 4000, scale 0.1: extents 40, 100,
    200, 400 with 4 cascades)."""
    import numpy as np

    from luxgi_gb300.sdf import MeshSDF, box_distance, sphere_distance, trs

    meshes = [MeshSDF.bake(box_distance((2.0, 1.0, 1.5)), (-2, -1, -1.5), (2, 1, 1.5), (48, 32, 40)),
              MeshSDF.bake(sphere_distance(1.5), (-1.5,) * 3, (1.5,) * 3, (40, 40, 40)),
              MeshSDF.bake(box_distance((0.4, 4.0, 0.4)), (-0.4, -4, -0.4), (0.4, 4, 0.4), (32, 64, 32)),
              MeshSDF.bake(box_distance((6.0, 0.25, 6.0)), (-6, -0.25, -6), (6, 0.25, 6), (64, 32, 64))]
    rng = np.random.default_rng(seed)
    objs = [(trs(rng.uniform(-36, 36, 3), rng.normal(size=3), rng.uniform(0, 6), rng.uniform(0.7, 2.5, 3)), i % 4)
            for i in range(count)]
    return meshes, objs


def run_sdf_build(args, rank: int, world: int):
    """Global SDF from placed mesh SDFs: a 256^3 x 4-cascade FP16 SDF (the
    reference's R16F) and its mip from 96 objects.  A step is one
    luxgi_sdf_build: clear, per cascade the host plan, the chunk
    rasterisation and the mip with its flood passes.  Metric: SDF voxels
    built per second."""
    import ctypes

    import numpy as np
    import torch

    import oracle
    from luxgi_gb300 import _native as N
    from luxgi_gb300.sdf import GlobalSDF, build_desc, objects_array, plan

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev_t = torch.device("cuda", local)
    meshes, objs = sdf_build_scene()
    d = build_desc(resolution=256, cascades=4, storage=N.STORAGE_FP16)
    g = GlobalSDF(d, device=f"cuda:{local}")
    descs = g.upload(meshes)
    md = (N.MeshSdf * len(descs))(*descs)
    ob = objects_array(objs)
    lib = N.ddgi()
    stream = torch.cuda.current_stream()
    voxels = d.resolution ** 3 * d.cascades
    chunk_voxels = sum(len(plan(d, meshes, objs, c)[2]) for c in range(d.cascades)) * 32 ** 3

    def step():
        N.check(lib.luxgi_sdf_build(ctypes.byref(d), md, len(descs), ob, len(objs), g.sdf.data_ptr(),
                                    g.mip.data_ptr(), g.tmp.data_ptr(), ctypes.byref(g.data), stream.cuda_stream),
                "sdf_build")

    K, W = args.steps, args.warmup
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev_t)
    for _ in range(W):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = Clocks(local)
    launches0 = lib.luxgi_launch_count()
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        step()
        e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = lib.luxgi_launch_count() - launches0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    if world > 1:
        t = torch.tensor([ms], device=dev_t)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * voxels * K / (ms / 1e3)
    # e2e: the public call with host inputs -- every mesh volume uploaded from
    # pinned memory, the build, the mip read back
    e2e = None
    if not args.no_e2e:
        pinned = [[torch.from_numpy(np.ascontiguousarray(v).view(np.int16).reshape(-1)).pin_memory() for v in m.mips]
                  for m in meshes]
        mip_h = torch.empty(g.mip.shape, dtype=g.mip.dtype).pin_memory()
        h2d = sum(p.numel() * 2 for vols in pinned for p in vols)

        def e2e_step():
            for vols, dvols in zip(pinned, g._meshes):
                for p, dv in zip(vols, dvols):
                    dv.copy_(p, non_blocking=True)
            step()
            mip_h.copy_(g.mip, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(K):
            e2e_step()
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        e2e = {"value": world * voxels * K / te, "unit": "SDF voxels/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(mip_h.numel() * mip_h.element_size())}
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu and world == 1:
        t0 = time.perf_counter()
        oracle.sdf_build(d, meshes, objs)
        el = time.perf_counter() - t0
        cpu = {"value": voxels / el, "unit": "SDF voxels/s", "cores": oracle.num_threads(), "kind": "port",
               "sample": f"one whole build (oracle FP32 rasterisation + mips, {el:.2f} s)"}
    line = {
        "metric": "global-SDF voxels built/s (rasterise placed mesh SDFs + cascade mips)", "value": round(value, 1),
        "unit": "SDF voxels/s", "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": round(ms / K, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 arithmetic, fp16 (R16F) SDF",
        "data": "synthetic (analytic shapes baked like SDFBaker)",
        "config": {"workload": "sdf_build_256x4_objects96", "resolution": d.resolution, "cascades": d.cascades,
                   "objects": len(objs), "meshes": len(meshes), "voxels": voxels, "chunk_voxels": chunk_voxels,
                   "parallelism": f"replicas{world}", "l2": "256 MB flush between builds (outside the events)"},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- serve
def measure_serve(ws, hosts, rate: float, seconds: float, budget_gb: float, warm_seconds: float = 3.0,
                  seed: int = 0x5EED) -> dict:
    """Sessions (one per workload) behind a server with a device-memory
    budget, Poisson arrivals at `rate` over all sessions for `seconds`.
    `value` is the probe-rays/s the server completed (submit of the first
    request to completion of the last); latency is submit to completion
    seen by the host."""
    import torch

    from luxgi_gb300 import Server

    budget = int(budget_gb * (1 << 30))
    srv = Server(budget, max_group=64, max_inflight=3)
    ids = [srv.add_session(w.volume, h) for w, h in zip(ws, hosts)]
    t0 = time.perf_counter()
    for sid in ids:
        try:
            srv.touch(sid)
        except Exception:
            break                        # budget full: the rest are admitted on demand
    admit_s = time.perf_counter() - t0
    # warm-up: every session's first frames, untimed
    srv.run_poisson(ids, rate=rate, seconds=min(warm_seconds, seconds), seed=seed)
    srv.stats(reset=True)
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    srv.run_poisson(ids, rate=rate, seconds=seconds, seed=seed + 1)
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    value = st["probe_rays"] / st["wall_s"] if st["wall_s"] > 0 else 0.0
    return {"value": round(value, 1), "unit": "probe-rays/s",
            "latency_ms": {"p50": round(st["latency_ms_p50"], 3), "p95": round(st["latency_ms_p95"], 3),
                           "p99": round(st["latency_ms_p99"], 3), "mean": round(st["latency_ms_mean"], 3),
                           "max": round(st["latency_ms_max"], 3)},
            "served": {k: st[k] for k in ("submitted", "completed", "admissions", "evictions", "rejected", "groups",
                                          "max_overlap", "resident_sessions", "peak_resident_bytes")},
            "mean_group": round(st["mean_group"], 2), "wall_s": round(st["wall_s"], 3),
            "admission_s": round(admit_s, 2), "clocks": clk}


def run_serve(args, rank: int, world: int):
    """Serving form: sessions with batching-form volumes and scenes, Poisson
    arrivals, admission by a device-memory budget with LRU eviction."""
    import torch

    from luxgi_gb300 import HostScene
    from luxgi_gb300.scene import batch_workloads

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    count = int(args.workload[len("serve"):] or 200)
    t0 = time.perf_counter()
    ws = batch_workloads(count, seed=0xC0FFEE + 5)
    hosts = [HostScene(w.scene) for w in ws]
    gen_s = time.perf_counter() - t0
    s = measure_serve(ws, hosts, args.serve_rate, args.serve_seconds, args.serve_budget_gb, seed=0x5EED + rank)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(s["value"] * world, 1), "unit": "probe-rays/s", "n_gpus": world,
        "steps": int(s["served"]["completed"]), "warmup": 0, "ms_per_step": s["latency_ms"]["mean"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 march, fp16 tensor-core blend operands, fp32 accumulate",
        "data": "synthetic (seeded analytic scenes, one per session)",
        "config": {"workload": f"serve{count}_poisson{int(args.serve_rate)}_budget{args.serve_budget_gb:g}GB",
                   "sessions": count, "rate_per_s": args.serve_rate, "seconds": args.serve_seconds,
                   "budget_bytes": int(args.serve_budget_gb * (1 << 30)), "max_group": 64, "streams": 3,
                   "parallelism": f"replicas{world}"},
        "latency_ms": s["latency_ms"], "served": s["served"], "mean_group": s["mean_group"], "wall_s": s["wall_s"],
        "setup_s": {"scenes": round(gen_s, 2), "admission": s["admission_s"]},
        "e2e": {"value": round(s["value"] * world, 1), "unit": "probe-rays/s", "h2d_bytes_per_step": 36,
                "d2h_bytes_per_step": 0},
        "clocks": s["clocks"],
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- reference
def run_reference(args, rank: int, world: int):
    """The CPU restatement of the reference shaders on the host cores, on
    the GPU arm's workload: each step is one whole frame of the volume
    (every probe and ray; trace with the per-hit bounce from the arm's own
    previous frame, blend, border), a bounded sample of the GPU arm's
    16-frame step.  Loads only the oracle and the scene generator."""
    if rank != 0:
        return
    import oracle
    from luxgi_gb300.scene import HostScene, WORKLOADS

    if world > 1:
        # torchrun sets OMP_NUM_THREADS=1 for every rank; rank 0 alone runs
        # here and takes every host core
        oracle.set_threads(os.cpu_count() or 1)
    w = WORKLOADS[args.workload]
    v = w.volume
    host = HostScene(w.scene)
    vd = v.desc(derive=oracle.derive_uniform)
    inp = oracle.HostInputs(host, v.light_mode)
    R = v.rays_per_probe
    fp16 = v.storage == 1
    rots = [oracle.frame_rotation(0x5EED, f) for f in range(args.warmup + args.steps)]
    state = {"irr": None, "dist": None, "frames": 0}

    def step(rot):
        f = state["frames"]
        rays, _ = oracle.trace(vd, inp, rot, f, state["irr"], state["dist"], precision=0, want_info=False)
        state["irr"], state["dist"] = oracle.blend(vd, oracle.ray_dirs(rot, R, 0, fp16), rays, state["irr"],
                                                   state["dist"], first=(f == 0), precision=0)
        state["frames"] = f + 1

    for f in range(args.warmup):
        step(rots[f])
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(rots[args.warmup + k])
    dt = time.perf_counter() - t0
    value = v.probes * R * args.steps / dt
    cores = oracle.num_threads()
    sample = (f"one whole frame per step ({v.probes} probes x {R} rays, per-hit bounce from the previous frame, "
              f"blend and border) of {w.name}, of the GPU arm's {args.frames_per_step}-frame steps; "
              "CPU restatement of the reference shaders, FP32")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": "probe-rays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded analytic scene)", "config": workload_config(w, world, args.frames_per_step),
            "cpu_baseline": {"value": round(value, 1), "unit": "probe-rays/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 1), "unit": "probe-rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload.startswith("batch"):
        run_batch(args, rank, world)
    elif args.workload.startswith("sdf_build"):
        run_sdf_build(args, rank, world)
    elif args.workload.startswith("surface_light"):
        run_surface(args, rank, world)
    elif args.workload.startswith("serve"):
        run_serve(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
