"""Benchmark of the render-and-encode hot path (one JSON line on rank 0).

Workload (the plain GPU drop-in configuration): the seeded scene (seed 0,
16 levels x 2^19 entries), one 1920x1080 mono view per request, 100 poses
uniform on the radius-1.5 sphere looking at the cube centre, 90 deg
horizontal FOV.  A step is one request: ray generation + march + composite
into RGB/depth, RGB24 quantisation, RGB24->YUV420P and depth packing to
uint16 mm, all on the device with the scene resident.  L2 is flushed (a
256 MiB write) before every timed step, outside the timed interval.

  value   Mrays/s (all pixels, misses included) of the device step, from
          CUDA events on the launching stream, summed over K steps, max over
          ranks, times the number of ranks (weak scaling: each rank renders
          its own requests).
  e2e     the same metric through nes_render_yuv (pose in host memory, YUV
          planes + packed depth copied back to pinned host buffers inside
          the timed region), plus p50/p99 pose->YUV latency.

--impl reference times the plain FP32 CPU render of the path (oracle/, all
host threads) on bounded random pixel samples of the same requests: the
reference's renderer is an external project and its swscale/libavcodec
dependencies are not installed, so the CPU restatement is the CPU arm.  That
arm loads only the oracle's library (poses and focal length are computed in
Python), and both arms print the same `config`.  The default run's
cpu_baseline times the same FP32 CPU render and the FP64 oracle (the
checker) on one pixel sample, with the parity of the tensor-core render
against the FP64 oracle on those pixels.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "ngp-encode-server_gb300"))

W, H, FOV, NPOSES, RADIUS = 1920, 1080, 90.0, 100, 1.5
FLOP_PER_SAMPLE = 18688          # 2 x 9,344 MLP multiply-adds
GATHER_BYTES = {"fp32": 1024, "fp16": 512}  # 16 levels x 8 corners x 2 features
# dram__bytes_read.sum + dram__bytes_write.sum of one full 1920x1080 march
# launch: the tensor-core march with records of levels 0..12 from a 1-pass
# ncu capture of `bench.py --steps 1 --warmup 1 --precision tc --no-extras
# --no-cpu-baseline --e2e-steps 1` (49.23 GB + 17.7 MB), the FP32 march from
# a capture of the same command with --precision fp32.
DRAM_BYTES_PER_LAUNCH = {"fp16": 49.23e9 + 17.72e6, "fp32": 73.651e6 + 7.437e6}
DRAM_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, one full 1920x1080 launch (1 pass)"
# The tensor-core march's binding unit is the L1 data pipe (ncu names it as
# the limiter: LSU wavefronts at 66 % of peak, long-scoreboard stalls
# dominant).  Its gather term is stated against that pipe: L1 LSU wavefronts
# per sample of a full 1920x1080 launch with records of levels 0..12 (1-pass
# ncu capture of the --precision tc command above: l1tex__data_pipe_lsu_
# wavefronts.sum / the launch's samples), and the pipe's peak of one wavefront
# per SM per cycle (l1tex__data_pipe_lsu_wavefronts.sum.peak_sustained = the
# SM count).
L1_WF_PER_SAMPLE = {("fp16", 13): 5250204369 / 285031892}  # 18.42
L1_WF_PER_SM_CYCLE = 1.0
L1_WF_SOURCE = ("ncu l1tex__data_pipe_lsu_wavefronts.sum of one full 1920x1080 launch (1 pass) / its samples; "
                "peak = 1 wavefront per SM per cycle x SMs x the median SM clock sampled during the timed steps")
WORKLOAD = "mono 1920x1080, 100 poses on r=1.5 sphere, 90 deg FOV, seed 0, T=2^19"
L2_RULE = "flushed (256 MiB write) before every timed GPU step"
REC_GB = {10: 1.30, 13: 24.05}  # per-cell corner records of a tensor-core context (32 B per cell)


def bench_config():
    """The `config` both arms print (identical, so their lines compare)."""
    return {"workload": WORKLOAD, "l2": L2_RULE, "parallelism": "replicas"}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["auto", "fp32", "tc"], default="auto")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--no-extras", action="store_true", help="skip the stereo and serving sections")
    p.add_argument("--serve-seconds", type=float, default=3.0)
    p.add_argument("--stereo-poses", type=int, default=200, help="poses of the stereo precision-form section")
    p.add_argument("--train-steps", type=int, default=20, help="refit steps timed in the training section")
    p.add_argument("--train-batch", type=int, default=1 << 18, help="rays per refit step")
    p.add_argument("--section", choices=["all", "training"], default="all",
                   help="'training' prints only the refit section (for profiling captures)")
    p.add_argument("--record-levels", type=int, default=13, choices=[10, 13],
                   help="tensor-core contexts: levels kept as per-cell records (10 only for small profiling captures)")
    p.add_argument("--width", type=int, default=1920, help="smaller sizes only for profiling captures")
    p.add_argument("--height", type=int, default=1080)
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def job_time_ms(local_ms, world, device="cpu"):
    """The whole job's timed region: the maximum of every rank's (an
    all-reduce over the initialised process group when world > 1)."""
    if world <= 1:
        return float(local_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mrays(world, pixels_per_step, steps, job_ms):
    """Whole-job Mrays/s: every rank renders its own requests (weak scaling)."""
    return world * pixels_per_step * steps / (job_ms / 1e3) / 1e6


def rank_poses(rank):
    """The request poses rank `rank` serves (each rank its own seeded set)."""
    import nes
    return nes.shell_poses(rank, NPOSES, RADIUS, RADIUS)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.lines, self.proc = device, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
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
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) != 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return pk["hbm_gbs"], pk["bf16_tflops"], pk["bf16_tflops_sustained"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, 1700.0, "fallback"


def cpu_sample(poses, steps_px, seed, fp32=True):
    """Times the CPU render (plain FP32, or the FP64 oracle) on random pixel
    subsets; returns (Mrays/s, s, px, threads)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import numpy as np
    import oracle
    scene = oracle.Scene(0, 19)
    f = oracle.focal_from_fov(W, FOV)
    rng = np.random.default_rng(seed)
    threads = os.cpu_count() or 1
    total_px, total_s = 0, 0.0
    for i, npx in enumerate(steps_px):
        pix = rng.choice(W * H, npx, replace=False).astype(np.int32)
        render = scene.render_f32 if fp32 else scene.render
        t0 = time.perf_counter()
        render(poses[i % len(poses)], W, H, f, pixels=pix, nthreads=threads)
        total_s += time.perf_counter() - t0
        total_px += npx
    return total_px / total_s / 1e6, total_s, total_px, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # Poses are pure Python (nes.shell_poses loads no library); the focal
    # length comes from the oracle: this arm maps only the oracle's library.
    import nes
    poses = nes.shell_poses(0, NPOSES, RADIUS, RADIUS)
    per_step = max(2048, (W * H) // 256)
    cpu_sample(poses, [per_step // 4] * max(1, args.warmup), 99)  # warm-up
    mrays, secs, px, threads = cpu_sample(poses, [per_step] * args.steps, 1)
    line = {"metric": "Mrays/s (pose->YUV render, all pixels)", "value": round(mrays, 6), "unit": "Mrays/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and poses)",
            "config": bench_config(),
            "cpu_baseline": {"value": round(mrays, 6), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": "plain FP32 CPU render (oracle/, pthreads) of %d random pixels of a "
                                       "1920x1080 request per step (misses included in proportion), %d steps; "
                                       "Mrays/s = sampled pixels / CPU time" % (per_step, args.steps)},
            "e2e": {"value": round(mrays, 6), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import nes
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)  # a real stream: NULL would mean the library's own
    torch.cuda.set_stream(stream)
    precisions = {"fp32": [nes.PREC_FP32], "tc": [nes.PREC_FP16_TC],
                  "auto": [nes.PREC_FP16_TC, nes.PREC_FP32]}[args.precision]

    poses = rank_poses(rank)
    focal = nes.focal_from_fov(W, FOV)
    views = [nes.make_view(m, W, H, focal) for m in poses]
    ls = nes.linesizes(W)
    ch = (H + 1) // 2
    rgb = torch.empty(W * H * 3, device=dev)
    dep = torch.empty(W * H, device=dev)
    rgb8 = torch.empty(W * H * 3, dtype=torch.uint8, device=dev)
    yuv = torch.empty(ls[0] * H + (ls[1] + ls[2]) * ch, dtype=torch.uint8, device=dev)
    dmm = torch.empty(W * H, dtype=torch.int16, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    lib = nes.load()
    yp, up, vp = yuv.data_ptr(), yuv.data_ptr() + ls[0] * H, yuv.data_ptr() + ls[0] * H + ls[1] * ch
    sptr = stream.cuda_stream

    results, renderer_used = {}, None
    for prec in precisions:
        try:
            r = nes.Renderer(precision=prec, max_pixels=W * H, device=local, record_levels=args.record_levels)
        except nes.NesError as e:
            results[prec] = {"error": str(e)}
            continue
        r.set_profiling(True)

        def step(i):
            r.render_views([views[i % NPOSES]], [rgb.data_ptr()], [dep.data_ptr()], sptr)
            nes.check(lib.nes_rgb_to_rgb24(rgb.data_ptr(), W * H * 3, rgb8.data_ptr(), sptr), "rgb24")
            nes.rgb24_to_yuv420p(rgb8.data_ptr(), W, H, W * 3, yp, up, vp, ls, sptr)
            nes.depth_pack_u16mm(dep.data_ptr(), W * H, dmm.data_ptr(), sptr)

        try:
            for i in range(args.warmup):
                flush.zero_()
                step(i)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            march_ms, raygen_ms, samples = [], [], []
            with ClockSampler(local) as clk:
                for i in range(args.steps):
                    flush.zero_()
                    ev[i][0].record(stream)
                    step(i)
                    ev[i][1].record(stream)
                    rg, mm = r.last_timings()
                    raygen_ms.append(rg)
                    march_ms.append(mm)
                    samples.append(r.last_sample_count())
                torch.cuda.synchronize()
            step_ms = [a.elapsed_time(b) for a, b in ev]
            total_ms = job_time_ms(sum(step_ms), world, dev)
            res = {"total_ms": total_ms, "ms_per_step": total_ms / args.steps,
                   "mrays": job_mrays(world, W * H, args.steps, total_ms),
                   "march_ms": statistics.mean(march_ms), "raygen_ms": statistics.mean(raygen_ms),
                   "samples_per_step": statistics.mean(samples), "clocks": clk.summary(),
                   # hitting rays of the last timed request (a miss has depth 0)
                   "rays_per_step": int((dep > 0).sum().item())}
            if prec == nes.PREC_FP16_TC and rank == 0:
                # The replay covers the timed steps' poses in turn, one per replay.
                res["gather"] = measure_gather_ceilings(r, [views[0]], flush, stream, dev)
                res["gather"]["replay_pose"] = 0
                res["march_ms_pose0"] = march_ms[0]
                res["samples_pose0"] = samples[0]

            # End to end through the host-buffer C-ABI call.
            ke = args.e2e_steps or args.steps
            hy = torch.empty(ls[0] * H, dtype=torch.uint8).pin_memory()
            hu = torch.empty(ls[1] * ch, dtype=torch.uint8).pin_memory()
            hv = torch.empty(ls[2] * ch, dtype=torch.uint8).pin_memory()
            hd = torch.empty(W * H, dtype=torch.int16).pin_memory()
            r.set_profiling(False)
            for i in range(args.warmup):
                r.render_yuv(views[i % NPOSES], hy.data_ptr(), hu.data_ptr(), hv.data_ptr(), ls, hd.data_ptr())
            lat = []
            for i in range(ke):
                flush.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r.render_yuv(views[i % NPOSES], hy.data_ptr(), hu.data_ptr(), hv.data_ptr(), ls, hd.data_ptr())
                lat.append(time.perf_counter() - t0)
            lat_sorted = sorted(lat)
            res["e2e"] = {"mrays": world * W * H * ke / sum(lat) / 1e6,
                          "p50_ms": 1e3 * lat_sorted[len(lat) // 2],
                          "p99_ms": 1e3 * lat_sorted[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)],
                          "h2d": 48 + 8, "d2h": hy.numel() + hu.numel() + hv.numel() + 2 * hd.numel()}
            results[prec] = res
            if renderer_used is None:
                renderer_used = prec
        finally:
            r.close()

    if rank != 0:
        return
    if renderer_used is None:
        print(json.dumps({"metric": "Mrays/s (pose->YUV render, all pixels)", "value": None,
                          "error": {str(k): v for k, v in results.items()}}), flush=True)
        sys.exit(1)
    head = results[renderer_used]
    hbm, tf_burst, tf_sust, src = load_peaks()
    kind = "fp16" if renderer_used == nes.PREC_FP16_TC else "fp32"
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roof = roofline_terms(head, kind, tf_sust, src, hbm, sms, args.record_levels)
    line = {
        "metric": "Mrays/s (pose->YUV render, all pixels)", "value": round(head["mrays"], 3), "unit": "Mrays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(head["ms_per_step"], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": kind, "data": "synthetic (seeded scene and poses)",
        "config": bench_config(),
        "precision": "FP16 table + FP16 MLP on tcgen05, FP32 accumulate and compositing; hash-grid levels 0..%d "
                     "also kept as per-cell corner records (%.1f GB)" % (args.record_levels - 1,
                                                                         REC_GB[args.record_levels])
                     if kind == "fp16" else "FP32 CUDA cores",
        "e2e": {"value": round(head["e2e"]["mrays"], 3), "unit": "Mrays/s",
                "h2d_bytes_per_step": head["e2e"]["h2d"], "d2h_bytes_per_step": head["e2e"]["d2h"],
                "p50_ms": round(head["e2e"]["p50_ms"], 3), "p99_ms": round(head["e2e"]["p99_ms"], 3)},
        "gpu_launches": 5 * args.steps,
        "roofline": roof,
        "clocks": head["clocks"],
        "paths": {("fp16_tc" if k == nes.PREC_FP16_TC else "fp32"):
                  ({"mrays": round(v["mrays"], 3), "ms_per_step": round(v["ms_per_step"], 3),
                    "e2e_mrays": round(v["e2e"]["mrays"], 3), "p99_ms": round(v["e2e"]["p99_ms"], 3)}
                   if "mrays" in v else v) for k, v in results.items()},
    }
    if world == 1 and not args.no_extras:
        line["stereo"] = run_stereo(dev, nposes=args.stereo_poses)
        line["serving"] = run_serving(dev, args.serve_seconds)
        line["serving_delay_bounded"] = run_serving(dev, args.serve_seconds, max_queue_ms=100.0)
        line["glue"] = run_glue(dev, {"hbm_gbs": hbm})
        if args.train_steps > 0:
            line["training"] = run_training(dev, args.train_steps, batch=args.train_batch)
    if not args.no_cpu_baseline:
        per = (W * H) // 32
        cb = cpu_baseline_with_parity(dev, poses[0], per)
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)


def roofline_terms(head, kind, tf_sust, src, hbm, sms, rec_levels):
    """The march's two roofline terms per launch: the MLP contraction
    (18,688 FLOP per sample) against the measured bf16 tensor peak, and the
    hash-table gathers (512 B per sample) against the unit that carries
    them, the L1 data pipe: its wavefronts per sample (ncu) x samples / the
    launch's CUDA-event time, over one wavefront per SM per cycle at the SM
    clock sampled during the timed steps.  `bound` names the term with the
    larger floor; achieved / peak / frac are that term's (the gather term in
    algorithmic GB/s: its peak is the gather rate at which the L1 pipe would
    be saturated)."""
    ms, n = head["march_ms"], head["samples_per_step"]
    tflops = n * FLOP_PER_SAMPLE / (ms / 1e3) / 1e12
    t_tensor = n * FLOP_PER_SAMPLE / (tf_sust * 1e12) * 1e3
    out = {"kernel": "march", "march_ms": round(ms, 3), "raygen_ms": round(head["raygen_ms"], 4),
           "samples_per_step": int(n), "msamples_per_s": round(n / (ms / 1e3) / 1e6, 1),
           "frames_per_s": round(1e3 / head["ms_per_step"], 2),
           "tensor": {"achieved": round(tflops, 3), "peak": tf_sust, "unit": "TFLOP/s",
                      "frac": round(tflops / tf_sust, 5), "floor_ms": round(t_tensor, 3),
                      "peak_source": src + " bf16 sustained (MEASURED_PEAKS.json)",
                      "per_unit": "18,688 FLOP per sample (2 x 9,344 MLP multiply-adds)"},
           "tensor_frac": round(tflops / tf_sust, 5)}
    gbytes = n * GATHER_BYTES[kind]
    gbs = gbytes / (ms / 1e3) / 1e9
    out["gather_achieved_gbs"] = round(gbs, 1)
    wf = L1_WF_PER_SAMPLE.get((kind, rec_levels)) if (W, H) == (1920, 1080) else None
    clk = head["clocks"].get("sm_mhz") or head["clocks"].get("sm_max_mhz")
    bound = "tensor"
    if wf and clk:
        ach_wf = wf * n / (ms / 1e3)
        peak_wf = sms * clk * 1e6 * L1_WF_PER_SM_CYCLE
        frac = ach_wf / peak_wf
        out["gather"] = {"achieved": round(gbs, 1), "peak": round(gbs / frac, 1), "unit": "GB/s",
                         "frac": round(frac, 4), "floor_ms": round(ms * frac, 3),
                         "unit_limit": "L1 data pipe (LSU wavefronts)",
                         "l1_wavefronts_per_sample": wf, "l1_wavefronts_per_s": round(ach_wf / 1e9, 2),
                         "l1_wavefront_peak_per_s": round(peak_wf / 1e9, 2), "rate_unit": "G wavefronts/s",
                         "sm_mhz": clk, "peak_source": L1_WF_SOURCE,
                         "per_unit": "512 B per sample (16 levels x 8 corners x 2 FP16 features)"}
        out["gather_frac"] = out["gather"]["frac"]
        if ms * frac > t_tensor:
            bound = "gather"
    g = head.get("gather")
    if g:
        # Supporting measurements: the same load stream replayed alone, and
        # the hardware's random-gather rate (no locality).
        out["gather_probes"] = dict(g)
        out["gather_probes"]["replay_ms_scaled"] = round(g["replay_ms"] * n / head["samples_pose0"], 3)
    term = out["gather"] if bound == "gather" else out["tensor"]
    out.update({"bound": bound, "achieved": term["achieved"], "peak": term["peak"], "unit": term["unit"],
                "frac": term["frac"]})
    traffic = DRAM_BYTES_PER_LAUNCH.get(kind) if (W, H) == (1920, 1080) and rec_levels == 13 else None
    rays = head.get("rays_per_step") or W * H
    algo = (16 << 19) * (2 if kind == "fp16" else 4) * 2 + rays * 32 + W * H * 16
    out.update({"traffic": traffic, "traffic_source": DRAM_SOURCE if traffic else None,
                "algorithmic_hbm_bytes": int(algo),
                "traffic_ratio": round(traffic / algo, 1) if traffic else None,
                "traffic_note": "algorithmic HBM bytes: the table read once, the ray list (32 B per hitting ray) "
                                "and the FP32 RGB + depth written (16 B per pixel).  The measured excess is "
                                "by design: the per-cell corner records of levels 7-12 (copies of table "
                                "entries, 24 GB) are read from HBM, one 32-byte sector per level and sample "
                                "(~2 TB/s, under a third of HBM bandwidth; levels 10-12 with an L2 "
                                "evict-first policy), in place of eight scattered L1/L2 gathers each; with "
                                "records of levels 0-9 only (2.8 GB per launch) the march is 6-8 % slower",
                "hbm_peak_gbs": hbm,
                "limiter": "hash-table gathers through L1: L1 data pipe at 66% of its wavefront rate, "
                           "long-scoreboard stalls dominant, tensor pipe 10%, DRAM 3% (ncu full sections, "
                           "960x540 request, records of levels 0-9)"})
    return out


def measure_gather_ceilings(r, views, flush, stream, dev, reps=5):
    """Gather probes beside the march's roofline: the march's own load
    stream replayed without arithmetic on the same views
    (nes_probe_gather_replay, 512 ray slots per SM, L2 flushed before each
    replay, median), and the random-gather rates of 4-, 16- and 32-byte loads
    over an L2-resident 32 MiB table (nes_probe_gather, CUDA events, median of
    `reps` launches)."""
    import ctypes
    import torch
    import nes
    lib = nes.load()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sink = torch.empty(max(sms * 512, sms * 2048), dtype=torch.int32, device=dev)
    arr = (nes.NesView * len(views))(*views)
    ms = ctypes.c_float(0)
    rep = []
    for i in range(reps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        nes.check(lib.nes_probe_gather_replay(r.h, arr, len(views), 512, sink.data_ptr(), sink.numel(),
                                              ctypes.byref(ms)), "nes_probe_gather_replay")
        if i:
            rep.append(ms.value)
    out = {"replay_ms": round(statistics.median(rep), 3),
           "replay_note": "the march's load stream alone (same rays, addresses and per-tile pacing, no "
                          "interpolation, MLP or compositing): it runs no faster than the march, which "
                          "overlaps its gathers with the MLP warps' work"}
    table = torch.randint(0, 1 << 30, ((32 << 20) // 4,), dtype=torch.int32, device=dev)
    threads, loads = sms * 2048, 256
    for nbytes in (4, 16, 32):
        t = []
        for i in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            nes.check(lib.nes_probe_gather(table.data_ptr(), table.numel() * 4, nbytes, loads, threads,
                                           sink.data_ptr(), ctypes.c_void_p(stream.cuda_stream)), "nes_probe_gather")
            b.record(stream)
            b.synchronize()
            if i:
                t.append(a.elapsed_time(b))
        sec = statistics.median(t) / 1e3
        out["random_%dB" % nbytes] = {"gbs": round(threads * loads * nbytes / sec / 1e9, 1),
                                      "gloads_per_s": round(threads * loads / sec / 1e9, 2)}
    out["random_note"] = ("uniformly random loads over a 32 MiB L2-resident table, %d threads x %d loads, "
                          "no locality: the hardware's gather rate" % (threads, loads))
    return out


def cpu_baseline_with_parity(dev, pose, npx):
    """The FP64 oracle timed on a random pixel sample of one request; the same
    pixels of the tensor-core render are compared against it (PSNR, depth)."""
    import numpy as np
    import torch
    import nes
    f = nes.focal_from_fov(W, FOV)
    with nes.Renderer(precision=nes.PREC_FP16_TC, max_pixels=W * H, device=dev.index) as r:
        rgb = torch.empty(W * H * 3, device=dev)
        dep = torch.empty(W * H, device=dev)
        r.render_views([nes.make_view(pose, W, H, f)], [rgb.data_ptr()], [dep.data_ptr()])
        torch.cuda.synchronize()
        g_rgb = rgb.cpu().numpy().reshape(-1, 3)
        g_dep = dep.cpu().numpy()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    scene = oracle.Scene(0, 19)
    pix = np.random.default_rng(7).choice(W * H, npx, replace=False).astype(np.int32)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    scene.render_f32(pose, W, H, f, pixels=pix, nthreads=threads)
    secs32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    orgb, odep, _ = scene.render(pose, W, H, f, pixels=pix, nthreads=threads)
    secs = time.perf_counter() - t0
    mse = float(np.mean((g_rgb[pix] - orgb) ** 2))
    return {"value": round(npx / secs32 / 1e6, 6), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": "%d random pixels of one 1920x1080 request, plain FP32 CPU render (%.1f s)" % (npx, secs32),
            "fp64_oracle": {"value": round(npx / secs / 1e6, 6), "unit": "Mrays/s", "seconds": round(secs, 2)},
            "parity_fp16_tc": {"psnr_db": round(10 * math.log10(1.0 / mse), 2) if mse > 0 else None,
                               "max_abs_depth_err": float(np.abs(g_dep[pix] - odep).max()), "pixels": npx,
                               "against": "FP64 oracle"}}


def _pct(vals, q):
    v = sorted(vals)
    return v[min(len(v) - 1, max(0, int(math.ceil(q * len(v))) - 1))]


def run_stereo(dev, nposes=200, parity_px=512, sweep_poses=20, log2_tables=(14, 19, 22)):
    """Precision form: stereo 2x1920x1832 per request (100 deg FOV, IPD
    0.063), nposes poses on the r = 1.2..2.0 shell, FP16 tcgen05, T = 2^19.

      device  CUDA events around raygen + march + RGB24 + YUV420P + depth
              packing of both eyes (pose already on the host);
      host    pose -> YUV420P + uint16 depth of both eyes in pinned host
              memory through nes_render_yuv_views (host clock, D2H inside);
      parity  for EVERY pose, `parity_px` seeded random pixels per eye of
              the tensor-core render against the FP64 oracle: PSNR and max
              |depth error| (scene extent 1);
      sweep   T = 2^14 / 2^19 / 2^22: device Mrays/s over sweep_poses poses
              and the parity of one pose per table size."""
    import numpy as np
    import torch
    import nes
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    SW, SH = 1920, 1832
    px_eye = SW * SH
    f = nes.focal_from_fov(SW, 100.0)
    poses = nes.shell_poses(0, nposes, 1.2, 2.0)
    ls = nes.linesizes(SW)
    ch = (SH + 1) // 2
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    lib = nes.load()
    bufs = []
    for _ in range(2):
        bufs.append(dict(rgb=torch.empty(px_eye * 3, device=dev), dep=torch.empty(px_eye, device=dev),
                         rgb8=torch.empty(px_eye * 3, dtype=torch.uint8, device=dev),
                         yuv=torch.empty(ls[0] * SH + 2 * ls[1] * ch, dtype=torch.uint8, device=dev),
                         dmm=torch.empty(px_eye, dtype=torch.int16, device=dev)))
    host = [[torch.empty(n, dtype=torch.uint8).pin_memory() for n in (ls[0] * SH, ls[1] * ch, ls[2] * ch)] +
            [torch.empty(px_eye, dtype=torch.int16).pin_memory()] for _ in range(2)]
    rng = np.random.default_rng(2024)
    pix_sets = [[np.sort(rng.choice(px_eye, parity_px, replace=False)).astype(np.int64) for _ in range(2)]
                for _ in range(nposes)]

    def eyes_of(i, focal=f):
        return [nes.make_view(m, SW, SH, focal) for m in nes.stereo_pair(poses[i % len(poses)], 0.063)]

    def device_request(r, i):
        r.render_views(eyes_of(i), [b["rgb"].data_ptr() for b in bufs], [b["dep"].data_ptr() for b in bufs], sptr)
        for b in bufs:
            y = b["yuv"].data_ptr()
            nes.check(lib.nes_rgb_to_rgb24(b["rgb"].data_ptr(), px_eye * 3, b["rgb8"].data_ptr(), sptr), "rgb24")
            nes.rgb24_to_yuv420p(b["rgb8"].data_ptr(), SW, SH, SW * 3, y, y + ls[0] * SH,
                                 y + ls[0] * SH + ls[1] * ch, ls, sptr)
            nes.depth_pack_u16mm(b["dep"].data_ptr(), px_eye, b["dmm"].data_ptr(), sptr)

    def timed_device(r, n, collect=None):
        ms, samples = [], []
        for i in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            device_request(r, i)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
            samples.append(r.last_sample_count())
            if collect is not None:
                collect(i)
        return ms, samples

    gpu_px = []  # per pose: (rgb [2, parity_px, 3], depth [2, parity_px]) of the device render

    def grab(i):
        rr, dd = [], []
        for e, b in enumerate(bufs):
            idx = torch.from_numpy(pix_sets[i][e]).to(dev)
            rr.append(b["rgb"].view(-1, 3).index_select(0, idx).cpu().numpy())
            dd.append(b["dep"].index_select(0, idx).cpu().numpy())
        gpu_px.append((rr, dd))

    out = {"workload": "stereo 2x1920x1832 per request, 100 deg FOV, IPD 0.063, %d poses on r=1.2..2.0 shell, "
                       "FP16 tcgen05, seed 0" % nposes}
    with nes.Renderer(precision=nes.PREC_FP16_TC, max_pixels=2 * px_eye, device=dev.index) as r:
        for i in range(3):
            device_request(r, i)
        torch.cuda.synchronize()
        ms, samples = timed_device(r, nposes, collect=grab)
        # Pose -> YUV on the host (D2H of both eyes' planes and depth inside).
        hy, hu, hv, hd = ([h[k].data_ptr() for h in host] for k in range(4))
        for i in range(3):
            r.render_yuv_views(eyes_of(i), hy, hu, hv, ls, hd)
        lat = []
        for i in range(nposes):
            t0 = time.perf_counter()
            r.render_yuv_views(eyes_of(i), hy, hu, hv, ls, hd)
            lat.append(1e3 * (time.perf_counter() - t0))
    out["device"] = {"requests": nposes, "p50_ms": round(_pct(ms, 0.5), 3), "p99_ms": round(_pct(ms, 0.99), 3),
                     "mrays": round(2 * px_eye * nposes / (sum(ms) / 1e3) / 1e6, 3),
                     "samples_per_pixel": round(statistics.mean(samples) / (2 * px_eye), 2),
                     "timing": "CUDA events around each request (pose already on the host)"}
    d2h = 2 * (host[0][0].numel() + host[0][1].numel() + host[0][2].numel() + 2 * host[0][3].numel())
    out["host_pose_to_yuv"] = {"requests": nposes, "p50_ms": round(_pct(lat, 0.5), 3),
                               "p99_ms": round(_pct(lat, 0.99), 3),
                               "mrays": round(2 * px_eye * nposes / (sum(lat) / 1e3) / 1e6, 3),
                               "d2h_bytes_per_request": d2h,
                               "timing": "host clock around nes_render_yuv_views (pose on the host -> YUV420P + "
                                         "uint16 depth of both eyes in pinned host memory)"}
    # Per-pose parity against the FP64 oracle.
    scene = oracle.Scene(0, 19)
    threads = os.cpu_count() or 1
    psnrs, derr = [], []
    t0 = time.perf_counter()
    for i in range(nposes):
        for e, m in enumerate(nes.stereo_pair(poses[i], 0.063)):
            o_rgb, o_dep, _ = scene.render(m, SW, SH, f, pixels=pix_sets[i][e].astype(np.int32), nthreads=threads)
            g_rgb, g_dep = gpu_px[i][0][e], gpu_px[i][1][e]
            psnrs.append(oracle.psnr(g_rgb, o_rgb))
            derr.append(float(np.abs(g_dep - o_dep).max()))
    out["parity"] = {"against": "FP64 oracle", "pixels_per_eye_per_pose": parity_px, "poses": nposes,
                     "per_pose_min_psnr_db": round(min(psnrs), 2), "median_psnr_db": round(statistics.median(psnrs), 2),
                     "max_depth_err": max(derr), "all_pass": bool(min(psnrs) >= 45.0 and max(derr) <= 1e-3),
                     "oracle_seconds": round(time.perf_counter() - t0, 1)}
    # Table-size sweep.
    sweep = {}
    for lg in log2_tables:
        with nes.Renderer(precision=nes.PREC_FP16_TC, max_pixels=2 * px_eye, device=dev.index,
                          log2_table_size=lg) as r:
            for i in range(2):
                device_request(r, i)
            torch.cuda.synchronize()
            gpu_px.clear()
            ms_t, samp_t = timed_device(r, sweep_poses, collect=lambda i: grab(i) if i == 0 else None)
        sc = scene if lg == 19 else oracle.Scene(0, lg)
        ps, de = [], []
        for e, m in enumerate(nes.stereo_pair(poses[0], 0.063)):
            o_rgb, o_dep, _ = sc.render(m, SW, SH, f, pixels=pix_sets[0][e].astype(np.int32), nthreads=threads)
            ps.append(oracle.psnr(gpu_px[0][0][e], o_rgb))
            de.append(float(np.abs(gpu_px[0][1][e] - o_dep).max()))
        sweep["2^%d" % lg] = {"mrays": round(2 * px_eye * sweep_poses / (sum(ms_t) / 1e3) / 1e6, 3),
                              "p50_ms": round(_pct(ms_t, 0.5), 3), "table_mib_fp16": (16 << lg) * 4 // (1 << 20),
                              "pose0_min_psnr_db": round(min(ps), 2), "pose0_max_depth_err": max(de)}
        del sc
    out["table_sweep"] = sweep
    out["table_sweep_note"] = ("device Mrays/s over %d poses per table size (2 warm-up requests each); parity of "
                               "pose 0 (%d pixels per eye) against the FP64 oracle of the same table size"
                               % (sweep_poses, parity_px))
    return out


def run_glue(dev, peaks):
    """Frame glue on its configured inputs: 30 frames of 1280x720 RGB24 (50/50
    blend of U(0,255) bytes and a horizontal gradient) and FP32 depth
    U(0.1, 10), per kernel timed with CUDA events over the 30 frames after an
    L2 flush (a 1280x720 launch moves 4.1 MB: launch-latency bound); plus one
    7680x4320 frame per kernel, L2 flushed, for the HBM roofline.  Frame 0 is
    checked bit for bit against the oracle's integer restatement."""
    import numpy as np
    import torch
    import nes
    lib = nes.load()
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    hbm = peaks.get("hbm_gbs")

    def frames(w, h, n, seed):
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        noise = torch.randint(0, 256, (n, h, w, 3), generator=g, device=dev, dtype=torch.int32)
        grad = (torch.arange(w, device=dev, dtype=torch.int32) * 255 // max(1, w - 1)).view(1, 1, w, 1)
        rgb = ((noise + grad) // 2).to(torch.uint8).reshape(n, -1)
        dep = (torch.rand((n, h * w), generator=g, device=dev) * 9.9 + 0.1).contiguous()
        return rgb, dep

    def timed(fn, n):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for i in range(n):
            fn(i)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / n

    out = {}
    for tag, (w, h, n) in {"1280x720_x30": (1280, 720, 30), "7680x4320": (7680, 4320, 1)}.items():
        rgb, dep = frames(w, h, n, 5)
        ls = nes.linesizes(w)
        ch = (h + 1) // 2
        ysz = ls[0] * h + 2 * ls[1] * ch
        yuv = torch.empty((n, ysz), dtype=torch.uint8, device=dev)
        gray = torch.empty((n, w * h), dtype=torch.uint8, device=dev)
        dmm = torch.empty((n, w * h), dtype=torch.int16, device=dev)

        def to_yuv(i, src=rgb, gray_src=False):
            y = yuv[i].data_ptr()
            fn = nes.gray8_to_yuv420p if gray_src else nes.rgb24_to_yuv420p
            fn(src[i].data_ptr(), w, h, w if gray_src else 3 * w, y, y + ls[0] * h, y + ls[0] * h + ls[1] * ch,
               ls, sptr)

        for i in range(min(n, 3)):  # warm-up
            to_yuv(i)
        px = w * h
        ms_rgb = timed(to_yuv, n)
        ms_dep = timed(lambda i: nes.depth_pack_u16mm(dep[i].data_ptr(), px, dmm[i].data_ptr(), sptr), n)
        ms_g8 = timed(lambda i: nes.check(lib.nes_depth_to_gray8(dep[i].data_ptr(), px, 4.0, gray[i].data_ptr(),
                                                                 sptr), "gray8"), n)
        ms_gy = timed(lambda i: to_yuv(i, gray, True), n)
        rows = [("rgb24_to_yuv420p", ms_rgb, 4.5), ("depth_pack_u16mm", ms_dep, 6.0),
                ("depth_to_gray8", ms_g8, 5.0), ("gray8_to_yuv420p", ms_gy, 2.5)]
        if n > 1:  # the same frames in one launch per kernel (nes_*_batch)
            yp = [yuv[i].data_ptr() for i in range(n)]
            up = [p + ls[0] * h for p in yp]
            vp = [p + ls[0] * h + ls[1] * ch for p in yp]
            rp, gp = [rgb[i].data_ptr() for i in range(n)], [gray[i].data_ptr() for i in range(n)]
            dp, mp = [dep[i].data_ptr() for i in range(n)], [dmm[i].data_ptr() for i in range(n)]
            nes.yuv420p_batch(rp, w, h, 3 * w, yp, up, vp, ls, sptr)  # warm-up
            rows += [("rgb24_to_yuv420p_batch", timed(lambda i: nes.yuv420p_batch(rp, w, h, 3 * w, yp, up, vp, ls, sptr), 1) / n, 4.5),
                     ("depth_pack_u16mm_batch", timed(lambda i: nes.depth_pack_u16mm_batch(dp, px, mp, sptr), 1) / n, 6.0),
                     ("gray8_to_yuv420p_batch", timed(lambda i: nes.yuv420p_batch(gp, w, h, w, yp, up, vp, ls, sptr,
                                                                                  gray=True), 1) / n, 2.5)]
        ent = {}
        for k, ms, bpp in rows:
            gbs = px * bpp / (ms / 1e3) / 1e9
            ent[k] = {"us_per_frame": round(ms * 1e3, 2), "gbs": round(gbs, 1),
                      "frac_of_hbm": round(gbs / hbm, 3) if hbm else None, "bytes_per_px": bpp}
        if tag.startswith("1280"):
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import oracle
            torch.cuda.synchronize()
            img = rgb[0].cpu().numpy()
            oy, ou, ov = oracle.rgb24_to_yuv420p(img, w, h, 3 * w, ls)
            to_yuv(0)  # the timed gray8 loop reused the YUV buffers
            torch.cuda.synchronize()
            got = yuv[0].cpu().numpy()
            exact = (np.array_equal(got[:ls[0] * h], oy) and np.array_equal(got[ls[0] * h:ls[0] * h + ls[1] * ch], ou)
                     and np.array_equal(got[ls[0] * h + ls[1] * ch:], ov))
            exact_d = np.array_equal(dmm[0].cpu().numpy().view(np.uint16), oracle.depth_pack_u16mm(dep[0].cpu().numpy()))
            ent["bit_exact_vs_oracle"] = bool(exact and exact_d)
        out[tag] = ent
    out["timing"] = ("CUDA events over back-to-back launches after a 256 MiB L2 flush (one launch per frame; "
                     "*_batch: one launch for all 30 frames); GB/s from algorithmic bytes per pixel")
    return out


def run_training(dev, steps, nviews=64, side=800, batch=1 << 18, curve_points=16):
    """Differentiation form: an FP32 teacher (seed 1, T=2^19) renders nviews
    side x side targets (60 deg FOV) from the r = 1.2..2.0 shell; an FP32
    student (seed 2) takes Adam steps of `batch` rays sampled uniformly over
    the views (lr 1e-2, betas (0.9, 0.99), eps 1e-15, L2 RGB + 0.1 L2
    depth).  Each step is synchronous; its device phases come from CUDA
    events on the trainer's stream and the step time from the host clock
    around the call.  PSNR of the student against the teacher on a held-out
    view before and after the steps."""
    import numpy as np
    import torch
    import nes
    f = nes.focal_from_fov(side, 60.0)
    poses = nes.shell_poses(11, nviews + 1, 1.2, 2.0)
    views = [nes.make_view(m, side, side, f) for m in poses[:nviews]]
    held = nes.make_view(poses[nviews], side, side, f)
    px = side * side
    rgb = torch.empty((nviews * px, 3), device=dev)
    dep = torch.empty(nviews * px, device=dev)
    hr, hd = torch.empty((px, 3), device=dev), torch.empty(px, device=dev)
    with nes.Renderer(precision=nes.PREC_FP32, seed=1, max_pixels=nviews * px, device=dev.index) as teacher:
        teacher.render_views(views, [rgb[i * px:].data_ptr() for i in range(nviews)],
                             [dep[i * px:].data_ptr() for i in range(nviews)])
        teacher.render_views([held], [hr.data_ptr()], [hd.data_ptr()])
        torch.cuda.synchronize()
    sr, sd = torch.empty((px, 3), device=dev), torch.empty(px, device=dev)

    def psnr(r):
        r.render_views([held], [sr.data_ptr()], [sd.data_ptr()])
        torch.cuda.synchronize()
        mse = float(torch.mean((sr - hr) ** 2))
        return round(10 * math.log10(1.0 / mse), 2) if mse > 0 else None

    with nes.Renderer(precision=nes.PREC_FP32, seed=2, max_pixels=px, device=dev.index) as student:
        p0 = psnr(student)
        with nes.Trainer(student, batch_rays=batch) as tr:
            tr.set_targets(views, rgb.data_ptr(), dep.data_ptr())
            losses = [tr.step(1000 + i) for i in range(3)]  # warm-up steps (part of the refit)
            wall, phases, samples = [], [], []
            t_all = time.perf_counter()
            for i in range(steps):
                t0 = time.perf_counter()
                losses.append(tr.step(i))
                wall.append(time.perf_counter() - t0)
                phases.append(tr.last_timings())
                samples.append(tr.last_samples())
            t_all = time.perf_counter() - t_all
        p1 = psnr(student)
    ms = 1e3 * statistics.median(wall)
    fwd, bwd, adam = (statistics.median(p[k] for p in phases) for k in range(3))
    every = max(1, len(losses) // curve_points)
    return {"workload": "refit teacher seed 1 -> student seed 2, T=2^19, %d views %dx%d (60 deg FOV, r=1.2..2.0 "
                        "shell), %d rays/step sampled uniformly over the views, Adam lr 1e-2 betas (0.9, 0.99) "
                        "eps 1e-15, loss L2 RGB + 0.1 L2 depth" % (nviews, side, side, batch),
            "steps": steps, "warmup_steps": 3, "ms_per_step": round(ms, 2), "mrays_per_s": round(batch / ms / 1e3, 3),
            "total_s": round(t_all, 1),
            "samples_per_step": int(statistics.median(samples)),
            "msamples_per_s": round(statistics.median(samples) / ms / 1e3, 1),
            "phase_ms": {"forward": round(fwd, 2), "backward": round(bwd, 2), "adam": round(adam, 2)},
            "loss": {"first": round(losses[0], 7), "last": round(losses[-1], 7),
                     "curve_every": every, "curve": [round(v, 7) for v in losses[::every]]},
            "held_out_psnr_db": {"before": p0, "after": p1},
            "timing": "host clock around each synchronous step (median); phases from CUDA events (median)"}


def random_walk_poses(seed, n, rmin=1.2, rmax=2.0, jitter_deg=0.5):
    """Seeded random walk on the shell: each pose turns the eye direction by
    a random rotation of std jitter_deg and moves the radius a little."""
    import numpy as np
    import nes
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    r = 0.5 * (rmin + rmax)
    out = []
    for _ in range(n):
        axis = rng.normal(size=3)
        axis -= axis.dot(d) * d
        axis /= np.linalg.norm(axis)
        ang = math.radians(jitter_deg) * rng.normal()
        d = d * math.cos(ang) + np.cross(axis, d) * math.sin(ang)
        d /= np.linalg.norm(d)
        r = float(np.clip(r + 0.005 * rng.normal(), rmin, rmax))
        out.append(nes.look_at(tuple(0.5 + r * d)))
    return out


def run_serving(dev, seconds, max_queue_ms=0.0):
    """Serving form: open-loop Poisson arrivals, resolutions mixed uniformly
    over mono 640x360, 1280x720, 1920x1080 and stereo 2x1920x1832, random-walk
    poses; latency = submit -> YUV + depth ready on the device.  With
    max_queue_ms > 0 the server rejects a request at submit when its expected
    pose -> YUV time exceeds that bound."""
    import threading as th
    import numpy as np
    import nes
    res = [(640, 360, False), (1280, 720, False), (1920, 1080, False), (1920, 1832, True)]
    out = {}
    with nes.Renderer(precision=nes.PREC_FP16_TC, max_pixels=2 * 1920 * 1832, device=dev.index) as r:
        srv = nes.Server(r, max_inflight_batches=2, max_batch_pixels=2 * 1920 * 1832,
                         hbm_budget_bytes=80 << 30, max_pending=16, max_queue_ms=max_queue_ms)
        import torch
        st0 = srv.stats()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        try:
            # An untimed second at the lowest rate first: graphs for the common
            # batch shapes, the output pool and the throughput estimate settle.
            for rate, secs, timed_run in ((90, 1.0, False), (90, seconds, True), (360, seconds, True),
                                          (720, seconds, True)):
                rng = np.random.default_rng(rate + (0 if timed_run else 7))
                n = int(rate * secs)
                gaps = rng.exponential(1.0 / rate, n)
                kinds = rng.integers(0, 4, n)
                poses = random_walk_poses(rate, n)
                tickets, lock = [], th.Lock()
                done = th.Event()
                lat, pix = [], [0]

                def collect():
                    i = 0
                    while True:
                        with lock:
                            item = tickets[i] if i < len(tickets) else None
                        if item is None:
                            if done.is_set():
                                with lock:
                                    if i >= len(tickets):
                                        return
                                continue
                            time.sleep(0.0005)
                            continue
                        t, px = item
                        res_ = srv.wait(t)
                        lat.append(res_.latency_ms)
                        pix[0] += px
                        srv.release(t)
                        i += 1

                col = th.Thread(target=collect)
                col.start()
                dropped = 0
                t0 = time.perf_counter()
                due = t0
                for i in range(n):
                    due += gaps[i]
                    while time.perf_counter() < due:
                        time.sleep(max(0.0, min(0.001, due - time.perf_counter())))
                    w, h, stereo = res[kinds[i]]
                    f = nes.focal_from_fov(w, 100.0 if stereo else 90.0)
                    mats = nes.stereo_pair(poses[i], 0.063) if stereo else [poses[i]]
                    t = srv.submit([nes.make_view(m, w, h, f) for m in mats])
                    if t is None:
                        dropped += 1
                    else:
                        with lock:
                            tickets.append((t, w * h * len(mats)))
                done.set()
                col.join()
                wall = time.perf_counter() - t0
                if not timed_run:
                    continue
                ls = sorted(lat)
                out[str(rate)] = {"offered": n, "completed": len(lat), "dropped": dropped,
                                  "p50_ms": round(ls[len(ls) // 2], 3) if ls else None,
                                  "p99_ms": round(ls[min(len(ls) - 1, int(math.ceil(0.99 * len(ls))) - 1)], 3)
                                  if ls else None,
                                  "mrays": round(pix[0] / wall / 1e6, 3)}
            st = srv.stats()
            free1 = torch.cuda.mem_get_info(dev)[0]
        finally:
            srv.close()
    out["workload"] = ("Poisson arrivals for %.1f s per rate after 1 s untimed at 90 req/s; mono 640x360 / "
                       "1280x720 / 1920x1080 and stereo "
                       "2x1920x1832 uniformly; random-walk poses on the r=1.2..2.0 shell (0.5 deg jitter); "
                       "FP16 tcgen05; 2 batches in flight; latency = submit -> YUV+depth ready on the device; admission: "
                       "80 GB budget, 16 pending, %s" % (seconds, "expected delay <= %g ms" % max_queue_ms
                                                          if max_queue_ms else "no delay bound"))
    out["batches"] = st["batches"]
    out["graph_instantiations"] = {"at_creation": st0["graph_instantiations"],
                                   "while_serving": st["graph_instantiations"] - st0["graph_instantiations"]}
    out["graph_updates"] = st["graph_updates"]
    out["device_free_bytes_change_while_serving"] = int(free1 - free0)
    out["allocation_note"] = ("outputs are carved from the output arena reserved at server creation; one graph "
                              "per slot, instantiated at creation, replays every batch shape")
    return out


def main():
    args = parse_args()
    global W, H, WORKLOAD
    if (args.width, args.height) != (W, H):
        W, H = args.width, args.height
        WORKLOAD = WORKLOAD.replace("1920x1080", "%dx%d (profiling case)" % (W, H))
    if args.impl == "reference":
        run_reference(args)
    elif args.section == "training":
        import torch
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        print(json.dumps({"training": run_training(dev, args.train_steps, batch=args.train_batch)}), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
