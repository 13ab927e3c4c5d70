"""Benchmark: frames/s registered + warped + stacked on GB300.

Workload (the headline configuration): 2000 synthetic mono uint16 frames of
1280x960 (Gaussian-blurred banded disk, per-frame seeing blur U(0.8, 2.5) px,
random homography, Poisson + read noise), registered against the noiseless
reference with a 4-level c_ecch pyramid, inverse-compositional ECC, affine
then homography, gated by rho >= 0.8, weighted by Laplacian energy and
stacked with compensated FP32 sums. One step = one pass of that whole
sequence through sst_stack_frames.

  value : frames already resident in HBM when the timed region starts
  e2e   : the same call with pinned HOST frames (H2D inside the timed region)
          plus the D2H of every result and of the stacked image

--impl reference times the CPU restatement of the reference path (FP32, the
reference's sequence of full-image passes, OpenMP static row partitions over
all host cores; oracle/sst_refcpu.cc) on a bounded sample of the same workload.
Multi-GPU runs (torchrun) are replicas: each rank stacks its own sequence.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/sec registered+warped+stacked, batched vs plain on GB300 at ≤0.02 px"
WIDTH, HEIGHT = 1280, 960
GAIN = 64.0
SCALE = 1.0 / 65535.0
SEED = 1001


# sst_stack_frames weighting modes
WEIGHTING = {0: "unweighted", 1: "Laplacian-energy frame weights",
             2: "focus-stacking per-pixel weights (6 lap^2 + |grad|^2)^2, Gaussian sigma 3",
             3: "local-variance per-pixel weights (kradius 2, dscale 1, uscale 3)"}
_weighting = 1


def workload_cfg(frames: int):
    return {
        "workload": f"{frames} x {WIDTH}x{HEIGHT} u16 frames; c_ecch 4 levels, inverse-compositional ECC, "
                    f"affine then homography; rho>=0.8 gate; {WEIGHTING[_weighting]}; "
                    "compensated FP32 weighted average",
        "frames": frames, "width": WIDTH, "height": HEIGHT, "levels": 4, "method": "INVERSE_COMPOSITIONAL",
        "passes": ["AFFINE", "HOMOGRAPHY"], "epsx": 0.01, "max_iterations": 50,
        "l2": "inputs (frames x 2.46 MB > 129 MB L2) stream from HBM every step; no flush needed",
    }


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes of one level-0 IC pass launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ecc_ic_pass_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except (OSError, ValueError):
            return None
    return None


def make_workload(n: int, device):
    import torch
    from serstacker_gb300 import synth
    sc = synth.scene_config1()
    frames_i32, Hs, blurs = synth.make_sequence_torch(sc, n, SEED, kind="config1", gain=GAIN,
                                                      blur_range=(0.8, 2.5), device=device)
    frames = torch.where(frames_i32 > 32767, frames_i32 - 65536, frames_i32).to(torch.int16)
    del frames_i32
    ref = (synth.reference_np(sc) * GAIN).astype(np.float32)
    return frames, ref, Hs


def warp_rms_vs_truth(params: np.ndarray, Hs: np.ndarray, status: np.ndarray, step: int = 40):
    ys, xs = np.mgrid[0:HEIGHT:step, 0:WIDTH:step].astype(np.float64)
    out = []
    for p, H, s in zip(params, Hs, status):
        if s != 0:
            continue
        w = p[6] * xs + p[7] * ys + 1.0
        X = (p[0] * xs + p[1] * ys + p[2]) / w
        Y = (p[3] * xs + p[4] * ys + p[5]) / w
        wt = H[2, 0] * xs + H[2, 1] * ys + 1.0
        Xt = (H[0, 0] * xs + H[0, 1] * ys + H[0, 2]) / wt
        Yt = (H[1, 0] * xs + H[1, 1] * ys + H[1, 2]) / wt
        out.append(math.sqrt(float(np.mean((X - Xt) ** 2 + (Y - Yt) ** 2))))
    return float(np.median(out)) if out else None, float(np.max(out)) if out else None


CPU_BASELINE_DESC = ("FP32 reference-semantics CPU restatement (oracle/sst_refcpu.cc: the reference's sequence of "
                     "full-image passes per frame, -O3 -ffast-math, OpenMP static row partitions over all host cores)")


def cpu_reference_rate(frames_host: np.ndarray, ref: np.ndarray, sample: int, threads: int):
    """The FP32 reference-semantics CPU restatement of the path (register +
    warp + running-mean stack) on `sample` frames: frames/s."""
    import oracle as O
    O.set_num_threads(threads)
    po = O.pipeline_opts(passes=(O.AFFINE, O.HOMOGRAPHY), method=O.IC, maxlevel=4, max_iterations=50, epsx=0.01,
                         min_rho=0.8, minimum_image_size=16)
    sub = frames_host[:sample]
    r = (ref.astype(np.float64) * SCALE).astype(np.float32)
    t0 = time.perf_counter()
    O.refcpu_register_and_stack(po, r, sub, SCALE)
    dt = time.perf_counter() - t0
    return sample / dt, dt


def run_reference_arm(args, ws, rank):
    """--impl reference: the reference path's CPU implementation, timed per step."""
    if rank != 0:
        return
    import oracle as O
    O.build()
    from serstacker_gb300 import synth
    threads = os.cpu_count() or 1
    sample = args.ref_sample
    sc = synth.scene_config1()
    frames, _, _ = synth.make_sequence_np(sc, sample, SEED, kind="config1", dtype=np.uint16, gain=GAIN,
                                          blur_range=(0.8, 2.5))
    ref = synth.reference_np(sc) * GAIN
    for _ in range(min(args.warmup, 1)):
        cpu_reference_rate(frames, ref, min(4, sample), threads)
    rates = []
    t_all = 0.0
    for _ in range(args.steps):
        r, dt = cpu_reference_rate(frames, ref, sample, threads)
        rates.append(r)
        t_all += dt
    v = float(np.median(rates))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_all / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_cfg(args.frames),
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} frames of the workload per step; {CPU_BASELINE_DESC}"},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def accuracy_vs_oracle(frames_host: np.ndarray, ref: np.ndarray, opts, passes, threads: int):
    """Registration and stack of `frames_host` through sst_stack_frames against
    the FP64 oracle pipeline (outside every timed region): per-frame warp RMS
    vs the oracle's warp, the stack arithmetic error (the GPU's transforms and
    weights summed in FP64) and the end-to-end stack error, both as maxima
    over the settled pixels (oracle.stack_compare_region)."""
    import oracle as O
    from serstacker_gb300 import capi as C
    O.build()
    O.set_num_threads(threads)
    k = frames_host.shape[0]
    reg = C.c_ecch(opts)
    reg.set_reference_image(ref, scale=SCALE)
    acc = C.c_weigthed_average(WIDTH, HEIGHT)
    out = C.stack_frames(reg, acc, frames_host, passes, SCALE, weighting=1)
    avg, _ = acc.compute()
    po = O.pipeline_opts(passes=(O.AFFINE, O.HOMOGRAPHY), method=O.IC, maxlevel=4, max_iterations=50, epsx=0.01,
                         min_rho=0.8, minimum_image_size=16)
    states, status, rho, S, W = O.register_and_stack(po, ref.astype(np.float64) * SCALE, frames_host, SCALE)
    m = O.model(O.HOMOGRAPHY)
    rms = []
    for i in range(k):
        if status[i] != 0 or out["status"][i] != 0:
            continue
        s_g = O.set_params(m, O.identity(m), out["params"][i][:8].astype(np.float64))
        xa, ya = O.warp_grid(m, s_g, WIDTH, HEIGHT)
        xb, yb = O.warp_grid(m, states[i], WIDTH, HEIGHT)
        rms.append(math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2)[::8, ::8].mean())))
    rep = O.stack_error_report(frames_host, SCALE, O.HOMOGRAPHY, out["params"], out["status"], out["weight"], avg,
                               states, status, S, W)
    return {"frames": k, "status_equal": bool(np.array_equal(out["status"], status)),
            "warp_rms_vs_oracle_px_median": float(np.median(rms)) if rms else None,
            "warp_rms_vs_oracle_px_max": float(np.max(rms)) if rms else None,
            "stack_arith_rel_err_max": rep["arith_max"],
            "stack_rel_err_vs_oracle_max": rep["e2e_max"],
            "stack_rel_err_vs_oracle_median": rep["e2e_median"],
            "stack_err_of_registration_bound": rep["e2e_bound_frac"],
            "note": "stack_arith: the GPU stack vs FP64 sums with the GPU's transforms and weights; "
                    "stack_rel_err_vs_oracle: vs the oracle pipeline's own registration and weights "
                    "(relative to max(|value|, 1% of the image maximum), settled pixels only)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--frames", type=int, default=2000)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--chunk", type=int, default=1280,
                    help="largest streamed chunk of the e2e leg (chunks grow from a quarter of it; "
                         "a quarter of it for the raw Bayer frames)")
    ap.add_argument("--ref-sample", type=int, default=128, help="frames per step of the --impl reference arm")
    ap.add_argument("--cpu-sample", type=int, default=1024,
                    help="frames of the cpu_baseline sample (the FP32 CPU restatement on all host cores)")
    ap.add_argument("--plain-frames", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no autotuner)")
    ap.add_argument("--accuracy-frames", type=int, default=48,
                    help="frames of the workload checked against the FP64 oracle (0: skip)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form leg (profiling runs)")
    ap.add_argument("--unrolled-schedule", action="store_true",
                    help="level iterations as the unrolled launch schedule instead of graph WHILE loops "
                         "(per-kernel profilers do not profile kernels of graphs with conditional nodes)")
    ap.add_argument("--workload", choices=["mono", "bayer", "roi", "flow", "config0", "steps"], default="mono",
                    help="mono: the headline 1280x960 sequence; bayer: raw RGGB 3096x2080 frames; "
                         "roi: uneven-ROI crops (--frames crops); flow: c_eccflow on 1024^2 frames; "
                         "config0: 64 u8 640x480 frames, plain FA euclidean; steps: read_input_frame's debayer and "
                         "bad-pixel filter, LPG weights, the FFT / canvas / focus-stacking accumulators and the "
                         "linear inpaint, each timed on its own")
    ap.add_argument("--roi-method", choices=["fa", "lm"], default="fa")
    ap.add_argument("--roi-sample", type=int, default=8, help="crops checked against the oracle")
    ap.add_argument("--flow-sample", type=int, default=32, help="frames checked against the oracle (flow)")
    ap.add_argument("--ser-file", action="store_true",
                    help="mono workload: also write the frames to a SER file and time sst_stack_ser on it")
    ap.add_argument("--ser-dir", default="/tmp", help="directory of the --ser-file leg's temporary file")
    ap.add_argument("--ser-chunk", type=int, default=256, help="frames per file chunk of the --ser-file leg")
    ap.add_argument("--weighting", type=int, choices=sorted(WEIGHTING), default=1,
                    help="stacking weights of the mono / bayer workloads (1, the Laplacian-energy frame weight, "
                         "is the headline; the oracle's cpu_baseline implements only that one)")
    args = ap.parse_args()
    global _weighting
    _weighting = args.weighting
    if args.weighting != 1:
        args.no_cpu_baseline = True

    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload in ("bayer", "roi", "flow", "config0", "steps"):
        {"bayer": main_bayer, "roi": main_roi, "flow": main_flow, "config0": main_config0,
         "steps": main_steps}[args.workload](
            args, ws, rank, local)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import torch
    from serstacker_gb300 import capi as C
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    C.lib()
    n = args.frames
    frames, ref, Hs = make_workload(n, device)
    frame_bytes = WIDTH * HEIGHT * 2
    opts = C.default_options(method=C.IC, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16,
                             min_rho=0.8)
    reg = C.c_ecch(opts)
    reg.set_level_loops(not args.unrolled_schedule)
    reg.set_reference_image(ref, scale=SCALE)
    acc = C.c_weigthed_average(WIDTH, HEIGHT)
    passes = [C.AFFINE, C.HOMOGRAPHY]
    dev_out = {"params": torch.zeros((n, 12), dtype=torch.float32, device=device),
               "status": torch.zeros(n, dtype=torch.int32, device=device),
               "rho": torch.zeros(n, dtype=torch.float32, device=device),
               "weight": torch.zeros(n, dtype=torch.float32, device=device)}
    tuning = None
    if not args.no_tune:
        # launch shapes chosen by the project's autotuner on a sample of these frames
        # (outside every timed region; cached per device and workload)
        from serstacker_gb300 import autotune
        tuning = autotune.tune_stack_frames(reg, acc, frames, n, WIDTH, HEIGHT, C.DEPTH_U16, WIDTH * 2, frame_bytes,
                                            passes, SCALE, weighting=_weighting, sample=512)

    def step_device():
        acc.clear()
        reg.set_chunk_frames(n)
        C.stack_frames(reg, acc, frames, passes, SCALE, weighting=_weighting, on_device=True, n=n, width=WIDTH,
                       height=HEIGHT, depth=C.DEPTH_U16, row_stride=WIDTH * 2, frame_stride=frame_bytes,
                       outputs=dev_out)

    # ---------------------------------------------------------------- value
    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    C.kernel_launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step_device()
    e1.record()
    torch.cuda.synchronize()
    barrier(ws)
    launches = C.kernel_launch_count()
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, ws)
    clk = clocks.stop()
    value = ws * n / (ms / 1000.0)

    # roofline of the dominant kernel: the level-0 Gauss-Newton passes
    peak, peak_kind = measured_peaks()
    lv_ms, lv_bytes, lv_fi = 0.0, 0.0, 0.0
    level_table = []
    for k in range(len(passes)):
        for lvl in range(reg.num_levels()):
            t, fi, ab = reg.level_stats(k, lvl)
            level_table.append({"pass": k, "level": lvl, "ms": t, "frame_iterations": fi, "alg_bytes": ab})
            if lvl == 0:
                lv_ms += t
                lv_bytes += ab
                lv_fi += fi
    achieved = lv_bytes / (lv_ms / 1000.0) / 1e9 if lv_ms > 0 else 0.0
    tr = traffic_per_launch()
    # ncu DRAM bytes of one level-0 launch covering all n frames (small-case capture scaled
    # by frames; the per-frame traffic does not depend on the batch size)
    traffic = tr["dram_bytes_per_frame_iteration"] * n if tr else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "alg_bytes_per_launch": 16.0 * WIDTH * HEIGHT * n,
            "traffic_note": "DRAM bytes of a level-0 launch with all frames active (ncu, scaled from 64 frames)",
            "kernel": "k_pass_pointwise_tma<IC> level 0 (1280x960), all frames x iterations",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "alg_bytes_model": "16 B per pixel and frame-iteration (warped source 4 + template 4 + gradients 8)",
            "level0_ms_per_step": lv_ms, "level0_frame_iterations": lv_fi}

    res = {k: v.cpu().numpy() for k, v in dev_out.items()}
    med_rms, max_rms = warp_rms_vs_truth(res["params"][:, :8].astype(np.float64), Hs, res["status"])

    # ---------------------------------------------------------------- e2e
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ws, n, frames, reg, acc, passes, frame_bytes)
    plain_fps = run_plain(args, n, frames, ref, opts, passes) if not args.no_plain else None
    pn = min(args.plain_frames, n)
    ser_leg = run_ser_file(args, n, frames, ref, opts, passes) if args.ser_file and rank == 0 else None

    # ---------------------------------------------------------- CPU baseline
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle as O
        O.build()
        threads = os.cpu_count() or 1
        cs = max(1, min(args.cpu_sample, n))
        sub = frames[:cs].cpu().numpy().view(np.uint16)
        rate, dt = cpu_reference_rate(sub, ref, cs, threads)
        cpu = {"value": rate, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": f"{cs} frames of the workload ({dt:.1f} s); {CPU_BASELINE_DESC}"}

    acc_oracle = None
    if rank == 0 and args.accuracy_frames > 0 and _weighting == 1:
        ka = min(args.accuracy_frames, n)
        acc_oracle = accuracy_vs_oracle(frames[:ka].cpu().numpy().view(np.uint16), ref, opts, passes,
                                        os.cpu_count() or 1)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_cfg(n), "parallelism": f"replicas x{ws}", "tuning": tuning,
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
                "clocks": clk, "gpu_launches": launches,
                "plain": None if plain_fps is None else {
                    "value": plain_fps, "unit": "frames/s", "frames": pn,
                    "form": "one frame per call, one launch per Gauss-Newton step, host sync per step"},
                "batched_over_plain": None if plain_fps is None else value / ws / plain_fps,
                "accuracy": {"warp_rms_vs_truth_px_median": med_rms, "warp_rms_vs_truth_px_max": max_rms,
                             "frames_ok": int((res["status"] == 0).sum()), "vs_oracle": acc_oracle},
                "levels": level_table}
        if ser_leg is not None:
            line["ser_file"] = ser_leg
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_e2e(args, ws, n, frames, reg, acc, passes, frame_bytes):
    import torch
    from serstacker_gb300 import capi as C
    host_frames = torch.empty((n, HEIGHT, WIDTH), dtype=torch.int16, pin_memory=True)
    host_frames.copy_(frames)
    torch.cuda.synchronize()
    pinned_out = {"params": torch.zeros((n, 12), dtype=torch.float32, pin_memory=True),
                  "status": torch.zeros(n, dtype=torch.int32, pin_memory=True),
                  "rho": torch.zeros(n, dtype=torch.float32, pin_memory=True),
                  "weight": torch.zeros(n, dtype=torch.float32, pin_memory=True)}
    avg_host = torch.zeros((HEIGHT, WIDTH), dtype=torch.float32, pin_memory=True)
    mask_host = torch.zeros((HEIGHT, WIDTH), dtype=torch.uint8, pin_memory=True)

    def step_e2e():
        acc.clear()
        reg.set_chunk_frames(args.chunk)
        C.stack_frames(reg, acc, host_frames.data_ptr(), passes, SCALE, weighting=_weighting, on_device=True, n=n,
                       width=WIDTH, height=HEIGHT, depth=C.DEPTH_U16, row_stride=WIDTH * 2,
                       frame_stride=frame_bytes, outputs=pinned_out, host_input=True)
        C.lib().sst_weighted_average_compute(acc.handle, avg_host.data_ptr(), mask_host.data_ptr(), 0, None)

    for _ in range(max(1, args.warmup)):
        step_e2e()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    barrier(ws)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1000.0 / args.steps, ws)
    d2h = n * (12 * 4 + 3 * 4) + WIDTH * HEIGHT * 5
    # this host's copy rate for the same pinned frames in chunk-sized copies: the
    # step cannot finish before its frames have crossed
    total = n * frame_bytes
    dev = torch.empty(min(n, args.chunk) * frame_bytes, dtype=torch.uint8, device="cuda")
    src = host_frames.view(torch.uint8).view(-1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    off = 0
    while off < total:
        m = min(dev.numel(), total - off)
        dev[:m].copy_(src[off:off + m], non_blocking=True)
        off += m
    ev1.record()
    torch.cuda.synchronize()
    copy_ms = ev0.elapsed_time(ev1)
    del dev
    return {"value": ws * n / (e2e_ms / 1000.0), "unit": "frames/s", "h2d_bytes_per_step": total,
            "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
            "h2d_copy_gbs": total / (copy_ms * 1e6), "h2d_copy_ms": copy_ms,
            "api": "sst_stack_frames (host pinned) + sst_weighted_average_compute"}


def run_ser_file(args, n, frames, ref, opts, passes):
    """The workload written to a SER file (16-bit mono, read back from the page
    cache) and stacked by sst_stack_ser: file reads into pinned chunks overlap
    registration + stacking. Frames are scaled by 1 / 2^16 as read_input_frame
    does, so the reference is set with that scale. Returns the leg's figures."""
    import torch
    from serstacker_gb300 import capi as C
    path = os.path.join(args.ser_dir, f"sst_bench_{os.getpid()}.ser")
    host = frames.cpu().numpy().view(np.uint16)
    w = C.c_ser_writer(path, WIDTH, HEIGHT, 0, 16)
    try:
        w.write(host)
        w.close()
        del host
        reg_s = C.c_ecch(opts)
        reg_s.set_reference_image(ref, scale=1.0 / 65536)
        acc_s = C.c_weigthed_average(WIDTH, HEIGHT)
        passes_s = list(passes)

        def step():
            acc_s.clear()
            ser = C.c_ser_reader(path)
            out = C.stack_ser(reg_s, acc_s, ser, passes_s, chunk=args.ser_chunk, weighting=_weighting)
            ser.close()
            return out

        for _ in range(max(1, args.warmup)):
            out = step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out = step()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    finally:
        w.close()
        if os.path.exists(path):
            os.remove(path)
    return {"value": n / (ms / 1000.0), "unit": "frames/s", "ms_per_step": ms, "file_bytes": 178 + n * WIDTH * HEIGHT * 2
            + n * 8, "chunk": args.ser_chunk, "frames_ok": int((out["status"] == 0).sum()),
            "api": "sst_stack_ser (16-bit mono SER file in the page cache)"}


def run_plain(args, n, frames, ref, opts, passes):
    """The plain one-frame-per-launch form on a subset of the sequence: frames/s."""
    import torch
    from serstacker_gb300 import capi as C
    pn = min(args.plain_frames, n)
    sub = frames[:pn].cpu().numpy().view(np.uint16)
    reg_p = C.c_ecch(opts)
    reg_p.set_reference_image(ref, scale=SCALE)
    acc_p = C.c_weigthed_average(WIDTH, HEIGHT)
    reg_p.align(sub[:1], passes, scale=SCALE, plain=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(pn):
        o = reg_p.align(sub[i:i + 1], passes, scale=SCALE, plain=True)
        acc_p.add_warped(sub[i:i + 1], C.HOMOGRAPHY, o["params"], status=o["status"], weights=o["weight"],
                         scale=SCALE)
    torch.cuda.synchronize()
    return pn / (time.perf_counter() - t0)


# ------------------------------------------------------------------ config-0 workload

C0_W, C0_H = 640, 480


def config0_cfg(n: int):
    return {
        "workload": f"{n} x {C0_W}x{C0_H} u8 frames (banded disk of radius 180 px, euclidean warps tx, ty ~ "
                    "U(-8, 8) px and theta ~ N(0, 0.5 deg) about (0, 0), Poisson peak 200 + read noise 2); plain "
                    "forward-additive ECC, EUCLIDEAN (fixed scale: the reference's eps never converges, every "
                    "frame runs max_iterations 30), one pyramid level; bilinear remap; unweighted FP32 average",
        "frames": n, "width": C0_W, "height": C0_H, "levels": 1, "method": "FORWARD_ADDITIVE",
        "passes": ["EUCLIDEAN"], "max_iterations": 30,
        "l2": f"inputs ({n} x 0.31 MB) fit in L2; the step is latency-bound, not HBM-bound",
    }


def main_config0(args, ws_, rank, local):
    """BASELINE's CPU-runnable case: 64 u8 640x480 frames, FA euclidean, one
    level, unweighted stack, through sst_stack_frames."""
    import torch
    from serstacker_gb300 import capi as C
    from serstacker_gb300 import synth
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    C.lib()
    n = args.frames if args.frames != 2000 else 64
    sc = synth.scene_config0()
    fr, Hs, _ = synth.make_sequence_torch(sc, n, SEED, kind="config0", gain=1.0, blur_range=None, device=device,
                                          maxval=255)
    frames = fr.to(torch.uint8)
    del fr
    ref = synth.reference_np(sc).astype(np.float32)
    opts = C.default_options(method=C.FA, maxlevel=0, max_iterations=30, epsx=0.2, minimum_image_size=16,
                             min_rho=0.0)
    reg = C.c_ecch(opts)
    reg.set_level_loops(not args.unrolled_schedule)
    reg.set_reference_image(ref, scale=1.0)
    acc = C.c_weigthed_average(C0_W, C0_H)
    passes = [C.EUCLIDEAN]
    dev_out = {"params": torch.zeros((n, 12), dtype=torch.float32, device=device),
               "status": torch.zeros(n, dtype=torch.int32, device=device),
               "rho": torch.zeros(n, dtype=torch.float32, device=device),
               "weight": torch.zeros(n, dtype=torch.float32, device=device)}

    def step(ptr, on_device, host_input, outputs):
        acc.clear()
        reg.set_chunk_frames(n)
        C.stack_frames(reg, acc, ptr, passes, 1.0, weighting=0, on_device=on_device, n=n, width=C0_W, height=C0_H,
                       depth=C.DEPTH_U8, row_stride=C0_W, frame_stride=C0_W * C0_H, outputs=outputs,
                       host_input=host_input)

    for _ in range(args.warmup):
        step(frames, True, False, dev_out)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws_)
    torch.cuda.synchronize()
    C.kernel_launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step(frames, True, False, dev_out)
    e1.record()
    torch.cuda.synchronize()
    barrier(ws_)
    launches = C.kernel_launch_count()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws_)
    clk = clocks.stop()
    value = ws_ * n / (ms / 1000.0)
    t0_ms, fi0, ab0 = reg.level_stats(0, 0)
    peak, peak_kind = measured_peaks()
    achieved = ab0 / (t0_ms / 1000.0) / 1e9 if t0_ms > 0 else 0.0
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "k_pass_stencil<FA, EUCLIDEAN> (the single level), all frames x iterations",
            "alg_bytes_model": "8 B per pixel and frame-iteration (warped source 4 + template 4)",
            "peak_source": peak_kind, "level0_ms_per_step": t0_ms, "frame_iterations": fi0}
    res = {k: v.cpu().numpy() for k, v in dev_out.items()}

    # e2e: pinned host frames through the same call, results and the stack read back
    host = torch.empty((n, C0_H, C0_W), dtype=torch.uint8, pin_memory=True)
    host.copy_(frames)
    pout = {k: torch.zeros_like(v, device="cpu").pin_memory() for k, v in dev_out.items()}
    avg_host = torch.zeros((C0_H, C0_W), dtype=torch.float32, pin_memory=True)
    mask_host = torch.zeros((C0_H, C0_W), dtype=torch.uint8, pin_memory=True)

    def step_e2e():
        step(host.data_ptr(), True, True, pout)
        C.lib().sst_weighted_average_compute(acc.handle, avg_host.data_ptr(), mask_host.data_ptr(), 0, None)

    for _ in range(max(1, args.warmup)):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1000.0 / args.steps, ws_)
    e2e = {"value": ws_ * n / (e2e_ms / 1000.0), "unit": "frames/s", "h2d_bytes_per_step": n * C0_W * C0_H,
           "d2h_bytes_per_step": n * 16 * 4 + C0_W * C0_H * 5, "ms_per_step": e2e_ms,
           "api": "sst_stack_frames (host pinned) + sst_weighted_average_compute"}

    # plain one-frame-per-launch form
    sub = frames[:min(args.plain_frames, n)].cpu().numpy()
    reg_p = C.c_ecch(opts)
    reg_p.set_reference_image(ref, scale=1.0)
    acc_p = C.c_weigthed_average(C0_W, C0_H)
    reg_p.align(sub[:1], passes, plain=True)
    torch.cuda.synchronize()
    tp = time.perf_counter()
    for i in range(sub.shape[0]):
        o = reg_p.align(sub[i:i + 1], passes, plain=True)
        acc_p.add_warped(sub[i:i + 1], C.EUCLIDEAN, o["params"], status=o["status"])
    torch.cuda.synchronize()
    plain_fps = sub.shape[0] / (time.perf_counter() - tp)

    acc_o = None
    if rank == 0 and args.accuracy_frames > 0:
        import oracle as O
        O.build()
        O.set_num_threads(os.cpu_count() or 1)
        k = min(8, n)
        host_np = frames[:k].cpu().numpy()
        m = O.model(O.EUCLIDEAN)
        oo = O.ecch_opts(method=O.FA, maxlevel=0, max_iterations=30, epsx=0.2, minimum_image_size=16)
        rms, its = [], []
        for i in range(k):
            st, it, _ = O.ecch_align(m, O.identity(m), ref.astype(np.float64), host_np[i].astype(np.float64), oo)
            s_g = O.set_params(m, O.identity(m), res["params"][i][:3].astype(np.float64))
            xa, ya = O.warp_grid(m, s_g, C0_W, C0_H)
            xb, yb = O.warp_grid(m, st, C0_W, C0_H)
            rms.append(math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2)[::8, ::8].mean())))
            its.append(it)
        acc_o = {"frames": k, "warp_rms_vs_oracle_px_max": max(rms), "oracle_iterations": sorted(set(its))}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws_, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {**config0_cfg(n), "parallelism": f"replicas x{ws_}"}, "e2e": e2e, "roofline": roof,
                "cpu_baseline": None, "clocks": clk, "gpu_launches": launches,
                "plain": {"value": plain_fps, "unit": "frames/s", "frames": int(sub.shape[0])},
                "batched_over_plain": value / ws_ / plain_fps,
                "accuracy": {"gpu_iterations_per_frame": fi0 / n, "frames_ok": int((res["status"] == 0).sum()),
                             "vs_oracle": acc_o}}
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ Bayer workload

BAYER_W, BAYER_H = 3096, 2080
BAYER_SCALE = 1.0 / 4096.0


def bayer_cfg(frames: int):
    return {
        "workload": f"{frames} x {BAYER_W}x{BAYER_H} raw RGGB u16 12-bit frames (peak 1500 ADU, Poisson + read "
                    "noise); translation-only inverse-compositional c_ecch (4 levels) on the 2x2-binned "
                    f"luminance ({BAYER_W // 2}x{BAYER_H // 2}); rho>=0.8 gate; {WEIGHTING[_weighting]}; "
                    "the four Bayer planes warped and stacked with compensated FP32 sums",
        "frames": frames, "width": BAYER_W, "height": BAYER_H, "levels": 4, "method": "INVERSE_COMPOSITIONAL",
        "passes": ["TRANSLATION"], "epsx": 0.01, "max_iterations": 50,
        "l2": "inputs (frames x 12.9 MB > 129 MB L2) stream from HBM every step; no flush needed",
    }


def bayer_cpu_rate(frames: np.ndarray, ref_bin: np.ndarray, sample: int, threads: int):
    """The oracle's Bayer path on `sample` raw frames: bin, register, weight,
    extract planes, warp + accumulate four planes. Returns (frames/s, seconds)."""
    import oracle as O
    O.set_num_threads(threads)
    m = O.model(O.TRANSLATION)
    oo = O.ecch_opts(method=O.IC, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16)
    pw, ph = BAYER_W // 2, BAYER_H // 2
    ref = ref_bin.astype(np.float64) * BAYER_SCALE
    S = np.zeros((4, ph, pw))
    W = np.zeros((ph, pw))
    t0 = time.perf_counter()
    for i in range(sample):
        b = O.average_bayer_planes(frames[i]).astype(np.float64) * BAYER_SCALE
        st, _, _ = O.ecch_align(m, O.identity(m), ref, b, oo)
        lw = O.laplacian_energy(O.pyrdown(O.smooth(b, 1.0)))
        planes = O.extract_bayer_planes(frames[i])
        for k in range(4):
            dst, msk = O.stack_remap(m, st, planes[..., k].astype(np.float64) * BAYER_SCALE, pw, ph)
            wt = np.where(msk > 0, lw, 0.0)
            S[k] += wt * dst
            if k == 0:
                W += wt
    dt = time.perf_counter() - t0
    return sample / dt, dt


def make_bayer_workload(n: int, device):
    import torch
    from serstacker_gb300 import synth
    sc = synth.scene_bayer()
    fr32, Hs, _ = synth.make_sequence_torch(sc, n, SEED + 2, kind="translation", gain=1.0, blur_range=(0.8, 2.5),
                                            device=device, chunk=8, cell_gains=synth.BAYER_GAINS, maxval=4095)
    frames = fr32.to(torch.int16)                       # values <= 4095: the same bits as u16
    del fr32
    cg = np.tile(np.asarray(synth.BAYER_GAINS), (BAYER_H // 2, BAYER_W // 2))
    ref_raw = np.clip(np.rint(synth.reference_np(sc) * cg), 0, 4095).astype(np.uint16)
    return frames, ref_raw, Hs


def main_bayer(args, ws, rank, local):
    import torch
    from serstacker_gb300 import capi as C
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    C.lib()
    n = args.frames
    frames, ref_raw, Hs = make_bayer_workload(n, device)
    ref_bin = C.bayer_planes(ref_raw, average=True)   # sst_average_bayer_planes_u16
    pw, ph = BAYER_W // 2, BAYER_H // 2
    frame_bytes = BAYER_W * BAYER_H * 2
    opts = C.default_options(method=C.IC, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16,
                             min_rho=0.8)
    reg = C.c_ecch(opts)
    reg.set_level_loops(not args.unrolled_schedule)
    reg.set_reference_image(ref_bin.astype(np.float32), scale=BAYER_SCALE)
    accs = [C.c_weigthed_average(pw, ph) for _ in range(4)]
    passes = [C.TRANSLATION]
    dev_out = {"params": torch.zeros((n, 12), dtype=torch.float32, device=device),
               "status": torch.zeros(n, dtype=torch.int32, device=device),
               "rho": torch.zeros(n, dtype=torch.float32, device=device),
               "weight": torch.zeros(n, dtype=torch.float32, device=device)}

    def step(ptr, on_device, host_input, outputs, chunk):
        for a in accs:
            a.clear()
        reg.set_chunk_frames(chunk)
        C.stack_bayer_frames(reg, accs, ptr, passes, BAYER_SCALE, weighting=_weighting, on_device=on_device, n=n,
                             width=BAYER_W, height=BAYER_H, row_stride=BAYER_W * 2, frame_stride=frame_bytes,
                             outputs=outputs, host_input=host_input)

    for _ in range(args.warmup):
        step(frames, True, False, dev_out, n)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    C.kernel_launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step(frames, True, False, dev_out, n)
    e1.record()
    torch.cuda.synchronize()
    barrier(ws)
    launches = C.kernel_launch_count()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws)
    clk = clocks.stop()
    value = ws * n / (ms / 1000.0)
    peak, peak_kind = measured_peaks()
    lv_ms, lv_bytes = 0.0, 0.0
    level_table = []
    for lvl in range(reg.num_levels()):
        t, fi, ab = reg.level_stats(0, lvl)
        level_table.append({"pass": 0, "level": lvl, "ms": t, "frame_iterations": fi, "alg_bytes": ab})
        if lvl == 0:
            lv_ms, lv_bytes = t, ab
    achieved = lv_bytes / (lv_ms / 1000.0) / 1e9 if lv_ms > 0 else 0.0
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": f"k_pass_pointwise_tma<IC> level 0 ({pw}x{ph}), all frames x iterations",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "alg_bytes_model": "16 B per pixel and frame-iteration"}
    res = {k: v.cpu().numpy() for k, v in dev_out.items()}
    ok = res["status"] == 0
    err = np.hypot(res["params"][ok, 0] - Hs[ok, 0, 2] / 2, res["params"][ok, 1] - Hs[ok, 1, 2] / 2)

    e2e = None
    if not args.no_e2e:
        host = torch.empty((n, BAYER_H, BAYER_W), dtype=torch.int16, pin_memory=True)
        host.copy_(frames)
        pinned = {"params": torch.zeros((n, 12), dtype=torch.float32, pin_memory=True),
                  "status": torch.zeros(n, dtype=torch.int32, pin_memory=True),
                  "rho": torch.zeros(n, dtype=torch.float32, pin_memory=True),
                  "weight": torch.zeros(n, dtype=torch.float32, pin_memory=True)}
        avg_host = torch.zeros((4, ph, pw), dtype=torch.float32, pin_memory=True)
        mask_host = torch.zeros((ph, pw), dtype=torch.uint8, pin_memory=True)

        def step_e2e():
            # raw frames are 5x the mono frame: a quarter of the mono chunk keeps the
            # first, unoverlapped copy short
            step(host.data_ptr(), True, True, pinned, max(32, args.chunk // 4))
            for k, a in enumerate(accs):
                C.lib().sst_weighted_average_compute(a.handle, avg_host[k].data_ptr(),
                                                     mask_host.data_ptr() if k == 0 else None, 0, None)

        for _ in range(max(1, args.warmup)):
            step_e2e()
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_e2e()
        torch.cuda.synchronize()
        barrier(ws)
        e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1000.0 / args.steps, ws)
        e2e = {"value": ws * n / (e2e_ms / 1000.0), "unit": "frames/s", "h2d_bytes_per_step": n * frame_bytes,
               "d2h_bytes_per_step": n * 60 + pw * ph * (16 + 1), "ms_per_step": e2e_ms,
               "api": "sst_stack_bayer_frames (host pinned) + 4 x sst_weighted_average_compute"}
        del host

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = max(1, min(args.cpu_sample, n))
        sub = frames[:sample].cpu().numpy().view(np.uint16)
        rate, dt = bayer_cpu_rate(sub, ref_bin, sample, threads)
        cpu = {"value": rate, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": f"{sample} raw frames of the workload (oracle FP64 Bayer path, OpenMP, {dt:.1f} s)"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {**bayer_cfg(n), "parallelism": f"replicas x{ws}"},
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
                "accuracy": {"translation_err_vs_truth_px_median": float(np.median(err)) if err.size else None,
                             "translation_err_vs_truth_px_max": float(np.max(err)) if err.size else None,
                             "frames_ok": int(ok.sum())},
                "levels": level_table}
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ ROI workload

ROI_CANVAS = 4096


def roi_cfg(n: int, method: str):
    return {
        "workload": f"{n} f32 crops, width and height ~ U(128, 1024) independently, cut from a {ROI_CANVAS}^2 "
                    "tiled banded-disk scene; each crop registered against its own reference crop by c_ecch "
                    f"({method}, QUADRATIC 12-parameter motion, 4 levels, epsx 0.01, 50 iterations); warps: "
                    "translation U(-12, 12) px, scale 1 + U(-0.01, 0.01), quadratic terms <= 1 px at the corner",
        "crops": n, "method": method, "motion": "QUADRATIC", "levels": 4, "epsx": 0.01, "max_iterations": 50,
        "l2": "pools (2 x ~5.4 GB) stream from HBM every step; no flush needed",
    }


def tiled_scene_torch(X, Y):
    """banded disks (radius 200, edge sigma 2, bands of period 24) tiled every
    512 px over a faint two-frequency ripple, so that every crop has texture"""
    import torch
    P, Rd, es = 512.0, 200.0, 2.0
    cx = torch.remainder(X, P) - P / 2
    cy = torch.remainder(Y, P) - P / 2
    r = torch.hypot(cx, cy)
    disk = 0.5 * torch.special.erfc((r - Rd) / (math.sqrt(2.0) * es))
    amp = 0.2 * math.exp(-2.0 * math.pi ** 2 * es ** 2 / 24.0 ** 2)
    bands = 1.0 + amp * torch.sin(2 * math.pi * cy / 24.0)
    ripple = 20.0 * (1.0 + 0.5 * torch.sin(2 * math.pi * X / 37.0) * torch.sin(2 * math.pi * Y / 53.0))
    return 200.0 * disk * bands / 1.2 + ripple


def make_roi_workload(n: int, device, seed: int = SEED + 1):
    """crop sizes, offsets and quadratic warps (seeded), rendered on the device into two packed pools"""
    import torch
    rng = np.random.default_rng(seed)
    ws = rng.integers(128, 1025, size=n)
    hs = rng.integers(128, 1025, size=n)
    ox = rng.uniform(16, ROI_CANVAS - 16 - ws)
    oy = rng.uniform(16, ROI_CANVAS - 16 - hs)
    t = rng.uniform(-12, 12, size=(n, 2))
    sc = 1.0 + rng.uniform(-0.01, 0.01, size=n)
    qx = rng.uniform(-1, 1, size=(n, 3))      # x*y, x*x, y*y terms, scaled to <= 1 px at the corner
    qy = rng.uniform(-1, 1, size=(n, 3))
    sizes = ws * hs
    offs = np.concatenate([[0], np.cumsum(sizes)])
    ref_pool = torch.empty(int(offs[-1]), dtype=torch.float32, device=device)
    cur_pool = torch.empty(int(offs[-1]), dtype=torch.float32, device=device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    for i in range(n):
        w, h = int(ws[i]), int(hs[i])
        y, x = torch.meshgrid(torch.arange(h, device=device, dtype=torch.float64),
                              torch.arange(w, device=device, dtype=torch.float64), indexing="ij")
        ref_pool[offs[i]:offs[i + 1]] = tiled_scene_torch(x + ox[i], y + oy[i]).reshape(-1).float()
        d = 3.0 * float(max(w, h)) ** 2
        X = sc[i] * x + t[i, 0] + (qx[i, 0] * x * y + qx[i, 1] * x * x + qx[i, 2] * y * y) / d
        Y = sc[i] * y + t[i, 1] + (qy[i, 0] * x * y + qy[i, 1] * x * x + qy[i, 2] * y * y) / d
        img = tiled_scene_torch(X + ox[i], Y + oy[i])
        img = img + torch.randn(img.shape, generator=g, device=device, dtype=img.dtype)
        cur_pool[offs[i]:offs[i + 1]] = img.reshape(-1).float()
    return ref_pool, cur_pool, ws, hs, offs


def main_roi(args, ws_, rank, local):
    import torch
    from serstacker_gb300 import capi as C
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    C.lib()
    n = args.frames
    method = C.FA if args.roi_method == "fa" else C.LM
    ref_pool, cur_pool, wv, hv, offs = make_roi_workload(n, device)
    rois = (C.Roi * n)()
    for i in range(n):
        rois[i] = C.Roi(int(offs[i]) * 4, int(offs[i]) * 4, int(wv[i]) * 4, int(wv[i]) * 4, int(wv[i]), int(hv[i]))
    opts = C.default_options(method=method, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16)
    rb = C.c_roi_batch(opts)
    outs = {"params": torch.zeros((n, 12), dtype=torch.float32, device=device),
            "status": torch.zeros(n, dtype=torch.int32, device=device),
            "iterations": torch.zeros(n, dtype=torch.int32, device=device),
            "eps": torch.zeros(n, dtype=torch.float32, device=device),
            "rho": torch.zeros(n, dtype=torch.float32, device=device)}

    def step():
        rb.align_device(n, rois, ref_pool, cur_pool, C.DEPTH_F32, [C.QUADRATIC], 1.0, outs)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws_)
    torch.cuda.synchronize()
    C.kernel_launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    barrier(ws_)
    launches = C.kernel_launch_count()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws_)
    clk = clocks.stop()
    value = ws_ * n / (ms / 1000.0)
    # dominant kernel: the level-0 stencil passes
    peak, peak_kind = measured_peaks()
    t0_ms, fi0, px0, ab0 = rb.level_stats(0, 0)
    levels = []
    for lvl in range(4):
        try:
            t, fi, px, ab = rb.level_stats(0, lvl)
        except C.SSTError:
            break
        levels.append({"level": lvl, "ms": t, "frame_iterations": fi, "pixel_iterations": px, "alg_bytes": ab})
    M = 12
    nH = M * (M + 1) // 2
    flops_px = 2 * nH + 4 * M + M if method == C.FA else 2 * nH + 2 * M + 2
    achieved = ab0 / (t0_ms / 1000.0) / 1e9 if t0_ms > 0 else 0.0
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = sms * 128 * 2 * (clk["sm_max_mhz"] if clk else 2070.0) * 1e6 / 1e12
    tflops = flops_px * px0 / (t0_ms / 1000.0) / 1e12 if t0_ms > 0 else 0.0
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "k_pass_stencil<ROI> level 0, all crops x iterations",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "alg_bytes_model": "8 B per pixel-iteration (warped source + template; gradients on chip)",
            "fp32": {"achieved_tflops": tflops, "nominal_peak_tflops": fp32_peak, "frac": tflops / fp32_peak,
                     "flops_per_pixel_iteration": flops_px,
                     "note": "M = 12: the Hessian and projection FMAs make the pass FP32-bound"}}
    res = {k: v.cpu().numpy() for k, v in outs.items()}

    # accuracy against the FP64 oracle on a sample of crops, and the CPU baseline on the same sample
    acc = None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle as O
        O.build()
        threads = os.cpu_count() or 1
        O.set_num_threads(threads)
        m = O.model(O.QUADRATIC)
        oo = O.ecch_opts(method=method, maxlevel=4, max_iterations=50, epsx=0.01, minimum_image_size=16)
        k = max(1, min(args.roi_sample, n))
        rp, cp = ref_pool.cpu().numpy(), cur_pool.cpu().numpy()
        rms_l = []
        t0 = time.perf_counter()
        states = []
        for i in range(k):
            w, h = int(wv[i]), int(hv[i])
            r = rp[offs[i]:offs[i + 1]].reshape(h, w).astype(np.float64)
            c = cp[offs[i]:offs[i + 1]].reshape(h, w).astype(np.float64)
            s_o, _, _ = O.ecch_align(m, O.identity(m), r, c, oo)
            states.append(s_o)
        dt = time.perf_counter() - t0
        for i in range(k):
            w, h = int(wv[i]), int(hv[i])
            s_g = O.set_params(m, O.identity(m), res["params"][i][:12].astype(np.float64))
            ys, xs = np.mgrid[0:h:16, 0:w:16]
            d2 = [(np.subtract(O.warp(m, states[i], float(x), float(y)), O.warp(m, s_g, float(x), float(y))) ** 2).sum()
                  for y, x in zip(ys.ravel(), xs.ravel())]
            rms_l.append(math.sqrt(float(np.mean(d2))))
        fin = [v for v in rms_l if math.isfinite(v)]
        acc = {"warp_rms_vs_oracle_px_median": float(np.median(fin)) if fin else None,
               "warp_rms_vs_oracle_px_max": float(max(fin)) if fin else None,
               "sample_crops": k, "oracle_nonfinite": len(rms_l) - len(fin),
               "status_sample": [int(v) for v in res["status"][:k]]}
        cpu = {"value": k / dt, "unit": "crops/s", "cores": threads, "kind": "port",
               "sample": f"the first {k} crops (oracle FP64 c_ecch, OpenMP, {dt:.1f} s)"}
    if rank == 0:
        line = {"metric": "crops/sec registered (uneven-ROI batch, quadratic c_ecch)", "value": value,
                "unit": "crops/s", "n_gpus": ws_, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": {**roi_cfg(n, "FORWARD_ADDITIVE" if method == C.FA else "LM"),
                                                "parallelism": f"replicas x{ws_}"},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
                "accuracy": acc, "frames_ok": int((res["status"] == 0).sum()),
                "iterations_median": float(np.median(res["iterations"])), "levels": levels}
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- flow workload

FLOW_W = FLOW_H = 1024


def flow_cfg(n: int):
    return {
        "workload": f"{n} f32 frames {FLOW_W}x{FLOW_H} of a textured scene warped by smooth random fields "
                    "(Gaussian-filtered white noise, correlation length 64 px, 3 px RMS); c_eccflow with the "
                    "registration defaults (support_scale 4, scale_factor 0.75, 3 iterations per level, "
                    "update_multiplier 1.5); adjoint leg: warp residual + gradients to params, template and flow",
        "frames": n, "width": FLOW_W, "height": FLOW_H, "support_scale": 4, "scale_factor": 0.75,
        "max_iterations": 3, "l2": "frames (n x 4 MB) and flow planes stream from HBM; no flush needed",
    }


def make_flow_workload(n: int, device, seed: int = SEED + 4):
    """frames_f(y) = scene(y - d_f(y)), d_f smooth (FFT Gaussian filter of white noise)"""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    ys, xs = torch.meshgrid(torch.arange(FLOW_H, device=device, dtype=torch.float64),
                            torch.arange(FLOW_W, device=device, dtype=torch.float64), indexing="ij")
    ref = tiled_scene_torch(xs + 300.0, ys + 200.0).float()
    fy = torch.fft.fftfreq(FLOW_H, device=device, dtype=torch.float64)
    fx = torch.fft.rfftfreq(FLOW_W, device=device, dtype=torch.float64)
    sigma = 64.0
    tf = torch.exp(-2 * math.pi ** 2 * sigma ** 2 * (fy[:, None] ** 2 + fx[None, :] ** 2))
    frames = torch.empty((n, FLOW_H, FLOW_W), dtype=torch.float32, device=device)
    truth = torch.empty((n, FLOW_H, FLOW_W, 2), dtype=torch.float32, device=device)
    for i in range(n):
        d = []
        for _ in range(2):
            wn = torch.randn((FLOW_H, FLOW_W), generator=g, device=device, dtype=torch.float64)
            f = torch.fft.irfft2(torch.fft.rfft2(wn) * tf, s=(FLOW_H, FLOW_W))
            d.append(f * (3.0 / math.sqrt(2.0)) / f.std())
        truth[i] = torch.stack(d, dim=-1).float()
        img = tiled_scene_torch(xs - d[0] + 300.0, ys - d[1] + 200.0)
        frames[i] = (img + torch.randn(img.shape, generator=g, device=device, dtype=img.dtype)).float()
    return frames, ref, truth


def main_flow(args, ws_, rank, local):
    import torch
    from serstacker_gb300 import capi as C
    from serstacker_gb300 import adjoint
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    C.lib()
    n = args.frames
    frames, ref, truth = make_flow_workload(n, device)
    opts = C.eccflow_options(support_scale=4, scale_factor=0.75, max_iterations=3, update_multiplier=1.5,
                             min_image_size=-1)
    fl = C.c_eccflow(opts)
    fl.set_reference_image(ref.cpu().numpy())
    rmap = torch.empty((n, FLOW_H, FLOW_W, 2), dtype=torch.float32, device=device)

    def step():
        fl.compute_device(frames, n, C.DEPTH_F32, FLOW_W * 4, FLOW_W * FLOW_H * 4, rmap)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws_)
    torch.cuda.synchronize()
    C.kernel_launch_count(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    barrier(ws_)
    launches = C.kernel_launch_count()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws_)
    clk = clocks.stop()
    value = ws_ * n / (ms / 1000.0)
    # algorithmic bytes: per level and iteration, the fused residual + area pass reads {T, gx, gy} (16 B),
    # the flow (8 B) and the warped frame (4 B); the cubic update reads and writes the flow (16 B);
    # per level change the flow is rewritten (8 B); plus the frame read and pyramid writes
    import oracle as O
    oo = O.flow_opts(support_scale=4, scale_factor=0.75, max_iterations=3, update_multiplier=1.5, min_image_size=-1)
    levels = O.eccflow_levels(FLOW_W, FLOW_H, oo)
    px = sum(w * h for w, h in levels)
    bytes_frame = 4 * FLOW_W * FLOW_H + 4 * px + 3 * 44 * px + 8 * px + 8 * FLOW_W * FLOW_H
    achieved = n * bytes_frame / (ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "whole c_eccflow step (k_flow_area + k_flow_solve + k_resample)",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "alg_bytes_model": "per pixel of every level: 3 iterations x (28 B residual/area + 16 B flow update) "
                               "+ 8 B level change + 4 B pyramid; + 12 B per level-0 pixel (frame in, rmap out)",
            "alg_bytes_per_frame": bytes_frame, "levels": len(levels)}
    # accuracy: the flow against the true deformation (interior), all frames
    y, x = torch.meshgrid(torch.arange(FLOW_H, device=device, dtype=torch.float32),
                          torch.arange(FLOW_W, device=device, dtype=torch.float32), indexing="ij")
    fl_est = rmap - torch.stack([x, y], dim=-1)
    err = (fl_est - truth)[:, 32:-32, 32:-32].norm(dim=-1)
    acc = {"flow_err_vs_truth_px_median": float(err.median()), "truth_rms_px": float(truth.norm(dim=-1).pow(2).mean().sqrt())}

    # adjoint leg: loss + gradients (params, template, flow) + Gauss-Newton matrices, all frames
    T = ref.contiguous()
    p = torch.tensor([[1.0, 0.0, 0.0, 0.0, 1.0, 0.0]], device=device).repeat(n, 1)
    flow_in = fl_est.contiguous()
    p12 = adjoint._pad12(p)
    loss = torch.empty(n, dtype=torch.float64, device=device)
    gp = torch.zeros((n, 12), dtype=torch.float32, device=device)
    gt = torch.zeros((FLOW_H, FLOW_W), dtype=torch.float32, device=device)
    gu = torch.zeros((n, FLOW_H, FLOW_W, 2), dtype=torch.float32, device=device)
    hs = torch.zeros((n, 144), dtype=torch.float64, device=device)

    def adj_step():
        adjoint._call(frames, T, p12, flow_in, C.AFFINE, loss=loss, grad_params=gp, grad_template=gt,
                      grad_flow=gu, hessian=hs)

    for _ in range(max(1, args.warmup)):
        adj_step()
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record()
    for _ in range(args.steps):
        adj_step()
    a1.record()
    torch.cuda.synchronize()
    adj_ms = a0.elapsed_time(a1) / args.steps
    # per frame: frame gathers (4), template (4) twice (tiles + template pass), flow read twice (16),
    # flow gradient write (8)
    adj_bytes = n * FLOW_W * FLOW_H * (4 + 4 + 16 + 8 + 4)
    adjoint_line = {"value": n / (adj_ms / 1000.0), "unit": "frames/s", "ms_per_step": adj_ms,
                    "achieved_gbs": adj_bytes / (adj_ms / 1000.0) / 1e9,
                    "outputs": "loss, dL/dp (affine), dL/dT, dL/du, J^T J per frame"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        O.build()
        threads = os.cpu_count() or 1
        O.set_num_threads(threads)
        k = max(1, min(args.flow_sample, n))
        refd = ref.double().cpu().numpy()
        t0 = time.perf_counter()
        diffs = []
        for i in range(k):
            f_o = O.eccflow(oo, refd, frames[i].double().cpu().numpy())
            diffs.append(float(np.sqrt(np.mean((fl_est[i].double().cpu().numpy() - f_o) ** 2))))
        dt = time.perf_counter() - t0
        cpu = {"value": k / dt, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": f"the first {k} frames (oracle FP64 c_eccflow, OpenMP, {dt:.1f} s)"}
        acc["flow_rms_vs_oracle_px"] = diffs
    if rank == 0:
        line = {"metric": "frames/sec of c_eccflow dense flow", "value": value, "unit": "frames/s", "n_gpus": ws_,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {**flow_cfg(n), "parallelism": f"replicas x{ws_}"}, "roofline": roof,
                "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches, "accuracy": acc,
                "adjoint": adjoint_line}
        print(json.dumps(line), flush=True)


STEPS_RAW_W, STEPS_RAW_H = 3096, 2080


def main_steps(args, ws_, rank, local):
    """The steps either side of the stacking loop and the other accumulators,
    each timed on its own with device-resident synthetic inputs (CUDA events,
    warm-up first): read_input_frame's NN2 debayer and bad-pixel filter on raw
    RGGB 3096x2080 u16 frames; LPG maps, the FFT average, the Laplacian focus
    stack and the canvas average on 1280x960 frames; linear_interpolation_inpaint
    of one 1280x960 image. Each entry gives frames/s, the algorithmic bytes per
    pixel and GB/s against the measured HBM peak, and the FP64 oracle timed on
    one frame on one host core (cpu_baseline, kind port)."""
    import ctypes as Cty
    import torch
    import oracle as O
    from serstacker_gb300 import capi as C
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    lib = C.lib()
    O.build()
    peak, peak_kind = measured_peaks()
    n = min(args.frames, 64)
    reps = max(1, args.steps)
    gen = torch.Generator(device=device)
    gen.manual_seed(SEED + 7)

    def timeit(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def cpu_rate(fn):
        t0 = time.perf_counter()
        fn()
        return 1.0 / (time.perf_counter() - t0)

    def entry(ms, frames, px, bytes_per_px, what, cpu, sample="one frame of the same size through the FP64 oracle"):
        gbs = frames * px * bytes_per_px / (ms / 1e3) / 1e9
        return {"frames_per_s": frames / (ms / 1e3), "ms_per_call": ms, "frames_per_call": frames,
                "alg_bytes_per_px": bytes_per_px, "achieved_gbs": gbs, "frac_of_hbm": gbs / peak,
                "workload": what, "cpu_baseline": {"value": cpu, "unit": "frames/s", "cores": 1, "kind": "port",
                                                   "sample": sample}}

    res = {}
    raw_px = STEPS_RAW_W * STEPS_RAW_H
    raw = torch.randint(0, 4096, (n, STEPS_RAW_H, STEPS_RAW_W), generator=gen, device=device,
                        dtype=torch.int32).to(torch.int16)
    bgr = torch.empty((n, STEPS_RAW_H, STEPS_RAW_W, 3), dtype=torch.int16, device=device)
    raw0 = raw[0].cpu().numpy().view(np.uint16)

    def nn2():
        C._check(lib.sst_debayer_nn2(raw.data_ptr(), C.DEPTH_U16, n, STEPS_RAW_W, STEPS_RAW_H, STEPS_RAW_W * 2,
                                     raw_px * 2, 8, bgr.data_ptr(), 0, 0, None), "sst_debayer_nn2")
    res["debayer_nn2"] = entry(timeit(nn2), n, raw_px, 8, f"{n} raw RGGB {STEPS_RAW_W}x{STEPS_RAW_H} u16 -> BGR u16",
                               cpu_rate(lambda: O.debayer_nn2(raw0, 8)))
    flt = torch.empty_like(raw)

    def bad():
        C._check(lib.sst_filter_bad_pixels(raw.data_ptr(), C.DEPTH_U16, n, STEPS_RAW_W, STEPS_RAW_H, STEPS_RAW_W * 2,
                                           raw_px * 2, 8, 3.0, flt.data_ptr(), 0, 0, None), "sst_filter_bad_pixels")
    res["bad_pixels_bayer"] = entry(timeit(bad), n, raw_px, 4,
                                    f"{n} raw RGGB {STEPS_RAW_W}x{STEPS_RAW_H} u16, bayer_denoise k = 3",
                                    cpu_rate(lambda: O.filter_bad_pixels(raw0, 8, 3.0)))
    del raw, bgr, flt
    torch.cuda.empty_cache()

    px = WIDTH * HEIGHT
    frames, _, _ = make_workload(n, device)
    fr32 = (frames.to(torch.int32) & 0xffff).to(torch.float32) * SCALE
    f0 = fr32[0].cpu().numpy().astype(np.float64)
    lpg = C.c_lpg_sharpness_measure()
    maps = torch.empty((n, HEIGHT, WIDTH), dtype=torch.float32, device=device)
    mets = (Cty.c_double * n)()

    def lpg_run():
        C._check(lib.sst_lpg_compute(lpg._h, frames.data_ptr(), C.DEPTH_U16, n, WIDTH, HEIGHT, WIDTH * 2, px * 2, None,
                                     0, 0, 1, maps.data_ptr(), mets, None), "sst_lpg_compute")
    res["lpg"] = entry(timeit(lpg_run), n, px, 6, f"{n} u16 1280x960 frames, c_lpg_options defaults (k 2, p 2, "
                       "dscale 2, uscale 6), maps + metrics", cpu_rate(lambda: O.lpg(f0)))
    fft = C.c_frame_accumulation_with_fft()

    def fft_run():
        C._check(lib.sst_fft_average_clear(fft._h), "clear")
        C._check(lib.sst_fft_average_add(fft._h, fr32.data_ptr(), C.DEPTH_F32, n, WIDTH, HEIGHT, 1, WIDTH * 4, px * 4,
                                         1.0, 1, None), "sst_fft_average_add")
    fsmall = f0[:240, :320]
    res["fft_average_add"] = entry(timeit(fft_run), n, px, 4,
                                   f"{n} f32 1280x960 frames (an optimal DFT size): R2C + spectral weights",
                                   cpu_rate(lambda: O.fft_average(fsmall[None])),
                                   "one 320x240 frame through the FP64 oracle's direct DFT")
    fs = C.c_laplacian_pyramid_focus_stacking()
    nf = min(n, 16)

    def focus_run():
        C._check(lib.sst_focus_stack_clear(fs._h), "clear")
        C._check(lib.sst_focus_stack_add(fs._h, fr32.data_ptr(), C.DEPTH_F32, nf, WIDTH, HEIGHT, 1, WIDTH * 4, px * 4,
                                         1.0, None, 0, 0, 1, None), "sst_focus_stack_add")
    res["focus_stack_add"] = entry(timeit(focus_run), nf, px, 4, f"{nf} f32 1280x960 frames, select_max_energy",
                                   cpu_rate(lambda: O.focus_stack(f0[None])))
    cv = C.c_canvas_average((WIDTH * 3 // 2, HEIGHT * 3 // 2))
    bw, bh = WIDTH - 64, HEIGHT - 64
    yy, xx = torch.meshgrid(torch.arange(bh, device=device, dtype=torch.float32),
                            torch.arange(bw, device=device, dtype=torch.float32), indexing="ij")
    rmap = torch.stack([xx + 17.3, yy + 9.6], dim=-1).contiguous()
    box = (Cty.c_int32 * 4)(300, 250, bw, bh)

    def canvas_run():
        C._check(lib.sst_canvas_average_clear(cv._h), "clear")
        for i in range(n):
            C._check(lib.sst_canvas_average_add(cv._h, fr32[i].data_ptr(), C.DEPTH_F32, WIDTH, HEIGHT, 1, WIDTH * 4, 1.0,
                                                None, 0, 0, None if i == 0 else rmap.data_ptr(),
                                                None if i == 0 else box, 1, None), "sst_canvas_average_add")
    rmap_np = rmap.cpu().numpy().astype(np.float64)
    boxes = np.array([[0, 0, 0, 0], [300, 250, bw, bh]], np.int32)
    res["canvas_average_add"] = entry(
        timeit(canvas_run), n, bw * bh, 16,
        f"{n} f32 1280x960 frames remapped onto a 1920x1440 canvas (one launch per frame)",
        2 * cpu_rate(lambda: O.canvas_average(np.stack([f0, f0]), boxes=boxes, rmaps=[None, rmap_np],
                                               canvas=(WIDTH * 3 // 2, HEIGHT * 3 // 2))),
        "two frames (the first placed, the second remapped) through the FP64 oracle")
    img = fr32[0].clone()
    holes = (torch.rand((HEIGHT, WIDTH), generator=gen, device=device) > 0.05).to(torch.uint8) * 255

    def inpaint_run():
        C._check(lib.sst_linear_interpolation_inpaint(img.data_ptr(), 0, WIDTH, HEIGHT, 1, holes.data_ptr(), 0, 1, None),
                 "sst_linear_interpolation_inpaint")
    hm = holes.cpu().numpy()
    res["linear_inpaint"] = entry(timeit(inpaint_run), 1, px, 13, "one f32 1280x960 image, 5 % random holes",
                                  cpu_rate(lambda: O.linear_inpaint(f0, hm)))
    if rank == 0:
        line = {"metric": "read_input_frame steps, LPG weights and the other accumulators on GB300 (each on its own)",
                "workload": "steps", "n_gpus": ws_, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
                "peak_gbs": peak, "peak_source": peak_kind, "results": res,
                "note": "device-resident inputs, CUDA events; alg_bytes_per_px counts the frame bytes read and the "
                        "result bytes written; cpu_baseline: the FP64 oracle on one host core"}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
