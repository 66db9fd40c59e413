#!/usr/bin/env python
"""Benchmark: nonuniform points/s of forward + adjoint NFFT, 3D N = 128^3, M = 2^21.

Workload (the reference's headline 3D size): d = 3, N = 128^3, n = 256^3
(sigma = 2), Gaussian window m = 6, M = 2^21 nodes iid uniform in
[-0.5, 0.5)^3, coefficients and samples with real/imaginary parts iid
uniform [-1, 1] (seeded synthetic data; the reference publishes no dataset).

A step = bind the node set (FP64 node reduction + binning) + forward NFFT +
adjoint NFFT, i.e. one pass of the hot path over one batch of nodes;
value = M * n_gpus / (time per step), max over ranks.  ``value`` is the FP32
form (FP32 gridding, FFT and accumulation; FP64 node reduction and roll-off);
the FP64 form (the reference's arithmetic) is timed in the same run and
reported as ``fp64_plain``.  Errors are relative l2 against the FP64 direct
NDFT on a 4096-node subsample (forward) and 4096 coefficients (adjoint).  The
same step with the ES window of the extension API (cunfft_x_set_window) is
timed and checked in both forms and reported as ``es_window``.

``--impl reference`` times the reference method on the host CPU cores instead
(the CPU restatement in oracle/, OpenMP over all host threads; the reference
itself is GPU code for a Fermi-era toolchain and does not build here).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NU points/s fwd+adj 3D N=128^3 M=2^21: FP32-batched vs FP64 plain at stated l2 err"
UNIT = "points/s"
N3 = [128, 128, 128]
M_FULL = 1 << 21
M_CUT = 6


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the clustered, batched and autograd legs")
    ap.add_argument("--sustain-s", type=float, default=1.0,
                    help="length of the sustained run after the headline steps (seconds)")
    # The plan's default tiling (T0 = 8, tensor-core kernels) is what the autotuner picks
    # on this workload when timed without a profiler; under ncu its per-launch overhead
    # tips the choice, so the default run skips the autotuner and profiles the same kernels.
    ap.add_argument("--autotune", action="store_true", help="run the autotuner before the timed steps")
    ap.add_argument("--no-autotune", action="store_true", help="(default) keep the plan's default tiling")
    ap.add_argument("--case", choices=["interp", "spread", "step", "spread2d", "interp2d"],
                    help="profiling case: bind nodes once, then launch only this stage (3 times); the 2D cases "
                         "run the batched 2D workload (64 x N=256^2, m=5, log-uniform M)")
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--M", type=int, default=M_FULL)
    ap.add_argument("--tile", default="", help="tile extents for --case, e.g. 8,4,16")
    ap.add_argument("--kernel", default="auto", choices=["auto", "shared", "register", "tensor"],
                    help="gridding kernel form for --case (spreading: shared, register or tensor; "
                         "interpolation: shared or tensor)")
    return ap.parse_args()


def run_case2d(args):
    """Three launches of 2D spreading or interpolation on the batched 2D workload."""
    import numpy as np
    import torch

    from cunfft_gb300.nfft import NFFT

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(404)
    B, N, m = 64, [256, 256], 5
    Ms = np.round(10 ** rng.uniform(3, 6, B)).astype(np.int64)
    Mt = int(Ms.sum())
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (Mt, 2))).to(dev)
    f = _crand_t(Mt, rng, dev, torch.complex64)
    p = NFFT(N, m=m, precision="f32", batch=B, device=dev).set_nodes(x, Ms.tolist())
    if args.kernel != "auto":
        (p.set_spread_kernel if args.case == "spread2d" else p.set_interp_kernel)(args.kernel)
    grid = p.grid()
    out = torch.empty(Mt, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(3):
        if args.case == "spread2d":
            grid.zero_()
        a.record(stream)
        if args.case == "spread2d":
            p.spread(f, grid)
        else:
            p.interp(grid, out=out)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    print(json.dumps({"case": args.case, "M": Mt, "tiling": p.tiling(), "ms": times}))
    p.close()


def run_case(args):
    """A few launches of one stage on the benchmark workload, for ncu captures."""
    import torch

    from cunfft_gb300.nfft import NFFT

    if args.case in ("spread2d", "interp2d"):
        return run_case2d(args)

    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(20240)
    M = args.M
    x = torch.rand(M, 3, generator=g, device=dev, dtype=torch.float64) - 0.5
    cd = torch.complex64 if args.precision == "f32" else torch.complex128
    fh = torch.complex(torch.rand(N3, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                       torch.rand(N3, generator=g, device=dev, dtype=torch.float64) * 2 - 1).to(cd)
    f = torch.complex(torch.rand(M, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                      torch.rand(M, generator=g, device=dev, dtype=torch.float64) * 2 - 1).to(cd)
    p = NFFT(N3, m=M_CUT, precision=args.precision, device=dev)
    if args.tile:
        p.set_tiling([int(v) for v in args.tile.split(",")])
    p.set_nodes(x)
    if args.kernel != "auto":
        if args.case in ("spread", "step"):
            p.set_spread_kernel(args.kernel)
        if args.case in ("interp", "step") and args.kernel != "register":
            p.set_interp_kernel(args.kernel)
    grid = p.grid()
    out = torch.empty(M, dtype=cd, device=dev)
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(3):
        if args.case == "spread":
            grid.zero_()
        a.record(stream)
        if args.case == "interp":
            p.interp(grid, out=out)
        elif args.case == "spread":
            p.spread(f, grid)
        else:
            p.set_nodes(x)
            p.forward(fh, out=out)
            p.adjoint(f)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    print(json.dumps({"case": args.case, "precision": args.precision, "M": M, "tiling": p.tiling(),
                      "ms": times}))
    p.close()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_tensor_peak():
    """Dense bf16 TFLOP/s (measured burst; FP16 runs at the same dense rate)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured bf16_tflops (burst)"
    except Exception:
        return 1900.0, "fallback"


def load_traffic():
    """dram bytes per launch of the dominant kernels from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from before the timed
    region (start() returns once sampling is live) to after it; the summary is over the
    samples stamped inside the region (all samples when none fell inside)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        deadline = time.time() + 5.0
        while time.time() < deadline and os.path.getsize(self.path) == 0:
            time.sleep(0.01)

    def region(self, begin):
        """Mark the start (begin=True) or the end of the timed region (host clock)."""
        import datetime
        now = datetime.datetime.now()
        if begin:
            self.t0 = now
        else:
            self.t1 = now

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        import datetime
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                try:
                    parts[0] = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                except ValueError:
                    parts[0] = None
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        inside = [r for r in rows if r[0] is not None and self.t0 is not None and self.t1 is not None
                  and self.t0 <= r[0] <= self.t1 + datetime.timedelta(milliseconds=50)]
        use = inside or rows
        sm = [float(r[2]) for r in use if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in use if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in use for i in range(4) if r[6 + i].lower() == "active"})
        load = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(use), "samples_in_region": len(inside),
                "interval_ms": 50}


def rel_l2(ref, got):
    import torch
    ref = ref.to(torch.complex128).reshape(-1)
    got = got.to(torch.complex128).reshape(-1)
    return float(torch.linalg.norm(ref - got) / torch.linalg.norm(ref))


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def max_over_ranks_on(v, world, device):
    """Largest per-rank time: the job's step time when every rank runs its own replica."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_points_per_s(M, world, ms_max):
    """Whole-job throughput of `world` replicas of M nodes each, timed by the slowest rank."""
    return M * world / (ms_max * 1e-3)


def run_ours(args):
    import torch
    import torch.distributed as dist

    from cunfft_gb300.nfft import NFFT

    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def max_over_ranks(v):
        return max_over_ranks_on(v, world, dev)

    g = torch.Generator(device=dev).manual_seed(20240 + rank)
    M = M_FULL
    x = torch.rand(M, 3, generator=g, device=dev, dtype=torch.float64) - 0.5
    fh64 = torch.complex(torch.rand(N3, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                         torch.rand(N3, generator=g, device=dev, dtype=torch.float64) * 2 - 1)
    f64 = torch.complex(torch.rand(M, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                        torch.rand(M, generator=g, device=dev, dtype=torch.float64) * 2 - 1)
    fh32, f32 = fh64.to(torch.complex64), f64.to(torch.complex64)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, steps):
        """ms per call of fn over `steps` calls, events on the plan stream, synchronised both sides"""
        barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / steps

    # ---------------- FP32 form (headline) ----------------
    p32 = NFFT(N3, m=M_CUT, precision="f32", device=dev)
    p32.set_nodes(x)
    tuned = None
    if args.autotune and not args.no_autotune:
        tuned = p32.autotune(reps=2)
    out_f = torch.empty(M, dtype=torch.complex64, device=dev)
    out_fh = torch.empty(N3, dtype=torch.complex64, device=dev)

    def step32():
        p32.set_nodes(x)
        p32.forward(fh32, out=out_f)
        p32.adjoint(f32, out=out_fh)

    warm = max(3, args.warmup)
    for _ in range(warm):
        step32()
    barrier()
    clocks = ClockSampler(dev.index)
    clocks.start()
    # the headline: exactly --steps steps, bracketed by a barrier and a synchronize
    clocks.region(True)
    ms32 = timed(step32, args.steps)
    # the same step repeated for at least one second (at least --sustain-s), so that the
    # clock record holds enough samples and the headline is checked against a long run
    sus_steps = max(args.steps, int(math.ceil(args.sustain_s * 1e3 / max(ms32, 1e-3))))
    ms32_sus = timed(step32, sus_steps)
    clocks.region(False)
    clk = clocks.stop()
    ms32_max = max_over_ranks(ms32)
    ms32_sus_max = max_over_ranks(ms32_sus)

    # binning amortised: forward + adjoint on an already-binned node set
    p32.set_nodes(x)

    def fwdadj32():
        p32.forward(fh32, out=out_f)
        p32.adjoint(f32, out=out_fh)

    ms32_amort = max_over_ranks(timed(fwdadj32, args.steps))

    # stage breakdown of one FP32 step (events on the plan stream)
    p32.set_nodes(x)
    p32.forward(fh32, out=out_f)
    st_f = p32.stage_times()
    p32.adjoint(f32, out=out_fh)
    st_a = p32.stage_times()
    stages32 = {"bin_ms": st_f["bin"] * 1e3, "fwd_roc_ms": st_f["roc"] * 1e3, "fwd_fft_ms": st_f["fft"] * 1e3,
                "fwd_interp_ms": st_f["conv"] * 1e3, "adj_spread_ms": st_a["conv"] * 1e3,
                "adj_fft_ms": st_a["fft"] * 1e3, "adj_roc_ms": st_a["roc"] * 1e3}

    # ---------------- dominant-kernel roofline (spreading and interpolation alone) ----------------
    grid = p32.grid()
    reps = 5
    for _ in range(2):
        grid.zero_()
        p32.spread(f32, grid)
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ks_ms = []
    for _ in range(reps):
        grid.zero_()
        k0.record(stream)
        p32.spread(f32, grid)
        k1.record(stream)
        k1.synchronize()
        ks_ms.append(k0.elapsed_time(k1))
    ki_ms = []
    for _ in range(reps):
        k0.record(stream)
        p32.interp(grid, out=out_f)
        k1.record(stream)
        k1.synchronize()
        ki_ms.append(k0.elapsed_time(k1))
    spread_ms = statistics.median(ks_ms)
    interp_ms = statistics.median(ki_ms)
    n_total = 256 ** 3
    c32 = 8
    alg_bytes = M * (8 * 3 + c32) + n_total * c32   # nodes + samples + grid, counted once
    W3 = (2 * M_CUT + 2) ** 3
    peak, peak_kind = load_peaks()
    dominant = "spread" if spread_ms >= interp_ms else "interp"
    dom_ms = max(spread_ms, interp_ms)
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    traffic = load_traffic().get(f"{dominant}_fp32_3d_full")
    # algorithmic flops per pass: a weight product and a complex x real FMA pair per tap,
    # plus one evaluation per tap and dimension; FP32 CUDA-core peak (nominal)
    flops = M * W3 * 5 + M * 3 * (2 * M_CUT + 2)
    fp32_peak_tflops = 152 * 128 * 2 * 2.07e9 / 1e12
    # the tensor-core formulation's MMA work: per node E0 E1 (plane, row) pairs times
    # 2 E2 (column, re|im) outputs, 2 flops each, for the three FP16 products; of it
    # the useful part is the node's own window, W^3 taps x 2 (re|im) x 2 flops x 3
    Wt = 2 * M_CUT + 2
    T = p32.tiling()["T"]
    E0, E1, E2 = T[0] + Wt - 1, T[1] + Wt - 1, T[2] + Wt - 1
    mma_flops = M * E0 * E1 * 2 * E2 * 2 * 3
    useful_flops = M * W3 * 2 * 2 * 3
    tpeak, tpeak_kind = load_tensor_peak()
    tensor_roof = {"issued_mma_flops_per_launch": mma_flops, "useful_mma_flops_per_launch": useful_flops,
                   "achieved_tflops_issued": round(mma_flops / (dom_ms * 1e-3) / 1e12, 1),
                   "achieved_tflops_useful": round(useful_flops / (dom_ms * 1e-3) / 1e12, 1),
                   "peak_tflops": tpeak, "peak_source": tpeak_kind,
                   "frac_issued": round(mma_flops / (dom_ms * 1e-3) / 1e12 / tpeak, 4),
                   "frac_useful": round(useful_flops / (dom_ms * 1e-3) / 1e12 / tpeak, 4),
                   "note": "FP16 hi/lo products hi*hi + hi*lo + lo*hi on tcgen05 kind::f16. Issued: the padded tile's "
                           "E0 E1 rows x 2 E2 columns per node (padding rows and columns of the MMA tiles not "
                           "counted); useful: the node's own W^3 window"}
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                "compute": {"algorithmic_flops_per_launch": flops,
                            "achieved_tflops": round(flops / (dom_ms * 1e-3) / 1e12, 2),
                            "peak_tflops": round(fp32_peak_tflops, 1),
                            "peak_source": "nominal FP32 CUDA-core peak, 152 SMs x 128 lanes x 2 flop x 2.07 GHz",
                            "frac": round(flops / (dom_ms * 1e-3) / 1e12 / fp32_peak_tflops, 4)},
                "tensor": tensor_roof,
                "spread_ms": round(spread_ms, 4), "interp_ms": round(interp_ms, 4),
                "taps_per_s": {"spread": M * W3 / (spread_ms * 1e-3), "interp": M * W3 / (interp_ms * 1e-3)}}

    # ---------------- FP64 plain form ----------------
    p64 = NFFT(N3, m=M_CUT, precision="f64", device=dev)
    o64f = torch.empty(M, dtype=torch.complex128, device=dev)
    o64h = torch.empty(N3, dtype=torch.complex128, device=dev)

    def step64():
        p64.set_nodes(x)
        p64.forward(fh64, out=o64f)
        p64.adjoint(f64, out=o64h)

    for _ in range(3):
        step64()
    k64 = max(20, args.steps)
    ms64 = max_over_ranks(timed(step64, k64))

    # ---------------- accuracy against the FP64 NDFT, and of the FP32 kernels against the FP64 form ----------------
    gsub = torch.Generator(device=dev).manual_seed(7)
    idx = torch.randperm(M, generator=gsub, device=dev)[:4096]
    kidx = torch.randperm(n_total // 8, generator=gsub, device=dev)[:4096]
    sub = NFFT(N3, m=M_CUT, precision="f64", device=dev).set_nodes(x[idx].contiguous())
    nd_f = sub.ndft_forward(fh64)
    nd_h = p64.ndft_adjoint_at(f64, kidx)
    p32.set_nodes(x)
    r32f = p32.forward(fh32)
    r32h_full = p32.adjoint(f32)
    r32h = r32h_full.reshape(-1)[kidx]
    r64f = o64f[idx]
    r64h = o64h.reshape(-1)[kidx]
    err = {"fp32_forward": rel_l2(nd_f, r32f[idx]), "fp32_adjoint": rel_l2(nd_h, r32h),
           "fp64_forward": rel_l2(nd_f, r64f), "fp64_adjoint": rel_l2(nd_h, r64h)}
    # the FP32 form against the FP64 form on the same nodes, window and inputs (all 2^21
    # samples, all 128^3 coefficients): the FP32 kernels' own error, which the window
    # error against the NDFT (about 1e-6 at m = 6) would hide
    err_form = {"forward": rel_l2(o64f, r32f), "adjoint": rel_l2(o64h, r32h_full)}
    # the gridding kernels alone, FP32 against FP64 on identical inputs: interpolation of
    # the FP64 forward's post-FFT grid (rounded to c64 for the FP32 kernel), spreading of
    # the samples into a cleared grid; no FFT, roll-off or input rounding in between
    p64.set_nodes(x)
    p64.forward(fh64, out=o64f)
    g64 = p64.grid().clone()
    i64 = p64.interp(g64)
    i32 = p32.interp(g64.to(torch.complex64))
    s64 = p64.spread(f64)
    s32 = p32.spread(f32)
    err_grid = {"interp": rel_l2(i64, i32), "spread": rel_l2(s64, s32),
                "note": "FP32 tensor-core gridding (FP16 hi/lo x3, FP32 accumulate) against the FP64 gridding on "
                        "the same nodes, grid and samples: the kernels' own error"}
    del g64, i64, i32, s64, s32
    p64.forward(fh64, out=o64f)
    sub.close()

    # ---------------- ES window (cunfft_x_set_window): same step, same NDFT subsamples ----------------
    p64.set_window("es")
    p32.set_window("es")
    step64()
    ms64_es = max_over_ranks(timed(step64, k64))
    step32()
    ms32_es = max_over_ranks(timed(step32, args.steps))
    es_r32f = p32.forward(fh32)
    es_r32h = p32.adjoint(f32)
    es = {"window": "exponential of semicircle, alpha = m + 1/2, beta = 0.97 pi (2m+1)(1 - 1/(2 sigma))",
          "fp32": {"value": replica_points_per_s(M, world, ms32_es), "ms_per_step": ms32_es, "steps": args.steps,
                   "rel_l2_vs_ndft": {"forward": rel_l2(nd_f, es_r32f[idx]),
                                      "adjoint": rel_l2(nd_h, es_r32h.reshape(-1)[kidx])},
                   "rel_l2_vs_fp64_form": {"forward": rel_l2(o64f, es_r32f), "adjoint": rel_l2(o64h, es_r32h)}},
          "fp64": {"value": replica_points_per_s(M, world, ms64_es), "ms_per_step": ms64_es, "steps": k64,
                   "rel_l2_vs_ndft": {"forward": rel_l2(nd_f, o64f[idx]), "adjoint": rel_l2(nd_h, o64h.reshape(-1)[kidx])}},
          "ratio_fp32_vs_fp64": ms64_es / ms32_es}
    p64.set_window("gaussian")
    p32.set_window("gaussian")
    p32.set_nodes(x)

    # ---------------- end to end through the C ABI from pinned host buffers ----------------
    # cunfft_x_forward_host / cunfft_x_adjoint_host: nodes, coefficients and samples
    # upload and download on the plan's two copy streams, overlapped with its kernels;
    # host wall clock from an idle device to the last download landed in host memory.
    xh = x.cpu().pin_memory()
    fhh = fh32.cpu().pin_memory()
    fh_h_out = torch.empty(N3, dtype=torch.complex64).pin_memory()
    fin_h = f32.cpu().pin_memory()
    fout_h = torch.empty(M, dtype=torch.complex64).pin_memory()

    def step_e2e():
        p32.forward_host(fhh, fout_h, x=xh)
        p32.adjoint_host(fin_h, fh_h_out)

    for _ in range(warm):
        step_e2e()
    p32.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    p32.synchronize()
    ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
    e2e_err = {"forward": rel_l2(r32f.cpu(), fout_h), "adjoint": rel_l2(r32h_full.cpu().reshape(-1),
                                                                       fh_h_out.reshape(-1))}
    h2d = xh.numel() * 8 + fhh.numel() * 8 + fin_h.numel() * 8
    d2h = fout_h.numel() * 8 + fh_h_out.numel() * 8
    launches_per_step = (4 + 2 + 2 + (1 if p32.spread_kernel() == "tensor" else 0)
                         + interp_prep_launches(p32))
    tiling = p32.tiling()
    p32.close()
    p64.close()

    # ---------------- the other workloads, each a parity-checked leg of its own ----------------
    legs = {}
    if not args.no_configs:
        legs["clustered_2d"] = leg_clustered_2d(dev, args.steps, timed)
        legs["batched_2d"] = leg_batched_2d(dev, args.steps, timed)
        legs["autograd_2d"] = leg_autograd_2d(dev, args.steps, timed)

    # ---------------- CPU baselines (rank 0, N = 1): the reference method and the direct NDFT ----------------
    cpu = cpu_ndft = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_reference_method(x, fh64, f64, steps=2)
        cpu_ndft = cpu_ndft_baseline(x, fh64, f64)

    result = {
        "metric": METRIC, "value": replica_points_per_s(M, world, ms32_max), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": ms32_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64: gridding on tcgen05 kind::f16 with FP16 hi/lo operands, three products "
                 "(hi*hi + hi*lo + lo*hi) per tap, FP32 accumulate; FP32 FFT; FP64 node reduction and "
                 "roll-off factors",
        "data": "synthetic (seeded uniform nodes and coefficients, the reference's 3D workload shape)",
        "config": {"workload": "3D NFFT fwd+adj, N=128^3, n=256^3 (sigma=2), Gaussian m=6, M=2^21 uniform nodes",
                   "step": "bin nodes + forward + adjoint", "form": "FP32", "parallelism": f"replicas x{world}",
                   "l2_cache": "working set (grid 134 MB + nodes 50 MB + coefficients/samples 34 MB) exceeds L2",
                   "tiling": tiling, "autotuned": tuned is not None},
        "sustained": {"value": replica_points_per_s(M, world, ms32_sus_max), "ms_per_step": ms32_sus_max,
                      "steps": sus_steps, "seconds": ms32_sus_max * sus_steps * 1e-3,
                      "note": "the headline step repeated back to back for at least --sustain-s seconds right "
                              "after the headline steps; the clock record covers both"},
        "binning_amortised": {"value": replica_points_per_s(M, world, ms32_amort), "ms_per_step": ms32_amort,
                              "step": "forward + adjoint on an already-binned node set"},
        "fp64_plain": {"value": replica_points_per_s(M, world, ms64), "ms_per_step": ms64, "steps": k64},
        "ratio_fp32_vs_fp64": ms64 / ms32_max,
        "es_window": es,
        "rel_l2_vs_ndft": err,
        "rel_l2_fp32_vs_fp64_form": err_form,
        "rel_l2_fp32_vs_fp64_gridding": err_grid,
        "stages_fp32": stages32,
        "e2e": {"value": replica_points_per_s(M, world, ms_e2e), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e,
                "path": "cunfft_x_forward_host + cunfft_x_adjoint_host (C ABI) from pinned host buffers, "
                        "copies on two copy streams overlapped with the kernels; host wall clock",
                "rel_l2_vs_device_path": e2e_err},
        "roofline": roofline,
        # binning 4 (count, scan, scatter, items) + forward 2 (roll-off, interpolation)
        # + adjoint 2 (spreading, crop) + the sample permutation of the tensor-core
        # spreading + the grid split of the tensor-core interpolation
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clk,
        "configs": legs,
    }
    if cpu is not None:
        result["cpu_baseline"] = cpu
        result["cpu_ndft"] = cpu_ndft
        result["fp64_vs_cpu_ratio"] = replica_points_per_s(M, world, ms64) / cpu["value"]
        result["fp32_vs_cpu_ratio"] = replica_points_per_s(M, world, ms32_max) / cpu["value"]
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def interp_prep_launches(p):
    """Launches per forward that prepare the tensor-core interpolation's operands (the
    grid's padded FP16 hi/lo planes, one kernel)."""
    return 1 if p.interp_kernel() == "tensor" else 0


def _crand_t(shape, rng, dev, dtype):
    import torch
    a = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    return torch.from_numpy(a).to(dev, dtype)


def clustered_nodes(rng):
    """512 radial spokes x 1024 samples (uniform angles in [0, pi), radius in [-0.5, 0.5))
    plus 2^18 nodes from an isotropic Gaussian (std 0.02) at the origin, wrapped to the torus."""
    import numpy as np
    spokes, samples = 512, 1024
    theta = np.pi * np.arange(spokes) / spokes
    r = -0.5 + np.arange(samples) / samples
    rad = np.stack([np.outer(np.cos(theta), r).ravel(), np.outer(np.sin(theta), r).ravel()], axis=1)
    gs = rng.normal(0.0, 0.02, (1 << 18, 2))
    gs = np.mod(gs + 0.5, 1.0) - 0.5
    return np.concatenate([rad, gs])


def leg_clustered_2d(dev, steps, timed):
    """2D clustered nodes, N = 512^2, n = 1024^2, m = 6, M = 786,432: FP32 and FP64 forms, a
    step being bind + forward + adjoint; errors against the FP64 NDFT on 2048 nodes and
    2048 coefficients, and of the FP32 form against the FP64 form."""
    import numpy as np
    import torch

    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(303)
    N = [512, 512]
    x = torch.from_numpy(clustered_nodes(rng)).to(dev)
    M = x.shape[0]
    fh64 = _crand_t(N, rng, dev, torch.complex128)
    f64 = _crand_t(M, rng, dev, torch.complex128)
    fh32, f32 = fh64.to(torch.complex64), f64.to(torch.complex64)
    out = {}
    res = {}
    for prec, fh, f in (("f32", fh32, f32), ("f64", fh64, f64)):
        p = NFFT(N, m=6, precision=prec, device=dev)
        of = torch.empty(M, dtype=fh.dtype, device=dev)
        oh = torch.empty(N, dtype=fh.dtype, device=dev)

        def step():
            p.set_nodes(x)
            p.forward(fh, out=of)
            p.adjoint(f, out=oh)

        for _ in range(3):
            step()
        ms = timed(step, steps)
        p.set_nodes(x)
        p.forward(fh, out=of)
        sf = p.stage_times()
        p.adjoint(f, out=oh)
        sa = p.stage_times()
        res[prec] = (of.clone(), oh.clone())
        out[prec] = {"value": M / (ms * 1e-3), "ms_per_step": ms, "steps": steps,
                     "stages_ms": {"bin": sf["bin"] * 1e3, "fwd_roc": sf["roc"] * 1e3, "fwd_fft": sf["fft"] * 1e3,
                                   "fwd_interp": sf["conv"] * 1e3, "adj_spread": sa["conv"] * 1e3,
                                   "adj_fft": sa["fft"] * 1e3, "adj_roc": sa["roc"] * 1e3},
                     "kernels": {"spread": p.spread_kernel(), "interp": p.interp_kernel()}}
        if prec == "f64":
            gsub = np.random.default_rng(3031)
            idx = torch.from_numpy(gsub.choice(M, 2048, replace=False)).to(dev)
            kidx = torch.from_numpy(gsub.choice(N[0] * N[1], 2048, replace=False)).to(dev)
            sub = NFFT(N, m=6, device=dev).set_nodes(x[idx].contiguous())
            nd_f = sub.ndft_forward(fh64)
            nd_h = p.ndft_adjoint_at(f64, kidx)
            sub.close()
        p.close()
    for prec in ("f32", "f64"):
        of, oh = res[prec]
        out[prec]["rel_l2_vs_ndft"] = {"forward": rel_l2(nd_f, of[idx]), "adjoint": rel_l2(nd_h, oh.reshape(-1)[kidx])}
    out["f32"]["rel_l2_vs_fp64_form"] = {"forward": rel_l2(res["f64"][0], res["f32"][0]),
                                         "adjoint": rel_l2(res["f64"][1], res["f32"][1])}
    out["workload"] = ("2D NFFT fwd+adj, N=512^2, n=1024^2, Gaussian m=6, M=786432: 512 radial spokes x 1024 "
                       "samples + 2^18 Gaussian (std 0.02) nodes at the origin")
    out["M"] = M
    out["ratio_fp32_vs_fp64"] = out["f64"]["ms_per_step"] / out["f32"]["ms_per_step"]
    return out


def leg_batched_2d(dev, steps, timed):
    """64 independent 2D instances, N = 256^2, n = 512^2, m = 5, per-instance M log-uniform in
    [1e3, 1e6], FP32: adjoint + forward replayed from captured CUDA graphs on a bound node set;
    errors against the FP64 NDFT on 2048 nodes / 2048 coefficients per instance, and of the
    FP32 form against the FP64 batched form."""
    import numpy as np
    import torch

    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(404)
    B, N, m = 64, [256, 256], 5
    Ms = np.round(10 ** rng.uniform(3, 6, B)).astype(np.int64)
    Mt = int(Ms.sum())
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (Mt, 2))).to(dev)
    fh64 = _crand_t([B] + N, rng, dev, torch.complex128)
    f64 = _crand_t(Mt, rng, dev, torch.complex128)
    fh32, f32 = fh64.to(torch.complex64), f64.to(torch.complex64)
    side = torch.cuda.Stream(dev)  # graph capture needs a non-default stream
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        p = NFFT(N, m=m, precision="f32", batch=B, device=dev).set_nodes(x, Ms.tolist())
        of = torch.empty(Mt, dtype=torch.complex64, device=dev)
        oh = torch.empty([B] + N, dtype=torch.complex64, device=dev)

        def step():
            p.adjoint_graph(f32, oh)
            p.forward_graph(fh32, of)

        for _ in range(3):
            step()  # the first call of each captures, the others replay
        side.synchronize()
    # time on the side stream (where the plan runs)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(side)
    with torch.cuda.stream(side):
        for _ in range(steps):
            step()
    ev1.record(side)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    with torch.cuda.stream(side):
        p.set_nodes(x, Ms.tolist())
        p.forward(fh32, out=of)
        sf = p.stage_times()
        p.adjoint(f32, out=oh)
        sa = p.stage_times()
        kinds = {"spread": p.spread_kernel(), "interp": p.interp_kernel()}
        p.close()
    side.synchronize()
    # FP64 batched form on the same inputs, and the FP64 NDFT on subsamples
    p64 = NFFT(N, m=m, batch=B, device=dev).set_nodes(x, Ms.tolist())
    of64 = p64.forward(fh64)
    oh64 = p64.adjoint(f64)
    sub_idx, off = [], 0
    for k in Ms:
        sub_idx.append(off + rng.choice(int(k), min(2048, int(k)), replace=False))
        off += int(k)
    sidx = torch.from_numpy(np.concatenate(sub_idx)).to(dev)
    sub = NFFT(N, m=m, batch=B, device=dev).set_nodes(x[sidx].contiguous(), [len(s) for s in sub_idx])
    nd_f = sub.ndft_forward(fh64)
    kidx = torch.from_numpy(rng.choice(N[0] * N[1], 2048, replace=False)).to(dev)
    nd_h = p64.ndft_adjoint_at(f64, kidx).reshape(B, -1)
    err = {"forward": rel_l2(nd_f, of[sidx]), "adjoint": rel_l2(nd_h, oh.reshape(B, -1)[:, kidx])}
    err_form = {"forward": rel_l2(of64, of), "adjoint": rel_l2(oh64, oh)}
    sub.close()
    p64.close()
    return {"workload": "64 x 2D NFFT adj+fwd, N=256^2, n=512^2, Gaussian m=5, per-instance M log-uniform in "
                        "[1e3, 1e6], FP32, graph replay on a bound node set",
            "M": Mt, "value": Mt / (ms * 1e-3), "ms_per_step": ms, "steps": steps,
            "step": "cunfft_x_adjoint_graph + cunfft_x_forward_graph (two graph launches)",
            "bin_ms": sf["bin"] * 1e3,
            "stages_ms": {"fwd_roc": sf["roc"] * 1e3, "fwd_fft": sf["fft"] * 1e3, "fwd_interp": sf["conv"] * 1e3,
                          "adj_spread": sa["conv"] * 1e3, "adj_fft": sa["fft"] * 1e3, "adj_roc": sa["roc"] * 1e3},
            "kernels": kinds, "rel_l2_vs_ndft": err, "rel_l2_vs_fp64_form": err_form}


def leg_autograd_2d(dev, steps, timed):
    """Differentiable 2D NFFT, N = 256^2, m = 6, M = 2^18 FP64 nodes: a step is the forward
    through NFFTFunction and the backward of ||A(x) f_hat - y||^2 (adjoint for f_hat, the
    derivative-of-window gridding for x); the gradients checked against the exact adjoint
    and against the FP64 NDFT gradient on 512 nodes."""
    import numpy as np
    import torch

    from cunfft_gb300.autograd import NFFTFunction
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(505)
    N, M, m = [256, 256], 1 << 18, 6
    x0 = rng.uniform(-0.5, 0.5, (M, 2))
    fh0 = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    xpert = np.mod(x0 + rng.normal(0, 1e-3, x0.shape) + 0.5, 1.0) - 0.5
    fhd = torch.from_numpy(fh0).to(dev)
    yp = NFFT(N, m=m, device=dev).set_nodes(torch.from_numpy(xpert).to(dev))
    y = yp.forward(fhd)
    yp.close()
    plan = NFFT(N, m=m, device=dev)
    xd = torch.from_numpy(x0).to(dev)
    state = {}

    def step():
        xx = xd.clone().requires_grad_(True)
        fh = fhd.clone().requires_grad_(True)
        loss = (NFFTFunction.apply(xx, fh, plan) - y).abs().pow(2).sum()
        loss.backward()
        state["gx"], state["gfh"] = xx.grad, fh.grad

    for _ in range(3):
        step()
    ms = timed(step, steps)
    with torch.no_grad():
        r = plan.set_nodes(xd).forward(fhd) - y
        g_fh = plan.adjoint(2 * r)
    err_fh = rel_l2(g_fh, state["gfh"])
    idx = rng.choice(M, 512, replace=False)
    sub = NFFT(N, m=m, device=dev).set_nodes(torch.from_numpy(x0[idx]).to(dev))
    k = [torch.arange(-(n // 2), n - n // 2, device=dev, dtype=torch.float64) for n in N]
    kk = torch.meshgrid(*k, indexing="ij")
    ref = np.zeros((512, 2))
    rj = r[torch.from_numpy(idx).to(dev)]
    for t in range(2):
        df = sub.ndft_forward((-2j * np.pi) * kk[t] * fhd)
        ref[:, t] = (torch.conj(2 * rj) * df).real.cpu().numpy()
    got = state["gx"].cpu().numpy()[idx]
    err_x = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    sub.close()
    plan.close()
    return {"workload": "2D NFFT in torch.autograd, N=256^2, n=512^2, Gaussian m=6, M=2^18 FP64 nodes, loss "
                        "||A(x) f_hat - y||^2",
            "M": M, "value": M / (ms * 1e-3), "ms_per_step": ms, "steps": steps,
            "step": "forward (NFFT) + loss + backward (adjoint NFFT + node gradient)",
            "rel_l2": {"grad_fhat_vs_adjoint": err_fh, "grad_x_vs_fp64_ndft_gradient": err_x}}


def cpu_reference_method(x, fh64, f64, steps=2):
    """The reference method (the oracle's FP64 restatement of the CUNFFT NFFT, OpenMP on
    all host cores) at the full benchmark size: roll-off, FFT and interpolation, then
    spreading, FFT and roll-off, timed over `steps` whole steps."""
    import oracle as O

    xs = x.cpu().numpy()
    fh = fh64.cpu().numpy()
    f = f64.cpu().numpy()
    cores = O.num_threads()
    ts = [_reference_step(O, xs, fh, f) for _ in range(steps)]
    t = statistics.median(ts)
    return {"value": xs.shape[0] / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the whole workload (M = {xs.shape[0]} nodes, N = 128^3): the reference method restated in "
                      f"C (oracle, FP64, OpenMP {cores} threads), {steps} full forward + adjoint steps, median "
                      f"{t:.2f} s"}


def _reference_step(O, xs, fh, f):
    n3 = [256, 256, 256]
    s = time.perf_counter()
    G = O.fft(O.roc_forward(fh, N3, n3, M_CUT), -1)
    O.interp(xs, G, N3, n3, M_CUT)
    Ga = O.fft(O.spread(xs, f, N3, n3, M_CUT), +1)
    O.roc_adjoint(Ga, N3, n3, M_CUT)
    return time.perf_counter() - s


def cpu_ndft_baseline(x, fh64, f64, sample=None):
    """FP64 direct NDFT on the host cores: forward on `sample` nodes and adjoint on
    `sample` coefficients, extrapolated to the full M nodes and N coefficients."""
    import numpy as np

    import oracle as O

    xs = x.cpu().numpy()
    fh = fh64.cpu().numpy()
    f = f64.cpu().numpy()
    cores = O.num_threads()
    if sample is None:
        sample = max(64, 8 * cores)
    rng = np.random.default_rng(3)
    idx = rng.choice(xs.shape[0], sample, replace=False).astype(np.int64)
    kidx = rng.choice(fh.size, sample, replace=False).astype(np.int64)
    t0 = time.perf_counter()
    O.ndft_forward_subset(xs, fh, N3, idx)
    t1 = time.perf_counter()
    O.ndft_adjoint_subset(xs, f, N3, kidx)
    t2 = time.perf_counter()
    t_full = (t1 - t0) * xs.shape[0] / sample + (t2 - t1) * fh.size / sample
    return {"value": xs.shape[0] / t_full, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"FP64 direct NDFT (oracle, OpenMP): forward on {sample} of {xs.shape[0]} nodes and adjoint on "
                      f"{sample} of {fh.size} coefficients, {t2 - t0:.1f} s measured, extrapolated linearly "
                      f"to the full transform pair ({t_full:.0f} s)"}


# ---------------------------------------------------------------------------
# reference arm: the reference method on the host CPU cores
# ---------------------------------------------------------------------------
def run_reference(args):
    import numpy as np

    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O

    cores = O.num_threads()
    rng = np.random.default_rng(20240)
    fh = rng.uniform(-1, 1, N3) + 1j * rng.uniform(-1, 1, N3)
    xs = rng.uniform(-0.5, 0.5, (M_FULL, 3))
    fs = rng.uniform(-1, 1, M_FULL) + 1j * rng.uniform(-1, 1, M_FULL)
    for _ in range(args.warmup):
        _reference_step(O, xs, fh, fs)
    t0 = time.perf_counter()
    ts = [_reference_step(O, xs, fh, fs) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    t_step = wall / max(1, args.steps)
    value = M_FULL / t_step
    sample = (f"the whole workload every step (M = {M_FULL} nodes, N = 128^3, no sampling or extrapolation): the "
              f"reference method restated in C (oracle, FP64, OpenMP {cores} threads), roll-off + FFT + "
              f"interpolation and spreading + FFT + roll-off; {args.steps} steps in {wall:.1f} s (median step "
              f"{statistics.median(ts):.2f} s)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
        "data": "synthetic (seeded uniform nodes and coefficients)",
        "config": {"workload": "3D NFFT fwd+adj, N=128^3, n=256^3 (sigma=2), Gaussian m=6, M=2^21 uniform nodes",
                   "form": "FP64 reference method on host CPU"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def spawn_local_ranks(args):
    """--gpus N without a launcher: run N local ranks of this script under
    torch.distributed.run (one per GPU); with a launcher, WORLD_SIZE must equal N."""
    if "WORLD_SIZE" in os.environ:
        world = int(os.environ["WORLD_SIZE"])
        if world != args.gpus:
            print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}", file=sys.stderr)
            sys.exit(2)
        return False
    if args.gpus <= 1 or args.impl == "reference":
        return False
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    sys.exit(subprocess.call(cmd))


def main():
    args = parse_args()
    spawn_local_ranks(args)
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
