"""Benchmark of the TGV-DCT deshade hot path on one GB300 (or N independent replicas).

Workload (the 256x256x192 full deshade): the 5-class tissue phantom times a smooth
bias exp(b), Rician-like noise (seed 2), taken to the log domain; 1500 TGV2-L1
iterations (lambda=1, alpha0=2, alpha1=1, reference steps tau=sigma=1/sqrt(20)),
then the DCT Poisson integration of v and r = u - l.  One "step" is one whole
deshade of the volume.  Metric: voxel-iterations per second.

  value  device-timed, input already in HBM, through tgvdct_process_dev
  e2e    the reference-facing call tgvdct_process_tgv2_l1 with host buffers
         (host->device copy of f and device->host copies of u, l, r inside)
  roofline  the TGV iteration kernels, timed live with CUDA events on the stream
         they run on; algorithmic bytes per voxel-iteration from ALGO_BYTES

``--impl reference`` times the reference algorithm's CPU restatement (the oracle
port; the reference itself has no CPU path) on the host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # name: (D, H, W, iterations)
    "deshade_256x256x192": (192, 256, 256, 1500),
    "deshade_128x128x128": (128, 128, 128, 2000),
}
# algorithmic bytes per voxel-iteration of one TGV2 iteration (read f, u, ubar, v3,
# vbar3, p3, q6; write u, ubar, v3, vbar3, p3, q6), by state precision
ALGO_BYTES = {0: 140, 1: 104, 2: 104}
# the shifted pass (primal of one iteration, dual of the next) keeps ubar and vbar on
# chip: read f, u, v3, p3, q6, write u, v3, p3, q6 (p, q in the dual element size)
ALGO_BYTES_SHIFTED = {0: 108, 1: 72, 2: 72}
KERNELS = {"shifted": 4, "fused": 2, "two_pass": 1}
ADJOINT_KERNELS = {"auto": 0, "two_pass": 1, "shifted": 4}
# the kernel a roofline line times, per --kernel
KERNEL_NAMES = {"shifted": "tgv_shifted_tma_kernel", "fused": "tgv_fused_tma_kernel",
                "two_pass": "tgv_dual_kernel + tgv_primal_kernel"}


def algo_bytes(kernel, precision):
    """Algorithmic bytes per voxel-iteration of the iteration kernel that runs."""
    return (ALGO_BYTES_SHIFTED if kernel == "shifted" else ALGO_BYTES)[precision]
# the extra measurements a default run adds to its line, in the order they run
EXTRAS = ["iteration_variants", "dct_poisson_256cube", "adjoint", "adjoint_256x256x192",
          "other_configs", "downsampled_deshade", "masked_deshade", "accuracy_vs_fp64"]
PREC_NAMES = {0: "fp32", 1: "bf16_dual", 2: "fx16_dual"}
DCT_MODES = {"fp32": 0, "tf32": 1, "bf16x3": 2}


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, period_ms=200):
        self.index, self.period_ms = index, period_ms
        self.proc, self.lines = None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", f"-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value, dist, device):
    """Time-like figure of the slowest rank (every rank calls; all receive the max).
    dist is torch.distributed or None (one process)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, ms):
    """Whole-job units per second: every replica processes units_per_rank in ms (the
    slowest rank's time)."""
    return world * units_per_rank / (ms * 1e-3)


def hbm_peak():
    try:
        with open(PEAKS_FILE) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def make_input(workload):
    from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
    d, h, w, _ = WORKLOADS[workload]
    return tissue_phantom_3d(d, h, w, seed=2)


# ---------------------------------------------------------------------------------
def cpu_reference(args, f, iterations_sample, threads=None):
    """The reference algorithm on the host cores (oracle port, FP32, OpenMP)."""
    import oracle
    cores = oracle.set_threads(threads or os.cpu_count() or 1)
    flog = np.log(f).astype(np.float32)
    t0 = time.perf_counter()
    oracle.tgv2_deshade(flog, 1.0, 2.0, 1.0, iterations_sample, dtype=np.float32)
    dt = time.perf_counter() - t0
    return f.size * iterations_sample / dt, cores, dt


def run_reference_arm(args):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    f = make_input(args.workload)
    d, h, w, iters = WORKLOADS[args.workload]
    # bounded sample: a few iterations of the same volume per step
    sample_it = args.ref_sample_iterations
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_reference(args, f, 1)
    rates, cores = [], 1
    t_all = time.perf_counter()
    for _ in range(args.steps):
        r, cores, _ = cpu_reference(args, f, sample_it)
        rates.append(r)
    wall = time.perf_counter() - t_all
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": "voxel_iters_per_s", "value": value,
        "unit": "voxel-iter/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "shape_dhw": [d, h, w], "iterations": iters,
                   "sample_iterations_per_step": sample_it},
        "cpu_baseline": {"value": value, "unit": "voxel-iter/s", "cores": cores, "kind": "port",
                         "sample": f"{sample_it} TGV2-L1 iterations of the {d}x{h}x{w} volume "
                                   "per step (the reference has no CPU implementation; this is "
                                   "its kernel sequence restated in C++/OpenMP)"},
        "e2e": {"value": value, "unit": "voxel-iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------------
# DRAM bytes (read + write) of one launch of the iteration kernel on this workload,
# FP32 state: dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of that
# launch (the summaries are under profiles/).
TRAFFIC_256x256x192 = {("fused", 0): 914891776 + 801782528,
                       ("shifted", 0): 715630000 + 606720000}


def time_shifted_pass(pkg, torch, w, h, d, f, stream, precision=0, n_pass=100):
    """Milliseconds per launch of the shifted pass: tgvdct_tgv2_step_dev runs n iterations
    as one dual step, n - 1 shifted passes and one primal step, so the difference of
    runs of n_pass + 2 and 2 iterations is n_pass launches of the pass alone (CUDA events
    on `stream`)."""
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=1,
                             state_precision=precision, iteration_kernel=KERNELS["shifted"])
    L = pkg.lib()
    sh = ctypes.c_void_p(stream.cuda_stream)
    with pkg.Context(prm) as ctx:
        def run(n):
            assert L.tgvdct_state_init_dev(ctx._ctx, ctypes.c_void_p(f.data_ptr()), sh) == pkg.OK
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert L.tgvdct_tgv2_step_dev(ctx._ctx, n, sh) == pkg.OK
            e1.record(stream)
            torch.cuda.synchronize()
            assert ctx.loop_launches() == n + 1
            return e0.elapsed_time(e1)
        run(n_pass + 2)  # warm-up
        t_long = min(run(n_pass + 2) for _ in range(2))
        t_short = min(run(2) for _ in range(3))
        ctx.check_device_error(stream.cuda_stream)
    return (t_long - t_short) / n_pass


def time_iterations(pkg, torch, w, h, d, f, kernel, precision, n_it, stream):
    """Milliseconds per iteration of the TGV loop alone (CUDA events on `stream`)."""
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=n_it,
                             state_precision=precision, iteration_kernel=KERNELS[kernel])
    u, vx, vy, vz = (torch.empty_like(f) for _ in range(4))
    with pkg.Context(prm) as ctx:
        def run():
            ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr(),
                        stream=stream.cuda_stream)
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.check_device_error(stream.cuda_stream)
    return e0.elapsed_time(e1) / n_it


def time_dct_poisson(pkg, torch, stream, n=256, reps=10):
    """The 256^3 DCT Poisson solve per precision mode: ms per solve and flop rate
    (12 N^4 flops of the six contractions; three times that in tensor flops for BF16x3)."""
    from ambient_image_processor_gb300.phantoms import cosine_modes_rhs
    rhs = torch.from_numpy(cosine_modes_rhs(n, n, n, seed=3)).cuda()
    out = torch.empty_like(rhs)
    res = {}
    for mode, name in ((pkg.DCT_FP32, "fp32"), (pkg.DCT_TF32, "tf32"), (pkg.DCT_BF16X3, "bf16x3")):
        prm = pkg.default_params(width=n, height=n, depth=n, dct_mode=mode,
                                 poisson_eigen=pkg.EIGEN_ACCURATE)
        with pkg.Context(prm) as ctx:
            for _ in range(3):
                ctx.poisson_solve_dev(rhs.data_ptr(), out.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                ctx.poisson_solve_dev(rhs.data_ptr(), out.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ctx.check_device_error(stream.cuda_stream)
        ms = e0.elapsed_time(e1) / reps
        flops = 12.0 * n ** 4
        res[name] = {"ms": ms, "useful_tflops": flops / (ms * 1e-3) / 1e12,
                     "hbm_gbs": 48.0 * n ** 3 / (ms * 1e-3) / 1e9}
    return res


def time_other_configs(pkg, torch, stream):
    """The remaining configurations of the reference's benchmark set, device-timed:
    the 2-D 512x512 TGV2-L1 denoise (rectangles-and-ellipses phantom, noise 0.05,
    1000 iterations, tau = sigma = 1/sqrt(12), the 2-D operators) and the whole 3-D
    deshade of the 128^3 tissue phantom in the log domain (2000 iterations + DCT)."""
    import math
    from ambient_image_processor_gb300.phantoms import rectangles_ellipses_2d, tissue_phantom_3d
    res = {}
    f2 = torch.from_numpy(rectangles_ellipses_2d(512, 512, seed=1)).cuda()
    prm = pkg.default_params(width=512, height=512, depth=1, iteration_count=1000,
                             geometry=pkg.GEOMETRY_2D)
    prm.tau = prm.sigma = 1.0 / math.sqrt(12.0)
    u, vx, vy = (torch.empty_like(f2) for _ in range(3))
    with pkg.Context(prm) as ctx:
        run = lambda: ctx.run_dev(f2.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                                  None, stream=stream.cuda_stream)
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    res["denoise2d_512x512_1000it"] = {"ms": ms, "pixel_iters_per_s": 512 * 512 * 1000 / (ms * 1e-3)}
    f3 = torch.from_numpy(tissue_phantom_3d(128, 128, 128, seed=2)).cuda()
    prm = pkg.default_params(width=128, height=128, depth=128, iteration_count=2000)
    u, l, r = (torch.empty_like(f3) for _ in range(3))
    with pkg.Context(prm) as ctx:
        run = lambda: ctx.process_dev(f3.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                                      set_negative_values_to_zero=False, log_domain=True,
                                      stream=stream.cuda_stream)
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    res["deshade_128x128x128_2000it"] = {"ms": ms,
                                          "voxel_iters_per_s": 128 ** 3 * 2000 / (ms * 1e-3)}
    return res


def time_downsampled(pkg, torch, stream):
    """The down-sampled deshade (TGVKDeshadeDownsampledProcessor, order 2) of the
    256x256x192 tissue phantom at factor 1/2, 1500 iterations, with an ellipsoid mask,
    the clamp and the background add-back (the reference CLI's settings), device-timed
    end to end; and the cubic B-spline resizes alone (down 256x256x192 -> 128x128x96,
    up back)."""
    import ctypes
    import numpy as np
    from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
    d, h, w = 192, 256, 256
    f = torch.from_numpy(tissue_phantom_3d(d, h, w, seed=2)).cuda()
    z, y, x = np.meshgrid(np.linspace(-1, 1, d), np.linspace(-1, 1, h), np.linspace(-1, 1, w),
                          indexing="ij")
    mask = torch.from_numpy(((x / 0.9) ** 2 + (y / 0.85) ** 2 + (z / 0.95) ** 2 < 1)
                            .astype(np.float32)).cuda()
    u, l, r = (torch.empty_like(f) for _ in range(3))
    alpha = np.array([1.0, 2.0], dtype=np.float32)
    sh = stream.cuda_stream
    L = pkg.lib()

    def run():
        pkg._check(L.tgvdct_process_tgvk_l1_downsampled_dev(
            f.data_ptr(), mask.data_ptr(), w, h, d, 0.5, 1.0, 2, alpha, 1500, 1, 1, 0, 0,
            pkg.CALLBACK(), None, u.data_ptr(), l.data_ptr(), r.data_ptr(), None, sh))

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    res = {"workload": "256x256x192 tissue phantom, factor 0.5 (128x128x96 loop), 1500 "
                       "iterations, ellipsoid mask, clamp and add-back"}
    ms = timed(run)
    res["ms"] = ms
    res["full_res_voxel_iters_per_s"] = w * h * d * 1500 / (ms * 1e-3)
    small = torch.empty((96, 128, 128), device="cuda")
    res["resize_down_ms"] = timed(lambda: pkg._check(L.tgvdct_resize_bspline3_dev(
        f.data_ptr(), w, h, d, small.data_ptr(), 128, 128, 96, sh)))
    res["resize_up_ms"] = timed(lambda: pkg._check(L.tgvdct_resize_bspline3_dev(
        small.data_ptr(), 128, 128, 96, u.data_ptr(), w, h, d, sh)))
    return res


def time_masked(pkg, torch, stream):
    """The masked deshade (TGVDeshadeMaskedProcessor) of the 256x256x192 tissue phantom
    with an ellipsoid mask (38% of the voxels inside), 1500 iterations, the clamp
    and the background add-back, device-timed; the loop runs the masked instance of
    the shifted pass."""
    import numpy as np
    from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
    d, h, w = 192, 256, 256
    f = torch.from_numpy(tissue_phantom_3d(d, h, w, seed=2)).cuda()
    z, y, x = np.meshgrid(np.linspace(-1, 1, d), np.linspace(-1, 1, h), np.linspace(-1, 1, w),
                          indexing="ij")
    m = ((x / 0.9) ** 2 + (y / 0.85) ** 2 + (z / 0.95) ** 2 < 1).astype(np.float32)
    mask = torch.from_numpy(m).cuda()
    u, l, r = (torch.empty_like(f) for _ in range(3))
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=1500)
    with pkg.Context(prm) as ctx:
        ctx.set_domain_mask_dev(mask.data_ptr(), stream.cuda_stream)
        run = lambda: ctx.process_dev(f.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                                      add_background_back=True, stream=stream.cuda_stream)
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.check_device_error()
    ms = e0.elapsed_time(e1)
    return {"workload": "256x256x192 tissue phantom, ellipsoid mask (%.0f%% inside), 1500 "
                        "iterations, clamp and add-back" % (100 * float(m.mean())),
            "ms": ms, "voxel_iters_per_s": w * h * d * 1500 / (ms * 1e-3)}


def time_adjoint(pkg, torch, stream, shape=(96, 96, 96), K=200, every=20, kernel=0):
    """Backward over forward time of the checkpointed reverse mode (default: 96^3,
    K = 200, checkpoints every 20).  `kernel` is the context's iteration kernel, which
    also picks the reverse sweep's passes (0, automatic: the fused adjoint pass for
    large volumes; 4, shifted passes: the fused adjoint pass always)."""
    from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
    d, h, w = shape
    f = torch.from_numpy(tissue_phantom_3d(d, h, w, bias=False, noise=0.05, rician=False,
                                           seed=4)).cuda()
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=K,
                             iteration_kernel=kernel)
    u, vx, vy, vz, gu, gf = (torch.empty_like(f) for _ in range(6))
    gu.normal_()
    gp = torch.empty(3, dtype=torch.float64, device=f.device)
    sh = stream.cuda_stream
    with pkg.Context(prm) as ctx:
        calls = {
            "forward": lambda: ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(),
                                           vy.data_ptr(), vz.data_ptr(), stream=sh),
            "forward_checkpointed": lambda: ctx.forward_checkpointed_dev(
                f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), every,
                sh),
            "backward": lambda: ctx.backward_dev(gu.data_ptr(), None, None, None, gf.data_ptr(),
                                                 gp.data_ptr(), sh),
        }
        for fn in calls.values():
            fn()
        torch.cuda.synchronize()
        out = {}
        for name, fn in calls.items():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out[name + "_ms"] = e0.elapsed_time(e1)
    out["backward_over_forward"] = out["backward_ms"] / out["forward_ms"]
    # the forward a gradient computation runs: the same loop keeping its checkpoints
    out["backward_over_forward_checkpointed"] = out["backward_ms"] / out["forward_checkpointed_ms"]
    out["workload"] = f"{w}x{h}x{d}, K = {K}, checkpoints every {every}"
    return out


def run_ours(args):
    import torch
    import ambient_image_processor_gb300 as pkg

    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("nccl")

    d, h, w, iters = WORKLOADS[args.workload]
    if args.iterations:
        iters = args.iterations
    V = d * h * w
    f_host = make_input(args.workload)
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=iters,
                             state_precision=args.precision, dct_mode=DCT_MODES[args.dct],
                             poisson_eigen=args.eigen, iteration_kernel=KERNELS[args.kernel],
                             z_chunk=args.z_chunk)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    dev = torch.device("cuda", local)
    f = torch.from_numpy(f_host).to(dev)
    u, l, r = (torch.empty_like(f) for _ in range(3))
    ctx = pkg.Context(prm)

    def step():
        ctx.process_dev(f.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                        set_negative_values_to_zero=False, log_domain=True, stream=sh)

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- the headline: whole deshades, input resident in HBM (state 1.6 GB > L2)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ctx.check_device_error(sh)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, dist, dev)
    value = replica_throughput(V * iters, world, ms)
    loop_launches = ctx.loop_launches()  # iteration kernels of one deshade (the last step)
    ctx.close()

    # ---- roofline of the iteration kernel, timed alone on its stream
    it_ms = time_iterations(pkg, torch, w, h, d, f, args.kernel, args.precision,
                            args.profile_iterations, stream)
    launches_per_it = 2 if args.kernel == "two_pass" else 1
    launch_ms = it_ms / launches_per_it
    if args.kernel == "shifted":  # the pass alone, without the steps around each run
        launch_ms = time_shifted_pass(pkg, torch, w, h, d, f, stream, args.precision)
    peak, peak_kind = hbm_peak()
    algo = algo_bytes(args.kernel, args.precision)
    # algorithmic bytes of one iteration per second of the dominant kernel
    achieved = algo * V / (launch_ms * launches_per_it * 1e-3) / 1e9
    traffic = TRAFFIC_256x256x192.get((args.kernel, args.precision)) \
        if args.workload == "deshade_256x256x192" else None

    # ---- e2e through the host-buffer C-ABI call (reference-facing)
    e2e_ms, e2e_calls, e2e_clocks = None, [], None
    if not args.no_e2e:
        # pinned host buffers (numpy views of page-locked torch tensors), as a caller
        # streaming volumes through the library would hold them
        pinned = [torch.from_numpy(np.ascontiguousarray(f_host)).pin_memory()]
        pinned += [torch.empty(f_host.shape, dtype=torch.float32).pin_memory() for _ in range(3)]
        fh, uo, lo, ro = (t.numpy() for t in pinned)
        times = []
        with ClockSampler(local) as e2e_clocks:
            for k in range(args.e2e_steps + 1):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                st = pkg.lib().tgvdct_process_tgv2_l1(ctypes.byref(prm), fh, None, 0, 0, 1,
                                                      pkg.CALLBACK(), None, uo, lo, ro)
                torch.cuda.synchronize()
                if st != pkg.OK:
                    raise RuntimeError(pkg.lib().tgvdct_last_error().decode())
                times.append(time.perf_counter() - t0)
        e2e_calls = [round(1e3 * t, 3) for t in times]  # the first builds the context
        e2e_ms = 1e3 * float(np.median(times[1:]))
    if not args.no_e2e:
        e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    e2e_value = replica_throughput(V * iters, world, e2e_ms) if e2e_ms else None

    line = None
    if rank == 0:
        extra = {}
        want = set(filter(None, args.extras.split(","))) or set(EXTRAS)
        if not args.no_variants:
            if "iteration_variants" in want:
                var = {}
                for kernel, prec in (("two_pass", 0), ("fused", 0), ("shifted", 0),
                                     ("two_pass", 2), ("fused", 2), ("fused", 1),
                                     ("shifted", 2), ("shifted", 1)):
                    t = time_iterations(pkg, torch, w, h, d, f, kernel, prec, 200, stream)
                    var[f"{kernel}_{PREC_NAMES[prec]}"] = {
                        "ms_per_iteration": t, "voxel_iters_per_s": V / (t * 1e-3),
                        "algorithmic_gbs": algo_bytes(kernel, prec) * V / (t * 1e-3) / 1e9}
                extra["iteration_variants"] = var
            if "dct_poisson_256cube" in want:
                extra["dct_poisson_256cube"] = time_dct_poisson(pkg, torch, stream)
            akern = ADJOINT_KERNELS[args.adjoint_kernel]
            if "adjoint" in want:
                extra["adjoint"] = time_adjoint(pkg, torch, stream, kernel=akern)
            if "adjoint_256x256x192" in want:
                extra["adjoint_256x256x192"] = time_adjoint(pkg, torch, stream, (192, 256, 256),
                                                            K=100, every=20, kernel=akern)
            if "other_configs" in want:
                extra["other_configs"] = time_other_configs(pkg, torch, stream)
            if "downsampled_deshade" in want:
                extra["downsampled_deshade"] = time_downsampled(pkg, torch, stream)
            if "masked_deshade" in want:
                extra["masked_deshade"] = time_masked(pkg, torch, stream)
        cpu = None
        if not args.no_cpu_baseline:
            rate, cores, dt = cpu_reference(args, f_host, args.cpu_sample_iterations)
            cpu = {"value": rate, "unit": "voxel-iter/s", "cores": cores, "kind": "port",
                   "sample": f"{args.cpu_sample_iterations} TGV2-L1 iterations of the same "
                             f"{d}x{h}x{w} log volume ({dt:.1f} s)"}
        if not args.no_variants and "accuracy_vs_fp64" in want:
            # last: the FP64 oracle occupies every host core for about two minutes
            extra["accuracy_vs_fp64"] = accuracy_vs_fp64(pkg, torch, f_host, iters, stream)
        # the loop; the six DCT contractions (the tensor-core passes take the divergence
        # as a kernel of its own); the epilogue; the log of f and the exp of u, l, r
        dct_launches = 6 if args.dct == "fp32" else 7
        gpu_launches = loop_launches + dct_launches + 1 + 4
        line = {
            "metric": "voxel_iters_per_s", "value": value, "unit": "voxel-iter/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == 0 else "f32+" + PREC_NAMES[args.precision],
            "data": "synthetic",
            "config": {"workload": args.workload, "shape_dhw": [d, h, w], "iterations": iters,
                       "state_precision": PREC_NAMES[args.precision], "dct": args.dct,
                       "poisson_eigen": "accurate" if args.eigen else "reference",
                       "iteration_kernel": args.kernel,
                       "l2": "inputs larger than L2 (TGV state 1.6 GB per replica)",
                       "parallelism": f"replicas{world}"},
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_value, "unit": "voxel-iter/s",
                    "h2d_bytes_per_step": V * 4, "d2h_bytes_per_step": 3 * V * 4,
                    "ms_per_step": e2e_ms, "call_ms": e2e_calls,
                    "clocks": e2e_clocks.summary() if e2e_clocks else None,
                    "call": "tgvdct_process_tgv2_l1, pinned host buffers; the library keeps "
                            "its context between calls (the first, untimed call builds it)"},
            "gpu_launches": gpu_launches * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": KERNEL_NAMES[args.kernel],
                         "algorithmic_bytes_per_launch": algo * V / launches_per_it,
                         "launch_ms": launch_ms,
                         "loop_ms_per_iteration": it_ms,
                         "peak_source": peak_kind},
            "cpu_baseline": cpu,
        }
        line.update(extra)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


# the precision forms whose error against the FP64 oracle the line reports:
# (state precision name, state precision, DCT mode, eigenvalue mode)
ACCURACY_FORMS = [("fp32", 0, "fp32", 0), ("fp32", 0, "fp32", 1), ("fp32", 0, "bf16x3", 1),
                  ("fp32", 0, "tf32", 1), ("fx16_dual", 2, "fp32", 1), ("bf16_dual", 1, "fp32", 1),
                  ("fx16_dual", 2, "bf16x3", 1)]
# the target bound on the relative L2 error (against FP64) of the corrected image and the
# shading field for a mixed-precision form
ACCURACY_TOL = 1e-4


def accuracy_vs_fp64(pkg, torch, f_host, iters, stream):
    """Error of the whole deshade against the FP64 oracle, per precision form.

    The FP64 oracle runs the same workload (log domain, no clamp) on the host cores
    (about two minutes at 256x256x192 x 1500 on 16 cores); each GPU form runs once.
    Returns the relative L2 error of the denoised image u, the shading field l and the
    corrected image r (all exponentiated back, as the user gets them), whether l and r
    meet ACCURACY_TOL, and the voxel-iterations per second of each form's deshade."""
    import oracle
    d, h, w = f_host.shape
    threads = oracle.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    ou, ol, orr = oracle.process_tgv2_l1(np.log(f_host.astype(np.float64)), 1.0, 2.0, 1.0, iters,
                                         set_negative_values_to_zero=False, dtype=np.float64)
    t_oracle = time.perf_counter() - t0
    ref = {"u": np.exp(ou), "l": np.exp(ol), "r": np.exp(orr)}
    del ou, ol, orr
    f = torch.from_numpy(f_host).cuda()
    u, l, r = (torch.empty_like(f) for _ in range(3))
    res = []
    for name, prec, dct, eig in ACCURACY_FORMS:
        prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=iters,
                                 state_precision=prec, dct_mode=DCT_MODES[dct],
                                 poisson_eigen=eig)
        with pkg.Context(prm) as ctx:
            # the first deshade builds the context's DCT plan; the second is timed
            for timed in (False, True):
                e0, e1 = (torch.cuda.Event(enable_timing=True),
                          torch.cuda.Event(enable_timing=True))
                e0.record(stream)
                ctx.process_dev(f.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                                set_negative_values_to_zero=False, log_domain=True,
                                stream=stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize()
            ctx.check_device_error(stream.cuda_stream)
        got = {"u": u.cpu().numpy(), "l": l.cpu().numpy(), "r": r.cpu().numpy()}
        err = {k: float(np.linalg.norm(got[k] - ref[k]) / np.linalg.norm(ref[k])) for k in ref}
        ms = e0.elapsed_time(e1)
        res.append({"state": name, "dct": dct, "eigen": "accurate" if eig else "reference",
                    "rel_l2": err, "meets_tol_l_r": err["l"] <= ACCURACY_TOL and
                    err["r"] <= ACCURACY_TOL, "ms_per_deshade": ms,
                    "voxel_iters_per_s": d * h * w * iters / (ms * 1e-3)})
    return {"tolerance_rel_l2": ACCURACY_TOL, "iterations": iters, "forms": res,
            "oracle": f"FP64 oracle on {threads} host threads, {t_oracle:.0f} s"}


def run_accuracy(args):
    """Only the error of every precision form against the FP64 oracle (one JSON line)."""
    import torch
    import ambient_image_processor_gb300 as pkg

    d, h, w, iters = WORKLOADS[args.workload]
    if args.iterations:
        iters = args.iterations
    res = accuracy_vs_fp64(pkg, torch, make_input(args.workload), iters,
                           torch.cuda.current_stream())
    print(json.dumps({"accuracy_vs_fp64": res, "workload": args.workload}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="deshade_256x256x192", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1, 2])
    # the headline integrates v with the tensor-core DCT (BF16 hi/lo products, FP32
    # accumulation) and the cancellation-free eigenvalues: within 6.3e-7 of the FP64
    # shading field, against 7.2e-6 for the reference's float formula
    ap.add_argument("--eigen", type=int, default=1, choices=[0, 1])
    ap.add_argument("--dct", default="bf16x3", choices=sorted(DCT_MODES))
    ap.add_argument("--kernel", default="shifted", choices=sorted(KERNELS))
    ap.add_argument("--adjoint-kernel", default="auto", choices=sorted(ADJOINT_KERNELS),
                    help="iteration kernel of the adjoint extras (it picks the reverse "
                         "sweep's passes: shifted forces the fused adjoint pass)")
    ap.add_argument("--z-chunk", type=int, default=0)
    ap.add_argument("--iterations", type=int, default=0, help="override the iteration count")
    ap.add_argument("--profile-iterations", type=int, default=200)
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-sample-iterations", type=int, default=100,
                    help="iterations of the CPU baseline sample in the ours line (~10 s)")
    ap.add_argument("--ref-sample-iterations", type=int, default=24,
                    help="iterations per step of the reference arm's CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--extras", default="",
                    help="comma-separated subset of the extra measurements (default: all of "
                         + ", ".join(EXTRAS) + ")")
    ap.add_argument("--accuracy", action="store_true",
                    help="error of every precision form against the FP64 oracle instead")
    args = ap.parse_args()
    unknown = sorted(set(filter(None, args.extras.split(","))) - set(EXTRAS))
    if unknown:  # before any device work
        ap.error(f"unknown --extras {unknown}; known: {', '.join(EXTRAS)}")
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.accuracy:
        return run_accuracy(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
