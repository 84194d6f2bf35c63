"""Benchmark of the GB300 randomization-method summation.

Workload (one "step"): the 3-D anisotropic Exponential field -- var 2,
len_scale [20, 10, 5], 2000 modes drawn by the reference's RNG (inversion
sampling, stored in tests/golden/workloads.npz) -- summed on the structured
256^3 grid with unit spacing: 2000 * 16 777 216 = 3.36e10 mode*point
evaluations per step.

Metric: G mode*point evals/s of the fastest path at its stated error against
the FP64 kernel, with the plain FP64 kernel's throughput reported beside it.

* ``value``  -- device-resident inputs, CUDA-event timing of one step of the
                separable tensor-core path (per-axis tables + 3xTF32
                contraction; L2 flushed between steps);
* ``e2e``    -- the public API ``gstools_gb300.summate_grid`` called with host
                numpy arrays: host->device copy of the modes and axes, the
                kernels, and the device->host copy of the float32 field, all
                inside the timed region;
* ``f64_plain`` / ``other_paths`` -- the plain FP64 kernel (on a slab) and
                the mixed-precision pointwise kernel on the same workload;
* ``cpu_baseline`` -- the FP64 C/OpenMP oracle on a bounded slab of the same
                grid, all host cores;
* ``--impl reference`` -- the same oracle as the reference arm (the
                reference's own kernels are in the external gstools-cython
                package and cannot be built here), on the same config.

Multi-GPU (``torchrun --nproc-per-node N``): every rank runs the full
workload on its own GPU (replicas, weak scaling), timing is the max over
ranks.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("G mode·point evals/s at stated error vs FP64: plain FP64 vs "
          "mixed/batched")
UNIT = "G mode*point/s"
GRID = 256
N_MODES = 2000
VAR = 2.0
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2
# DRAM bytes (read + write) of one contraction launch on this workload, from
# the ncu capture summarised in profiles/grid_tc_kernel_exp3d_grid256.md.
TC_DRAM_BYTES_PER_LAUNCH = 34.4e6


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--grid", type=int, default=GRID)
    p.add_argument("--path", default="auto",
                   choices=["auto", "mixed", "tensor", "f64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def load_modes():
    data = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
    cov = data["exp3d/cov"]
    iso = data["exp3d/isometrize"]
    return iso.T @ cov, data["exp3d/z1"], data["exp3d/z2"]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.proc = None
        self.index = index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded),
                "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(cov, z1, z2, axes, target_s=10.0):
    """FP64 C/OpenMP oracle on a z-slab of the grid (all host cores)."""
    import oracle

    oracle.build()
    threads = oracle.num_threads()
    nx, ny, nz = (len(a) for a in axes)
    # calibrate on a small slab, then size the sample for ~target_s
    slab = 1
    x_sub = axes[0][:max(1, nx // 16)]
    grid = np.array(np.meshgrid(x_sub, axes[1], axes[2][:slab],
                                indexing="ij")).reshape(3, -1)
    t0 = time.perf_counter()
    oracle.c_summate(cov, z1, z2, grid)
    dt = time.perf_counter() - t0
    rate = cov.shape[1] * grid.shape[1] / max(dt, 1e-6)
    want_pts = int(rate * target_s / cov.shape[1])
    n_x = int(np.clip(want_pts // (ny * slab), 1, nx))
    grid = np.array(np.meshgrid(axes[0][:n_x], axes[1], axes[2][:slab],
                                indexing="ij")).reshape(3, -1)
    t0 = time.perf_counter()
    oracle.c_summate(cov, z1, z2, grid)
    dt = time.perf_counter() - t0
    value = cov.shape[1] * grid.shape[1] / dt / 1e9
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"FP64 C/OpenMP oracle, {cov.shape[1]} modes x "
                       f"{grid.shape[1]} grid points ({n_x}x{ny}x{slab} slab "
                       f"of the {nx}x{ny}x{nz} grid), {dt:.2f} s")}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cov, z1, z2 = load_modes()
    axes = [np.arange(float(args.grid))] * 3
    import oracle

    oracle.build()
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        base = cpu_baseline(cov, z1, z2, axes, target_s=6.0)
        if i >= args.warmup:
            vals.append(base["value"])
    value = statistics.median(vals)
    base["value"] = value
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"exp3d_grid{args.grid}_modes{N_MODES}",
                   "grid": [args.grid] * 3, "modes": N_MODES,
                   "model": "Exponential(dim=3, var=2, len_scale=[20,10,5])",
                   "l2": "inputs smaller than L2; CPU run"},
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("reference summators (gstools-cython / gstools_core) are "
                 "external to the reference tree; the FP64 C/OpenMP "
                 "restatement of generator.py:193-199 stands in"),
    }
    print(json.dumps(line), flush=True)


def tensor_peak():
    """Measured dense bf16 tensor peak (TFLOP/s) and where it came from."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def run_ours(args):
    import torch

    from gstools_gb300 import _native, build
    import gstools_gb300 as gg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    build.build()
    _native.load()

    cov, z1, z2 = load_modes()
    n = args.grid
    axes = [np.arange(float(n))] * 3
    n_pts = n ** 3
    work = N_MODES * n_pts
    scale = float(np.sqrt(VAR / N_MODES))
    path = "tensor" if args.path == "auto" else args.path

    d_cov = torch.from_numpy(np.ascontiguousarray(cov)).to(dev)
    d_z1 = torch.from_numpy(z1).to(dev)
    d_z2 = torch.from_numpy(z2).to(dev)
    d_axes = torch.from_numpy(np.concatenate(axes)).to(dev)
    lens = (ctypes.c_int64 * 4)(n, n, n, 1)
    out32 = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    ws_bytes = ctypes.c_size_t(0)
    _native.call("gst_grid_tc_workspace_size", 3, N_MODES, lens,
                 ctypes.byref(ws_bytes))
    ws = torch.empty(max(ws_bytes.value, 1), dtype=torch.uint8, device=dev)

    def p(t):
        return ctypes.c_void_p(t.data_ptr())

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        import torch.distributed as dist

        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def tc_tables():
        _native.call("gst_grid_tc_tables", 3, N_MODES, lens, p(d_axes),
                     p(d_cov), p(d_z1), p(d_z2), p(ws), ws_bytes, sp)

    def tc_contract():
        _native.call("gst_grid_tc_contract", 3, N_MODES, lens, p(ws),
                     ws_bytes, p(out32), _native.GST_OUT_F32, scale, sp)

    def step_mixed():
        _native.call("gst_summate_grid_mixed", 3, N_MODES, lens, p(d_axes),
                     p(d_cov), p(d_z1), p(d_z2), p(out32), _native.GST_OUT_F32,
                     scale, sp)

    if path == "tensor":
        parts = [tc_tables, tc_contract]
        launches_per_step = 2
        desc = "separable 3xTF32 tensor-core grid path (tables + contraction)"
    else:
        parts = [step_mixed]
        launches_per_step = 2
        desc = "mixed-precision pointwise grid kernel"

    def timed(parts, steps, warmup):
        """Per step: L2 flush, then events around each part."""
        for _ in range(warmup):
            for fn in parts:
                fn()
        torch.cuda.synchronize()
        barrier()
        per_part = [[] for _ in parts]
        totals = []
        for _ in range(steps):
            flush.fill_(1.0)
            evs = [torch.cuda.Event(enable_timing=True)
                   for _ in range(len(parts) + 1)]
            evs[0].record(stream)
            for i, fn in enumerate(parts):
                fn()
                evs[i + 1].record(stream)
            evs[-1].synchronize()
            for i in range(len(parts)):
                per_part[i].append(evs[i].elapsed_time(evs[i + 1]) / 1e3)
            totals.append(evs[0].elapsed_time(evs[-1]) / 1e3)
        torch.cuda.synchronize()
        barrier()
        return totals, per_part

    # -- headline ----------------------------------------------------------
    clocks = Clocks(local)
    clocks.start()
    totals, per_part = timed(parts, args.steps, args.warmup)
    clk = clocks.stop()
    t_step = max_over_ranks(statistics.mean(totals))
    value = world * work / t_step / 1e9
    t_main = max_over_ranks(statistics.mean(per_part[-1]))

    # -- error of the headline output vs the FP64 kernel on a sub-grid ------
    stride = max(1, n // 32)
    sub = [a[::stride] for a in axes]
    ref64 = gg.summate_grid(cov, z1, z2, sub, scale=scale)
    got = out32[::stride, ::stride, ::stride].double().cpu().numpy()
    diff = got - ref64
    sigma = np.sqrt(VAR)
    err = {"rms_sigma": float(np.sqrt(np.mean(diff**2)) / sigma),
           "max_abs_sigma": float(np.max(np.abs(diff)) / sigma),
           "vs": "FP64 grid kernel (reference op order)",
           "points": int(diff.size)}

    # -- the other paths, for the record ------------------------------------
    others = {}
    if path == "tensor":
        t_mx, _ = timed([step_mixed], 3, 1)
        others["mixed_pointwise"] = world * work / max_over_ranks(
            statistics.mean(t_mx)) / 1e9
    slab = max(1, n // 16)
    lens64 = (ctypes.c_int64 * 4)(slab, n, n, 1)
    out64 = torch.empty((slab, n, n), dtype=torch.float64, device=dev)

    def step_f64():
        _native.call("gst_summate_grid_f64", 3, N_MODES, lens64, p(d_axes),
                     p(d_cov), p(d_z1), p(d_z2), p(out64), sp)

    t64, _ = timed([step_f64], 2, 1)
    f64_value = world * N_MODES * slab * n * n / max_over_ranks(
        statistics.mean(t64)) / 1e9

    # -- end to end through the public API (host arrays in and out) --------
    method = "tensor" if path == "tensor" else "pointwise"

    def step_e2e():
        return gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                               method=method, out_dtype="float32",
                               scale=scale)

    for _ in range(2):
        res = step_e2e()
    torch.cuda.synchronize()
    barrier()
    e2e_times = []
    for _ in range(max(3, min(args.steps, 5))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = step_e2e()
        e2e_times.append(time.perf_counter() - t0)
    e2e_t = max_over_ranks(statistics.mean(e2e_times))
    h2d = cov.nbytes + z1.nbytes + z2.nbytes + sum(a.nbytes for a in axes)
    d2h = res.nbytes

    # -- roofline of the dominant kernel -------------------------------------
    sink = torch.zeros(256, dtype=torch.float32, device=dev)
    ops = ctypes.c_double(0.0)

    def probe(kind, iters):
        best = 0.0
        for _ in range(3):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            _native.call("gst_peak_probe", kind, iters, p(sink),
                         ctypes.byref(ops), sp)
            ev1.record(stream)
            ev1.synchronize()
            best = max(best, ops.value / (ev0.elapsed_time(ev1) / 1e3))
        return best

    peaks = {"fp32_tflops": probe(0, 4096) / 1e12,
             "fp64_tflops": probe(1, 64) / 1e12,
             "sfu_tops": probe(2, 512) / 1e12}
    if path == "tensor":
        peak, peak_src = tensor_peak()
        alg = 4.0 * work / t_main / 1e12
        n_pad = -(-N_MODES // 8) * 8
        executed = 12.0 * n_pad * (-(-n // 128) * 128) * n * n / t_main / 1e12
        roof = {"bound": "tensor", "achieved": alg, "peak": peak,
                "unit": "TFLOP/s", "frac": alg / peak,
                "traffic": TC_DRAM_BYTES_PER_LAUNCH,
                "traffic_note": ("dram read+write bytes per contraction "
                                 "launch (ncu); the 67 MB float32 field "
                                 "stays in L2 at launch end"),
                "kernel": "grid_tc_kernel (contraction)",
                "kernel_ms": t_main * 1e3,
                "note": (f"achieved = 4 algorithmic flops per mode*point "
                         f"(Re of a complex MAC) / contraction time; peak = "
                         f"{peak_src} dense bf16; the kernel executes "
                         f"{executed:.0f} TFLOP/s of TF32 MMAs (3xTF32 "
                         f"split, padded), TF32 runs at half the bf16 rate")}
    else:
        alg = 10.0 * work / t_main / 1e12
        roof = {"bound": "fp32", "achieved": alg, "peak": peaks["fp32_tflops"],
                "unit": "TFLOP/s", "frac": alg / peaks["fp32_tflops"],
                "traffic": None, "kernel": "pointwise_kernel (mixed)",
                "note": "10 algorithmic flops per mode*point vs measured FP32"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("tf32x3 (fp32 accumulate)" if path == "tensor"
                  else "fp32 + exact turn reduction"),
        "data": "synthetic (modes from the reference RNG, fixture)",
        "config": {
            "workload": f"exp3d_grid{n}_modes{N_MODES}",
            "model": "Exponential(dim=3, var=2, len_scale=[20,10,5])",
            "grid": [n, n, n], "modes": N_MODES,
            "mode_points_per_step": work,
            "path": desc,
            "output": "float32, scaled by sqrt(var/N)",
            "l2": "512 MB buffer written between timed steps",
            "parallelism": f"replicas x{world}",
        },
        "error_vs_fp64": err,
        "f64_plain": {"value": f64_value, "unit": UNIT,
                      "sample": f"{slab}x{n}x{n} slab, FP64 grid kernel",
                      "value_over_f64": value / f64_value},
        "other_paths": others,
        "e2e": {"value": world * work / e2e_t / 1e9, "unit": UNIT,
                "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": roof,
        "measured_peaks": peaks,
        "clocks": clk,
        "gpu_launches": launches_per_step * args.steps,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cov, z1, z2, axes)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
