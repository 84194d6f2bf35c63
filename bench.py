"""Benchmark of the GB300 randomization-method summation.

Workload (one "step"): the 3-D anisotropic Exponential field -- var 2,
len_scale [20, 10, 5], 2000 modes drawn by the reference's RNG (inversion
sampling, stored in tests/golden/workloads.npz) -- summed on the structured
256^3 grid with unit spacing: 2000 * 16 777 216 = 3.36e10 mode*point
evaluations per step.

Metric: G mode*point evals/s of the fastest path at its stated error against
the FP64 oracle, with the plain FP64 kernel's throughput reported beside it.

* ``value``  -- device-resident inputs, CUDA-event timing of one step of the
                separable tensor-core path (per-axis tables + 3xFP16
                contraction, FP32 accumulation; L2 flushed between steps);
* ``error_vs_fp64`` -- the headline output against the FP64 C oracle: on a
                32^3 sub-grid recomputed here, and on the sub-grid the
                reference's own pipeline (its RNG, its isometrized meshgrid)
                evaluated when the fixture was made;
* ``e2e``    -- the public API ``gstools_gb300.summate_grid`` called with host
                numpy arrays: host->device copy of the modes and axes, the
                kernels, and the device->host copy of the float32 field, all
                inside the timed region (clocks sampled over it);
* ``e2e_reference_call`` -- the summation a structured ``SRF`` of the
                reference runs once ``install()`` routes it
                (``summate_structured``: unmapped modes, isometrize matrix,
                axes in; the float64 flat field the reference expects out);
* ``f64_plain`` / ``other_paths`` -- the plain FP64 kernel (on a slab), the
                mixed-precision pointwise kernel on the same workload, and
                bounded runs of the other four configurations (2-D points,
                512-realization ensemble, incompressible 192^3 field,
                gradients), each with its error against the oracle and its
                own clock record;
* ``cpu_baseline`` -- the FP64 C/OpenMP oracle on a bounded slab of the same
                grid, all host cores;
* ``--impl reference`` -- the same oracle as the reference arm (the
                reference's own kernels are in the external gstools-cython
                package and cannot be built here), on the same config: each
                step is a bounded slab of the grid; the line reports the
                throughput, the measured time of a step and the points it
                covered.

Defaults: 200 timed steps after 3 warm-up steps (about 70 ms of timed
work, so the 10 ms clock sampler sees the timed region); ``clocks`` reports
the samples taken inside it.

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
# DRAM bytes (read + write) of one contraction launch on this workload
# (dram__bytes_read.sum + dram__bytes_write.sum of grid_tc_kernel, one ncu
# capture of this build: 20.2 MB + 14.5 MB).
TC_DRAM_BYTES_PER_LAUNCH = 34.7e6


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default 200 for the headline grid, "
                        "10 for the other workloads)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--min-timed-s", dest="min_timed_s", type=float, default=0.25,
                   help="other workloads: the timed steps of the measurement "
                        "behind `value` go on until they span this many "
                        "seconds (at least --steps), so that the clock "
                        "samples fall inside the timed region")
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--grid", type=int, default=GRID)
    p.add_argument("--path", default="auto",
                   choices=["auto", "mixed", "tensor", "f64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-workloads", dest="workloads", action="store_false",
                   help="leave the bounded runs of the other configurations "
                        "out of the headline line")
    p.add_argument("--size", default="full", choices=["full", "small"],
                   help="small: reduced problem sizes of the krige and vario "
                        "workloads (for profiler captures)")
    p.add_argument("--operands", default="f16", choices=["f16", "tf32"],
                   help="operand format of the tensor-core split GEMM")
    p.add_argument("--workload", default="grid",
                   choices=["grid", "points", "ensemble", "incompr", "adjoint",
                            "krige", "vario"],
                   help="grid: the headline (3-D Exponential, 256^3, 2000 "
                        "modes); points: 2-D Gaussian, 100k points; ensemble: "
                        "512 Matern realizations; incompr: 3-D incompressible "
                        "field, 192^3; adjoint: gradients of a 3-D field; "
                        "krige: ordinary kriging; vario: empirical variogram")
    args = p.parse_args()
    if args.steps is None:
        args.steps = 200 if args.workload == "grid" else 10
    return args


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

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,"
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
                 "-lms", "10"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    @staticmethod
    def _stamp(text):
        import datetime

        try:
            return datetime.datetime.strptime(
                text, "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def stop(self, window=None):
        """Median SM clock and throttle reasons of the samples taken inside
        `window` = (t0, t1) (host time.time()), or of all samples when none
        falls inside it."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        rows = []
        for line in out.strip().splitlines():
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                row = (self._stamp(parts[0]), float(parts[1]), float(parts[2]),
                       {n for n, v in zip(names, parts[5:9])
                        if v.lower().startswith("active")})
            except ValueError:
                continue
            rows.append(row)
        inside = [r for r in rows if window is not None and r[0] is not None
                  and window[0] <= r[0] <= window[1]]
        use = inside or rows
        if not use:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [r[1] for r in use]
        loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded),
                "sm_max_mhz": max(r[2] for r in use),
                "reasons": sorted(set().union(*(r[3] for r in use))),
                "samples": len(use), "samples_in_timed_region": len(inside),
                "interval_ms": 10}


def workload_config(n, world):
    """The ``config`` of both arms' lines (identical keys and values)."""
    return {"workload": f"exp3d_grid{n}_modes{N_MODES}",
            "model": "Exponential(dim=3, var=2, len_scale=[20,10,5])",
            "grid": [n, n, n], "modes": N_MODES,
            "mode_points_per_step": N_MODES * n ** 3,
            "parallelism": f"replicas x{world}"}


def _grid_sample(axes, n):
    """The first n points of the grid spanned by axes (flattened "ij")."""
    shape = tuple(len(a) for a in axes)
    idx = np.unravel_index(np.arange(n), shape)
    return np.array([a[i] for a, i in zip(axes, idx)])


def cpu_baseline(cov, z1, z2, axes, target_s=10.0):
    """FP64 C/OpenMP oracle on the first points of the grid (flattened "ij"
    order), sized for about ``target_s`` seconds on all host cores."""
    import oracle

    oracle.build()
    threads = oracle.num_threads()
    shape = tuple(len(a) for a in axes)
    total = int(np.prod(shape))
    pts = _grid_sample(axes, min(total, 65536))
    t0 = time.perf_counter()
    oracle.c_summate(cov, z1, z2, pts)
    dt = time.perf_counter() - t0
    rate = cov.shape[1] * pts.shape[1] / max(dt, 1e-6)
    n = int(np.clip(rate * target_s / cov.shape[1], 1, total))
    pts = _grid_sample(axes, n)
    t0 = time.perf_counter()
    oracle.c_summate(cov, z1, z2, pts)
    dt = time.perf_counter() - t0
    value = cov.shape[1] * n / dt / 1e9
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "points_timed": n, "seconds": dt,
            "sample": (f"FP64 C/OpenMP oracle, {cov.shape[1]} modes x {n} "
                       f"grid points (the first {n} of the "
                       f"{'x'.join(map(str, shape))} grid), {dt:.2f} s on "
                       f"{threads} threads")}


def run_reference(args):
    """The reference arm: the FP64 C/OpenMP restatement of the reference's
    summate on the same workload, all host cores.  A step is a bounded slab
    of the grid (the same first points every step), sized so the whole run
    takes about two and a half minutes; ``value`` is its throughput and
    ``ms_per_step`` its measured time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cov, z1, z2 = load_modes()
    axes = [np.arange(float(args.grid))] * 3
    import oracle

    oracle.build()
    threads = oracle.num_threads()
    per_step_s = float(np.clip(150.0 / (args.warmup + args.steps), 0.2, 5.0))
    # size the slab once, then time every step on the same points
    probe = cpu_baseline(cov, z1, z2, axes, target_s=per_step_s)
    n = probe["points_timed"]
    pts = _grid_sample(axes, n)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.c_summate(cov, z1, z2, pts)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    t_step = statistics.mean(times)
    value = N_MODES * n / t_step / 1e9
    sample = (f"FP64 C/OpenMP oracle, {N_MODES} modes x {n} grid points (the "
              f"first {n} of the {args.grid}^3 grid) per step, {threads} "
              f"threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.grid, world),
        "points_timed": n,
        "full_grid_ms_extrapolated": N_MODES * args.grid ** 3 / (value * 1e9) * 1e3,
        "notes": {"step": "a bounded slab of the grid; value = its mode*point "
                          "throughput (linear in points)",
                  "l2": "CPU run", "output": "float64"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("reference summators (gstools-cython / gstools_core) are "
                 "external to the reference tree; the FP64 C/OpenMP "
                 "restatement of generator.py:193-199 stands in"),
    }
    print(json.dumps(line), flush=True)


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s), or None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


# GB300's nominal FP64 rate: 2 DFMA per clock per SM x 152 SMs x 2.07 GHz.
# The FMA-chain probe (gst_peak_probe kind 1) tops out near 1.0 TFLOP/s,
# below the 1.15 TFLOP/s the kriging GEMM sustains (ncu: FP64 pipe 94 % busy),
# so FP64 fractions are quoted against the nominal figure.
FP64_NOMINAL_TFLOPS = 1.25


def peak_probe(torch, kind, iters):
    """Best of three timed launches of gst_peak_probe (after one untimed):
    0 FP32 FMA, 1 FP64 FMA (flop/s), 2 SFU sin (op/s), on the current stream."""
    from gstools_gb300 import _native

    sink = torch.zeros(256, dtype=torch.float32, device="cuda")
    ops = ctypes.c_double(0.0)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    sk = ctypes.c_void_p(sink.data_ptr())
    _native.call("gst_peak_probe", kind, iters, sk, ctypes.byref(ops), sp)
    best = 0.0
    for _ in range(3):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        _native.call("gst_peak_probe", kind, iters, sk, ctypes.byref(ops), sp)
        ev1.record(stream)
        ev1.synchronize()
        best = max(best, ops.value / (ev0.elapsed_time(ev1) / 1e3))
    return best


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

    _native.set_tc_operands(args.operands)
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
        # grid_prep_kernel + grid_tables_kernel, then zero_split_tiles_kernel
        # (the 256 pair tiles leave a partial last wave) + grid_tc_kernel
        launches_per_step = 4
        desc = (f"separable 3x{args.operands.upper()} tensor-core grid path "
                f"(tables + contraction)")
    else:
        parts = [step_mixed]
        launches_per_step = 2   # pack_modes_kernel + pointwise_kernel
        desc = "mixed-precision pointwise grid kernel"

    window = [None, None]   # host time of the last timed region

    def timed(parts, steps, warmup):
        """Per step: L2 flush, then events around each part."""
        for _ in range(warmup):
            for fn in parts:
                fn()
        torch.cuda.synchronize()
        barrier()
        per_part = [[] for _ in parts]
        totals = []
        window[0] = time.time()
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
        window[1] = time.time()
        barrier()
        return totals, per_part

    # -- headline ----------------------------------------------------------
    clocks = Clocks(local)
    clocks.start()
    totals, per_part = timed(parts, args.steps, args.warmup)
    clk = clocks.stop(tuple(window))
    t_step = max_over_ranks(statistics.mean(totals))
    value = world * work / t_step / 1e9
    t_main = max_over_ranks(statistics.mean(per_part[-1]))

    # -- error of the headline output vs the FP64 oracle --------------------
    import oracle

    oracle.build()
    stride = max(1, n // 32)
    sub = [a[::stride] for a in axes]
    pts_sub = np.array(np.meshgrid(*sub, indexing="ij")).reshape(3, -1)
    ref64 = scale * oracle.c_summate(cov, z1, z2, pts_sub)
    got = out32[::stride, ::stride, ::stride].double().cpu().numpy().reshape(-1)
    diff = got - ref64
    sigma = np.sqrt(VAR)
    err = {"rms_sigma": float(np.sqrt(np.mean(diff**2)) / sigma),
           "max_abs_sigma": float(np.max(np.abs(diff)) / sigma),
           "vs": "FP64 C oracle (reference formula and operation order), "
                 "mapped modes on the raw sub-grid",
           "points": int(diff.size)}
    if n == GRID:
        # the sub-grid the reference's own pipeline evaluated (its RNG, its
        # isometrized meshgrid, the oracle as its summator) for the fixture
        wl = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
        ix = [torch.from_numpy(wl[f"exp3d/sub_{c}"].astype(np.int64)).to(dev)
              for c in "xyz"]
        got_ref = out32.index_select(0, ix[0]).index_select(1, ix[1]) \
            .index_select(2, ix[2])
        d_ref = got_ref.double().cpu().numpy().reshape(-1) - \
            scale * wl["exp3d/summed_sub"]
        err["reference_pipeline"] = {
            "rms_sigma": float(np.sqrt(np.mean(d_ref**2)) / sigma),
            "max_abs_sigma": float(np.max(np.abs(d_ref)) / sigma),
            "points": int(d_ref.size),
            "vs": "the reference's RandMeth on its isometrized meshgrid with "
                  "the FP64 oracle as summator (fixture)"}

    # -- the other paths, for the record ------------------------------------
    others = {}
    if path == "tensor":
        t_mx, _ = timed([step_mixed], 3, 1)
        others["mixed_pointwise"] = world * work / max_over_ranks(
            statistics.mean(t_mx)) / 1e9
        # the other operand format of the split GEMM, same workload
        alt = "tf32" if args.operands == "f16" else "f16"
        _native.set_tc_operands(alt)
        alt_bytes = ctypes.c_size_t(0)
        _native.call("gst_grid_tc_workspace_size", 3, N_MODES, lens,
                     ctypes.byref(alt_bytes))
        alt_ws = torch.empty(max(alt_bytes.value, 1), dtype=torch.uint8,
                             device=dev)

        def alt_tables():
            _native.call("gst_grid_tc_tables", 3, N_MODES, lens, p(d_axes),
                         p(d_cov), p(d_z1), p(d_z2), p(alt_ws), alt_bytes, sp)

        def alt_contract():
            _native.call("gst_grid_tc_contract", 3, N_MODES, lens, p(alt_ws),
                         alt_bytes, p(out32), _native.GST_OUT_F32, scale, sp)

        t_alt, _ = timed([alt_tables, alt_contract], 5, 2)
        _native.set_tc_operands(args.operands)
        others[f"tensor_{alt}_operands"] = world * work / max_over_ranks(
            statistics.mean(t_alt)) / 1e9
        del alt_ws
        # the 2-D form of the tensor-core path: 2-D Gaussian modes (1000,
        # reference RNG, fixture) on an 8192^2 grid, float32 output
        wl = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
        cov2, z12, z22 = wl["gau2d/cov"], wl["gau2d/z1"], wl["gau2d/z2"]
        n2, m2 = 8192, cov2.shape[1]
        lens2 = (ctypes.c_int64 * 4)(n2, n2, 1, 1)
        t2 = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
              for a in (np.concatenate([np.arange(float(n2))] * 2), cov2, z12, z22)]
        out2 = torch.empty((n2, n2), dtype=torch.float32, device=dev)
        ws2_bytes = ctypes.c_size_t(0)
        _native.call("gst_grid_tc_workspace_size", 2, m2, lens2,
                     ctypes.byref(ws2_bytes))
        ws2 = torch.empty(max(ws2_bytes.value, 1), dtype=torch.uint8, device=dev)

        def tables2():
            _native.call("gst_grid_tc_tables", 2, m2, lens2, p(t2[0]), p(t2[1]),
                         p(t2[2]), p(t2[3]), p(ws2), ws2_bytes, sp)

        def contract2():
            _native.call("gst_grid_tc_contract", 2, m2, lens2, p(ws2), ws2_bytes,
                         p(out2), _native.GST_OUT_F32, 1.0, sp)

        t_2d, _ = timed([tables2, contract2], 5, 2)
        others["tensor_2d_gau2d_grid8192_modes1000"] = world * m2 * n2 * n2 / \
            max_over_ranks(statistics.mean(t_2d)) / 1e9
        del ws2, out2
    slab = max(1, n // 16)
    lens64 = (ctypes.c_int64 * 4)(slab, n, n, 1)
    out64 = torch.empty((slab, n, n), dtype=torch.float64, device=dev)
    d_axes64 = torch.from_numpy(np.concatenate(
        [axes[0][:slab], axes[1], axes[2]])).to(dev)

    def step_f64():
        _native.call("gst_summate_grid_f64", 3, N_MODES, lens64, p(d_axes64),
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

    def host_timed(fn, calls, warmup=3):
        """Wall-clock time per call of fn (host inputs and result), L2
        flushed before each call, clocks sampled over the loop."""
        for _ in range(warmup):
            res = fn()
        torch.cuda.synchronize()
        barrier()
        ck = Clocks(local)
        ck.start()
        times = []
        t_begin = time.time()
        for _ in range(calls):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = fn()
            times.append(time.perf_counter() - t0)
        window_e2e = (t_begin, time.time())
        return res, max_over_ranks(statistics.mean(times)), ck.stop(window_e2e)

    e2e_calls = max(20, min(args.steps, 200))
    res, e2e_t, e2e_clk = host_timed(step_e2e, e2e_calls)
    h2d = cov.nbytes + z1.nbytes + z2.nbytes + sum(a.nbytes for a in axes)
    d2h = res.nbytes

    # -- the routed structured SRF call of the reference ---------------------
    # install() hands a structured SRF evaluation to summate_structured with
    # the generator's (unmapped) modes, the model's isometrize matrix and the
    # axis arrays, and returns the float64 flat sum the reference scales.
    wl = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
    cov_raw, iso = wl["exp3d/cov"], wl["exp3d/isometrize"]

    def step_routed():
        return gg.summate_structured(cov_raw, z1, z2, axes, iso,
                                     precision="mixed")

    res_r, routed_t, routed_clk = host_timed(step_routed, max(20, e2e_calls // 4))
    routed = {"value": world * work / routed_t / 1e9, "unit": UNIT,
              "ms_per_call": routed_t * 1e3, "calls": max(20, e2e_calls // 4),
              "h2d_bytes_per_step": int(cov_raw.nbytes + z1.nbytes + z2.nbytes
                                        + iso.nbytes
                                        + sum(a.nbytes for a in axes)),
              "d2h_bytes_per_step": int(res_r.nbytes),
              "output": "float64 (the reference's summator contract)",
              "clocks": routed_clk}
    del res_r

    # -- roofline of the dominant kernel -------------------------------------
    peaks = {"fp32_tflops": peak_probe(torch, 0, 4096) / 1e12,
             "fp64_tflops": peak_probe(torch, 1, 256) / 1e12,
             "sfu_tops": peak_probe(torch, 2, 512) / 1e12}
    if path == "tensor":
        peak, peak_src = tensor_peak()
        alg = 4.0 * work / t_main / 1e12
        mps = 32 if args.operands == "f16" else 16   # modes per pipeline stage
        n_pad = -(-N_MODES // mps) * mps
        nt = _native.grid_tile_cols(n)        # z tile width (MMA N)
        executed = 12.0 * n_pad * (-(-n // nt) * nt) * n * n / t_main / 1e12
        op_note = ("FP16 MMAs (3xFP16 split, padded), FP16 runs at the bf16 "
                   "rate" if args.operands == "f16" else
                   "TF32 MMAs (3xTF32 split, padded), TF32 runs at half the "
                   "bf16 rate")
        roof = {"bound": "tensor", "achieved": alg, "peak": peak,
                "unit": "TFLOP/s", "frac": alg / peak,
                "traffic": TC_DRAM_BYTES_PER_LAUNCH,
                "traffic_note": ("dram read+write bytes per contraction "
                                 "launch, from one ncu --set full capture of "
                                 "this build on this workload (a constant: "
                                 "no counter is read during a timed run); "
                                 "the 67 MB float32 field stays in L2 at "
                                 "launch end"),
                "kernel": "grid_tc_kernel (contraction)",
                "kernel_ms": t_main * 1e3,
                "note": (f"achieved = 4 algorithmic flops per mode*point "
                         f"(Re of a complex MAC) / contraction time; peak = "
                         f"{peak_src} dense bf16; the kernel executes "
                         f"{executed:.0f} TFLOP/s of {op_note}; the three-"
                         f"product hi/lo split executes 3 MMA flops per "
                         f"algorithmic flop, so frac is at most 1/3 (FP16) "
                         f"or 1/6 (TF32)")}
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
        "dtype": (f"{args.operands}x3 (fp32 accumulate)" if path == "tensor"
                  else "fp32 + exact turn reduction"),
        "data": "synthetic (modes from the reference RNG, fixture)",
        "config": workload_config(n, world),
        "notes": {"path": desc, "output": "float32, scaled by sqrt(var/N)",
                  "l2": "512 MB buffer written between timed steps"},
        "error_vs_fp64": err,
        "f64_plain": {"value": f64_value, "unit": UNIT,
                      "sample": f"{slab}x{n}x{n} slab, FP64 grid kernel",
                      "value_over_f64": value / f64_value},
        "other_paths": others,
        "e2e": {"value": world * work / e2e_t / 1e9, "unit": UNIT,
                "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "calls": e2e_calls, "ms_per_call": e2e_t * 1e3,
                "clocks": e2e_clk},
        "e2e_reference_call": routed,
        "roofline": roof,
        "measured_peaks": peaks,
        "clocks": clk,
        "gpu_launches": launches_per_step * args.steps,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cov, z1, z2, axes)
    if args.workloads and world == 1 and n == GRID:
        line["other_paths"]["configs"] = other_configs(args, torch, gg, flush)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)



# ---------------------------------------------------------------------------
# The other workloads (not the headline; run explicitly with --workload).
# Each prints one JSON line with the same timing rules.
# ---------------------------------------------------------------------------

# The timed region of the measurement a workload line's `value` comes from:
# host window (for the clock record) and the number of timed steps.
_MAIN = {"window": None, "steps": 0}


def _timed_events(torch, fn, steps, warmup, flush, main=False, min_s=0.0):
    """Mean CUDA-event time of `steps` calls of fn (L2 flushed before each)
    after `warmup` calls; with min_s > 0 the timed calls go on until they
    span at least min_s seconds, so that the clock sampler (10 ms period)
    sees the timed region.  main: record the window and step count in
    _MAIN."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    w0 = time.time()
    while len(times) < steps or time.time() - w0 < min_s:
        if flush is not None:
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    if main:
        _MAIN["window"] = (w0, time.time())
        _MAIN["steps"] = len(times)
    return statistics.mean(times)


def _line(args, workload, value, t_step, dtype, config, **extra):
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic", "config": dict(workload=workload, **config)}
    line.update(extra)
    return line


def _cpu_sample(fn, items, work_of, target_s=5.0, what="items", skip=False):
    """Time the oracle (all host cores) on the first items of a workload,
    growing the sample until it runs about target_s seconds or covers every
    item; returns a cpu_baseline dict in G mode*point/s."""
    if skip:
        return None
    import oracle

    oracle.build()
    done, t, n = 0, 0.0, 1
    while True:
        n = min(n, len(items))
        t0 = time.perf_counter()
        for it in items[:n]:
            fn(it)
        t = time.perf_counter() - t0
        done = sum(work_of(it) for it in items[:n])
        if t >= target_s * 0.3 or n == len(items):
            break
        n = max(n + 1, int(n * min(8.0, target_s / max(t, 1e-3))))
    return {"value": done / t / 1e9, "unit": UNIT, "cores": oracle.num_threads(),
            "kind": "port",
            "sample": f"FP64 C/OpenMP oracle on the first {n} of {len(items)} {what} "
                      f"({done:.3g} mode*point, {t:.2f} s)"}


def wl_krige(args, torch, gg, flush):
    """Ordinary kriging with an exponential covariance (var 1, length scale
    50): 1000 conditioning points and 65 536 target points uniform in
    [0, 500]^2; the kernels' inputs built the reference's way
    (src/gstools/krige/base.py:330-405): M = inverse of the bordered
    covariance matrix, V = covariances to the targets plus the unbiasedness
    row.  Work unit: the 2 (K+1)^2 n flops of the nested sums."""
    import oracle
    from scipy.spatial.distance import cdist

    rng = np.random.RandomState(20170519)
    n_cond, n_pts = (1000, 65536) if args.size == "full" else (1000, 16384)
    cpos = rng.uniform(0.0, 500.0, (2, n_cond))
    tpos = rng.uniform(0.0, 500.0, (2, n_pts))
    cond = np.append(rng.normal(size=n_cond), 0.0)
    cov = lambda h: np.exp(-h / 50.0)
    a = np.empty((n_cond + 1, n_cond + 1))
    a[:n_cond, :n_cond] = cov(cdist(cpos.T, cpos.T))
    a[n_cond, :n_cond] = a[:n_cond, n_cond] = 1.0
    a[n_cond, n_cond] = 0.0
    mat = np.linalg.inv(a)
    vecs = np.empty((n_cond + 1, n_pts))
    vecs[:n_cond] = cov(cdist(cpos.T, tpos.T))
    vecs[n_cond] = 1.0
    k = n_cond + 1
    flops = 2.0 * k * k * n_pts
    dev = torch.device("cuda", torch.cuda.current_device())
    dm, dv, dc = (torch.from_numpy(np.ascontiguousarray(x)).to(dev)
                  for x in (mat, vecs, cond))
    step = lambda: gg.calc_field_krige_and_variance(dm, dv, dc)
    t = _timed_events(torch, step, args.steps, args.warmup, flush, main=True,
                      min_s=args.min_timed_s)
    f, e = step()
    # the field alone: V^T (M^T c), one pass over V (HBM-bound)
    t_field = _timed_events(torch, lambda: gg.calc_field_krige(dm, dv, dc),
                            args.steps, args.warmup, flush)
    field_bytes = 8.0 * (k * k + k * n_pts + n_pts)
    hbm = hbm_peak()
    f_only = gg.calc_field_krige(dm, dv, dc)
    sample = 512
    t0 = time.perf_counter()
    fo, eo = oracle.c_krige(mat, vecs[:, :sample], cond)
    t_cpu = time.perf_counter() - t0
    _, _, scale = oracle.np_krige(mat, vecs[:, :sample], cond)
    err = float(max(np.max(np.abs(f[:sample].cpu().numpy() - fo) / scale),
                    np.max(np.abs(e[:sample].cpu().numpy() - eo) / scale),
                    np.max(np.abs(f_only[:sample].cpu().numpy() - fo) / scale)))
    t0 = time.perf_counter()
    fe = gg.calc_field_krige_and_variance(mat, vecs, cond)
    te2e = time.perf_counter() - t0
    peak64 = peak_probe(torch, 1, 256) / 1e12
    # the variance runs as FP16 tensor-core products of error-free slices of
    # M and V (6-bit digits, 9 slices, the 45 slice pairs of levels 2..10,
    # inner dimensions padded to multiples of 8): executed MMA flops
    kp, npad = -(-k // 8) * 8, -(-n_pts // 8) * 8
    slice_flops = 2.0 * k * npad * kp * 45
    bf16_peak, bf16_source = tensor_peak()
    achieved = slice_flops / t / 1e12
    return dict(
        metric="GFLOP/s of the kriging field + variance (FP64)",
        value=flops / t / 1e9, unit="GFLOP/s", n_gpus=1, steps=args.steps,
        warmup=args.warmup, ms_per_step=t * 1e3, higher_is_better=True,
        scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
        config={"workload": f"ordinary_krige_exp2d_cond1000_pts{n_pts}",
                "n_cond": k, "n_pts": n_pts},
        error_vs_oracle={"max_rel_to_term_scale": err, "points": sample},
        field_only={"ms": t_field * 1e3, "GB_per_s": field_bytes / t_field / 1e9,
                    "hbm_frac_of_measured": (field_bytes / t_field / 1e9 / hbm
                                             if hbm else None),
                    "equivalent_GFLOP_per_s": flops / 2 / t_field / 1e9,
                    "note": "calc_field_krige: V^T (M^T c), bytes = 8 (K^2 + K n + n)"},
        roofline={"bound": "tensor", "achieved": achieved, "peak": bf16_peak,
                  "unit": "TFLOP/s", "frac": achieved / bf16_peak,
                  "kernel": "slice GEMMs (cuBLAS FP16, FP32 accumulate) + FP64 folds",
                  "peak_source": f"dense bf16 ({bf16_source})",
                  "note": "achieved = executed slice-product flops (45 slice pairs "
                          "x 2 K Kp n) over the whole step; the step also holds the "
                          "slicing passes and the FP64 folds of each GEMM result",
                  "fp64_equivalent_tflops": flops / t / 1e12,
                  "fp64_nominal_tflops": FP64_NOMINAL_TFLOPS,
                  "fma_chain_probe_tflops": peak64},
        cpu_baseline={"value": 2.0 * k * k * sample / t_cpu / 1e9,
                      "unit": "GFLOP/s", "cores": oracle.num_threads(),
                      "kind": "port", "sample": f"{sample} target points"},
        e2e={"value": flops / te2e / 1e9, "unit": "GFLOP/s",
             "h2d_bytes_per_step": int(mat.nbytes + vecs.nbytes + cond.nbytes),
             "d2h_bytes_per_step": int(fe[0].nbytes + fe[1].nbytes)},
        # per step: 2 field sums, 2 exponent and 2 slicing passes, 9 folds,
        # 1 finish (plus 9 cuBLAS GEMMs, not counted)
        gpu_launches=16 * _MAIN["steps"])


def wl_vario(args, torch, gg, flush):
    """Omnidirectional Matheron variogram of 50 000 points uniform in
    [0, 1000]^2 (one field), 40 bins up to 400: 1.25e9 point pairs per step;
    plus the axis variogram of a 256^3 field.  Work unit: point pairs."""
    import oracle
    import gstools_gb300.variogram as gv
    from gstools_gb300 import _native

    rng = np.random.RandomState(20170519)
    n, nb = (50_000, 40) if args.size == "full" else (20_000, 40)
    pos = rng.uniform(0.0, 1000.0, (2, n))
    f = rng.normal(size=(1, n))
    edges = np.linspace(0.0, 400.0, nb + 1)
    dev = torch.device("cuda", torch.cuda.current_device())
    dp, dfd, de = (torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                   for a in (pos, f, edges))
    vario = torch.zeros(nb, dtype=torch.float64, device=dev)
    counts = torch.zeros(nb, dtype=torch.int64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())

    def step():
        _native.call("gst_vario_unstructured", 2, n, 1, p(dfd), nb, p(de), p(dp),
                     ord("m"), ord("e"), p(vario), p(counts), stream)

    t = _timed_events(torch, step, args.steps, args.warmup, flush, main=True,
                      min_s=args.min_timed_s)
    pairs = n * (n - 1) / 2
    # directional: the two axes, tolerance pi/8, bandwidth 20
    dirs = torch.tensor([[1.0, 0.0], [0.0, 1.0]], dtype=torch.float64, device=dev)
    vario_d = torch.zeros(2 * nb, dtype=torch.float64, device=dev)
    counts_d = torch.zeros(2 * nb, dtype=torch.int64, device=dev)

    def step_dir():
        _native.call("gst_vario_directional", 2, n, 1, p(dfd), nb, p(de), p(dp), 2,
                     p(dirs), float(np.pi / 8), 20.0, 0, ord("m"), p(vario_d),
                     p(counts_d), stream)

    t_dir = _timed_events(torch, step_dir, args.steps, args.warmup, flush)
    sample = 3000
    t0 = time.perf_counter()
    go, co = oracle.c_vario_unstructured(f[:, :sample], edges, pos[:, :sample])
    t_cpu = time.perf_counter() - t0
    gs_, cs_ = gv.unstructured(f[:, :sample], edges, pos[:, :sample])
    err = float(np.max(np.abs(gs_ - go) / np.maximum(np.abs(go), 1e-300)))
    exact_counts = bool(np.array_equal(cs_, co))
    t0 = time.perf_counter()
    gv.unstructured(f, edges, pos)
    te2e = time.perf_counter() - t0
    na = 256 if args.size == "full" else 128
    fld = torch.from_numpy(rng.normal(size=(na, na * na))).to(dev)
    vs = torch.zeros(na, dtype=torch.float64, device=dev)

    def axis_step():
        _native.call("gst_vario_structured", na, na * na, p(fld),
                     ctypes.c_void_p(0), ord("m"), p(vs), stream)

    t_axis = _timed_events(torch, axis_step, args.steps, args.warmup, flush)
    axis_pairs = na * (na - 1) / 2 * na * na
    return dict(
        metric="G point pairs/s of the empirical variogram (FP64)",
        value=pairs / t / 1e9, unit="G pairs/s", n_gpus=1, steps=args.steps,
        warmup=args.warmup, ms_per_step=t * 1e3, higher_is_better=True,
        scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
        config={"workload": f"vario_unstructured_2d_pts{n}_bins{nb}",
                "pairs_per_step": pairs, "bins": nb},
        error_vs_oracle={"max_rel": err, "counts_exact": exact_counts,
                         "points": sample},
        directional={"value": pairs / t_dir / 1e9, "unit": "G pairs/s",
                     "ms": t_dir * 1e3, "directions": 2, "angles_tol": "pi/8",
                     "bandwidth": 20.0},
        axis_variogram={"value": axis_pairs / t_axis / 1e9, "unit": "G pairs/s",
                        "ms": t_axis * 1e3, "field": [na, na, na],
                        "kernel": "vario_structured_tiled_kernel",
                        "fp64_tflops": 3.0 * axis_pairs / t_axis / 1e12,
                        "fp64_frac_of_nominal": 3.0 * axis_pairs / t_axis / 1e12
                        / FP64_NOMINAL_TFLOPS,
                        "note": "3 FP64 flops per pair (DADD + DFMA)"},
        cpu_baseline={"value": sample * (sample - 1) / 2 / t_cpu / 1e9,
                      "unit": "G pairs/s", "cores": oracle.num_threads(),
                      "kind": "port",
                      "sample": f"{sample} points (the restated loop runs the "
                                "bins outermost, as the reference's does)"},
        e2e={"value": pairs / te2e / 1e9, "unit": "G pairs/s",
             "h2d_bytes_per_step": int(pos.nbytes + f.nbytes + edges.nbytes),
             "d2h_bytes_per_step": int(nb * 16)},
        gpu_launches=2)


def wl_points(args, torch, gg, flush):
    """2-D Gaussian, var 1, len_scale 10, 1000 modes (reference RNG, seed
    20170519), 100 000 points uniform in [0, 100]^2."""
    import oracle

    gen = gg.RandMeth(gg.Gaussian(dim=2, var=1.0, len_scale=10.0),
                      mode_no=1000, seed=20170519)
    pos = np.random.RandomState(20170519).uniform(0.0, 100.0, (2, 100_000))
    dev = torch.device("cuda", torch.cuda.current_device())
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
         for a in (gen.cov_samples, gen.z_1, gen.z_2, pos)]
    work = 1000 * 100_000
    f64 = lambda: gg.summate(*t)
    mixed = lambda: gg.summate(*t, precision="mixed")
    t64 = _timed_events(torch, f64, args.steps, args.warmup, flush)
    tmx = _timed_events(torch, mixed, args.steps, args.warmup, flush, main=True,
                        min_s=args.min_timed_s)
    t0 = time.perf_counter()
    ref = oracle.c_summate(gen.cov_samples, gen.z_1, gen.z_2, pos)
    t_cpu = time.perf_counter() - t0
    got64 = f64().cpu().numpy()
    gotmx = mixed().cpu().numpy()
    s = np.sqrt(1.0 / 1000)
    e2e = gg.summate(gen.cov_samples, gen.z_1, gen.z_2, pos, precision="mixed")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(20):
        e2e = gg.summate(gen.cov_samples, gen.z_1, gen.z_2, pos, precision="mixed")
    te2e = (time.perf_counter() - t0) / 20
    return _line(
        args, "gau2d_points100k_modes1000", work / tmx / 1e9, tmx,
        "fp32 + exact turn reduction", {"points": 100_000, "modes": 1000},
        f64_plain={"value": work / t64 / 1e9, "unit": UNIT,
                   "max_rel_err_vs_oracle": float(np.max(np.abs(got64 - ref))
                                                  / np.max(np.abs(ref)))},
        error_vs_fp64={"rms_sigma": float(np.sqrt(np.mean((s * (gotmx - ref)) ** 2))),
                       "max_abs_sigma": float(np.max(np.abs(s * (gotmx - ref)))),
                       "vs": "FP64 C oracle, all 100 000 points"},
        e2e={"value": work / te2e / 1e9, "unit": UNIT,
             "h2d_bytes_per_step": int(pos.nbytes + 4 * 8 * 1000),
             "d2h_bytes_per_step": int(e2e.nbytes)},
        cpu_baseline={"value": work / t_cpu / 1e9, "unit": UNIT,
                      "cores": oracle.num_threads(), "kind": "port",
                      "sample": "the whole workload (FP64 C/OpenMP oracle)"},
        roofline={"bound": "fp32 issue",
                  "achieved_alg_tflops": 8.0 * work / tmx / 1e12,
                  "note": "algorithmic 2d+4 = 8 flops per mode*point plus 2 SFU "
                          "sin/cos; the exact turn reduction issues ~20 FP32 "
                          "operations per mode*point, and ncu measures the FMA "
                          "pipe 64.8 % active (profiles: pointwise summary)"},
        gpu_launches=2 * _MAIN["steps"])


def make_ensemble(n_items=512, seed=20170519):
    """512 realizations: 2-D Matern nu=1.5, var 1, len_scale log-uniform in
    [2, 50], mode_no uniform in {1000, 2000, 4000}, own seed (MasterRNG) and
    own point set of log-uniform size 1k-200k in [0, 500]^2."""
    import gstools_gb300 as gg

    seeds = gg.MasterRNG(seed)
    rng = np.random.RandomState(seed + 1)
    gens, pos = [], []
    for _ in range(n_items):
        ls = float(np.exp(rng.uniform(np.log(2.0), np.log(50.0))))
        n_modes = int(rng.choice([1000, 2000, 4000]))
        n_pts = int(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
        gens.append(gg.RandMeth(gg.Matern(dim=2, nu=1.5, var=1.0, len_scale=ls),
                                mode_no=n_modes, seed=seeds()))
        pos.append(rng.uniform(0.0, 500.0, size=(2, n_pts)))
    return gens, pos


def wl_ensemble(args, torch, gg, flush):
    from gstools_gb300 import _native

    gens, pos = make_ensemble()
    modes = [g.mode_no for g in gens]
    pts = [p.shape[1] for p in pos]
    work = int(sum(m * n for m, n in zip(modes, pts)))
    scales = [np.sqrt(1.0 / m) for m in modes]
    bs = gg.BatchedSummator(2, modes, pts, out_dtype="float32", graph=True)
    bs.load([g.cov_samples for g in gens], [g.z_1 for g in gens],
            [g.z_2 for g in gens], pos, scales)
    tune = bs.tune()
    t_batch = _timed_events(torch, bs.run, args.steps, args.warmup, flush, main=True,
                            min_s=args.min_timed_s)
    batched = [f.astype(np.float64) for f in bs.split()]
    # modes drawn on the device (one Philox stream per realization seed) vs
    # the host mirror's per-realization reset_seed loop (the reference's way)
    model = gg.Matern(dim=2, nu=1.5, var=1.0)
    seeds_r = np.array([g.seed for g in gens], dtype=np.uint64)
    ls_r = np.array([g.model.len_scale for g in gens])
    bs_dev = gg.BatchedSummator(2, modes, pts, out_dtype="float32", graph=True)
    bs_dev.load_points(pos)

    def sample_dev():
        bs_dev.sample(model, seeds_r, len_scales=ls_r)

    sample_dev()
    bs_dev.tune()

    def sample_and_sum():
        sample_dev()
        bs_dev.run()

    t_sample = _timed_events(torch, sample_dev, args.steps, args.warmup, flush)
    t_ss = _timed_events(torch, sample_and_sum, args.steps, args.warmup, flush)
    t0 = time.perf_counter()
    for g in gens:
        g.reset_seed(g.seed)
    t_host_sample = time.perf_counter() - t0
    # 512 sequential calls on the same device-resident data
    cov, z1, z2, xx = bs.cov, bs.z1, bs.z2, bs.pos
    outs = [torch.empty(n, dtype=torch.float64, device=bs.dev) for n in pts]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    covs = [cov[:, bs.mode_off[r]:bs.mode_off[r + 1]].contiguous() for r in range(len(gens))]
    poss = [xx[:, bs.point_off[r]:bs.point_off[r + 1]].contiguous() for r in range(len(gens))]

    def sequential(name, extra):
        for r in range(len(gens)):
            m0, m1 = bs.mode_off[r], bs.mode_off[r + 1]
            args_ = [2, modes[r], pts[r], ctypes.c_void_p(covs[r].data_ptr()),
                     ctypes.c_void_p(z1[m0:m1].data_ptr()),
                     ctypes.c_void_p(z2[m0:m1].data_ptr()),
                     ctypes.c_void_p(poss[r].data_ptr()),
                     ctypes.c_void_p(outs[r].data_ptr())] + extra + [stream]
            _native.call(name, *args_)

    t_seq64 = _timed_events(torch, lambda: sequential("gst_summate_f64", []),
                            1, 1, flush)
    ref = [o.cpu().numpy() * s for o, s in zip(outs, scales)]
    t_seqmx = _timed_events(
        torch, lambda: sequential("gst_summate_mixed", [_native.GST_OUT_F64]),
        2, 1, flush)
    import oracle

    # every realization against the FP64 oracle on 256 of its points
    rng_s = np.random.RandomState(3)
    sq, cnt, mx, worst = 0.0, 0, 0.0, 0.0
    for r, g in enumerate(gens):
        idx = np.sort(rng_s.choice(pts[r], size=min(256, pts[r]), replace=False))
        ref_o = scales[r] * oracle.c_summate(g.cov_samples, g.z_1, g.z_2,
                                             np.ascontiguousarray(pos[r][:, idx]))
        d = batched[r][idx] - ref_o
        sq += float(np.sum(d ** 2))
        cnt += d.size
        mx = max(mx, float(np.max(np.abs(d))))
        worst = max(worst, float(np.sqrt(np.mean(d ** 2))))
    err = np.sqrt(sq / cnt)
    seq_err = max(float(np.max(np.abs(b - r))) for b, r in zip(batched, ref))
    # end to end: host arrays in, per-realization host arrays out
    cov_l = [g.cov_samples for g in gens]
    z1_l = [g.z_1 for g in gens]
    z2_l = [g.z_2 for g in gens]
    bs(cov_l, z1_l, z2_l, pos, scales)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = bs(cov_l, z1_l, z2_l, pos, scales)
    te2e = time.perf_counter() - t0
    cpu = _cpu_sample(
        lambda r: oracle.c_summate(gens[r].cov_samples, gens[r].z_1, gens[r].z_2, pos[r]),
        list(range(len(gens))), lambda r: modes[r] * pts[r], what="realizations",
        skip=args.no_cpu_baseline)
    return _line(
        args, "matern2d_ensemble512", work / t_batch / 1e9, t_batch,
        "fp32 + exact turn reduction",
        {"realizations": len(gens), "mode_points_per_step": work,
         "total_points": int(sum(pts)), "total_modes": int(sum(modes))},
        autotune={"chosen_variant": bs.variant,
                  "chosen_shape": dict(zip(("points_per_tile", "modes_per_stage",
                                            "ctas_per_sm"),
                                           gg.batched.VARIANT_SHAPES[bs.variant])),
                  "candidates_ms": {str(k): v for k, v in tune.items()},
                  "spread": (max(tune.values()) / min(tune.values())
                             if tune else None),
                  "chosen_over_variant0": (tune[0] / tune[bs.variant]
                                           if tune and 0 in tune else None)},
        sequential_f64={"value": work / t_seq64 / 1e9, "unit": UNIT,
                        "ms": t_seq64 * 1e3, "calls": len(gens)},
        sequential_mixed={"value": work / t_seqmx / 1e9, "unit": UNIT,
                          "ms": t_seqmx * 1e3, "calls": len(gens)},
        value_over_sequential_f64=t_seq64 / t_batch,
        device_sampling={"ms": t_sample * 1e3,
                         "host_mirror_reset_seed_ms": t_host_sample * 1e3,
                         "speedup": t_host_sample / t_sample,
                         "stream": "Philox4x64-10 per realization seed "
                                   "(not the reference's MT19937 stream)"},
        sample_and_sum={"value": work / t_ss / 1e9, "unit": UNIT,
                        "ms": t_ss * 1e3},
        error_vs_fp64={"rms_sigma": err, "max_abs_sigma": mx,
                       "worst_realization_rms_sigma": worst,
                       "vs": "FP64 C oracle, 256 points of every realization",
                       "max_abs_vs_sequential_fp64_gpu": seq_err},
        e2e={"value": work / te2e / 1e9, "unit": UNIT,
             "h2d_bytes_per_step": int(sum(p.nbytes for p in pos)
                                       + sum(c.nbytes for c in cov_l) * 2),
             "d2h_bytes_per_step": int(sum(r.nbytes for r in res))},
        cpu_baseline=cpu,
        gpu_launches=2 * _MAIN["steps"])


def wl_incompr(args, torch, gg, flush):
    """3-D Gaussian incompressible field, var 1, len_scale 8, 2000 modes,
    mean velocity 1, 192^3 unit grid, float32 3-component output."""
    from gstools_gb300 import _native

    data = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
    cov, z1, z2 = data["incompr3d/cov"], data["incompr3d/z1"], data["incompr3d/z2"]
    n, nm = 192, 2000
    scale = float(np.sqrt(1.0 / nm))
    dev = torch.device("cuda", torch.cuda.current_device())
    d = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (cov, z1, z2)]
    axes = torch.from_numpy(np.concatenate([np.arange(float(n))] * 3)).to(dev)
    lens = (ctypes.c_int64 * 4)(n, n, n, 1)
    out = torch.empty((3, n, n, n), dtype=torch.float32, device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    mixed = lambda: _native.call("gst_summate_incompr_grid_mixed", 3, nm, lens,
                                 p(axes), p(d[0]), p(d[1]), p(d[2]), p(out),
                                 _native.GST_OUT_F32, scale, stream)
    out_tc = torch.empty((3, n, n, n), dtype=torch.float32, device=dev)
    tensor = lambda: _native.call("gst_summate_incompr_grid_tc", 3, nm, lens,
                                  p(axes), p(d[0]), p(d[0]), p(d[1]), p(d[2]),
                                  p(out_tc), _native.GST_OUT_F32, scale, stream)
    ttc = _timed_events(torch, tensor, args.steps, args.warmup, flush, main=True,
                        min_s=args.min_timed_s)
    tmx = _timed_events(torch, mixed, args.steps, args.warmup, flush)
    slab = 12
    lens64 = (ctypes.c_int64 * 4)(slab, n, n, 1)
    out64 = torch.empty((3, slab, n, n), dtype=torch.float64, device=dev)
    axes64 = torch.from_numpy(np.concatenate(
        [np.arange(float(slab)), np.arange(float(n)), np.arange(float(n))])).to(dev)
    f64 = lambda: _native.call("gst_summate_incompr_grid_f64", 3, nm, lens64,
                               p(axes64), p(d[0]), p(d[1]), p(d[2]), p(out64),
                               stream)
    t64 = _timed_events(torch, f64, 1, 1, flush)
    mixed()
    tensor()
    import oracle

    # the FP64 oracle on every 8th grid point per axis (24^3 points)
    sub = np.arange(0, n, 8)
    pts_sub = np.array(np.meshgrid(sub, sub, sub, indexing="ij"),
                       dtype=np.float64).reshape(3, -1)
    ref = scale * oracle.c_summate_incompr(cov, z1, z2, pts_sub)
    isub = torch.from_numpy(sub).to(dev)

    def at_sub(t):
        t = t.index_select(1, isub).index_select(2, isub).index_select(3, isub)
        return t.double().cpu().numpy().reshape(3, -1)

    diff = at_sub(out) - ref
    diff_tc = at_sub(out_tc) - ref
    # the FP64 kernel's slab (x < 12) at the sub-grid points it covers
    ref4 = ref.reshape(3, len(sub), len(sub), len(sub))
    xs = np.nonzero(sub < slab)[0]
    o64 = scale * out64.cpu().numpy()[:, sub[xs]][:, :, ::8, ::8]
    f64_rel = float(np.max(np.abs(o64 - ref4[:, xs])) / np.max(np.abs(ref4[:, xs])))
    # divergence of the float32 field by central differences (unit spacing)
    u = out_tc.double()
    div = ((u[0, 2:, 1:-1, 1:-1] - u[0, :-2, 1:-1, 1:-1])
           + (u[1, 1:-1, 2:, 1:-1] - u[1, 1:-1, :-2, 1:-1])
           + (u[2, 1:-1, 1:-1, 2:] - u[2, 1:-1, 1:-1, :-2])) / 2.0
    grad_scale = ((u[0, 2:, 1:-1, 1:-1] - u[0, :-2, 1:-1, 1:-1]) / 2.0).std()
    work = nm * n ** 3
    import oracle

    g1 = np.arange(float(n))

    def cpu_row(ix):
        yz = np.array(np.meshgrid(g1, g1, indexing="ij")).reshape(2, -1)
        row = np.concatenate([np.full((1, yz.shape[1]), float(ix)), yz])
        oracle.c_summate_incompr(cov, z1, z2, row)

    cpu = _cpu_sample(cpu_row, list(range(n)), lambda ix: nm * n * n, what="x rows",
                      skip=args.no_cpu_baseline)
    return _line(
        args, "gau3d_incompr_grid192_modes2000", work / ttc / 1e9, ttc,
        "f16x3 (fp32 accumulate)",
        {"grid": [n] * 3, "modes": nm, "components": 3, "output": "float32",
         "path": "tensor-core grid path, one weighted contraction per component"},
        f64_plain={"value": nm * slab * n * n / t64 / 1e9, "unit": UNIT,
                   "sample": f"{slab}x{n}x{n} slab",
                   "max_rel_err_vs_oracle": f64_rel},
        mixed_pointwise={"value": work / tmx / 1e9, "unit": UNIT,
                         "rms_sigma": float(np.sqrt(np.mean(diff ** 2)))},
        error_vs_fp64={"rms_sigma": float(np.sqrt(np.mean(diff_tc ** 2))),
                       "max_abs_sigma": float(np.max(np.abs(diff_tc))),
                       "vs": "FP64 C oracle on every 8th grid point per axis "
                             f"({pts_sub.shape[1]} points, 3 components)"},
        divergence={"fd_rms_over_grad_rms": float(div.std() / grad_scale),
                    "note": "central differences, h=1; O(h^2) truncation"},
        cpu_baseline=cpu,
        gpu_launches=2 * _MAIN["steps"])


def wl_adjoint(args, torch, gg, flush):
    """3-D Gaussian, 4000 modes (reference RNG, anisotropic and rotated),
    128^3 grid + 50 000 points in [0, 128]^3; loss = mean squared misfit at
    10 000 random observation points against a field from another seed;
    gradients w.r.t. z_1, z_2, len_scale, anisotropy and rotation angles.
    The grid is passed as its axes (structured forward), the points as
    coordinates."""
    from gstools_gb300.grad import isometrize_matrix, randmeth_field

    data = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
    dev = torch.device("cuda", torch.cuda.current_device())
    cov_ref = torch.tensor(data["gau3d_grad/cov"], device=dev)
    z1 = torch.tensor(data["gau3d_grad/z1"], device=dev, requires_grad=True)
    z2 = torch.tensor(data["gau3d_grad/z2"], device=dev, requires_grad=True)
    rng = np.random.RandomState(7)
    g = np.arange(128.0)
    grid = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1)
    pts = np.concatenate([grid, rng.uniform(0.0, 128.0, (3, 50_000))], axis=1)
    x = torch.tensor(pts[:, g.size ** 3:], device=dev)   # the 50 000 points
    axes = [torch.tensor(g, device=dev)] * 3
    obs = torch.tensor(rng.choice(pts.shape[1], 10_000, replace=False), device=dev)
    other = gg.RandMeth(gg.Gaussian(dim=3, var=1.0, len_scale=16.0), mode_no=4000,
                        seed=4242, sampling="analytic")
    target = torch.tensor(other(pts[:, obs.cpu().numpy()], add_nugget=False),
                          device=dev)
    params = {"var": torch.tensor(1.0, dtype=torch.float64, device=dev),
              "len_scale": torch.tensor(16.0, dtype=torch.float64, device=dev,
                                        requires_grad=True),
              "anis": torch.tensor([0.8, 0.6], dtype=torch.float64, device=dev,
                                   requires_grad=True),
              "angles": torch.tensor([0.3, 0.2, 0.1], dtype=torch.float64,
                                     device=dev, requires_grad=True)}

    def fwd(prec):
        # the 128^3 grid (tensor-core contraction forward in mixed precision)
        # followed by the 50 000 points
        return randmeth_field(cov_ref, 16.0, z1, z2, x, axes=axes, precision=prec,
                              **params)

    def loss_of(u):
        return torch.mean((u[obs] - target) ** 2)

    def step_fwd():
        with torch.no_grad():
            fwd("mixed")

    def step_fwd_bwd(prec="mixed"):
        for t in (z1, z2, params["len_scale"], params["anis"], params["angles"]):
            t.grad = None
        loss_of(fwd(prec)).backward()

    t_f = _timed_events(torch, step_fwd, args.steps, args.warmup, flush, main=True,
                        min_s=args.min_timed_s)
    t_fb = _timed_events(torch, step_fwd_bwd, args.steps, args.warmup, flush)
    # the adjoint over every point (the cotangent is zero off the 10 000
    # observations, which the default backward leaves out)
    gg.grad.SPARSE_COTANGENT = False
    try:
        t_fb_dense = _timed_events(torch, step_fwd_bwd, args.steps, args.warmup,
                                   flush)
    finally:
        gg.grad.SPARSE_COTANGENT = True
    grads_mixed = [t.grad.clone() for t in (z1, z2, params["len_scale"],
                                            params["anis"], params["angles"])]
    step_fwd_bwd("f64")
    grads_f64 = [t.grad.clone() for t in (z1, z2, params["len_scale"],
                                          params["anis"], params["angles"])]
    rel = {name: float(torch.max(torch.abs(a - b)) / torch.max(torch.abs(b)))
           for name, a, b in zip(("z1", "z2", "len_scale", "anis", "angles"),
                                 grads_mixed, grads_f64)}
    work = 4000 * pts.shape[1]
    import oracle

    # forward field vs the FP64 oracle on 4096 of the points
    with torch.no_grad():
        u_mx = fwd("mixed").cpu().numpy()
        k_map = (isometrize_matrix(3, params["angles"], params["anis"]).T
                 @ cov_ref).cpu().numpy()
    sel = np.sort(np.random.RandomState(11).choice(pts.shape[1], 4096,
                                                   replace=False))
    u_or = np.sqrt(1.0 / 4000) * oracle.c_summate(
        k_map, data["gau3d_grad/z1"], data["gau3d_grad/z2"],
        np.ascontiguousarray(pts[:, sel]))
    d_fwd = u_mx[sel] - u_or

    cov_np = data["gau3d_grad/cov"]
    z1_np, z2_np = data["gau3d_grad/z1"], data["gau3d_grad/z2"]
    chunks = list(range(0, pts.shape[1], 4096))
    cpu = _cpu_sample(lambda c: oracle.c_summate(cov_np, z1_np, z2_np, pts[:, c:c + 4096]),
                      chunks, lambda c: 4000 * min(4096, pts.shape[1] - c),
                      what="4096-point chunks (forward summate only; a CPU gradient "
                           "by finite differences needs two forwards per parameter)",
                      skip=args.no_cpu_baseline)
    return _line(
        args, "gau3d_adjoint_grid128_pts50k_modes4000", work / t_f / 1e9, t_f,
        "f16x3 (grid) + fp32 with exact turn reduction (points)",
        {"points": int(pts.shape[1]), "modes": 4000, "observations": 10_000},
        notes={"path": "randmeth_field(pos=50k points, axes=128^3 grid): the "
                       "grid forward through the tensor-core contraction "
                       "(SummateGridFunction), the points through the mixed "
                       "pointwise kernel; the backward runs the adjoint "
                       "kernels at the points with a nonzero cotangent"},
        fwd_ms=t_f * 1e3, fwd_bwd_ms=t_fb * 1e3, fwd_bwd_over_fwd=t_fb / t_f,
        fwd_bwd_all_points={"ms": t_fb_dense * 1e3, "over_fwd": t_fb_dense / t_f,
                            "note": "adjoint kernels over all 2.15 M points, "
                                    "not only the 10 000 with a nonzero "
                                    "cotangent"},
        error_vs_fp64={"rms_sigma": float(np.sqrt(np.mean(d_fwd ** 2))),
                       "max_abs_sigma": float(np.max(np.abs(d_fwd))),
                       "vs": "FP64 C oracle, forward field at 4096 points"},
        grad_rel_err_mixed_vs_f64=rel, cpu_baseline=cpu, gpu_launches=None)


_LINE_ONLY = ("metric", "n_gpus", "steps", "warmup", "higher_is_better",
              "scaling", "vs_baseline", "data")


def other_configs(args, torch, gg, flush):
    """Bounded runs of the other four configurations for the headline line:
    at least 5 timed steps spanning at least --min-timed-s seconds after 3
    warm-up steps each, every one with its error against the oracle and the
    clocks sampled inside the timed region of its `value`."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.size = 5, 3, "full"
    out = {}
    for fn in (wl_points, wl_ensemble, wl_incompr, wl_adjoint):
        ck = Clocks(torch.cuda.current_device())
        ck.start()
        _MAIN["window"], _MAIN["steps"] = None, 0
        line = fn(sub, torch, gg, flush)
        clk = ck.stop(window=_MAIN["window"])
        keep = {k: v for k, v in line.items() if k not in _LINE_ONLY}
        keep["clocks"] = clk
        keep["steps"], keep["warmup"] = _MAIN["steps"], sub.warmup
        out[line["config"]["workload"]] = keep
    return out


def run_workload(args):
    import torch

    import gstools_gb300 as gg
    from gstools_gb300 import build

    torch.cuda.set_device(0)
    build.build()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    fn = {"points": wl_points, "ensemble": wl_ensemble, "krige": wl_krige,
          "vario": wl_vario,
          "incompr": wl_incompr, "adjoint": wl_adjoint}[args.workload]
    clocks = Clocks(0)
    clocks.start()
    line = fn(args, torch, gg, flush)
    line["clocks"] = clocks.stop(window=_MAIN["window"])
    if _MAIN["steps"]:
        line["steps"] = _MAIN["steps"]
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "grid":
        run_ours(args)
    else:
        run_workload(args)


if __name__ == "__main__":
    main()
