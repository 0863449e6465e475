"""Benchmark of the sparse x dense mul! hot path on one GB300 (or N replicas under torchrun).

Headline: plain Float64 CSR SpMV ``mul!(y, A, x)`` of the 2D 5-point Laplacian on a 2048 x 2048
grid (n = 4,194,304, nnz = 20,963,328, Int32 indices, alpha = 1, beta = 0), synthetic and
generated on the host from the stated formula.  Metric: algorithmic HBM GB/s under the
minimal-bytes model  nnz*(8+4) + (m+1)*4 + n*8 + m*8 = 335.45 MB per SpMV.

* ``value``     device time of K SpMVs with A, x, y resident in HBM; L2 is flushed (a 512 MB
                write, then a 256 MB read so that no dirty line is left for the timed step to
                write back) before every timed SpMV, and only the SpMV sits between the events
* ``roofline``  the dominant kernel (row-block gather) timed by events the library records
                right around it; algorithmic bytes / its average duration vs the measured
                HBM copy bandwidth in MEASURED_PEAKS.json
* ``e2e``       the same metric through the public API from pinned host buffers: per step the
                host->device copy of x, mul!, the device->host copy of y (steps alternate
                between two streams so uploads overlap downloads; the one-stream sequential
                figure is reported beside it)
* ``cpu_baseline``  the oracle's C restatement of the reference kernel (OpenMP, all host
                cores) on the same matrix, a bounded number of SpMVs
* ``extras``    the other benchmark rows (CSC, SpMM k=16, F32, Int64 indices, power-law
                ComplexF64 CSR/COO, n=1e5 random CSR/CSC/COO, COO->CSR conversion) and the
                batched uneven-size mix (4096 banded ComplexF64 matrices: grouped launch from a
                CUDA graph against per-call mul!, mul!/s and p50/p99 batch latency)

``--impl reference`` times the CPU restatement of the reference (the reference itself is
Julia, absent on this machine) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 512 << 20
METRIC = "SpMV/SpMM HBM GB/s (% of peak); batched mul!/s + p99 vs plain GPU at 1e-12"


def spmv_bytes(m, n, nnz, vs, is_, k=1, beta_read=False):
    b = nnz * (vs + is_) + (m + 1) * is_ + n * k * vs + m * k * vs
    return b + (m * k * vs if beta_read else 0)


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(key):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
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
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------

def replica_value(total_ms, world, nbytes, steps, device):
    """Whole-job GB/s of `world` replicas that each ran `steps` steps of `nbytes`: all ranks'
    bytes over the slowest rank's time (the max over ranks; weak scaling, no data exchange).
    Returns (GB/s, max ms)."""
    import torch
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    max_ms = float(t.item())
    return world * nbytes * steps / (max_ms / 1e3) / 1e9, max_ms


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def host_threads() -> int:
    """CPUs this process may run on.  OMP_NUM_THREADS is not consulted (torchrun sets it to 1):
    the CPU legs run on rank 0 alone and take the whole host."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_spmv_sample(oracle, m, n, rp, cv, nz, x, budget_s=10.0, max_reps=200):
    """Time the C restatement of kernel_spmatmul_csr_N! (OpenMP, all host threads)."""
    threads = host_threads()
    y = np.zeros(m)
    oracle.mul("csr", "N", m, n, rp, cv, nz, 1, x, y, nthreads=threads)  # warm-up
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < max_reps and (time.perf_counter() < t_end or len(times) < 3):
        t0 = time.perf_counter()
        oracle.mul("csr", "N", m, n, rp, cv, nz, 1, x, y, nthreads=threads)
        times.append(time.perf_counter() - t0)
    return statistics.median(times), len(times), threads


def run_reference(args, world, rank):
    """CPU restatement of the reference on the headline workload (rank 0 only)."""
    if rank != 0:
        return
    from oracle import oracle
    import genericsparsearrays_gb300  # noqa: F401  (registered by __graft_entry__)
    wl = genericsparsearrays_gb300.workloads
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=np.int32, dtype=np.float64)
    x = np.random.default_rng(0).uniform(-1, 1, n)
    threads = host_threads()
    y = np.zeros(m)
    for _ in range(args.warmup):
        oracle.mul("csr", "N", m, n, rp, cv, nz, 1, x, y, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.mul("csr", "N", m, n, rp, cv, nz, 1, x, y, nthreads=threads)
        times.append(time.perf_counter() - t0)
    nbytes = spmv_bytes(m, n, cv.size, 8, 4)
    total = sum(times)
    value = nbytes * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total / len(times) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "laplacian_2048x2048_csr_spmv_f64_i32", "n": m, "nnz": int(cv.size),
                   "bytes_per_step": nbytes, "impl_note":
                   "C/OpenMP restatement of kernel_spmatmul_csr_N! (Julia reference absent)"},
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full SpMVs of the 2048^2 Laplacian"},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------

class DeviceTimer:
    """Per-step CUDA-event timing on the current stream, with an L2 flush between steps.

    The flush writes a 512 MB buffer (evicting every line of the 129 MB L2) and then reads a
    256 MB buffer, so that L2 holds clean lines when the timed step starts: otherwise the
    step would pay for writing the flush's dirty lines back to HBM.  Both passes sit outside
    the timed events."""

    def __init__(self, torch, device):
        self.torch = torch
        self.flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
        self.clean_buf = torch.ones(L2_FLUSH_BYTES // 8, dtype=torch.float32, device=device)

    def flush(self):
        self.flush_buf.fill_(1.0)
        self._sink = self.clean_buf.sum()

    def run(self, fn, steps, warmup, flush=True, kernel_events=None, lib=None):
        torch = self.torch
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        kb = [torch.cuda.Event(enable_timing=True) for _ in range(steps)] if kernel_events else None
        ka = [torch.cuda.Event(enable_timing=True) for _ in range(steps)] if kernel_events else None
        if kernel_events:  # torch creates the CUDA event on first record; the library re-records it
            for e in kb + ka:
                e.record()
        torch.cuda.synchronize()
        for i in range(steps):
            if flush:
                self.flush()
            if kernel_events:
                lib.gsa_set_kernel_timer(ctypes.c_void_p(kb[i].cuda_event), ctypes.c_void_p(ka[i].cuda_event))
            starts[i].record()
            fn()
            ends[i].record()
        if kernel_events:
            lib.gsa_set_kernel_timer(None, None)
        torch.cuda.synchronize()
        total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
        kern_ms = sum(b.elapsed_time(a) for b, a in zip(kb, ka)) if kernel_events else None
        return total_ms, kern_ms


def run_gpu(args, world, rank, local):
    import torch
    import __graft_entry__
    gsa = __graft_entry__.load_package()
    from genericsparsearrays_gb300 import workloads as wl
    from genericsparsearrays_gb300 import _lib

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    timer = DeviceTimer(torch, dev)
    peak, peak_kind = measured_peak()

    # ---- headline workload ------------------------------------------------
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=np.int32, dtype=np.float64)
    nnz = int(cv.size)
    nbytes = spmv_bytes(m, n, nnz, 8, 4)
    rng = np.random.default_rng(0)
    x_host = rng.uniform(-1, 1, n)
    A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    x = torch.from_numpy(x_host).to(dev)
    y = torch.empty(m, dtype=torch.float64, device=dev)
    ws_bytes = lib.gsa_mul_workspace_size(0, _lib.F64, _lib.IDX32, m, n, nnz, 0, 1, 0)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
    one, zero = np.array([1.0]), np.array([0.0])
    pone, pzero = one.ctypes.data_as(ctypes.c_void_p), zero.ctypes.data_as(ctypes.c_void_p)

    def spmv_capi(algo=0):
        st = lib.gsa_csr_mul(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), _lib.F64,
                             _lib.IDX32, m, n, nnz, ctypes.c_void_p(A.rowptr.data_ptr()),
                             ctypes.c_void_p(A.colval.data_ptr()), ctypes.c_void_p(A.nzval.data_ptr()),
                             1, 0, 1, ctypes.c_void_p(x.data_ptr()), n, 0,
                             ctypes.c_void_p(y.data_ptr()), m, pone, pzero, algo,
                             ctypes.c_void_p(ws.data_ptr()), ws.numel())
        if st:
            raise RuntimeError(_lib.last_error())

    # correctness guard on the benchmarked call
    spmv_capi()
    torch.cuda.synchronize()
    import scipy.sparse as sp
    S = sp.csr_matrix((nz, cv.astype(np.int64) - 1, rp.astype(np.int64) - 1), shape=(m, n))
    ref = S @ x_host
    scale = abs(S) @ np.abs(x_host)
    err = float(np.max(np.abs(y.cpu().numpy() - ref) / scale))
    if err > 1e-12:
        raise SystemExit(f"benchmark result check failed: max rel error {err}")

    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        total_ms, kern_ms = timer.run(spmv_capi, args.steps, args.warmup, flush=True,
                                      kernel_events=True, lib=lib)
        value, max_ms = replica_value(total_ms, world, nbytes, args.steps, dev)
        kern_avg_s = kern_ms / args.steps / 1e3
        achieved = nbytes / kern_avg_s / 1e9

        # e2e through the public API: every step copies its x from pinned host memory to the
        # device, runs mul!, and copies its y back to pinned host memory.  Steps rotate over
        # three (--e2e-sets) streams and buffer sets, so one step's upload, the previous step's
        # product and the one before's download run at once (the host link is full duplex;
        # three sets measured 0.211 ms per step against 0.248 ms with two); a step's buffers
        # are reused only after its result is on the host.  The sequential form (one stream,
        # a synchronize per step) is reported beside it.
        SETS = args.e2e_sets
        xh = [torch.from_numpy(x_host).pin_memory() for _ in range(SETS)]
        yh = [torch.empty(m, dtype=torch.float64).pin_memory() for _ in range(SETS)]
        xd = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(SETS)]
        yd = [torch.empty(m, dtype=torch.float64, device=dev) for _ in range(SETS)]
        streams = [torch.cuda.Stream(dev) for _ in range(SETS)]

        def e2e_run(nsteps):
            done = []
            for i in range(nsteps):
                j = i % SETS
                if i >= SETS:
                    done[i - SETS].synchronize()  # that step's y is on the host: its buffers are free
                with torch.cuda.stream(streams[j]):
                    xd[j].copy_(xh[j], non_blocking=True)
                    gsa.mul_(yd[j], A, xd[j])
                    yh[j].copy_(yd[j], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(streams[j])
                    done.append(ev)
            for ev in done[-SETS:]:
                ev.synchronize()

        def e2e_seq():
            xd[0].copy_(xh[0], non_blocking=True)
            gsa.mul_(yd[0], A, xd[0])
            yh[0].copy_(yd[0], non_blocking=True)
            torch.cuda.current_stream().synchronize()

        e2e_run(max(args.warmup, SETS))
        t0 = time.perf_counter()
        e2e_run(args.steps)
        e2e_s = time.perf_counter() - t0
        e2e_ok = all(float(np.max(np.abs(y.numpy() - ref) / scale)) <= 1e-12 for y in yh)
        e2e_value = nbytes * args.steps / e2e_s / 1e9
        for _ in range(args.warmup):
            e2e_seq()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_seq()
        e2e_seq_s = time.perf_counter() - t0

        import bench_support
        fma_rate = bench_support.fma_rate(torch.cuda.current_stream().cuda_stream, "f64")
        extras = {} if args.no_extras else run_extras(gsa, wl, torch, dev, lib, timer, args, fma_rate)
        if not args.no_extras:
            extras["batched_uneven_mix"] = run_batched(gsa, torch, dev, args)
        if not args.no_extras and not args.no_serving:
            extras["served_stream"] = run_serving(gsa, torch, dev, args, fma_rate)

    # arithmetic roofline: FP64 FMAs the SMs retire per second (the row-block kernel does
    # one FMA per stored entry; alpha = 1 adds no multiply)
    fp64_ops = nnz
    clk = clocks.summary()
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle
        t_cpu, reps, threads = cpu_spmv_sample(oracle, m, n, rp, cv, nz, x_host, budget_s=args.cpu_budget)
        cpu = {"value": round(nbytes / t_cpu / 1e9, 2), "unit": "GB/s", "cores": threads,
               "kind": "port",
               "sample": f"{reps} full SpMVs of the 2048^2 Laplacian (median), C/OpenMP restatement"}
    traffic = committed_traffic("rowblock_kernel/laplacian_2048_csr_spmv_f64_i32")
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(max_ms / args.steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 2048x2048 5-point Laplacian, x U(-1,1))",
        "config": {"workload": "laplacian_2048x2048_csr_spmv_f64_i32", "n": m, "nnz": nnz,
                   "bytes_per_step": nbytes, "l2": "flushed before every timed step (512 MB write, then 256 MB read so L2 is clean)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "pct_of_peak": round(100 * value / world / peak, 1), "max_rel_error": err},
        "roofline": {"bound": "hbm", "kernel": "rowblock_kernel<double,int,1>",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "kernel_us": round(kern_avg_s * 1e6, 2),
                     "traffic": traffic,
                     "fp64": {"fma_per_launch": fp64_ops,
                              "achieved_gfma_s": round(fp64_ops / kern_avg_s / 1e9, 1),
                              "peak_gfma_s": round(fma_rate / 1e9, 1),
                              "frac": round(fp64_ops / kern_avg_s / fma_rate, 4),
                              "peak_kind": "measured by bench_support's FMA-rate probe in this run"}},
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": m * 8, "ms_per_step": round(e2e_s / args.steps * 1e3, 4),
                "within_tolerance": e2e_ok, "api": "genericsparsearrays_gb300.mul_",
                "steps_overlap": f"{SETS} streams and buffer sets: upload, product and download of consecutive steps run at once",
                "sequential": {"value": round(nbytes * args.steps / e2e_seq_s / 1e9, 2),
                               "ms_per_step": round(e2e_seq_s / args.steps * 1e3, 4)}},
        "gpu_launches": args.steps,  # one rowblock_kernel per SpMV
        "clocks": clk,
        "cpu_baseline": cpu,
        "extras": extras,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def fp64_error(S, X, Y):
    """max over outputs of |Y - S X| / (|S| |X|) with S X computed by scipy in float64 /
    complex128 (the FP64 reference the error statements use); S a scipy sparse matrix, X and Y
    numpy arrays (Y may be a lower precision)."""
    wide = np.complex128 if np.iscomplexobj(S.data) or np.iscomplexobj(X) else np.float64
    S64 = S.astype(wide)
    X64 = np.asarray(X).astype(wide)
    ref = S64 @ X64
    scale = abs(S64) @ np.abs(X64)
    err = np.abs(np.asarray(Y).astype(wide) - ref) / np.where(scale > 0, scale, 1.0)
    return float(err.max()) if err.size else 0.0


def scipy_csr(m, n, rp, cv, nz):
    import scipy.sparse as sp
    return sp.csr_matrix((nz, cv.astype(np.int64) - 1, rp.astype(np.int64) - 1), shape=(m, n))


def run_extras(gsa, wl, torch, dev, lib, timer, args, fma_rate):
    """Other benchmark rows, fewer steps each: GB/s under the minimal-bytes model, the error
    against an FP64 reference (scipy in float64/complex128) of each row's last result, and
    for FP64-bound rows the fraction of the FP64 FMA rate measured in this run."""
    out = {}
    steps, warm = max(5, args.steps // 4), 3

    def time_call(fn, flush=True):
        total_ms, kern_ms = timer.run(fn, steps, warm, flush=flush, kernel_events=True, lib=lib)
        return total_ms / steps / 1e3, kern_ms / steps / 1e3

    def fp64_frac(fmas, secs):
        return round(fmas / secs / fma_rate, 4)

    rng = np.random.default_rng(1)
    # Laplacian: F64/I64, F32/I32, F32/I64 CSR; CSC F64/I32; SpMM k=16; COO->CSR
    for it, dt, tag in ((np.int64, np.float64, "f64_i64"), (np.int32, np.float32, "f32_i32"),
                        (np.int64, np.float32, "f32_i64")):
        m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=it, dtype=dt)
        A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
        xh = rng.uniform(-1, 1, n).astype(dt)
        x = torch.from_numpy(xh).to(dev)
        y = torch.empty(m, dtype=x.dtype, device=dev)
        t, tk = time_call(lambda: gsa.mul_(y, A, x))
        b = spmv_bytes(m, n, cv.size, np.dtype(dt).itemsize, np.dtype(it).itemsize)
        out[f"laplacian_csr_spmv_{tag}"] = {"GBps": round(b / t / 1e9, 1), "kernel_GBps": round(b / tk / 1e9, 1),
                                             "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                             "max_rel_error": fp64_error(scipy_csr(m, n, rp, cv, nz), xh,
                                                                         y.cpu().numpy())}
        del A
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=np.int32, dtype=np.float64)
    S = scipy_csr(m, n, rp, cv, nz)
    A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    xh = rng.uniform(-1, 1, n)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty(m, dtype=torch.float64, device=dev)
    b1 = spmv_bytes(m, n, cv.size, 8, 4)
    t, tk = time_call(lambda: gsa.mul_(y, A, x, algo=gsa.ALGO_VECTOR))
    out["laplacian_csr_spmv_f64_i32_vector"] = {"GBps": round(b1 / t / 1e9, 1), "kernel_GBps": round(b1 / tk / 1e9, 1),
                                                 "us": round(t * 1e6, 2),
                                                 "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.adapt(dev, gsa.GenericSparseMatrixCSC(m, n, cp, rv, cz))
    t, tk = time_call(lambda: gsa.mul_(y, K, x))
    out["laplacian_csc_spmv_f64_i32"] = {"GBps": round(b1 / t / 1e9, 1), "kernel_GBps": round(b1 / tk / 1e9, 1),
                                          "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                          "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    Xh = rng.uniform(-1, 1, (n, 16))
    X = torch.empty((16, n), dtype=torch.float64, device=dev).t()
    X.copy_(torch.from_numpy(Xh))
    Y = torch.empty((16, m), dtype=torch.float64, device=dev).t()
    bk = spmv_bytes(m, n, cv.size, 8, 4, k=16)
    t, tk = time_call(lambda: gsa.mul_(Y, A, X))
    out["laplacian_csr_spmm_k16_f64_i32"] = {"GBps": round(bk / t / 1e9, 1), "kernel_GBps": round(bk / tk / 1e9, 1),
                                              "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                              "fp64_frac": fp64_frac(16 * cv.size, tk),
                                              "max_rel_error": fp64_error(S, Xh, Y.cpu().numpy())}
    t, tk = time_call(lambda: gsa.mul_(Y, K, X))
    out["laplacian_csc_spmm_k16_f64_i32"] = {"GBps": round(bk / t / 1e9, 1), "kernel_GBps": round(bk / tk / 1e9, 1),
                                              "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                              "fp64_frac": fp64_frac(16 * cv.size, tk),
                                              "max_rel_error": fp64_error(S, Xh, Y.cpu().numpy())}
    del X, Y, K
    _, _, r, c, v = wl.permuted_coo(m, n, rp, cv, nz, seed=7)
    C = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, r.astype(np.int64), c.astype(np.int64), v))
    bc = cv.size * (8 + 16) + cv.size * (8 + 8) + (m + 1) * 8
    holder = {}
    t, tk = time_call(lambda: holder.__setitem__("B", gsa.GenericSparseMatrixCSR(C)))
    B = holder.pop("B")
    exact = (np.array_equal(B.rowptr.cpu().numpy(), rp.astype(np.int64))
             and np.array_equal(B.colval.cpu().numpy(), cv.astype(np.int64))
             and np.array_equal(B.nzval.cpu().numpy(), nz))
    del B
    out["laplacian_coo_to_csr_f64_i64"] = {"GBps": round(bc / t / 1e9, 1), "us": round(t * 1e6, 1),
                                           "sort_GBps": round(bc / tk / 1e9, 1), "sort_us": round(tk * 1e6, 1),
                                           "bit_exact": bool(exact)}

    def wall(fn, reps=max(3, steps // 2)):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            timer.flush()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts))

    # COO sum A + transpose(A): 2 x 21M entries sorted column-major, runs summed, zeros dropped
    t = wall(lambda: C + gsa.transpose(C))
    R = C + gsa.transpose(C)
    Rs = (S + S.T).tocsc()
    Rs.sort_indices()
    rr, rc_, rv_ = (R.rowind.cpu().numpy(), R.colind.cpu().numpy(), R.nzval.cpu().numpy())
    cols = np.repeat(np.arange(n), np.diff(Rs.indptr))
    sum_exact = (np.array_equal(rr - 1, Rs.indices) and np.array_equal(rc_ - 1, cols)
                 and np.array_equal(rv_, Rs.data))
    del R, Rs, rr, rc_, rv_, cols
    out["laplacian_coo_plus_transpose_f64_i64"] = {
        "us": round(t * 1e6, 1), "entries_per_s": round(2 * cv.size / t, 1),
        "bit_exact_vs_scipy": bool(sum_exact),
        "note": "wall time of A + transpose(A) through the API (count, allocation, copy)"}
    del C
    # SpGEMM A * A of the Laplacian: 25 products per interior row, all rows in shared memory
    fl = int(np.diff(rp.astype(np.int64))[cv.astype(np.int64) - 1].sum())  # products of A * A
    sq = A @ A
    nnz_sq = gsa.nnz(sq)
    S2 = (S @ S).tocsr()
    S2.sort_indices()
    gem_exact = (np.array_equal(sq.rowptr.cpu().numpy().astype(np.int64) - 1, S2.indptr)
                 and np.array_equal(sq.colval.cpu().numpy().astype(np.int64) - 1, S2.indices)
                 and np.array_equal(sq.nzval.cpu().numpy(), S2.data))
    del sq, S2
    t = wall(lambda: A @ A)
    out["laplacian_spgemm_a_times_a_f64_i32"] = {
        "us": round(t * 1e6, 1), "products": fl, "products_per_s": round(fl / t, 1), "nnz_c": nnz_sq,
        "bit_exact_vs_scipy": bool(gem_exact),
        "note": "wall time of A * A through the API (symbolic, allocation, numeric)"}
    del A
    # power-law ComplexF64 CSR and COO
    m, n, rp, cv, nz = wl.power_law(1_000_000, seed=0, itype=np.int64, dtype=np.complex128)
    S = scipy_csr(m, n, rp, cv, nz)
    A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    xh = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty(m, dtype=torch.complex128, device=dev)
    bp = spmv_bytes(m, n, cv.size, 16, 8)
    t, tk = time_call(lambda: gsa.mul_(y, A, x))
    out["powerlaw_csr_spmv_c64_i64"] = {"GBps": round(bp / t / 1e9, 1), "kernel_GBps": round(bp / tk / 1e9, 1),
                                         "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                         "nnz": int(cv.size), "fp64_frac": fp64_frac(4 * cv.size, tk),
                                         "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    Cp = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, wl.csr_rows(rp), cv, nz))
    bq = cv.size * (16 + 16) + n * 16 + m * 16
    t, tk = time_call(lambda: gsa.mul_(y, Cp, x))
    out["powerlaw_coo_spmv_c64_i64"] = {"GBps": round(bq / t / 1e9, 1), "kernel_GBps": round(bq / tk / 1e9, 1),
                                         "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                         "fp64_frac": fp64_frac(4 * cv.size, tk),
                                         "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    # the same COO with its triplets in random order: the atomic COO kernel (no row pointers)
    _, _, r, c, v = wl.permuted_coo(m, n, rp, cv, nz, seed=3)
    Cr = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, r, c, v))
    del r, c, v
    t, tk = time_call(lambda: gsa.mul_(y, Cr, x))
    out["powerlaw_coo_random_order_spmv_c64_i64"] = {
        "GBps": round(bq / t / 1e9, 1), "kernel_GBps": round(bq / tk / 1e9, 1), "us": round(t * 1e6, 2),
        "kernel_us": round(tk * 1e6, 2), "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    del Cr
    # three-argument dot(x, A, y) on the same matrix (the call returns the scalar to the host)
    xl = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    xd = torch.from_numpy(xl).to(dev)
    val = gsa.dot(xd, A, x)
    torch.cuda.synchronize()
    ref = np.vdot(xl, S @ xh)
    dscale = float(np.abs(xl) @ (abs(S) @ np.abs(xh)))
    ts = []
    for _ in range(max(5, steps)):
        timer.flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gsa.dot(xd, A, x)
        ts.append(time.perf_counter() - t0)
    td = float(np.median(ts))
    out["powerlaw_csr_dot_c64_i64"] = {"GBps": round(bp / td / 1e9, 1), "us": round(td * 1e6, 2),
                                       "rel_error": float(abs(complex(val) - ref) / dscale),
                                       "note": "wall time of gsa.dot incl. the scalar's copy to the host"}
    del A, Cp
    # n = 1e5 Poisson(10): CSR / CSC / COO (18 MB: L2-resident unless flushed; timed both ways,
    # the main figures with L2 flushed, the l2_warm_* ones back to back with the operands in L2)
    m, n, rp, cv, nz = wl.random_poisson(100_000, seed=0)
    S = scipy_csr(m, n, rp, cv, nz)
    A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.adapt(dev, gsa.GenericSparseMatrixCSC(m, n, cp, rv, cz))
    Co = gsa.GenericSparseMatrixCOO(K)
    xh = rng.uniform(-1, 1, n)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty(m, dtype=torch.float64, device=dev)
    br = spmv_bytes(m, n, cv.size, 8, 8)
    for name, M in (("csr", A), ("csc", K), ("coo", Co)):
        t, tk = time_call(lambda: gsa.mul_(y, M, x))
        tw, tkw = time_call(lambda: gsa.mul_(y, M, x), flush=False)
        out[f"random1e5_{name}_spmv_f64_i64"] = {"GBps": round(br / t / 1e9, 1), "kernel_GBps": round(br / tk / 1e9, 1),
                                                 "us": round(t * 1e6, 2), "kernel_us": round(tk * 1e6, 2),
                                                 "l2_warm_us": round(tw * 1e6, 2), "l2_warm_kernel_us": round(tkw * 1e6, 2),
                                                 "l2_warm_kernel_GBps": round(br / tkw / 1e9, 1),
                                                 "max_rel_error": fp64_error(S, xh, y.cpu().numpy())}
    return out


def batched_products(gsa, wl, torch, dev, count=4096, seed=11, ks=(1, 4, 8)):
    """The uneven-size mix: ``count`` banded ComplexF64 CSR matrices (n log-uniform in
    [64, 8192], half-band 3 plus Poisson(8) off-band entries per row), each with its own
    column-major X of k in ``ks`` (cycled) columns U(-1,1) + iU(-1,1), alpha = 1, beta = 0."""
    sizes, rp, cv, nz, ro, eo = wl.banded_batch(count=count, lo=64, hi=8192, seed=seed,
                                                itype=np.int64, dtype=np.complex128, device=dev)
    g = torch.Generator(device=dev).manual_seed(seed + 2)
    prods, a_bytes, xy_bytes = [], 0, 0
    for i, m in enumerate(sizes):
        A = gsa.GenericSparseMatrixCSR(m, m, rp[int(ro[i]) + i: int(ro[i + 1]) + i + 1],
                                       cv[int(eo[i]): int(eo[i + 1])], nz[int(eo[i]): int(eo[i + 1])])
        k = ks[i % len(ks)]
        shape = (m,) if k == 1 else (k, m)
        X = torch.complex(torch.rand(shape, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                          torch.rand(shape, generator=g, device=dev, dtype=torch.float64) * 2 - 1)
        Y = torch.zeros(shape, dtype=torch.complex128, device=dev)
        if k > 1:
            X, Y = X.t(), Y.t()
        prods.append((A, X, Y, 1, 0))
        a_bytes += int(A.nzval.numel()) * (16 + 8) + (m + 1) * 8
        xy_bytes += 2 * m * k * 16
    del rp, cv, nz
    return prods, a_bytes + xy_bytes


def run_batched(gsa, torch, dev, args):
    """Batched mul!/s on the uneven-size mix: one grouped launch replayed from a CUDA graph,
    against one C-ABI mul! per product and one public-API ``mul_`` per product."""
    from genericsparsearrays_gb300 import autotune, batch, workloads as wl
    prods, nbytes = batched_products(gsa, wl, torch, dev)
    count = len(prods)
    cols, g1 = autotune.tune(prods, reps=3)
    b = batch.BatchedMul(prods, columns=cols, g1_avg=g1)
    steps, warm = max(10, args.steps // 10), 3

    def timed(fn, n):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        t0 = time.perf_counter()
        for s, e in ev:
            s.record()
            fn()
            e.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        ms = np.array([s.elapsed_time(e) for s, e in ev])
        return ms, wall

    g_ms, g_wall = timed(lambda: b.run("graph"), steps)
    gr_ms, _ = timed(lambda: b.run("grouped"), steps)
    pc_ms, pc_wall = timed(lambda: b.run("per_call"), max(3, steps // 4))

    def api_loop():
        for A, X, Y, al, be in prods:
            gsa.mul_(Y, A, X, al, be)
    api_ms, api_wall = timed(api_loop, 3)
    # error of every product against the FP64 reference (beta = 0: Y = A X)
    b.run("graph")
    torch.cuda.synchronize()
    err = 0.0
    for A, X, Y, al, be in prods:
        S = scipy_csr(A.m, A.n, A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy())
        err = max(err, fp64_error(S, X.cpu().numpy(), Y.cpu().numpy()))
    b.close()
    graph_rate = count * steps / g_wall
    api_rate = count * 3 / api_wall
    return {
        "workload": f"{count} banded ComplexF64 CSR (n log-uniform [64, 8192], half-band 3 + Poisson(8)), "
                    "k cycled 1/4/8, Int64 indices",
        "mul_per_s_graph": round(graph_rate, 1),
        "mul_per_s_per_call_capi": round(count * pc_ms.size / pc_wall, 1),
        "mul_per_s_per_call_api": round(api_rate, 1),
        "speedup_vs_per_call_api": round(graph_rate / api_rate, 2),
        "speedup_vs_per_call_capi": round(graph_rate / (count * pc_ms.size / pc_wall), 2),
        "batch_ms_p50": round(float(np.percentile(g_ms, 50)), 4),
        "batch_ms_p99": round(float(np.percentile(g_ms, 99)), 4),
        "grouped_ms_p50": round(float(np.percentile(gr_ms, 50)), 4),
        "per_call_capi_batch_ms_p50": round(float(np.percentile(pc_ms, 50)), 4),
        "per_call_api_batch_ms_p50": round(float(np.percentile(api_ms, 50)), 4),
        "GBps_graph": round(nbytes / (float(np.median(g_ms)) / 1e3) / 1e9, 1),
        "bytes_per_batch": nbytes, "columns": cols, "g1_avg": g1,
        "max_rel_error": err, "products_checked": count,
    }


def run_serving(gsa, torch, dev, args, fma_rate):
    """Served mul! stream: Poisson arrivals against a resident registry, continuous batching
    (work-capped grouped launches on four streams) against one ``mul_`` per request as it
    arrives.  First at the configured rate (far above what the FP64 pipe serves: both paths
    saturate), then both at 80 % of the per-call path's measured capacity."""
    from genericsparsearrays_gb300 import serving
    t_gen = time.perf_counter()
    mats = serving.registry_matrices(count=args.serve_matrices, n_lo=1_000, n_hi=args.serve_n_hi,
                                     seed=21, device=dev)
    reg = serving.Registry(150 * 10**9)
    ids = [reg.add(A) for A in mats]
    del mats
    kmax = 32
    g = torch.Generator(device=dev).manual_seed(22)
    xs = {}
    for mid in ids:  # row-major (n, 32) blocks: an entry's k values share cache lines
        A = reg[mid]
        re = torch.rand((A.n, kmax), generator=g, device=dev, dtype=torch.float64) * 2 - 1
        if A.dtype == torch.complex128:
            xs[mid] = torch.complex(re, torch.rand((A.n, kmax), generator=g, device=dev,
                                                   dtype=torch.float64) * 2 - 1)
        else:
            xs[mid] = re
        if not reg.reserve(xs[mid].numel() * xs[mid].element_size()):
            raise SystemExit("serving workload: right-hand sides exceed the HBM budget")
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen

    def mk(rate, duration, seed):
        reqs = serving.poisson_requests(reg, xs, rate=rate, duration=duration, k_lo=1, k_hi=kmax, seed=seed)
        t0 = time.perf_counter() + 0.05
        for r in reqs:
            r.arrival += t0
        return reqs

    ex = serving.GroupedExecutor(dev, slots=args.serve_slots)

    def server():
        return serving.Server(reg, ex, slots=args.serve_slots, keep_outputs=False)

    # warm-up: one short stream through each path (plans, launch shapes, pinned buffers)
    server().run(mk(args.serve_rate, 0.02, 1))
    serving.serve_per_call(reg, mk(args.serve_rate, 0.02, 2), dev, keep_outputs=False)
    torch.cuda.synchronize()

    def both(rate, duration, seed):
        srv = server()
        reqs = mk(rate, duration, seed)
        with torch.cuda.device(dev):
            srv.run(reqs)
        torch.cuda.synchronize()
        st = srv.stats()
        pc = serving.serve_per_call(reg, mk(rate, duration, seed), dev, keep_outputs=False)
        for d in (st, pc):
            d["fp64_frac"] = d.get("fma_per_s", 0.0) / fma_rate
        return len(reqs), st, pc

    def rnd(d):
        return {k: (round(v, 4) if isinstance(v, float) else v) for k, v in d.items()}

    nreq, batched, per_call = both(args.serve_rate, args.serve_seconds, 3)
    capacity = per_call.get("mul_per_s", 0.0)
    rate2 = 0.8 * capacity
    nreq2, batched2, per_call2 = both(rate2, args.serve_seconds_low, 4)
    # error statement: a sample of requests recomputed and checked against the FP64 reference
    err = serving_error_sample(reg, xs, dev, ex)
    nnz_total = sum(int(reg[i].nzval.numel()) for i in ids)
    return {
        "workload": f"{len(ids)} resident CSR matrices (n log-uniform [1e3, {args.serve_n_hi:.0e}], "
                    "5-40 nnz/row uniform or truncated Pareto, Float64 and ComplexF64, Int32 indices); "
                    f"Poisson arrivals {args.serve_rate}/s for {args.serve_seconds}s, k uniform in [1, 32] "
                    "(X: the first k columns of a resident row-major n x 32 block per matrix), "
                    "150 GB HBM budget",
        "requests": nreq, "registry_nnz": nnz_total, "registry_bytes": reg.resident,
        "setup_s": round(t_gen, 1), "slots": args.serve_slots,
        "fp64_fma_rate_probe": round(fma_rate, 1),
        "continuous_batching": rnd(batched), "per_call_mul": rnd(per_call),
        "speedup_mul_per_s": round(batched.get("mul_per_s", 0) / max(per_call.get("mul_per_s", 1e-9), 1e-9), 3),
        "at_80pct_of_per_call_capacity": {
            "rate_per_s": round(rate2, 1), "requests": nreq2, "seconds": args.serve_seconds_low,
            "continuous_batching": rnd(batched2), "per_call_mul": rnd(per_call2),
            "speedup_mul_per_s": round(batched2.get("mul_per_s", 0) / max(per_call2.get("mul_per_s", 1e-9), 1e-9), 3)},
        "max_rel_error_sampled": err,
    }


def serving_error_sample(reg, xs, dev, ex, count=64, seed=5):
    """Error of ``count`` served requests (a grouped launch through the executor, as the server
    runs them) against the FP64 reference."""
    import torch
    from genericsparsearrays_gb300 import serving
    reqs = serving.poisson_requests(reg, xs, rate=1e6, duration=count / 1e6 * 4, k_lo=1, k_hi=32, seed=seed)[:count]
    small = [r for r in reqs if serving.product_fma(reg[r.matrix], r.k) < (1 << 24)][:count // 2]
    err = 0.0
    for batch in (small, reqs[:4]):
        if not batch:
            continue
        h = ex.launch(0, [(reg[r.matrix], r) for r in batch])
        h.synchronize()
        for r in batch:
            A = reg[r.matrix]
            S = scipy_csr(A.m, A.n, A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy())
            err = max(err, fp64_error(S, r.X.cpu().numpy(), r.Y.cpu().numpy()))
            r.Y = None
    torch.cuda.synchronize()
    return err


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gsa", choices=["gsa", "reference"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-matrices", type=int, default=512)
    ap.add_argument("--serve-n-hi", type=float, default=2e6)
    ap.add_argument("--serve-rate", type=float, default=20_000)
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-seconds-low", type=float, default=2.0,
                    help="seconds of arrivals at 80%% of the per-call capacity")
    ap.add_argument("--serve-slots", type=int, default=4, help="launch slots (CUDA streams) of the server")
    ap.add_argument("--e2e-sets", type=int, default=3,
                    help="steps in flight in the end-to-end run (streams and buffer sets)")
    args = ap.parse_args()
    if args.e2e_sets < 1:
        ap.error("--e2e-sets must be at least 1")
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    import __graft_entry__
    __graft_entry__.load_package()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
