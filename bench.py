"""Benchmark: batched log|Pf| + gradient over uneven skew matrices on GB300.

Workload (one step): 4096 real skew-symmetric Float64 matrices with even sizes n
drawn uniformly from {16, 18, ..., 256}, entries (B - B^T)/2 with B iid
N(0, 1/n) (seeded, synthetic); for every matrix log|Pf(A)|, its sign and the
gradient 1/2 A^{-T} through the batched C-ABI entry point.  The inputs (766 MB)
and gradients (766 MB) are each larger than L2, so no flush is needed between
steps.

value: matrices/s with inputs resident in HBM.  e2e: the same through the public
API with pinned host buffers, the H2D copy of the inputs and the D2H copy of
log|Pf|, sign and gradients inside the timed region.

Multi-GPU (torchrun): every rank solves its own batch (weak scaling, no
collective on the data path); value = all matrices / max-over-ranks time.

--impl reference: the reference's CPU algorithm (the oracle's FP64 restatement of
SkewLinearAlgebra.jl, since Julia is not available on the box) on the host
cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "skewlinearalgebra.jl_gb300"))

# dram__bytes_read.sum + dram__bytes_write.sum over the four batch_kernel launches of one
# step of the default workload (4096 matrices, even n in [16, 256]), from one ncu capture
# of the timed step (-s 12 -c 4)
STEP_DRAM_BYTES = 20_753_729_792
METRIC = "batched log|Pf|+grad matrices/s & n=8192 hessenberg GFLOP/s vs plain GPU, err≤1e-11"
UNIT = "matrices/s"
COUNT = 4096
NMIN, NMAX = 16, 256
SEED = 20261203


def workload_sizes(count=COUNT, seed=SEED, rank=0, nmin=NMIN, nmax=NMAX):
    rng = np.random.default_rng(seed + 7919 * rank)
    return (2 * rng.integers(nmin // 2, nmax // 2 + 1, count)).astype(np.int64)


def packed_inputs(sizes, seed=SEED, rank=0):
    """Column-major matrices back to back; returns (buffer, offsets)."""
    offs = np.zeros(len(sizes), dtype=np.int64)
    offs[1:] = np.cumsum(sizes[:-1].astype(np.int64) ** 2)
    total = int(offs[-1] + sizes[-1] ** 2)
    buf = np.empty(total, dtype=np.float64)
    rng = np.random.default_rng(seed + 104729 * (rank + 1))
    for b, n in enumerate(sizes):
        B = rng.standard_normal((n, n)) / np.sqrt(n)
        buf[offs[b]:offs[b] + n * n] = ((B - B.T) / 2).ravel(order="F")
    return buf, offs


def dense_skew_input(n):
    """The single dense real matrix of size n: A = (B - B^T)/2 with B iid N(0,1),
    seeded by n (the n = 512 and n = 8192 single-matrix workloads)."""
    rng = np.random.default_rng(SEED + n)
    B = rng.standard_normal((n, n))
    return (B - B.T) / 2


def dense_skewh_input(n):
    """The single dense ComplexF64 skew-Hermitian matrix of size n: A = (C - C^H)/2
    with the real and imaginary parts of C iid N(0,1), seeded by n."""
    rng = np.random.default_rng(SEED + 3 * n)
    C = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (C - C.conj().T) / 2, rng


def pfaffian_adjoint_inputs(count=1024, n=128):
    """The batched Pfaffian-adjoint workload: (B - B^T)/2 + 0.5 J with B iid
    N(0, 1/n) and J the canonical symplectic form, packed column-major back to
    back, and the loss weights w ~ U(-1, 1)."""
    rng = np.random.default_rng(SEED + 128)
    J = np.kron(np.eye(n // 2), np.array([[0.0, 1.0], [-1.0, 0.0]]))
    buf = np.empty(count * n * n)
    for b in range(count):
        B = rng.standard_normal((n, n)) / np.sqrt(n)
        buf[b * n * n:(b + 1) * n * n] = ((B - B.T) / 2 + 0.5 * J).ravel(order="F")
    w = rng.uniform(-1.0, 1.0, count)
    return buf, w


def exp_adjoint_inputs(count=512):
    """The real exp-adjoint workload: n uniform in {32, 64, ..., 512}, each
    (B - B^T)/2 scaled to a spectral radius ~ U(0.5, 8), cotangents iid N(0,1);
    returns (sizes, offsets, packed inputs, packed cotangents)."""
    rng = np.random.default_rng(SEED + 5)
    sizes = (32 * rng.integers(1, 17, count)).astype(np.int64)
    offs = np.zeros(count, dtype=np.int64)
    offs[1:] = np.cumsum(sizes[:-1] ** 2)
    total = int(offs[-1] + sizes[-1] ** 2)
    buf = np.empty(total)
    cot = rng.standard_normal(total)
    for b, n in enumerate(sizes):
        B = rng.standard_normal((n, n))
        A = (B - B.T) / 2
        rho = np.abs(np.linalg.eigvalsh(1j * A)).max()
        A *= rng.uniform(0.5, 8.0) / rho
        buf[offs[b]:offs[b] + n * n] = A.ravel(order="F")
    return sizes, offs, buf, cot


def complex_exp_adjoint_inputs(count=64, n=256):
    """The complex exp-adjoint workload: ComplexF64 skew-Hermitian (C - C^H)/2
    scaled to a spectral radius ~ U(0.5, 8), cotangents iid complex N(0,1)."""
    rng = np.random.default_rng(SEED + 64)
    mats, cots = [], []
    for _ in range(count):
        C = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        A = (C - C.conj().T) / 2
        A *= rng.uniform(0.5, 8.0) / np.abs(np.linalg.eigvalsh(1j * A)).max()
        mats.append(A)
        cots.append(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return mats, cots


def flops_per_matrix(n):
    """Algorithmic FP64 work: Householder tridiagonalisation 4/3 n^3 plus the
    gradient Q (-1/2 T^{-1}) Q^T by two-sided reflector application 2 n^3."""
    n = np.asarray(n, dtype=np.float64)
    return 4.0 / 3.0 * n ** 3 + 2.0 * n ** 3


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(sizes_all, steps, warmup, sample, nthreads, rank):
    """The reference's CPU algorithm (oracle FP64 restatement) on a bounded sample."""
    from oracle import oracle as O

    sizes = sizes_all[:sample]
    buf, offs = packed_inputs(sizes, rank=rank)
    for _ in range(warmup):
        O.batch_logabspfaffian_grad_packed(buf, offs, sizes, nthreads)
    times = []
    out = None
    for _ in range(steps):
        t0 = time.perf_counter()
        out = O.batch_logabspfaffian_grad_packed(buf, offs, sizes, nthreads)
        times.append(time.perf_counter() - t0)
    return len(sizes) / float(np.mean(times)), out, float(np.mean(times))


def _lapack_share(job):
    """One worker process: LAPACK through scipy's OpenBLAS (one thread) on its share of
    the workload's sizes, entries of the same distribution: dsytrd (Householder
    tridiagonalisation, the same 4/3 n^3 as the skew reduction; LAPACK has no skew
    routine) and dgetrf + dgetri (the inverse that gives the gradient, 2 n^3).
    Returns the seconds spent in the LAPACK calls."""
    sizes, seed = job
    from scipy.linalg import lapack

    rng = np.random.default_rng(seed)
    mats = []
    for n in sizes:
        B = rng.standard_normal((int(n), int(n))) / np.sqrt(n)
        mats.append(np.asfortranarray((B - B.T) / 2))
    t0 = time.perf_counter()
    for A in mats:
        lapack.dsytrd(A, lower=1)
        lu, piv, _ = lapack.dgetrf(A)
        lapack.dgetri(lu, piv)
    return time.perf_counter() - t0


def lapack_context(sizes, procs):
    """BLAS-backed CPU context for the headline: the same sizes through LAPACK, one
    single-threaded process per core (spawned), matrices dealt round robin; one
    untimed pass (imports, page faults), then one timed pass.  Matrices/s over the
    slowest process."""
    import multiprocessing as mp

    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ["OPENBLAS_NUM_THREADS"] = "1"  # inherited by the spawned workers
    os.environ["OMP_NUM_THREADS"] = "1"
    try:
        with mp.get_context("spawn").Pool(procs) as pool:
            shares = [sizes[i::procs] for i in range(procs)]
            pool.map(_lapack_share, [(sh, 100 + i) for i, sh in enumerate(shares)])
            secs = pool.map(_lapack_share, [(sh, 200 + i) for i, sh in enumerate(shares)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return {"value": len(sizes) / max(secs), "unit": UNIT, "cores": procs,
            "calls": "per matrix: dsytrd + dgetrf + dgetri (scipy's OpenBLAS, one thread per process)",
            "sample": f"all {len(sizes)} matrices of the workload's sizes, entries of the same distribution",
            "note": "context only: LAPACK's symmetric tridiagonalisation has the skew reduction's cost; "
                    "the inverse gives the gradient"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    sizes = workload_sizes()
    sample = args.cpu_sample
    value, _, sec = cpu_reference(sizes, max(1, args.steps), min(args.warmup, 1), sample, nthreads, 0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"batched_logabspf_grad_{COUNT}x_even_n{NMIN}-{NMAX}", "count": COUNT,
                   "n_range": [NMIN, NMAX], "entries": "(B-B^T)/2, B~N(0,1/n)", "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": (f"all {sample} matrices of the workload per step" if sample >= COUNT else
                                    f"first {sample} matrices of the workload per step") +
                                   "; Julia is absent on the box, so the oracle's FP64 restatement of "
                                   "SkewLinearAlgebra.jl (logabspfaffian) plus an FP64 Gauss-Jordan inverse for the "
                                   "gradient, OpenMP over matrices, scalar C++ -O3 without BLAS"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=COUNT)
    ap.add_argument("--plain-sample", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--count", type=int, default=COUNT, help="matrices per step (profiling cases)")
    ap.add_argument("--nmin", type=int, default=NMIN)
    ap.add_argument("--nmax", type=int, default=NMAX)
    ap.add_argument("--large-n", type=int, default=8192, help="single-matrix hessenberg leg (0 = skip)")
    ap.add_argument("--only-large", action="store_true", help="run only the single-matrix hessenberg leg")
    ap.add_argument("--no-legs", action="store_true", help="skip the eigvals / n=512 / adjoint legs")
    ap.add_argument("--only-legs", action="store_true", help="run only the eigvals / n=512 / adjoint legs")
    ap.add_argument("--leg", default=None, help="with --only-legs: run only this leg (profiling)")
    ap.add_argument("--complex-n", type=int, default=4096,
                    help="with --only-legs: size of the single ComplexF64 leg (profiling cases)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only_legs:
        import torch

        import skewgpu

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        peak = skewgpu.measure_fp64_peak()
        sizes = workload_sizes(args.count, nmin=args.nmin, nmax=args.nmax)
        buf, offs = packed_inputs(sizes)
        d_in = torch.from_numpy(buf).to("cuda")
        plan = skewgpu.BatchPlan(sizes)
        legs = {"eigvals_batched": lambda: leg_eigvals_batched(plan, d_in, offs, sizes, max(1, args.steps)),
                "plain_n512": lambda: leg_plain_n512(peak, cpu=not args.no_cpu),
                "pfaffian_adjoint_1024x128": lambda: leg_pfaffian_adjoint(peak, max(1, args.steps)),
                "exp_adjoint_512_mixed": lambda: leg_exp_adjoint(peak, max(1, min(args.steps, 3))),
                "exp_adjoint_complex_64x256": lambda: leg_complex_exp_adjoint(peak),
                "complex_n4096": lambda: leg_complex_large(args.complex_n, peak),
                "complex_pfaffian_2048x128": lambda: leg_complex_pfaffian(peak, cpu=not args.no_cpu)}
        out = {k: f() for k, f in legs.items() if args.leg is None or k == args.leg}
        plan.close()
        print(json.dumps({"legs": out}), flush=True)
        return 0
    if args.only_large:
        import torch

        import skewgpu

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        peak = skewgpu.measure_fp64_peak()
        out = {"hessenberg": bench_hessenberg_large(args.large_n, max(1, args.steps), peak)}
        if not args.no_legs:
            out["eigen"] = leg_eigen_large(args.large_n, peak)
        print(json.dumps(out), flush=True)
        return 0

    import torch

    import skewgpu
    from skewgpu import replicas

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    world, rank, local, dist = replicas.init_from_env("nccl")

    count = args.count
    sizes = workload_sizes(count, rank=rank, nmin=args.nmin, nmax=args.nmax)
    buf, offs = packed_inputs(sizes, rank=rank)
    total = buf.size
    h_in = torch.from_numpy(buf).pin_memory()
    d_in = h_in.to("cuda")
    d_grad = torch.empty(total, dtype=torch.float64, device="cuda")
    base_in, base_g = d_in.data_ptr(), d_grad.data_ptr()
    a_ptrs = torch.tensor((base_in + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    g_ptrs = torch.tensor((base_g + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    plan = skewgpu.BatchPlan(sizes)
    logpf = torch.empty(count, dtype=torch.float64, device="cuda")
    sign = torch.empty_like(logpf)
    status = torch.empty(count, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fp64_peak = skewgpu.measure_fp64_peak()

    def step():
        plan.logabspfaffian(a_ptrs, g_ptrs, logpf, sign, status)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    st = status.cpu().numpy()
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    barrier()
    wall = time.perf_counter() - t0
    ms_dev = ev0.elapsed_time(ev1)
    sec = replicas.max_over_ranks(ms_dev / 1e3, dist, "cuda")
    value = replicas.weak_scaling_throughput(count, world, args.steps, sec)

    # e2e through the public host-buffer call (skew_batch_logabspf_host_d): page-locked
    # host inputs in, log|Pf|, sign, status and every gradient back in host memory;
    # the kernels move each matrix over the host link themselves.
    h_lp = torch.empty(count, dtype=torch.float64).pin_memory()
    h_sg = torch.empty_like(h_lp).pin_memory()
    h_st = torch.empty(count, dtype=torch.int32).pin_memory()
    h_g = torch.empty(total, dtype=torch.float64).pin_memory()
    e2e_steps = max(1, min(args.steps, 5))
    plan.logabspfaffian_host(h_in, h_g, h_lp, h_sg, h_st)  # host-path workspace, outside the timing
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        plan.logabspfaffian_host(h_in, h_g, h_lp, h_sg, h_st)
    e1.record(stream)
    barrier()
    e2e_sec = replicas.max_over_ranks(e0.elapsed_time(e1) / 1e3, dist, "cuda")
    e2e_value = replicas.weak_scaling_throughput(count, world, e2e_steps, e2e_sec)
    e2e_ok = bool((h_st.numpy() == st).all())
    # the same with whole-batch copies around the device-pointer call on one stream
    e0.record(stream)
    for _ in range(e2e_steps):
        d_in.copy_(h_in, non_blocking=True)
        step()
        h_lp.copy_(logpf, non_blocking=True)
        h_sg.copy_(sign, non_blocking=True)
        h_g.copy_(d_grad, non_blocking=True)
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    staged_sec = replicas.max_over_ranks(e0.elapsed_time(e1) / 1e3, dist, "cuda")
    staged_value = replicas.weak_scaling_throughput(count, world, e2e_steps, staged_sec)

    # roofline of the dominant kernel (batch_kernel: every launch of a step)
    flops = float(flops_per_matrix(sizes).sum())
    achieved_tflops = flops / (ms_dev / args.steps / 1e3) / 1e12

    # plain per-matrix GPU path: single-matrix C-ABI call looped over a sample
    plain = None
    if args.plain_sample > 0:
        idx = np.arange(min(args.plain_sample, count))
        mats = [d_in[offs[b]:offs[b] + sizes[b] ** 2].view(int(sizes[b]), int(sizes[b])) for b in idx]
        gbuf = [torch.empty_like(m) for m in mats]
        import ctypes

        L = skewgpu._lib.load()
        h = skewgpu.handle().bind()
        work = [m.clone() for m in mats]
        outs = torch.empty(2 * len(idx), dtype=torch.float64, device="cuda")
        info = torch.empty(len(idx), dtype=torch.int32, device="cuda")

        def refill():
            for k in range(len(idx)):
                work[k].copy_(mats[k])

        def plain_pass():
            for k, b in enumerate(idx):
                L.skew_logabspf_grad_d(h, ctypes.c_void_p(work[k].data_ptr()), int(sizes[b]), int(sizes[b]),
                                       ctypes.c_void_p(outs.data_ptr() + 16 * k),
                                       ctypes.c_void_p(outs.data_ptr() + 16 * k + 8),
                                       ctypes.c_void_p(gbuf[k].data_ptr()), int(sizes[b]),
                                       ctypes.c_void_p(info.data_ptr() + 4 * k))

        refill()
        plain_pass()
        refill()
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        plain_pass()
        p1.record(stream)
        torch.cuda.synchronize()
        plain_val = len(idx) / (p0.elapsed_time(p1) / 1e3)
        # same sample through the batched path (a plan over the sample only)
        splan = skewgpu.BatchPlan(sizes[idx])
        sa = a_ptrs[: len(idx)]
        sg_ = g_ptrs[: len(idx)]
        slp = torch.empty(len(idx), dtype=torch.float64, device="cuda")
        ssg = torch.empty_like(slp)
        sst = torch.empty(len(idx), dtype=torch.int32, device="cuda")
        splan.logabspfaffian(sa, sg_, slp, ssg, sst)
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        for _ in range(3):
            splan.logabspfaffian(sa, sg_, slp, ssg, sst)
        q1.record(stream)
        torch.cuda.synchronize()
        batched_sample_val = 3 * len(idx) / (q0.elapsed_time(q1) / 1e3)
        splan.close()
        plain = {"value": plain_val, "unit": UNIT, "sample": int(len(idx)),
                 "batched_same_sample": batched_sample_val, "speedup_full_batch": value / world / plain_val,
                 "speedup_same_sample": batched_sample_val / plain_val}

    cpu = None
    check = None
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        cval, (clp, csg, cgrad), _ = cpu_reference(sizes, 1, 0, args.cpu_sample, nthreads, rank)
        cpu = {"value": cval, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"first {args.cpu_sample} of the {count} matrices of the workload, one pass; oracle FP64 "
                         "restatement of logabspfaffian + FP64 Gauss-Jordan gradient, OpenMP over matrices, "
                         "scalar C++ -O3 without BLAS"}
        try:
            cpu["lapack_context"] = lapack_context(sizes, nthreads)
        except Exception as e:  # scipy missing: the context is optional
            cpu["lapack_context"] = {"unavailable": f"{type(e).__name__}: {e}"}
        k = args.cpu_sample
        glp = logpf[:k].cpu().numpy()
        gsg = sign[:k].cpu().numpy()
        rel = np.abs(glp - clp) / np.maximum(1.0, np.abs(clp))
        gg = d_grad[: int(offs[k - 1] + sizes[k - 1] ** 2)].cpu().numpy()
        gerr = 0.0
        for b in range(k):
            a, e = int(offs[b]), int(offs[b] + sizes[b] ** 2)
            gerr = max(gerr, float(np.abs(gg[a:e] - cgrad[a:e]).max() / np.abs(cgrad[a:e]).max()))
        check = {"max_rel_logpf_vs_cpu": float(rel.max()), "sign_mismatches": int((gsg != csg).sum()),
                 "max_rel_grad_vs_cpu": gerr, "matrices": k, "status_nonzero": int((st != 0).sum())}

    large = None
    eig_large = None
    if rank == 0 and args.large_n > 0:
        large = bench_hessenberg_large(args.large_n, 2, fp64_peak)
        if not args.no_cpu:
            large["leading_256_vs_cpu_port"] = leading_256_check(args.large_n)
        eig_large = leg_eigen_large(args.large_n, fp64_peak)
    legs = {}
    if rank == 0 and not args.no_legs:
        legs["eigvals_batched"] = leg_eigvals_batched(plan, d_in, offs, sizes, args.steps)
        legs["plain_n512"] = leg_plain_n512(fp64_peak, cpu=not args.no_cpu)
        legs["pfaffian_adjoint_1024x128"] = leg_pfaffian_adjoint(fp64_peak, args.steps)
        legs["exp_adjoint_512_mixed"] = leg_exp_adjoint(fp64_peak, max(1, min(args.steps, 3)))
        legs["exp_adjoint_complex_64x256"] = leg_complex_exp_adjoint(fp64_peak)
        legs["complex_n4096"] = leg_complex_large(4096, fp64_peak)
        legs["complex_pfaffian_2048x128"] = leg_complex_pfaffian(fp64_peak, cpu=not args.no_cpu)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"batched_logabspf_grad_{count}x_even_n{args.nmin}-{args.nmax}", "count": count,
                       "n_range": [args.nmin, args.nmax], "entries": "(B-B^T)/2, B~N(0,1/n)",
                       "l2": "inputs and gradients each 766 MB > L2; no flush", "parallelism": f"replica x{world}"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(total * 8),
                    "d2h_bytes_per_step": int(total * 8 + count * 20), "steps": e2e_steps,
                    "call": "skew_batch_logabspf_host_d (page-locked host buffers)", "status_match": e2e_ok,
                    "staged_copies": {"value": staged_value, "note": "whole-batch cudaMemcpyAsync in and out "
                                      "around skew_batch_logabspf_d on one stream"}},
            "roofline": {"bound": "fp64", "achieved": achieved_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved_tflops / fp64_peak, "traffic": STEP_DRAM_BYTES if (count, args.nmin, args.nmax) == (COUNT, NMIN, NMAX) else None,
                         "traffic_unit": "bytes per step (DRAM read + write of the step's batch_kernel "
                                         "launches, one ncu capture of the default workload)",
                         "algorithmic_bytes_per_step": int(2 * total * 8),
                         "peak_source": "FP64 DFMA peak measured live by skew_measure_fp64_peak "
                                        "(MEASURED_PEAKS.json has no FP64 figure)",
                         "algorithmic_flops_per_step": flops, "kernel": "batch_kernel"},
            "gpu_launches": int(args.steps * _launches_per_call(sizes)),
            "tuning": skewgpu.tuning_source(),
            "fp64_pipes_tflops": skewgpu.measure_fp64_pipes(),
            "clocks": clk,
            "wall_s": wall,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if check:
            line["check"] = check
        if plain:
            line["plain_gpu"] = plain
        if large:
            line[f"hessenberg_n{args.large_n}"] = large
        if eig_large:
            line[f"eigen_n{args.large_n}"] = eig_large
        if legs:
            line["legs"] = legs
        print(json.dumps(line), flush=True)
    plan.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def bench_hessenberg_large(n, reps, fp64_peak):
    """Single dense skew matrix: blocked Householder tridiagonalisation on the
    whole GPU (skew_hessenberg_d), timed with CUDA events per call; the input is
    restored from a pristine device copy outside the timed region."""
    import ctypes

    import torch

    import skewgpu

    A = dense_skew_input(n)
    pristine = skewgpu.to_device(A)
    work = torch.empty_like(pristine)
    tau = torch.empty(n - 1, dtype=torch.float64, device="cuda")
    ev = torch.empty(n - 1, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    times = []
    for r in range(reps + 1):
        work.copy_(pristine)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.skew_hessenberg_d(h, ctypes.c_void_p(work.data_ptr()), n, n, ctypes.c_void_p(tau.data_ptr()),
                                 ctypes.c_void_p(ev.data_ptr()), ctypes.c_void_p(info.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        assert st == 0, st
        if r > 0:
            times.append(e0.elapsed_time(e1) / 1e3)
    sec = float(np.median(times))
    flops = 4.0 / 3.0 * n ** 3
    e = ev.cpu().numpy()
    fro_rel = abs(np.sqrt(2.0 * np.sum(e * e)) - np.linalg.norm(A)) / np.linalg.norm(A)
    # logabspfaffian of the same matrix (skew_logabspf_d: the reduction, then log|Pf| and
    # the sign from ev and tau), checked against 1/2 log|det A| from cuSOLVER's LU
    out2 = torch.zeros(2, dtype=torch.float64, device="cuda")
    lp_times = []
    for r in range(reps + 1):
        work.copy_(pristine)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.skew_logabspf_d(h, ctypes.c_void_p(work.data_ptr()), n, n, ctypes.c_void_p(out2.data_ptr()),
                               ctypes.c_void_p(out2.data_ptr() + 8), 0, ctypes.c_void_p(info.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        assert st == 0, st
        if r > 0:
            lp_times.append(e0.elapsed_time(e1) / 1e3)
    lp, sg = (float(x) for x in out2.cpu().numpy())
    sdet, ldet = torch.linalg.slogdet(pristine)
    del work
    return {"n": n, "ms": sec * 1e3, "gflops": flops / sec / 1e9, "frac_fp64": flops / sec / 1e12 / fp64_peak,
            "algorithmic_flops": flops, "reps": reps, "check_frobenius_rel": float(fro_rel),
            "logabspfaffian": {"ms": float(np.median(lp_times)) * 1e3, "logpf": lp, "sign": sg,
                               "check_rel_vs_half_logdet": float(abs(lp - 0.5 * ldet.item()) / abs(0.5 * ldet.item())),
                               "det_sign": float(sdet.item())}}


def leading_256_check(n=8192, k=256):
    """The single large dense matrix's leading k x k principal submatrix through the
    single-matrix calls, next to the oracle's FP64 restatement of the reference
    (the CPU port, one host core): hessenberg ev, eigvals (the reference's order) and
    log|Pf|, with the port's times and the largest differences."""
    import skewgpu
    from oracle import oracle as O

    A = np.ascontiguousarray(dense_skew_input(n)[:k, :k])
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    vals = skewgpu.eigvals(A).imag
    lp, sg = skewgpu.logabspfaffian(A)
    t0 = time.perf_counter()
    _, _, evo = O.hessenberg(A)
    t1 = time.perf_counter()
    vo, _ = O.eigvals(A)
    t2 = time.perf_counter()
    lpo, sgo = O.logabspfaffian(A)
    t3 = time.perf_counter()
    return {"k": k, "cpu_port_ms": {"hessenberg": (t1 - t0) * 1e3, "eigvals": (t2 - t1) * 1e3,
                                    "logabspfaffian": (t3 - t2) * 1e3, "cores": 1},
            "max_rel_ev_vs_port": float(np.abs(ev - evo).max() / np.abs(evo).max()),
            "max_rel_eigvals_vs_port_same_order": float(np.abs(vals - vo).max() / np.abs(vo).max()),
            "logpf_rel_vs_port": float(abs(lp - lpo) / abs(lpo)), "sign_equal": bool(sg == sgo)}


def leg_eigen_large(n, fp64_peak, reps=1):
    """eigen with vectors of one dense n x n skew matrix (A = (B - B^T)/2, B iid
    N(0,1)) through skew_eigen_d: blocked reduction, bisection, twisted
    eigenvectors, blocked back-transformation; input restored outside the timed
    region.  Checked on 16 sampled eigenpairs: residual |A v - i lambda v| and
    orthonormality of the sample (torch FP64 on the device, outside the timing)."""
    import ctypes

    import torch

    import skewgpu

    A = dense_skew_input(n)
    rng = np.random.default_rng(SEED + n + 1)
    pristine = skewgpu.to_device(A)
    work = torch.empty_like(pristine)
    vals = torch.empty(n, dtype=torch.float64, device="cuda")
    Vr = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.empty((n, n), dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    times = []
    for r in range(reps + 1):
        work.copy_(pristine)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.skew_eigen_d(h, P(work), n, n, P(vals), P(Vr), P(Vi), n, P(info))
        e1.record(stream)
        torch.cuda.synchronize()
        assert st == 0, st
        if r:
            times.append(e0.elapsed_time(e1) / 1e3)
    sec = float(np.median(times))
    # device buffers hold A^T (column-major A); V columns are Vr.T[:, k] in torch terms
    At = pristine.T
    idx = torch.tensor(np.sort(rng.choice(n, 16, replace=False)), device="cuda")
    Vs = torch.complex(Vr.T[:, idx], Vi.T[:, idx])
    lam = 1j * vals[idx]
    Ac = torch.complex(At, torch.zeros_like(At))
    res = (Ac @ Vs - Vs * lam).abs().max().item() / vals.abs().max().item()
    orth = (Vs.conj().T @ Vs - torch.eye(16, dtype=Vs.dtype, device="cuda")).abs().max().item()
    # the work of this algorithm: reduction 4/3 n^3, back-transformation of the n real
    # columns that carry the -sigma vectors (the +sigma ones are their conjugates) 2 n^3
    flops = (4.0 / 3.0 + 2.0) * n ** 3
    return {"n": n, "ms": sec * 1e3, "algorithmic_flops": flops, "gflops": flops / sec / 1e9,
            "frac_fp64": flops / sec / 1e12 / fp64_peak, "reps": reps,
            "check_sample": {"pairs": 16, "max_residual_rel": res, "max_orthonormality_err": orth}}


def leg_complex_large(n, fp64_peak, reps=1):
    """One ComplexF64 skew-Hermitian n x n matrix, A = (C - C^H)/2 with re/im of C
    iid N(0,1): hessenberg (skew_hessenberg_z) and eigen with vectors
    (skew_eigen_z), each timed with CUDA events, input restored outside the timed
    region; eigen checked on 16 sampled pairs."""
    import ctypes

    import torch

    import skewgpu

    A, rng = dense_skewh_input(n)
    pristine = skewgpu.to_device_complex(A)
    work = torch.empty_like(pristine)
    tau = torch.empty(n - 1, dtype=torch.complex128, device="cuda")
    ev = torch.empty(n - 1, dtype=torch.float64, device="cuda")
    dvim = torch.empty(n, dtype=torch.float64, device="cuda")
    vals = torch.empty(n, dtype=torch.float64, device="cuda")
    V = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    calls = {
        "hessenberg": lambda: L.skew_hessenberg_z(h, P(work), n, n, P(tau), P(ev), P(dvim), P(info)),
        "eigen": lambda: L.skew_eigen_z(h, P(work), n, n, P(vals), P(V), n, P(info)),
    }
    res = {"n": n}
    for name, fn in calls.items():
        times = []
        for r in range(reps + 1):
            work.copy_(pristine)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert fn() == 0
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
        res[f"{name}_ms"] = float(np.median(times))
    flops_h = 16.0 / 3.0 * n ** 3  # complex reduction in real flops
    res["hessenberg_gflops"] = flops_h / (res["hessenberg_ms"] / 1e3) / 1e9
    res["hessenberg_frac_fp64"] = res["hessenberg_gflops"] / 1e3 / fp64_peak
    At = pristine.T  # device buffer holds A^T (column-major A)
    idx = torch.tensor(np.sort(rng.choice(n, 16, replace=False)), device="cuda")
    Vs = V.T[:, idx]
    lam = 1j * vals[idx]
    r = (At @ Vs - Vs * lam).abs().max().item() / vals.abs().max().item()
    o = (Vs.conj().T @ Vs - torch.eye(16, dtype=Vs.dtype, device="cuda")).abs().max().item()
    res["check_sample"] = {"pairs": 16, "max_residual_rel": r, "max_orthonormality_err": o}
    return res


def leg_complex_exp_adjoint(fp64_peak, count=64, n=256, steps=3):
    """The exp-adjoint workload's complex part: 64 ComplexF64 skew-Hermitian
    matrices, n = 256, scaled to a spectral radius ~ U(0.5, 8), cotangents iid
    complex N(0,1); all G_i in one batched call (skew_batch_exp_vjp_z), inputs
    resident in HBM."""
    import ctypes

    import torch

    import skewgpu

    mats, cots = complex_exp_adjoint_inputs(count, n)
    dA = skewgpu._stack_complex(mats)
    dC = skewgpu._stack_complex(cots)
    dG = torch.empty_like(dA)
    st = torch.zeros(count, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def run():
        assert L.skew_batch_exp_vjp_z(h, P(dA), n, count, P(dC), P(dG), P(st)) == 0

    for _ in range(2):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / steps
    # algorithmic work in real flops: reduction 16/3 n^3, back-transformation of the complex
    # eigenvectors 8 n^3, the exp assembly V e^L V^H 8 n^3 and the adjoint's three complex
    # products 24 n^3 (the real count (4/3 + 4 + 4 + 6) n^3 with complex arithmetic)
    flops = count * (16.0 / 3.0 + 8.0 + 8.0 + 24.0) * n ** 3
    return {"value": count / sec, "unit": "matrices/s", "ms_per_step": sec * 1e3, "count": count, "n": n,
            "steps": steps, "gflops": flops / sec / 1e9, "frac_fp64": flops / sec / 1e12 / fp64_peak,
            "status_ok": int((st.cpu().numpy() == 0).sum())}


def pfz_flops(n):
    """Real flops of the complex Parlett-Reid elimination on the lower triangle:
    8 complex-multiply-adds (16 real flops) per trailing entry and step."""
    return float(sum(16 * (n - k - 2) * (n - k - 3) // 2 for k in range(0, n - 1, 2)))


def leg_complex_pfaffian(fp64_peak, count=2048, n=128, large_n=4096, steps=3, cpu=True):
    """Complex skew-symmetric Pfaffian (Parlett-Reid, pfaffian.jl:98-137, :193-233):
    a batch of `count` matrices n x n (C iid complex N(0, 1/n), A = (C - C^T)/2) in one
    skew_batch_logabspf_z call, inputs resident in HBM (count*n^2*16 B > L2); the same
    through host buffers (e2e); one n = large_n matrix on the cooperative grid; the
    oracle's FP64 restatement on a sample of the batch, one thread."""
    import ctypes
    import time

    import torch

    import skewgpu

    rng = np.random.default_rng(SEED + 77)
    host = np.empty((count, n, n), dtype=np.complex128)
    for b in range(count):
        C = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
        host[b] = ((C - C.T) / 2).T  # row-major storage of A^T = column-major A
    dA = torch.from_numpy(host).cuda()
    lp = torch.zeros(count, dtype=torch.float64, device="cuda")
    ph = torch.zeros(count, dtype=torch.complex128, device="cuda")
    st = torch.zeros(count, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def run():
        assert L.skew_batch_logabspf_z(h, P(dA), n, count, P(lp), P(ph), None, 1, P(st)) == 0

    for _ in range(3):
        run()
    torch.cuda.synchronize()
    sec = _time_events(run, steps, stream)
    flops = count * pfz_flops(n)
    out = {"value": count / sec, "unit": "matrices/s", "ms_per_step": sec * 1e3, "count": count, "n": n,
           "gflops": flops / sec / 1e9, "frac_fp64": flops / sec / 1e12 / fp64_peak,
           "algorithmic_flops_per_step": flops, "status_ok": int((st.cpu().numpy() == 0).sum())}
    # e2e through the host-buffer call (skew_batch_logabspf_host_z): page-locked input
    # read by the kernels, log|Pf|, cis(phase) and status in host memory on return
    pin = torch.from_numpy(host).pin_memory()
    out_lp = torch.zeros(count, dtype=torch.float64).pin_memory()
    out_ph = torch.zeros(count, dtype=torch.complex128).pin_memory()
    out_st = torch.zeros(count, dtype=torch.int32).pin_memory()

    def e2e():
        assert L.skew_batch_logabspf_host_z(h, P(pin), n, count, P(out_lp), P(out_ph), None, 1, P(out_st)) == 0

    e2e()
    torch.cuda.synchronize()
    sec_e = _time_events(e2e, steps, stream)

    def staged():
        dA.copy_(pin, non_blocking=True)
        run()
        out_lp.copy_(lp, non_blocking=True)
        out_ph.copy_(ph, non_blocking=True)

    staged()
    torch.cuda.synchronize()
    sec_s = _time_events(staged, steps, stream)
    out["e2e"] = {"value": count / sec_e, "unit": "matrices/s", "h2d_bytes_per_step": int(host.nbytes),
                  "d2h_bytes_per_step": int(count * 28), "call": "skew_batch_logabspf_host_z",
                  "staged_copies": {"value": count / sec_s, "note": "whole-batch copies around the device call"}}
    # parity of a sample against the oracle (FP64 restatement)
    if cpu:
        from oracle import oracle as O

        k = 48
        mats = [host[b].T for b in range(k)]
        t0 = time.perf_counter()
        refs = [O.pfaffian_complex(M) for M in mats]
        cpu_sec = time.perf_counter() - t0
        glp = lp[:k].cpu().numpy()
        gph = ph[:k].cpu().numpy()
        out["check"] = {"matrices": k,
                        "max_rel_logpf_vs_oracle": float(max(abs(glp[b] - refs[b][0]) / max(1.0, abs(refs[b][0]))
                                                             for b in range(k))),
                        "max_phase_diff_vs_oracle": float(max(abs(gph[b] - refs[b][1]) for b in range(k)))}
        out["cpu_baseline"] = {"value": k / cpu_sec, "unit": "matrices/s", "cores": 1, "kind": "port",
                               "sample": f"{k} of the {count} matrices, oracle FP64 restatement (full-matrix "
                                         "update as the reference), one thread"}
    # one large matrix on the cooperative grid (in place on a fresh copy per repetition)
    if large_n:
        C = (rng.standard_normal((large_n, large_n)) + 1j * rng.standard_normal((large_n, large_n))) / np.sqrt(large_n)
        src = skewgpu.to_device_complex((C - C.T) / 2)
        W = torch.empty_like(src)
        o = torch.zeros(3, dtype=torch.float64, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        times = []
        for r in range(3):
            W.copy_(src)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert L.skew_logabspf_z(h, P(W), large_n, large_n, P(o), ctypes.c_void_p(o.data_ptr() + 8), 0,
                                     P(info)) == 0
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                times.append(e0.elapsed_time(e1) / 1e3)
        sec_l = float(np.median(times))
        fl = pfz_flops(large_n)
        sign, logdet = np.linalg.slogdet(skewgpu.from_device_complex(src)) if large_n <= 4096 else (None, None)
        out[f"single_n{large_n}"] = {"ms": sec_l * 1e3, "gflops": fl / sec_l / 1e9, "frac_fp64": fl / sec_l / 1e12 / fp64_peak,
                                     "info": int(info.item()),
                                     "logpf_minus_half_logdet": None if logdet is None else float(o[0].item() - logdet / 2)}
    return out


def _time_events(fn, reps, stream):
    """Median device time (s) of fn() over reps calls, each bracketed by CUDA events."""
    import torch

    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    return float(np.median(times))


def leg_eigvals_batched(plan, d_in, offs, sizes, steps):
    """The batched workload's eigvals (hessenberg + skewtrieigvals! per matrix,
    reference order) through skew_batch_eigvals_d; the inputs stay unmodified."""
    import torch

    count = len(sizes)
    base = d_in.data_ptr()
    a_ptrs = torch.tensor((base + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    voff = np.zeros(count, dtype=np.int64)
    voff[1:] = np.cumsum(sizes[:-1])
    vals = torch.empty(int(sizes.sum()), dtype=torch.float64, device="cuda")
    v_ptrs = torch.tensor((vals.data_ptr() + 8 * voff).tolist(), dtype=torch.int64, device="cuda")
    st = torch.empty(count, dtype=torch.int32, device="cuda")
    for _ in range(3):
        plan.eigvals(a_ptrs, v_ptrs, st)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        plan.eigvals(a_ptrs, v_ptrs, st)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / steps
    s = st.cpu().numpy()
    return {"value": count / sec, "unit": "matrices/s", "ms_per_step": sec * 1e3, "steps": steps,
            "status_ok": int((s == 0).sum()), "status_fallback": int((s == 8).sum())}


def leg_plain_n512(fp64_peak, reps=5, cpu=True):
    """One real n=512 matrix, A = (B - B^T)/2 with B iid N(0,1): hessenberg,
    eigvals and logabspfaffian through the single-matrix C-ABI calls (median of
    reps, input restored outside the timed region), next to the oracle's FP64
    restatement of the reference on one host core.  eigvals returns the values in
    the reference's QR deflation order (the QR chain on one GPU thread);
    eigvals_sorted is eigvals(A, 1:n), the same values sorted by bisection."""
    import ctypes

    import torch

    import skewgpu

    n = 512
    A = dense_skew_input(n)
    pristine = skewgpu.to_device(A)
    work = torch.empty_like(pristine)
    tau = torch.empty(n - 1, dtype=torch.float64, device="cuda")
    ev = torch.empty(n - 1, dtype=torch.float64, device="cuda")
    vals = torch.empty(n, dtype=torch.float64, device="cuda")
    out2 = torch.empty(2, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    stream = torch.cuda.current_stream()
    P = lambda t, off=0: ctypes.c_void_p(t.data_ptr() + off)  # noqa: E731
    calls = {
        "hessenberg": lambda: L.skew_hessenberg_d(h, P(work), n, n, P(tau), P(ev), P(info)),
        "eigvals_sorted": lambda: L.skew_eigvals_irange_d(h, P(work), n, n, 1, n, P(vals), P(info)),
        "eigvals": lambda: L.skew_eigvals_d(h, P(work), n, n, P(vals), P(info)),
        "logabspfaffian": lambda: L.skew_logabspf_d(h, P(work), n, n, P(out2), P(out2, 8), 0, P(info)),
    }
    res = {"n": n}
    for name, fn in calls.items():
        times = []
        for r in range(reps + 1):
            work.copy_(pristine)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert fn() == 0
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
        res[f"{name}_ms"] = float(np.median(times))
    res["hessenberg_gflops"] = 4.0 / 3.0 * n ** 3 / (res["hessenberg_ms"] / 1e3) / 1e9
    if cpu:
        from oracle import oracle as O

        t0 = time.perf_counter()
        O.hessenberg(A)
        t1 = time.perf_counter()
        cv, _ = O.eigvals(A)
        t2 = time.perf_counter()
        clp, csg = O.logabspfaffian(A)
        t3 = time.perf_counter()
        res["cpu_port_ms"] = {"hessenberg": (t1 - t0) * 1e3, "eigvals": (t2 - t1) * 1e3,
                              "logabspfaffian": (t3 - t2) * 1e3, "cores": 1}
        g = out2.cpu().numpy()
        gv = vals.cpu().numpy()
        res["check"] = {"logpf_rel_vs_cpu": float(abs(g[0] - clp) / abs(clp)), "sign_equal": bool(g[1] == csg),
                        "eigvals_rel_vs_cpu_same_order": float(np.abs(gv - cv).max() / np.abs(cv).max())}
    return res


def leg_pfaffian_adjoint(fp64_peak, steps, count=1024, n=128):
    """1024 real n=128 matrices (B - B^T)/2 + 0.5 J, B iid N(0,1/n); loss
    sum_i w_i log|Pf(A_i)| with w ~ U(-1,1); forward + gradient per step through
    skew_batch_logabspf_d, gradient scaled by w on the device."""
    import torch

    import skewgpu

    buf, w_host = pfaffian_adjoint_inputs(count, n)
    w = torch.from_numpy(w_host).to("cuda")
    d_in = torch.from_numpy(buf).to("cuda")
    d_g = torch.empty_like(d_in)
    offs = np.arange(count, dtype=np.int64) * n * n
    a_ptrs = torch.tensor((d_in.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    g_ptrs = torch.tensor((d_g.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    plan = skewgpu.BatchPlan([n] * count)
    lp = torch.empty(count, dtype=torch.float64, device="cuda")
    sg = torch.empty_like(lp)
    st = torch.empty(count, dtype=torch.int32, device="cuda")
    gv = d_g.view(count, n * n)

    def step():
        plan.logabspfaffian(a_ptrs, g_ptrs, lp, sg, st)
        gv.mul_(w[:, None])
        return torch.dot(w, lp)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        loss = step()
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / steps
    flops = count * float(flops_per_matrix(n))
    plan.close()
    return {"value": count / sec, "unit": "matrices/s", "ms_per_step": sec * 1e3, "steps": steps,
            "gflops": flops / sec / 1e9, "frac_fp64": flops / sec / 1e12 / fp64_peak, "loss": float(loss.item()),
            "status_ok": int((st.cpu().numpy() == 0).sum())}


def exp_adjoint_flops(n):
    """Algorithmic FP64 work of one exp adjoint: the eigendecomposition, reduction
    4/3 n^3 and back-transformation of Vr and Vi 4 n^3; the exp assembly 4 n^3; the
    Daleckii-Krein adjoint 6 n^3 (the QR chain is O(n^2))."""
    n = np.asarray(n, dtype=np.float64)
    return (4.0 / 3.0 + 4.0 + 4.0 + 6.0) * n ** 3


def exp_adjoint_flops_executed(n):
    """FP64 work the exp adjoint executes: reduction 4/3 n^3, back-transformation of
    the real Schur basis Q 2 n^3, and the four real n x n products of the assembly
    8 n^3 (G = Q T' Q^T with T = Q^T C Q)."""
    n = np.asarray(n, dtype=np.float64)
    return (4.0 / 3.0 + 2.0 + 8.0) * n ** 3


def leg_exp_adjoint(fp64_peak, steps, count=512):
    """512 real matrices, n uniform in {32, 64, ..., 512}, each scaled to a spectral
    radius ~ U(0.5, 8); cotangents C_i iid N(0,1); G_i = d<C_i, exp(A_i)>/dA_i
    through skew_batch_exp_vjp_d."""
    import torch

    import skewgpu

    sizes, offs, buf, cot = exp_adjoint_inputs(count)
    d_in = torch.from_numpy(buf).to("cuda")
    d_c = torch.from_numpy(cot).to("cuda")
    d_g = torch.empty_like(d_in)
    ptr = lambda t: torch.tensor((t.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")  # noqa: E731
    a_ptrs, c_ptrs, g_ptrs = ptr(d_in), ptr(d_c), ptr(d_g)
    plan = skewgpu.BatchPlan(sizes)
    st = torch.empty(count, dtype=torch.int32, device="cuda")
    plan.exp_vjp(a_ptrs, c_ptrs, g_ptrs, st)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        plan.exp_vjp(a_ptrs, c_ptrs, g_ptrs, st)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / steps
    flops = float(exp_adjoint_flops(sizes).sum())
    xflops = float(exp_adjoint_flops_executed(sizes).sum())
    s = st.cpu().numpy()
    plan.close()
    return {"value": count / sec, "unit": "matrices/s", "ms_per_step": sec * 1e3, "steps": steps,
            "gflops": flops / sec / 1e9, "frac_fp64": flops / sec / 1e12 / fp64_peak,
            "algorithmic_flops": flops, "algorithmic_flops_per_matrix": "(4/3 + 4 + 4 + 6) n^3",
            "executed_flops": xflops, "frac_fp64_executed": xflops / sec / 1e12 / fp64_peak,
            "status_ok": int((s == 0).sum()), "status_fallback": int((s == 8).sum()),
            "complex_part": "reported separately as exp_adjoint_complex_64x256"}


def _launches_per_call(sizes):
    """batch_kernel launches of one batched call: one per size bucket of
    skew_batch_plan_create (tuning key bucket_edges), the buckets whose working copies
    live in global memory (above batch_smem_nmax) merged into one launch when
    batch_merge_global is set."""
    import skewgpu

    edges = skewgpu.tuning_get("bucket_edges")
    smem_nmax = skewgpu.tuning_get("batch_smem_nmax")
    merge = skewgpu.tuning_get("batch_merge_global")
    buckets = {next((e for e in edges if n <= e), 1 << 30): 0 for n in sizes}
    for n in sizes:
        e = next((e for e in edges if n <= e), 1 << 30)
        buckets[e] = max(buckets[e], int(n))
    smem = sum(1 for e, nmax in buckets.items() if nmax <= smem_nmax)
    glob = len(buckets) - smem
    return smem + (min(glob, 1) if merge else glob)


if __name__ == "__main__":
    sys.exit(main())
