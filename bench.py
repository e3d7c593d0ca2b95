#!/usr/bin/env python
"""Benchmark: MPO-MPS apply + SVD compression sweeps per second.

Workload (one step = one unit): transverse-field Ising MPO (D=3, J=1, h=0.5)
on N=64 sites, d=2, applied to a seeded random complex128 MPS with bond
chi=256 (normalised), the result compressed back to chi=256 by
``MatrixProductState.svd_compress`` (QR left sweep, truncating SVD right
sweep) -- tncontract's ``contract_mps_mpo`` + ``svd_compress``.

Arms:
  (default)          this project on the GPU.  ``value``: sweeps/s with the
                     input MPS/MPO resident in HBM; ``e2e``: the same through
                     the public API from pinned host buffers, host->device
                     copies of the inputs and the device->host read of the
                     compressed MPS inside the timed region.
  --impl reference   the reference algorithm on the host cores (the NumPy
                     restatement in oracle/, same LAPACK calls), on a bounded
                     sample of the same workload, scaled to sweeps/s by the
                     algorithmic flop ratio.

Multi-GPU (torchrun): a sweep does not shard; every rank runs its own
replica (weak scaling) and ``value`` = total sweeps / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SITES, PHYS, MPO_D, CHI = 64, 2, 3, 256
# admission stagger of the work queue (seconds between workers' first jobs):
# identical instances started together run their QR and SVD phases in
# lockstep and contend for the same resources at the same time
STAGGER = 0.02
METRIC = "MPO-MPS apply+compress sweeps/s at chi=256 (TFIM D=3, N=64, d=2, complex128)"
# dram bytes (read + write) per call of the native ops at the workload's bulk
# shape, from ncu captures of their Jacobi kernels at that shape (the matrix
# once in and once out; the working set stays in L2): the FP32 Jacobi on the
# 512 x 512 complex64 factor 2.410 MB read + 0.488 MB written, the FP64 finish
# on the 512 x 512 complex128 rows 5.191 MB + 0.435 MB, the double-float finish
# on the 512 x 512 DF rows 4.279 MB + 0.052 MB; absent = not captured.
TRAFFIC_PER_CALL = {"tnc_svd_rows": 2.898e6, "tnc_svd_rows_fp64_finish": 5.626e6, "tnc_svd_rows_df": 4.331e6}
# the bond-core finish of the mixed precision, by its arithmetic
FINISH_OP = {"df": "tnc_svd_rows_df", "fp64": "tnc_svd_rows_fp64_finish"}
# FP32 pipe: 152 SMs x 128 lanes x 2.07 GHz operations/s (x 2 for FMA flops)
FP32_OPS_T = 152 * 128 * 2.07e9 / 1e12


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nsites", type=int, default=N_SITES)
    p.add_argument("--chi", type=int, default=CHI)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batch", type=int, default=12, help="independent instances per GPU")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "fp64"])
    p.add_argument("--block-rows", type=int, default=0, choices=[0, 2, 4, 8, 16],
                   help="Jacobi half-block height of the sweep (0: the library's default, 8)")
    p.add_argument("--core", default="df", choices=["df", "fp64"],
                   help="the mixed precision's bond-core finish: double-float or FP64 arithmetic")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 engine arm")
    p.add_argument("--fp64-steps", type=int, default=1, help="timed steps of the plain FP64 engine arm")
    p.add_argument("--workload", default="tfim", choices=["tfim", "uneven", "learned"],
                   help="tfim: the headline sweep; uneven: the uneven batch of independent MPS; learned: "
                        "config 5 (XXZ D=5, N=128, chi=512, learned rank against the plain and FP64 sweeps)")
    p.add_argument("--instances", type=int, default=512, help="instances of the uneven batch")
    p.add_argument("--micro", default=None,
                   help="time one native op instead: svd:MxN:DT, qr:MxN:DT, gemm:MxNxK:DT, svdrows[H]:MxN:DT "
                        "or dffinish:MxN:DT (DT in f32,f64,c64,c128); used for kernel profiling")
    return p.parse_args()


def run_micro(args):
    """One native op at a fixed shape, timed with CUDA events (3 warm-up calls)."""
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import _ops
    op, shape, dt = args.micro.split(":")
    dims = [int(x) for x in shape.split("x")]
    npdt = {"f32": np.float32, "f64": np.float64, "c64": np.complex64, "c128": np.complex128}[dt]
    rng = np.random.default_rng(0)

    def mat(r, c):
        a = rng.standard_normal((r, c))
        if np.iscomplexobj(np.zeros(0, npdt)):
            a = a + 1j * rng.standard_normal((r, c))
        return torch.from_numpy(a.astype(npdt)).cuda()

    infos = []
    if op == "svd":
        A = mat(*dims)
        fn = lambda: _ops.svd(A, check=False, info_out=infos)
    elif op == "qr":
        A = mat(*dims)
        fn = lambda: _ops.qr(A, check=False)
    elif op in ("qrr", "qrrh"):
        A = mat(*dims)
        fn = lambda: _ops.qr_r(A, adjoint=(op == "qrrh"), check=False)
    elif op in ("gemm", "gemmtc", "gemmsimt"):
        A, B = mat(dims[0], dims[2]), mat(dims[2], dims[1])
        Cm = torch.empty((dims[0], dims[1]), dtype=A.dtype, device="cuda")
        tc = {"gemm": None, "gemmtc": True, "gemmsimt": False}[op]
        fn = lambda: _ops.gemm(0, 0, dims[0], dims[1], dims[2], A, dims[2], B, dims[1], Cm, dims[1], tc=tc)
    elif op == "dffinish":
        # the mixed sweep's bond-core finish: FP32 Jacobi rows (3e-6, sorted by
        # norm) orthogonalised in double-float to 1e-7
        A = mat(*dims)
        W32, _s, o32, _i = _ops.svd_rows(A, max_sweeps=14, tol=3e-6)
        kall = torch.tensor([dims[0]], dtype=torch.int64, device="cuda")
        rows = _ops.gather_rows(W32, o32, kall, dims[0])

        def fn():
            r = _ops.svd_rows_df(rows, tol=1e-7)
            infos.append(r[3])
            return r
    elif op.startswith("svdrows"):
        A = mat(*dims)
        h = int(op[7:]) if len(op) > 7 else None

        def fn():
            r = _ops.svd_rows(A, block_rows=h)
            infos.append(r[3])
            return r
    else:
        raise SystemExit("unknown micro op " + op)
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    _ops.PROFILE = {}
    for _ in range(max(args.steps, 1)):
        fn()
    torch.cuda.synchronize()
    summ = _ops.profile_summary(_ops.PROFILE)
    _ops.PROFILE = None
    name = {"svd": "tnc_svd", "qr": "tnc_qr", "qrr": "tnc_qr_r", "qrrh": "tnc_qr_r",
            "gemmsimt": "tnc_gemm", "gemmtc": "tnc_gemm_tc",
            "gemm": "tnc_gemm_tc" if "tnc_gemm_tc" in summ else "tnc_gemm",
            "dffinish": "tnc_svd_rows_df"}.get(op, "tnc_svd_rows")
    n, ms, fl = summ[name]
    extra = {}
    if infos:
        st, sweeps, last = (int(v) for v in infos[-1][:3].cpu())
        extra = {"status": st, "jacobi_sweeps": sweeps}
    print(json.dumps(dict({"micro": args.micro, "calls": n, "ms_per_call": ms / n,
                           "algorithmic_tflops": fl / (ms / 1e3) / 1e12}, **extra)), flush=True)
    return 0


# ------------------------------------------------------------------ clocks


class ClockSampler:
    """nvidia-smi samples (every 200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU legs


def oracle_sweep(seed, nsites, chi, discarded_fraction=None):
    """One full apply + svd_compress sweep of instance ``seed`` through the
    reference algorithm on the host cores (the NumPy restatement in oracle/,
    the reference's own LAPACK / BLAS calls, every host thread OpenBLAS
    takes).  Returns (output sites, seconds of the sweep)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import tn_oracle as O
    from tncontract_gb300 import workloads as W
    sites = W.random_mps_arrays(seed, nsites, PHYS, chi, np.complex128, normalise=True)
    mpo = W.tfim_mpo_arrays(nsites)
    t = time.perf_counter()
    out = O.apply_compress_sweep(sites, mpo, chi, discarded_fraction=discarded_fraction)
    return out, time.perf_counter() - t


def run_reference(args):
    """The reference algorithm on the machine's host cores: every step is one
    full sweep of the benchmark workload (N sites at chi, complex128), no
    sampling or scaling.  One untimed warm-up sweep (the CPU path has no
    caches to fill beyond the BLAS threads)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count()
    oracle_sweep(0, 8, 16)  # start the BLAS threads
    if args.warmup > 0:
        oracle_sweep(0, args.nsites, args.chi)
    times = [oracle_sweep(0, args.nsites, args.chi)[1] for _ in range(max(args.steps, 1))]
    total = sum(times)
    value = len(times) / total
    sample = ("%d full sweeps (apply + svd_compress, N=%d, chi=%d, complex128), one at a time, after one "
              "warm-up sweep" % (len(times), args.nsites, args.chi))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded random MPS, TFIM MPO)",
            "config": {"workload": "tfim_apply_svd_compress", "nsites": args.nsites, "phys_dim": PHYS,
                       "mpo_bond": MPO_D, "chi": args.chi, "dtype": "complex128"},
            "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def errors_vs_oracle(got_sites, log_norm, discarded, ref_sites, ref_discarded):
    """Per-output error of one instance against the FP64 oracle's result of
    the same sweep: fidelity error of the compressed states, the largest
    per-bond difference of the discarded fraction of the squared spectrum,
    and the relative error of the state norm."""
    import numpy as np
    import tn_oracle as O
    got = [np.asarray(a, dtype=np.complex128) for a in got_sites]
    f = O.fidelity(ref_sites, got)
    n_ref = O.mps_norm(ref_sites)
    n_got = O.mps_norm(got)
    if log_norm is not None:   # sites without the norm folded in
        n_got = float(np.exp(log_norm))
    dw = max(abs(a - b) for a, b in zip(discarded, ref_discarded)) if discarded else None
    return {"fidelity_error": 1.0 - f, "discarded_weight_max_abs_error": dw,
            "discarded_weight_max": max(ref_discarded) if ref_discarded else None,
            "norm_rel_error": abs(n_got - n_ref) / n_ref, "norm": n_got, "norm_oracle": n_ref}


# ------------------------------------------------------------------ GPU leg


def run_ours(args):
    import ctypes
    import numpy as np
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import _lib
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W

    N, chi, B = args.nsites, args.chi, args.batch
    warm = max(args.warmup, 3)
    core = args.core if args.precision == "mixed" else None
    E.MIXED_CORE = args.core
    # instance b of rank r uses seed (r * B + b); every instance is a full
    # workload; the caller's data is complex128 on the host
    host_batch = [W.random_mps_arrays(rank * B + b, N, PHYS, chi, np.complex128, normalise=True)
                  for b in range(B)]
    host_mpo = W.tfim_mpo_arrays(N)
    streams = [torch.cuda.Stream() for _ in range(B)]

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    # ---- value: inputs resident in HBM (balanced and cast before timing)
    dt = E.compute_dtype(args.precision, True)
    balanced = [E.balance(sites) for sites in host_batch]
    log_norms = [ln for _, ln in balanced]
    dev_batch = [E.to_sites(sites, dt) for sites, _ in balanced]
    dev_mpo = E.to_sites(host_mpo, dt)
    last = [None] * B
    last_stats = [None] * B
    OPS = ("tnc_qr", "tnc_qr_r", "tnc_svd_rows", FINISH_OP[args.core])

    def sweep_job(b, prof=None, precision_core=core, batch=dev_batch, mpo=dev_mpo, out=last, stats=last_stats):
        def job():
            st = E.SweepStats()
            out[b] = E.apply_compress_native(batch[b], mpo, chi, log_norm_in=log_norms[b], profile=prof,
                                             stats=st, core=precision_core, block_rows=args.block_rows)
            stats[b] = st
        return job

    def run_steps(k, profs=None, **kw):
        jobs = [sweep_job(b, profs[j * B + b] if profs else None, **kw) for j in range(k) for b in range(B)]
        E.run_queue(jobs, B, streams=streams, stagger=STAGGER)

    run_steps(warm)
    barrier()
    launches0 = _lib.kernel_launches()
    st = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(st)
        run_steps(args.steps)
        ev1.record(st)
        barrier()
    launches = _lib.kernel_launches() - launches0
    elapsed = ev0.elapsed_time(ev1) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * B * args.steps / elapsed
    out_sites = [[a.cpu().numpy() for a in o] for o in last]
    out_stats = list(last_stats)

    # per-op durations: one more step in which every sweep brackets its QR,
    # R-only QR, Jacobi and FP64 finish calls by CUDA events on its
    # instance's stream (timing events recorded on many concurrent streams
    # slow the batch down, so the timed region above runs without them)
    profs = [(ctypes.c_double * 12)() for _ in range(B)]
    run_steps(1, profs)
    barrier()
    timed = {op: (sum(p[3 * o + 1] for p in profs), sum(p[3 * o] for p in profs), sum(p[3 * o + 2] for p in profs))
             for o, op in enumerate(OPS)}
    timed = {k: v for k, v in timed.items() if v[0] > 0}
    dom_name = max(timed.items(), key=lambda kv: kv[1][1])[0]

    # ---- e2e: through the public host-array API (engine.apply_compress_host):
    # the caller's pinned complex128 arrays in, complex128 host arrays out;
    # the host->device copy, balancing and casting on the device, the sweep,
    # the cast back and the device->host copy are inside the timed region
    pinned_batch = [[torch.from_numpy(a).pin_memory() for a in sites] for sites in host_batch]
    pinned_mpo = [torch.from_numpy(w).pin_memory() for w in host_mpo]
    h2d = sum(a.numel() * a.element_size() for sites in pinned_batch for a in sites) + \
        B * sum(w.numel() * w.element_size() for w in pinned_mpo)
    e2e_last = [None] * B

    def e2e_job(b):
        def job():
            e2e_last[b] = E.apply_compress_host(pinned_batch[b], pinned_mpo, chi, precision=args.precision)
        return job

    E.run_queue([e2e_job(b) for b in range(B)], B, streams=streams, stagger=STAGGER)
    barrier()
    t0 = time.perf_counter()
    E.run_queue([e2e_job(b) for _ in range(args.steps) for b in range(B)], B, streams=streams, stagger=STAGGER)
    barrier()
    e2e_el = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_el], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_el = float(t.item())
    d2h = sum(a.nbytes for r in e2e_last for a in r)  # per step: B instances' results
    e2e_value = world * B * args.steps / e2e_el

    # ---- the same sweep with the FP32 Jacobi alone on the bond cores (no FP64
    # finish): the speed the FP64 core costs, and its accuracy
    extra = {}
    fp32_sites, fp32_stats = None, None
    if args.precision == "mixed" and not args.no_plain:
        last32, stats32 = [None] * B, [None] * B
        kw32 = dict(precision_core=None, out=last32, stats=stats32)
        run_steps(1, **kw32)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(st)
        run_steps(1, **kw32)
        e1.record(st)
        barrier()
        t32 = e0.elapsed_time(e1) / 1e3
        if world > 1:
            t = torch.tensor([t32], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            t32 = float(t.item())
        extra["fp32_core"] = {"value": world * B / t32, "unit": "sweeps/s", "steps": 1, "warmup": 1,
                              "path": "the same native sweep with the FP32 Jacobi alone on every bond core"}
        fp32_sites = [a.cpu().numpy() for a in last32[0]]
        fp32_stats = stats32[0]

    # ---- the plain FP64 method of this project: the same native sweep and
    # work queue in complex128 end to end (QR, Jacobi, products, decision)
    fp64_sites, fp64_stats = None, None
    if not args.no_plain:
        dt64 = torch.complex128
        batch64 = [E.to_sites(sites, dt64) for sites, _ in balanced]
        mpo64 = E.to_sites(host_mpo, dt64)
        last64, stats64 = [None] * B, [None] * B
        kw = dict(precision_core=None, batch=batch64, mpo=mpo64, out=last64, stats=stats64)
        run_steps(1, **kw)   # warm-up (workspaces, first launches)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(st)
        run_steps(args.fp64_steps, **kw)
        e1.record(st)
        barrier()
        t64 = e0.elapsed_time(e1) / 1e3
        if world > 1:
            t = torch.tensor([t64], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            t64 = float(t.item())
        v64 = world * B * args.fp64_steps / t64
        fp64_sites = [a.cpu().numpy() for a in last64[0]]
        fp64_stats = stats64[0]
        extra["plain_fp64"] = {"value": v64, "unit": "sweeps/s", "steps": args.fp64_steps, "warmup": 1,
                               "path": "the same native sweep and %d-stream work queue in complex128 (FP64 QR, "
                                       "Jacobi, products and truncation decision)" % B}
        extra["speedup_vs_plain_fp64"] = value / v64
        del batch64, mpo64, last64

    name = dom_name
    ncalls, ms, flops = timed[name]
    ncalls = int(ncalls)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["bf16_tflops"]), "measured"
    except Exception:
        peak, peak_src = 1900.0, "fallback"
    achieved = flops / (ms / 1e3) / 1e12 if ms > 0 else 0.0
    fp64_op = name.endswith("fp64_finish")
    df_op = name == FINISH_OP["df"]
    if df_op:
        pipe = ("FP32 (double-float operations)", round(FP32_OPS_T, 1))
        fp_note = ("CUDA-core arithmetic; achieved counts the FP32 operations the double-float Jacobi executed "
                   "(44 n^2 L per rotating sweep and 24 n^2 L for the checking one: 12 per Dot2 step, 7 per "
                   "compensated update), frac is against the measured bf16 tensor peak, frac_of_pipe_nominal "
                   "against the FP32 pipe's operation rate (152 SMs x 128 lanes x 2.07 GHz = %.1f T ops/s)"
                   % FP32_OPS_T)
    else:
        pipe = ("FP64", 1.25) if fp64_op else ("FP32", 80.5)
        fp_note = ("CUDA-core arithmetic (Jacobi rotations, Householder); frac is against the measured bf16 "
                   "tensor peak, frac_of_pipe_nominal against GB300's nominal %s CUDA-core rate (%s TFLOP/s%s); "
                   "flops are %s" % (pipe[0], pipe[1], "" if fp64_op else ": 152 SMs x 128 FMA x 2 x 2.07 GHz",
                                     "the FP64 Jacobi's executed flops (14 n^2 L per rotating sweep, 4 n^2 L for "
                                     "the checking one)" if fp64_op else "the op's fixed algorithmic count"))
    roofline = {"bound": "tensor", "kernel": name, "launches": ncalls, "achieved": achieved,
                "measured": "CUDA events around every %s call, recorded by the native sweep on its instance's "
                            "stream in one profiled step of the same workload after the timed region (%d streams "
                            "run concurrently, so durations include time shared with other instances)" % (name, B),
                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": peak_src,
                "traffic": TRAFFIC_PER_CALL.get(name), "pipe": pipe[0], "pipe_nominal_tflops": pipe[1],
                "frac_of_pipe_nominal": achieved / pipe[1], "note": fp_note}
    tot_ms = sum(x[1] for x in timed.values())
    share = {k: round(v[1] / tot_ms, 4) for k, v in timed.items() if tot_ms > 0}
    dtype_name = {"mixed": "c64+%score" % {"df": "df", "fp64": "f64"}[args.core], "fp32": "c64",
                  "fp64": "c128"}[args.precision]
    path = {"mixed": "engine (mixed: complex64 sites and FP32 products and QR, FP32 Jacobi finished by a %s "
                     "Jacobi on every bond core, truncation decided on its singular values)"
                     % {"df": "double-float (FP32-pipe, ~48-bit)", "fp64": "FP64"}[args.core],
            "fp32": "engine (fp32)", "fp64": "engine (fp64)"}[args.precision]
    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": elapsed / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype_name, "data": "synthetic (seeded random MPS, TFIM MPO)",
            "config": {"workload": "tfim_apply_svd_compress", "path": path, "precision": args.precision,
                       "batch_per_gpu": B, "nsites": N, "phys_dim": PHYS, "mpo_bond": MPO_D, "chi": chi,
                       "block_rows": args.block_rows or 8,
                       "input_dtype": "complex128", "parallelism": "replicas" if world > 1 else "single",
                       "scheduling": "K steps x %d sweeps as one work queue on %d CUDA streams (continuous "
                                     "batching), workers admitted %d ms apart, each sweep one native call"
                                     % (B, B, int(STAGGER * 1e3)),
                       "l2": "inputs larger than L2 (%d MPS of 67 MB complex64 on the device, 0.6 GB applied "
                             "each)" % B},
            "e2e": {"value": e2e_value, "unit": "sweeps/s", "h2d_bytes_per_step": h2d // 1,
                    "d2h_bytes_per_step": d2h,
                    "path": "engine.apply_compress_host: pinned complex128 host arrays -> device, balance and "
                            "cast on the device, native sweep, complex128 host arrays back"},
            "gpu_launches": launches,
            "roofline": roofline,
            "stage_share": share,
            "clocks": clk.summary(),
            "sweep_tflop": W.sweep_flops(N, PHYS, MPO_D, chi)["total"] / 1e12}
    line.update(extra)
    if rank == 0 and not args.no_cpu_baseline:
        # the FP64 oracle on instance 0 (seed 0): timed as the CPU baseline,
        # and the reference result every output of the GPU paths is checked
        # against
        ref_df = []
        ref, t_cpu = oracle_sweep(0, N, chi, discarded_fraction=ref_df)
        line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": "one full sweep (N=%d, chi=%d, complex128) of instance 0" % (N, chi)}
        st0 = out_stats[0]
        errs = {args.precision: errors_vs_oracle(out_sites[0], None if st0.norm_folded else st0.log_norm,
                                                 st0.discarded, ref, ref_df)}
        errs[args.precision]["bond_dims_match"] = [1] + list(st0.bonds) + [1] == \
            [1] + [a.shape[2] for a in ref[:-1]] + [1]
        if fp32_sites is not None:
            errs["fp32_core"] = errors_vs_oracle(fp32_sites, None if fp32_stats.norm_folded else fp32_stats.log_norm,
                                                 fp32_stats.discarded, ref, ref_df)
            errs["fp32_core"]["bond_dims_match"] = list(fp32_stats.bonds) == [a.shape[2] for a in ref[:-1]]
        if fp64_sites is not None:
            errs["fp64"] = errors_vs_oracle(fp64_sites, None if fp64_stats.norm_folded else fp64_stats.log_norm,
                                            fp64_stats.discarded, ref, ref_df)
            errs["fp64"]["bond_dims_match"] = list(fp64_stats.bonds) == [a.shape[2] for a in ref[:-1]]
        e2e0 = e2e_last[0]
        errs["e2e_" + args.precision] = {"fidelity_error": 1.0 - __import__("tn_oracle").fidelity(ref, e2e0)}
        line["errors_vs_fp64_oracle"] = errs
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_uneven(args):
    """The uneven batch: ``--instances`` independent random MPS (seed 1: N in
    [16, 128], d in {2, 3, 4}, chi in [16, 256], float32 / complex64
    alternating, ``workloads.config3_specs``), each left-canonised, svd-
    compressed to chi // 2 (QR sweep + truncating SVD sweep, one native call
    with an identity MPO) and its norm evaluated.  Under torchrun every rank
    runs its flop-balanced share (``workloads.run_sharded``: the same split
    on every rank, no data exchanged), the time is the max over ranks, and
    the per-instance scalars (log norm, bonds) are gathered to rank 0.
    Inputs are generated on the device from per-instance seeds (Gaussian
    entries, each site scaled to unit expected norm) before the timed region;
    the jobs run heaviest first on a work queue of ``--batch`` streams.  A
    sample of instances is checked against the oracle on the rank that ran
    it (fidelity error) and timed on rank 0's host cores as the CPU baseline,
    scaled to the whole batch by the flop ratio."""
    import numpy as np
    import torch
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import _ops
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    specs = W.config3_specs(1, args.instances)
    mine = set(W.partition_by_flops(specs, world)[rank])
    tdt = {np.float32: torch.float32, np.complex64: torch.complex64}
    inputs, idents = {}, {}
    for i in sorted(mine):
        N, d, chi, dt, seed = specs[i]
        td = tdt[dt]
        bonds = [1] + [chi] * (N - 1) + [1]
        sites = []
        for j in range(N):
            a = _ops.fill_gaussian((d, bonds[j], bonds[j + 1]), td, seed * 1000 + j)
            n = a.numel() * (2 if td == torch.complex64 else 1)
            sites.append(_ops.scale(a, 1.0 / np.sqrt(n)))
        inputs[i] = sites
        if (d, td) not in idents:
            idents[(d, td)] = _ops.to_device(np.eye(d).reshape(d, d, 1, 1), td)
    torch.cuda.synchronize()
    small = sorted(range(len(specs)), key=lambda i: W.spec_flops(specs[i]))
    sample = set(small[:6] + small[len(small) // 4: len(small) // 4 + 2])
    outputs = {}

    def make_job(i):
        def f():
            N, d, chi, dt, _ = specs[i]
            st = E.SweepStats()
            out = E.apply_compress_native(inputs[i], [idents[(d, tdt[dt])]] * N, chi // 2, stats=st)
            if i in sample:
                outputs[i] = out
            return {"log_norm": st.log_norm, "bonds": list(st.bonds)}
        return f

    B = args.batch
    streams = [torch.cuda.Stream() for _ in range(B)]

    def run_jobs(jobs):
        return E.run_queue(jobs, B, streams=streams, stagger=STAGGER)

    warm = sorted(mine, key=lambda i: -W.spec_flops(specs[i]))[:B]
    run_jobs([make_job(i) for i in warm])   # warm-up
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e0.record()
        local = W.run_sharded(specs, make_job, run_jobs, rank, world)
        e1.record()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    # parity on the sample instances this rank ran
    import tn_oracle as O
    fid_err, cpu_s, checked = 0.0, 0.0, 0
    for i in sorted(sample & mine):
        N, d, chi, dt, _ = specs[i]
        host = [a.cpu().numpy().astype(np.complex128 if dt == np.complex64 else np.float64) for a in inputs[i]]
        t0 = time.perf_counter()
        ref = O.svd_compress_method(O.left_canonical_form_mps(host), chi // 2)
        cpu_s += time.perf_counter() - t0
        got = [o.cpu().numpy().astype(np.complex128) for o in outputs[i]]
        fid_err = max(fid_err, 1 - O.fidelity(ref, got))
        checked += 1
    merged = W.gather_results(local, world)
    if world > 1:
        stats = [None] * world if rank == 0 else None
        dist.gather_object((fid_err, cpu_s, checked), stats, dst=0)
        if rank == 0:
            fid_err = max(s[0] for s in stats)
            checked = sum(s[2] for s in stats)
    if rank == 0:
        assert merged is not None and sorted(merged) == list(range(len(specs)))
        ratio_local = sum(W.spec_flops(specs[i]) for i in sample & mine) / sum(W.spec_flops(sp) for sp in specs)
        cpu_rate = len(specs) * ratio_local / cpu_s if cpu_s > 0 else None
        line = {"metric": "uneven-batch instances/s (left-canonise + svd_compress to chi/2 + norm; N 16-128, "
                          "d 2-4, chi 16-256)",
                "value": len(specs) / elapsed, "unit": "instances/s", "n_gpus": world, "steps": 1, "warmup": 1,
                "ms_per_step": elapsed * 1e3, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f32/c64", "data": "synthetic (seeded Gaussian MPS generated on the "
                                                                  "device)",
                "config": {"workload": "uneven_batch", "instances": len(specs), "seed": 1, "streams": B,
                           "parallelism": "flop-partitioned instances over %d rank(s), per-instance scalars "
                                          "gathered to rank 0" % world,
                           "scheduling": "heaviest first on a work queue, workers admitted %d ms apart"
                                         % int(STAGGER * 1e3)},
                "instances_gathered": len(merged),
                "fidelity_error_max_vs_oracle": fid_err, "oracle_sample": checked,
                "clocks": clk.summary(),
                "cpu_baseline": {"value": cpu_rate, "unit": "instances/s", "cores": os.cpu_count(),
                                 "kind": "port",
                                 "sample": "rank 0's instances of the oracle sample through the oracle "
                                           "(left_canonical_form + svd_compress), scaled by their flop share %.4f"
                                           % ratio_local}}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_learned(args):
    """Config 5, learned-rank truncation at full size: a random float32 MPS
    (N=128, d=2, chi=512, seed 5) under the Heisenberg XXZ MPO (Delta=0.8,
    D=5), compressed with the discarded-weight rule (tolerance 1e-8, at most
    chi).  The rank predictor is first trained on the GPU by the library's
    own MLP kernels on spectra of plain sweeps of configs 1-3
    (``learned.train_rank_model``); then the sweep runs without it (full SVD
    at every bond) and with it (randomized SVD sized by the prediction,
    oversampling 16, 2 power iterations, the full SVD as fallback when the
    sketch fails its residual check), and once in FP64 as the reference both
    are compared with.  One step =
    one sweep; sweeps/s with and without the predictor, the fallback rate and
    the fidelity errors are reported."""
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import learned as LR
    from tncontract_gb300 import workloads as W
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    E.MIXED_CORE = args.core
    N, chi, tol = args.nsites, args.chi, 1e-8
    t0 = time.perf_counter()
    model, hist, ntrain = LR.train_rank_model(tol)
    t_train = time.perf_counter() - t0
    sites, mpo = LR.config5_inputs(N, 2, chi)
    LR.config5(sites[:8], mpo[:8], min(chi, 64), tol)          # warm-up (first launches)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        plain, t_plain, rs_plain, st_plain = LR.config5(sites, mpo, chi, tol)
        learn, t_learn, rs_learn, st_learn = LR.config5(sites, mpo, chi, tol, model=model)
    f32, t_f32, _rs32, _st32 = LR.config5(sites, mpo, chi, tol, precision="fp32")
    ref, t_ref, _rs, st_ref = LR.config5(sites, mpo, chi, tol, precision="fp64")

    def fid(a, b):
        return 1.0 - E.fidelity([x.to(torch.float64) for x in a], [x.to(torch.float64) for x in b])
    bonds = lambda P: [int(a.shape[2]) for a in P[:-1]]  # noqa: E731
    flops = W.sweep_flops(N, 2, 5, chi, complex_=False)["total"]
    line = {"metric": "config 5 learned-rank apply+compress sweeps/s (XXZ D=5, N=%d, chi=%d, float32, "
                      "discarded weight <= 1e-8)" % (N, chi),
            "value": 1.0 / t_learn, "unit": "sweeps/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": t_learn * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+%score" % {"df": "df", "fp64": "f64"}[E.MIXED_CORE],
            "data": "synthetic (seeded random MPS, XXZ MPO)",
            "config": {"workload": "config5_learned_rank", "nsites": N, "phys_dim": 2, "mpo_bond": 5, "chi": chi,
                       "dw_tol": tol, "oversample": 16, "power_iters": 2,
                       "timing": "one sweep each, host wall clock around a synchronised sweep"},
            "precision": "mixed (float32 sites and products, %s Jacobi finish of every bond core)"
                         % {"df": "double-float", "fp64": "FP64"}[E.MIXED_CORE],
            "plain_sweeps_per_s": 1.0 / t_plain, "fp64_sweeps_per_s": 1.0 / t_ref,
            "fp32_core_sweeps_per_s": 1.0 / t_f32, "fidelity_error_fp32_core_vs_fp64": fid(f32, ref),
            "speedup_learned_vs_plain": t_plain / t_learn,
            "fallback_rate": LR.fallback_rate(rs_learn), "bonds_sketched": rs_learn.sketched,
            "bonds_fallback": rs_learn.fallbacks, "bonds_full_svd": rs_learn.full,
            "bonds_declined_cap_bound": rs_learn.declined,
            "rows_factored_learned_over_plain": rs_learn.rows_factored / max(rs_plain.rows_factored, 1),
            "fidelity_error_plain_vs_fp64": fid(plain, ref), "fidelity_error_learned_vs_fp64": fid(learn, ref),
            "bond_dims_match_fp64": {"plain": bonds(plain) == bonds(ref), "learned": bonds(learn) == bonds(ref)},
            "training": {"bonds": ntrain, "loss_first": hist[0], "loss_last": hist[-1], "seconds": t_train},
            "sweep_tflop_fixed_count": flops / 1e12,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.micro:
        return run_micro(args)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.workload == "learned":
        if args.nsites == N_SITES and args.chi == CHI:
            args.nsites, args.chi = 128, 512
        return run_learned(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
