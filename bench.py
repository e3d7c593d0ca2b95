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
# dram bytes (read + write) per call of the dominant native op at the
# workload's bulk shape (the Jacobi kernel of tnc_svd_rows on the 512 x 512
# complex64 triangular factor: 2.412 MB read + 0.470 MB written), from an
# ncu capture of that kernel at that shape; absent = not captured.
TRAFFIC_PER_CALL = {"tnc_svd_rows": 2.882e6}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nsites", type=int, default=N_SITES)
    p.add_argument("--chi", type=int, default=CHI)
    p.add_argument("--cpu-sample-sites", type=int, default=28)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batch", type=int, default=12, help="independent instances per GPU")
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 drop-in comparison")
    p.add_argument("--workload", default="tfim", choices=["tfim", "uneven"],
                   help="tfim: the headline sweep; uneven: the uneven batch of independent MPS")
    p.add_argument("--instances", type=int, default=512, help="instances of the uneven batch")
    p.add_argument("--micro", default=None,
                   help="time one native op instead: svd:MxN:DT, qr:MxN:DT or gemm:MxNxK:DT "
                        "(DT in f32,f64,c64,c128); used for kernel profiling")
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
            "gemm": "tnc_gemm_tc" if "tnc_gemm_tc" in summ else "tnc_gemm"}.get(op, "tnc_svd_rows")
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


def cpu_sample(nsites, chi, steps=1, target=N_SITES):
    """Reference algorithm (oracle restatement, NumPy/LAPACK) on N=nsites at
    the full bond dimension; returns (seconds per sample, the flop ratio of
    the sample to a sweep of ``target`` sites)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import tn_oracle as O
    from tncontract_gb300 import workloads as W
    sites = O.random_mps(0, nsites, PHYS, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(nsites)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        O.apply_compress_sweep(sites, mpo, chi)
        times.append(time.perf_counter() - t)
    ratio = W.sweep_flops(nsites, PHYS, MPO_D, chi)["total"] / W.sweep_flops(target, PHYS, MPO_D, chi)["total"]
    return times, ratio


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count()
    cpu_sample(8, 16)  # warm the BLAS threads
    w = max(args.warmup, 0)
    if w:
        cpu_sample(args.cpu_sample_sites, args.chi, steps=1, target=args.nsites)
    times, ratio = cpu_sample(args.cpu_sample_sites, args.chi, steps=max(args.steps, 1), target=args.nsites)
    per_sweep = statistics.median(times) / ratio
    value = 1.0 / per_sweep
    sample = ("apply+svd_compress on N=%d sites at chi=%d (same d, D, dtype), scaled by the "
              "algorithmic flop ratio %.4f to N=%d" % (args.cpu_sample_sites, args.chi, ratio, args.nsites))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sweep * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded random MPS, TFIM MPO)",
            "config": {"workload": "tfim_apply_svd_compress", "nsites": args.nsites, "phys_dim": PHYS,
                       "mpo_bond": MPO_D, "chi": args.chi, "dtype": "complex128"},
            "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU leg


def run_ours(args):
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
    import tncontract_gb300 as tn
    from tncontract_gb300 import _lib, _ops
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W

    N, chi, B = args.nsites, args.chi, args.batch
    warm = max(args.warmup, 3)
    # instance b of rank r uses seed (r * B + b); every instance is a full workload
    host_batch = [W.random_mps_arrays(rank * B + b, N, PHYS, chi, np.complex128, normalise=True)
                  for b in range(B)]
    host_mpo = W.tfim_mpo_arrays(N)
    dt = E.compute_dtype(args.precision, True)
    np_dt = np.complex64 if dt == torch.complex64 else np.complex128
    # FP32 storage needs balanced sites (see engine.balance); the log norms
    # travel with the host buffers
    balanced = [E.balance(sites) for sites in host_batch]
    log_norms = [ln for _, ln in balanced]
    pinned_batch = [[torch.from_numpy(a.astype(np_dt)).pin_memory() for a in sites] for sites, _ in balanced]
    pinned_mpo = [torch.from_numpy(w.astype(np_dt)).pin_memory() for w in host_mpo]
    # e2e bytes per step: every sweep job copies its instance's sites and the MPO
    h2d = sum(a.numel() * a.element_size() for sites in pinned_batch for a in sites) + \
        B * sum(w.numel() * w.element_size() for w in pinned_mpo)

    dev_batch = [E.to_sites(sites, dt) for sites in pinned_batch]
    dev_mpo = E.to_sites(pinned_mpo, dt)
    streams = [torch.cuda.Stream() for _ in range(B)]

    # the timed work: K steps of B sweeps as one queue of K*B jobs on B
    # streams (continuous batching: an instance that finishes its sweep takes
    # the next one), each sweep one native call (tnc_sweep_apply_compress)
    import ctypes
    last = [None] * B
    OPS = ("tnc_qr", "tnc_qr_r", "tnc_svd_rows")

    def sweep_job(b, prof=None):
        def job():
            last[b] = E.apply_compress_native(dev_batch[b], dev_mpo, chi, log_norm_in=log_norms[b], profile=prof)
        return job

    def run_steps(k, profs=None):
        jobs = [sweep_job(b, profs[j * B + b] if profs else None) for j in range(k) for b in range(B)]
        E.run_queue(jobs, B, streams=streams, stagger=STAGGER)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

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
    out = last
    launches = _lib.kernel_launches() - launches0
    elapsed = ev0.elapsed_time(ev1) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * B * args.steps / elapsed
    # per-op durations: one more step of the same workload in which every
    # sweep brackets its QR, R-only QR and Jacobi calls by CUDA events on its
    # instance's stream (timing events recorded on many concurrent streams
    # slow the batch down, so the timed region above runs without them)
    profs = [(ctypes.c_double * 9)() for _ in range(B)]
    run_steps(1, profs)
    barrier()
    timed = {op: (sum(p[3 * o + 1] for p in profs), sum(p[3 * o] for p in profs), sum(p[3 * o + 2] for p in profs))
             for o, op in enumerate(OPS)}
    dom_name = max(timed.items(), key=lambda kv: kv[1][1])[0]

    # end to end through the public API: pinned host arrays in, host arrays
    # out, every sweep job copying its own inputs and results
    e2e_last = [None] * B

    def e2e_job(b):
        def job():
            sites = E.to_sites(pinned_batch[b], dt)
            mpo = E.to_sites(pinned_mpo, dt)
            r = E.apply_compress_native(sites, mpo, chi, log_norm_in=log_norms[b])
            e2e_last[b] = [t.cpu().numpy() for t in r]
        return job

    E.run_queue([e2e_job(b) for b in range(B)], B, streams=streams, stagger=STAGGER)
    barrier()
    t0 = time.perf_counter()
    E.run_queue([e2e_job(b) for _ in range(args.steps) for b in range(B)], B, streams=streams, stagger=STAGGER)
    barrier()
    e2e_el = time.perf_counter() - t0
    res = e2e_last
    if world > 1:
        t = torch.tensor([e2e_el], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_el = float(t.item())
    d2h = sum(a.nbytes for r in res for a in r)  # per step: B instances' results
    e2e_value = world * B * args.steps / e2e_el

    # plain FP64 drop-in path (this project's straightforward FP64 method) on
    # instance 0, and the fidelity error of the measured path against it
    extra = {}
    if rank == 0 and not args.no_plain:
        psi = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in host_batch[0]])
        mpo = tn.onedim.MatrixProductOperator([tn.Tensor(w, ["physout", "physin", "left", "right"])
                                               for w in host_mpo])

        def plain():
            phi = tn.onedim.contract_mps_mpo(psi, mpo)
            phi.svd_compress(chi=chi)
            return phi

        plain()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref = plain()
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        ref_sites = []
        for t in ref:
            lab = t.labels
            ref_sites.append(_ops.permute(t.data, [lab.index(ref.phys_label), lab.index(ref.left_label),
                                                   lab.index(ref.right_label)]))
        fid = E.fidelity(ref_sites, [_ops.cast(x, torch.complex128) for x in out[0]])
        extra = {"plain_fp64_sweeps_per_s": 1.0 / t_plain,
                 "speedup_vs_plain_fp64": value / (1.0 / t_plain),
                 "fidelity_error_vs_plain_fp64": 1.0 - fid}

    name = dom_name
    ncalls, ms, flops = timed[name]
    ncalls = int(ncalls)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["bf16_tflops"]), "measured"
    except Exception:
        peak, peak_src = 1900.0, "fallback"
    achieved = flops / (ms / 1e3) / 1e12 if ms > 0 else 0.0
    fp_note = ("FP32 CUDA-core arithmetic (Jacobi rotations, Householder); frac is against the "
               "measured bf16 tensor peak, frac_of_fp32_nominal against GB300's nominal FP32 rate "
               "(152 SMs x 128 FMA x 2 x 2.07 GHz = 80.5 TFLOP/s)")
    roofline = {"bound": "tensor", "kernel": name, "launches": ncalls, "achieved": achieved,
                "measured": "CUDA events around every %s call, recorded by the native sweep on its instance's "
                            "stream in one profiled step of the same workload after the timed region (%d streams "
                            "run concurrently, so durations include time shared with other instances)" % (name, B),
                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": peak_src,
                "traffic": TRAFFIC_PER_CALL.get(name), "fp32_nominal_tflops": 80.5,
                "frac_of_fp32_nominal": achieved / 80.5, "note": fp_note}
    tot_ms = sum(x[1] for x in timed.values())
    # of the three factorisation stages' event time in the timed region
    share = {k: round(v[1] / tot_ms, 4) for k, v in timed.items() if tot_ms > 0}

    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": elapsed / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64" if dt == torch.complex64 else "c128",
            "data": "synthetic (seeded random MPS, TFIM MPO)",
            "config": {"workload": "tfim_apply_svd_compress", "path": "engine (%s)" % args.precision,
                       "batch_per_gpu": B, "nsites": N, "phys_dim": PHYS, "mpo_bond": MPO_D, "chi": chi,
                       "input_dtype": "complex128", "parallelism": "replicas" if world > 1 else "single",
                       "scheduling": "K steps x %d sweeps as one work queue on %d CUDA streams (continuous "
                                     "batching), workers admitted %d ms apart, each sweep one native call"
                                     % (B, B, int(STAGGER * 1e3)),
                       "l2": "inputs larger than L2 (%d MPS of 67 MB complex64 on the device, 0.6 GB applied "
                             "each)" % B},
            "e2e": {"value": e2e_value, "unit": "sweeps/s", "h2d_bytes_per_step": h2d // 1,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roofline,
            "stage_share": share,
            "clocks": clk.summary(),
            "sweep_tflop": W.sweep_flops(N, PHYS, MPO_D, chi)["total"] / 1e12}
    line.update(extra)
    if rank == 0 and not args.no_cpu_baseline:
        times, ratio = cpu_sample(args.cpu_sample_sites, chi, steps=1, target=N)
        v = ratio / times[0]
        line["cpu_baseline"] = {"value": v, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": "apply+svd_compress on N=%d sites at chi=%d, scaled by the "
                                          "algorithmic flop ratio %.4f to N=%d" % (
                                              args.cpu_sample_sites, chi, ratio, N)}
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
    with an identity MPO) and its norm evaluated.  Inputs are generated on
    the device from per-instance seeds (Gaussian entries, each site scaled to
    unit expected norm) before the timed region; the jobs run heaviest first
    on a work queue of ``--batch`` streams.  A sample of instances is checked
    against the oracle (fidelity error) and timed on the host cores as the
    CPU baseline, scaled to the whole batch by the flop ratio."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__
    __graft_entry__.build()
    from tncontract_gb300 import _ops
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    specs = W.config3_specs(1, args.instances)
    tdt = {np.float32: torch.float32, np.complex64: torch.complex64}
    inputs, idents = [], {}
    for (N, d, chi, dt, seed) in specs:
        td = tdt[dt]
        bonds = [1] + [chi] * (N - 1) + [1]
        sites = []
        for i in range(N):
            a = _ops.fill_gaussian((d, bonds[i], bonds[i + 1]), td, seed * 1000 + i)
            n = a.numel() * (2 if td == torch.complex64 else 1)
            sites.append(_ops.scale(a, 1.0 / np.sqrt(n)))
        inputs.append(sites)
        if (d, td) not in idents:
            idents[(d, td)] = _ops.to_device(np.eye(d).reshape(d, d, 1, 1), td)
    torch.cuda.synchronize()
    order = sorted(range(len(specs)), key=lambda i: -W.spec_flops(specs[i]))
    results = [None] * len(specs)

    def job(i):
        def f():
            N, d, chi, dt, _ = specs[i]
            st = E.SweepStats()
            out = E.apply_compress_native(inputs[i], [idents[(d, tdt[dt])]] * N, chi // 2, stats=st)
            results[i] = (st.log_norm, st.bonds, out if i in sample else None)
        return f

    small = sorted(range(len(specs)), key=lambda i: W.spec_flops(specs[i]))
    sample = set(small[:6] + small[len(small) // 4: len(small) // 4 + 2])
    B = args.batch
    streams = [torch.cuda.Stream() for _ in range(B)]
    E.run_queue([job(i) for i in order[:B]], B, streams=streams, stagger=STAGGER)   # warm-up
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        torch.cuda.synchronize()
        e0.record()
        E.run_queue([job(i) for i in order], B, streams=streams, stagger=STAGGER)
        e1.record()
        torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1) / 1e3
    # parity and CPU baseline on the sample
    import tn_oracle as O
    fid_err, cpu_s = 0.0, 0.0
    for i in sorted(sample):
        N, d, chi, dt, _ = specs[i]
        host = [a.cpu().numpy().astype(np.complex128 if dt == np.complex64 else np.float64) for a in inputs[i]]
        t0 = time.perf_counter()
        ref = O.svd_compress_method(O.left_canonical_form_mps(host), chi // 2)
        cpu_s += time.perf_counter() - t0
        got = [o.cpu().numpy().astype(np.complex128) for o in results[i][2]]
        fid_err = max(fid_err, 1 - O.fidelity(ref, got))
    ratio = sum(W.spec_flops(specs[i]) for i in sample) / sum(W.spec_flops(sp) for sp in specs)
    cpu_rate = len(specs) * ratio / cpu_s if cpu_s > 0 else None
    line = {"metric": "uneven-batch instances/s (left-canonise + svd_compress to chi/2 + norm; N 16-128, "
                      "d 2-4, chi 16-256)",
            "value": len(specs) / elapsed, "unit": "instances/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": elapsed * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/c64", "data": "synthetic (seeded Gaussian MPS generated on the device)",
            "config": {"workload": "uneven_batch", "instances": len(specs), "seed": 1, "streams": B,
                       "scheduling": "heaviest first on a work queue, workers admitted %d ms apart"
                                     % int(STAGGER * 1e3)},
            "fidelity_error_max_vs_oracle": fid_err, "oracle_sample": len(sample),
            "clocks": clk.summary(),
            "cpu_baseline": {"value": cpu_rate, "unit": "instances/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d instances of the batch through the oracle (left_canonical_form + "
                                       "svd_compress), scaled by their flop share %.4f" % (len(sample), ratio)}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.micro:
        return run_micro(args)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
