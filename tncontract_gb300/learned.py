"""Learned-rank truncation at benchmark scale (the rank predictor of
``rank_model`` in the truncating sweep of ``engine.svd_right_sweep``).

``train_rank_model`` trains the predictor on the GPU, by the library's own
MLP kernels, on singular spectra that the plain method produces on small
instances of the other workloads (config 1: a real random MPS compressed to
half its bond; config 2: the TFIM D=3 MPO applied to a complex random MPS;
config 3: the smallest instances of the uneven batch), with the discarded-
weight rank rule it will be used with.  ``config5`` runs the apply + compress
sweep of a random float32 MPS (N=128, d=2, chi=512) under the Heisenberg XXZ
MPO (Delta=0.8, D=5) with the rule "smallest rank whose discarded weight is
at most dw_tol of the total, at most chi" -- with or without the predictor
(which sizes a randomized SVD, oversampling 16, 2 power iterations, and
falls back to the full SVD when the sketch leaves more than dw_tol of the
weight uncaptured).  The truncation the predictor replaces is the full SVD
of left_canonise (tncontract/onedim/onedim_core.py:317); the discarded-
weight rule and the sweep's learned part have no counterpart in the
reference.  Where the bond cap, not the tolerance, sets a bond's rank (the
neighbouring bond discarded more than 10 dw_tol) no sketch can pass the
tolerance check, so none is tried there (``RankStats.declined``).""" 
from __future__ import annotations

import time

import numpy as np
import torch

from . import engine as E
from . import rank_model as RM
from . import workloads as W


def _collect(rs_feats, rs_targets, sites, mpo, cap, dw_tol, precision):
    dt = E.compute_dtype(precision, any(np.iscomplexobj(a) for a in sites))
    bal, ln = E.balance(sites)
    rs = E.RankStats()
    E.apply_compress(E.to_sites(bal, dt), E.to_sites(mpo, dt), cap, log_norm_in=ln, dw_tol=dw_tol, rank_stats=rs)
    rs_feats += rs.features
    rs_targets += rs.targets


def training_spectra(dw_tol, precision="fp32", uneven=6):
    """(features, targets) of every bond of plain sweeps on small instances
    of configs 1-3 under the discarded-weight rule."""
    feats, targets = [], []
    ident = lambda n, d: [np.eye(d).reshape(d, d, 1, 1) for _ in range(n)]  # noqa: E731
    # config 1: real, N=32, d=2, chi=32, compressed to 16
    _collect(feats, targets, W.random_mps_arrays(0, 32, 2, 32, np.float64), ident(32, 2), 16, dw_tol, precision)
    # config 2 (scaled): TFIM D=3 on complex N=32, chi=64
    for seed in range(2):
        _collect(feats, targets, W.random_mps_arrays(seed, 32, 2, 64, np.complex128, normalise=True),
                 W.tfim_mpo_arrays(32), 64, dw_tol, precision)
    # config 3: the smallest instances of the uneven batch, compressed to chi / 2
    specs = W.config3_specs(1, 512)
    for i in sorted(range(len(specs)), key=lambda j: W.spec_flops(specs[j]))[:uneven]:
        N, d, chi, dt, seed = specs[i]
        sites = W.random_mps_arrays(seed, N, d, chi, np.complex128 if dt == np.complex64 else np.float64)
        _collect(feats, targets, sites, ident(N, d), chi // 2, dw_tol, precision)
    return np.array(feats, np.float32), np.array(targets, np.float32)


def train_rank_model(dw_tol, precision="fp32", steps=400, seed=0):
    """The rank predictor trained on ``training_spectra``; returns (model,
    loss history, number of training bonds)."""
    X, T = training_spectra(dw_tol, precision)
    model = RM.RankMLP(seed=seed)
    hist = model.fit(X, T, steps=steps)
    return model, hist, len(T)


def config5_inputs(N=128, d=2, chi=512, seed=5):
    """Seeded random MPS (float64 draws, not normalised: the sweep carries the
    norm as a logarithm, and <psi|psi> of N=128 sites at chi=512 is ~1e385)
    and the XXZ MPO."""
    return W.random_mps_arrays(seed, N, d, chi, np.float64), W.xxz_mpo_arrays(N)


def config5(sites, mpo, chi=512, dw_tol=1e-8, precision="mixed", model=None):
    """One apply + compress sweep of config 5 on the device; returns (sites,
    seconds, RankStats, SweepStats).  ``precision``: "fp32", "mixed" (float32
    sites, every bond core finished by the double-float Jacobi) or "fp64"."""
    dt = E.compute_dtype(precision, False)
    bal, ln = E.balance(sites)
    S, Mo = E.to_sites(bal, dt), E.to_sites(mpo, dt)
    rs, st = E.RankStats(), E.SweepStats()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = E.apply_compress(S, Mo, chi, log_norm_in=ln, dw_tol=dw_tol, rank_model=model, rank_stats=rs, stats=st,
                           core=E.mixed_core(precision))
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0, rs, st


def fallback_rate(rs):
    tried = rs.sketched + rs.fallbacks
    return rs.fallbacks / tried if tried else None
