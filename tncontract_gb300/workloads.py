"""Seeded synthetic workloads and the algorithmic flop model of one
MPO-MPS apply + compress sweep.

The reference ships only a D=2 one-body MPO builder (onebody_sum_mpo,
tncontract/onedim/onedim_utils.py:122-172) and NumPy-global random states
(init_mps_random, :23-60); the benchmark workloads need seeded generators and
the transverse-field Ising (D=3) and XXZ (D=5) MPOs, stated here.  Draw order:
sites in order, each of shape (d, chi_l, chi_r), bonds [1, chi, ..., chi, 1],
entries N(0,1) (complex: real part then imaginary part per site).
"""
from __future__ import annotations

import numpy as np


def random_mps_arrays(seed, N, d, chi, dtype=np.complex128, normalise=False):
    rng = np.random.default_rng(seed)
    bd = [1] + [chi] * (N - 1) + [1]
    cplx = np.iscomplexobj(np.zeros(0, dtype))
    sites = []
    for i in range(N):
        shp = (d, bd[i], bd[i + 1])
        a = rng.standard_normal(shp) + 1j * rng.standard_normal(shp) if cplx else rng.standard_normal(shp)
        sites.append(a.astype(dtype))
    if normalise:
        # <psi|psi> by a left-to-right environment sweep (float64 on the host)
        C = np.ones((1, 1))
        for a in sites:
            T = np.tensordot(C, np.conj(a), (0, 1))
            C = np.tensordot(T, a, ([0, 1], [1, 0]))
        sites[0] = (sites[0] / np.sqrt(np.real(C.reshape(-1)[0]))).astype(dtype)
    return sites


def tfim_mpo_arrays(N, J=1.0, h=0.5, dtype=np.float64):
    """H = -J sum Z_i Z_{i+1} - h sum X_i as a lower-triangular D=3 MPO,
    W = [[I,0,0],[Z,0,0],[-hX,-JZ,I]], first site the last row, last site the
    first column.  Sites are (physout, physin, left, right)."""
    I = np.eye(2)
    X = np.array([[0., 1.], [1., 0.]])
    Z = np.diag([1., -1.])
    W = np.zeros((3, 3, 2, 2))
    W[0, 0], W[1, 0], W[2, 0], W[2, 1], W[2, 2] = I, Z, -h * X, -J * Z, I
    return _mpo_sites(W, N, dtype)


def xxz_mpo_arrays(N, delta=0.8, dtype=np.float64):
    """Heisenberg XXZ, H = sum (S+S- + S-S+)/2 + delta Sz Sz, as a D=5 MPO."""
    I = np.eye(2)
    Sp = np.array([[0., 1.], [0., 0.]])
    Sm = Sp.T
    Sz = np.diag([0.5, -0.5])
    W = np.zeros((5, 5, 2, 2))
    W[0, 0], W[1, 0], W[2, 0], W[3, 0] = I, Sp, Sm, Sz
    W[4, 1], W[4, 2], W[4, 3], W[4, 4] = 0.5 * Sm, 0.5 * Sp, delta * Sz, I
    return _mpo_sites(W, N, dtype)


def _mpo_sites(W, N, dtype):
    D = W.shape[0]
    out = []
    for i in range(N):
        w = W
        if i == 0:
            w = w[D - 1:D]
        if i == N - 1:
            w = w[:, 0:1]
        out.append(np.ascontiguousarray(np.transpose(w, (2, 3, 0, 1))).astype(dtype))
    return out


def random_peps_arrays(seed, nrows, ncols, D, d, dtype=np.float64):
    """Open-boundary PEPS, sites (phys, up, right, down, left), uniform[0,1)."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(nrows):
        row = []
        for j in range(ncols):
            u = 1 if i == 0 else D
            dn = 1 if i == nrows - 1 else D
            lft = 1 if j == 0 else D
            rgt = 1 if j == ncols - 1 else D
            row.append(rng.uniform(0, 1, (d, u, rgt, dn, lft)).astype(dtype))
        rows.append(row)
    return rows


def config3_specs(seed=1, count=512):
    """The uneven batch: per instance N ~ U{16..128}, d ~ {2, 3, 4},
    chi ~ U{16..256}, dtype alternating float32 / complex64 (drawn in this
    order from one generator); the instance's sites use seed (seed*100000 + b)."""
    rng = np.random.default_rng(seed)
    specs = []
    for b in range(count):
        N = int(rng.integers(16, 129))
        d = int(rng.choice([2, 3, 4]))
        chi = int(rng.integers(16, 257))
        specs.append((N, d, chi, np.complex64 if b % 2 else np.float32, seed * 100000 + b))
    return specs


def double_layer_arrays(peps_rows):
    """Double-layer norm tensors conj(ket).ket over phys with legs
    (down, left, right, up), each the bra-major fusion of the two layers
    (inner_product_peps + consolidate_indices, square_lattice.py:283-304)."""
    out = []
    for row in peps_rows:
        r = []
        for k in row:
            t = np.tensordot(np.conj(k), k, (0, 0))  # (u,r,dn,l | u,r,dn,l)
            u, rr, dn, lf = k.shape[1:]
            t = t.transpose(2, 6, 3, 7, 1, 5, 0, 4).reshape(dn * dn, lf * lf, rr * rr, u * u)
            r.append(np.ascontiguousarray(t))
        out.append(r)
    return out


def sweep_flops(N, d, D, chi, complex_=True, chi_in=None):
    """Algorithmic flops of one apply + svd_compress sweep (fixed count,
    implementation independent), from the bond dimensions the plain method
    produces.  Per site: apply 2 d^2 D_l D_r chi_l chi_r; QR of m x n (m >= n)
    2 m n^2 - 2/3 n^3; R absorption 2 k n (d chi'_next); thin SVD with U, V
    (m >= n) 6 m n^2 + 20 n^3 (Golub & Van Loan's R-SVD count); U S absorption
    2 m_prev n k.  Complex operations count 4 real flops.  Returns a dict of
    the parts and the total."""
    chi_in = chi if chi_in is None else chi_in
    mps_b = [1] + [chi_in] * (N - 1) + [1]
    mpo_b = [1] + [D] * (N - 1) + [1]
    bp = [mps_b[i] * mpo_b[i] for i in range(N + 1)]  # applied bonds
    f = {"apply": 0.0, "qr": 0.0, "r_absorb": 0.0, "svd": 0.0, "us_absorb": 0.0}
    for i in range(N):
        f["apply"] += 2.0 * d * d * mpo_b[i] * mpo_b[i + 1] * mps_b[i] * mps_b[i + 1]
    # QR left sweep
    b = [1] * (N + 1)
    b[0] = bp[0]
    for i in range(N - 1):
        m, n = d * b[i], bp[i + 1]
        k = min(m, n)
        mm, nn = max(m, n), min(m, n)
        f["qr"] += 2.0 * mm * nn * nn - 2.0 / 3.0 * nn ** 3
        f["r_absorb"] += 2.0 * k * n * d * bp[i + 2]
        b[i + 1] = k
    b[N] = bp[N]
    # truncating SVD right sweep (reversed frame)
    kr = b[N]
    for i in range(N - 1, 0, -1):
        m, n = d * kr, b[i]
        mm, nn = max(m, n), min(m, n)
        f["svd"] += 6.0 * mm * nn * nn + 20.0 * nn ** 3
        k = min(chi, nn)
        f["us_absorb"] += 2.0 * d * b[i - 1] * n * k
        kr = k
    scale = 4.0 if complex_ else 1.0
    for key in f:
        f[key] *= scale
    f["total"] = sum(f.values())
    return f


def instance_flops(N, d, chi, complex_=True):
    """Estimated flops of one left-canonise + svd_compress of an N-site MPS
    (phys d, bond chi): the sweep count above with no MPO (D = 1)."""
    return sweep_flops(N, d, 1, chi, complex_=complex_)["total"]


def spec_flops(spec):
    """instance_flops of one (N, d, chi, dtype, seed) spec of the uneven batch."""
    N, d, chi, dt, _seed = spec
    return instance_flops(N, d, chi, bool(np.iscomplexobj(np.zeros(0, dt))))


def partition_by_flops(specs, world):
    """Split independent instances across ``world`` ranks, balancing the
    estimated flops (greedy longest-processing-time: heaviest first, each to
    the least-loaded rank).  ``specs`` are (N, d, chi, dtype, seed) tuples;
    returns one sorted list of instance indices per rank.  Deterministic, so
    every rank computes the same split without communicating."""
    cost = [spec_flops(sp) for sp in specs]
    order = sorted(range(len(specs)), key=lambda i: (-cost[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += cost[i]
    return [sorted(p) for p in parts]


def run_sharded(specs, make_job, run_jobs, rank=0, world=1):
    """Run this rank's share of independent instances: the flop-balanced
    split of ``partition_by_flops`` (every rank computes the same split, so
    no data moves between ranks), heaviest first.  ``make_job(i)`` returns a
    callable computing instance i's result; ``run_jobs(jobs)`` runs a list of
    them (on the GPU: ``engine.run_queue`` over worker streams) and returns
    their results in order.  Returns {instance index: result} for this rank."""
    mine = partition_by_flops(specs, world)[rank]
    mine = sorted(mine, key=lambda i: (-spec_flops(specs[i]), i))
    results = run_jobs([make_job(i) for i in mine])
    return dict(zip(mine, results))


def gather_results(local, world, dst=0):
    """The only exchange of a sharded batch: every rank's {index: per-instance
    scalars} gathered to rank ``dst`` (torch.distributed.gather_object over
    the default process group).  Returns the merged dict on ``dst``, None on
    the other ranks; with one rank, ``local`` itself."""
    if world <= 1:
        return local
    import torch.distributed as dist
    got = [None] * world if dist.get_rank() == dst else None
    dist.gather_object(local, got, dst=dst)
    if dist.get_rank() != dst:
        return None
    merged = {}
    for part in got:
        merged.update(part)
    return merged
