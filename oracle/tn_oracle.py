"""CPU oracle for the tncontract hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain NumPy, the algorithms of the reference library
(andrewdarmawan/tncontract) on the path that ``tncontract_gb300`` accelerates:
labelled pairwise contraction, matricised SVD / QR, truncation rules, MPS
canonisation, SVD compression, MPO-MPS application, MPS inner products and the
2-D boundary-MPS column contraction.  Every function names the reference
``file:line`` it follows.  The numerical kernels are the same LAPACK/BLAS
calls the reference makes (``np.tensordot``, ``np.linalg.svd`` (gesdd),
``np.linalg.qr`` (geqrf/orgqr)), so results agree with the reference to
rounding.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference legs may import this module, and only as the checker / the
timed CPU implementation; the product package never imports it.

Parity of this restatement is pinned against fixtures produced by running the
reference itself (``tests/golden/gen_golden.py``); see
``tests/test_oracle_golden.py``.

Layout convention used throughout the MPS helpers: a site is an ndarray of
shape ``(phys, left, right)``; an MPO site is ``(physout, physin, left,
right)``.  The reference keeps labels instead of a fixed layout; the label
bookkeeping (which only permutes axes) is restated separately in
``contract_labelled`` / ``consolidate``.
"""
from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------
# Labelled tensors: tncontract/tensor.py
# ---------------------------------------------------------------------------


def _as_list(x):
    return x if isinstance(x, list) else [x]


def contract_labelled(d1, l1, d2, l2, labels1, labels2,
                      index_slice1=None, index_slice2=None):
    """Pairwise labelled contraction, ``tensor.py:635-770``.

    All axes of ``d1`` whose label is in ``labels1`` (in the order of
    ``labels1``, every occurrence of a repeated label, ``:702-712``) are
    contracted with the matching axes of ``d2``; ``index_slice`` picks a subset,
    ``-1`` meaning the last match (``:716-731``).  Output labels are the
    uncontracted labels of ``d1`` then of ``d2`` in their original order
    (``:764-768``).
    """
    labels1 = _as_list(labels1)
    labels2 = _as_list(labels2)
    ax1 = []
    for lab in labels1:
        ax1.extend(i for i, x in enumerate(l1) if x == lab)
    ax2 = []
    for lab in labels2:
        ax2.extend(i for i, x in enumerate(l2) if x == lab)
    if index_slice1 is not None:
        sl = [x if x != -1 else len(ax1) - 1 for x in index_slice1]
        ax1 = [a for i, a in enumerate(ax1) if i in sl]
    if index_slice2 is not None:
        sl = [x if x != -1 else len(ax2) - 1 for x in index_slice2]
        ax2 = [a for i, a in enumerate(ax2) if i in sl]
    out = np.tensordot(d1, d2, (ax1, ax2))
    lab = [x for j, x in enumerate(l1) if j not in ax1] + \
          [x for j, x in enumerate(l2) if j not in ax2]
    return out, lab


def consolidate(data, labels, only=()):
    """Fuse all axes sharing a label, ``tensor.py:340-370``.

    Labels are visited in sorted order; the axes of label number ``p`` are
    rolled (in their original relative order) to position ``p`` and fused with
    the first occurrence most significant.  With ``only`` non-empty, only those
    labels are fused (and only they move).
    """
    labels = list(labels)
    uniq = sorted(set(labels))
    if only:
        uniq = [x for x in uniq if x in only]
    for p, lab in enumerate(uniq):
        idx = [i for i, x in enumerate(labels) if x == lab]
        for k, q in enumerate(idx):
            data = np.rollaxis(data, q, p + k)
        tot = 1
        for r in range(len(idx)):
            tot *= data.shape[p + r]
        data = data.reshape(data.shape[:p] + (tot,) + data.shape[p + len(idx):])
        rest = [x for x in labels if x != lab]
        rest.insert(p, lab)
        labels = rest
    return data, labels


def move_index(data, labels, label, position):
    """``Tensor.move_index``, ``tensor.py:380-394``."""
    labels = list(labels)
    i = labels.index(label)
    labels.pop(i)
    labels.insert(position, label)
    if position <= i:
        data = np.rollaxis(data, i, position)
    else:
        data = np.rollaxis(data, i, position + 1)
    return data, labels


def matricise(data, labels, row_labels):
    """Row labels to the front in the given order, then reshape
    (``tensor_svd`` ``tensor.py:903-912``, ``tensor_to_matrix`` ``:805-818``)."""
    for i, lab in enumerate(row_labels):
        data, labels = move_index(data, labels, lab, i)
    nrow = int(np.prod(data.shape[:len(row_labels)], dtype=np.int64))
    mat = data.reshape(nrow, -1)
    return mat, data.shape, labels


def tensor_svd(data, labels, row_labels, svd_label="svd_"):
    """``tensor_svd`` without absorption, ``tensor.py:830-943``.

    Returns ``(U, Ulabels, s, V, Vlabels)`` with ``s`` the singular values as a
    1-D array (the reference stores ``np.diag(s)``, ``:940``)."""
    mat, shp, lab = matricise(data, labels, row_labels)
    u, s, v = np.linalg.svd(mat, full_matrices=False)
    nr = len(row_labels)
    U = u.reshape(tuple(shp[:nr]) + (u.shape[1],))
    V = v.reshape((v.shape[0],) + tuple(shp[nr:]))
    return (U, list(row_labels) + [svd_label + "in"], s,
            V, [svd_label + "out"] + lab[nr:])


def truncation_keep(s, chi=0, threshold=1e-15, absolute=True):
    """Number of singular values ``truncated_svd`` keeps, ``tensor.py:1137-1152``:
    cut to ``chi`` first, then keep ``s > threshold`` (absolute) or
    ``s > s[0]*threshold`` (relative).  ``s`` is sorted descending."""
    keep = s[:chi] if chi else s
    thr = threshold if absolute else s[0] * threshold
    return int(np.count_nonzero(keep > thr))


def canonise_keep(s, chi, threshold):
    """Number of singular values ``left_canonise`` keeps,
    ``onedim_core.py:332-339``: ``s/s[0] > threshold`` (strict), then ``[:chi]``.
    """
    k = int(np.count_nonzero(s / s[0] > threshold))
    if chi:
        k = min(k, chi)
    return k


def tensor_qr(data, labels, row_labels, qr_label="qr_"):
    """``tensor_qr``, ``tensor.py:962-1055`` (reduced QR, ``:1044``)."""
    row_labels = _as_list(row_labels)
    # move_indices(row_labels, 0) without preserve_relative_order
    # (tensor.py:452-478): row labels end up first, in the given order.
    for i, lab in enumerate(row_labels):
        data, labels = move_index(data, labels, lab, i)
    nr = len(row_labels)
    nrow = int(np.prod(data.shape[:nr], dtype=np.int64))
    q, r = np.linalg.qr(data.reshape(nrow, -1), mode="reduced")
    Q = q.reshape(tuple(data.shape[:nr]) + (q.shape[1],))
    R = r.reshape((r.shape[0],) + tuple(data.shape[nr:]))
    return Q, list(row_labels) + [qr_label + "in"], R, [qr_label + "out"] + labels[nr:]


# ---------------------------------------------------------------------------
# MPS algorithms: tncontract/onedim/onedim_core.py, sites in (phys,left,right)
# ---------------------------------------------------------------------------


def mps_reverse(sites):
    """``OneDimensionalTensorNetwork.reverse``, ``onedim_core.py:84-88``: the
    site order flips and the roles of the left/right legs swap."""
    return [np.ascontiguousarray(np.transpose(a, (0, 2, 1))) for a in sites[::-1]]


def _zero_product_state(sites):
    # onedim_core.py:273-278, 305-309, 323-330
    return [np.zeros((a.shape[0], 1, 1), dtype=a.dtype) for a in sites]


def left_canonise_qr(sites, normalise=False):
    """QR branch of ``left_canonise``, ``onedim_core.py:267-294``."""
    sites = [a.copy() for a in sites]
    N = len(sites)
    for i in range(N):
        a = sites[i]
        if i == N - 1:
            nrm = np.linalg.norm(a)
            if nrm == 0.0:
                return _zero_product_state(sites)
            if normalise:
                sites[i] = a / nrm
            return sites
        d, l, r = a.shape
        q, rr = np.linalg.qr(a.reshape(d * l, r), mode="reduced")
        k = q.shape[1]
        sites[i] = q.reshape(d, l, k)
        # contract(R, next, right, left) then relabel, :291-294
        nxt = np.tensordot(rr, sites[i + 1], (1, 1))  # (k, phys, right)
        sites[i + 1] = np.ascontiguousarray(nxt.transpose(1, 0, 2))
    return sites


def left_canonise_svd(sites, chi=None, threshold=1e-14, normalise=False,
                      spectra=None, discarded=None, discarded_fraction=None):
    """SVD branch of ``left_canonise``, ``onedim_core.py:296-358``.

    Each site's singular values are divided by the largest one, whose product
    is tracked in ``norm`` (``:332-334``); ``s/s_max > threshold`` then
    ``[:chi]`` are kept (``:336-339``); ``S V`` is absorbed into the next site
    (``:347-351``); the last site is normalised or multiplied by ``norm``
    (``:301-314``).  If given, ``spectra`` / ``discarded`` /
    ``discarded_fraction`` receive per bond the kept singular values
    (un-normalised), the discarded weight sum(s[k:]^2) and that weight as a
    fraction of sum(s^2).
    """
    sites = [a.copy() for a in sites]
    N = len(sites)
    norm = 1.0
    for i in range(N):
        a = sites[i]
        if i == N - 1:
            if np.linalg.norm(a) == 0.0:
                return _zero_product_state(sites)
            if normalise:
                sites[i] = a / np.linalg.norm(a)
            else:
                sites[i] = a * norm
            return sites
        d, l, r = a.shape
        u, s, vh = np.linalg.svd(a.reshape(d * l, r), full_matrices=False)
        smax = s[0]
        if smax == 0.0:
            return _zero_product_state(sites)
        sn = s / smax
        norm *= smax
        k = int(np.count_nonzero(sn > threshold))
        if chi:
            k = min(k, chi)
        if spectra is not None:
            spectra.append(s[:k].copy())
        if discarded is not None:
            discarded.append(float(np.sum(s[k:] ** 2)))
        if discarded_fraction is not None:
            discarded_fraction.append(float(np.sum(s[k:] ** 2) / np.sum(s ** 2)))
        sites[i] = u[:, :k].reshape(d, l, k)
        sv = sn[:k, None] * vh[:k]
        nxt = np.tensordot(sv, sites[i + 1], (1, 1))  # (k, phys, right)
        sites[i + 1] = np.ascontiguousarray(nxt.transpose(1, 0, 2))
    return sites


def right_canonise_svd(sites, chi=None, threshold=1e-14, normalise=False,
                       spectra=None, discarded=None, discarded_fraction=None):
    """``right_canonise`` = reverse, left-canonise, reverse
    (``onedim_core.py:360-378``).  Spectra are reported right-to-left."""
    return mps_reverse(left_canonise_svd(mps_reverse(sites), chi, threshold,
                                         normalise, spectra, discarded, discarded_fraction))


def left_canonical_form_mps(sites, chi=0, threshold=1e-14, normalise=False):
    """``onedim_core.py:1425-1436``."""
    return left_canonise_svd(sites, chi, threshold, normalise)


def svd_compress_method(sites, chi=None, threshold=1e-15, normalise=False,
                        spectra=None, discarded=None, discarded_fraction=None):
    """``MatrixProductState.svd_compress``, ``onedim_core.py:463-484``: QR left
    sweep, divide by the norm, truncating SVD right sweep, restore the norm.
    Per-bond outputs of the truncating sweep (see ``left_canonise_svd``) are
    reported right-to-left."""
    s1 = left_canonise_qr(sites, normalise=False)
    nrm = np.linalg.norm(s1[-1])
    s1[-1] = s1[-1] / nrm
    s2 = right_canonise_svd(s1, chi, threshold, False, spectra, discarded, discarded_fraction)
    if not normalise:
        s2[0] = s2[0] * nrm
    return s2


def svd_compress_mps(sites, chi, threshold=1e-15, normalise=False,
                     spectra=None, discarded=None):
    """``svd_compress_mps``, ``onedim_core.py:1468-1473``: SVD left sweep
    (threshold only) then truncating SVD right sweep."""
    s1 = left_canonise_svd(sites, 0, threshold, normalise)
    return right_canonise_svd(s1, chi, threshold, normalise, spectra, discarded)


def contract_mps_mpo(sites, mpo):
    """``contract_mps_mpo``, ``onedim_core.py:1691-1708``.

    Per site ``contract(mps[i], mpo[i], phys, physin)`` then
    ``consolidate_indices`` (``tensor.py:340-370``): the fused bond index is
    ``a*D + b`` (MPS bond most significant).  Returned in (phys, left, right)
    layout with phys = the MPO's physout."""
    out = []
    for a, w in zip(sites, mpo):
        d, l, r = a.shape
        do, di, wl, wr = w.shape
        t = np.tensordot(a, w, (0, 1))  # (l, r, physout, wl, wr)
        t = t.transpose(2, 0, 3, 1, 4).reshape(do, l * wl, r * wr)
        out.append(np.ascontiguousarray(t))
    return out


def inner_product(bra, ket, complex_conjugate_bra=True):
    """``inner_product_mps`` via ``ladder_contract``, ``onedim_core.py:1491-1683``:
    left-to-right environment ``C[a,b]``, two contractions per site
    (``:1587-1607``)."""
    # open boundaries: the outer legs have dimension 1
    C = np.ones((bra[0].shape[1], ket[0].shape[1]))
    for a, b in zip(bra, ket):
        if complex_conjugate_bra:
            a = np.conj(a)
        T = np.tensordot(C, a, (0, 1))            # (b_left, phys, a_right)
        C = np.tensordot(T, b, ([0, 1], [1, 0]))  # (a_right, b_right)
    return C.reshape(-1)[0] if C.size == 1 else C


def mps_norm(sites):
    """``MatrixProductState.norm``, ``onedim_core.py:642-660``."""
    return float(np.sqrt(np.real(inner_product(sites, sites))))


def fidelity(a, b):
    """|<a|b>|^2 / (<a|a><b|b>)."""
    ab = inner_product(a, b)
    aa = inner_product(a, a)
    bb = inner_product(b, b)
    return float(abs(ab) ** 2 / (np.real(aa) * np.real(bb)))


def bond_spectra(sites):
    """Schmidt spectrum at every bond (gauge invariant), via an SVD
    left sweep without truncation."""
    spectra = []
    left_canonise_svd(sites, 0, 0.0, False, spectra=spectra)
    return spectra


# ---------------------------------------------------------------------------
# 2-D boundary MPS: tncontract/twodim/square_lattice.py
# ---------------------------------------------------------------------------


def double_layer(ket, bra=None):
    """Double-layer sites of ``inner_product_peps``, ``square_lattice.py:283-304``.

    ``ket[i][j]`` has shape (phys, up, right, down, left).  The result has
    the reference's consolidated label order (down, left, right, up), each leg
    the bra-major fusion of the bra and ket legs."""
    bra = ket if bra is None else bra
    out = []
    for i in range(len(ket)):
        row = []
        for j in range(len(ket[i])):
            b = np.conj(bra[i][j])
            k = ket[i][j]
            t = np.tensordot(b, k, (0, 0))  # (u,r,dn,l | u,r,dn,l)
            u1, r1, d1, l1 = b.shape[1:]
            u2, r2, d2, l2 = k.shape[1:]
            t = t.transpose(2, 6, 3, 7, 1, 5, 0, 4)  # down, left, right, up
            row.append(np.ascontiguousarray(
                t.reshape(d1 * d2, l1 * l2, r1 * r2, u1 * u2)))
        out.append(row)
    return out


def _column_mps_first(col):
    # column_to_mpo col 0, square_lattice.py:405-409: MPS(left=up, right=down,
    # phys=right); (down,left,right,up) -> (phys=right, left=up, right=down)
    return [np.ascontiguousarray(t[:, 0, :, :].transpose(1, 2, 0)) for t in col]


def _column_mps_last(col):
    # square_lattice.py:410-414: phys = left
    return [np.ascontiguousarray(t[:, :, 0, :].transpose(1, 2, 0)) for t in col]


def _column_mpo(col):
    # square_lattice.py:415-417: MPO(left=up, right=down, physout=right,
    # physin=left) -> (physout, physin, left, right)
    return [np.ascontiguousarray(t.transpose(2, 1, 3, 0)) for t in col]


def mps_contract(layer, chi, tolerance=1e-14):
    """``SquareLatticeTensorNetwork.mps_contract`` (svd), ``square_lattice.py:130-203``.

    ``layer[i][j]`` has labels (down, left, right, up).  Returns the scalar
    contraction as ``(mantissa, exponent10)`` plus the plain ``np.longdouble``
    value; the running norm is accumulated in ``np.longdouble`` like the
    reference (``:145, 158-163``)."""
    nrows, ncols = len(layer), len(layer[0])
    cols = [[layer[i][j] for i in range(nrows)] for j in range(ncols)]
    norm = np.longdouble(1)
    comp = None
    for c in range(ncols - 1):
        if c == 0:
            mps = _column_mps_first(cols[0])
        else:
            mps = contract_mps_mpo(comp, _column_mpo(cols[c]))
        comp = svd_compress_mps(mps, chi, threshold=tolerance, normalise=False)
        n = np.linalg.norm(comp[0])
        if n == 0.0:
            return 0.0
        comp[0] = comp[0] / n
        norm *= n
    last = _column_mps_last(cols[-1])
    val = inner_product(comp, last, complex_conjugate_bra=False)
    return np.longdouble(val) * norm if np.isrealobj(val) else val * norm


# ---------------------------------------------------------------------------
# Seeded workloads (the harness builds its own inputs)
# ---------------------------------------------------------------------------


def random_mps(seed, N, d, chi, dtype=np.float64, normalise=False):
    """Seeded random MPS: sites drawn in order, shape (d, chi_l, chi_r),
    bonds [1, chi, ..., chi, 1], entries N(0,1) (complex: re and im each)."""
    rng = np.random.default_rng(seed)
    bd = [1] + [chi] * (N - 1) + [1]
    cplx = np.iscomplexobj(np.zeros(0, dtype))
    sites = []
    for i in range(N):
        shp = (d, bd[i], bd[i + 1])
        if cplx:
            a = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
        else:
            a = rng.standard_normal(shp)
        sites.append(a.astype(dtype))
    if normalise:
        n = mps_norm(sites)
        sites[0] = (sites[0] / n).astype(dtype)
    return sites


def graded_mps(seed, N, d, chi, decades=20.0, dtype=np.float64):
    """Seeded MPS whose bond spectra fall over ``decades`` orders of
    magnitude: Gaussian sites whose right-bond columns are scaled by
    10**(-decades * j / (r - 1)).  A relative truncation threshold (not the
    bond cap) then decides every rank, as it does for the boundary MPS of a
    PEPS norm network.  Not in the reference (an input generator)."""
    rng = np.random.default_rng(seed)
    bonds = [1] + [min(chi, d ** (i + 1), d ** (N - 1 - i)) for i in range(N - 1)] + [1]
    out = []
    for i in range(N):
        r = bonds[i + 1]
        a = rng.standard_normal((d, bonds[i], r))
        if np.iscomplexobj(np.zeros(0, dtype)):
            a = a + 1j * rng.standard_normal((d, bonds[i], r))
        lam = 10.0 ** (-decades * np.arange(r) / max(r - 1, 1))
        out.append((a * lam[None, None, :]).astype(dtype))
    return out


def tfim_mpo(N, J=1.0, h=0.5, dtype=np.float64):
    """Transverse-field Ising MPO, H = -J sum Z_i Z_{i+1} - h sum X_i, bond D=3,
    lower-triangular W = [[I,0,0],[Z,0,0],[-hX,-JZ,I]] with boundary row/column
    slices.  Sites are (physout, physin, left, right)."""
    I = np.eye(2)
    X = np.array([[0., 1.], [1., 0.]])
    Z = np.diag([1., -1.])
    W = np.zeros((3, 3, 2, 2))
    W[0, 0] = I
    W[1, 0] = Z
    W[2, 0] = -h * X
    W[2, 1] = -J * Z
    W[2, 2] = I
    out = []
    for i in range(N):
        w = W
        if i == 0:
            w = w[2:3]
        if i == N - 1:
            w = w[:, 0:1]
        out.append(np.ascontiguousarray(np.transpose(w, (2, 3, 0, 1))).astype(dtype))
    return out


def xxz_mpo(N, delta=0.8, dtype=np.float64):
    """Heisenberg XXZ MPO, H = sum (X X + Y Y + delta Z Z)/4 written with
    S+ S- terms, bond D=5 (lower triangular)."""
    I = np.eye(2)
    Sp = np.array([[0., 1.], [0., 0.]])
    Sm = Sp.T
    Sz = np.diag([0.5, -0.5])
    W = np.zeros((5, 5, 2, 2))
    W[0, 0] = I
    W[1, 0] = Sp
    W[2, 0] = Sm
    W[3, 0] = Sz
    W[4, 1] = 0.5 * Sm
    W[4, 2] = 0.5 * Sp
    W[4, 3] = delta * Sz
    W[4, 4] = I
    out = []
    for i in range(N):
        w = W
        if i == 0:
            w = w[4:5]
        if i == N - 1:
            w = w[:, 0:1]
        out.append(np.ascontiguousarray(np.transpose(w, (2, 3, 0, 1))).astype(dtype))
    return out


def random_peps(seed, nrows, ncols, D, d, dtype=np.float64):
    """Seeded open-boundary PEPS, sites (phys, up, right, down, left), entries
    uniform[0,1); boundary legs have dimension 1."""
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


def apply_compress_sweep(sites, mpo, chi, threshold=1e-15, discarded_fraction=None):
    """One unit of the benchmark: ``contract_mps_mpo`` then
    ``MatrixProductState.svd_compress(chi)`` (QR left sweep, truncating SVD
    right sweep).  ``discarded_fraction`` (a list) receives the discarded
    fraction of the squared spectrum per bond, bonds left to right."""
    df = [] if discarded_fraction is not None else None
    out = svd_compress_method(contract_mps_mpo(sites, mpo), chi, threshold, discarded_fraction=df)
    if df is not None:
        discarded_fraction.extend(df[::-1])
    return out
