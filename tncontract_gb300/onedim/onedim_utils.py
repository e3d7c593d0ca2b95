"""MPS / MPO utilities on the GPU: the drop-in for
tncontract/onedim/onedim_utils.py (constructors of simple states, the
one-body-sum MPO, single-site expectation values and reduced density
matrices).  Host code builds the small constructor arrays; sites live on the
device and every contraction, factorisation and scaling runs in the native
library.
"""
from __future__ import annotations

import numpy as np

from .. import _ops
from .. import tensor as tsr
from . import onedim_core as onedim

__all__ = ['init_mps_random', 'init_mps_allzero', 'init_mps_logical', 'onebody_sum_mpo', 'expvals_mps',
           'ptrace_mps']


def _per_site(value, n):
    return list(value) if np.iterable(value) else [value] * n


def init_mps_random(nsites, physdim, bonddim=1, left_label='left', right_label='right', phys_label='phys'):
    """``onedim_utils.py:23-60``: sites with entries uniform in [0, 1) from
    NumPy's global generator (shape (physdim, left bond, right bond), open
    ends), each rescaled so its largest singular value (rows: phys, left) is
    1.  Not normalised."""
    physdim = _per_site(physdim, nsites)
    bonds = [1] + _per_site(bonddim, nsites - 1) + [1]
    sites = []
    for i in range(nsites):
        raw = tsr.Tensor(np.random.rand(physdim[i], bonds[i], bonds[i + 1]), [phys_label, left_label, right_label])
        U, S, V = tsr.tensor_svd(raw, [phys_label, left_label])
        smax = float(S.data[0, 0].real.item())
        S.data = _ops.scale(S.data, 1.0 / smax)
        site = U["svd_in", ] * S["svd_out", ]
        sites.append(site["svd_in", ] * V["svd_out", ])
    return onedim.MatrixProductState(sites, left_label=left_label, right_label=right_label, phys_label=phys_label)


def _product_state(nsites, levels, physdim, left_label, right_label, phys_label):
    physdim = _per_site(physdim, nsites)
    sites = []
    for j in range(nsites):
        v = np.zeros(physdim[j])
        v[levels[j]] = 1.0
        sites.append(tsr.Tensor(v.reshape(physdim[j], 1, 1), [phys_label, left_label, right_label]))
    return onedim.MatrixProductState(sites, left_label=left_label, right_label=right_label, phys_label=phys_label)


def init_mps_allzero(nsites, physdim, left_label='left', right_label='right', phys_label='phys'):
    """``onedim_utils.py:63-88``: the product state |00..0>."""
    return _product_state(nsites, [0] * nsites, physdim, left_label, right_label, phys_label)


def init_mps_logical(nsites, basis_state, physdim, left_label='left', right_label='right', phys_label='phys'):
    """``onedim_utils.py:91-119``: the product state |basis_state[0] ...>
    (the reference indexes ``basis_state`` per site)."""
    return _product_state(nsites, basis_state, physdim, left_label, right_label, phys_label)


def onebody_sum_mpo(terms, output_label=None):
    """``onedim_utils.py:122-172``: bond-2 MPO of sum_i term_i
    (Sanchez-Burillo et al., PRL 113, 263604, Supplemental Eqs. 3-4): the
    first site is [term, 1], the last [1, term]^T, the middle sites
    [[1, 0], [term, 1]]; complex entries, labels physout / physin /
    left / right.  A term is a 2-D array or a rank-2 Tensor (its
    ``output_label`` leg, or its first leg, is the output)."""
    sites = []
    n = len(terms)
    for i, term in enumerate(terms):
        if isinstance(term, tsr.Tensor):
            t = term.copy()
            if output_label is not None:
                t.move_index(output_label, 0)
            op = t.to_numpy()
        else:
            op = np.asarray(term)
        eye = np.eye(op.shape[0], op.shape[1])
        if i == 0:
            B = np.stack([op, eye], axis=-1).astype(complex)
            sites.append(tsr.Tensor(B, ['physout', 'physin', 'right']))
        elif i == n - 1:
            B = np.stack([eye, op], axis=-1).astype(complex)
            sites.append(tsr.Tensor(B, ['physout', 'physin', 'left']))
        else:
            B = np.zeros(op.shape + (2, 2), dtype=complex)
            B[:, :, 0, 0] = eye
            B[:, :, 1, 0] = op
            B[:, :, 1, 1] = eye
            sites.append(tsr.Tensor(B, ['physout', 'physin', 'left', 'right']))
    return onedim.MatrixProductOperator(sites, left_label='left', right_label='right', physin_label='physin',
                                        physout_label='physout')


def _orthogonality_walk(mps, canonised):
    """Bring ``mps`` to right-canonical form (or reverse a left-canonical
    one) as ``expvals_mps`` / ``ptrace_mps`` do (``onedim_utils.py:230-234``)."""
    if canonised == 'left':
        mps.reverse()
    elif canonised != 'right':
        mps.right_canonise()


def expvals_mps(mps, oplist=[], sites=None, output_label=None, canonised=None):
    """``onedim_utils.py:175-255``: <op_i> at each site in ``sites`` (all by
    default), moving the orthogonality centre site by site with
    ``left_canonise``; returns a complex NumPy array.  ``oplist`` is one
    rank-2 Tensor for every site or a list (one per requested site)."""
    if sites is None:
        sites = range(len(mps))
    if not np.iterable(sites):
        sites = [sites]
    n = len(sites)
    out = np.zeros(n, dtype=complex)
    ops = oplist if isinstance(oplist, list) else [oplist] * n
    if canonised == 'left':
        ops = ops[::-1]
    _orthogonality_walk(mps, canonised)
    centre = 0
    for i, site in enumerate(sites):
        mps.left_canonise(centre, site)
        centre = site
        op = ops[i]
        if output_label is None:
            out_leg, in_leg = op.labels[0], op.labels[1]
        else:
            out_leg = output_label
            in_leg = [x for x in op.labels if x != out_leg][0]
        A = mps[site]
        Ad = A.copy()
        Ad.conjugate()
        val = tsr.contract(A, op, mps.phys_label, in_leg)
        val = tsr.contract(Ad, val, mps.phys_label, out_leg)
        val.contract_internal(mps.left_label, mps.left_label, index1=0, index2=1)
        val.contract_internal(mps.right_label, mps.right_label, index1=0, index2=1)
        out[i] = complex(val.data.item())
    if canonised == 'left':
        mps.reverse()
        out = out[::-1]
    return out


def ptrace_mps(mps, sites=None, canonised=None):
    """``onedim_utils.py:258-313``: single-site reduced density matrices
    (legs: phys, phys primed) at each site in ``sites`` (all by default),
    moving the orthogonality centre site by site."""
    rhos = []
    _orthogonality_walk(mps, canonised)
    if sites is None:
        sites = range(len(mps))
    if not np.iterable(sites):
        sites = [sites]
    centre = 0
    for site in sites:
        mps.left_canonise(centre, site)
        centre = site
        A = mps[centre]
        Ad = A.copy()
        Ad.conjugate()
        Ad.prime_label(mps.phys_label)
        rhos.append(tsr.contract(A, Ad, [mps.left_label, mps.right_label], [mps.left_label, mps.right_label]))
    if canonised == 'left':
        mps.reverse()
        rhos = rhos[::-1]
    return rhos
