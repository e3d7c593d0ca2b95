"""1-D tensor networks on the GPU: the drop-in for
tncontract/onedim/onedim_core.py (hot-path part).

Control flow, label bookkeeping and truncation rules are restated from the
reference (line numbers cited per function); every contraction,
factorisation, norm and rescaling runs in the native library through
``tncontract_gb300.tensor`` / ``_ops``.  Site tensors keep the reference's
label order after every operation (e.g. sites are ``[phys, right, left]``
after a right canonisation), so ``.data`` layouts match the reference's.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _ops
from .. import tensor as tsr
from ..label import unique_label

__all__ = ['MatrixProductState', 'MatrixProductOperator',
           'OneDimensionalTensorNetwork', 'contract_mps_mpo', 'contract_multi_index_tensor_with_one_dim_array',
           'contract_virtual_indices', 'frob_distance_squared', 'inner_product_mps', 'ladder_contract',
           'left_canonical_form_mps', 'mps_complex_conjugate', 'reverse_mps', 'right_canonical_form_mps',
           'svd_compress_mps', 'check_canonical_form_mps']


def _objarray(items):
    arr = np.empty(len(items), dtype=object)
    for i, x in enumerate(items):
        arr[i] = x
    return arr


class OneDimensionalTensorNetwork:
    """Array of site tensors with left/right virtual legs
    (``onedim_core.py:31-183``).  Inputs are copied; missing boundary legs are
    added as dummy legs of dimension 1 (``:59-61``)."""

    def __init__(self, tensors, left_label="left", right_label="right"):
        self.left_label = left_label
        self.right_label = right_label
        self.data = _objarray([x.copy() for x in tensors])
        for x in self.data:
            if left_label not in x.labels:
                x.add_dummy_index(left_label)
            if right_label not in x.labels:
                x.add_dummy_index(right_label)

    def __iter__(self):
        return self.data.__iter__()

    def __len__(self):
        return self.data.__len__()

    def __getitem__(self, key):
        return self.data.__getitem__(key)

    def __setitem__(self, key, value):
        self.data.__setitem__(key, value)

    def copy(self):
        return OneDimensionalTensorNetwork([x.copy() for x in self], self.left_label, self.right_label)

    def reverse(self):
        """``:84-88``: flip the site order and swap the left/right roles."""
        self.data = self.data[::-1]
        self.left_label, self.right_label = self.right_label, self.left_label

    def complex_conjugate(self):
        for x in self.data:
            x.conjugate()

    def replace_labels(self, old_labels, new_labels):
        """``:129-145``"""
        if not isinstance(old_labels, list):
            old_labels = [old_labels]
        if not isinstance(new_labels, list):
            new_labels = [new_labels]
        for x in self.data:
            x.replace_label(old_labels, new_labels)
        if self.left_label in old_labels:
            self.left_label = new_labels[old_labels.index(self.left_label)]
        if self.right_label in old_labels:
            self.right_label = new_labels[old_labels.index(self.right_label)]

    def standard_virtual_labels(self, suffix=""):
        self.replace_labels([self.left_label, self.right_label],
                            ["left" + suffix, "right" + suffix])

    def unique_virtual_labels(self):
        self.replace_labels([self.left_label, self.right_label],
                            [unique_label(), unique_label()])

    def leftdim(self, site):
        return self.data[site].index_dimension(self.left_label)

    def rightdim(self, site):
        return self.data[site].index_dimension(self.right_label)

    def bonddims(self):
        """``:168-175``"""
        if self.nsites == 0:
            return []
        bonds = [self.leftdim(0)]
        for i in range(self.nsites):
            bonds.append(self.rightdim(i))
        return bonds

    @property
    def nsites(self):
        return len(self.data)

    @property
    def nsites_physical(self):
        return self.nsites


def _zero_product_state(mps, N):
    # onedim_core.py:273-278, 305-309, 323-330
    for k in range(N):
        d = mps[k].index_dimension(mps.phys_label)
        mps[k].data = _ops.zeros((d, 1, 1), torch.float64)  # np.zeros default dtype
        mps[k].labels = [mps.phys_label, mps.left_label, mps.right_label]


class MatrixProductState(OneDimensionalTensorNetwork):
    """Matrix product state (``onedim_core.py:186-877``)."""

    def __init__(self, tensors, left_label="left", right_label="right", phys_label="phys"):
        OneDimensionalTensorNetwork.__init__(self, tensors, left_label=left_label,
                                             right_label=right_label)
        self.phys_label = phys_label

    def __repr__(self):
        return ("MatrixProductState(tensors=%r, left_label=%r, right_label=%r,"
                "phys_label=%r)" % (self.data, self.left_label, self.right_label, self.phys_label))

    def __str__(self):
        return ("MatrixProductState object: " + "sites = " + str(len(self)) +
                ", left_label = " + self.left_label + ", right_label = " + self.right_label +
                ", phys_label = " + self.phys_label)

    def copy(self):
        return MatrixProductState([x.copy() for x in self], self.left_label,
                                  self.right_label, self.phys_label)

    def left_canonise(self, start=0, end=-1, chi=None, threshold=1e-14,
                      normalise=False, qr_decomposition=False):
        """``onedim_core.py:218-358``: sweep left to right with QR (no
        truncation) or SVD (keep s/s_max > threshold, then at most chi)."""
        N = len(self)
        if end == -1:
            end = N
        if qr_decomposition:
            for i in range(start, end):
                if i == N - 1:
                    norm = _ops.nrm2(self[i].data)
                    if norm == 0.0:
                        _zero_product_state(self, N)
                        return
                    if normalise and start == 0:
                        self[i].data = _ops.scale(self[i].data, 1.0 / norm)
                    return
                qr_label = unique_label()
                Q, R = tsr.tensor_qr(self[i], [self.phys_label, self.left_label], qr_label=qr_label)
                Q.replace_label(qr_label + "in", self.right_label)
                self[i] = Q
                self[i + 1] = tsr.contract(R, self[i + 1], self.right_label, self.left_label)
                self[i + 1].replace_label(qr_label + "out", self.left_label)
        else:
            norm = 1.0
            for i in range(start, end):
                if i == N - 1:
                    n_last = _ops.nrm2(self[i].data)
                    if n_last == 0.0:
                        _zero_product_state(self, N)
                        return
                    if normalise and start == 0:
                        self[i].data = _ops.scale(self[i].data, 1.0 / n_last)
                    else:
                        self[i].data = _ops.scale(self[i].data, norm)
                    return
                svd_label = unique_label()
                U, s, V = tsr._svd_parts(self[i], [self.phys_label, self.left_label], svd_label)
                # truncation decision on device (s/s_max > threshold, then chi)
                k, _ = _ops.truncation_rank(s, chi or 0, threshold, relative=True)
                smax = float(s[0].item()) if s.numel() else 0.0
                if smax == 0.0:
                    _zero_product_state(self, N)
                    return
                norm *= smax
                # U labels are [phys, left, svd_in]: keep the first k columns
                U = tsr._new(_ops.slice_last(U.data, k), U.labels)
                U.replace_label(svd_label + "in", self.right_label)
                self[i] = U
                # next = S (V next) with S = s[:k] / s_max (onedim_core.py:347-351)
                V = tsr._new(V.data[0:k], V.labels)
                nxt = tsr.contract(V, self[i + 1], self.right_label, self.left_label)
                sn = _ops.scale(s[:k].contiguous(), 1.0 / smax)
                flat = nxt.data.reshape(k, -1).clone()
                _ops.scale_rows(flat, sn, 0)
                nxt = tsr._new(flat.reshape(nxt.data.shape), nxt.labels)
                nxt.replace_label(svd_label + "out", self.left_label)
                self[i + 1] = nxt
                if i == end - 1:
                    self[i + 1].data = _ops.scale(self[i + 1].data, norm)

    def right_canonise(self, start=0, end=-1, chi=None, threshold=1e-14,
                       normalise=False, qr_decomposition=False):
        """``onedim_core.py:360-378``: mirror of ``left_canonise``."""
        self.reverse()
        N = len(self)
        if end == -1:
            end = N
        self.left_canonise(start=N - end, end=N - start, chi=chi, threshold=threshold,
                           normalise=normalise, qr_decomposition=qr_decomposition)
        self.reverse()

    def replace_labels(self, old_labels, new_labels):
        """``onedim_core.py:380-397``"""
        if not isinstance(old_labels, list):
            old_labels = [old_labels]
        if not isinstance(new_labels, list):
            new_labels = [new_labels]
        for x in self.data:
            x.replace_label(old_labels, new_labels)
        if self.left_label in old_labels:
            self.left_label = new_labels[old_labels.index(self.left_label)]
        if self.right_label in old_labels:
            self.right_label = new_labels[old_labels.index(self.right_label)]
        if self.phys_label in old_labels:
            self.phys_label = new_labels[old_labels.index(self.phys_label)]

    def standard_labels(self, suffix=""):
        self.replace_labels([self.left_label, self.right_label, self.phys_label],
                            ["left" + suffix, "right" + suffix, "phys" + suffix])

    def check_canonical_form(self, threshold=1e-14, print_output=True):
        """``onedim_core.py:408-461``: first site (from the left) that is not
        left-isometric and first (from the right) not right-isometric."""
        mps_cc = mps_complex_conjugate(self)
        first_not_left = len(self) - 1
        for i in range(len(self) - 1):
            I = tsr.contract(self[i], mps_cc[i], [self.phys_label, self.left_label],
                             [mps_cc.phys_label, mps_cc.left_label])
            if _identity_residual(I.data) > threshold:
                first_not_left = i
                break
        first_not_right = 0
        for i in range(len(self) - 1, 0, -1):
            I = tsr.contract(self[i], mps_cc[i], [self.phys_label, self.right_label],
                             [mps_cc.phys_label, mps_cc.right_label])
            if _identity_residual(I.data) > threshold:
                first_not_right = i
                break
        if print_output:
            print("first site not left canonised: %d, first site not right canonised: %d"
                  % (first_not_left, first_not_right))
        return (first_not_left, first_not_right)

    def svd_compress(self, chi=None, threshold=1e-15, normalise=False, reverse=False):
        """``onedim_core.py:463-484``: QR left sweep, normalise, truncating SVD
        right sweep, restore the norm (the state ends right-canonical)."""
        if reverse:
            self.reverse()
        self.left_canonise(normalise=False, qr_decomposition=True)
        norm = self.norm(canonical_form="left")
        self[-1].data = _ops.scale(self[-1].data, 1.0 / norm)
        self.right_canonise(chi=chi, threshold=threshold, normalise=False)
        if normalise is False:
            self[0].data = _ops.scale(self[0].data, norm)
        if reverse:
            self.reverse()

    def physical_site(self, n):
        return n

    def physdim(self, site):
        return self.data[site].index_dimension(self.phys_label)

    def norm(self, canonical_form=False):
        """``onedim_core.py:642-660``"""
        if canonical_form == "left":
            return _ops.nrm2(self[-1].data)
        elif canonical_form == "right":
            return _ops.nrm2(self[0].data)
        else:
            ip = inner_product_mps(self, self)
            return float(np.sqrt(_scalar(ip).real))


def _identity_residual(M):
    """|| M - I ||_F for a square device matrix (synchronises)."""
    n = M.shape[0]
    eye = _ops.diag_matrix(torch.ones(n, dtype=_ops.real_dtype(M.dtype), device=M.device), M.dtype)
    diff = M.contiguous().clone()
    _ops.axpby(-1.0, eye, 1.0, diff)
    return _ops.nrm2(diff)


def _scalar(x):
    if isinstance(x, torch.Tensor):
        return complex(x.item()) if x.is_complex() else complex(float(x.item()))
    return complex(x)


class MatrixProductOperator(OneDimensionalTensorNetwork):
    """``onedim_core.py:1329-1367``"""

    def __init__(self, tensors, left_label="left", right_label="right",
                 physout_label="physout", physin_label="physin"):
        OneDimensionalTensorNetwork.__init__(self, tensors, left_label, right_label)
        self.physout_label = physout_label
        self.physin_label = physin_label

    def __str__(self):
        return ("MatrixProductOperator object: " + "sites = " + str(len(self)) +
                ", left_label = " + self.left_label + ", right_label = " + self.right_label +
                ", physout_label = " + self.physout_label + ", physin_label = " + self.physin_label)

    def physoutdim(self, site):
        return self.data[site].index_dimension(self.physout_label)

    def physindim(self, site):
        return self.data[site].index_dimension(self.physin_label)


def contract_multi_index_tensor_with_one_dim_array(tensor, array, label1, label2):
    """``onedim_core.py:1370-1396``"""
    temp_label = unique_label()
    tensor.replace_label(label1, temp_label)
    C = tsr.contract(tensor, array[0], temp_label, label2, index_slice1=[0])
    for i in range(1, len(array)):
        C = tsr.contract(C, array[i], [array.right_label, temp_label],
                         [array.left_label, label2], index_slice1=[0, 1])
    C.contract_internal(array.right_label, array.left_label)
    tensor.replace_label(temp_label, label1)
    return C


def contract_virtual_indices(array_1d, start=0, end=None, periodic_boundaries=True):
    """``onedim_core.py:1399-1422``"""
    C = array_1d[start].copy()
    for x in array_1d[start + 1:end]:
        C = tsr.contract(C, x, array_1d.right_label, array_1d.left_label)
    if periodic_boundaries:
        C.contract_internal(array_1d.right_label, array_1d.left_label)
    return C


def left_canonical_form_mps(orig_mps, chi=0, threshold=1e-14, normalise=False):
    """``onedim_core.py:1425-1436``"""
    mps = orig_mps.copy()
    mps.left_canonise(chi=chi, threshold=threshold, normalise=normalise)
    return mps


def right_canonical_form_mps(orig_mps, chi=0, threshold=1e-14, normalise=False):
    """``onedim_core.py:1439-1445``"""
    mps = orig_mps.copy()
    mps.right_canonise(chi=chi, threshold=threshold, normalise=normalise)
    return mps


def reverse_mps(orig_mps):
    mps = orig_mps.copy()
    mps.reverse()
    return mps


def check_canonical_form_mps(mps, threshold=1e-14, print_output=True):
    return mps.check_canonical_form(threshold=threshold, print_output=print_output)


def svd_compress_mps(orig_mps, chi, threshold=1e-15, normalise=False):
    """``onedim_core.py:1468-1473``: SVD left sweep (threshold only), then
    truncating SVD right sweep."""
    mps = left_canonical_form_mps(orig_mps, threshold=threshold, normalise=normalise)
    return right_canonical_form_mps(mps, chi=chi, threshold=threshold, normalise=normalise)


def mps_complex_conjugate(mps):
    """``onedim_core.py:1482-1488``"""
    new_mps = mps.copy()
    for x in new_mps.data:
        x.conjugate()
    return new_mps


def ladder_contract(array1, array2, label1, label2, start=0, end=None,
                    complex_conjugate_array1=False, left_output_label="left",
                    right_output_label="right", return_intermediate_contractions=False):
    """``onedim_core.py:1491-1663``: contract two 1-D networks rung by rung."""
    if end is None:
        end = min(array1.nsites, array2.nsites) - 1
    if end < start:
        raise ValueError("Badly defined interval (end before start).")
    a1 = array1.copy()
    a2 = array2.copy()
    if complex_conjugate_array1:
        a1.complex_conjugate()
    a1.unique_virtual_labels()
    a2.unique_virtual_labels()
    rung_label = unique_label()
    a1.replace_labels(label1, rung_label)
    a2.replace_labels(label2, rung_label)
    inter = []
    if start == 0:
        for i in range(0, end + 1):
            if i == 0:
                C = tsr.contract(a1[0], a2[0], rung_label, rung_label)
            else:
                C.contract(a1[i], a1.right_label, a1.left_label)
                C.contract(a2[i], [a2.right_label, rung_label], [a2.left_label, rung_label])
            if return_intermediate_contractions:
                t = C.copy()
                t.replace_label([a1.right_label, a2.right_label],
                                [right_output_label + "1", right_output_label + "2"])
                t.remove_all_dummy_indices(labels=[x for x in t.labels if x not in
                                                   [right_output_label + "1", right_output_label + "2"]])
                inter.append(t)
        C.replace_label([a1.right_label, a2.right_label],
                        [right_output_label + "1", right_output_label + "2"])
        C.remove_all_dummy_indices()
    elif end == a1.nsites - 1 and end == a2.nsites - 1:
        for i in range(end, start - 1, -1):
            if i == end:
                C = tsr.contract(a1[end], a2[end], rung_label, rung_label)
            else:
                C.contract(a1[i], a1.left_label, a1.right_label)
                C.contract(a2[i], [a2.left_label, rung_label], [a2.right_label, rung_label])
            if return_intermediate_contractions:
                t = C.copy()
                t.replace_label([a1.left_label, a2.left_label],
                                [left_output_label + "1", left_output_label + "2"])
                t.remove_all_dummy_indices(labels=[x for x in t.labels if x not in
                                                   [left_output_label + "1", left_output_label + "2"]])
                inter.insert(0, t)
        C.replace_label([a1.left_label, a2.left_label],
                        [left_output_label + "1", left_output_label + "2"])
        C.remove_all_dummy_indices()
    else:
        for i in range(start, end + 1):
            t = tsr.contract(a1[i], a2[i], rung_label, rung_label)
            if i == start:
                C = t
            else:
                C.contract(t, [a1.right_label, a2.right_label], [a1.left_label, a2.left_label])
            if return_intermediate_contractions:
                t = C.copy()
                t.replace_label([a1.right_label, a2.right_label, a1.left_label, a2.left_label],
                                [right_output_label + "1", right_output_label + "2",
                                 left_output_label + "1", left_output_label + "2"])
                t.remove_all_dummy_indices(labels=[x for x in t.labels if x not in
                                                   [right_output_label + "1", right_output_label + "2",
                                                    left_output_label + "1", left_output_label + "2"]])
                t.remove_all_dummy_indices()
                inter.append(t)
        C.replace_label([a1.right_label, a2.right_label, a1.left_label, a2.left_label],
                        [right_output_label + "1", right_output_label + "2",
                         left_output_label + "1", left_output_label + "2"])
        C.remove_all_dummy_indices()
    if return_intermediate_contractions:
        return inter
    return C


def inner_product_mps(mps_bra, mps_ket, complex_conjugate_bra=True, return_whole_tensor=False):
    """``onedim_core.py:1666-1683``: <bra|ket> via ``ladder_contract``;
    returns the 0-d device array (``t.data``) or the whole Tensor."""
    t = ladder_contract(mps_bra, mps_ket, mps_bra.phys_label, mps_ket.phys_label,
                        complex_conjugate_array1=complex_conjugate_bra)
    if return_whole_tensor:
        return t
    return t.data


def frob_distance_squared(mps1, mps2):
    """``onedim_core.py:1686-1688``"""
    ip = lambda a, b: _scalar(inner_product_mps(a, b))
    return (ip(mps1, mps1) + ip(mps2, mps2) - 2 * ip(mps1, mps2).real).real


def contract_mps_mpo(mps, mpo):
    """``onedim_core.py:1691-1708``: per site contract(mps[i], mpo[i], phys,
    physin) then ``consolidate_indices``.  When the site and MPO labels are
    the standard ones the two steps run as one fused kernel writing the
    consolidated (left, physout, right) layout; otherwise the generic
    contract + consolidate path is taken."""
    N = len(mps)
    new_mps = []
    for i in range(N):
        a, w = mps[i], mpo[i]
        Lb, Rb, P, PO, PI = (mps.left_label, mps.right_label, mps.phys_label,
                             mpo.physout_label, mpo.physin_label)
        fast = (len(a.labels) == 3 and set(a.labels) == {P, Lb, Rb}
                and len(w.labels) == 4 and set(w.labels) == {PO, PI, Lb, Rb}
                and mpo.left_label == Lb and mpo.right_label == Rb
                and PO not in (Lb, Rb) and sorted([Lb, PO, Rb]) == [Lb, PO, Rb])
        if fast:
            A = _ops.permute(a.data, [a.labels.index(mps.phys_label), a.labels.index(mps.left_label),
                                      a.labels.index(mps.right_label)])
            W = _ops.permute(w.data, [w.labels.index(mpo.physout_label), w.labels.index(mpo.physin_label),
                                      w.labels.index(mpo.left_label), w.labels.index(mpo.right_label)])
            out = _ops.mps_mpo_site(A, W, layout=0)
            t = tsr._new(out, [mps.left_label, mpo.physout_label, mps.right_label])
        else:
            t = tsr.contract(a, w, mps.phys_label, mpo.physin_label)
            t.consolidate_indices()
        new_mps.append(t)
    return MatrixProductState(new_mps, mps.left_label, mps.right_label, mpo.physout_label)
