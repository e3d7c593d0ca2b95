"""1-D tensor networks on the GPU: the drop-in for
tncontract/onedim/onedim_core.py (MPS / MPO containers, canonisation, SVD and
variational compression, gates, expectation values, the Γ-Λ canonical form
and its converters).

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

__all__ = ['MatrixProductState', 'MatrixProductStateCanonical', 'MatrixProductOperator',
           'OneDimensionalTensorNetwork', 'check_canonical_form_mps', 'contract_mps_mpo',
           'contract_multi_index_tensor_with_one_dim_array', 'contract_virtual_indices', 'frob_distance_squared',
           'inner_product_mps', 'ladder_contract', 'left_canonical_form_mps', 'mps_complex_conjugate',
           'reverse_mps', 'right_canonical_form_mps', 'canonical_form_mps', 'svd_compress_mps',
           'variational_compress_mps', 'tensor_to_mpo', 'tensor_to_mps', 'right_canonical_to_canonical',
           'left_canonical_to_canonical', 'canonical_to_right_canonical', 'canonical_to_left_canonical']


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

    def swap_gate(self, i, threshold=1e-15):
        """``onedim_core.py:95-127``: exchange every non-virtual leg of sites i
        and i+1 through one SVD of the merged pair (Shi, Duan & Vidal, PRA 74,
        022320): the new site i carries i+1's legs, sqrt(S) goes both ways."""
        virtual = (self.left_label, self.right_label)
        a_legs = [l for l in self[i].labels if l not in virtual]
        b_legs = [l for l in self[i + 1].labels if l not in virtual]
        self[i].prime_label(a_legs)
        pair = tsr.contract(self[i], self[i + 1], self.right_label, self.left_label)
        U, V, _ = tsr.truncated_svd(pair, [self.left_label] + b_legs, chi=0, threshold=threshold,
                                    absorb_singular_values='both')
        U.replace_label('svd_in', self.right_label)
        V.unprime_label(a_legs)
        V.replace_label('svd_out', self.left_label)
        self[i] = U
        self[i + 1] = V

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

    def variational_compress(self, chi, max_iter=10, initial_guess=None, tolerance=1e-15, normalise=False):
        """``onedim_core.py:486-631``: fit an MPS of bond ``chi`` (or of the
        bonds of ``initial_guess``) to ``self`` by alternating single-site
        updates (Schollwöck, Ann. Phys. 326 (2011) 96, sec. 4.5.2).

        Start: an SVD compression of a copy (``reverse=True``, so the start is
        left-canonical) or ``initial_guess`` itself, QR left-canonised.  A full
        update is a right-to-left sweep, then the mirrored sweep (both networks
        reversed); each site is the target contracted with the two
        environments, then LQ-split with L absorbed into the next site.
        Converged when successive site norms of the second sweep differ by
        less than ``tolerance`` (relative); ``RuntimeError`` after
        ``max_iter`` full updates.  Every contraction and LQ runs on the
        device; the convergence test reads one norm per site."""
        if initial_guess is None:
            approx = self.copy()
            approx.svd_compress(chi=chi, reverse=True)
        else:
            approx = initial_guess
            approx.left_canonise(qr_decomposition=True)
        approx.replace_labels([approx.left_label, approx.right_label, approx.phys_label],
                              [unique_label(), unique_label(), unique_label()])
        envs = ladder_contract(approx, self, approx.phys_label, self.phys_label,
                               return_intermediate_contractions=True, right_output_label=unique_label(),
                               complex_conjugate_array1=True)
        for it in range(max_iter):
            envs, _ = _variational_sweep(approx, self, envs)
            approx.reverse()
            self.reverse()
            envs, norms = _variational_sweep(approx, self, envs)
            approx.reverse()
            self.reverse()
            if np.all(np.abs(norms[1:] - norms[:-1]) / norms[1:] < tolerance):
                approx.replace_labels([approx.left_label, approx.right_label, approx.phys_label],
                                      [self.left_label, self.right_label, self.phys_label])
                if normalise is True:
                    approx[-1].data = _ops.scale(approx[-1].data, 1.0 / approx.norm(canonical_form="left"))
                return approx
            if it == max_iter - 1:
                raise RuntimeError("variational_compress did not converge.")

    def apply_gate(self, gate, firstsite, gate_outputs=None, gate_inputs=None, chi=None, threshold=1e-15,
                   canonise='left'):
        """``onedim_core.py:662-739``: contract sites ``firstsite`` ..
        ``firstsite + n - 1`` into one block, apply ``gate`` on their physical
        legs (the k-th input label on the k-th site) and split the block back
        into sites by truncated SVDs (``tensor_to_mps``), canonised towards
        the right end (``canonise='left'``) or the left end (``'right'``).
        As in the reference, the split uses the literal labels "left" and
        "right" for the block's virtual legs."""
        gate_outputs, gate_inputs = _gate_legs(gate, gate_outputs, gate_inputs)
        n = len(gate_inputs)
        block = contract_virtual_indices(self, firstsite, firstsite + n, periodic_boundaries=False)
        block = tsr.contract(block, gate, self.phys_label, gate_inputs)
        if canonise == 'right':
            split = tensor_to_mps(block, phys_labels=gate_outputs[::-1], mps_phys_label=self.phys_label,
                                  left_label='right', right_label='left', chi=chi, threshold=threshold)
            split.reverse()
        else:
            split = tensor_to_mps(block, phys_labels=gate_outputs, mps_phys_label=self.phys_label,
                                  left_label='left', right_label='right', chi=chi, threshold=threshold)
        self.data[firstsite:firstsite + n] = split.data

    def expval(self, gate, firstsite, left_canonised_up_to=0, right_canonised_up_to=-1,
               gate_outputs=None, gate_inputs=None):
        """``onedim_core.py:741-823``: <psi|gate|psi> on sites ``firstsite`` ..
        ``firstsite + n - 1`` after moving the orthogonality centre there
        (left-canonise from ``left_canonised_up_to``, right-canonise down to
        ``right_canonised_up_to``).  Returns the contracted Tensor."""
        gate_outputs, gate_inputs = _gate_legs(gate, gate_outputs, gate_inputs)
        n = len(gate_inputs)
        if right_canonised_up_to == -1:
            right_canonised_up_to = len(self)
        if left_canonised_up_to < firstsite:
            self.left_canonise(left_canonised_up_to, firstsite)
        if right_canonised_up_to > firstsite + n:
            self.right_canonise(firstsite + n, right_canonised_up_to)
        ket = contract_virtual_indices(self, firstsite, firstsite + n, periodic_boundaries=False)
        bra = ket.copy()
        bra.conjugate()
        out = tsr.contract(ket, gate, self.phys_label, gate_inputs)
        out = tsr.contract(bra, out, self.phys_label, gate_outputs)
        out.tr(self.left_label, self.left_label, index1=0, index2=1)
        out.tr(self.right_label, self.right_label, index1=0, index2=1)
        return out

    def ptrace(self, firstsite, lastsite=None, left_canonised_up_to=0, right_canonised_up_to=-1):
        """``onedim_core.py:825-877``: reduced density matrix of sites
        ``firstsite`` .. ``lastsite`` (orthogonality centre moved there as in
        ``expval``); physical legs at block axis j become ``phys_out<j>`` and
        ``phys_in<j>``."""
        if right_canonised_up_to == -1:
            right_canonised_up_to = self.nsites
        if lastsite is None:
            lastsite = firstsite
        if left_canonised_up_to < firstsite:
            self.left_canonise(left_canonised_up_to, firstsite)
        if right_canonised_up_to > lastsite:
            self.right_canonise(lastsite + 1, right_canonised_up_to)
        return _block_density(self, self.physical_site(firstsite), self.physical_site(lastsite) + 1)


def _gate_legs(gate, gate_outputs, gate_inputs):
    """Default output / input legs of a gate (``onedim_core.py:706-716``):
    first half / second half of its labels, or the complement of the list
    that is given."""
    if gate_outputs is None and gate_inputs is None:
        half = int(len(gate.labels) / 2)
        gate_outputs, gate_inputs = gate.labels[:half], gate.labels[half:]
    elif gate_outputs is None:
        gate_outputs = [x for x in gate.labels if x not in gate_inputs]
    elif gate_inputs is None:
        gate_inputs = [x for x in gate.labels if x not in gate_outputs]
    if len(gate_outputs) != len(gate_inputs):
        raise ValueError("len(gate_outputs) != len(gate_inputs)")
    return gate_outputs, gate_inputs


def _block_density(net, start, end):
    """rho = block . conj(block) over the block's outer virtual legs, the
    physical legs renamed by axis position (``onedim_core.py:868-877``)."""
    ket = contract_virtual_indices(net, start, end, periodic_boundaries=False)
    bra = ket.copy()
    bra.conjugate()
    for j, l in enumerate(ket.labels):
        if l == net.phys_label:
            ket.labels[j] = l + "_out" + str(j)
            bra.labels[j] = l + "_in" + str(j)
    return ket[net.left_label, net.right_label] * bra[net.left_label, net.right_label]


def _variational_sweep(approx, target, left_envs):
    """One right-to-left sweep of ``variational_compress``
    (``onedim_core.py:540-604``): returns the right environments (usable as
    left environments of the mirrored sweep) and the norm of the updated
    site after each step (the first entry: the last site before the sweep).

    ``left_envs[i]`` holds <approx|target> over sites 0..i with legs
    ``<base>1`` (approx) and ``<base>2`` (target)."""
    N = target.nsites
    le = left_envs[0].labels[0][:-1]
    re = unique_label()
    lq = unique_label()
    right_envs = []
    norms = [approx[-1].norm()]
    env = None
    for i in range(N - 1, 0, -1):
        site = tsr.contract(target[i], left_envs[i - 1], target.left_label, le + "2")
        if i != N - 1:
            site = tsr.contract(site, env, target.right_label, re + "2")
            site.replace_label(re + "1", approx.right_label)
        site.replace_label([le + "1", target.phys_label], [approx.left_label, approx.phys_label])
        L, Q = tsr.tensor_lq(site, approx.left_label, lq_label=lq)
        Q.replace_label(lq + "out", approx.left_label)
        L.replace_label(lq + "in", approx.right_label)
        approx[i] = Q
        approx[i - 1] = tsr.contract(approx[i - 1], L, approx.right_label, approx.left_label)
        norms.append(approx[i - 1].norm())
        # grow the right environment by site i
        if i == N - 1:
            env = tsr.contract(tsr.conjugate(approx[i]), target[i], approx.phys_label, target.phys_label)
            env.remove_all_dummy_indices(labels=[approx.right_label, target.right_label])
        else:
            env.contract(tsr.conjugate(approx[i]), re + "1", approx.right_label)
            env.contract(target[i], [approx.phys_label, re + "2"], [target.phys_label, target.right_label])
        env.replace_label([approx.left_label, target.left_label], [re + "1", re + "2"])
        right_envs.append(env.copy())
        if i == 1:
            first = tsr.contract(target[0], env, target.right_label, re + "2")
            first.replace_label([target.phys_label, re + "1"], [approx.phys_label, approx.right_label])
            approx[0] = first
    return right_envs, np.array(norms)


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


class MatrixProductStateCanonical(OneDimensionalTensorNetwork):
    """Vidal / Γ-Λ canonical form (``onedim_core.py:880-1327``): sites
    alternate Λ (diagonal singular-value matrix, even positions) and Γ
    (rank-3 site, odd positions), with 1x1 Λ at both ends; physical site n is
    position 2n+1.  The gate, swap and compression steps are local: merge
    Λ Γ Λ Γ Λ, SVD, restore Γ by the inverses of the outer Λ
    (Schollwöck, Ann. Phys. 326 (2011) 96, sec. 4.6)."""

    def __init__(self, tensors, left_label="left", right_label="right", phys_label="phys"):
        OneDimensionalTensorNetwork.__init__(self, tensors, left_label=left_label, right_label=right_label)
        self.phys_label = phys_label

    def __repr__(self):
        return ("MatrixProductStateCanonical(tensors=%r, left_label=%r,"
                "right_label=%r, phys_label=%r)" % (self.data, self.left_label, self.right_label,
                                                    self.phys_label))

    def __str__(self):
        return ("MatrixProductStateCanonical object: " + "sites (incl. singular value sites)= "
                + str(len(self)) + ", left_label = " + self.left_label + ", right_label = "
                + self.right_label + ", phys_label = " + self.phys_label)

    def copy(self):
        return MatrixProductStateCanonical([x.copy() for x in self], self.left_label, self.right_label,
                                           self.phys_label)

    def replace_labels(self, old_labels, new_labels):
        """``onedim_core.py:930-948``"""
        MatrixProductState.replace_labels(self, old_labels, new_labels)

    def standard_labels(self, suffix=""):
        self.replace_labels([self.left_label, self.right_label, self.phys_label],
                            ["left" + suffix, "right" + suffix, "phys" + suffix])

    def physical_site(self, n):
        return 2 * n + 1

    def singular_site(self, n):
        return 2 * n

    def physdim(self, site):
        return self.data[self.physical_site(site)].index_dimension(self.phys_label)

    def singulardim(self, site):
        return self.data[self.singular_site(site)].index_dimension(self.left_label)

    @property
    def nsites_physical(self):
        return int((self.nsites - 1) / 2)

    def norm(self, canonical_form=True):
        """``onedim_core.py:988-1002``: product of the two edge Λ norms, or
        sqrt(<psi|psi>) by the ladder when ``canonical_form`` is not True."""
        if canonical_form is True:
            return _ops.nrm2(self[-1].data) * _ops.nrm2(self[0].data)
        return float(np.sqrt(_scalar(inner_product_mps(self, self)).real))

    def check_canonical_form(self, threshold=1e-14, print_output=True):
        """``onedim_core.py:1004-1065``: Λ Γ must be left-isometric and Γ Λ
        right-isometric at every physical site; an edge site whose Gram
        matrix has a single entry above ``threshold`` counts as
        un-normalised rather than non-canonical."""
        not_left, not_right, not_normalised = [], [], []
        for side, bad in (("left", not_left), ("right", not_right)):
            for i in range(self.nsites_physical):
                p = self.physical_site(i)
                if side == "left":
                    A = self[p - 1][self.right_label, ] * self[p][self.left_label, ]
                    legs = [self.phys_label, self.left_label]
                else:
                    A = self[p][self.right_label, ] * self[p + 1][self.left_label, ]
                    legs = [self.phys_label, self.right_label]
                gram = tsr.contract(A, tsr.conjugate(A), legs, legs)
                if _identity_residual(gram.data) > threshold:
                    if i == 0 or i == self.nsites_physical - 1:
                        entries = np.abs(gram.to_numpy()).ravel()
                        if np.count_nonzero(entries > threshold) > 1:
                            bad.append(i)
                        else:
                            not_normalised.append(i)
                    else:
                        bad.append(i)
        if print_output:
            if len(not_left) == 0 and len(not_right) == 0:
                if len(not_normalised) == 0:
                    print("MPS in canonical form (normalised)")
                else:
                    print("MPS in canonical form (unnormalised)")
            else:
                print("Physical sites not left-canonical:")
                print(not_left)
                print("Physical sites not right-canonical:")
                print(not_right)
        return not_left, not_right, not_normalised

    def _outer_inverses(self, start, end):
        S1_inv = self[start].copy()
        S1_inv.inv()
        S2_inv = self[end].copy()
        S2_inv.inv()
        return S1_inv, S2_inv

    def _store_split(self, start, U, S, V, S1_inv, S2_inv):
        """Γ Λ Γ back from an SVD of the merged block: Γ_left = Λ1⁻¹ U,
        Λ = S, Γ_right = V Λ2⁻¹ (``onedim_core.py:1088-1095``)."""
        S.replace_label(["svd_out", "svd_in"], [self.left_label, self.right_label])
        self[start + 1] = S1_inv[self.right_label, ] * U[self.left_label, ]
        self[start + 2] = S
        self[start + 3] = V[self.right_label, ] * S2_inv[self.left_label, ]

    def compress_bond(self, singular_site, chi=None, threshold=1e-15):
        """``onedim_core.py:1067-1095``: truncate the Λ at
        ``singular_site(singular_site)`` by one SVD of its Λ Γ Λ Γ Λ block.
        The early return reads ``singulardim(2 * singular_site)`` (the
        reference maps the index twice)."""
        site = self.singular_site(singular_site)
        if self.singulardim(site) == 1:
            return
        start, end = site - 2, site + 2
        self[end - 1].prime_label(self.phys_label)
        block = contract_virtual_indices(self, start, end + 1, periodic_boundaries=False)
        S1_inv, S2_inv = self._outer_inverses(start, end)
        U, S, V = tsr.truncated_svd(block, [self.phys_label, self.left_label], chi=chi, threshold=threshold,
                                    absorb_singular_values=None)
        U.replace_label("svd_in", self.right_label)
        V.replace_label("svd_out", self.left_label)
        self._store_split(start, U, S, V, S1_inv, S2_inv)
        self[end - 1].unprime_label(self.phys_label)

    def compress_all(self, chi=None, threshold=1e-15, normalise=False):
        raise NotImplementedError

    def apply_gate(self, gate, firstsite, gate_outputs=None, gate_inputs=None, chi=None, threshold=1e-15):
        """``onedim_core.py:1100-1186``: one- or two-site gate on the Λ Γ (Λ Γ) Λ
        block; a two-site result is split by a truncated SVD (``chi``,
        ``threshold``) into Γ Λ Γ."""
        gate_outputs, gate_inputs = _gate_legs(gate, gate_outputs, gate_inputs)
        n = len(gate_inputs)
        if n > 2:
            raise NotImplementedError("gate acting on more than two sites.")
        start = self.physical_site(firstsite) - 1
        end = self.physical_site(firstsite + n - 1) + 1
        block = contract_virtual_indices(self, start, end + 1, periodic_boundaries=False)
        block = tsr.contract(block, gate, self.phys_label, gate_inputs)
        S1_inv, S2_inv = self._outer_inverses(start, end)
        if n == 1:
            block.replace_label([gate_outputs[0]], [self.phys_label])
            block = S1_inv[self.right_label, ] * block[self.left_label, ]
            self[start + 1] = block[self.right_label, ] * S2_inv[self.left_label, ]
        elif n == 2:
            U, S, V = tsr.truncated_svd(block, [gate_outputs[0], self.left_label], chi=chi,
                                        threshold=threshold, absorb_singular_values=None)
            U.replace_label(["svd_in", gate_outputs[0]], [self.right_label, self.phys_label])
            V.replace_label(["svd_out", gate_outputs[1]], [self.left_label, self.phys_label])
            self._store_split(start, U, S, V, S1_inv, S2_inv)

    def swap_gate(self, i, chi=None, threshold=1e-15):
        """``onedim_core.py:1188-1232``: swap the physical legs of physical
        sites i and i+1 through one SVD of their Λ Γ Λ Γ Λ block."""
        start = self.physical_site(i) - 1
        end = self.physical_site(i + 1) + 1
        self[start + 1].prime_label(self.phys_label)
        block = contract_virtual_indices(self, start, end + 1, periodic_boundaries=False)
        S1_inv, S2_inv = self._outer_inverses(start, end)
        U, S, V = tsr.truncated_svd(block, [self.left_label, self.phys_label], chi=chi, threshold=threshold,
                                    absorb_singular_values=None)
        V.unprime_label(self.phys_label)
        U.replace_label("svd_in", self.right_label)
        V.replace_label('svd_out', self.left_label)
        self._store_split(start, U, S, V, S1_inv, S2_inv)

    def expval(self, gate, firstsite, gate_outputs=None, gate_inputs=None):
        """``onedim_core.py:1234-1290``: <psi|gate|psi> from the Λ Γ .. Γ Λ
        block alone (canonical form assumed)."""
        gate_outputs, gate_inputs = _gate_legs(gate, gate_outputs, gate_inputs)
        start = self.physical_site(firstsite) - 1
        end = self.physical_site(firstsite + len(gate_inputs) - 1) + 1
        ket = contract_virtual_indices(self, start, end + 1, periodic_boundaries=False)
        bra = ket.copy()
        bra.conjugate()
        out = ket[self.phys_label, ] * gate[gate_inputs]
        out = bra[self.phys_label, ] * out[gate_outputs]
        out.tr(self.left_label, self.left_label, index1=0, index2=1)
        out.tr(self.right_label, self.right_label, index1=0, index2=1)
        return out

    def ptrace(self, firstsite, lastsite=None):
        """``onedim_core.py:1292-1327``: reduced density matrix of physical
        sites ``firstsite`` .. ``lastsite`` (canonical form assumed)."""
        if lastsite is None:
            lastsite = firstsite
        return _block_density(self, self.physical_site(firstsite) - 1, self.physical_site(lastsite) + 2)


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


def canonical_form_mps(orig_mps, chi=0, threshold=1e-14, normalise=False):
    """``onedim_core.py:1448-1454``: right-canonise a copy, then convert it
    to the Γ-Λ form."""
    mps = orig_mps.copy()
    mps.right_canonise(chi=chi, threshold=threshold, normalise=normalise)
    return right_canonical_to_canonical(mps, threshold=threshold)


def variational_compress_mps(mps, chi, max_iter=10, initial_guess=None, tolerance=1e-15):
    """``onedim_core.py:1476-1479``"""
    return mps.variational_compress(chi, max_iter=max_iter, initial_guess=initial_guess, tolerance=tolerance)


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


def tensor_to_mps(tensor, phys_labels=None, mps_phys_label='phys', left_label='left', right_label='right',
                  chi=0, threshold=1e-15):
    """``onedim_core.py:1711-1761``: split a tensor into a left-canonical MPS
    by successive truncated SVDs, peeling one physical leg (in the order of
    ``phys_labels``, by default every leg but ``left_label`` /
    ``right_label``) per site with S absorbed to the right."""
    if phys_labels is None:
        phys_labels = [x for x in tensor.labels if x not in [left_label, right_label]]
    rest = tensor.copy()
    sites = []
    for leg in phys_labels[:-1]:
        rows = ([left_label] if left_label in rest.labels else []) + [leg]
        U, rest, _ = tsr.truncated_svd(rest, rows, chi=chi, threshold=threshold, absorb_singular_values='right')
        U.replace_label('svd_in', right_label)
        U.replace_label(leg, mps_phys_label)
        sites.append(U)
        rest.replace_label('svd_out', left_label)
    rest.replace_label(phys_labels[-1], mps_phys_label)
    sites.append(rest)
    return MatrixProductState(sites, phys_label=mps_phys_label, left_label=left_label, right_label=right_label)


def tensor_to_mpo(tensor, physout_labels=None, physin_labels=None, mpo_physout_label='physout',
                  mpo_physin_label='physin', left_label='left', right_label='right', chi=0, threshold=1e-15):
    """``onedim_core.py:1764-1833``: split an operator tensor into an MPO by
    successive truncated SVDs, one (out, in) leg pair per site; by default
    the first half of the non-virtual legs are the outputs."""
    phys = [x for x in tensor.labels if x not in [left_label, right_label]]
    if physout_labels is None and physin_labels is None:
        physout_labels, physin_labels = phys[:int(len(phys) / 2)], phys[int(len(phys) / 2):]
    elif physout_labels is None:
        physout_labels = [x for x in phys if x not in physin_labels]
    elif physin_labels is None:
        physin_labels = [x for x in phys if x not in physout_labels]
    n = len(physin_labels)
    if len(physout_labels) != n:
        raise ValueError("len(physout_labels) != len(physin_labels)")
    rest = tensor.copy()
    sites = []
    for k in range(n - 1):
        rows = ([left_label] if left_label in rest.labels else []) + [physout_labels[k], physin_labels[k]]
        U, rest, _ = tsr.truncated_svd(rest, rows, chi=chi, threshold=threshold)
        U.replace_label('svd_in', right_label)
        U.replace_label(physout_labels[k], mpo_physout_label)
        U.replace_label(physin_labels[k], mpo_physin_label)
        sites.append(U)
        rest.replace_label('svd_out', left_label)
    rest.replace_label(physout_labels[n - 1], mpo_physout_label)
    rest.replace_label(physin_labels[n - 1], mpo_physin_label)
    sites.append(rest)
    return MatrixProductOperator(sites, physout_label=mpo_physout_label, physin_label=mpo_physin_label,
                                 left_label=left_label, right_label=right_label)


def right_canonical_to_canonical(mps, threshold=1e-14):
    """``onedim_core.py:1836-1884``: sweep left to right, SVD each site
    (rows: phys, left), keep singular values above ``threshold``
    (absolute), store Λ_prev and Γ = Λ_prev⁻¹ U, carry S Vᴴ into the next
    site; the last S (the norm) closes the chain.  Λ matrices hold the real
    singular values (as the reference's ``np.diag`` of them)."""
    L, R, P = mps.left_label, mps.right_label, mps.phys_label
    lam_prev = tsr.Tensor([[1.0]], labels=[L, R])
    lam_prev_inv = lam_prev.copy()
    B = mps[0]
    out = []
    svd_label = unique_label()
    for i in range(mps.nsites):
        U, s, V = tsr._svd_parts(B, [P, L], svd_label)
        k, _ = _ops.truncation_rank(s, 0, threshold, relative=False)
        lam = tsr._new(_ops.diag_matrix(s[:k].contiguous(), s.dtype), [L, R])
        U = tsr._new(_ops.slice_last(U.data, k), U.labels)
        V = tsr._new(V.data[0:k].contiguous(), V.labels)
        U.replace_label(svd_label + "in", R)
        V.replace_label(svd_label + "out", L)
        if i == mps.nsites - 1 and V.data.numel() == 1:
            # the last SVD has one column, so V is a 1x1 phase; LAPACK returns
            # 1 there (the reference drops V), this library's SVD may not:
            # keep the phase in the last Gamma so the state is unchanged
            v = V.data.reshape(()).item()
            U = tsr._new(_ops.scale(U.data, v), U.labels)
        out.append(lam_prev)
        out.append(lam_prev_inv[R, ] * U[L, ])
        if i == mps.nsites - 1:
            out.append(lam)  # 1x1: the norm of the state
        else:
            V = lam[R, ] * V[L, ]
            B = V[R, ] * mps[i + 1][L, ]
            lam_prev = lam.copy()
            lam_prev_inv = lam_prev.copy()
            lam_prev_inv.inv()
    return MatrixProductStateCanonical(out, left_label=L, right_label=R, phys_label=P)


def left_canonical_to_canonical(mps, threshold=1e-14):
    """``onedim_core.py:1887-1894``: the mirror of
    ``right_canonical_to_canonical`` through ``reverse``."""
    mpsc = right_canonical_to_canonical(reverse_mps(mps), threshold=threshold)
    mpsc.reverse()
    return mpsc


def canonical_to_right_canonical(mps):
    """``onedim_core.py:1897-1911``: B_i = Γ_i Λ_{i+1}; the edge Λ norms are
    folded into the first site."""
    N = mps.nsites_physical
    sites = [mps[mps.physical_site(i)][mps.right_label, ] * mps[mps.physical_site(i) + 1][mps.left_label, ]
             for i in range(N - 1)]
    sites.append(mps[mps.physical_site(N - 1)])
    sites[0].data = _ops.scale(sites[0].data, _ops.nrm2(mps[-1].data) * _ops.nrm2(mps[0].data))
    return MatrixProductState(sites, left_label=mps.left_label, right_label=mps.right_label,
                              phys_label=mps.phys_label)


def canonical_to_left_canonical(mps):
    """``onedim_core.py:1914-1928``: A_i = Λ_i Γ_i; the edge Λ norms are
    folded into the last site."""
    N = mps.nsites_physical
    sites = [mps[mps.physical_site(0)]]
    for i in range(1, N):
        sites.append(mps[mps.physical_site(i) - 1][mps.right_label, ] * mps[mps.physical_site(i)][mps.left_label, ])
    sites[-1].data = _ops.scale(sites[-1].data, _ops.nrm2(mps[-1].data) * _ops.nrm2(mps[0].data))
    return MatrixProductState(sites, left_label=mps.left_label, right_label=mps.right_label,
                              phys_label=mps.phys_label)
