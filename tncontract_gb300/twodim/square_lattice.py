"""2-D square-lattice networks on the GPU: the drop-in for
tncontract/twodim/square_lattice.py (boundary-MPS contraction path).

``mps_contract`` follows ``square_lattice.py:130-203`` column by column:
apply the column MPO (``contract_mps_mpo``), ``svd_compress_mps`` to
``chi``, divide by the norm and accumulate it in ``np.longdouble``; the last
column is closed with ``inner_product_mps``.  All tensor work runs on the
device; only the running norm (a host scalar) is kept in extended precision,
which is what lets the ~1e115 value of an 8x8 norm network survive FP32-class
storage.
"""
from __future__ import annotations

import numpy as np

from .. import _ops
from .. import onedim as od
from .. import tensor as tn

__all__ = ['SquareLatticeTensorNetwork', 'SquareLatticePEPS', 'SquareLatticePEPO',
           'inner_product_peps', 'outer_product_peps', 'column_to_mpo', 'apply_pepo_to_peps']


def _objarray2(rows):
    nr, nc = len(rows), len(rows[0])
    arr = np.empty((nr, nc), dtype=object)
    for i in range(nr):
        for j in range(nc):
            arr[i, j] = rows[i][j]
    return arr


class SquareLatticeTensorNetwork():
    """``square_lattice.py:13-214``: 2-D array of tensors with up/right/down/
    left legs; missing boundary legs become dummy legs of dimension 1."""

    def __init__(self, tensors, up_label="up", right_label="right",
                 down_label="down", left_label="left", copy_data=True):
        self.up_label = up_label
        self.right_label = right_label
        self.down_label = down_label
        self.left_label = left_label
        rows = [[(x.copy() if copy_data else x) for x in row] for row in tensors]
        self.data = _objarray2(rows)
        for _, x in np.ndenumerate(self.data):
            if left_label not in x.labels:
                x.add_dummy_index(left_label)
            if right_label not in x.labels:
                x.add_dummy_index(right_label)
            if up_label not in x.labels:
                x.add_dummy_index(up_label)
            if down_label not in x.labels:
                x.add_dummy_index(down_label)

    def __iter__(self):
        return self.data.__iter__()

    def __len__(self):
        return self.data.__len__()

    def __getitem__(self, key):
        return self.data.__getitem__(key)

    def __setitem__(self, key, value):
        self.data.__setitem__(key, value)

    def copy(self):
        return SquareLatticeTensorNetwork(self.data, up_label=self.up_label,
                                          right_label=self.right_label, down_label=self.down_label,
                                          left_label=self.left_label, copy_data=True)

    @property
    def shape(self):
        return self.data.shape

    def is_left_right_periodic(self):
        for x in self[:, 0]:
            if x.index_dimension(self.left_label) > 1:
                return True
        return False

    def can_contract(self):
        """``square_lattice.py:87-110``"""
        rows, cols = self.data.shape
        left_unmatched, up_unmatched = [], []
        for i in range(1, rows):
            for j in range(1, cols):
                if self[i, j].index_dimension(self.up_label) != self[i - 1, j].index_dimension(self.down_label):
                    left_unmatched.append((i, j))
                if self[i, j].index_dimension(self.left_label) != self[i, j - 1].index_dimension(self.right_label):
                    up_unmatched.append((i, j))
        if not left_unmatched and not up_unmatched:
            return True
        print("Unmatched bonds found between the following sites:")
        for k in left_unmatched:
            print("(" + str(k[0] - 1) + ", " + str(k[1]) + ")" + " and " + str(k))
        for k in up_unmatched:
            print("(" + str(k[0]) + ", " + str(k[1] - 1) + ")" + " and " + str(k))
        return False

    def exact_contract(self, until_column=-1):
        """``square_lattice.py:112-128``: exact column-by-column contraction
        (exponential cost; for small networks)."""
        rows, cols = self.data.shape
        mpo = column_to_mpo(self, 0)
        C = od.contract_virtual_indices(mpo)
        for i in range(1, cols):
            if i == until_column + 1:
                return C
            mpo = column_to_mpo(self, i)
            C = od.contract_multi_index_tensor_with_one_dim_array(C, mpo, self.right_label, self.left_label)
            C.remove_all_dummy_indices([self.left_label, self.up_label, self.down_label])
        return C

    def mps_contract(self, chi, compression_type="svd", until_column=-1,
                     max_iter=10, tolerance=1e-14, return_all_columns=False):
        """``square_lattice.py:130-203``: boundary-MPS contraction from the
        left, each column's MPS compressed by ``svd_compress_mps`` (the norm
        divided out of the first site) or ``variational_compress`` (out of the
        last site).  The running norm is a host ``np.longdouble`` as in the
        reference."""
        if compression_type not in ("svd", "variational"):
            raise ValueError("compression_type must be 'svd' or 'variational'")
        nrows, ncols = self.shape
        column_list = [] if return_all_columns else None
        norm = np.longdouble(1)
        compressed_mps = None
        for col in range(ncols - 1):
            if col == 0:
                mps_to_compress = column_to_mpo(self, 0)
            else:
                column_mpo = column_to_mpo(self, col)
                mps_to_compress = od.contract_mps_mpo(compressed_mps, column_mpo)
            if compression_type == "svd":
                compressed_mps = od.svd_compress_mps(mps_to_compress, chi, normalise=False,
                                                     threshold=tolerance)
                mps_norm = compressed_mps.norm(canonical_form="right")
                if mps_norm == 0.0:
                    return 0.0
                compressed_mps[0].data = _ops.scale(compressed_mps[0].data, 1.0 / mps_norm)
            else:
                compressed_mps = mps_to_compress.variational_compress(chi, max_iter=max_iter,
                                                                      tolerance=tolerance)
                mps_norm = compressed_mps.norm(canonical_form="left")
                if mps_norm == 0.0:
                    return 0.0
                compressed_mps[-1].data = _ops.scale(compressed_mps[-1].data, 1.0 / mps_norm)
            norm *= mps_norm
            if return_all_columns:
                mps_copy = compressed_mps.copy()
                mps_copy[0].data = _ops.scale(mps_copy[0].data, float(norm))
                column_list.append(mps_copy)
            if col == until_column:
                if return_all_columns:
                    return column_list
                compressed_mps.norm_factor = norm  # longdouble kept on the host
                site = 0 if compression_type == "svd" else -1
                compressed_mps[site].data = _ops.scale(compressed_mps[site].data, float(norm))
                return compressed_mps
        final_column_mps = column_to_mpo(self, ncols - 1)
        full = od.inner_product_mps(compressed_mps, final_column_mps,
                                    return_whole_tensor=True, complex_conjugate_bra=False)
        val = full.data.item()
        if isinstance(val, complex):
            result = val * complex(norm)
        else:
            result = np.longdouble(val) * norm
        if return_all_columns:
            column_list.append(result)
            return column_list
        return result

    def col_to_1D_array(self, col):
        new_data = [x.copy() for x in self[:, col]]
        return od.OneDimensionalTensorNetwork(new_data, left_label=self.up_label,
                                              right_label=self.down_label)

    def fliplr(self):
        """``square_lattice.py:217-229``"""
        mirror = self.copy()
        mirror.data = np.fliplr(mirror.data)
        mirror.right_label = self.left_label
        mirror.left_label = self.right_label
        return mirror


class SquareLatticePEPS(SquareLatticeTensorNetwork):
    """``square_lattice.py:232-281``"""

    def __init__(self, tensors, up_label="up", right_label="right", down_label="down",
                 left_label="left", phys_label="phys", copy_data=True):
        SquareLatticeTensorNetwork.__init__(self, tensors, up_label, right_label, down_label,
                                            left_label, copy_data=copy_data)
        self.phys_label = phys_label

    def copy(self):
        return SquareLatticePEPS(self.data, up_label=self.up_label, right_label=self.right_label,
                                 down_label=self.down_label, left_label=self.left_label,
                                 phys_label=self.phys_label, copy_data=True)

    def outer_product(self, physin_label="physin", physout_label="physout"):
        """``square_lattice.py:251-278``"""
        rows = []
        for r in range(self.shape[0]):
            new_row = []
            for c in range(self.shape[1]):
                outer = tn.contract(self[r, c], self[r, c], [], [])
                outer.labels[outer.labels.index(self.phys_label)] = physin_label
                outer.labels[outer.labels.index(self.phys_label)] = physout_label
                outer.consolidate_indices(labels=[self.left_label, self.right_label,
                                                  self.up_label, self.down_label])
                new_row.append(outer)
            rows.append(new_row)
        return SquareLatticePEPO(rows, up_label=self.up_label, down_label=self.down_label,
                                 right_label=self.right_label, left_label=self.left_label,
                                 physin_label=physin_label, physout_label=physout_label)

    density_operator = outer_product


def inner_product_peps(peps_ket, peps_bra, exact_contract="True", complex_conjugate_bra=True,
                       compression_type="svd", chi=2, max_iter=10, tolerance=1e-14,
                       contract_virtual=True):
    """``square_lattice.py:283-304``: double-layer network conj(bra)·ket over
    phys, consolidated, then exact or boundary-MPS contraction."""
    rows = []
    for i in range(peps_ket.shape[0]):
        new_row = []
        for j in range(peps_ket.shape[1]):
            t = (tn.conjugate(peps_bra[i, j])["phys"] * peps_ket[i, j]["phys"])
            t.consolidate_indices()
            new_row.append(t)
        rows.append(new_row)
    ip = SquareLatticeTensorNetwork(rows)
    if not contract_virtual:
        return ip
    if exact_contract:
        return ip.exact_contract()
    return ip.mps_contract(chi, compression_type=compression_type, max_iter=max_iter,
                           tolerance=tolerance)


def outer_product_peps(peps1, peps2, physin_label="physin", physout_label="physout"):
    """``square_lattice.py:306-342``"""
    if peps1.shape != peps2.shape:
        raise ValueError("Peps input do not have same dimension.")
    rows = []
    for r in range(peps1.shape[0]):
        new_row = []
        for c in range(peps1.shape[1]):
            outer = tn.contract(peps1[r, c], tn.conjugate(peps2[r, c]), [], [])
            outer.labels[outer.labels.index(peps1.phys_label)] = physout_label
            outer.labels[outer.labels.index(peps2.phys_label)] = physin_label
            outer.consolidate_indices(labels=[peps1.left_label, peps1.right_label,
                                              peps1.up_label, peps1.down_label])
            new_row.append(outer)
        rows.append(new_row)
    return SquareLatticePEPO(rows, up_label=peps1.up_label, down_label=peps1.down_label,
                             right_label=peps1.right_label, left_label=peps1.left_label,
                             physin_label=physin_label, physout_label=physout_label)


class SquareLatticePEPO(SquareLatticeTensorNetwork):
    """``square_lattice.py:345-375``"""

    def __init__(self, tensors, up_label="up", right_label="right", down_label="down",
                 left_label="left", physin_label="physin", physout_label="physout", copy_data=True):
        SquareLatticeTensorNetwork.__init__(self, tensors, up_label, right_label, down_label,
                                            left_label, copy_data=copy_data)
        self.physin_label = physin_label
        self.physout_label = physout_label

    def copy(self):
        return SquareLatticePEPO(self.data, up_label=self.up_label, right_label=self.right_label,
                                 down_label=self.down_label, left_label=self.left_label,
                                 physin_label=self.physin_label, physout_label=self.physout_label,
                                 copy_data=True)

    def trace(self):
        rows = []
        for i in range(self.shape[0]):
            row = []
            for j in range(self.shape[1]):
                tmp = self[i, j].copy()
                tmp.trace(self.physin_label, self.physout_label)
                row.append(tmp)
            rows.append(row)
        return SquareLatticeTensorNetwork(rows, up_label=self.up_label, down_label=self.down_label,
                                          right_label=self.right_label, left_label=self.left_label)


def apply_pepo_to_peps(peps, pepo):
    """``square_lattice.py:377-392``"""
    nrows, ncols = peps.shape
    rows = []
    for i in range(nrows):
        new_row = []
        for j in range(ncols):
            t = peps[i, j][peps.phys_label] * pepo[i, j][pepo.physin_label]
            t.replace_label(pepo.physout_label, peps.phys_label)
            t.consolidate_indices()
            new_row.append(t)
        rows.append(new_row)
    return SquareLatticePEPS(rows, up_label=peps.up_label, right_label=peps.right_label,
                             down_label=peps.down_label, left_label=peps.left_label,
                             phys_label=peps.phys_label)


def column_to_mpo(square_tn, col):
    """``square_lattice.py:394-417``: first/last column -> MPS, others -> MPO."""
    new_data = [x.copy() for x in square_tn[:, col]]
    if col == 0 or col == square_tn.shape[1] - 1:
        if col == 0:
            new_mps = od.MatrixProductState(new_data, square_tn.up_label, square_tn.down_label,
                                            square_tn.right_label)
            for x in new_mps.data:
                x.remove_all_dummy_indices(square_tn.left_label)
        else:
            new_mps = od.MatrixProductState(new_data, square_tn.up_label, square_tn.down_label,
                                            square_tn.left_label)
            for x in new_mps.data:
                x.remove_all_dummy_indices(square_tn.right_label)
        return new_mps
    return od.MatrixProductOperator(new_data, square_tn.up_label, square_tn.down_label,
                                    square_tn.right_label, square_tn.left_label)
