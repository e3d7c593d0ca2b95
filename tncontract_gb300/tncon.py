"""Network contraction ``con``: the drop-in for tncontract/tncon.py.

The plan (argument flattening, uniqueness checks, grouping of multi-edge
pairs, traces first, pairwise contractions in argument order, tensor product
of the disconnected components) is host logic restated from
``tncon.py:68-158``; each step is a device ``contract`` / ``trace``.
"""
from __future__ import annotations

import numpy as np

from . import tensor as tn


def con(*args):
    """Contract a network given tensors and label pairs (``tncon.py:4-159``).

    Arguments are Tensors, lists of Tensors, label pairs ``(a, b)`` or lists
    of pairs.  Labels must be unique across the network."""
    tensor_list = []
    contract_list = []
    for x in args:
        if isinstance(x, list):
            if isinstance(x[0], tn.Tensor):
                tensor_list.extend(x)
            else:
                contract_list.extend(x)
        elif isinstance(x, tn.Tensor):
            tensor_list.append(x)
        else:
            contract_list.append(x)

    tensor_list = [t.copy() for t in tensor_list]
    all_tensor_indices = [t.labels for t in tensor_list]

    contracted = [item for pair in contract_list for item in pair]
    if len(set(contracted)) != len(contracted):
        raise ValueError("Index found in more than one contraction pair.")

    index_lookup = {}
    for i, labels in enumerate(all_tensor_indices):
        for lab in labels:
            if lab in index_lookup.keys():
                raise ValueError("Index label " + lab + " found in two tensors." +
                                 " Tensors must have unique index labelling.")
            index_lookup[lab] = i

    internal_contract = []
    pairwise_contract = []
    tensor_pairs = []
    for c in contract_list:
        if index_lookup[c[0]] == index_lookup[c[1]]:
            internal_contract.append(c)
        else:
            key = tuple(np.sort((index_lookup[c[0]], index_lookup[c[1]])))
            if key in tensor_pairs:
                # several edges between the same two tensors: one contraction
                # (the reference looks the pair up unsorted, tncon.py:110-111)
                idx = tensor_pairs.index((index_lookup[c[0]], index_lookup[c[1]]))
                if not isinstance(pairwise_contract[idx][0], list):
                    pairwise_contract[idx][0] = [pairwise_contract[idx][0]]
                    pairwise_contract[idx][1] = [pairwise_contract[idx][1]]
                pairwise_contract[idx][0].append(c[0])
                pairwise_contract[idx][1].append(c[1])
            else:
                pairwise_contract.append(list(c))
                tensor_pairs.append(key)

    for c in internal_contract:
        tensor_list[index_lookup[c[0]]].trace(c[0], c[1])

    connected_component = [i for i in range(len(tensor_list))]
    for c in pairwise_contract:
        if isinstance(c[0], list):
            d = index_lookup[c[0][0]]
            e = index_lookup[c[1][0]]
        else:
            d = index_lookup[c[0]]
            e = index_lookup[c[1]]
        if d == e:
            tensor_list[d].trace(c[0], c[1])
        else:
            if d < e:
                tensor_list[d] = tn.contract(tensor_list[d], tensor_list[e], c[0], c[1])
                connected_component[e] = d
            else:
                tensor_list[e] = tn.contract(tensor_list[e], tensor_list[d], c[1], c[0])
                connected_component[d] = e
            for lab in tensor_list[min(d, e)].labels:
                index_lookup[lab] = min(d, e)

    return tn.tensor_product(*[tensor_list[connected_component.index(x)]
                               for x in set(connected_component)])
