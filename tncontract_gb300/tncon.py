"""Network contraction ``con``: the drop-in for tncontract/tncon.py.

The reference contracts a network in argument order (``tncon.py:68-158``:
argument flattening, uniqueness checks, grouping of multi-edge pairs,
traces first, pairwise contractions in the order the pairs are given, then
the tensor product of the disconnected components).  That control flow is
restated here once, over an executor: the device executor runs it, and a
label-only executor replays it on the host to find the reference's output
label order.

By default the pairwise contractions are instead ordered by cost: traces
first, then repeatedly the connected pair of tensors whose contraction
needs the fewest multiply-adds (ties: the smaller result), all edges between
the two contracted in one call; the result is permuted to the reference's
label order.  Values equal the argument-order ones up to floating-point
summation order.  ``order="argument"`` runs the reference's order itself, and
so does the default where the reference's result is not the network's
contraction: a repeated label inside one tensor, or a pair order for which
its component bookkeeping (``tncon.py:151-158``) keeps a merged tensor twice
(e.g. pairs A-B, C-D, B-C of a chain return A·B·C·D times D) -- the drop-in
returns what the reference returns.  Every step is a device ``contract`` /
``trace`` / permute.
"""
from __future__ import annotations

import numpy as np

from . import _ops
from . import tensor as tn


def _split_args(args):
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
    return tensor_list, contract_list


def _index_lookup(all_labels, contract_list):
    """Uniqueness checks and label -> tensor map (``tncon.py:85-100``)."""
    contracted = [item for pair in contract_list for item in pair]
    if len(set(contracted)) != len(contracted):
        raise ValueError("Index found in more than one contraction pair.")
    index_lookup = {}
    for i, labels in enumerate(all_labels):
        for lab in labels:
            if lab in index_lookup.keys():
                raise ValueError("Index label " + lab + " found in two tensors." +
                                 " Tensors must have unique index labelling.")
            index_lookup[lab] = i
    return index_lookup


def _group_pairs(contract_list, index_lookup):
    """Internal pairs and pairwise groups, several edges between the same two
    tensors merged into one group (``tncon.py:102-125``; the reference looks
    a repeated pair up unsorted, ``:110-111``)."""
    internal_contract = []
    pairwise_contract = []
    tensor_pairs = []
    for c in contract_list:
        if index_lookup[c[0]] == index_lookup[c[1]]:
            internal_contract.append(c)
        else:
            key = tuple(np.sort((index_lookup[c[0]], index_lookup[c[1]])))
            if key in tensor_pairs:
                idx = tensor_pairs.index((index_lookup[c[0]], index_lookup[c[1]]))
                if not isinstance(pairwise_contract[idx][0], list):
                    pairwise_contract[idx][0] = [pairwise_contract[idx][0]]
                    pairwise_contract[idx][1] = [pairwise_contract[idx][1]]
                pairwise_contract[idx][0].append(c[0])
                pairwise_contract[idx][1].append(c[1])
            else:
                pairwise_contract.append(list(c))
                tensor_pairs.append(key)
    return internal_contract, pairwise_contract


class _Device:
    """Executor over device Tensors."""

    @staticmethod
    def labels(t):
        return t.labels

    @staticmethod
    def trace(t, a, b):
        t.trace(a, b)
        return t

    @staticmethod
    def contract(t1, t2, l1, l2):
        return tn.contract(t1, t2, l1, l2)

    @staticmethod
    def product(ts):
        return tn.tensor_product(*ts)


class _ListTrace(Exception):
    """The argument order would trace a multi-edge group (two tensors already
    merged by earlier pairs); that case runs the argument order itself."""


class _Labels:
    """Executor over label lists only (unique labels): the reference's label
    order of a trace, a contraction and a tensor product."""

    @staticmethod
    def labels(t):
        return t

    @staticmethod
    def trace(t, a, b):
        if isinstance(a, list):
            raise _ListTrace()
        return [x for x in t if x not in (a, b)]

    @staticmethod
    def contract(t1, t2, l1, l2):
        l1 = l1 if isinstance(l1, list) else [l1]
        l2 = l2 if isinstance(l2, list) else [l2]
        return [x for x in t1 if x not in l1] + [x for x in t2 if x not in l2]

    @staticmethod
    def product(ts):
        return [x for t in ts for x in t]


def _argument_order(ex, tensors, internal_contract, pairwise_contract, index_lookup):
    """Traces, then the pairwise groups in argument order, then the tensor
    product of the components (``tncon.py:127-158``)."""
    tensors = list(tensors)
    index_lookup = dict(index_lookup)
    for c in internal_contract:
        i = index_lookup[c[0]]
        tensors[i] = ex.trace(tensors[i], c[0], c[1])
    connected_component = [i for i in range(len(tensors))]
    for c in pairwise_contract:
        if isinstance(c[0], list):
            d, e = index_lookup[c[0][0]], index_lookup[c[1][0]]
        else:
            d, e = index_lookup[c[0]], index_lookup[c[1]]
        if d == e:
            tensors[d] = ex.trace(tensors[d], c[0], c[1])
        else:
            if d < e:
                tensors[d] = ex.contract(tensors[d], tensors[e], c[0], c[1])
                connected_component[e] = d
            else:
                tensors[e] = ex.contract(tensors[e], tensors[d], c[1], c[0])
                connected_component[d] = e
            for lab in ex.labels(tensors[min(d, e)]):
                index_lookup[lab] = min(d, e)
    return ex.product([tensors[connected_component.index(x)] for x in set(connected_component)])


def _greedy_plan(shapes, labels, partner):
    """Order of pairwise contractions by cost on shapes alone.

    ``shapes[i]`` / ``labels[i]``: dims and labels of node i (after traces);
    ``partner``: label -> the label it contracts with.  Returns the merge list
    [(i, j, labels of i, labels of j)] (node j is absorbed into node i) and
    the multiply-adds it needs."""
    dims = {}
    for sh, lb in zip(shapes, labels):
        for d, l in zip(sh, lb):
            dims[l] = int(d)
    nodes = {i: list(lb) for i, lb in enumerate(labels)}
    owner = {l: i for i, lb in nodes.items() for l in lb}
    partner = dict(partner)
    steps = []
    total = 0
    while True:
        best = None
        for i in sorted(nodes):
            for j in sorted({owner[partner[l]] for l in nodes[i] if l in partner}):
                if j <= i:
                    continue
                la = [l for l in nodes[i] if l in partner and owner[partner[l]] == j]
                shared = int(np.prod([dims[l] for l in la], dtype=np.float64))
                size_i = int(np.prod([dims[l] for l in nodes[i]], dtype=np.float64))
                size_j = int(np.prod([dims[l] for l in nodes[j]], dtype=np.float64))
                cost = size_i * size_j // max(shared, 1)
                out = cost // max(shared, 1)
                key = (cost, out, i, j)
                if best is None or key < best[0]:
                    best = (key, i, j, la)
        if best is None:
            break
        (cost, _, _, _), i, j, la = best
        lb = [partner[l] for l in la]
        steps.append((i, j, la, lb))
        total += cost
        nodes[i] = [l for l in nodes[i] if l not in la] + [l for l in nodes[j] if l not in lb]
        del nodes[j]
        for l in nodes[i]:
            owner[l] = i
        for l in la + lb:
            partner.pop(l, None)
    return steps, total


def plan_waves(steps):
    """Group a merge list [(i, j, ...)] (node j absorbed into node i) into
    waves of independent merges: a merge goes one wave after the last merge
    that wrote either of its nodes, so the merges of a wave touch disjoint
    nodes and can run together (one grouped GEMM launch).  Order inside a
    wave and of the waves follows the plan."""
    level = {}
    waves = []
    for st in steps:
        i, j = st[0], st[1]
        w = max(level.get(i, -1), level.get(j, -1)) + 1
        level[i] = w
        level[j] = w
        if w == len(waves):
            waves.append([])
        waves[w].append(st)
    return waves


def _argument_cost(shapes, labels, internal_contract, pairwise_contract, index_lookup):
    """Multiply-adds of the reference's argument order (for comparison)."""
    dims = {}
    for sh, lb in zip(shapes, labels):
        for d, l in zip(sh, lb):
            dims[l] = int(d)
    total = [0]

    class _Count(_Labels):
        @staticmethod
        def contract(t1, t2, l1, l2):
            l1 = l1 if isinstance(l1, list) else [l1]
            total[0] += int(np.prod([dims[l] for l in t1 + t2], dtype=np.float64)) // max(
                int(np.prod([dims[l] for l in l1], dtype=np.float64)), 1)
            return _Labels.contract(t1, t2, l1, l2)

    _argument_order(_Count, labels, internal_contract, pairwise_contract, index_lookup)
    return total[0]


def _traced_labels(labels, internal_contract, index_lookup):
    out = [list(l) for l in labels]
    for c in internal_contract:
        i = index_lookup[c[0]]
        out[i] = _Labels.trace(out[i], c[0], c[1])
    return out


def plan_costs(*args):
    """(argument-order, cost-order) multiply-adds of ``con(*args)``: the
    estimate both plans are chosen by, computed on the host without
    contracting anything."""
    tensor_list, contract_list = _split_args(args)
    labels = [list(t.labels) for t in tensor_list]
    shapes = [tuple(t.shape) for t in tensor_list]
    index_lookup = _index_lookup(labels, contract_list)
    internal, pairwise = _group_pairs(contract_list, index_lookup)
    try:
        arg = _argument_cost(shapes, labels, internal, pairwise, index_lookup)
    except _ListTrace:
        arg = None
    traced = _traced_labels(labels, internal, index_lookup)
    tshapes = [[dict(zip(lb, sh))[l] for l in tl] for sh, lb, tl in zip(shapes, labels, traced)]
    partner = {}
    for c in contract_list:
        if index_lookup[c[0]] != index_lookup[c[1]]:
            partner[c[0]], partner[c[1]] = c[1], c[0]
    _, greedy = _greedy_plan(tshapes, traced, partner)
    return arg, greedy


def con(*args, order="cost"):
    """Contract a network given tensors and label pairs (``tncon.py:4-159``).

    Arguments are Tensors, lists of Tensors, label pairs ``(a, b)`` or lists
    of pairs.  Labels must be unique across the network.  ``order``:
    ``"cost"`` (default) contracts the cheapest connected pair first and
    returns the reference's label order; ``"argument"`` follows the order of
    the pairs as the reference does."""
    if order not in ("cost", "argument"):
        raise ValueError("order must be 'cost' or 'argument'")
    tensor_list, contract_list = _split_args(args)
    tensor_list = [t.copy() for t in tensor_list]
    all_labels = [t.labels for t in tensor_list]
    index_lookup = _index_lookup(all_labels, contract_list)
    internal, pairwise = _group_pairs(contract_list, index_lookup)
    repeated = any(len(set(l)) != len(l) for l in all_labels)
    if order == "argument" or repeated or len(tensor_list) < 3:
        return _argument_order(_Device, tensor_list, internal, pairwise, index_lookup)

    try:
        ref_labels = _argument_order(_Labels, [list(l) for l in all_labels], internal, pairwise, index_lookup)
    except _ListTrace:
        return _argument_order(_Device, tensor_list, internal, pairwise, index_lookup)
    contracted = {l for c in contract_list for l in c}
    free = [l for labels in all_labels for l in labels if l not in contracted]
    if sorted(ref_labels) != sorted(free):
        # the argument order's component bookkeeping (tncon.py:151-158) does
        # not follow merges of merged tensors, so some orders return a
        # component twice; reproduce the reference's result exactly
        return _argument_order(_Device, tensor_list, internal, pairwise, index_lookup)
    for c in internal:
        i = index_lookup[c[0]]
        tensor_list[i].trace(c[0], c[1])
    partner = {}
    for c in contract_list:
        if index_lookup[c[0]] != index_lookup[c[1]]:
            partner[c[0]], partner[c[1]] = c[1], c[0]
    steps, _ = _greedy_plan([t.shape for t in tensor_list], [list(t.labels) for t in tensor_list], partner)
    nodes = {i: t for i, t in enumerate(tensor_list)}
    for wave in plan_waves(steps):
        results = tn.contract_many([(nodes[i], nodes[j], la, lb) for i, j, la, lb in wave])
        for (i, j, _la, _lb), r in zip(wave, results):
            nodes[i] = r
            del nodes[j]
    result = tn.tensor_product(*[nodes[i] for i in sorted(nodes)])
    if result.labels != ref_labels:
        perm = [result.labels.index(l) for l in ref_labels]
        result = tn._new(_ops.permute(result.data, perm), list(ref_labels))
    return result
