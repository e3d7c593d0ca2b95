"""``con`` with the cost-ordered plan against the reference's argument order
(host logic, CPU stand-in for the device ops): same labels, same values up
to summation order, never a costlier plan on networks where the argument
order is poor.  The argument order itself is pinned to the reference's
fixtures by the label-case tests."""
import numpy as np
import pytest

import api_cases as K
from host_fake import cpu_ops


def test_con_fixture_networks_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_con_cases(tn)


def _t(tn, rng, shape, labels, cplx=False):
    a = rng.standard_normal(shape)
    if cplx:
        a = a + 1j * rng.standard_normal(shape)
    return tn.Tensor(a, labels)


def _networks(tn, rng):
    # a chain given in an order whose first pair is an outer product of the ends
    A = _t(tn, rng, (2, 30), ["a0", "a1"])
    B = _t(tn, rng, (30, 30), ["b0", "b1"])
    C = _t(tn, rng, (30, 30), ["c0", "c1"])
    D = _t(tn, rng, (30, 2), ["d0", "d1"])
    yield "chain", [D, A, B, C, [("d1", "a0"), ("a1", "b0"), ("b1", "c0"), ("c1", "d0")]]
    # a ring with a multi-edge, a trace and a dangling vector (disconnected)
    P = _t(tn, rng, (3, 4, 5, 5), ["p0", "p1", "p2", "p3"], cplx=True)
    Q = _t(tn, rng, (4, 6, 3), ["q0", "q1", "q2"], cplx=True)
    R = _t(tn, rng, (6, 7), ["r0", "r1"])
    S = _t(tn, rng, (7, 2), ["s0", "s1"])
    V = _t(tn, rng, (9,), ["v0"])
    yield "ring", [[P, Q, R, S], V, ("p2", "p3"), ("p1", "q0"), ("q1", "r0"), ("r1", "s0"), ("p0", "q2")]
    # star: a hub contracted with leaves, full contraction to a scalar
    H = _t(tn, rng, (3, 4, 5), ["h0", "h1", "h2"])
    L = [_t(tn, rng, (n,), ["l%d" % i]) for i, n in enumerate((3, 4, 5))]
    yield "star", [H, L, [("h0", "l0"), ("h1", "l1"), ("h2", "l2")]]
    # a 2x3 grid (PEPS-like, open legs kept)
    G = {}
    for r in range(2):
        for c in range(3):
            G[r, c] = _t(tn, rng, (2, 1 if r == 0 else 3, 3 if r == 0 else 1, 1 if c == 0 else 3,
                                   3 if c < 2 else 1), ["g%d%d%s" % (r, c, x) for x in "pudlr"])
    pairs = [("g%d%dr" % (r, c), "g%d%dl" % (r, c + 1)) for r in range(2) for c in range(2)]
    pairs += [("g0%dd" % c, "g1%du" % c) for c in range(3)]
    yield "grid", [[G[k] for k in sorted(G)], pairs]


def test_con_cost_order_matches_argument_order():
    import tncontract_gb300 as tn
    rng = np.random.default_rng(3)
    with cpu_ops():
        for name, args in _networks(tn, rng):
            ref = tn.con(*args, order="argument")
            got = tn.con(*args)
            assert got.labels == ref.labels, name
            a, b = got.to_numpy(), ref.to_numpy()
            assert a.shape == b.shape, name
            assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1e-300), name


def test_con_plan_cost_never_worse():
    import tncontract_gb300 as tn
    from tncontract_gb300 import tncon
    rng = np.random.default_rng(4)
    with cpu_ops():
        costs = {name: tncon.plan_costs(*args) for name, args in _networks(tn, rng)}
    for name, (arg, greedy) in costs.items():
        assert greedy <= arg, (name, arg, greedy)
    # the chain's argument order starts with the 30 x 30 outer product D.A
    arg, greedy = costs["chain"]
    assert greedy * 2 < arg


def test_con_order_argument_validation():
    import tncontract_gb300 as tn
    rng = np.random.default_rng(5)
    with cpu_ops():
        A = _t(tn, rng, (2, 2), ["x", "y"])
        B = _t(tn, rng, (2, 2), ["z", "w"])
        with pytest.raises(ValueError):
            tn.con(A, B, ("y", "z"), order="fastest")
        with pytest.raises(ValueError):
            tn.con(A, B, ("y", "z"), ("y", "w"))


def test_con_waves_of_independent_pairs():
    """The cost-ordered plan of the reference's 2x3 grid network (breadth-first pair order) has a wave
    of two or more independent merges (one grouped GEMM launch on the
    device); waves touch disjoint nodes and keep every merge once; the values
    stay the reference's (CPU stand-in)."""
    import tncontract_gb300 as tn
    from tncontract_gb300 import tncon
    with cpu_ops():
        tensors, pairs, want, want_labels = K.con_fixture_network(tn, "grid_2x3_bfs")
    waves = K.con_waves(tn, tensors, pairs)
    assert max(len(w) for w in waves) >= 2
    for w in waves:
        touched = [n for st in w for n in st[:2]]
        assert len(touched) == len(set(touched))
    assert sum(len(w) for w in waves) == len(tensors) - 1
    # a chain whose two end pairs are independent: [[A.B, C.D], [AB.CD]]
    steps = [(0, 1, ["a"], ["b"]), (2, 3, ["c"], ["d"]), (0, 2, ["x"], ["y"])]
    assert [[s[:2] for s in w] for w in tncon.plan_waves(steps)] == [[(0, 1), (2, 3)], [(0, 2)]]
    with cpu_ops():
        r = tn.con(tensors, pairs)
    assert r.labels == want_labels and K.close(r.to_numpy(), want, 1e-12)
