"""Randomised cross-check of the drop-in's host logic against the reference
library itself (not collected by pytest: it needs the reference checkout).

    python tests/golden/fuzz_vs_reference.py /path/to/tncontract-checkout [trials]

The device ops run on the CPU stand-in of ``tests/host_fake.py``; the
reference runs on NumPy with the same inputs.  Checked: ``contract`` on
random label sets (repeated labels included), ``consolidate_indices``,
``move_index(es)``, the labels and shapes of ``tensor_svd / qr / lq`` and
``truncated_svd``; ``con`` on random networks (traces, multi-edges,
disconnected parts; same result or the same exception class); and random
sequences of MPS operations (canonisations, compressions, reverse, gates,
swaps, expectation values) compared by bond dimensions, labels, norm and
fidelity; the Gamma-Lambda form (Schmidt values, canonical check, gates,
expval, ptrace, converters); the chain helpers (frob_distance_squared,
contract_virtual_indices, ladder_contract, the multi-index contraction); and
PEPS inner products (exact and boundary MPS).  Truncation to chi / threshold is applied to generic spectra only:
on an already canonical state the singular values are degenerate and the
kept subspace is a gauge choice.
"""
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)
if not hasattr(np, "product"):
    np.product = np.prod
if not hasattr(np, "float"):
    np.float = float


def outcome(fn):
    try:
        return ("ok", fn())
    except Exception as e:  # noqa: BLE001 -- the class name is compared
        return ("err", type(e).__name__)


def same_tensor(r, g):
    a, b = np.asarray(r.data), g.to_numpy()
    return list(r.labels) == list(g.labels) and a.shape == b.shape and np.allclose(a, b, atol=1e-9)


def fuzz_tensor(R, G, trials, rng, nprng):
    bad = 0
    for _ in range(trials):
        l1 = [rng.choice("abcd") for _ in range(rng.randint(1, 4))]
        l2 = [rng.choice("abcde") for _ in range(rng.randint(1, 4))]
        dims = {l: rng.randint(1, 3) for l in "abcde"}
        A = nprng.standard_normal([dims[l] for l in l1])
        B = nprng.standard_normal([dims[l] for l in l2])
        ra, rb, ga, gb = R.Tensor(A, list(l1)), R.Tensor(B, list(l2)), G.Tensor(A, list(l1)), G.Tensor(B, list(l2))
        common = sorted({l for l in l1 if l in l2})
        if common:
            c = rng.sample(common, rng.randint(1, len(common)))
            o1, o2 = outcome(lambda: R.contract(ra, rb, c, c)), outcome(lambda: G.contract(ga, gb, c, c))
            bad += o1[0] != o2[0] or (o1[0] == "ok" and not same_tensor(o1[1], o2[1])) or \
                (o1[0] == "err" and o1[1] != o2[1])
        t1, t2 = ra.copy(), ga.copy()
        t1.consolidate_indices()
        t2.consolidate_indices()
        bad += not same_tensor(t1, t2)
        labs = rng.sample(sorted(set(l1)), rng.randint(1, len(set(l1))))
        pos, keep = rng.randint(0, len(l1) - 1), rng.choice([True, False])
        t1, t2 = ra.copy(), ga.copy()
        o1 = outcome(lambda: t1.move_indices(labs, pos, preserve_relative_order=keep))
        o2 = outcome(lambda: t2.move_indices(labs, pos, preserve_relative_order=keep))
        bad += o1[0] != o2[0] or (o1[0] == "ok" and not same_tensor(t1, t2))
        if len(set(l1)) == len(l1) >= 2:
            rows = rng.sample(l1, rng.randint(1, len(l1) - 1))
            for fn in ("tensor_svd", "tensor_qr", "tensor_lq"):
                for x, y in zip(getattr(R.tensor, fn)(ra, rows), getattr(G.tensor, fn)(ga, rows)):
                    bad += list(x.labels) != list(y.labels) or tuple(x.data.shape) != tuple(y.shape)
            for absorb in ("left", "right", "both", None):
                chi = rng.randint(0, 3)
                r = R.truncated_svd(ra, rows, chi=chi, absorb_singular_values=absorb)
                g = G.truncated_svd(ga, rows, chi=chi, absorb_singular_values=absorb)
                for x, y in zip(r[:2] if absorb else r, g[:2] if absorb else g):
                    bad += list(x.labels) != list(y.labels) or tuple(x.data.shape) != tuple(y.shape)
    return bad


def fuzz_con(R, G, trials, rng, nprng):
    bad = 0
    for _ in range(trials):
        labels = [["t%d_%d" % (i, j) for j in range(rng.randint(1, 4))] for i in range(rng.randint(1, 6))]
        slots = [(i, j) for i, ls in enumerate(labels) for j in range(len(ls))]
        rng.shuffle(slots)
        pairs, dims = [], {}
        for k in range(0, 2 * rng.randint(0, len(slots) // 2), 2):
            la, lb = labels[slots[k][0]][slots[k][1]], labels[slots[k + 1][0]][slots[k + 1][1]]
            dims[la] = dims[lb] = rng.randint(1, 3)
            pairs.append((la, lb))
        data = [nprng.standard_normal([dims.get(l, rng.randint(1, 3)) for l in ls]) for ls in labels]
        rt = [R.Tensor(d, list(ls)) for d, ls in zip(data, labels)]
        gt = [G.Tensor(d, list(ls)) for d, ls in zip(data, labels)]
        o1 = outcome(lambda: R.con(rt, pairs) if pairs else R.con(rt))
        o2 = outcome(lambda: G.con(gt, pairs) if pairs else G.con(gt))
        bad += o1[0] != o2[0] or (o1[0] == "err" and o1[1] != o2[1]) or \
            (o1[0] == "ok" and not same_tensor(o1[1], o2[1]))
    return bad


def fuzz_mps(R, G, trials, rng):
    import tn_oracle as O

    def sites(m, host):
        out = []
        for t in m:
            lab = list(t.labels)
            out.append(np.transpose(host(t), [lab.index(m.phys_label), lab.index(m.left_label),
                                              lab.index(m.right_label)]))
        return out

    def close(r, g):
        if r.bonddims() != g.bonddims() or [list(t.labels) for t in r] != [list(t.labels) for t in g]:
            return False
        a, b = sites(r, lambda t: np.asarray(t.data)), sites(g, lambda t: t.to_numpy())
        try:
            na, nb = O.mps_norm(a), O.mps_norm(b)
        except (ValueError, TypeError):      # the network does not chain (e.g. a gate after reverse)
            return [x.shape for x in a] == [x.shape for x in b]
        return abs(na - nb) <= 1e-9 * max(na, 1e-300) and (na < 1e-12 or 1 - O.fidelity(a, b) < 1e-9)

    bad = 0
    for trial in range(trials):
        N, d, chi = rng.randint(2, 7), rng.randint(2, 3), rng.randint(1, 5)
        dt = np.complex128 if rng.random() < 0.5 else np.float64
        s = O.random_mps(trial, N, d, chi, dt, normalise=rng.random() < 0.5)
        rm = R.onedim.MatrixProductState([R.Tensor(a, ["phys", "left", "right"]) for a in s])
        gm = G.onedim.MatrixProductState([G.Tensor(a, ["phys", "left", "right"]) for a in s])
        for step in range(4):
            op = rng.choice(["lc", "rc", "svdc", "svdcn", "rev", "gate", "swap", "lcqr", "expval"])
            c, thr = (rng.choice([None, 1, 2, 3]), rng.choice([1e-14, 1e-2, 0.3])) if step == 0 else (None, 1e-14)
            i = rng.randint(0, N - 2)
            gate = np.random.default_rng(trial * 10 + step).standard_normal((d, d, d, d))
            can = rng.choice(["left", "right"])
            fns = {"lc": lambda m, T: m.left_canonise(chi=c, threshold=thr),
                   "rc": lambda m, T: m.right_canonise(chi=c, threshold=thr),
                   "svdc": lambda m, T: m.svd_compress(chi=c, threshold=thr),
                   "svdcn": lambda m, T: m.svd_compress(chi=c, normalise=True),
                   "rev": lambda m, T: m.reverse(),
                   "swap": lambda m, T: m.swap_gate(i),
                   "lcqr": lambda m, T: m.left_canonise(qr_decomposition=True),
                   "gate": lambda m, T: m.apply_gate(T(gate, ["o1", "o2", "i1", "i2"]), i, chi=c, canonise=can),
                   "expval": lambda m, T: m.expval(T(gate, ["o1", "o2", "i1", "i2"]), i)}
            o1, o2 = outcome(lambda: fns[op](rm, R.Tensor)), outcome(lambda: fns[op](gm, G.Tensor))
            if o1[0] != o2[0]:
                bad += 1
                break
            if o1[0] == "err":
                break
            if op == "expval":
                v1, v2 = complex(np.asarray(o1[1].data)), complex(o2[1].to_numpy())
                bad += abs(v1 - v2) > 1e-9 * max(1.0, abs(v1))
            if not close(rm, gm):
                bad += 1
                break
    return bad


def fuzz_canonical(R, G, trials, rng):
    """Gamma-Lambda form: canonical_form_mps (Schmidt values, canonical-form
    check, norm), a two-site gate on it, expval / ptrace, and the converters
    back to left / right canonical form (same state)."""
    import tn_oracle as O

    def lam(net, host):
        return [np.sort(np.abs(np.diag(host(net[2 * i]))))[::-1] for i in range(net.nsites_physical + 1)]

    def sites(m, host):
        out = []
        for t in m:
            lab = list(t.labels)
            out.append(np.transpose(host(t), [lab.index(m.phys_label), lab.index(m.left_label),
                                              lab.index(m.right_label)]))
        return out

    rh, gh = (lambda t: np.asarray(t.data)), (lambda t: t.to_numpy())
    bad = 0
    for trial in range(trials):
        N, d, chi = rng.randint(2, 6), rng.randint(2, 3), rng.randint(1, 4)
        dt = np.complex128 if rng.random() < 0.5 else np.float64
        s = O.random_mps(1000 + trial, N, d, chi, dt, normalise=rng.random() < 0.5)
        rc = R.onedim.onedim_core.canonical_form_mps(
            R.onedim.MatrixProductState([R.Tensor(a, ["phys", "left", "right"]) for a in s]))
        gc = G.onedim.canonical_form_mps(G.onedim.MatrixProductState([G.Tensor(a, ["phys", "left", "right"])
                                                                      for a in s]))
        if rc.bonddims() != gc.bonddims():
            bad += 1
            continue
        bad += any(not np.allclose(a, b, rtol=1e-8, atol=1e-12) for a, b in zip(lam(rc, rh), lam(gc, gh)))
        c1 = rc.check_canonical_form(threshold=1e-10, print_output=False)
        c2 = gc.check_canonical_form(threshold=1e-10, print_output=False)
        bad += [list(x) for x in c1] != [list(x) for x in c2]
        i = rng.randint(0, N - 2)
        gate = np.random.default_rng(trial).standard_normal((d, d, d, d))
        e1 = complex(np.asarray(rc.expval(R.Tensor(gate, ["o1", "o2", "i1", "i2"]), i).data))
        e2 = complex(gc.expval(G.Tensor(gate, ["o1", "o2", "i1", "i2"]), i).to_numpy())
        bad += abs(e1 - e2) > 1e-8 * max(1.0, abs(e1))
        p1, p2 = rc.ptrace(i), gc.ptrace(i)
        bad += list(p1.labels) != list(p2.labels) or not np.allclose(np.asarray(p1.data), p2.to_numpy(), atol=1e-9)
        rc.apply_gate(R.Tensor(gate, ["o1", "o2", "i1", "i2"]), i)
        gc.apply_gate(G.Tensor(gate, ["o1", "o2", "i1", "i2"]), i)
        for conv in ("canonical_to_left_canonical", "canonical_to_right_canonical"):
            a = sites(getattr(R.onedim, conv)(rc.copy()), rh)
            b = sites(getattr(G.onedim, conv)(gc.copy()), gh)
            na, nb = O.mps_norm(a), O.mps_norm(b)
            bad += abs(na - nb) > 1e-8 * max(na, 1e-300) or (na > 1e-12 and 1 - O.fidelity(a, b) > 1e-8)
    return bad


def fuzz_chain_helpers(R, G, trials, rng, nprng):
    """frob_distance_squared, contract_virtual_indices (open and periodic:
    the periodic trace can pair legs of different lengths, which np.trace
    accepts), ladder_contract over every start / end / option, and
    contract_multi_index_tensor_with_one_dim_array."""
    import tn_oracle as O
    bad = 0
    for trial in range(trials):
        N, chi = rng.randint(2, 5), rng.randint(1, 3)
        s1 = O.random_mps(2000 + trial, N, 2, chi, np.complex128)
        s2 = O.random_mps(3000 + trial, N, 2, chi + 1, np.complex128)
        mk = lambda M, s: M.onedim.MatrixProductState([M.Tensor(a, ["phys", "left", "right"]) for a in s])
        r1, r2, g1, g2 = mk(R, s1), mk(R, s2), mk(G, s1), mk(G, s2)
        v1, v2 = complex(R.onedim.frob_distance_squared(r1, r2)), complex(G.onedim.frob_distance_squared(g1, g2))
        bad += abs(v1 - v2) > 1e-8 * max(1.0, abs(v1))
        st = rng.randint(0, N - 1)
        en, per = rng.randint(st + 1, N), rng.choice([True, False])
        o1 = outcome(lambda: R.onedim.contract_virtual_indices(r1, st, en, periodic_boundaries=per))
        o2 = outcome(lambda: G.onedim.contract_virtual_indices(g1, st, en, periodic_boundaries=per))
        bad += o1[0] != o2[0] or (o1[0] == "ok" and not same_tensor(o1[1], o2[1]))
        st = rng.randint(0, N - 1)
        kw = dict(start=st, end=rng.randint(st, N - 1), complex_conjugate_array1=rng.choice([True, False]),
                  return_intermediate_contractions=rng.choice([True, False]))
        o1 = outcome(lambda: R.onedim.ladder_contract(r1, r2, "phys", "phys", **kw))
        o2 = outcome(lambda: G.onedim.ladder_contract(g1, g2, "phys", "phys", **kw))
        if o1[0] != o2[0]:
            bad += 1
        elif o1[0] == "ok":
            a = o1[1] if kw["return_intermediate_contractions"] else [o1[1]]
            b = o2[1] if kw["return_intermediate_contractions"] else [o2[1]]
            bad += len(a) != len(b) or any(not same_tensor(x, y) for x, y in zip(a, b))
        T = nprng.standard_normal([2] * N)
        o1 = outcome(lambda: R.onedim.contract_multi_index_tensor_with_one_dim_array(
            R.Tensor(T, ["p"] * N), r1, "p", "phys"))
        o2 = outcome(lambda: G.onedim.contract_multi_index_tensor_with_one_dim_array(
            G.Tensor(T, ["p"] * N), g1, "p", "phys"))
        bad += o1[0] != o2[0] or (o1[0] == "ok" and not same_tensor(o1[1], o2[1]))
    return bad


def fuzz_peps(R, G, trials, rng, nprng):
    """inner_product_peps on random small lattices: exact and boundary-MPS
    contraction at chi 2 and 4."""
    def val(x):
        if hasattr(x, "to_numpy"):
            return complex(x.to_numpy().reshape(()))
        if hasattr(x, "data"):
            return complex(np.asarray(x.data).reshape(()))
        return complex(x)

    bad = 0
    for trial in range(trials):
        L, M, D, d = rng.randint(2, 4), rng.randint(2, 4), rng.randint(1, 2), 2
        rows = [[nprng.random((d, 1 if r == 0 else D, 1 if c == M - 1 else D, 1 if r == L - 1 else D,
                               1 if c == 0 else D)) for c in range(M)] for r in range(L)]
        legs = ["phys", "up", "right", "down", "left"]
        rp = R.twodim.SquareLatticePEPS([[R.Tensor(a, legs) for a in r] for r in rows])
        gp = G.twodim.SquareLatticePEPS([[G.Tensor(a, legs) for a in r] for r in rows])
        for kw in ({"exact_contract": True}, {"exact_contract": False, "chi": 4},
                   {"exact_contract": False, "chi": 2}):
            o1 = outcome(lambda: R.twodim.inner_product_peps(rp, rp, **kw))
            o2 = outcome(lambda: G.twodim.inner_product_peps(gp, gp, **kw))
            bad += o1[0] != o2[0] or (o1[0] == "ok" and abs(val(o1[1]) - val(o2[1])) > 1e-8 * abs(val(o1[1])))
    return bad


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    trials = int(sys.argv[2]) if len(sys.argv) > 2 else 200
    sys.path.insert(0, ref)
    import tncontract as R
    import tncontract_gb300 as G
    from host_fake import cpu_ops
    rng, nprng = random.Random(0), np.random.default_rng(0)
    with cpu_ops():
        res = {"tensor": fuzz_tensor(R, G, trials, rng, nprng), "con": fuzz_con(R, G, trials, rng, nprng),
               "mps": fuzz_mps(R, G, max(trials // 2, 1), rng),
               "canonical": fuzz_canonical(R, G, max(trials // 3, 1), rng),
               "chain_helpers": fuzz_chain_helpers(R, G, max(trials // 2, 1), rng, nprng),
               "peps": fuzz_peps(R, G, max(trials // 10, 1), rng, nprng)}
    print("mismatches:", res)
    return 1 if any(res.values()) else 0


if __name__ == "__main__":
    sys.exit(main())
