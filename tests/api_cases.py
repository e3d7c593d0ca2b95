"""Drop-in API checks against fixtures generated by the reference itself
(tests/golden/gen_golden.py).  Shared by the CPU host-logic tests (with the
test-only CPU stand-in for the device ops) and the GPU tests (real kernels).
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = json.load(open(os.path.join(GOLDEN, name + ".json")))
    return g, m


def unpack(g, prefix):
    return [g["%s_%d" % (prefix, i)] for i in range(int(g[prefix + "_n"]))]


def close(a, b, rtol):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(b), 1e-300)


def sites_of(mps):
    out = []
    for t in mps:
        lab = t.labels
        out.append(np.transpose(t.to_numpy(), [lab.index(mps.phys_label), lab.index(mps.left_label),
                                                lab.index(mps.right_label)]))
    return out


def check_label_cases(tn, rtol=1e-13):
    g, m = load("labels_and_fixture")
    A = tn.Tensor(g["lc_A"], labels=["spam", "eggs"])
    B = tn.Tensor(g["lc_B"])
    C = tn.contract(A, B, "spam", "i2")
    assert C.labels == m["lc_C_labels"] and close(C.to_numpy(), g["lc_C"], rtol)
    D = tn.contract(A, B, ["spam", "eggs"], ["i0", "i2"])
    assert D.labels == m["lc_D_labels"] and close(D.to_numpy(), g["lc_D"], rtol)
    E = A["spam", "eggs"] * B["i0", "i2"]
    assert E.labels == m["lc_E_labels"] and close(E.to_numpy(), g["lc_E"], rtol)
    T1 = tn.Tensor(g["lc_T1"], labels=["a", "b", "a", "c"])
    T2 = tn.Tensor(g["lc_T2"], labels=["x", "y", "x"])
    F = tn.contract(T1, T2, "a", "x")
    assert F.labels == m["lc_F_labels"] and close(F.to_numpy(), g["lc_F"], rtol)
    G = tn.contract(T1, T2, "a", "x", index_slice1=[-1], index_slice2=[0])
    assert G.labels == m["lc_G_labels"] and close(G.to_numpy(), g["lc_G"], rtol)
    H = tn.Tensor(g["lc_H"], labels=["z", "b", "z", "a"])
    H.consolidate_indices()
    assert H.labels == m["lc_Hc_labels"] and close(H.to_numpy(), g["lc_Hc"], rtol)
    P = tn.tensor_product(A, tn.Tensor(g["lc_P"].reshape(2, 2, 3)[0, 0] * 0 + 1, labels=["q"]))
    assert P.labels == m["lc_P_labels"]
    R = tn.Tensor(g["lc_R"], labels=["left", "right"])
    ring = tn.con([R.suf(str(i)) for i in range(5)],
                  [("right" + str(j), "left" + str(j + 1)) for j in range(4)], ("right4", "left0"))
    assert ring.labels == m["lc_ring_labels"] and close(ring.to_numpy(), g["lc_ring"], rtol)
    X = tn.Tensor(g["lc_X"], labels=["x1", "x2", "x3"])
    Y = tn.Tensor(g["lc_Y"], labels=["y1", "y2", "y3"])
    Z = tn.Tensor(g["lc_Z"], labels=["z1", "z2", "z3"])
    W = tn.Tensor(g["lc_W"], labels=["w1"])
    K = tn.con(X, Y, Z, W, ("x2", "y1"), ("x3", "y2"), ("z1", "z2"), ("x1", "z3"))
    assert K.labels == m["lc_K_labels"] and close(K.to_numpy(), g["lc_K"], rtol)


def check_factorisation_labels(tn, rtol=1e-12):
    g, m = load("labels_and_fixture")
    S0 = tn.Tensor(g["lc_S0"], labels=["i0", "i1", "i2"])
    U, S, V = tn.tensor_svd(S0, ["i0", "i2"])
    assert [U.labels, S.labels, V.labels] == m["svd_labels"]
    assert [list(U.shape), list(S.shape), list(V.shape)] == m["svd_shapes"]
    assert close(np.diag(S.to_numpy()), g["svd_s"], rtol)
    # recombination (tensor.py:889-894 docstring)
    b = tn.contract(U, tn.contract(S, V, "svd_in", "svd_out"), "svd_in", "svd_out")
    assert tn.distance(S0, b) < 1e-10
    U2, V2, tr = tn.truncated_svd(S0, ["i0", "i2"], chi=2)
    assert [U2.labels, V2.labels] == m["tsvd_labels"]
    assert [list(U2.shape), list(V2.shape)] == m["tsvd_shapes"]
    assert close(tr.cpu().numpy(), g["tsvd_trunc"], rtol)
    U3, V3, tr3 = tn.truncated_svd(S0, ["i0", "i2"], chi=0, threshold=0.3, absolute=False,
                                   absorb_singular_values="both")
    assert [list(U3.shape), list(V3.shape)] == m["tsvd_rel_shapes"]
    assert close(tr3.cpu().numpy(), g["tsvd_rel_trunc"], rtol)
    Q, R = tn.tensor_qr(S0, ["i0", "i2"])
    assert [Q.labels, R.labels] == m["qr_labels"]
    assert [list(Q.shape), list(R.shape)] == m["qr_shapes"]
    assert tn.distance(tn.contract(Q, R, "qr_in", "qr_out"), S0) < 1e-10
    L, Q2 = tn.tensor_lq(S0, ["i0", "i2"])
    assert [L.labels, Q2.labels] == m["lq_labels"]
    assert [list(L.shape), list(Q2.shape)] == m["lq_shapes"]


def check_contract_errors(tn):
    import pytest
    A = tn.Tensor(np.ones((2, 3)), labels=["a", "b"])
    B = tn.Tensor(np.ones((3, 4)), labels=["c", "d"])
    with pytest.raises(ValueError, match="Number of indices in contraction does not match"):
        tn.contract(A, B, ["a", "b"], "c")
    with pytest.raises(ValueError, match="a with dim=2 does not match c with dim=3"):
        tn.contract(A, B, "a", "c")
    with pytest.raises(ValueError, match="Labels do not match shape of data"):
        tn.Tensor(np.ones((2, 3)), labels=["a"])


def check_fixture_mps(tn, rtol=1e-10):
    """The reference's own test MPS and what its tests pin
    (tncontract/tests/test_canonical_form_mps_conversion.py:31-80)."""
    g, m = load("labels_and_fixture")
    sites = unpack(g, "fx_site")
    psi = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    assert abs(psi.norm() - float(g["fx_norm"])) < rtol
    a = psi.copy()
    a.svd_compress(threshold=1e-12, normalise=False)
    assert abs(a.norm() - float(g["fx_c_norm"])) < rtol
    assert a.bonddims() == m["fx_c_bonds"]
    assert [t.labels for t in a] == m["fx_c_labels"]
    import tn_oracle as O
    spec = O.bond_spectra(sites_of(a))
    for s, s_ref in zip(spec, unpack(g, "fx_c_spectra")):
        assert close(s, s_ref, 1e-9)
    b = psi.copy()
    b.svd_compress(threshold=1e-12, normalise=True)
    assert abs(b.norm() - 1.0) < rtol
    # right-canonical after svd_compress: first site not right-canonised is 0
    assert b.check_canonical_form(threshold=1e-10, print_output=False)[1] == 0
    c = psi.copy()
    c.left_canonise()
    assert c.bonddims() == m["fx_lc_bonds"]
    assert list(c.check_canonical_form(threshold=1e-10, print_output=False)) == m["fx_lc_canon"]
    ip = complex(np.asarray(tn.onedim.inner_product_mps(psi, c).cpu()).reshape(()))
    assert abs(ip - complex(g["fx_ip"])) < rtol


def check_config1(tn, fid_tol=1e-10):
    import tn_oracle as O
    g, m = load("config1")
    sites = O.random_mps(0, 32, 2, 32, np.float64)
    mps = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    lc = tn.onedim.left_canonical_form_mps(mps)
    comp = lc.copy()
    comp.svd_compress(chi=16)
    assert lc.bonddims() == m["c1_lc_bonds"]
    assert comp.bonddims() == m["c1_c_bonds"]
    assert [t.labels for t in comp][:3] == m["c1_c_labels"]
    assert abs(comp.norm() - float(g["c1_norm_c"])) < 1e-9 * float(g["c1_norm_c"])
    cs = sites_of(comp)
    f = O.fidelity(sites, cs)
    assert abs(f - float(g["c1_fid_vs_input"])) < fid_tol
    for s, s_ref in zip(O.bond_spectra(cs), unpack(g, "c1_c_spectra")):
        assert close(s, s_ref, 1e-8)


def check_config2_small(tn, fid_tol=1e-10):
    import tn_oracle as O
    g, m = load("config2_small")
    N, chi = 12, 16
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    psi = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    W = tn.onedim.MatrixProductOperator([tn.Tensor(w, ["physout", "physin", "left", "right"]) for w in mpo])
    phi = tn.onedim.contract_mps_mpo(psi, W)
    assert list(phi[1].labels) == m["c2s_phi_labels"] and list(phi[1].shape) == m["c2s_phi_shape"]
    assert phi.phys_label == m["c2s_phi_phys"]
    assert close(phi[1].to_numpy(), g["c2s_phi_site1"], 1e-13)
    mm = phi.copy()
    mm.svd_compress(chi=chi)
    assert mm.bonddims() == m["c2s_m_bonds"]
    assert [t.labels for t in mm][:3] == m["c2s_m_labels"]
    ms = sites_of(mm)
    ref = O.svd_compress_method(sites_of(phi), chi)
    assert 1 - O.fidelity(ref, ms) < fid_tol
    assert abs(O.mps_norm(ms) - float(np.real(g["c2s_norm_m"]))) < 1e-10
    for s, s_ref in zip(O.bond_spectra(ms), unpack(g, "c2s_m_spectra")):
        assert close(s, s_ref, 1e-8)
    f = tn.onedim.svd_compress_mps(phi, chi)
    assert f.bonddims() == m["c2s_f_bonds"]
    fs = sites_of(f)
    assert abs(O.fidelity(fs, ms) - float(np.real(g["c2s_fid_f_m"]))) < fid_tol


def _mps_sites(net, phys=None):
    """(phys, left, right) arrays of an MPS-like network's sites."""
    phys = phys or net.phys_label
    out = []
    for t in net:
        lab = t.labels
        out.append(np.transpose(t.to_numpy(), [lab.index(phys), lab.index(net.left_label),
                                                lab.index(net.right_label)]))
    return out


def _same_state(ref_sites, got_sites, tol):
    """The two site lists describe the same state: fidelity and norm."""
    import tn_oracle as O
    nr, ng = O.mps_norm(ref_sites), O.mps_norm(got_sites)
    assert abs(nr - ng) <= tol * nr, (nr, ng)
    assert 1.0 - O.fidelity(ref_sites, got_sites) < tol


def _lambdas(net):
    return [np.diag(net[2 * i].to_numpy()) for i in range(net.nsites_physical + 1)]


def _full_tensor(net, legs):
    """Contract an open MPO / MPS chain on the host into one array with the
    given per-site leg groups (e.g. [["physout", "physin"]] * n)."""
    acc = None
    out_legs = []
    for t, group in zip(net, legs):
        lab = list(t.labels)
        a = np.transpose(t.to_numpy(), [lab.index(net.left_label)] + [lab.index(x) for x in group]
                         + [lab.index(net.right_label)])
        acc = a if acc is None else np.tensordot(acc, a, axes=([acc.ndim - 1], [0]))
        out_legs += group
    return acc.reshape(acc.shape[1:-1])


def check_onedim_extras(tn, tol=1e-10):
    """Gates, expectation values, reduced density matrices, variational
    compression, the Gamma-Lambda canonical form, tensor -> MPS / MPO and the
    onedim_utils constructors against the reference's fixtures.  States are
    compared gauge-invariantly (fidelity, norm, Schmidt values, density
    matrices, expectation values); constructor outputs exactly."""
    g, m = load("onedim_extras")
    oc = tn.onedim
    sites6 = unpack(g, "x_psi")

    def mps_of(sites):
        return oc.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])

    g2 = tn.Tensor(g["x_G2"], ["o1", "o2", "i1", "i2"])
    g3 = tn.Tensor(g["x_G3"], ["o1", "o2", "o3", "i1", "i2", "i3"])
    op1 = tn.Tensor(g["x_op1"], ["o", "i"])
    # swap_gate
    a = mps_of(sites6)
    a.swap_gate(2)
    assert a.bonddims() == m["x_swap_bonds"] and [t.labels for t in a] == m["x_swap_labels"]
    _same_state(unpack(g, "x_swap"), _mps_sites(a), tol)
    # apply_gate
    for tag, gate, first, kw in [("x_ag2l", g2, 2, {}), ("x_ag2r", g2, 2, {"canonise": "right"}),
                                 ("x_ag3c", g3, 1, {"chi": 3})]:
        b = mps_of(sites6)
        b.apply_gate(gate, first, **kw)
        assert b.bonddims() == m[tag + "_bonds"], tag
        assert [t.labels for t in b] == m[tag + "_labels"], tag
        _same_state(unpack(g, tag), _mps_sites(b), tol)
    # expval, ptrace
    e = mps_of(sites6)
    val = complex(e.expval(g2, 2).to_numpy().reshape(()))
    assert abs(val - complex(g["x_expval"])) <= tol * max(abs(complex(g["x_expval"])), 1.0)
    assert e.bonddims() == m["x_expval_bonds"]
    f = mps_of(sites6)
    rho = f.ptrace(1, 2)
    assert rho.labels == m["x_ptrace_labels"] and close(rho.to_numpy(), g["x_ptrace"], tol)
    # variational compression (iterative: looser bound)
    p8 = mps_of(unpack(g, "x_psi8"))
    v = p8.variational_compress(4, max_iter=20, tolerance=1e-8)
    assert v.bonddims() == m["x_var_bonds"] and [t.labels for t in v] == m["x_var_labels"]
    _same_state(unpack(g, "x_var"), _mps_sites(v), 1e-7)
    v2 = oc.variational_compress_mps(mps_of(unpack(g, "x_psi8")), 3, max_iter=40, tolerance=1e-6)
    _same_state(unpack(g, "x_var3"), _mps_sites(v2), 1e-5)
    # canonical form
    pc = oc.canonical_form_mps(mps_of(sites6))
    assert [list(x) for x in pc.check_canonical_form(threshold=1e-10, print_output=False)] == m["x_can_check"]
    assert pc.bonddims() == m["x_can_bonds"]
    assert abs(pc.norm() - float(g["x_can_norm"])) <= tol
    for lam, ref in zip(_lambdas(pc), unpack(g, "x_can_lam")):
        assert close(lam, ref, tol)
    val = complex(pc.expval(g2, 1).to_numpy().reshape(()))
    assert abs(val - complex(g["x_can_expval"])) <= tol * max(abs(complex(g["x_can_expval"])), 1.0)
    assert close(pc.ptrace(2).to_numpy(), g["x_can_ptrace"], tol)
    pg = pc.copy()
    pg.apply_gate(g2, 1, chi=3)
    pg.apply_gate(op1, 3)
    pg.swap_gate(2)
    for lam, ref in zip(_lambdas(pg), unpack(g, "x_cang_lam")):
        assert close(lam, ref, 1e-9)
    _same_state(unpack(g, "x_cang_left"), _mps_sites(oc.canonical_to_left_canonical(pg)), 1e-9)
    _same_state(unpack(g, "x_cang_right"), _mps_sites(oc.canonical_to_right_canonical(pg)), 1e-9)
    pb = pc.copy()
    pb.compress_bond(1, chi=2)
    for lam, ref in zip(_lambdas(pb), unpack(g, "x_canb_lam")):
        assert close(lam, ref, 1e-9)
    lc = oc.left_canonical_to_canonical(oc.left_canonical_form_mps(mps_of(sites6)))
    for lam, ref in zip(_lambdas(lc), unpack(g, "x_lcan_lam")):
        assert close(lam, ref, tol)
    # tensor -> MPS / MPO
    T = g["x_T"]
    mt = oc.tensor_to_mps(tn.Tensor(T, ["a", "b", "c", "d"]))
    assert mt.bonddims() == m["x_t2m_bonds"]
    assert close(_full_tensor(mt, [["phys"]] * 4), T, tol)
    mc = oc.tensor_to_mps(tn.Tensor(T, ["a", "b", "c", "d"]), chi=2)
    assert mc.bonddims() == m["x_t2mc_bonds"]
    _same_state(unpack(g, "x_t2mc"), _mps_sites(mc), tol)
    Top = g["x_Top"]
    mo = oc.tensor_to_mpo(tn.Tensor(Top, ["o1", "o2", "o3", "i1", "i2", "i3"]))
    assert mo.bonddims() == m["x_t2o_bonds"] and [t.labels for t in mo] == m["x_t2o_labels"]
    full = _full_tensor(mo, [["physout", "physin"]] * 3)            # (o1, i1, o2, i2, o3, i3)
    assert close(np.transpose(full, [0, 2, 4, 1, 3, 5]), Top, tol)
    # onedim_utils
    sz = np.diag([1.0, -1.0])
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sy = np.array([[0.0, -1j], [1j, 0.0]])
    ob = oc.onebody_sum_mpo([tn.matrices.sigmaz(), tn.matrices.sigmax(), tn.matrices.sigmay(), sz])
    assert [t.labels for t in ob] == m["x_obs_labels"]
    for t, ref in zip(ob, unpack(g, "x_obs")):
        assert t.data.dtype == _torch_dtype(ref.dtype) and np.array_equal(t.to_numpy(), ref)
    ev = oc.expvals_mps(mps_of(sites6), tn.Tensor(sz, ["o", "i"]))
    assert close(ev, g["x_expvals"], tol)
    ev2 = oc.expvals_mps(mps_of(sites6), [op1] * 3, sites=[0, 2, 5])
    assert close(ev2, g["x_expvals_sites"], tol)
    rhos = oc.ptrace_mps(mps_of(sites6))
    assert rhos[0].labels == m["x_rhos_labels"]
    for r, ref in zip(rhos, unpack(g, "x_rhos")):
        assert close(r.to_numpy(), ref, tol)
    for got, ref in [(oc.init_mps_allzero(4, 3), unpack(g, "x_zero")),
                     (oc.init_mps_logical(3, [1, 0, 2], 3), unpack(g, "x_logical"))]:
        for t, r in zip(got, ref):
            assert np.array_equal(t.to_numpy(), r)
    np.random.seed(7)
    rnd = oc.init_mps_random(5, 2, 3)
    assert [t.labels for t in rnd] == m["x_random_labels"]
    for t, r in zip(rnd, unpack(g, "x_random")):
        assert close(t.to_numpy(), r, 1e-12)
    assert sx.shape == sy.shape
    # boundary-MPS PEPS contraction with variational compression
    import tn_oracle as O
    rows = O.random_peps(2, 4, 4, 2, 2)
    peps = tn.twodim.SquareLatticePEPS(
        [[tn.Tensor(a, ["phys", "up", "right", "down", "left"]) for a in r] for r in rows])
    val = tn.twodim.inner_product_peps(peps, peps, exact_contract=False, chi=3,
                                       compression_type="variational", max_iter=30, tolerance=1e-8)
    val = complex(np.asarray(val.to_numpy() if hasattr(val, "to_numpy") else val).reshape(()))
    ref = complex(g["x_peps_var"])
    assert abs(val - ref) <= 1e-7 * abs(ref), (val, ref, complex(g["x_peps_exact"]))


def _torch_dtype(np_dtype):
    import torch
    return {np.dtype(np.float64): torch.float64, np.dtype(np.complex128): torch.complex128,
            np.dtype(np.float32): torch.float32, np.dtype(np.complex64): torch.complex64}[np.dtype(np_dtype)]


def check_con_cases(tn, rtol=1e-12):
    """con on the reference's fixture networks: the default (cost-ordered)
    plan and the argument order give the reference's labels and values,
    including the orders for which the reference returns a merged tensor
    twice."""
    g, m = load("con_cases")
    names = sorted({k[:-len("_out_labels")] for k in m if k.endswith("_out_labels")})
    for name in names:
        tensors = [tn.Tensor(g["%s_in%d" % (name, i)], labels)
                   for i, labels in enumerate(m[name + "_in_labels"])]
        pairs = [tuple(p) for p in m[name + "_pairs"]]
        for order in ("cost", "argument"):
            r = tn.con(tensors, pairs, order=order)
            assert r.labels == m[name + "_out_labels"], (name, order, r.labels)
            assert close(r.to_numpy(), g[name + "_out"], rtol), (name, order)


def check_canonical_conversions(tn, decimal=10):
    """The reference's own unit tests of the canonical-form converters
    (tncontract/tests/test_canonical_form_mps_conversion.py:31-80) on the
    same pickled 10-site MPS, with the same assertions and tolerances."""
    from numpy import testing
    g, m = load("labels_and_fixture")
    sites = unpack(g, "fx_site")
    oc = tn.onedim

    def fresh():
        return oc.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])

    def ip(a, b):
        return complex(np.asarray(oc.inner_product_mps(a, b).cpu()).reshape(()))

    # test_right_and_left_canonical_to_canonical (the reference mutates one
    # module-level MPS through both tests; the same sequence is replayed)
    psi = fresh()
    psi.svd_compress(threshold=1e-12, normalise=False)
    psicr = oc.right_canonical_to_canonical(psi, threshold=1e-12)
    testing.assert_almost_equal(psi.norm(), psicr.norm(), decimal=decimal)
    l, r, n = psicr.check_canonical_form(threshold=1e-10, print_output=False)
    assert (len(l), len(r), len(n)) == (0, 0, 1)
    psi.left_canonise()
    psicl = oc.left_canonical_to_canonical(psi, threshold=1e-12)
    testing.assert_almost_equal(psi.norm(), psicr.norm(), decimal=decimal)
    l, r, n = psicl.check_canonical_form(threshold=1e-10, print_output=False)
    assert (len(l), len(r), len(n)) == (0, 0, 1)
    testing.assert_almost_equal(ip(psicr, psicl), psi.norm() ** 2, decimal=decimal)
    psi.svd_compress(threshold=1e-12, normalise=True)
    psicr = oc.right_canonical_to_canonical(psi, threshold=1e-12)
    assert [len(x) for x in psicr.check_canonical_form(threshold=1e-10, print_output=False)] == [0, 0, 0]
    psi.left_canonise()
    psicl = oc.left_canonical_to_canonical(psi, threshold=1e-12)
    assert [len(x) for x in psicl.check_canonical_form(threshold=1e-10, print_output=False)] == [0, 0, 0]
    testing.assert_almost_equal(ip(psicr, psicl), 1.0, decimal=decimal)
    # test_right_canonical_to_canonical_and_back
    psi.svd_compress(threshold=1e-12, normalise=True)
    psic = oc.right_canonical_to_canonical(psi, threshold=1e-12)
    psir = oc.canonical_to_right_canonical(psic)
    psil = oc.canonical_to_left_canonical(psic)
    testing.assert_almost_equal(ip(psi, psil), 1.0, decimal=decimal)
    testing.assert_almost_equal(ip(psi, psir), 1.0, decimal=decimal)
    assert psir.check_canonical_form(threshold=1e-10, print_output=False)[1] == 0
    assert psil.check_canonical_form(threshold=1e-10, print_output=False)[0] == len(psi) - 1


def _raises_name(fn):
    try:
        fn()
    except Exception as e:  # noqa: BLE001 -- compared with the reference's class name
        return type(e).__name__
    return None


def check_onedim_edges(tn, tol=1e-10):
    """Argument variants and error behaviour of the 1-D API against the
    reference's fixtures (tests/golden/gen_golden.py: gen_onedim_edges)."""
    g, m = load("onedim_edges")
    oc = tn.onedim
    sites = unpack(g, "e_psi")

    def mps_of(s):
        return oc.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in s])

    gate = tn.Tensor(g["e_G"], ["a", "b", "c", "d"])
    b = mps_of(sites)
    b.apply_gate(gate, 1, gate_inputs=["a", "c"])
    _same_state(unpack(g, "e_ag_in"), _mps_sites(b), tol)
    c = mps_of(sites)
    c.apply_gate(gate, 2, gate_outputs=["d", "b"])
    _same_state(unpack(g, "e_ag_out"), _mps_sites(c), tol)
    assert _raises_name(lambda: mps_of(sites).apply_gate(gate, 1, gate_inputs=["a"], gate_outputs=["b", "c"])) \
        == m["e_ag_mismatch"]
    e = mps_of(sites)
    e.left_canonise(0, 2)
    val = complex(e.expval(gate, 2, left_canonised_up_to=2, right_canonised_up_to=4).to_numpy().reshape(()))
    ref = complex(g["e_expval_bounds"])
    assert abs(val - ref) <= tol * max(abs(ref), 1.0)
    assert e.bonddims() == m["e_expval_bounds_bonds"]
    f = mps_of(sites)
    rho = f.ptrace(3)
    assert rho.labels == m["e_ptrace1_labels"] and close(rho.to_numpy(), g["e_ptrace1"], tol)
    op = tn.Tensor(g["e_op"], ["o", "i"])
    lc = oc.left_canonical_form_mps(mps_of(sites))
    assert close(oc.expvals_mps(lc, op, canonised="left"), g["e_expvals_left"], tol)
    rc = oc.right_canonical_form_mps(mps_of(sites))
    assert close(oc.expvals_mps(rc, [op, op], sites=[1, 3], canonised="right"), g["e_expvals_right"], tol)
    lc2 = oc.left_canonical_form_mps(mps_of(sites))
    for r, ref in zip(oc.ptrace_mps(lc2, sites=[0, 4], canonised="left"), unpack(g, "e_rhos_left")):
        assert close(r.to_numpy(), ref, tol)
    mpo = oc.MatrixProductOperator([tn.Tensor(w, ["physout", "physin", "left", "right"]) for w in unpack(g, "e_mpo")])
    mpo.swap_gate(1)
    assert [t.labels for t in mpo] == m["e_mpo_swap_labels"] and mpo.bonddims() == m["e_mpo_swap_bonds"]
    assert close(_full_tensor(mpo, [["physout", "physin"]] * 4), g["e_mpo_swap_full"], tol)
    big = unpack(g, "e_big")
    guess = oc.svd_compress_mps(mps_of(big), 3)
    v = mps_of(big).variational_compress(3, max_iter=40, initial_guess=guess, tolerance=1e-8)
    _same_state(unpack(g, "e_var_guess"), _mps_sites(v), 1e-6)
    vn = mps_of(big).variational_compress(4, max_iter=40, tolerance=1e-8, normalise=True)
    _same_state(unpack(g, "e_var_norm"), _mps_sites(vn), 1e-6)
    assert abs(vn.norm() - complex(g["e_var_norm_value"]).real) < 1e-8
    pc = oc.canonical_form_mps(mps_of(sites))
    pc[3].data = pc[3].data * 1.5
    assert [list(x) for x in pc.check_canonical_form(threshold=1e-10, print_output=False)] == m["e_can_bad"]
    g3 = tn.Tensor(np.ones((2,) * 6), ["o1", "o2", "o3", "i1", "i2", "i3"])
    assert _raises_name(lambda: pc.copy().apply_gate(g3, 0)) == m["e_can_gate3"]
    assert _raises_name(lambda: pc.copy().compress_all()) == m["e_can_compress_all"]
    T = tn.Tensor(g["e_Tmpo"], ["o1", "o2", "i1", "i2"])
    mo = oc.tensor_to_mpo(T, physin_labels=["i1", "i2"])
    assert [t.labels for t in mo] == m["e_t2o_in_labels"]
    full = _full_tensor(mo, [["physout", "physin"]] * 2)             # (o1, i1, o2, i2)
    assert close(np.transpose(full, [0, 2, 1, 3]), g["e_Tmpo"], tol)
    assert _raises_name(lambda: oc.tensor_to_mpo(T, physout_labels=["o1"], physin_labels=["i1", "i2"])) \
        == m["e_t2o_mismatch"]


def con_fixture_network(tn, name):
    """Tensors and pairs of one of the reference's con fixture networks."""
    g, m = load("con_cases")
    tensors = [tn.Tensor(g["%s_in%d" % (name, i)], labels) for i, labels in enumerate(m[name + "_in_labels"])]
    return tensors, [tuple(p) for p in m[name + "_pairs"]], g[name + "_out"], m[name + "_out_labels"]


def con_waves(tn, tensors, pairs):
    """The waves of con's cost-ordered plan for a network (host only)."""
    from tncontract_gb300 import tncon
    labels = [list(t.labels) for t in tensors]
    index_lookup = tncon._index_lookup(labels, pairs)
    internal, _pw = tncon._group_pairs(pairs, index_lookup)
    traced = tncon._traced_labels(labels, internal, index_lookup)
    shapes = [[dict(zip(lb, t.shape))[l] for l in tl] for t, lb, tl in zip(tensors, labels, traced)]
    partner = {}
    for c in pairs:
        if index_lookup[c[0]] != index_lookup[c[1]]:
            partner[c[0]], partner[c[1]] = c[1], c[0]
    steps, _ = tncon._greedy_plan(shapes, traced, partner)
    return tncon.plan_waves(steps)
