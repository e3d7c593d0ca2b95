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
