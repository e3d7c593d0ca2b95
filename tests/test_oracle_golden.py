"""The CPU oracle (oracle/tn_oracle.py) pinned against fixtures produced by
running the reference itself (tests/golden/gen_golden.py)."""
import numpy as np

import api_cases as K
import tn_oracle as O


def test_label_rules_against_reference():
    g, m = K.load("labels_and_fixture")
    d, lab = O.contract_labelled(g["lc_A"], ["spam", "eggs"], g["lc_B"], ["i0", "i1", "i2", "i3"], "spam", "i2")
    assert lab == m["lc_C_labels"] and np.allclose(d, g["lc_C"])
    d, lab = O.contract_labelled(g["lc_T1"], ["a", "b", "a", "c"], g["lc_T2"], ["x", "y", "x"], "a", "x")
    assert lab == m["lc_F_labels"] and np.allclose(d, g["lc_F"])
    d, lab = O.contract_labelled(g["lc_T1"], ["a", "b", "a", "c"], g["lc_T2"], ["x", "y", "x"], "a", "x",
                                 index_slice1=[-1], index_slice2=[0])
    assert lab == m["lc_G_labels"] and np.allclose(d, g["lc_G"])
    d, lab = O.consolidate(g["lc_H"], ["z", "b", "z", "a"])
    assert lab == m["lc_Hc_labels"] and np.array_equal(d, g["lc_Hc"])
    U, ul, s, V, vl = O.tensor_svd(g["lc_S0"], ["i0", "i1", "i2"], ["i0", "i2"])
    assert [ul, ["svd_out", "svd_in"], vl] == m["svd_labels"] and np.allclose(s, g["svd_s"])
    assert list(U.shape) == m["svd_shapes"][0] and list(V.shape) == m["svd_shapes"][2]
    k = O.truncation_keep(s, 2, 1e-15, True)
    assert np.allclose(s[k:], g["tsvd_trunc"])
    k = O.truncation_keep(s, 0, 0.3, False)
    assert np.allclose(s[k:], g["tsvd_rel_trunc"])
    Q, ql, R, rl = O.tensor_qr(g["lc_S0"], ["i0", "i1", "i2"], ["i0", "i2"])
    assert [ql, rl] == m["qr_labels"] and [list(Q.shape), list(R.shape)] == m["qr_shapes"]


def test_reference_fixture_mps():
    g, m = K.load("labels_and_fixture")
    sites = K.unpack(g, "fx_site")
    assert abs(O.mps_norm(sites) - float(g["fx_norm"])) < 1e-12
    spectra = []
    c = O.svd_compress_method(sites, None, 1e-12, False, spectra=spectra)
    assert abs(O.mps_norm(c) - float(g["fx_c_norm"])) < 1e-12
    bonds = [1] + [a.shape[2] for a in c]
    assert bonds == m["fx_c_bonds"]
    for s, s_ref in zip(O.bond_spectra(c), K.unpack(g, "fx_c_spectra")):
        assert K.close(s, s_ref, 1e-10)
    cn = O.svd_compress_method(sites, None, 1e-12, True)
    assert abs(O.mps_norm(cn) - 1.0) < 1e-12
    lc = O.left_canonise_svd(sites, None, 1e-14, False)
    assert [1] + [a.shape[2] for a in lc] == m["fx_lc_bonds"]
    assert abs(O.inner_product(sites, lc) - complex(g["fx_ip"])) < 1e-12


def test_config1():
    g, m = K.load("config1")
    sites = O.random_mps(0, 32, 2, 32, np.float64)
    lc = O.left_canonical_form_mps(sites)
    assert [1] + [a.shape[2] for a in lc] == m["c1_lc_bonds"]
    c = O.svd_compress_method(lc, 16)
    assert [1] + [a.shape[2] for a in c] == m["c1_c_bonds"]
    assert abs(O.fidelity(sites, c) - float(g["c1_fid_vs_input"])) < 1e-12
    for s, s_ref in zip(O.bond_spectra(c), K.unpack(g, "c1_c_spectra")):
        assert K.close(s, s_ref, 1e-10)


def test_config2_small():
    g, m = K.load("config2_small")
    N, chi = 12, 16
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    phi = O.contract_mps_mpo(sites, O.tfim_mpo(N))
    assert K.close(np.transpose(phi[1], (1, 0, 2)), g["c2s_phi_site1"], 1e-14)
    c = O.svd_compress_method(phi, chi)
    assert [1] + [a.shape[2] for a in c] == m["c2s_m_bonds"]
    for s, s_ref in zip(O.bond_spectra(c), K.unpack(g, "c2s_m_spectra")):
        assert K.close(s, s_ref, 1e-10)
    f = O.svd_compress_mps(phi, chi)
    assert abs(O.fidelity(f, c) - float(np.real(g["c2s_fid_f_m"]))) < 1e-12


def test_config2_chi128_apply_compress():
    """The benchmark unit at chi=128 (N=64): ~2 s of LAPACK."""
    g, m = K.load("config2_chi128")
    N, chi = 64, 128
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    phi = O.contract_mps_mpo(sites, O.tfim_mpo(N))
    c = O.svd_compress_method(phi, chi)
    assert [1] + [a.shape[2] for a in c] == m["c2_m_bonds"]
    assert abs(O.fidelity(phi, c) - float(np.real(g["c2_fid_m_phi"]))) < 1e-10
    assert abs(O.mps_norm(c) - float(np.real(g["c2_norm_m"]))) < 1e-10


def test_config2_chi256_apply_compress():
    """The benchmark's own configuration (N=64, chi=256, complex128): the
    oracle against the reference's bond dimensions, norm, fidelity to the
    applied state and per-bond spectra.  About half a minute of LAPACK."""
    g, m = K.load("config2_chi256")
    N, chi = 64, 256
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    phi = O.contract_mps_mpo(sites, O.tfim_mpo(N))
    df = []
    c = O.svd_compress_method(phi, chi, discarded_fraction=df)
    assert [1] + [a.shape[2] for a in c] == m["c2x_m_bonds"]
    assert abs(O.mps_norm(c) - float(np.real(g["c2x_norm_m"]))) < 1e-10
    assert abs(O.fidelity(phi, c) - float(np.real(g["c2x_fid_m_phi"]))) < 1e-10
    for s, s_ref in zip(O.bond_spectra(c), K.unpack(g, "c2x_m_spectra")):
        assert K.close(s, s_ref, 1e-10)
    # each truncation keeps (1 - df) of the current squared norm, so their
    # product is the reference's squared norm ratio of the result to phi
    assert len(df) == N - 1 and all(0.0 <= x < 1.0 for x in df)
    kept = float(np.prod([1.0 - x for x in df]))
    ratio = (float(np.real(g["c2x_norm_m"])) / float(np.real(g["c2x_norm_phi"]))) ** 2
    assert abs(kept - ratio) < 1e-10 * ratio


def test_graded_rank_rule():
    """Spectra over 20 decades, svd_compress(threshold=1e-14) without a cap:
    the threshold decides every rank (tests/golden/graded)."""
    g, m = K.load("graded")
    for tag, dt in (("gr", np.float64), ("grc", np.complex128)):
        sites = O.graded_mps(m[tag + "_seed"], 16, 2, 32, 20.0, dt)
        assert [1] + [a.shape[2] for a in sites] == m[tag + "_input_bonds"]
        c = O.svd_compress_method(sites, None, 1e-14)
        assert [1] + [a.shape[2] for a in c] == m[tag + "_bonds"]
        assert abs(O.mps_norm(c) - float(np.real(g[tag + "_norm"]))) < 1e-12 * float(np.real(g[tag + "_norm"]))
        for s, s_ref in zip(O.bond_spectra(c), K.unpack(g, tag + "_spectra")):
            assert K.close(s, s_ref, 1e-10)


def test_peps_small_against_reference():
    g, m = K.load("peps")
    layer = O.double_layer(O.random_peps(2, 4, 4, 2, 2))
    v = O.mps_contract(layer, 4)
    assert abs(float(v) - float(g["p4_value"])) < 1e-10 * abs(float(g["p4_value"]))
    assert abs(float(v) - float(g["p4_exact"])) < 1e-6 * abs(float(g["p4_exact"]))


def test_workload_generators_match_oracle():
    from tncontract_gb300 import workloads as W
    for a, b in zip(W.random_mps_arrays(3, 6, 3, 5, np.complex64, True), O.random_mps(3, 6, 3, 5, np.complex64, True)):
        assert np.array_equal(a, b)
    for a, b in zip(W.tfim_mpo_arrays(5), O.tfim_mpo(5)):
        assert np.array_equal(a, b)
    for a, b in zip(W.xxz_mpo_arrays(5), O.xxz_mpo(5)):
        assert np.array_equal(a, b)
    for ra, rb in zip(W.random_peps_arrays(2, 3, 3, 2, 2), O.random_peps(2, 3, 3, 2, 2)):
        for a, b in zip(ra, rb):
            assert np.array_equal(a, b)
