"""Generate the golden fixtures in this folder by running the reference
library (andrewdarmawan/tncontract, pure Python on NumPy/SciPy) itself.

Run from the repository root with the reference checkout importable:

    python tests/golden/gen_golden.py /path/to/tncontract-checkout [--only=NAME ...]

(``--only=onedim_extras`` regenerates one fixture file).

The reference predates NumPy 2; two aliases it uses (``np.product``,
``np.float``) are restored at run time before it is imported.  The checkout is
only read.  Outputs (small ``.npz`` / ``.json`` files) are committed and are
what the tests compare against; the tests never import the reference.

Inputs are regenerated from seeds by ``oracle/tn_oracle.py``'s generators
(``numpy.random.default_rng``), except the reference's own pickled 10-site
test MPS, whose arrays are stored here verbatim.
"""
import json
import os
import pickle
import sys
import time

import numpy as np

if not hasattr(np, "product"):
    np.product = np.prod
if not hasattr(np, "float"):
    np.float = float

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.dont_write_bytecode = True
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import tn_oracle as O  # noqa: E402


def _ref(path):
    sys.path.insert(0, path)
    import tncontract as tn  # noqa
    return tn


def to_sites(mps, tn):
    """Reference MPS -> list of (phys,left,right) arrays (label-aware)."""
    out = []
    for t in mps:
        lab = list(t.labels)
        perm = [lab.index(mps.phys_label), lab.index(mps.left_label),
                lab.index(mps.right_label)]
        out.append(np.ascontiguousarray(np.transpose(t.data, perm)))
    return out


def spectra_of(sites):
    return [np.asarray(s) for s in O.bond_spectra(sites)]


def pack_list(prefix, arrs, store):
    store[prefix + "_n"] = np.array(len(arrs))
    for i, a in enumerate(arrs):
        store["%s_%d" % (prefix, i)] = np.asarray(a)


def gen_label_cases(tn, store, meta):
    rng = np.random.default_rng(11)
    # README / docstring label cases (tensor.py:659-683, README.md:37-128)
    A = tn.Tensor(rng.random((2, 2)), labels=["spam", "eggs"])
    B = tn.Tensor(rng.random((2, 3, 2, 4)))
    store["lc_A"] = A.data
    store["lc_B"] = B.data
    C = tn.contract(A, B, "spam", "i2")
    D = tn.contract(A, B, ["spam", "eggs"], ["i0", "i2"])
    E = A["spam", "eggs"] * B["i0", "i2"]
    store["lc_C"] = C.data
    store["lc_D"] = D.data
    store["lc_E"] = E.data
    meta["lc_C_labels"] = C.labels
    meta["lc_D_labels"] = D.labels
    meta["lc_E_labels"] = E.labels
    # duplicate labels and index_slice (tensor.py:702-731)
    T1 = tn.Tensor(rng.random((2, 3, 2, 4)), labels=["a", "b", "a", "c"])
    T2 = tn.Tensor(rng.random((2, 5, 2)), labels=["x", "y", "x"])
    store["lc_T1"] = T1.data
    store["lc_T2"] = T2.data
    F = tn.contract(T1, T2, "a", "x")
    G = tn.contract(T1, T2, "a", "x", index_slice1=[-1], index_slice2=[0])
    store["lc_F"] = F.data
    store["lc_G"] = G.data
    meta["lc_F_labels"] = F.labels
    meta["lc_G_labels"] = G.labels
    # consolidate_indices (tensor.py:340-370)
    H = tn.Tensor(rng.random((2, 3, 4, 5)), labels=["z", "b", "z", "a"])
    store["lc_H"] = H.data
    H2 = H.copy()
    H2.consolidate_indices()
    store["lc_Hc"] = H2.data
    meta["lc_Hc_labels"] = H2.labels
    # tensor product and con (tncon.py:4-159)
    P = tn.tensor_product(A, tn.Tensor(rng.random(3), labels=["q"]))
    store["lc_P"] = P.data
    meta["lc_P_labels"] = P.labels
    # con docstring-style ring: A_i labelled left_i/right_i, periodic trace
    R = tn.Tensor(rng.random((2, 2)), labels=["left", "right"])
    store["lc_R"] = R.data
    tl = [R.suf(str(i)) for i in range(5)]
    pairs = [("right" + str(j), "left" + str(j + 1)) for j in range(4)]
    ring = tn.con(tl, pairs, ("right4", "left0"))
    store["lc_ring"] = np.asarray(ring.data)
    meta["lc_ring_labels"] = ring.labels
    # con with a multi-edge pair, an internal trace and a disconnected tensor
    X = tn.Tensor(rng.random((2, 3, 4)), labels=["x1", "x2", "x3"])
    Y = tn.Tensor(rng.random((3, 4, 5)), labels=["y1", "y2", "y3"])
    Z = tn.Tensor(rng.random((6, 6, 2)), labels=["z1", "z2", "z3"])
    W = tn.Tensor(rng.random(7), labels=["w1"])
    store["lc_X"], store["lc_Y"], store["lc_Z"], store["lc_W"] = X.data, Y.data, Z.data, W.data
    K = tn.con(X, Y, Z, W, ("x2", "y1"), ("x3", "y2"), ("z1", "z2"), ("x1", "z3"))
    store["lc_K"] = np.asarray(K.data)
    meta["lc_K_labels"] = K.labels
    # tensor_svd / truncated_svd / tensor_qr / tensor_lq labels & shapes
    S0 = tn.Tensor(rng.random((2, 3, 4)), labels=["i0", "i1", "i2"])
    store["lc_S0"] = S0.data
    U, S, V = tn.tensor_svd(S0, ["i0", "i2"])
    meta["svd_labels"] = [U.labels, S.labels, V.labels]
    meta["svd_shapes"] = [list(U.shape), list(S.shape), list(V.shape)]
    store["svd_s"] = np.diag(S.data)
    U2, V2, tr = tn.truncated_svd(S0, ["i0", "i2"], chi=2)
    meta["tsvd_labels"] = [U2.labels, V2.labels]
    meta["tsvd_shapes"] = [list(U2.shape), list(V2.shape)]
    store["tsvd_trunc"] = np.asarray(tr)
    U3, V3, tr3 = tn.truncated_svd(S0, ["i0", "i2"], chi=0, threshold=0.3,
                                   absolute=False, absorb_singular_values="both")
    meta["tsvd_rel_shapes"] = [list(U3.shape), list(V3.shape)]
    store["tsvd_rel_trunc"] = np.asarray(tr3)
    Q, Rr = tn.tensor.tensor_qr(S0, ["i0", "i2"])
    meta["qr_labels"] = [Q.labels, Rr.labels]
    meta["qr_shapes"] = [list(Q.shape), list(Rr.shape)]
    L, Q2 = tn.tensor.tensor_lq(S0, ["i0", "i2"])
    meta["lq_labels"] = [L.labels, Q2.labels]
    meta["lq_shapes"] = [list(L.shape), list(Q2.shape)]


def gen_fixture_10site(tn, ref_path, store, meta):
    """The reference's own test MPS (tests/random_10site_mps.dat) and what its
    tests pin (test_canonical_form_mps_conversion.py:31-80)."""
    with open(os.path.join(ref_path, "tncontract/tests/random_10site_mps.dat"), "rb") as f:
        psi = pickle.load(f, encoding="latin1")
    meta["fx_labels"] = [list(t.labels) for t in psi]
    meta["fx_mps_labels"] = [psi.left_label, psi.right_label, psi.phys_label]
    sites = to_sites(psi, tn)
    pack_list("fx_site", sites, store)
    store["fx_norm"] = np.array(psi.norm())
    a = psi.copy()
    a.svd_compress(threshold=1e-12, normalise=False)
    store["fx_c_norm"] = np.array(a.norm())
    meta["fx_c_bonds"] = [int(x) for x in a.bonddims()]
    meta["fx_c_labels"] = [list(t.labels) for t in a]
    pack_list("fx_c_spectra", spectra_of(to_sites(a, tn)), store)
    b = psi.copy()
    b.svd_compress(threshold=1e-12, normalise=True)
    store["fx_cn_norm"] = np.array(b.norm())
    c = psi.copy()
    c.left_canonise()
    meta["fx_lc_bonds"] = [int(x) for x in c.bonddims()]
    meta["fx_lc_canon"] = list(c.check_canonical_form(threshold=1e-10, print_output=False))
    store["fx_ip"] = np.array(tn.onedim.inner_product_mps(psi, c))


def gen_config1(tn, store, meta):
    """Config: N=32, d=2, chi=32 float64 seed 0; left_canonical_form_mps then
    svd_compress(chi=16)."""
    sites = O.random_mps(0, 32, 2, 32, np.float64)
    mps = tn.onedim.MatrixProductState(
        [tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    t0 = time.perf_counter()
    lc = tn.onedim.left_canonical_form_mps(mps)
    comp = lc.copy()
    comp.svd_compress(chi=16)
    meta["c1_ref_seconds"] = time.perf_counter() - t0
    meta["c1_lc_bonds"] = [int(x) for x in lc.bonddims()]
    meta["c1_c_bonds"] = [int(x) for x in comp.bonddims()]
    meta["c1_c_labels"] = [list(t.labels) for t in comp][:3]
    cs = to_sites(comp, tn)
    store["c1_norm_in"] = np.array(mps.norm())
    store["c1_norm_lc"] = np.array(lc.norm())
    store["c1_norm_c"] = np.array(comp.norm())
    ip = tn.onedim.inner_product_mps
    store["c1_fid_vs_input"] = np.array(abs(ip(mps, comp)) ** 2 /
                                        (ip(mps, mps) * ip(comp, comp)))
    pack_list("c1_c_spectra", spectra_of(cs), store)


def gen_config2(tn, store, meta, N, chi, tag):
    """TFIM (D=3) MPO applied to a normalised random complex128 MPS, then
    svd_compress(chi) (method) and svd_compress_mps(chi) (function)."""
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    mps = tn.onedim.MatrixProductState(
        [tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    W = tn.onedim.MatrixProductOperator(
        [tn.Tensor(w, ["physout", "physin", "left", "right"]) for w in mpo])
    t0 = time.perf_counter()
    phi = tn.onedim.contract_mps_mpo(mps, W)
    t1 = time.perf_counter()
    m = phi.copy()
    m.svd_compress(chi=chi)
    t2 = time.perf_counter()
    meta[tag + "_ref_seconds_apply"] = t1 - t0
    meta[tag + "_ref_seconds_method"] = t2 - t1
    meta[tag + "_phi_labels"] = list(phi[1].labels)
    meta[tag + "_phi_shape"] = list(phi[1].shape)
    meta[tag + "_phi_phys"] = phi.phys_label
    if N <= 16:
        store[tag + "_phi_site1"] = phi[1].data
    meta[tag + "_m_bonds"] = [int(x) for x in m.bonddims()]
    meta[tag + "_m_labels"] = [list(t.labels) for t in m][:3]
    ip = tn.onedim.inner_product_mps
    store[tag + "_norm_phi"] = np.array(phi.norm())
    store[tag + "_norm_m"] = np.array(m.norm())
    store[tag + "_fid_m_phi"] = np.array(abs(ip(phi, m)) ** 2 / (ip(phi, phi) * ip(m, m)))
    ms = to_sites(m, tn)
    pack_list(tag + "_m_spectra", spectra_of(ms), store)
    if N <= 16:
        f = tn.onedim.svd_compress_mps(phi, chi)
        meta[tag + "_f_bonds"] = [int(x) for x in f.bonddims()]
        store[tag + "_norm_f"] = np.array(f.norm())
        store[tag + "_fid_f_m"] = np.array(abs(ip(f, m)) ** 2 / (ip(f, f) * ip(m, m)))
        pack_list(tag + "_f_spectra", spectra_of(to_sites(f, tn)), store)


def gen_graded(tn, store, meta):
    """svd_compress(threshold=1e-14) without a bond cap on MPS whose spectra
    fall over 20 decades (oracle.graded_mps): the threshold decides every
    rank, so the bond dimensions pin the rank rule itself.  Real float64 and
    complex128 inputs; the seeds are chosen so that every singular value the
    truncations see lies at least 0.4 decades from the threshold (a count
    closer to it would depend on rounding)."""
    for tag, dt, seed in (("gr", np.float64, 11), ("grc", np.complex128, 2)):
        sites = O.graded_mps(seed, 16, 2, 32, 20.0, dt)
        mps = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
        m = mps.copy()
        m.svd_compress(threshold=1e-14)
        meta[tag + "_seed"] = seed
        meta[tag + "_bonds"] = [int(x) for x in m.bonddims()]
        meta[tag + "_input_bonds"] = [1] + [a.shape[2] for a in sites]
        store[tag + "_norm"] = np.array(m.norm())
        pack_list(tag + "_spectra", spectra_of(to_sites(m, tn)), store)


def gen_peps(tn, store, meta, L, D, d, chi, tag, seed=2):
    rows = O.random_peps(seed, L, L, D, d)
    peps = tn.twodim.SquareLatticePEPS(
        [[tn.Tensor(a, ["phys", "up", "right", "down", "left"]) for a in r] for r in rows])
    t0 = time.perf_counter()
    v = tn.twodim.inner_product_peps(peps, peps, exact_contract=False, chi=chi)
    meta[tag + "_ref_seconds"] = time.perf_counter() - t0
    val = v.data if hasattr(v, "data") else v
    val = np.longdouble(np.real(val))
    m, e = np.frexp(np.float64(val / np.longdouble(10.0) ** int(np.floor(np.log10(float(val))))))
    meta[tag + "_value_str"] = repr(val)
    meta[tag + "_log10"] = float(np.log10(val))
    store[tag + "_value"] = np.array(float(val))
    if L <= 4:
        ex = tn.twodim.inner_product_peps(peps, peps, exact_contract=True)
        store[tag + "_exact"] = np.array(float(np.real(ex.data)))


def site_list(net, tn):
    """Sites of an MPS-like network as (phys, left, right) arrays; networks
    whose sites lack the physical leg (the Lambda sites of the canonical
    form) are stored as (left, right) matrices."""
    out = []
    for t in net:
        lab = list(t.labels)
        if net.phys_label in lab:
            perm = [lab.index(net.phys_label), lab.index(net.left_label), lab.index(net.right_label)]
        else:
            perm = [lab.index(net.left_label), lab.index(net.right_label)]
        out.append(np.ascontiguousarray(np.transpose(t.data, perm)))
    return out


def gen_onedim_extras(tn, store, meta):
    """Gates, expectation values, reduced density matrices, variational
    compression, the Gamma-Lambda canonical form and its converters,
    tensor -> MPS / MPO splits and the onedim_utils constructors
    (onedim_core.py:95-127, 486-1327, 1448-1479, 1711-1928;
    onedim_utils.py)."""
    oc = tn.onedim
    rng = np.random.default_rng(21)

    def cgauss(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    def mps_of(sites):
        return oc.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])

    sites6 = O.random_mps(5, 6, 2, 4, np.complex128, normalise=True)
    pack_list("x_psi", sites6, store)
    G2 = cgauss(2, 2, 2, 2)
    G3 = cgauss(2, 2, 2, 2, 2, 2)
    op1 = cgauss(2, 2)
    store["x_G2"], store["x_G3"], store["x_op1"] = G2, G3, op1
    g2 = tn.Tensor(G2, ["o1", "o2", "i1", "i2"])
    g3 = tn.Tensor(G3, ["o1", "o2", "o3", "i1", "i2", "i3"])
    # swap_gate (onedim_core.py:95-127)
    a = mps_of(sites6)
    a.swap_gate(2)
    pack_list("x_swap", site_list(a, tn), store)
    meta["x_swap_bonds"] = [int(x) for x in a.bonddims()]
    meta["x_swap_labels"] = [list(t.labels) for t in a]
    # apply_gate (onedim_core.py:662-739)
    for tag, gate, first, kw in [("x_ag2l", g2, 2, {}), ("x_ag2r", g2, 2, {"canonise": "right"}),
                                 ("x_ag3c", g3, 1, {"chi": 3})]:
        b = mps_of(sites6)
        b.apply_gate(gate, first, **kw)
        pack_list(tag, site_list(b, tn), store)
        meta[tag + "_bonds"] = [int(x) for x in b.bonddims()]
        meta[tag + "_labels"] = [list(t.labels) for t in b]
    # expval and ptrace (onedim_core.py:741-877)
    e = mps_of(sites6)
    store["x_expval"] = np.asarray(e.expval(g2, 2).data)
    meta["x_expval_bonds"] = [int(x) for x in e.bonddims()]
    f = mps_of(sites6)
    rho = f.ptrace(1, 2)
    store["x_ptrace"] = rho.data
    meta["x_ptrace_labels"] = list(rho.labels)
    # variational compression (onedim_core.py:486-631, 1476-1479)
    sites8 = O.random_mps(6, 8, 2, 8, np.complex128, normalise=True)
    pack_list("x_psi8", sites8, store)
    p8 = mps_of(sites8)
    v = p8.variational_compress(4, max_iter=20, tolerance=1e-8)
    pack_list("x_var", site_list(v, tn), store)
    meta["x_var_bonds"] = [int(x) for x in v.bonddims()]
    meta["x_var_labels"] = [list(t.labels) for t in v]
    store["x_var_norm"] = np.array(v.norm())
    v2 = oc.variational_compress_mps(mps_of(sites8), 3, max_iter=40, tolerance=1e-6)
    pack_list("x_var3", site_list(v2, tn), store)
    # canonical form (onedim_core.py:880-1327, 1448-1454, 1836-1928)
    pc = oc.onedim_core.canonical_form_mps(mps_of(sites6))
    meta["x_can_check"] = [list(map(int, x)) for x in pc.check_canonical_form(threshold=1e-10, print_output=False)]
    meta["x_can_bonds"] = [int(x) for x in pc.bonddims()]
    store["x_can_norm"] = np.array(pc.norm())
    pack_list("x_can_lam", [np.diag(pc[2 * i].data) for i in range(pc.nsites_physical + 1)], store)
    store["x_can_expval"] = np.asarray(pc.expval(g2, 1).data)
    store["x_can_ptrace"] = pc.ptrace(2).data
    pg = pc.copy()
    pg.apply_gate(g2, 1, chi=3)
    pg.apply_gate(tn.Tensor(op1, ["o", "i"]), 3)
    pg.swap_gate(2)
    pack_list("x_cang_lam", [np.diag(pg[2 * i].data) for i in range(pg.nsites_physical + 1)], store)
    pack_list("x_cang_left", site_list(oc.canonical_to_left_canonical(pg), tn), store)
    pack_list("x_cang_right", site_list(oc.canonical_to_right_canonical(pg), tn), store)
    pb = pc.copy()
    pb.compress_bond(1, chi=2)
    pack_list("x_canb_lam", [np.diag(pb[2 * i].data) for i in range(pb.nsites_physical + 1)], store)
    lc = oc.left_canonical_to_canonical(oc.left_canonical_form_mps(mps_of(sites6)))
    pack_list("x_lcan_lam", [np.diag(lc[2 * i].data) for i in range(lc.nsites_physical + 1)], store)
    # tensor -> MPS / MPO (onedim_core.py:1711-1833)
    T = cgauss(2, 3, 2, 2)
    store["x_T"] = T
    m = oc.tensor_to_mps(tn.Tensor(T, ["a", "b", "c", "d"]))
    meta["x_t2m_bonds"] = [int(x) for x in m.bonddims()]
    pack_list("x_t2m", site_list(m, tn), store)
    mc = oc.tensor_to_mps(tn.Tensor(T, ["a", "b", "c", "d"]), chi=2)
    meta["x_t2mc_bonds"] = [int(x) for x in mc.bonddims()]
    pack_list("x_t2mc", site_list(mc, tn), store)
    Top = cgauss(2, 2, 2, 2, 2, 2)
    store["x_Top"] = Top
    mo = oc.tensor_to_mpo(tn.Tensor(Top, ["o1", "o2", "o3", "i1", "i2", "i3"]))
    meta["x_t2o_bonds"] = [int(x) for x in mo.bonddims()]
    meta["x_t2o_labels"] = [list(t.labels) for t in mo]
    # onedim_utils
    import tncontract.matrices as mats
    terms = [mats.sigmaz(), mats.sigmax(), mats.sigmay(), mats.sigmaz()]
    ob = tn.onedim.onebody_sum_mpo(terms)
    pack_list("x_obs", [t.data for t in ob], store)
    meta["x_obs_labels"] = [list(t.labels) for t in ob]
    ev = tn.onedim.expvals_mps(mps_of(sites6), tn.Tensor(np.asarray(mats.sigmaz()), ["o", "i"]))
    store["x_expvals"] = np.asarray(ev)
    ev2 = tn.onedim.expvals_mps(mps_of(sites6), [tn.Tensor(op1, ["o", "i"])] * 3, sites=[0, 2, 5])
    store["x_expvals_sites"] = np.asarray(ev2)
    rhos = tn.onedim.ptrace_mps(mps_of(sites6))
    pack_list("x_rhos", [r.data for r in rhos], store)
    meta["x_rhos_labels"] = list(rhos[0].labels)
    z = tn.onedim.init_mps_allzero(4, 3)
    pack_list("x_zero", [t.data for t in z], store)
    lg = tn.onedim.init_mps_logical(3, [1, 0, 2], 3)
    pack_list("x_logical", [t.data for t in lg], store)
    np.random.seed(7)
    rnd = tn.onedim.init_mps_random(5, 2, 3)
    pack_list("x_random", [t.data for t in rnd], store)
    meta["x_random_labels"] = [list(t.labels) for t in rnd]
    # boundary-MPS PEPS contraction with variational compression
    # (square_lattice.py:164-173): 4 x 4, D=2, d=2, chi=3
    rows = O.random_peps(2, 4, 4, 2, 2)
    peps = tn.twodim.SquareLatticePEPS(
        [[tn.Tensor(a, ["phys", "up", "right", "down", "left"]) for a in r] for r in rows])
    val = tn.twodim.inner_product_peps(peps, peps, exact_contract=False, chi=3,
                                       compression_type="variational", max_iter=30, tolerance=1e-8)
    store["x_peps_var"] = np.array(complex(np.asarray(val.data).reshape(())))
    ex = tn.twodim.inner_product_peps(peps, peps, exact_contract=True)
    store["x_peps_exact"] = np.array(complex(np.asarray(ex.data).reshape(())))


def _raises(fn):
    """Name of the exception ``fn()`` raises, or None."""
    try:
        fn()
    except Exception as e:  # noqa: BLE001 -- the class name is the fixture
        return type(e).__name__
    return None


def gen_onedim_edges(tn, store, meta):
    """Argument variants and error behaviour of the 1-D API: explicit
    gate_inputs / gate_outputs, partial canonisation bounds, left-canonical
    inputs to expvals_mps / ptrace_mps, swap_gate on an MPO, variational
    compression from an initial guess and normalised, non-canonical
    Gamma-Lambda networks, and the errors each raises."""
    oc = tn.onedim
    rng = np.random.default_rng(41)

    def cgauss(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    def mps_of(sites):
        return oc.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])

    sites = O.random_mps(8, 5, 2, 3, np.complex128, normalise=True)
    pack_list("e_psi", sites, store)
    G = cgauss(2, 2, 2, 2)
    store["e_G"] = G
    g = tn.Tensor(G, ["a", "b", "c", "d"])
    b = mps_of(sites)
    b.apply_gate(g, 1, gate_inputs=["a", "c"])          # outputs: b, d
    pack_list("e_ag_in", site_list(b, tn), store)
    c = mps_of(sites)
    c.apply_gate(g, 2, gate_outputs=["d", "b"])         # inputs: a, c
    pack_list("e_ag_out", site_list(c, tn), store)
    meta["e_ag_mismatch"] = _raises(lambda: mps_of(sites).apply_gate(g, 1, gate_inputs=["a"],
                                                                    gate_outputs=["b", "c"]))
    e = mps_of(sites)
    e.left_canonise(0, 2)
    store["e_expval_bounds"] = np.asarray(e.expval(g, 2, left_canonised_up_to=2, right_canonised_up_to=4).data)
    meta["e_expval_bounds_bonds"] = [int(x) for x in e.bonddims()]
    f = mps_of(sites)
    rho = f.ptrace(3)
    store["e_ptrace1"] = rho.data
    meta["e_ptrace1_labels"] = list(rho.labels)
    op = tn.Tensor(cgauss(2, 2), ["o", "i"])
    store["e_op"] = op.data
    lc = oc.left_canonical_form_mps(mps_of(sites))
    store["e_expvals_left"] = np.asarray(oc.expvals_mps(lc, op, canonised="left"))
    rc = oc.right_canonical_form_mps(mps_of(sites))
    store["e_expvals_right"] = np.asarray(oc.expvals_mps(rc, [op, op], sites=[1, 3], canonised="right"))
    lc2 = oc.left_canonical_form_mps(mps_of(sites))
    rhos = oc.ptrace_mps(lc2, sites=[0, 4], canonised="left")
    pack_list("e_rhos_left", [r.data for r in rhos], store)
    # swap_gate on an MPO (all non-virtual legs move)
    W = [cgauss(2, 2, 1 if i == 0 else 3, 1 if i == 3 else 3) for i in range(4)]
    pack_list("e_mpo", W, store)
    mpo = oc.MatrixProductOperator([tn.Tensor(w, ["physout", "physin", "left", "right"]) for w in W])
    mpo.swap_gate(1)
    meta["e_mpo_swap_labels"] = [list(t.labels) for t in mpo]
    meta["e_mpo_swap_bonds"] = [int(x) for x in mpo.bonddims()]
    Wfull = None
    for t in mpo:
        lab = list(t.labels)
        a = np.transpose(t.data, [lab.index("left"), lab.index("physout"), lab.index("physin"), lab.index("right")])
        Wfull = a if Wfull is None else np.tensordot(Wfull, a, axes=([Wfull.ndim - 1], [0]))
    store["e_mpo_swap_full"] = Wfull.reshape(Wfull.shape[1:-1])
    # variational compression from an initial guess, and normalised
    big = O.random_mps(9, 6, 2, 6, np.complex128, normalise=False)
    pack_list("e_big", big, store)
    guess = oc.svd_compress_mps(mps_of(big), 3)
    v = mps_of(big).variational_compress(3, max_iter=40, initial_guess=guess, tolerance=1e-8)
    pack_list("e_var_guess", site_list(v, tn), store)
    vn = mps_of(big).variational_compress(4, max_iter=40, tolerance=1e-8, normalise=True)
    pack_list("e_var_norm", site_list(vn, tn), store)
    store["e_var_norm_value"] = np.array(vn.norm())
    # Gamma-Lambda: a perturbed network is not canonical; errors
    pc = oc.onedim_core.canonical_form_mps(mps_of(sites))
    pc[3].data = pc[3].data * 1.5
    meta["e_can_bad"] = [list(map(int, x)) for x in pc.check_canonical_form(threshold=1e-10, print_output=False)]
    g3 = tn.Tensor(cgauss(2, 2, 2, 2, 2, 2), ["o1", "o2", "o3", "i1", "i2", "i3"])
    meta["e_can_gate3"] = _raises(lambda: pc.copy().apply_gate(g3, 0))
    meta["e_can_compress_all"] = _raises(lambda: pc.copy().compress_all())
    T = tn.Tensor(cgauss(2, 2, 2, 2), ["o1", "o2", "i1", "i2"])
    store["e_Tmpo"] = T.data
    mo = oc.tensor_to_mpo(T, physin_labels=["i1", "i2"])
    meta["e_t2o_in_labels"] = [list(t.labels) for t in mo]
    meta["e_t2o_mismatch"] = _raises(lambda: oc.tensor_to_mpo(T, physout_labels=["o1"], physin_labels=["i1", "i2"]))


def con_networks(tn, rng):
    """Networks for the con fixtures: (name, tensors, pairs); data drawn from
    ``rng`` in a fixed order."""
    def t(shape, labels, cplx=False):
        a = rng.standard_normal(shape)
        if cplx:
            a = a + 1j * rng.standard_normal(shape)
        return tn.Tensor(a, labels)
    A, B = t((2, 6), ["a0", "a1"]), t((6, 6), ["b0", "b1"])
    C, D = t((6, 6), ["c0", "c1"]), t((6, 2), ["d0", "d1"])
    nets = [("chain_components", [A, B, C, D], [("a1", "b0"), ("c1", "d0"), ("b1", "c0")]),
            ("chain_outer_first", [D, A, B, C], [("d1", "a0"), ("a1", "b0"), ("b1", "c0"), ("c1", "d0")])]
    P, Q = t((3, 4, 5, 5), ["p0", "p1", "p2", "p3"], True), t((4, 6, 3), ["q0", "q1", "q2"], True)
    R, S, V = t((6, 7), ["r0", "r1"]), t((7, 2), ["s0", "s1"]), t((9,), ["v0"])
    nets.append(("ring_trace_multiedge", [P, Q, R, S, V],
                 [("p2", "p3"), ("p1", "q0"), ("q1", "r0"), ("r1", "s0"), ("p0", "q2")]))
    H = t((3, 4, 5), ["h0", "h1", "h2"])
    leaves = [t((n,), ["l%d" % i]) for i, n in enumerate((3, 4, 5))]
    nets.append(("star_scalar", [H] + leaves, [("h0", "l0"), ("h1", "l1"), ("h2", "l2")]))
    # 2 x 3 grid: physical leg 2, bonds 3 between neighbours, 1 at the boundary
    G = [t((2, 1 if r == 0 else 3, 3 if r == 0 else 1, 1 if c == 0 else 3, 3 if c < 2 else 1),
           ["g%d%d%s" % (r, c, x) for x in "pudlr"]) for r in range(2) for c in range(3)]
    pairs = [("g%d%dr" % (r, c), "g%d%dl" % (r, c + 1)) for r in range(2) for c in range(2)]
    pairs += [("g0%dd" % c, "g1%du" % c) for c in range(3)]
    nets.append(("grid_2x3", G, pairs))
    # the same grid with the pairs in breadth-first order from the corner (every
    # pair joins the growing component, so the reference contracts it exactly)
    bfs = [("g00r", "g01l"), ("g00d", "g10u"), ("g01r", "g02l"), ("g01d", "g11u"), ("g10r", "g11l"),
           ("g02d", "g12u"), ("g11r", "g12l")]
    nets.append(("grid_2x3_bfs", G, bfs))
    return nets


def gen_con_cases(tn, store, meta):
    """con (tncon.py:4-159) on networks that exercise its plan: a pair order
    whose component bookkeeping returns a tensor twice (the reference's
    result is kept as is), an order starting with an outer product, a ring
    with a trace and a multi-edge plus a disconnected vector, a full
    contraction to a scalar and a 2 x 3 grid with open legs."""
    rng = np.random.default_rng(31)
    for name, tensors, pairs in con_networks(tn, rng):
        for i, x in enumerate(tensors):
            store["%s_in%d" % (name, i)] = x.data
        meta[name + "_in_labels"] = [list(x.labels) for x in tensors]
        meta[name + "_pairs"] = [list(p) for p in pairs]
        r = tn.con(tensors, pairs)
        store[name + "_out"] = np.asarray(r.data)
        meta[name + "_out_labels"] = list(r.labels)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    if not args:
        raise SystemExit("usage: python tests/golden/gen_golden.py /path/to/tncontract-checkout [--only=NAME ...]")
    ref_path = args[0]
    tn = _ref(ref_path)
    if not only or "labels_and_fixture" in only:
        store, meta = {}, {}
        gen_label_cases(tn, store, meta)
        gen_fixture_10site(tn, ref_path, store, meta)
        np.savez_compressed(os.path.join(HERE, "labels_and_fixture.npz"), **store)
        with open(os.path.join(HERE, "labels_and_fixture.json"), "w") as f:
            json.dump(meta, f, indent=1)
    for fn, job in [("config1", lambda s, m: gen_config1(tn, s, m)),
                    ("config2_small", lambda s, m: gen_config2(tn, s, m, 12, 16, "c2s")),
                    ("config2_chi128", lambda s, m: gen_config2(tn, s, m, 64, 128, "c2")),
                    ("config2_chi256", lambda s, m: gen_config2(tn, s, m, 64, 256, "c2x")),
                    ("peps", lambda s, m: (gen_peps(tn, s, m, 4, 2, 2, 4, "p4"),
                                           gen_peps(tn, s, m, 8, 4, 2, 16, "p8c16"),
                                           gen_peps(tn, s, m, 8, 4, 2, 64, "p8c64"))),
                    ("onedim_extras", lambda s, m: gen_onedim_extras(tn, s, m)),
                    ("con_cases", lambda s, m: gen_con_cases(tn, s, m)),
                    ("onedim_edges", lambda s, m: gen_onedim_edges(tn, s, m)),
                    ("graded", lambda s, m: gen_graded(tn, s, m))]:
        if only and fn not in only:
            continue
        s, m = {}, {}
        t = time.perf_counter()
        job(s, m)
        print(fn, "%.1fs" % (time.perf_counter() - t), flush=True)
        np.savez_compressed(os.path.join(HERE, fn + ".npz"), **s)
        with open(os.path.join(HERE, fn + ".json"), "w") as f:
            json.dump(m, f, indent=1)


if __name__ == "__main__":
    main()
