"""The benchmark's own configuration on the GPU (TFIM D=3 MPO applied to the
seeded random complex128 MPS, N=64, chi=256, then svd_compress(256)) against
the reference's fixture (tests/golden/config2_chi256, made by running the
reference) and the FP64 oracle's result of the same sweep; and the rank rule
on graded spectra, where the threshold (not the bond cap) decides every rank
(tests/golden/graded).

Tolerances: FP64 storage -- fidelity error 1e-10, spectra 1e-8 relative,
discarded fractions 1e-10 absolute, norm 1e-9 relative; single-precision
storage ("fp32", and "mixed" with its double-float or FP64 bond-core
Jacobi finish) -- fidelity error 1e-6 (1e-8 with a finish), spectra 1e-4,
discarded fractions 1e-6, norm 1e-5.  Bond dimensions (integers) must match
exactly."""
import ctypes

import numpy as np
import pytest
import torch

import api_cases as K
import tn_oracle as O

pytestmark = pytest.mark.gpu

N, CHI = 64, 256
TOL = {"fp64": (1e-10, 1e-8, 1e-10, 1e-9), "fp32": (1e-6, 1e-4, 1e-6, 1e-5), "mixed": (1e-6, 1e-4, 1e-6, 1e-5),
       "mixed_fp64": (1e-6, 1e-4, 1e-6, 1e-5)}
# the mixed precision's bond-core finish: double-float ("mixed") or FP64 ("mixed_fp64");
# either brings the state to the oracle's within 1e-8 (FP32 cores alone: ~2e-7)
FID_CORE = {"mixed": 1e-8, "mixed_fp64": 1e-8}
CORE = {"fp64": None, "fp32": None, "mixed": "df", "mixed_fp64": "fp64"}


@pytest.fixture(scope="module")
def oracle256():
    """The FP64 oracle's sweep at the metric configuration (~10-30 s of LAPACK)."""
    sites = O.random_mps(0, N, 2, CHI, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    df = []
    ref = O.apply_compress_sweep(sites, mpo, CHI, discarded_fraction=df)
    return sites, mpo, ref, df


@pytest.mark.parametrize("precision", ["fp64", "fp32", "mixed", "mixed_fp64"])
def test_metric_config_native_sweep(gpu, oracle256, precision):
    from tncontract_gb300 import engine as E
    g, m = K.load("config2_chi256")
    sites, mpo, ref, df = oracle256
    fid_tol, s_tol, dw_tol, n_tol = TOL[precision]
    dt = E.compute_dtype(precision.split("_")[0], True)
    bal, ln = E.balance(sites)
    st = E.SweepStats()
    prof = (ctypes.c_double * 12)()
    out = E.apply_compress_native(E.to_sites(bal, dt), E.to_sites(mpo, dt), CHI, log_norm_in=ln, stats=st,
                                  profile=prof, core=CORE[precision])
    got = [o.cpu().numpy().astype(np.complex128) for o in out]
    # bond dimensions: exactly the reference's
    assert [1] + [a.shape[2] for a in got] == m["c2x_m_bonds"]
    assert [1] + list(st.bonds) + [1] == m["c2x_m_bonds"]
    # the state: against the oracle's compressed state and the reference's
    # norm and fidelity to the applied state
    err = 1.0 - O.fidelity(ref, got)
    assert err < FID_CORE.get(precision, fid_tol), err
    assert st.norm_folded
    n_ref = float(np.real(g["c2x_norm_m"]))
    assert abs(O.mps_norm(got) - n_ref) < n_tol * n_ref
    phi = O.contract_mps_mpo(sites, mpo)
    assert abs(O.fidelity(phi, got) - float(np.real(g["c2x_fid_m_phi"]))) < 10 * fid_tol
    # per-bond discarded fraction of the squared spectrum
    assert len(st.discarded) == N - 1
    assert max(abs(a - b) for a, b in zip(st.discarded, df)) < dw_tol
    # per-bond spectra of the result
    for s, s_ref in zip(O.bond_spectra(got), K.unpack(g, "c2x_m_spectra")):
        assert K.close(s, s_ref, s_tol)
    # "mixed" finished every bond core (profile op 3 = the finishing Jacobi)
    assert prof[3 * 3 + 1] == (N - 1 if precision.startswith("mixed") else 0)


def test_metric_config_host_api(gpu, oracle256):
    """engine.apply_compress_host (the e2e path of the benchmark): complex128
    host arrays in and out, mixed precision."""
    from tncontract_gb300 import engine as E
    sites, mpo, ref, df = oracle256
    st = E.SweepStats()
    got = E.apply_compress_host(sites, mpo, CHI, precision="mixed", stats=st)
    assert all(a.dtype == np.complex128 for a in got)
    assert 1.0 - O.fidelity(ref, got) < 1e-6
    assert abs(O.mps_norm(got) - O.mps_norm(ref)) < 1e-5 * O.mps_norm(ref)


@pytest.mark.parametrize("tag,dt", [("gr", np.float64), ("grc", np.complex128)])
def test_graded_rank_rule_exact(gpu, tag, dt):
    """svd_compress(threshold=1e-14), no bond cap, on spectra falling over 20
    decades: the native sweep, the Python engine and the drop-in method keep
    exactly the reference's number of singular values at every bond (FP64),
    with the reference's spectra and norm."""
    import tncontract_gb300 as tn
    from tncontract_gb300 import engine as E
    g, m = K.load("graded")
    sites = O.graded_mps(m[tag + "_seed"], 16, 2, 32, 20.0, dt)
    tdt = torch.float64 if dt == np.float64 else torch.complex128
    ident = [np.eye(2).reshape(2, 2, 1, 1) for _ in range(16)]
    want = m[tag + "_bonds"]
    n_ref = float(np.real(g[tag + "_norm"]))
    st = E.SweepStats()
    out = E.apply_compress_native(E.to_sites(sites, tdt), E.to_sites(ident, tdt), 0, threshold=1e-14, stats=st)
    got = [o.cpu().numpy() for o in out]
    assert [1] + [a.shape[2] for a in got] == want
    assert abs(O.mps_norm(got) - n_ref) < 1e-9 * n_ref
    for s, s_ref in zip(O.bond_spectra(got), K.unpack(g, tag + "_spectra")):
        assert K.close(s, s_ref, 1e-8)
    eng = E.apply_compress(E.to_sites(sites, tdt), E.to_sites(ident, tdt), 0, threshold=1e-14)
    assert [1] + [int(a.shape[2]) for a in eng] == want
    psi = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
    psi.svd_compress(threshold=1e-14)
    assert [int(x) for x in psi.bonddims()] == want
