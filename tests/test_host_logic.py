"""Host logic of the drop-in API (label resolution, axis-move simulation,
MPS control flow) on CPU, with the device ops replaced by the test-only CPU
stand-in in host_fake.py; results compared with the reference's fixtures."""
import api_cases as K
from host_fake import cpu_ops


def test_label_cases_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_label_cases(tn)


def test_factorisation_labels_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_factorisation_labels(tn)


def test_contract_errors_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_contract_errors(tn)


def test_reference_fixture_mps_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_fixture_mps(tn)


def test_config1_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_config1(tn)


def test_config2_small_host():
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_config2_small(tn)


def test_onedim_extras_host():
    """Gates, expvals, ptrace, variational compression, the canonical form
    and the onedim_utils constructors (host logic, CPU stand-in)."""
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_onedim_extras(tn)


def test_onedim_edges_host():
    """Argument variants and errors of the 1-D API (CPU stand-in)."""
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_onedim_edges(tn)


def test_canonical_conversions_host():
    """The reference's own converter tests, host logic on the CPU stand-in."""
    import tncontract_gb300 as tn
    with cpu_ops():
        K.check_canonical_conversions(tn)


def test_canonical_conversions_any_svd_phase_host():
    """The converters keep the state when the SVD of the last (one-column)
    site returns a V other than LAPACK's 1: the CPU stand-in's SVD is given a
    different, equally valid gauge (U and V^H times a phase) there."""
    import numpy as np
    import torch
    import tncontract_gb300 as tn
    import tncontract_gb300._ops as ops
    with cpu_ops():
        base = ops.svd

        def svd_other_gauge(M, *a, **k):
            u, s, vh = base(M, *a, **k)
            if M.shape[1] == 1:
                ph = -1.0 if not M.is_complex() else complex(np.exp(0.7j))
                u = u * (ph.conjugate() if isinstance(ph, complex) else ph)
                vh = vh * ph
            return u, s, vh
        ops.svd = svd_other_gauge
        try:
            K.check_canonical_conversions(tn)
            # complex input too (phase, not only a sign)
            g, m = K.load("onedim_extras")
            sites = [torch.from_numpy(a).numpy() for a in K.unpack(g, "x_psi")]
            psi = tn.onedim.MatrixProductState([tn.Tensor(a, ["phys", "left", "right"]) for a in sites])
            psi.right_canonise()
            c = tn.onedim.right_canonical_to_canonical(psi)
            back = tn.onedim.canonical_to_left_canonical(c)
            ip = complex(tn.onedim.inner_product_mps(psi, back).reshape(()).item())
            assert abs(ip - psi.norm() ** 2) < 1e-10
        finally:
            ops.svd = base


def test_engine_rank_rules():
    """The engine's host-side rank rule equals the reference's (s/s_max >
    threshold, then at most chi) and is capped at the storage noise floor."""
    import numpy as np
    import torch
    from tncontract_gb300 import engine as E
    s = np.array([1.0, 0.5, 1e-3, 1e-9, 1e-15, 0.0])
    assert E.reference_rank(s, 0, 1e-14) == 4
    assert E.reference_rank(s, 3, 1e-14) == 3
    assert E.reference_rank(s, 0, 1e-3) == 2          # strictly greater than threshold * s_max
    assert E.reference_rank(np.zeros(3), 0, 1e-14) == 0
    assert E.noise_rank(s, torch.float64) == 5        # 1e-15 > 4 eps |s| ~ 1e-15
    assert E.noise_rank(s, torch.float32) == 3        # FP32 floor ~ 5e-7
    assert E.noise_rank(s, torch.complex64) == 3


def test_boundary_mps_engine_host():
    """engine.boundary_mps_contract (control flow, layouts, log-norm
    bookkeeping) with the CPU stand-in, against the reference's PEPS norm
    values: 4x4 D=2 chi=4 and 8x8 D=4 chi=16."""
    import numpy as np
    import tn_oracle as O
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    g, m = K.load("peps")
    with cpu_ops():
        rows = O.random_peps(2, 4, 4, 2, 2)
        val, log10, _ = E.boundary_mps_contract(W.double_layer_arrays(rows), 4, precision="fp64")
        assert abs(val - float(g["p4_value"])) < 1e-10 * float(g["p4_value"])
        rows = W.random_peps_arrays(2, 8, 8, 4, 2)
        val, log10, _ = E.boundary_mps_contract(W.double_layer_arrays(rows), 16, precision="fp64")
        assert abs(log10 - m["p8c16_log10"]) < 1e-10
        assert np.isfinite(log10)


def test_high_rank_permute_and_trace_plans():
    """Permutations and traces of more axes than the kernels take are planned
    on the host as fused steps of at most eight axes (numpy applies the
    steps here; the device applies the same steps with tnc_permute)."""
    import random
    import numpy as np
    from tncontract_gb300._ops import permutation_steps, fuse_trace, MAX_KERNEL_RANK
    rng = random.Random(2)
    for n in (3, 8, 9, 12, 16, 21):
        for trial in range(20):
            shape = [rng.choice([1, 2, 2, 3]) for _ in range(n)]
            if np.prod(shape) > 300000:
                continue
            perm = list(range(n))
            rng.shuffle(perm)
            x = np.random.default_rng(trial).standard_normal(shape)
            cur = x
            for s, p in permutation_steps(shape, perm):
                assert len(s) <= MAX_KERNEL_RANK
                s, p = (s, p) if s else ([cur.size], [0])
                cur = np.ascontiguousarray(np.transpose(cur.reshape(s), p))
            assert np.array_equal(cur.reshape([shape[p] for p in perm]), np.transpose(x, perm))
    for shape, a1, a2 in [([2, 3, 3, 2, 1, 2, 2, 3, 2, 2], 1, 7), ([2] * 4 + [3] + [2] * 5 + [3, 2], 10, 4)]:
        x = np.random.default_rng(0).standard_normal(shape)
        fs, b1, b2 = fuse_trace(shape, a1, a2)
        got = np.trace(x.reshape(fs), axis1=b1, axis2=b2)
        ref = np.trace(x, axis1=a1, axis2=a2)
        assert np.allclose(got.reshape(ref.shape), ref)


def test_sweep_flop_count():
    """The metric's fixed flop count (per-site formula of the plain method's
    bonds): a hand-computed small case, internal consistency, and the value
    at the benchmark configuration."""
    from tncontract_gb300 import workloads as W
    f = W.sweep_flops(2, 2, 1, 1, complex_=False)
    # apply 2*8; QR of 2x1: 2*2*1 - 2/3; R absorption 2*1*1*2; SVD of 2x1: 6*2 + 20; U S absorption 2*2*1*1
    assert abs(f["total"] - (16 + (4 - 2.0 / 3.0) + 4 + 32 + 4)) < 1e-9
    fc = W.sweep_flops(2, 2, 1, 1, complex_=True)
    assert abs(fc["total"] - 4 * f["total"]) < 1e-9
    big = W.sweep_flops(64, 2, 3, 256)
    assert abs(sum(v for k, v in big.items() if k != "total") - big["total"]) < 1e-3 * big["total"]
    assert abs(big["total"] / 1e12 - 1.5721156823466667) < 1e-9


def test_balance_keeps_the_state():
    import numpy as np
    import tn_oracle as O
    from tncontract_gb300 import engine as E
    sites = O.random_mps(3, 8, 2, 6, np.complex128, normalise=True)
    sites[2] = sites[2] * 1e-30
    bal, log_norm = E.balance(sites)
    assert all(abs(np.linalg.norm(a) - 1.0) < 1e-12 for a in bal)
    n0 = O.mps_norm(sites)
    n1 = O.mps_norm(bal) * np.exp(log_norm)
    assert abs(n0 - n1) <= 1e-10 * n0
    assert 1.0 - O.fidelity(sites, bal) < 1e-12


def test_discarded_weight_rank():
    from tncontract_gb300 import rank_model as RM
    s = [1.0, 0.5, 0.1, 0.01]                      # s^2 total 1.2601
    assert RM.dw_rank(s, 1e-3) == 3                # tail 1e-4 <= 1.26e-3
    assert RM.dw_rank(s, 1e-3, chi=2) == 2
    assert RM.dw_rank(s, 1e-2) == 2                # tail 0.0101 <= 0.012601
    assert RM.dw_rank(s, 1.0) == 1                 # at least one value is kept
    assert RM.dw_rank([0.0, 0.0], 1e-3) == 1


def test_uneven_batch_specs():
    """The uneven batch's instance list: 512 specs, ranges and dtypes of the
    workload definition, deterministic in the seed."""
    import numpy as np
    from tncontract_gb300 import workloads as W
    specs = W.config3_specs()
    assert len(specs) == 512 and specs == W.config3_specs()
    assert all(16 <= N <= 128 and d in (2, 3, 4) and 16 <= chi <= 256 for N, d, chi, _, _ in specs)
    assert [dt for _, _, _, dt, _ in specs[:4]] == [np.float32, np.complex64, np.float32, np.complex64]
    assert len({seed for *_, seed in specs}) == 512
    assert {d for _, d, _, _, _ in specs} == {2, 3, 4}
    assert W.config3_specs(seed=2) != specs


def test_trace_of_unequal_axes_host():
    """contract_internal over axes of different lengths sums the common
    leading diagonal, as np.trace does (the reference's behaviour)."""
    import numpy as np
    import tncontract_gb300 as tn
    rng = np.random.default_rng(6)
    with cpu_ops():
        for shape, a1, a2 in [((2, 3), 0, 1), ((4, 2, 3), 0, 2), ((3, 2, 5, 2), 2, 0), ((1, 3), 1, 0)]:
            x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            labels = ["l%d" % i for i in range(len(shape))]
            t = tn.Tensor(x, list(labels))
            t.contract_internal(labels[a1], labels[a2])
            ref = np.trace(x, axis1=a1, axis2=a2)
            assert t.labels == [l for i, l in enumerate(labels) if i not in (a1, a2)]
            assert np.allclose(t.to_numpy(), ref)


def test_tensor_svd_retry_contract_host():
    """tensor_svd's failure contract (tncontract/tensor.py:914-929) on the
    CPU stand-in: a failed first SVD warns and is retried with the larger
    sweep cap; a non-finite matrix prints the inf / nan report and
    re-raises the ValueError."""
    import warnings as _w
    import numpy as np
    import tncontract_gb300 as tn
    from tncontract_gb300 import _ops
    calls = []
    with cpu_ops():
        real = _ops.svd

        def flaky(M, max_sweeps=0, **kw):
            calls.append(max_sweeps)
            if len(calls) == 1:
                raise _ops.LinAlgError("SVD did not converge")
            return real(M, max_sweeps=max_sweeps, **kw)
        _ops.svd = flaky
        try:
            t = tn.Tensor(np.arange(12.0).reshape(3, 4), ["r", "c"])
            with _w.catch_warnings(record=True) as rec:
                _w.simplefilter("always")
                U, S, V = tn.tensor_svd(t, ["r"])
        finally:
            _ops.svd = real
        assert any("retrying" in str(r.message) for r in rec)
        from tncontract_gb300 import tensor as T
        assert calls == [T.SVD_SWEEPS, T.SVD_RETRY_SWEEPS]


def test_committed_svd_rows_tuning():
    """The committed tuning table (tncontract_gb300/svd_rows_tuning.json,
    generated on a GB300 by tuning.generate): every bucket of the row
    kernels has a choice among the candidates; lookups round rows and
    length up to the next bucket and give None beyond the largest."""
    from tncontract_gb300 import tuning
    from tncontract_gb300 import _lib as L
    tab = tuning.load()
    assert tab, "svd_rows_tuning.json missing or empty"
    cands = {L.ROWS_GRAM, 4, 8}
    for name in tuning.DTYPES:
        for n in tuning.LENGTHS:
            if n > tuning.MAX_LEN[name]:
                continue
            for r in tuning.ROWS:
                if r <= n:
                    assert tab.get("%s:%d:%d" % (name, r, n)) in cands, (name, r, n)
    assert tuning.key("complex64", 300, 700) == "complex64:512:1024"
    assert tuning.key("complex64", 16, 64) == "complex64:16:64"
    assert tuning.key("float64", 16, 2000) is None
    fake = {"complex64:512:512": 4}
    assert tuning.lookup("complex64", 400, 500, table=fake) == 4
    assert tuning.lookup("complex64", 400, 600, table=fake) is None
