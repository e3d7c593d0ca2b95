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
