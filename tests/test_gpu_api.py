"""The drop-in API on the GPU against fixtures generated by the reference."""
import pytest

import api_cases as K

pytestmark = pytest.mark.gpu


def test_label_cases(gpu):
    K.check_label_cases(gpu)


def test_factorisation_labels(gpu):
    K.check_factorisation_labels(gpu)


def test_contract_errors(gpu):
    K.check_contract_errors(gpu)


def test_reference_fixture_mps(gpu):
    K.check_fixture_mps(gpu)


def test_config1_left_canonise_then_compress(gpu):
    K.check_config1(gpu)


def test_config2_small_apply_and_compress(gpu):
    K.check_config2_small(gpu)


def test_onedim_extras(gpu):
    K.check_onedim_extras(gpu)


def test_con_fixture_networks(gpu):
    K.check_con_cases(gpu)


def test_canonical_conversions(gpu):
    K.check_canonical_conversions(gpu)


def test_onedim_edges(gpu):
    K.check_onedim_edges(gpu)
