"""The FP32-class check (conftest.check_fp32_class) on synthetic fields: the plain normwise
bound, and the snow clamp's ill-conditioned rows, which may exceed it only when they are few,
all marked ill-conditioned, and the bulk of the rows stays in the FP32 class."""
import numpy as np
import pytest

from conftest import check_fp32_class


def fields(n=20000, seed=0):
    rng = np.random.default_rng(seed)
    o64 = rng.uniform(0.9, 1.1, size=(n, 3, 3))
    o32 = o64 + rng.normal(0.0, 1e-6, size=o64.shape)  # the FP32 oracle: ~1e-6 from FP64
    gpu = o64 + rng.normal(0.0, 1e-6, size=o64.shape)
    return {"F": gpu}, {"F": o32}, {"F": o64}


def test_within_the_class_passes():
    g, o32, o64 = fields()
    check_fp32_class(g, o32, o64, 1e-5, fields=("F",))


def test_a_row_far_off_fails_without_the_ill_set():
    g, o32, o64 = fields()
    g["F"][17] += 0.02
    with pytest.raises(AssertionError):
        check_fp32_class(g, o32, o64, 1e-5, fields=("F",))


def test_ill_conditioned_rows_may_exceed_the_maximum():
    g, o32, o64 = fields()
    g["F"][[17, 400]] += 0.02
    check_fp32_class(g, o32, o64, 1e-5, fields=("F",),
                     ill=lambda rows: np.isin(rows, [17, 400]))


def test_a_row_off_outside_the_ill_set_fails():
    g, o32, o64 = fields()
    g["F"][[17, 400]] += 0.02
    with pytest.raises(AssertionError):
        check_fp32_class(g, o32, o64, 1e-5, fields=("F",), ill=lambda rows: np.isin(rows, [17]))


def test_many_ill_rows_fail():
    g, o32, o64 = fields()
    rows = np.arange(0, 20000, 200)  # 100 rows: more than max(50, 1e-5 n)
    g["F"][rows] += 0.02
    with pytest.raises(AssertionError):
        check_fp32_class(g, o32, o64, 1e-5, fields=("F",), ill=lambda r: np.ones(len(r), bool))


def test_bulk_outside_the_class_fails_even_with_the_ill_set():
    g, o32, o64 = fields()
    g["F"] += np.random.default_rng(1).normal(0.0, 1e-4, size=g["F"].shape)  # 100x the oracle
    g["F"][17] += 0.02
    with pytest.raises(AssertionError):
        check_fp32_class(g, o32, o64, 1e-5, fields=("F",), ill=lambda r: np.ones(len(r), bool))
