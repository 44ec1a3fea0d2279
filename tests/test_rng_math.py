"""Philox known-answer vectors and the deterministic math (CPU)."""
import math

import numpy as np

from oracle import binding as ob


def test_philox4x32_10_known_answers():
    # Random123 kat_vectors for philox4x32_10
    assert list(ob.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(ob.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(ob.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_one_minus_exp_matches_libm():
    xs = np.concatenate([np.logspace(-12, -0.31, 400), np.linspace(0.49, 45, 400), [0.5, 1.0, 2.0, 37.9]])
    for x in xs:
        ref = -math.expm1(-x)
        got = ob.one_minus_exp(x)
        assert got == 0.0 and ref == 0.0 or abs(got - ref) <= 4 * math.ulp(ref), (x, got, ref)
    assert ob.one_minus_exp(0.0) == 0.0
    assert ob.one_minus_exp(-1.0) == 0.0
    assert ob.one_minus_exp(50.0) == 1.0


def test_one_minus_expf_accuracy():
    """The FP32 evaluation used for the hazard: a few ulp of the exact value
    over the whole range, no cancellation at small x."""
    xs = np.concatenate([np.logspace(-9, -0.31, 300), np.linspace(0.49, 25, 300)]).astype(np.float32)
    for x in xs:
        ref = -math.expm1(-float(x))
        got = ob.one_minus_expf(float(x))
        assert abs(got - ref) <= 4 * float(np.spacing(np.float32(ref))) + 1e-30, (x, got, ref)
    assert ob.one_minus_expf(0.0) == 0.0 and ob.one_minus_expf(30.0) == 1.0


def test_seasonality_day0():
    from pansim_gb300 import synth
    s = synth.make_snapshot(200, 50)
    v = ob.seasonality(s, 0)
    # d = 267 + 6 -> d_mod = 93 >= d_peak 81, c0 = 3.08 (infectionPolicies.h:443-478)
    d_mod, d_peak, c0 = 93, 81, 3.08
    ref = (0.5 * c0 * math.cos(2 * math.pi * (d_mod - d_peak) / 366) + 1 - 0.5 * c0) / (0.5 * c0 + 1 - 0.5 * c0)
    assert abs(v - max(min(ref, 1.0), 0.5)) < 1e-15
    assert 0.96 < v < 0.98


def test_modified_p_exact_daily_chain():
    from pansim_gb300 import synth
    # avgLength 1, maxlength 0: expectedLength is NaN and the secant method
    # returns its second start point 0.9 (basicLengthAbstract.cpp:16-29)
    assert synth.calculate_modified_p(1.0, 0.0) == 0.9
    assert synth.calculate_modified_p(-1.0, -1.0) == 1.0
    p = synth.calculate_modified_p(4.0, 13.0)
    assert 0.2 < p < 0.3
