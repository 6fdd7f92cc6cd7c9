"""Reconstruction constants against the reference's own doctest values."""
import json
import os

import numpy as np

import gen_coefficients as gc

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json")))


def test_centered4_float32_matches_reference_jldoctest():
    got = gc.symmetric_stencil(np.float32, 2)
    assert [np.float32(x) for x in GOLD["centered4_f32"]] == got


def test_upwind5_left_float32_matches_reference_jldoctest():
    # calc_reconstruction_stencil(Float32, 3, :left, :x) lists weights by offset -3..+1;
    # uniform_reconstruction_coefficients returns them in reverse order.
    coeff = gc.uniform_reconstruction_coefficients(np.float32, "left", 3)
    by_offset = list(coeff[::-1])
    assert [np.float32(x) for x in GOLD["upwind5_left_f32_by_offset"]] == by_offset


def test_centered2_float64():
    assert gc.symmetric_stencil(np.float64, 1) == GOLD["centered2_f64"]


def test_weno_constants_match_reference():
    from fractions import Fraction
    assert [Fraction(a, b) for a, b in GOLD["cstar_weno5"]] == gc.C_STAR[3]
    assert GOLD["smoothness_weno5"] == gc.SMOOTHNESS[3]
    assert GOLD["epsilon_literal"] == "1f-8"


def test_rk3_constants():
    want = {"γ¹": (8, 15), "γ²": (5, 12), "γ³": (3, 4), "ζ²": (-17, 60), "ζ³": (-5, 12)}
    assert {k: tuple(v) for k, v in GOLD["rk3"].items()} == want


def test_generated_header_is_current():
    here = os.path.dirname(os.path.abspath(gc.__file__))
    with open(os.path.join(here, "csrc", "gbo_coeffs.h")) as f:
        assert f.read() == gc.header_text()


def makhoul_dest(k, N):
    # the reordering used by the DCT kernels (gbo_fft.cuh: makhoul_dest), 0-based
    return N - 1 - (k >> 1) if k & 1 else (k >> 1)


def test_dct_reordering_matches_reference_permutation():
    for N, key in ((8, "permute_index_8"), (9, "permute_index_9")):
        assert [makhoul_dest(i - 1, N) + 1 for i in range(1, N + 1)] == GOLD[key]
    for N, key in ((8, "unpermute_index_8"), (9, "unpermute_index_9")):
        inv = [0] * N
        for k in range(N):
            inv[makhoul_dest(k, N)] = k
        assert [inv[i - 1] + 1 for i in range(1, N + 1)] == GOLD[key]
