"""CPU tests: the oracle is pinned against the reference's own golden outputs.

Fixtures (tests/golden, made by tests/golden/make_golden.py from the reference's tools):
  ref_order*/reference.bin + filter_taps.hpp   tools/ref_generate.py
  emulators.npz                                tools/{stcr,dtcr,plr}_emulator.py
  sosfilt_order2_uniform.npz                   scipy.signal.sosfilt, butter(2, 0.1) on 2^14 uniform samples
"""
import os

import numpy as np
import pytest

import oracle
from cuda_recursive_filtering_gb300 import formats
from conftest import GOLDEN

ORDERS = (2, 4, 8, 16)


@pytest.fixture(scope="module")
def emu():
    return np.load(os.path.join(GOLDEN, "emulators.npz"))


@pytest.mark.parametrize("order", ORDERS)
def test_sosfilt_f64_matches_reference_bin(order):
    """oracle FP64 cascade == the reference's reference.bin (FP64 sosfilt, stored float32)."""
    d = os.path.join(GOLDEN, f"ref_order{order}")
    taps = formats.parse_filter_taps(os.path.join(d, "filter_taps.hpp"))
    ref = formats.read_reference_bin(os.path.join(d, "reference.bin"))
    x = formats.reference_input(ref.size, taps["gain"])
    y = oracle.sosfilt_f64(taps["sos"].astype(np.float64), x.astype(np.float64)).astype(np.float32)
    # identical operation order as scipy's transposed DF-II: equal after float32 rounding
    mism = np.count_nonzero(y != ref)
    assert mism <= ref.size // 1000, f"{mism} samples differ"
    assert np.max(np.abs(y.astype(np.float64) - ref)) <= 2e-7 * np.max(np.abs(ref))


def test_sosfilt_f64_matches_scipy_order2_uniform():
    g = np.load(os.path.join(GOLDEN, "sosfilt_order2_uniform.npz"))
    y = oracle.sosfilt_f64(g["sos"], g["x"].astype(np.float64))
    assert np.max(np.abs(y - g["y"])) <= 1e-13 * np.max(np.abs(g["y"]))


@pytest.mark.parametrize("order", ORDERS)
def test_direct_f32_bit_exact_vs_plr_emulator(order, emu):
    """oracle float32 direct form == tools/plr_emulator.py direct_form_f32, bit for bit."""
    x = emu[f"x_direct_{order}"]
    with np.errstate(over="ignore", invalid="ignore"):
        y = oracle.direct_f32(x, emu[f"b_direct_{order}"], emu[f"a_direct_{order}"])
    ref = emu[f"direct_{order}"]
    both_nan = np.isnan(y) & np.isnan(ref)
    assert np.array_equal(y[~both_nan], ref[~both_nan])


@pytest.mark.parametrize("order", ORDERS)
def test_direct_form_verdicts_reproduce_reference(order, emu):
    """Direct form in float32: orders 2/4 pass the 1e-4 gate, 8 fails, 16 is non-finite
    (tools/plr_emulator.py Part B, reproduced)."""
    with np.errstate(over="ignore", invalid="ignore"):
        y = oracle.direct_f32(emu[f"x_direct_{order}"], emu[f"b_direct_{order}"], emu[f"a_direct_{order}"])
    e = oracle.errors(y, emu[f"ref_direct_{order}"])
    if order in (2, 4):
        assert e["finite"] and e["rel_max"] < 1e-4
    elif order == 8:
        assert e["finite"] and e["rel_max"] > 1e-4
    else:
        assert not e["finite"] or e["rel_max"] > 1e-2


@pytest.mark.parametrize("order", ORDERS)
def test_merge_sections_matches_direct_form_taps(order):
    """Product of the normalised float32 sections == the reference's butter(ba) taps."""
    taps = formats.parse_filter_taps(os.path.join(GOLDEN, f"ref_order{order}", "filter_taps.hpp"))
    b, a = oracle.merge_sections(taps["sos"].astype(np.float64))
    assert b.size == taps["plr_order"] == order
    scale_b = np.max(np.abs(taps["plr_b"]))
    scale_a = np.max(np.abs(taps["plr_a"]))
    # float32 rounding of the section coefficients bounds the agreement
    assert np.max(np.abs(b - taps["plr_b"])) <= 1e-5 * scale_b
    assert np.max(np.abs(a - taps["plr_a"])) <= 1e-5 * scale_a


@pytest.mark.parametrize("order", ORDERS)
def test_cascade_f32_within_reference_gate(order):
    """The float32 sequential cascade passes the reference's gate on its own test signal."""
    d = os.path.join(GOLDEN, f"ref_order{order}")
    taps = formats.parse_filter_taps(os.path.join(d, "filter_taps.hpp"))
    ref = formats.read_reference_bin(os.path.join(d, "reference.bin"))
    x = formats.reference_input(ref.size, taps["gain"])
    y = oracle.cascade_f32(x, taps["sos"])
    assert oracle.errors(y, ref)["rel_max"] < 1e-5


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("geom", ["32x32", "32x64", "32x128", "64x64"])
def test_emulator_fixtures_pass_gate(order, geom, emu):
    """Sanity of the fixtures themselves: the reference's STCR/DTCR emulators pass their gate."""
    ref = emu[f"ref_stcr_{order}_{geom}"]
    assert oracle.errors(emu[f"stcr_{order}_{geom}"], ref)["rel_max"] < 1e-4
    assert oracle.errors(emu[f"dtcr_{order}_{geom}"], ref)["rel_max"] < 1e-4


def test_normalise_and_reference_golden_consistent():
    from scipy import signal
    sos = signal.butter(4, 0.1, output="sos")
    norm, g = oracle.normalise_sos(sos)
    assert np.allclose(norm[:, 0], 1.0) and np.allclose(norm[:, 3], 1.0)
    assert np.isclose(g, np.prod(sos[:, 0]))
    x = np.random.default_rng(0).uniform(-1, 1, 4096).astype(np.float32)
    xd, gold = oracle.reference_golden(sos, x)
    y = signal.sosfilt(sos, x.astype(np.float64))
    assert np.max(np.abs(gold - y)) <= 1e-5 * np.max(np.abs(y))
