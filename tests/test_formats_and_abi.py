"""CPU tests: reference harness formats, workloads, and the C-ABI library surface."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from cuda_recursive_filtering_gb300 import _lib, formats
from conftest import GOLDEN, ROOT


@pytest.mark.parametrize("order", (2, 4, 8, 16))
def test_filter_taps_round_trip(order, tmp_path):
    src = os.path.join(GOLDEN, f"ref_order{order}", "filter_taps.hpp")
    t = formats.parse_filter_taps(src)
    assert t["n_sections"] == order // 2 and t["sos"].shape == (order // 2, 6)
    assert np.all(t["sos"][:, 0] == 1.0)
    out = tmp_path / "taps.hpp"
    formats.write_filter_taps(str(out), t["sos"], t["gain"], t["plr_b"], t["plr_a"])
    u = formats.parse_filter_taps(str(out))
    assert np.array_equal(u["sos"], t["sos"])
    assert u["gain"] == t["gain"]
    assert np.array_equal(u["plr_b"], t["plr_b"]) and np.array_equal(u["plr_a"], t["plr_a"])


def test_design_matches_reference_generator():
    for order in (2, 4, 8, 16):
        t = formats.parse_filter_taps(os.path.join(GOLDEN, f"ref_order{order}", "filter_taps.hpp"))
        d = formats.design_reference_filter(order // 2)
        assert np.array_equal(d["sos"], t["sos"])
        assert d["gain"] == pytest.approx(t["gain"], rel=1e-15)
        assert np.allclose(d["plr_b"], t["plr_b"], rtol=1e-12, atol=0)


def test_reference_bin_round_trip(tmp_path):
    y = np.random.default_rng(0).normal(size=1000)
    p = tmp_path / "r.bin"
    formats.write_reference_bin(str(p), y)
    assert np.array_equal(formats.read_reference_bin(str(p)), y.astype(np.float32))
    with pytest.raises(ValueError):
        formats.read_reference_bin(str(p), 2000)


def test_reference_input_formula():
    x = formats.reference_input(16, 0.5)
    i = np.arange(16, dtype=np.float64)
    assert np.array_equal(x, (0.5 * np.cos(2 * np.pi * 120 * i / 1000)).astype(np.float32))


def test_library_exports_every_declared_symbol(built_library):
    names = _lib.declared_functions()
    assert "iir_sos_filter" in names and "iir_plan_execute" in names
    lib = ctypes.CDLL(built_library)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    nm = subprocess.run(["nm", "-D", "--defined-only", built_library], capture_output=True, text=True).stdout
    for n in names:
        assert f" T {n}" in nm, n


def test_noalloc_limit_matches_header():
    import re
    text = open(_lib.HEADER).read()
    m = re.search(r"#define IIR_NOALLOC_MAX_SAMPLES \(1ull << (\d+)\)", text)
    assert m and (1 << int(m.group(1))) == _lib.IIR_NOALLOC_MAX_SAMPLES


def test_status_strings_and_argument_checks(built_library):
    L = _lib.load(built_library)
    assert L.iir_version() >= 10000
    for code in (0, -1, -2, -3, -4, -5, -6):
        assert L.iir_status_string(code)
    # argument validation happens before any CUDA call
    p = ctypes.c_void_p()
    sos = (ctypes.c_float * 6)(1, 0, 0, 1, 0, 0)
    assert L.iir_plan_create(ctypes.byref(p), sos, 0, 1, 32, 64, 1024) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_create(ctypes.byref(p), sos, 9, 1, 32, 64, 1024) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_create(ctypes.byref(p), None, 1, 1, 32, 64, 1024) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_create(ctypes.byref(p), sos, 1, 99, 32, 64, 1024) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_execute(None, None, None, 16, None) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_execute_host(None, None, None, 16, 0, None) == _lib.IIR_ERR_INVALID_ARGUMENT
    assert L.iir_plan_destroy(None) == _lib.IIR_ERR_INVALID_ARGUMENT


def test_header_kernel_ids_match_python():
    text = open(os.path.join(ROOT, "include", "iir_gb300.h")).read()
    for name, val in _lib.KERNELS.items():
        assert f"#define IIR_KERNEL_{name} " in text
        line = [l for l in text.splitlines() if l.startswith(f"#define IIR_KERNEL_{name} ")][0]
        assert int(line.split()[2]) == val


def test_workload_generators_are_seeded():
    from cuda_recursive_filtering_gb300 import workloads
    a = workloads.uniform_signal(1000, 1, device="cpu")
    b = workloads.uniform_signal(1000, 1, device="cpu")
    assert np.array_equal(a.numpy(), b.numpy())
    assert float(a.min()) >= -1.0 and float(a.max()) < 1.0
    sos, x = workloads.plain_order2_small(device="cpu")
    g = np.load(os.path.join(GOLDEN, "sosfilt_order2_uniform.npz"))
    assert np.array_equal(sos, g["sos"]) and np.array_equal(x.numpy()[: g["x"].size], g["x"])


@pytest.mark.parametrize("kind", ("butter", "cheby1"))
def test_generate_reference_files(kind, tmp_path):
    """generate_reference_files writes the reference generator's pair of files: the parsed taps
    reproduce the design, and reference.bin is FP64 sosfilt of the float32 sections and the
    float32 input (tools/ref_generate.py:56-131)."""
    from scipy import signal
    info = formats.generate_reference_files(str(tmp_path), 4, 12, cutoff=0.1, kind=kind)
    taps = formats.parse_filter_taps(str(tmp_path / "filter_taps.hpp"))
    ref = formats.read_reference_bin(str(tmp_path / "reference.bin"))
    assert ref.size == 1 << 12 and taps["n_sections"] == 4 and info["cross_check_rel"] <= 1e-4
    design = formats.design_reference_filter(4, 0.1, kind)
    np.testing.assert_array_equal(taps["sos"], design["sos"])
    assert abs(taps["gain"] - design["gain"]) <= 1e-15 * abs(design["gain"])
    x = formats.reference_input(ref.size, taps["gain"])
    want = signal.sosfilt(taps["sos"].astype(np.float64), x.astype(np.float64)).astype(np.float32)
    np.testing.assert_array_equal(ref, want)
    assert ("Chebyshev" in open(tmp_path / "filter_taps.hpp").read()) == (kind == "cheby1")
