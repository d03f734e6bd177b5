"""CPU oracle for the cascaded-biquad IIR path — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference legs may import
this package, and only to check results (or to time the reference's CPU golden path). The
library in ``cuda_recursive_filtering_gb300`` never imports it and has no CPU fallback.

Contents (each restated from the reference's behaviour; C sources in iir_oracle.c):
  * ``sosfilt_f64``     — FP64 cascade, the golden output of tools/ref_generate.py:89
                          (scipy.signal.sosfilt on float32-rounded normalised sections).
  * ``direct_f32``      — float32 sequential direct form (tools/plr_emulator.py:185-202).
  * ``cascade_f32``     — float32 sequential cascade in the kernels' coefficient convention.
  * ``merge_sections``  — normalised SOS -> one direct-form (b, a) pair (PLR route).
  * ``normalise_sos``   — b0/a0 normalisation + removed gain (tools/ref_generate.py:62-67).
  * accuracy metrics: the reference's gate max|err| <= 1e-4 * max|ref|
    (src/test_accuracy.cu:178-188) and max|err| / RMS(ref).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "iir_oracle.c")

REF_REL_TOL = 1e-4  # src/test_accuracy.cu:178


def build() -> str:
    """Compiles iir_oracle.c with gcc (host code only, portable C)."""
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, SRC, "-lm"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_sosfilt_f64.argtypes = [dp, ctypes.c_longlong, dp, ctypes.c_int, dp]
        L.oracle_direct_f32.argtypes = [fp, ctypes.c_longlong, fp, fp, ctypes.c_int, fp]
        L.oracle_cascade_f32.argtypes = [fp, ctypes.c_longlong, fp, ctypes.c_int, fp]
        L.oracle_normalise_sos.argtypes = [dp, ctypes.c_int, dp]
        L.oracle_normalise_sos.restype = ctypes.c_double
        L.oracle_merge_sections.argtypes = [dp, ctypes.c_int, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def sosfilt_f64(sos, x) -> np.ndarray:
    """FP64 cascade of `sos` (rows b0 b1 b2 a0 a1 a2) over x, zero initial state."""
    sos = np.ascontiguousarray(sos, dtype=np.float64).reshape(-1, 6)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib().oracle_sosfilt_f64(_dp(x), x.size, _dp(sos), sos.shape[0], _dp(y))
    return y


def direct_f32(x, b, a) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    a = np.ascontiguousarray(a, dtype=np.float32)
    y = np.empty_like(x)
    lib().oracle_direct_f32(_fp(x), x.size, _fp(b), _fp(a), b.size, _fp(y))
    return y


def cascade_f32(x_scaled, sos_norm_f32) -> np.ndarray:
    """float32 cascade of normalised rows (b0 = a0 = 1) over an already gain-scaled input."""
    s = np.asarray(sos_norm_f32, dtype=np.float32).reshape(-1, 6)
    coef = np.ascontiguousarray(np.stack([s[:, 1], s[:, 2], -s[:, 4], -s[:, 5]], axis=1), dtype=np.float32)
    x = np.ascontiguousarray(x_scaled, dtype=np.float32)
    y = np.empty_like(x)
    lib().oracle_cascade_f32(_fp(x), x.size, _fp(coef), s.shape[0], _fp(y))
    return y


def normalise_sos(sos):
    sos = np.ascontiguousarray(sos, dtype=np.float64).reshape(-1, 6)
    out = np.empty_like(sos)
    g = lib().oracle_normalise_sos(_dp(sos), sos.shape[0], _dp(out))
    return out, float(g)


def merge_sections(sos_norm):
    s = np.ascontiguousarray(sos_norm, dtype=np.float64).reshape(-1, 6)
    k = 2 * s.shape[0]
    b = np.empty(k, np.float64)
    a = np.empty(k, np.float64)
    lib().oracle_merge_sections(_dp(s), s.shape[0], _dp(b), _dp(a))
    return b, a


def reference_golden(sos, x_f32) -> np.ndarray:
    """The reference's golden: FP64 filtering of the float32 input through the float32-rounded
    normalised sections, gain applied to the input in FP64 then rounded to float32
    (tools/ref_generate.py:62-99). Returns (device_input_f32, golden_f64)."""
    norm, g = normalise_sos(sos)
    sos_f32 = norm.astype(np.float32).astype(np.float64)
    x_dev = (np.float64(g) * np.asarray(x_f32, np.float64)).astype(np.float32)
    return x_dev, sosfilt_f64(sos_f32, x_dev.astype(np.float64))


def errors(out, ref) -> dict:
    """max|err|, max|err|/max|ref| (reference gate, 1e-4) and max|err|/RMS(ref)."""
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    if not np.all(np.isfinite(out)):
        return {"max_abs": float("inf"), "rel_max": float("inf"), "rel_rms": float("inf"), "finite": False}
    err = float(np.max(np.abs(out - ref))) if out.size else 0.0
    mref = float(np.max(np.abs(ref))) if ref.size else 0.0
    rms = float(np.sqrt(np.mean(ref * ref))) if ref.size else 0.0
    return {"max_abs": err, "rel_max": err / max(mref, 1e-30), "rel_rms": err / max(rms, 1e-30), "finite": True}


def passes_reference_gate(out, ref) -> bool:
    e = errors(out, ref)
    return e["finite"] and e["rel_max"] <= REF_REL_TOL


REL_TOL_GATE = REF_REL_TOL
