"""The reference's harness formats and test-filter conventions.

* ``reference.bin`` — raw little-endian float32 golden output (tools/ref_generate.py:97,
  read by src/test_accuracy.cu:161-176).
* ``filter_taps.hpp`` — C header with FILTER_N_SECTIONS, FILTER_GAIN, INPUT_FS, INPUT_FREQ,
  FILTER_SOS[K][6] (b0-normalised float32 rows) and the PLR direct-form pair
  PLR_FILTER_ORDER / PLR_FILTER_B / PLR_FILTER_A (tools/ref_generate.py:101-131).
* the accuracy-test input x[i] = float32(FILTER_GAIN * cos(2*pi*INPUT_FREQ*i/INPUT_FS))
  (src/test_accuracy.cu:116-124).
"""
from __future__ import annotations

import re

import numpy as np

INPUT_FS = 1000.0
INPUT_FREQ = 120.0
REFERENCE_CUTOFF = 0.2


def read_reference_bin(path: str, n: int | None = None) -> np.ndarray:
    data = np.fromfile(path, dtype="<f4")
    if n is not None:
        if data.size < n:
            raise ValueError(f"{path} holds {data.size} floats, expected {n}")
        data = data[:n]
    return data


def write_reference_bin(path: str, y) -> None:
    np.asarray(y, dtype=np.float64).astype("<f4").tofile(path)


def _c_array(text: str, name: str) -> list[float]:
    m = re.search(name + r"\s*\[[^\]]*\](?:\s*\[[^\]]*\])?\s*=\s*\{(.*?)\};", text, flags=re.S)
    if not m:
        raise ValueError(f"{name} not found")
    body = m.group(1).replace("{", " ").replace("}", " ")
    return [float(t.rstrip("f")) for t in re.findall(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?f?", body)]


def _c_scalar(text: str, name: str, define: bool = False) -> float:
    pat = (r"#define\s+" + name + r"\s+([-+0-9.eE]+)") if define else (name + r"\s*=\s*([-+0-9.eE]+)\s*;")
    m = re.search(pat, text)
    if not m:
        raise ValueError(f"{name} not found")
    return float(m.group(1))


def parse_filter_taps(path: str) -> dict:
    """Parses a filter_taps.hpp written by the reference's tools/ref_generate.py."""
    text = open(path).read()
    ns = int(_c_scalar(text, "FILTER_N_SECTIONS", define=True))
    sos = np.array(_c_array(text, "FILTER_SOS"), dtype=np.float32).reshape(ns, 6)
    out = {
        "n_sections": ns,
        "gain": _c_scalar(text, "FILTER_GAIN"),
        "input_fs": _c_scalar(text, "INPUT_FS"),
        "input_freq": _c_scalar(text, "INPUT_FREQ"),
        "sos": sos,
    }
    if "PLR_FILTER_ORDER" in text:
        out["plr_order"] = int(_c_scalar(text, "PLR_FILTER_ORDER", define=True))
        out["plr_b"] = np.array(_c_array(text, "PLR_FILTER_B"), dtype=np.float64)
        out["plr_a"] = np.array(_c_array(text, "PLR_FILTER_A"), dtype=np.float64)
    return out


def write_filter_taps(path: str, sos_f32, gain: float, plr_b=None, plr_a=None, cutoff: float = REFERENCE_CUTOFF,
                      input_fs: float = INPUT_FS, input_freq: float = INPUT_FREQ) -> None:
    """Writes a header with the same symbols and conventions as the reference's generator."""
    sos_f32 = np.asarray(sos_f32, dtype=np.float32).reshape(-1, 6)
    ns = sos_f32.shape[0]
    rows = ",\n".join("    {" + ", ".join(f"{float(v):.9e}f" for v in r) + "}" for r in sos_f32)
    lines = [
        "// Cascaded-biquad filter taps (b0-normalised float32 sections; FILTER_GAIN must be",
        "// applied to the input). Format of the reference's filter_taps.hpp.",
        f"// Lowpass, order {2 * ns}, cutoff {cutoff} x Nyquist.",
        "#pragma once",
        "",
        f"#define FILTER_N_SECTIONS {ns}",
        f"static const double FILTER_GAIN = {float(gain)!r};",
        f"static const double INPUT_FS    = {float(input_fs)!r};",
        f"static const double INPUT_FREQ  = {float(input_freq)!r};",
        "",
        f"static const float FILTER_SOS[{ns}][6] = {{",
        rows,
        "};",
    ]
    if plr_b is not None and plr_a is not None:
        k = len(plr_b)
        lines += [
            "",
            f"#define PLR_FILTER_ORDER {k}",
            f"static const double PLR_FILTER_B[{k}] = {{",
            "    " + ",\n    ".join(repr(float(v)) for v in plr_b),
            "};",
            f"static const double PLR_FILTER_A[{k}] = {{",
            "    " + ",\n    ".join(repr(float(v)) for v in plr_a),
            "};",
        ]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def reference_input(n: int, gain: float, input_fs: float = INPUT_FS, input_freq: float = INPUT_FREQ) -> np.ndarray:
    """x[i] = float32(gain * cos(2 pi f i / fs)), computed in float64 (src/test_accuracy.cu:120-124)."""
    i = np.arange(n, dtype=np.float64)
    return (gain * np.cos(2.0 * np.pi * input_freq * i / input_fs)).astype(np.float32)


def normalise_sos(sos) -> tuple[np.ndarray, float]:
    """b0-normalised float32 rows and the removed FP64 gain (tools/ref_generate.py:62-67)."""
    s = np.asarray(sos, dtype=np.float64).reshape(-1, 6).copy()
    gain = float(np.prod(s[:, 0] / s[:, 3]))
    s[:, 0:3] /= s[:, 0:1]
    s[:, 3:6] /= s[:, 3:4]
    return s.astype(np.float32), gain


def design_reference_filter(n_sections: int, cutoff: float = REFERENCE_CUTOFF) -> dict:
    """The reference's test filter: Butterworth lowpass of order 2K designed in SOS form plus
    the direct-form taps of the same transfer function for PLR (tools/ref_generate.py:56-81)."""
    from scipy import signal
    sos = signal.butter(N=2 * n_sections, Wn=cutoff, btype="lowpass", output="sos")
    sos_f32, gain = normalise_sos(sos)
    bb, aa = signal.butter(N=2 * n_sections, Wn=cutoff, btype="lowpass", output="ba")
    return {"sos": sos_f32, "gain": gain, "plr_b": bb[1:] / bb[0], "plr_a": -aa[1:], "sos_f64": sos}
