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
                      input_fs: float = INPUT_FS, input_freq: float = INPUT_FREQ, kind: str = "butter") -> None:
    """Writes a header with the same symbols and conventions as the reference's generator."""
    sos_f32 = np.asarray(sos_f32, dtype=np.float32).reshape(-1, 6)
    ns = sos_f32.shape[0]
    rows = ",\n".join("    {" + ", ".join(f"{float(v):.9e}f" for v in r) + "}" for r in sos_f32)
    lines = [
        "// Cascaded-biquad filter taps (b0-normalised float32 sections; FILTER_GAIN must be",
        "// applied to the input). Format of the reference's filter_taps.hpp.",
        f"// {'Chebyshev type I' if kind == 'cheby1' else 'Butterworth'} lowpass, order {2 * ns}, cutoff {cutoff} x Nyquist.",
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


def design_reference_filter(n_sections: int, cutoff: float = REFERENCE_CUTOFF, kind: str = "butter",
                            rp: float = 1.0) -> dict:
    """The reference's test filter: a lowpass of order 2K designed in SOS form plus the
    direct-form taps of the same transfer function for PLR (tools/ref_generate.py:56-81).
    ``kind`` "butter" is the reference's design; "cheby1" (passband ripple ``rp`` dB) follows
    the same conventions (b0-normalised float32 sections, the removed gain applied to the
    input, b0-normalised direct-form taps with the recurrence sign y[n] += A[j] y[n-j-1])."""
    from scipy import signal
    if kind == "butter":
        design = lambda out: signal.butter(N=2 * n_sections, Wn=cutoff, btype="lowpass", output=out)
    elif kind == "cheby1":
        design = lambda out: signal.cheby1(N=2 * n_sections, rp=rp, Wn=cutoff, btype="lowpass", output=out)
    else:
        raise ValueError(f"unknown filter kind {kind!r} (butter, cheby1)")
    sos = design("sos")
    sos_f32, gain = normalise_sos(sos)
    bb, aa = design("ba")
    return {"sos": sos_f32, "gain": gain, "plr_b": bb[1:] / bb[0], "plr_a": -aa[1:], "sos_f64": sos,
            "kind": kind, "cutoff": cutoff}


def generate_reference_files(out_dir: str, n_sections: int, n_samples_log2: int, cutoff: float = REFERENCE_CUTOFF,
                             kind: str = "butter", rp: float = 1.0) -> dict:
    """Writes ``reference.bin`` and ``filter_taps.hpp`` into ``out_dir`` the way the reference's
    generator does (tools/ref_generate.py:56-131): the input is the accuracy test's cosine
    scaled by the removed gain, the golden output is FP64 sosfilt of the float32 sections and
    float32 input, and it is cross-checked (relative 1e-4) against the unnormalised design."""
    import os

    from scipy import signal
    f = design_reference_filter(n_sections, cutoff, kind, rp)
    n = 1 << n_samples_log2
    x = reference_input(n, f["gain"])
    ref = signal.sosfilt(f["sos"].astype(np.float64), x.astype(np.float64))
    i = np.arange(n, dtype=np.float64)
    check = signal.sosfilt(f["sos_f64"], np.cos(2.0 * np.pi * INPUT_FREQ * i / INPUT_FS))
    rel = float(np.max(np.abs(ref - check)) / max(np.max(np.abs(check)), 1e-30))
    if rel > 1e-4:
        raise RuntimeError(f"normalisation cross-check failed: relative {rel:.3e}")
    os.makedirs(out_dir, exist_ok=True)
    write_reference_bin(os.path.join(out_dir, "reference.bin"), ref)
    write_filter_taps(os.path.join(out_dir, "filter_taps.hpp"), f["sos"], f["gain"], f["plr_b"], f["plr_a"],
                      cutoff=cutoff, kind=kind)
    return {"n": n, "gain": f["gain"], "cross_check_rel": rel}


def check_reference_files(taps_path: str, ref_path: str, kernel: str = "DTCR_UNROLL", block_size: int = 0,
                          n_blocks: int = 0, device=None) -> dict:
    """The reference's accuracy driver (src/test_accuracy.cu:116-188) on this library: the
    input is rebuilt from filter_taps.hpp, filtered on the GPU (``kernel``; "PLR" uses the
    direct-form taps), and compared with reference.bin by the reference's gate
    max|err| <= 1e-4 * max|ref|. Returns the errors and the verdict."""
    import torch

    from .api import Plan, PlrPlan
    taps = parse_filter_taps(taps_path)
    ref = read_reference_bin(ref_path).astype(np.float64)
    n = ref.size
    x = torch.from_numpy(reference_input(n, taps["gain"], taps["input_fs"], taps["input_freq"]))
    x = x.to(device if device is not None else "cuda")
    if kernel.upper() == "PLR":
        # the direct-form lane: b0-normalised taps, the gain already in the input
        plan = PlrPlan(taps["plr_b"], taps["plr_a"], 1.0, block_size, n_blocks, max_n=n, device=x.device)
    else:
        # the sections are b0-normalised with FILTER_GAIN applied to the input, as in the reference
        plan = Plan(taps["sos"], kernel, block_size, n_blocks, max_n=n, device=x.device)
    y = plan(x)
    plan.check()
    out = y.cpu().numpy().astype(np.float64)
    plan.close()
    err = np.abs(out - ref)
    finite = bool(np.all(np.isfinite(out)))
    mref = float(np.max(np.abs(ref))) if n else 0.0
    max_abs = float(np.max(err)) if (n and finite) else (0.0 if not n else float("inf"))
    rel_max = max_abs / max(mref, 1e-30)
    return {"kernel": kernel.upper(), "n": n, "max_abs": max_abs, "rel_max": rel_max, "finite": finite,
            "pass": finite and rel_max <= 1e-4}


def main(argv=None) -> int:
    """Command line: ``generate`` writes reference.bin and filter_taps.hpp (the reference's
    generator), ``check`` runs one realization against them (the reference's accuracy driver)."""
    import argparse
    import json
    import os
    ap = argparse.ArgumentParser(prog="python -m cuda_recursive_filtering_gb300.formats")
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate")
    g.add_argument("--out", required=True)
    g.add_argument("--n-sections", type=int, required=True)
    g.add_argument("--n-samples-log2", type=int, default=16)
    g.add_argument("--cutoff", type=float, default=REFERENCE_CUTOFF)
    g.add_argument("--kind", default="butter", choices=("butter", "cheby1"))
    g.add_argument("--rp", type=float, default=1.0)
    c = sub.add_parser("check")
    c.add_argument("--dir", required=True, help="folder with reference.bin and filter_taps.hpp")
    c.add_argument("--kernel", default="DTCR_UNROLL")
    c.add_argument("--block-size", type=int, default=0)
    c.add_argument("--n-blocks", type=int, default=0)
    a = ap.parse_args(argv)
    if a.cmd == "generate":
        info = generate_reference_files(a.out, a.n_sections, a.n_samples_log2, a.cutoff, a.kind, a.rp)
        print(json.dumps(info))
        return 0
    res = check_reference_files(os.path.join(a.dir, "filter_taps.hpp"), os.path.join(a.dir, "reference.bin"),
                                a.kernel, a.block_size, a.n_blocks)
    print(json.dumps(res))
    return 0 if res["pass"] else 1


if __name__ == "__main__":
    raise SystemExit(main())

