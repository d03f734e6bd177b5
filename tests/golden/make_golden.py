"""Generates the golden fixtures under tests/golden/ from the reference's own Python tools.

Run once in a checkout where the reference repository is available (it is not needed at test
time; the fixtures are committed):

    python tests/golden/make_golden.py /path/to/cuda_recursive_filtering

What it produces (all small):
  ref_order{2,4,8,16}/reference.bin, filter_taps.hpp
      written by the reference's tools/ref_generate.py itself (its on-disk formats:
      float32 golden output of FP64 sosfilt, and the C header with FILTER_SOS / FILTER_GAIN /
      PLR_FILTER_B / PLR_FILTER_A), N_SAMPLES_LOG2 = 12.
  emulators.npz
      outputs of the reference's float32 emulators on their own 3-chunk cosine inputs:
        stcr_{order}_{B}x{N}   tools/stcr_emulator.py stcr(..., 'loop')
        dtcr_{order}_{B}x{N}   tools/dtcr_emulator.py dtcr(...)
        plr2_{B}_{X}           tools/plr_emulator.py plr_pass(...) (order 2, with a ragged tail)
        direct_{order}         tools/plr_emulator.py direct_form_f32 on 2^12 samples
      plus the matching inputs (x_*) and float64 references (ref_*).
  sosfilt_order2_uniform.npz
      butter(2, 0.1) on 2^14 samples of uniform[-1,1] from seed 0, with
      scipy.signal.sosfilt's FP64 output, and the scipy version used.
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(ref_root: str, name: str):
    path = os.path.join(ref_root, "tools", name + ".py")
    spec = importlib.util.spec_from_file_location("ref_" + name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_ref_generate(ref_root: str) -> None:
    script = os.path.join(ref_root, "tools", "ref_generate.py")
    for ns in (1, 2, 4, 8):
        out_dir = os.path.join(HERE, f"ref_order{2 * ns}")
        os.makedirs(out_dir, exist_ok=True)
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([sys.executable, script, "--n-samples-log2", "12", "--n-sections", str(ns),
                            "--output", os.path.join(td, "reference.bin"),
                            "--header", os.path.join(td, "filter_taps.hpp"), "--quiet"], check=True)
            for f in ("reference.bin", "filter_taps.hpp"):
                shutil.copy(os.path.join(td, f), os.path.join(out_dir, f))


def make_emulators(ref_root: str) -> None:
    stcr = _load(ref_root, "stcr_emulator")
    dtcr = _load(ref_root, "dtcr_emulator")
    plr = _load(ref_root, "plr_emulator")
    F32 = np.float32
    out: dict[str, np.ndarray] = {}
    for ns in (1, 2, 4, 8):
        order = 2 * ns
        sos, g = stcr.butter_norm_sos(ns)
        out[f"sos_{order}"] = sos
        out[f"gain_{order}"] = np.array(g, np.float64)
        for (B, N) in ((32, 32), (32, 64), (32, 128), (64, 64)):
            n = 3 * B * N
            x = np.array([np.cos(2 * np.pi * 120 * i / 1000.0) for i in range(n)], F32)
            out[f"x_stcr_{order}_{B}x{N}"] = x
            out[f"stcr_{order}_{B}x{N}"] = stcr.stcr(x, sos, g, B, N, "loop")
            out[f"ref_stcr_{order}_{B}x{N}"] = stcr.reference(x, sos, g)
            i = np.arange(n, dtype=np.float64)
            xd = (g * np.cos(2.0 * np.pi * 120.0 * i / 1000.0)).astype(F32)
            out[f"x_dtcr_{order}_{B}x{N}"] = xd
            out[f"dtcr_{order}_{B}x{N}"] = dtcr.dtcr(xd, sos, B, N, B == 64)
        print(f"order {order}: stcr/dtcr done", flush=True)
    bt, at, g = plr.butter_ba_norm(2)
    for B in (512, 1024):
        for X in (1, 4, 9, 10):
            n = 3 * B * X + B // 2
            i = np.arange(n, dtype=np.float64)
            x = (g * np.cos(2.0 * np.pi * 120.0 * i / 1000.0)).astype(F32)
            out[f"x_plr2_{B}_{X}"] = x
            out[f"plr2_{B}_{X}"] = plr.plr_pass(x, F32(bt[0]), F32(bt[1]), F32(at[0]), F32(at[1]), B, X, n)
    n = 1 << 12
    i = np.arange(n, dtype=np.float64)
    for order in (2, 4, 8, 16):
        bt, at, g = plr.butter_ba_norm(order)
        x = (g * np.cos(2.0 * np.pi * 120.0 * i / 1000.0)).astype(F32)
        out[f"x_direct_{order}"] = x
        out[f"b_direct_{order}"] = bt
        out[f"a_direct_{order}"] = at
        with np.errstate(over="ignore", invalid="ignore"):
            out[f"direct_{order}"] = plr.direct_form_f32(x, bt, at)
        out[f"ref_direct_{order}"] = plr.reference_f64(x, order)
    np.savez_compressed(os.path.join(HERE, "emulators.npz"), **out)


def make_sosfilt_order2_uniform() -> None:
    import scipy
    from scipy import signal
    sos = signal.butter(2, 0.1, output="sos")
    x = np.random.default_rng(0).uniform(-1.0, 1.0, 1 << 14).astype(np.float32)
    y = signal.sosfilt(sos, x.astype(np.float64))
    np.savez_compressed(os.path.join(HERE, "sosfilt_order2_uniform.npz"), sos=sos, x=x, y=y,
                        scipy_version=np.array(scipy.__version__))


def main() -> None:
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("IIR_REFERENCE_ROOT", "")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "tools")):
        sys.exit("usage: make_golden.py <reference checkout>")
    make_ref_generate(ref_root)
    make_sosfilt_order2_uniform()
    make_emulators(ref_root)


if __name__ == "__main__":
    main()
