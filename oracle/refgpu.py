"""Test and measurement infrastructure, not part of the product: the reference's own GPU kernels
(PH_32, STCR_32_LOOP, STCR_32_UNROLL_64, DTCR_32_LOOP and DTCR_32_UNROLL_64 of
include/{ph,stcr,dtcr}_kernels.cuh, from Haotian-RA/cuda_recursive_filtering) run on this GPU beside
this library, for a kernel-to-kernel comparison on the same inputs.

The reference configures a kernel at compile time (N_SECTIONS, BLOCK_SIZE, N_BLOCKS as macros) and
prepares it on the host: setup_kernel_coefficients (ph_kernels.cuh:151-200,
dtcr_kernels.cuh:203-289) computes float32 tables and copies them into the module's __constant__ and
__device__ arrays. Here:
  * build_cubins() compiles the reference's headers, where they lie, into device code (one cubin per
    header and number of sections under oracle/_ref/, holding every kernel of the header; the wrapper
    only includes them, as src/test_performance.cu does). It needs the reference's sources, so it
    runs only where they are; elsewhere the cubins are used as they were built, which device code
    allows, as it does not depend on the host's architecture.
  * the host setup is restated below in float32 (ph_tables / cr_tables, following the lines cited
    there) and written into the module with the CUDA driver API (cuModuleGetGlobal, cuMemcpyHtoD);
  * RefKernel launches the kernel under the reference's contract (ph_kernels.cuh:16-29): a status
    buffer zeroed once, the same grid on every launch of a module, launch index 0, 1, 2, ...; so each
    signal length gets its own module (its own ticket counter).
The kernels take b0-normalised sections and an input already multiplied by the cascade's gain, as
the reference's drivers give them (src/test_accuracy.cu:116-124).
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_INCLUDE = "/root/reference/include"  # only where the cubins are built
BLOCK_SIZE, N_BLOCKS = 32, 64
CHUNK = BLOCK_SIZE * N_BLOCKS
SECTIONS = (1, 2, 4, 8)
FAMILIES = {"PH": "ph_kernels.cuh", "STCR": "stcr_kernels.cuh", "DTCR": "dtcr_kernels.cuh"}
# this library's realization name -> (the header's family, the kernel's symbol, threads per block (x, y))
KERNELS = {
    "PH": ("PH", "_Z5PH_32PKfPfPViPVfS5_i", (BLOCK_SIZE, 1)),
    "STCR": ("STCR", "_Z12STCR_32_LOOPPKfPfPViPVfS5_i", (BLOCK_SIZE, 1)),
    "STCR_UNROLL": ("STCR", "_Z17STCR_32_UNROLL_64PKfPfPViPVfS5_i", (BLOCK_SIZE, 1)),
    "DTCR": ("DTCR", "_Z12DTCR_32_LOOPPKfPfPViPVfS5_i", (BLOCK_SIZE, 2)),
    "DTCR_UNROLL": ("DTCR", "_Z17DTCR_32_UNROLL_64PKfPfPViPVfS5_i", (BLOCK_SIZE, 2)),
}
WRAPPER = """#include "iir_utils.hpp"
#include "gpu_specs.hpp"
constexpr int N_TB_PER_SM = gpu_specs::compute_supply_tb_per_sm(BLOCK_SIZE, N_BLOCKS);
#include "{header}"
"""


def cubin_path(family: str, sections: int) -> str:
    return os.path.join(OUT, f"{family.lower()}_k{sections}_{BLOCK_SIZE}x{N_BLOCKS}.cubin")


def available() -> bool:
    return all(os.path.exists(cubin_path(f, s)) for f in FAMILIES for s in SECTIONS)


def build_cubins() -> bool:
    """Compiles every configuration from the reference's sources (sm_103a device code). Returns
    False, changing nothing, where the sources or nvcc are absent (the cubins built earlier are
    then used as they are)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not (os.path.isdir(REF_INCLUDE) and os.path.exists(nvcc)):
        return False
    os.makedirs(OUT, exist_ok=True)

    def one(job):
        family, k = job
        out = cubin_path(family, k)
        src = out[:-6] + ".cu"
        with open(src, "w") as f:
            f.write(WRAPPER.format(header=FAMILIES[family]))
        cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
               "-I", REF_INCLUDE, f"-DN_SECTIONS={k}", f"-DBLOCK_SIZE={BLOCK_SIZE}", f"-DN_BLOCKS={N_BLOCKS}",
               "-o", out, src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference kernel build failed ({family}, {k} sections):\n{r.stderr[-2000:]}")

    with cf.ThreadPoolExecutor(12) as ex:
        list(ex.map(one, [(f, s) for f in FAMILIES for s in SECTIONS]))
    return True


# ------------------------------------------------------------------------------------------------
# host setup of the reference, restated in float32
# ------------------------------------------------------------------------------------------------
f32 = np.float32


def _coeffs(sos_norm):
    """b1, b2, a1, a2 per section from b0-normalised rows (ph_kernels.cuh:157-161)."""
    s = np.asarray(sos_norm, dtype=np.float64).reshape(-1, 6).astype(np.float32)
    return [(f32(r[1]), f32(r[2]), f32(-r[4]), f32(-r[5])) for r in s]


def _impulse(a1, a2, n):
    """h0[0..n]: the recurrence's impulse response from y[-1] = 1 (ph_kernels.cuh:55-68)."""
    h0 = [f32(1.0), f32(a1)]
    for _ in range(2, n + 1):
        h0.append(f32(f32(a1 * h0[-1]) + f32(a2 * h0[-2])))
    h2 = [f32(a2 * h0[m]) for m in range(n)]
    h1 = [h0[m + 1] for m in range(n)]
    return h1, h2


def _mat2(a, b):
    return [f32(f32(a[0] * b[0]) + f32(a[1] * b[2])), f32(f32(a[0] * b[1]) + f32(a[1] * b[3])),
            f32(f32(a[2] * b[0]) + f32(a[3] * b[2])), f32(f32(a[2] * b[1]) + f32(a[3] * b[3]))]


def _cpow(c, n):
    """C^n by binary exponentiation in float32 (C_power, ph_kernels.cuh:70-106)."""
    if n == 1:
        return list(c)
    res, base = [f32(1), f32(0), f32(0), f32(1)], list(c)
    while n > 0:
        if n & 1:
            res = _mat2(res, base)
        base = _mat2(base, base)
        n >>= 1
    return res


def ph_tables(sos_norm) -> dict:
    """The arrays setup_kernel_coefficients fills for PH (ph_kernels.cuh:151-200)."""
    cf_ = _coeffs(sos_norm)
    K = len(cf_)
    t = {name: np.zeros(K, np.float32) for name in ("b1", "b2", "a1", "a2", "xi1", "xi2", "yi1", "yi2")}
    t["h1"] = np.zeros((K, N_BLOCKS), np.float32)
    t["h2"] = np.zeros((K, N_BLOCKS), np.float32)
    t["C_cross"] = np.zeros((K, BLOCK_SIZE, 4), np.float32)
    t["C_inner"] = np.zeros((K, 4 * BLOCK_SIZE), np.float32)
    for s, (b1, b2, a1, a2) in enumerate(cf_):
        t["b1"][s], t["b2"][s], t["a1"][s], t["a2"][s] = b1, b2, a1, a2
        h1, h2 = _impulse(a1, a2, N_BLOCKS)
        t["h1"][s], t["h2"][s] = h1, h2
        c = [h2[N_BLOCKS - 2], h1[N_BLOCKS - 2], h2[N_BLOCKS - 1], h1[N_BLOCKS - 1]]
        for m in range(BLOCK_SIZE):
            p = _cpow(c, m + 1)
            t["C_cross"][s, m] = p
            for j in range(4):
                t["C_inner"][s, j * BLOCK_SIZE + m] = p[j]  # C_power2 with stride BLOCK_SIZE
    return t


def cr_tables(sos_norm, decoupled: bool) -> dict:
    """The arrays setup_kernel_coefficients fills for STCR (stcr_kernels.cuh:93-275) and, with the
    decoupled first-round taps cb .. gb, for DTCR (dtcr_kernels.cuh:108-289): the elimination
    factors of every level, the block-filtering factors and C^(m+1)."""
    L = int(np.log2(N_BLOCKS))
    cf_ = _coeffs(sos_norm)
    K = len(cf_)
    t = {name: np.zeros(K, np.float32) for name in ("b1", "b2", "a1", "a2", "xi1", "xi2", "yi1", "yi2")}
    if decoupled:
        for name in ("cb", "db", "fb", "eb", "hb", "gb"):
            t[name] = np.zeros(K, np.float32)
    for name in ("e", "f", "fde", "cr_h", "cr_g", "cr_p", "cr_q", "cr_d", "cr_c"):
        t[name] = np.zeros((K, L + 1), np.float32)
    for name in ("h0", "hb2", "hb1", "he2", "he1"):
        t[name] = np.zeros((K, BLOCK_SIZE), np.float32)
    t["C_cross"] = np.zeros((K, BLOCK_SIZE, 4), np.float32)
    for s, (b1, b2, a1, a2) in enumerate(cf_):
        t["b1"][s], t["b2"][s], t["a1"][s], t["a2"][s] = b1, b2, a1, a2
        f, e, fde = [f32(0)] * (L + 1), [f32(0)] * (L + 1), [f32(0)] * (L + 1)
        h, g, p, q, d, c = ([f32(0)] * (L + 1) for _ in range(6))
        f[0], e[0] = f32(-a2), f32(-a1)
        fde[0] = f32(f[0] / e[0])
        h[0], g[0] = f[0], e[0]
        p[1], q[1] = f[0], e[0]
        for n in range(1, L + 1):
            f[n] = f32(f[n - 1] * f[n - 1])
            e[n] = f32(f32(2 * f[n - 1]) - f32(e[n - 1] * e[n - 1]))
            fde[n] = f32(f[n] / e[n])
            h[n] = f32(-e[n - 1] * h[n - 1])
            g[n] = f32(f[n - 1] - f32(e[n - 1] * g[n - 1]))
            d[n] = f32(f32(-f[n - 1] * f[n - 1]) / e[n - 1])
            c[n] = f32(e[n - 1] - f32(f[n - 1] / e[n - 1]))
            if n > 1:
                q[n] = f32(-e[n - 1] * q[n - 1])
                p[n] = f32(f[n - 1] - f32(e[n - 1] * p[n - 1]))
        dc = [f32(f32(f[0] * b1) - f32(e[0] * b2)), f32(b1 - e[0]), f32(b2 * f[0]),
              f32(f32(b2 + f[0]) - f32(b1 * e[0])), f32(b2 - f32(e[0] * b1)), f32(-e[0] * b2)]
        if decoupled:
            for name, v in zip(("cb", "db", "fb", "eb", "hb", "gb"), dc):
                t[name][s] = v
        for name, v in (("e", e), ("f", f), ("fde", fde), ("cr_h", h), ("cr_g", g), ("cr_p", p), ("cr_q", q),
                        ("cr_d", d), ("cr_c", c)):
            t[name][s] = v
        # block filtering factors: h0 over the top level's recurrence, head corrections
        h0 = [f32(1), f32(-e[L])]
        for m in range(2, BLOCK_SIZE):
            h0.append(f32(f32(-e[L] * h0[m - 1]) - f32(f[L] * h0[m - 2])))
        t["h0"][s] = h0
        for m in range(BLOCK_SIZE):
            prev = f32(0) if m == 0 else h0[m - 1]
            t["hb2"][s, m] = f32(h[L] * h0[m])
            t["he1"][s, m] = f32(q[L] * h0[m])
            t["hb1"][s, m] = f32(f32(f[L] * prev) + f32(g[L] * h0[m]))
            t["he2"][s, m] = f32(f32(f[L] * prev) + f32(p[L] * h0[m]))
        h1, h2 = _impulse(a1, a2, N_BLOCKS)
        cm = [h2[N_BLOCKS - 2], h1[N_BLOCKS - 2], h2[N_BLOCKS - 1], h1[N_BLOCKS - 1]]
        for m in range(BLOCK_SIZE):
            t["C_cross"][s, m] = _cpow(cm, m + 1)
    return t


# ------------------------------------------------------------------------------------------------
# driver API
# ------------------------------------------------------------------------------------------------
_cu = None


def _driver():
    global _cu
    if _cu is None:
        _cu = ctypes.CDLL("libcuda.so.1")
    return _cu


def _ck(r, what):
    if r != 0:
        raise RuntimeError(f"{what}: CUDA driver error {r}")


class RefKernel:
    """One reference kernel module for one filter and one signal length n (a multiple of the
    chunk, BLOCK_SIZE x N_BLOCKS). Call with device tensors x (gain already applied) and y."""

    def __init__(self, kernel: str, sos_norm, n: int, device="cuda"):
        import torch
        if n <= 0 or n % CHUNK:
            raise ValueError(f"the reference's kernels take whole chunks of {CHUNK} samples")
        family, sym, block = KERNELS[kernel]
        k = np.asarray(sos_norm).reshape(-1, 6).shape[0]
        path = cubin_path(family, k)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        torch.zeros(1, device=device)  # the primary context is current on this thread
        cu = _driver()
        self.mod = ctypes.c_void_p()
        _ck(cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = ctypes.c_void_p()
        _ck(cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, sym.encode()), "cuModuleGetFunction")
        tables = ph_tables(sos_norm) if family == "PH" else cr_tables(sos_norm, decoupled=family == "DTCR")
        for name, arr in tables.items():
            dptr, size = ctypes.c_uint64(), ctypes.c_size_t()
            _ck(cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(size), self.mod, name.encode()),
                f"cuModuleGetGlobal {name}")
            a = np.ascontiguousarray(arr, dtype=np.float32)
            if a.nbytes != size.value:
                raise RuntimeError(f"{name}: {a.nbytes} bytes for a {size.value}-byte symbol")
            _ck(cu.cuMemcpyHtoD_v2(dptr, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes)),
                f"cuMemcpyHtoD {name}")
        self.n, self.k, self.block = n, k, block
        self.grid = n // CHUNK
        self.status = torch.zeros(self.grid * k, dtype=torch.int32, device=device)  # zeroed once
        self.part = torch.zeros(self.grid * 2 * k, dtype=torch.float32, device=device)
        self.full = torch.zeros(self.grid * 2 * k, dtype=torch.float32, device=device)
        self.launch = 0

    def __call__(self, x, y, stream=None) -> None:
        import torch
        if x.numel() != self.n or y.numel() != self.n:
            raise ValueError("a module runs one signal length (its grid is fixed)")
        st = (stream or torch.cuda.current_stream()).cuda_stream
        args = [ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(self.part.data_ptr()),
                ctypes.c_void_p(self.full.data_ptr()), ctypes.c_int(self.launch)]
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        _ck(_driver().cuLaunchKernel(self.fn, ctypes.c_uint(self.grid), 1, 1, ctypes.c_uint(self.block[0]),
                                     ctypes.c_uint(self.block[1]), 1, 0, ctypes.c_void_p(st), params, None),
            "cuLaunchKernel")
        self.launch += 1

    def close(self) -> None:
        if self.mod:
            import torch
            torch.cuda.synchronize()
            _driver().cuModuleUnload(self.mod)
            self.mod = None
