"""Python mirror of the reference's filtering interface, on top of the C ABI.

Reference surface (header-only CUDA, compile-time configured):
  setup_kernel_coefficients(sos)               include/ph_kernels.cuh:151 (and stcr/dtcr/plr)
  KERNEL_FUNC<<<grid, block>>>(in, out, status, partcarry, fullcarry, launch)
                                               src/test_accuracy.cu:146
Here a :class:`Plan` owns what the reference's caller allocated (status / carries / launch
index); realization and BLOCK_SIZE x N_BLOCKS are constructor arguments. Device memory and
streams come from PyTorch; the filtering itself is the CUDA library (no fallback).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import KERNELS, KERNEL_NAMES, IirError, check

__all__ = ["Plan", "PlrPlan", "Batch", "sosfilt", "KERNELS", "IirError"]


def _kernel_id(kernel) -> int:
    if isinstance(kernel, str):
        k = kernel.upper()
        if k not in KERNELS:
            raise ValueError(f"unknown realization {kernel!r}; one of {sorted(KERNELS)}")
        return KERNELS[k]
    return int(kernel)


def _sos_array(sos) -> np.ndarray:
    s = np.ascontiguousarray(np.asarray(sos, dtype=np.float32).reshape(-1, 6))
    if s.shape[0] < 1:
        raise ValueError("sos needs at least one section")
    return s


def _stream_handle(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(int(stream.cuda_stream))


def _check_tensor(x: torch.Tensor, name: str) -> None:
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if x.dtype != torch.float32:
        raise TypeError(f"{name} must be float32")
    if not x.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


class Plan:
    """A filter bound to a realization and geometry (the reference's compile-time choice).

    Parameters mirror the reference's build variables: ``kernel`` = KERNEL (PH / STCR /
    STCR_UNROLL / DTCR / DTCR_UNROLL / PLR / AUTO), ``block_size`` = BLOCK_SIZE,
    ``n_blocks`` = N_BLOCKS (PLR: values per thread), 0 = tuned default.
    The plan's status buffer is zeroed once here and never reset (launch-versioned flags).
    Launches must be issued from one stream at a time.
    """

    def __init__(self, sos, kernel="AUTO", block_size: int = 0, n_blocks: int = 0, max_n: int = 1 << 20,
                 device=None):
        self._lib = _lib.load()
        self._sos = _sos_array(sos)
        self._ptr = ctypes.c_void_p()
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.device = dev
        with torch.cuda.device(dev):
            st = self._lib.iir_plan_create(ctypes.byref(self._ptr),
                                           self._sos.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           self._sos.shape[0], _kernel_id(kernel), int(block_size), int(n_blocks),
                                           int(max_n))
        check(st, "iir_plan_create")

    @classmethod
    def _from_ptr(cls, ptr, device):
        obj = cls.__new__(cls)
        obj._lib = _lib.load()
        obj._ptr = ptr
        obj.device = device
        obj._sos = None
        return obj

    def info(self) -> dict:
        vals = [ctypes.c_int() for _ in range(5)]
        check(self._lib.iir_plan_info(self._ptr, *[ctypes.byref(v) for v in vals]), "iir_plan_info")
        k, b, n, g, s = (v.value for v in vals)
        return {"kernel": KERNEL_NAMES.get(k, k), "block_size": b, "n_blocks": n, "grid": g, "n_sections": s}

    def __call__(self, x: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        _check_tensor(x, "x")
        if out is None:
            out = torch.empty_like(x)
        _check_tensor(out, "out")
        if out.numel() != x.numel():
            raise ValueError("out must have as many samples as x")
        st = self._lib.iir_plan_execute(self._ptr, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                        x.numel(), _stream_handle(stream))
        check(st, "iir_plan_execute")
        return out

    def filter_host(self, x: torch.Tensor, out: torch.Tensor | None = None, piece: int = 0,
                    stream=None) -> torch.Tensor:
        """The filter over HOST float32 tensors (C ABI: iir_plan_execute_host). Pinned tensors
        give overlapped copies; single-section plans on the two-pass schedule run in pieces
        of ``piece`` samples (0 = 2^24), each starting from the state the previous left.
        Stream-ordered: ``out`` is complete once ``stream`` (default: the current stream) is."""
        for name, t in (("x", x), ("out", out)):
            if t is None:
                continue
            if t.device.type != "cpu" or t.dtype != torch.float32 or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous float32 host tensor")
        if out is None:
            out = torch.empty(x.numel(), dtype=torch.float32, pin_memory=x.is_pinned())
        if out.numel() != x.numel():
            raise ValueError("out must have as many samples as x")
        st = self._lib.iir_plan_execute_host(self._ptr, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), x.numel(), int(piece),
                                             _stream_handle(stream))
        check(st, "iir_plan_execute_host")
        return out

    def launches_per_execute(self) -> int:
        return int(self._lib.iir_plan_launches_per_execute(self._ptr))

    def check(self, stream=None) -> None:
        """Synchronises the stream and raises IirError if a launch recorded a device error."""
        check(self._lib.iir_plan_check(self._ptr, _stream_handle(stream)), "device")

    def set_timeout_ns(self, ns: int) -> None:
        check(self._lib.iir_plan_set_timeout_ns(self._ptr, int(ns)))

    def debug_withhold(self, chunk: int) -> None:
        check(self._lib.iir_plan_debug_withhold(self._ptr, int(chunk)))

    def close(self) -> None:
        if getattr(self, "_ptr", None) is not None and self._ptr.value:
            self._lib.iir_plan_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlrPlan(Plan):
    """PLR plan from direct-form taps (filter_taps.hpp PLR_FILTER_B / PLR_FILTER_A)."""

    def __init__(self, b, a, gain: float = 1.0, block_size: int = 0, values_per_thread: int = 0,
                 max_n: int = 1 << 20, device=None):
        self._lib = _lib.load()
        self._sos = None
        b = np.ascontiguousarray(b, dtype=np.float64)
        a = np.ascontiguousarray(a, dtype=np.float64)
        if b.shape != a.shape:
            raise ValueError("b and a must have the same length (the order)")
        self._ptr = ctypes.c_void_p()
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.device = dev
        dp = ctypes.POINTER(ctypes.c_double)
        with torch.cuda.device(dev):
            st = self._lib.iir_plan_create_plr_ba(ctypes.byref(self._ptr), b.ctypes.data_as(dp), a.ctypes.data_as(dp),
                                                  b.size, float(gain), int(block_size), int(values_per_thread),
                                                  int(max_n))
        check(st, "iir_plan_create_plr_ba")


def sosfilt(sos, x: torch.Tensor, kernel="AUTO", block_size: int = 0, n_blocks: int = 0,
            out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """One-shot cascaded-biquad filtering of a CUDA float32 signal (zero initial state).

    ``sos`` rows are scipy's {b0, b1, b2, a0, a1, a2}; they are normalised in FP64 and the
    removed gain is applied to the input. Plans are cached per (stream, filter, realization).
    """
    lib = _lib.load()
    s = _sos_array(sos)
    _check_tensor(x, "x")
    if out is None:
        out = torch.empty_like(x)
    _check_tensor(out, "out")
    st = lib.iir_sos_filter_geom(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), x.numel(),
                                 s.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), s.shape[0], _kernel_id(kernel),
                                 int(block_size), int(n_blocks), _stream_handle(stream))
    check(st, "iir_sos_filter")
    return out


class Batch:
    """Many independent signals in one launch (C ABI: iir_batch_*), each with its own filter.

    ``filters`` is a list of SOS arrays (scipy rows), one per distinct filter. A call takes a
    list of segments ``(x, y, filter_index, zi, zf)``: CUDA float32 tensors for input and
    output, the filter's index, and optional device state in / out tensors of
    ``state_size(filter)`` floats (None = start at rest / do not report). Segments are filtered
    independently (PH solve; chunks of 8192 samples; the lookback stays inside a segment).
    State layout: x[-2], x[-1] of the raw input, then each section's y[-2], y[-1].
    """

    def __init__(self, filters, max_segments: int = 1024, max_chunks: int = 1 << 16, device=None):
        self._lib = _lib.load()
        soss = [_sos_array(f) for f in filters]
        if not soss:
            raise ValueError("at least one filter")
        self.n_sections = [int(s.shape[0]) for s in soss]
        flat = np.ascontiguousarray(np.concatenate(soss, axis=0), np.float32)
        ns = (ctypes.c_int * len(soss))(*self.n_sections)
        self._ptr = ctypes.c_void_p()
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.device = dev
        with torch.cuda.device(dev):
            st = self._lib.iir_batch_create(ctypes.byref(self._ptr), flat.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                            ns, len(soss), int(max_segments), int(max_chunks))
        check(st, "iir_batch_create")

    def state_size(self, filter_index: int) -> int:
        return 2 + 2 * self.n_sections[filter_index]

    SHAPES = ((128, 64), (128, 32), (128, 16), (64, 16))  # rows x samples per row (compiled)

    def set_shape(self, rows: int, samples_per_row: int) -> None:
        """Chunk shape of later launches (C ABI: iir_batch_set_shape); one of SHAPES."""
        check(self._lib.iir_batch_set_shape(self._ptr, int(rows), int(samples_per_row)), "iir_batch_set_shape")

    def shape(self) -> dict:
        """The current chunk shape: rows, samples_per_row, chunk, and its kernel's threads,
        registers per thread, shared memory per block and resident blocks per SM."""
        v = [ctypes.c_int() for _ in range(6)]
        check(self._lib.iir_batch_get_shape(self._ptr, *[ctypes.byref(t) for t in v]), "iir_batch_get_shape")
        r, n, th, rg, sm, b = (t.value for t in v)
        return {"rows": r, "samples_per_row": n, "chunk": r * n, "threads": th, "regs_per_thread": rg,
                "smem_bytes": sm, "blocks_per_sm": b}

    def __call__(self, segments, stream=None) -> None:
        arr = (_lib.IirSegment * max(1, len(segments)))()
        for i, seg in enumerate(segments):
            x, y, f = seg[0], seg[1], int(seg[2])
            zi = seg[3] if len(seg) > 3 else None
            zf = seg[4] if len(seg) > 4 else None
            _check_tensor(x, "x")
            _check_tensor(y, "y")
            if y.numel() != x.numel():
                raise ValueError("y must have as many samples as x")
            for z, name in ((zi, "zi"), (zf, "zf")):
                if z is not None:
                    _check_tensor(z, name)
                    if z.numel() != self.state_size(f):
                        raise ValueError(f"{name} must hold {self.state_size(f)} floats")
            arr[i] = _lib.IirSegment(x.data_ptr(), y.data_ptr(), x.numel(), f,
                                     zi.data_ptr() if zi is not None else None,
                                     zf.data_ptr() if zf is not None else None)
        check(self._lib.iir_batch_execute(self._ptr, arr, len(segments), _stream_handle(stream)), "iir_batch_execute")

    _SEG_DTYPE = np.dtype({"names": ["x", "y", "n", "filter", "zi", "zf"],
                           "formats": [np.uint64, np.uint64, np.uint64, np.int32, np.uint64, np.uint64],
                           "offsets": [0, 8, 16, 24, 32, 40], "itemsize": 48})

    def packed(self, x: torch.Tensor, y: torch.Tensor, offsets, filters, zi: torch.Tensor | None = None,
               zf: torch.Tensor | None = None, stream=None) -> None:
        """Segments packed back to back: segment i is x[offsets[i]:offsets[i+1]] -> y[...],
        filtered with filters[i]. Optional zi / zf are (n_segments, state_len) device tensors
        whose row i holds segment i's state (state_len = the largest state_size of the used
        filters; rows are read / written up to the segment's own state size). The segment
        table is built with array operations, so this path costs no per-segment Python work."""
        _check_tensor(x, "x")
        _check_tensor(y, "y")
        if y.numel() != x.numel():
            raise ValueError("y must have as many samples as x")
        off = np.asarray(offsets, dtype=np.int64)
        flt = np.asarray(filters, dtype=np.int32)
        nseg = flt.size
        tab = self._packed_table(x, y, off, flt, nseg, zi, zf)
        self.execute_table(tab, nseg, stream)

    def segment_table(self, n: int) -> np.ndarray:
        """An empty segment table (numpy structured array laid out as iir_segment) of n rows,
        for callers that fill pointers themselves (see execute_table)."""
        return np.zeros(max(n, 1), dtype=self._SEG_DTYPE)

    def execute_table(self, tab: np.ndarray, n: int, stream=None) -> None:
        """Launches the first n rows of a segment table (fields x, y, n, filter, zi, zf as
        device addresses / counts, as iir_segment)."""
        if tab.dtype != self._SEG_DTYPE or tab.size < n:
            raise ValueError("segment table of the wrong layout or size")
        st = self._lib.iir_batch_execute(self._ptr, tab.ctypes.data_as(ctypes.POINTER(_lib.IirSegment)), int(n),
                                         _stream_handle(stream))
        check(st, "iir_batch_execute")

    def bind(self, x: torch.Tensor, y: torch.Tensor, offsets, filters, zi=None, zf=None) -> "BoundBatch":
        """Packed segments (as :meth:`packed`) uploaded once; the returned object launches
        them with a single kernel launch per call, which CUDA graphs can capture."""
        _check_tensor(x, "x")
        _check_tensor(y, "y")
        off = np.asarray(offsets, dtype=np.int64)
        flt = np.asarray(filters, dtype=np.int32)
        tab = self._packed_table(x, y, off, flt, flt.size, zi, zf)
        h = ctypes.c_void_p()
        check(self._lib.iir_batch_bind(self._ptr, tab.ctypes.data_as(ctypes.POINTER(_lib.IirSegment)), flt.size,
                                       ctypes.byref(h)), "iir_batch_bind")
        return BoundBatch(self, h, (x, y, zi, zf))

    def _packed_table(self, x, y, off, flt, nseg, zi, zf):
        if off.shape != (nseg + 1,) or (nseg and (off[0] < 0 or off[-1] > x.numel() or np.any(np.diff(off) < 0))):
            raise ValueError("offsets must be nondecreasing, n_segments + 1 long, within x")
        if nseg and (flt.min() < 0 or flt.max() >= len(self.n_sections)):
            raise ValueError("filter index out of range")
        tab = np.zeros(max(nseg, 1), dtype=self._SEG_DTYPE)
        tab["x"][:nseg] = x.data_ptr() + 4 * off[:-1]
        tab["y"][:nseg] = y.data_ptr() + 4 * off[:-1]
        tab["n"][:nseg] = np.diff(off)
        tab["filter"][:nseg] = flt
        for z, name in ((zi, "zi"), (zf, "zf")):
            if z is not None:
                _check_tensor(z, name)
                need = max(self.state_size(int(f)) for f in np.unique(flt)) if nseg else 0
                if z.dim() != 2 or z.shape[0] != nseg or z.shape[1] < need:
                    raise ValueError(f"{name} must be (n_segments, >= {need})")
                tab[name][:nseg] = z.data_ptr() + 4 * z.shape[1] * np.arange(nseg, dtype=np.uint64)
        return tab

    def check(self, stream=None) -> None:
        check(self._lib.iir_batch_check(self._ptr, _stream_handle(stream)), "device")

    def set_timeout_ns(self, ns: int) -> None:
        check(self._lib.iir_batch_set_timeout_ns(self._ptr, int(ns)))

    def debug_withhold(self, chunk: int) -> None:
        check(self._lib.iir_batch_debug_withhold(self._ptr, int(chunk)))

    def close(self) -> None:
        if getattr(self, "_ptr", None) is not None and self._ptr.value:
            self._lib.iir_batch_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BoundBatch:
    """A batch's packed segments uploaded once (iir_batch_bind); calling it launches them."""

    def __init__(self, batch: Batch, handle, keep):
        self._batch = batch
        self._h = handle
        self._keep = keep  # the tensors the device table points into

    def __call__(self, stream=None) -> None:
        check(self._batch._lib.iir_batch_launch_bound(self._h, _stream_handle(stream)), "iir_batch_launch_bound")

    def close(self) -> None:
        if self._h is not None and self._h.value:
            self._batch._lib.iir_batch_unbind(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
