"""Thin wrappers of libfloodgb's surrogate kernels over CUDA tensors.

Every wrapper checks shapes, dtypes and strides on the host and calls one
C-ABI entry point; there is no fallback path.
"""

from __future__ import annotations

import ctypes as C

from .. import native as N


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def gemm(segments, b, *, bias=None, residual=None, out_f32=None, out_bf16=None, relu=False, k_splits=1):
    """out = act(cat_k(seg_rows) . b^T + bias) (+ residual) on the tensor cores.

    segments: list of (tensor bf16 [rows, >= width], row_index int32 [m] or None, width);
    b: bf16 [n, K]; outputs [m, >= n] (f32 and/or bf16).  With k_splits > 1,
    out_f32 is [k_splits, m, ldo] and receives one partial product per slice.
    """

    import torch

    lib = N.load()
    d = N.FlGemmDesc()
    if not 1 <= len(segments) <= 3:
        raise ValueError("1..3 A segments")
    m = None
    for i, (t, rows, width) in enumerate(segments):
        if t.dtype != torch.bfloat16 or t.dim() != 2 or t.stride(1) != 1:
            raise ValueError("A segments must be row-major bf16 matrices")
        if rows is not None:
            if rows.dtype != torch.int32:
                raise ValueError("row maps are int32")
            mi = rows.numel()
        else:
            mi = t.shape[0]
        m = mi if m is None else m
        if mi != m:
            raise ValueError("segments disagree on the number of rows")
        d.a[i] = N.FlGemmSegment(C.c_void_p(t.data_ptr()), _ptr(rows), t.stride(0), int(width))
    if b.dtype != torch.bfloat16 or b.stride(1) != 1:
        raise ValueError("B must be row-major bf16")
    out = out_f32 if out_f32 is not None else out_bf16
    d.n_seg = len(segments)
    d.m = int(m)
    d.n = int(b.shape[0])
    d.b = C.c_void_p(b.data_ptr())
    d.ldb = b.stride(0)
    d.bias = _ptr(bias)
    d.residual = _ptr(residual)
    d.ldr = residual.stride(0) if residual is not None else 0
    d.out_f32 = _ptr(out_f32)
    d.out_bf16 = _ptr(out_bf16)
    d.ldo = out.stride(-2)
    d.relu = int(bool(relu))
    d.k_splits = int(k_splits)
    N.check(lib.fl_gemm_bf16(C.byref(d), _stream()), "fl_gemm_bf16")


def status():
    N.check(N.load().fl_gemm_status(_stream()), "fl_gemm_status")
