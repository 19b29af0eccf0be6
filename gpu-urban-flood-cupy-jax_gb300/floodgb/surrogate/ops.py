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


def gemm(segments, b, *, bias=None, residual=None, out_f32=None, out_bf16=None, relu=False, k_splits=1,
         force_tiled=False):
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
    d.force_tiled = int(bool(force_tiled))
    N.check(lib.fl_gemm_bf16(C.byref(d), _stream()), "fl_gemm_bf16")


def status():
    N.check(N.load().fl_gemm_status(_stream()), "fl_gemm_status")


def _seg_array(segments):
    arr = (N.FlGemmSegment * 3)()
    for i, (t, rows, width) in enumerate(segments):
        arr[i] = N.FlGemmSegment(C.c_void_p(t.data_ptr()), _ptr(rows), t.stride(0), int(width))
    return arr


def transpose(segments, m, dst):
    """dst[k, r] = cat_k(segments)[r, k]; dst columns m.. zeroed."""

    N.check(N.load().fl_transpose_bf16(_seg_array(segments), len(segments), int(m), C.c_void_p(dst.data_ptr()),
                                       dst.stride(0), _stream()), "fl_transpose_bf16")


def segment_sum(src, col0, start, order, n_out, width, dst, dst_bf16=None, accumulate=False):
    """Fixed-order row sums; dst None (with dst_bf16, no accumulation) writes the bf16 copy only."""
    N.check(N.load().fl_segment_sum(C.c_void_p(src.data_ptr()), src.stride(0), int(col0), C.c_void_p(start.data_ptr()),
                                    _ptr(order), int(n_out), int(width), _ptr(dst), dst.stride(0) if dst is not None else 4,
                                    _ptr(dst_bf16), dst_bf16.stride(0) if dst_bf16 is not None else 0,
                                    int(bool(accumulate)), _stream()), "fl_segment_sum")


def relu_bwd(dx, z, out_bf16, out_f32=None):
    m, n = dx.shape[0], out_bf16.shape[1]
    N.check(N.load().fl_relu_bwd(C.c_void_p(dx.data_ptr()), dx.stride(0), _ptr(z), z.stride(0) if z is not None else 0,
                                 int(m), int(n), C.c_void_p(out_bf16.data_ptr()), out_bf16.stride(0), _ptr(out_f32),
                                 out_f32.stride(0) if out_f32 is not None else 0, _stream()), "fl_relu_bwd")


def colsum(x, m, n, scratch, out, accumulate=False):
    N.check(N.load().fl_colsum(C.c_void_p(x.data_ptr()), x.stride(0), int(m), int(n), C.c_void_p(scratch.data_ptr()),
                               C.c_void_p(out.data_ptr()), int(bool(accumulate)), _stream()), "fl_colsum")


def adam(w, m1, m2, g, lr, step, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0, w_bf16=None, wt_bf16=None):
    rows, cols = w.shape
    N.check(N.load().fl_adam(C.c_void_p(w.data_ptr()), C.c_void_p(m1.data_ptr()), C.c_void_p(m2.data_ptr()),
                             C.c_void_p(g.data_ptr()), int(rows), int(cols), float(lr), float(b1), float(b2),
                             float(eps), int(step), float(weight_decay), _ptr(w_bf16), _ptr(wt_bf16),
                             wt_bf16.stride(0) if wt_bf16 is not None else 0, _stream()), "fl_adam")


def cast_bf16(src, dst):
    m, n = dst.shape
    N.check(N.load().fl_cast_bf16(C.c_void_p(src.data_ptr()), src.stride(0), int(m), int(n),
                                  C.c_void_p(dst.data_ptr()), dst.stride(0), _stream()), "fl_cast_bf16")
