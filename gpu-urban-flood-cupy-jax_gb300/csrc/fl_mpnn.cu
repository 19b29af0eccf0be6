// Memory-bound kernels of the surrogate's message passing and training, next
// to the tensor-core GEMM (fl_mlp.cu):
//   k_transpose_seg  bf16 [m, K] (K = concatenated, optionally gathered,
//                    segments, as the GEMM's A) -> bf16 [K, ldd] with the
//                    columns m .. ldd-1 zeroed: the K-major operands of the
//                    weight-gradient products (reduction over rows)
//   k_segment_sum    fixed-order CSR row sums (message aggregation at the
//                    receiving cell; scatter of input gradients back to
//                    cells), optional row permutation, accumulate, bf16 copy
//   k_relu_bwd       dz = dx * (z > 0) -> bf16 (and fp32)
//   k_colsum_*       deterministic two-pass column sums (bias gradients)
//   k_adam           Adam step on fp32 master weights, refreshing the bf16
//                    weight and its transpose
//   k_cast_bf16      fp32 -> bf16 rows
// All sums run in a fixed order, so training is reproducible.
#include <cuda_bf16.h>

#include "fl_device.cuh"

namespace fl {

int set_error(int code, const char *fmt, ...);
void add_launches(int64_t n);

struct TSeg {
    const __nv_bfloat16 *base;
    const int32_t *rows;
    int64_t ld;
    int32_t width;
};

struct TArgs {
    TSeg s[3];
    int32_t n_seg, m, K;
    __nv_bfloat16 *dst;
    int64_t ldd;
};

// 32 x 32 tiles through shared memory: block (32, 8), tile (rows r0.., cols k0..)
__global__ void __launch_bounds__(256) k_transpose_seg(const __grid_constant__ TArgs a) {
    __shared__ __nv_bfloat16 t[32][33];
    const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // which segment holds columns k0 .. k0+31 (widths are multiples of 64)
    int seg = 0, kin = k0;
    while (seg + 1 < a.n_seg && kin >= a.s[seg].width) {
        kin -= a.s[seg].width;
        ++seg;
    }
    const TSeg s = a.s[seg];
    for (int j = ty; j < 32; j += 8) {
        const int r = r0 + j;
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (r < a.m && k0 + tx < a.K) {
            const int64_t row = s.rows ? (int64_t)s.rows[r] : (int64_t)r;
            v = s.base[row * s.ld + kin + tx];
        }
        t[j][tx] = v;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int k = k0 + j, r = r0 + tx;
        if (k < a.K && r < a.ldd) a.dst[(int64_t)k * a.ldd + r] = t[tx][j];
    }
}

// One warp per output row, four columns per lane per pass.
__global__ void __launch_bounds__(256) k_segment_sum(const float *__restrict__ src, int64_t lds, int32_t col0,
                                                     const int32_t *__restrict__ start,
                                                     const int32_t *__restrict__ order, int32_t n_out, int32_t width,
                                                     float *dst, int64_t ldd, __nv_bfloat16 *dst_bf16, int64_t ldb,
                                                     int32_t accumulate) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_out) return;
    const int p0 = start[warp], p1 = start[warp + 1];
    for (int c = lane * 4; c < width; c += 128) {
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll 4
        for (int p = p0; p < p1; ++p) {  // (unrolled: the loads of several rows in flight, the sum in order)
            const int64_t row = order ? (int64_t)order[p] : (int64_t)p;
            const float4 v = *(const float4 *)(src + row * lds + col0 + c);
            acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
        }
        if (dst) {  // (null: the bf16 copy only, for inference)
            float4 *d = (float4 *)(dst + (int64_t)warp * ldd + c);
            if (accumulate) {
                const float4 o = *d;
                acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
            }
            *d = acc;
        }
        if (dst_bf16) {
            __nv_bfloat162 h0 = __floats2bfloat162_rn(acc.x, acc.y), h1 = __floats2bfloat162_rn(acc.z, acc.w);
            uint2 w;
            w.x = *(uint32_t *)&h0;
            w.y = *(uint32_t *)&h1;
            *(uint2 *)(dst_bf16 + (int64_t)warp * ldb + c) = w;
        }
    }
}

__global__ void k_relu_bwd(const float *__restrict__ dx, int64_t ldx, const __nv_bfloat16 *__restrict__ z, int64_t ldz,
                           int32_t m, int32_t n, __nv_bfloat16 *out, int64_t ldo, float *out_f32, int64_t ldf) {
    const int64_t total = (int64_t)m * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n, c = i - r * n;
        float g = dx[r * ldx + c];
        if (z && !(__bfloat162float(z[r * ldz + c]) > 0.0f)) g = 0.0f;
        out[r * ldo + c] = __float2bfloat16(g);
        if (out_f32) out_f32[r * ldf + c] = g;
    }
}

constexpr int COLSUM_BLOCKS = 256;

// pass 1: block b sums rows b, b + B, ... into partial[b][:]
__global__ void k_colsum_partial(const float *__restrict__ x, int64_t ldx, int32_t m, int32_t n, float *partial) {
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        float s = 0.0f;
        for (int r = blockIdx.x; r < m; r += gridDim.x) s += x[(int64_t)r * ldx + c];
        partial[(int64_t)blockIdx.x * n + c] = s;
    }
}

__global__ void k_colsum_final(const float *__restrict__ partial, int32_t nb, int32_t n, float *out, int32_t accumulate) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int b = 0; b < nb; ++b) s += partial[(int64_t)b * n + c];
        out[c] = accumulate ? out[c] + s : s;
    }
}

// Adam (Kingma & Ba 2015) with bias correction; w is [rows, cols] (row = output feature).
__global__ void k_adam(float *w, float *m1, float *m2, const float *__restrict__ g, int32_t rows, int32_t cols, float lr,
                       float b1, float b2, float eps, float c1, float c2, float wd, __nv_bfloat16 *w_bf16,
                       __nv_bfloat16 *wt_bf16, int64_t ldt) {
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * w[i];
        const float a = b1 * m1[i] + (1.0f - b1) * gi;
        const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        const float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        w[i] = wi;
        const __nv_bfloat16 h = __float2bfloat16(wi);
        if (w_bf16) w_bf16[i] = h;
        if (wt_bf16) {
            const int64_t r = i / cols, c = i - r * cols;
            wt_bf16[c * ldt + r] = h;
        }
    }
}

__global__ void k_cast_bf16(const float *__restrict__ src, int64_t lds, int32_t m, int32_t n, __nv_bfloat16 *dst,
                            int64_t ldd) {
    const int64_t total = (int64_t)m * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n, c = i - r * n;
        dst[r * ldd + c] = __float2bfloat16(src[r * lds + c]);
    }
}

static int grid_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace fl

using namespace fl;

#define FM_CHECK(cond, msg)                                          \
    do {                                                             \
        if (!(cond)) return set_error(FL_E_INVALID, "%s", msg);      \
    } while (0)
#define FM_LAUNCHED(name)                                                                               \
    do {                                                                                                \
        cudaError_t _e = cudaGetLastError();                                                            \
        if (_e != cudaSuccess) return set_error(FL_E_CUDA, "%s launch: %s", name, cudaGetErrorString(_e)); \
        add_launches(1);                                                                                \
        return FL_OK;                                                                                   \
    } while (0)

extern "C" {

FL_API int fl_transpose_bf16(const FlGemmSegment *segs, int32_t n_seg, int32_t m, void *dst, int64_t ldd,
                             void *stream) {
    FM_CHECK(segs && dst && n_seg >= 1 && n_seg <= 3 && m >= 1, "fl_transpose_bf16: bad arguments");
    FM_CHECK(ldd >= m, "fl_transpose_bf16: ldd < m");
    TArgs a{};
    a.n_seg = n_seg;
    a.m = m;
    for (int i = 0; i < n_seg; ++i) {
        FM_CHECK(segs[i].base && segs[i].width > 0 && segs[i].width % 64 == 0 && segs[i].ld >= segs[i].width,
                 "fl_transpose_bf16: segment widths must be multiples of 64");
        a.s[i].base = (const __nv_bfloat16 *)segs[i].base;
        a.s[i].rows = segs[i].rows;
        a.s[i].ld = segs[i].ld;
        a.s[i].width = segs[i].width;
        a.K += segs[i].width;
    }
    a.dst = (__nv_bfloat16 *)dst;
    a.ldd = ldd;
    dim3 grid((unsigned)((ldd + 31) / 32), (unsigned)((a.K + 31) / 32));
    k_transpose_seg<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(a);
    FM_LAUNCHED("k_transpose_seg");
}

FL_API int fl_segment_sum(const float *src, int64_t lds, int32_t col0, const int32_t *start, const int32_t *order,
                          int32_t n_out, int32_t width, float *dst, int64_t ldd, void *dst_bf16, int64_t ldb,
                          int32_t accumulate, void *stream) {
    FM_CHECK(src && start && (dst || (dst_bf16 && !accumulate)) && n_out >= 1 && width > 0 && width % 4 == 0 &&
                 lds % 4 == 0 && ldd % 4 == 0 && col0 % 4 == 0 && (!dst_bf16 || ldb % 4 == 0),
             "fl_segment_sum: bad arguments (widths and strides must be multiples of 4; a null dst needs "
             "dst_bf16 and no accumulation)");
    const int64_t threads = (int64_t)n_out * 32;
    k_segment_sum<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        src, lds, col0, start, order, n_out, width, dst, ldd, (__nv_bfloat16 *)dst_bf16, ldb, accumulate);
    FM_LAUNCHED("k_segment_sum");
}

FL_API int fl_relu_bwd(const float *dx, int64_t ldx, const void *z_bf16, int64_t ldz, int32_t m, int32_t n,
                       void *out_bf16, int64_t ldo, float *out_f32, int64_t ldf, void *stream) {
    FM_CHECK(dx && out_bf16 && m >= 1 && n >= 1, "fl_relu_bwd: bad arguments");
    k_relu_bwd<<<grid_for((int64_t)m * n), 256, 0, (cudaStream_t)stream>>>(
        dx, ldx, (const __nv_bfloat16 *)z_bf16, ldz, m, n, (__nv_bfloat16 *)out_bf16, ldo, out_f32, ldf);
    FM_LAUNCHED("k_relu_bwd");
}

FL_API int fl_colsum(const float *x, int64_t ldx, int32_t m, int32_t n, float *scratch, float *out, int32_t accumulate,
                     void *stream) {
    FM_CHECK(x && scratch && out && m >= 1 && n >= 1, "fl_colsum: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    k_colsum_partial<<<COLSUM_BLOCKS, 128, 0, st>>>(x, ldx, m, n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "k_colsum_partial launch: %s", cudaGetErrorString(e));
    add_launches(1);
    k_colsum_final<<<(n + 127) / 128, 128, 0, st>>>(scratch, COLSUM_BLOCKS, n, out, accumulate);
    FM_LAUNCHED("k_colsum_final");
}

FL_API int fl_adam(float *w, float *m1, float *m2, const float *g, int32_t rows, int32_t cols, float lr, float b1,
                   float b2, float eps, int32_t step, float weight_decay, void *w_bf16, void *wt_bf16, int64_t ldt,
                   void *stream) {
    FM_CHECK(w && m1 && m2 && g && rows >= 1 && cols >= 1 && step >= 1 && (!wt_bf16 || ldt >= rows),
             "fl_adam: bad arguments");
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<grid_for((int64_t)rows * cols), 256, 0, (cudaStream_t)stream>>>(
        w, m1, m2, g, rows, cols, lr, b1, b2, eps, c1, c2, weight_decay, (__nv_bfloat16 *)w_bf16,
        (__nv_bfloat16 *)wt_bf16, ldt);
    FM_LAUNCHED("k_adam");
}

FL_API int fl_cast_bf16(const float *src, int64_t lds, int32_t m, int32_t n, void *dst, int64_t ldd, void *stream) {
    FM_CHECK(src && dst && m >= 1 && n >= 1, "fl_cast_bf16: bad arguments");
    k_cast_bf16<<<grid_for((int64_t)m * n), 256, 0, (cudaStream_t)stream>>>(src, lds, m, n, (__nv_bfloat16 *)dst, ldd);
    FM_LAUNCHED("k_cast_bf16");
}

}  // extern "C"
