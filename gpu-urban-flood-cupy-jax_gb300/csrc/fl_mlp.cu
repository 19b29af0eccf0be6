// Dense layers of the learned surrogate on the 5th-generation tensor cores.
//
// k_gemm_bf16: C[M, N] = act(A[M, K] . B[N, K]^T + bias[N]) (+ residual), A and
// B bf16, accumulation in fp32 in tensor memory (TMEM).  One CTA (4 warps)
// computes a 128 x 128 tile of C:
//   * A and B are staged in shared memory in 64-wide K chunks (128-byte rows)
//     in the canonical K-major 128-byte-swizzle layout, four stages deep, by
//     16-byte cp.async -- each A row of a chunk may come from a different
//     source row ("gathered" A: the concatenated [receiver, sender, edge]
//     input of a message MLP is never materialised);
//   * one elected thread issues tcgen05.mma (kind::f16, M = 128, N = 128,
//     K = 16 per instruction, four per chunk) and tcgen05.commit to the
//     stage's mbarrier, which frees the stage for the next chunk's copies;
//   * the epilogue reads the accumulator with tcgen05.ld (each warp its 32
//     TMEM lanes = 32 rows), adds bias / ReLU / residual and stores fp32
//     and/or bf16.
// K is split into up to three segments {base, row index, leading dimension,
// width}; a segment's chunk for output row r reads base + idx[r] * ld.
// A grid z-dimension splits K (chunks) for the weight-gradient products,
// each split writing its own fp32 partial tile.
//
// Every mbarrier wait is bounded in time; a wait that gives up records an
// error flag, drains the outstanding MMAs (bounded again), frees TMEM and
// returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "fl_device.cuh"

namespace fl {

constexpr int MM_BM = 128, MM_BN = 128, MM_BK = 64, MM_STAGES = 4, MM_THREADS = 128;
constexpr int MM_CHUNK_BYTES = MM_BM * MM_BK * 2;  // 16 KB per operand per stage
constexpr uint64_t MM_WAIT_NS = 1000000000ull;

struct GemmSeg {
    const __nv_bfloat16 *base;
    const int32_t *idx;  // row map (nullptr: identity)
    int64_t ld;          // elements between rows
    int32_t width;       // K elements of this segment (multiple of 64)
};

struct GemmArgs {
    GemmSeg a[3];
    int32_t n_seg;
    int32_t M, N, K;                 // K = sum of segment widths
    const __nv_bfloat16 *b;          // [N, ldb] rows = output features, K contiguous
    int64_t ldb;
    const float *bias;               // [N] or nullptr
    const float *residual;           // [M, ldr] fp32 or nullptr
    int64_t ldr;
    float *out_f32;                  // [M, ldo] or nullptr (split z writes out_f32 + z * M * ldo)
    __nv_bfloat16 *out_bf16;         // [M, ldo] or nullptr
    int64_t ldo;
    int32_t relu;
    int32_t k_chunks_per_split;      // chunks per z slice
    int32_t stages;                  // A ring depth (persistent kernel)
    int32_t wide;                    // bias / residual / outputs allow 32-byte accesses (persistent kernel)
    int32_t *error;                  // set to FL_E_TIMEOUT if a wait gave up
};

__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address (16-byte units)
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                    // descriptor version
    d |= (uint64_t)2 << 61;                    // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: fp32 accumulator, bf16 A and B, both
// K-major, M = 128, N = 128.
__device__ __forceinline__ uint32_t umma_idesc_bf16_128x128() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(MM_BN >> 3) << 17) | ((uint32_t)(MM_BM >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.u32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Copy one 64-wide chunk (128 rows x 128 B) into the swizzled stage layout:
// 16-byte piece c of row R lands at R * 128 + ((c ^ (R & 7)) * 16).
__device__ __forceinline__ void load_chunk_a(const GemmArgs &g, int m0, int chunk, uint32_t sdst) {
    int seg = 0, kin = chunk * MM_BK;
    while (seg + 1 < g.n_seg && kin >= g.a[seg].width) {
        kin -= g.a[seg].width;
        ++seg;
    }
    const GemmSeg s = g.a[seg];
    for (int p = threadIdx.x; p < MM_BM * 8; p += MM_THREADS) {
        const int R = p >> 3, c = p & 7;
        const uint32_t dst = sdst + (uint32_t)(R * 128 + ((c ^ (R & 7)) << 4));
        const int r = m0 + R;
        if (r < g.M) {
            const int64_t row = s.idx ? (int64_t)s.idx[r] : (int64_t)r;
            cp_async16(dst, s.base + row * s.ld + kin + c * 8);
        } else {
            asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(dst), "r"(0u) : "memory");
        }
    }
}

__device__ __forceinline__ void load_chunk_b(const GemmArgs &g, int n0, int chunk, uint32_t sdst) {
    for (int p = threadIdx.x; p < MM_BN * 8; p += MM_THREADS) {
        const int R = p >> 3, c = p & 7;
        const uint32_t dst = sdst + (uint32_t)(R * 128 + ((c ^ (R & 7)) << 4));
        const int n = n0 + R;
        if (n < g.N) cp_async16(dst, g.b + (int64_t)n * g.ldb + chunk * MM_BK + c * 8);
        else asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(dst), "r"(0u) : "memory");
    }
}

__global__ void __launch_bounds__(MM_THREADS, 1) k_gemm_bf16(const __grid_constant__ GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned stages: A0..A3, B0..B3, then barriers and the TMEM address
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA = smem_addr(smem), sB = sA + MM_STAGES * MM_CHUNK_BYTES;
    uint64_t *bars = (uint64_t *)(smem + 2 * MM_STAGES * MM_CHUNK_BYTES);
    uint32_t *tmem_slot = (uint32_t *)(bars + MM_STAGES);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * MM_BM, n0 = blockIdx.y * MM_BN;
    const int total_chunks = g.K / MM_BK;
    const int c_begin = blockIdx.z * g.k_chunks_per_split;
    const int c_end = min(total_chunks, c_begin + g.k_chunks_per_split);
    const int nk = c_end - c_begin;

    if (tid == 0) {
        for (int s = 0; s < MM_STAGES; ++s) mbar_init(smem_addr(&bars[s]), 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(128u));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = umma_idesc_bf16_128x128();
    bool bad = false;
    uint32_t issued_mask = 0u;  // stages with an MMA batch not yet waited for (thread 0)
    uint32_t par = 0u;          // bit s: parity of the next wait on stage s

    // prologue: chunks 0 .. STAGES-2
    for (int j = 0; j < MM_STAGES - 1; ++j) {
        if (j < nk) {
            load_chunk_a(g, m0, c_begin + j, sA + j * MM_CHUNK_BYTES);
            load_chunk_b(g, n0, c_begin + j, sB + j * MM_CHUNK_BYTES);
        }
        cp_async_commit();
    }
    for (int kc = 0; kc < nk; ++kc) {
        // refill the stage of chunk kc + STAGES - 1 once its previous MMAs are done
        const int j = kc + MM_STAGES - 1;
        const int sj = j % MM_STAGES;
        if (j < nk) {
            if (j >= MM_STAGES) {
                if (!mbar_wait_bounded(smem_addr(&bars[sj]), (par >> sj) & 1u, MM_WAIT_NS)) bad = true;
                par ^= 1u << sj;
                issued_mask &= ~(1u << sj);
            }
            if (!bad) {
                load_chunk_a(g, m0, c_begin + j, sA + sj * MM_CHUNK_BYTES);
                load_chunk_b(g, n0, c_begin + j, sB + sj * MM_CHUNK_BYTES);
            }
        }
        cp_async_commit();
        asm volatile("cp.async.wait_group %0;" ::"n"(MM_STAGES - 1) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // copies -> tensor-core reads
        if (__syncthreads_or(bad)) break;
        const int s = kc % MM_STAGES;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = sA + s * MM_CHUNK_BYTES, b0 = sB + s * MM_CHUNK_BYTES;
#pragma unroll
            for (int k = 0; k < MM_BK / 16; ++k)
                umma_bf16(tmem, umma_desc_sw128(a0 + k * 32), umma_desc_sw128(b0 + k * 32), idesc,
                          (kc > 0 || k > 0) ? 1u : 0u);
            umma_commit(smem_addr(&bars[s]));
        }
        issued_mask |= 1u << s;
    }
    cp_async_wait_all();
    // the accumulator is complete when every stage's last batch is done
    if (!bad) {
        for (int s = 0; s < MM_STAGES; ++s) {
            if (issued_mask & (1u << s)) {
                if (!mbar_wait_bounded(smem_addr(&bars[s]), (par >> s) & 1u, MM_WAIT_NS)) bad = true;
                par ^= 1u << s;
                issued_mask &= ~(1u << s);
            }
        }
    }
    if (__syncthreads_or(bad)) {
        if (tid == 0) {
            atomicCAS(g.error, 0, FL_E_TIMEOUT);
            for (int s = 0; s < MM_STAGES; ++s)
                if (issued_mask & (1u << s)) (void)mbar_wait_bounded(smem_addr(&bars[s]), (par >> s) & 1u, MM_WAIT_NS);
        }
        __syncthreads();
    } else if (nk > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int r = m0 + warp * 32 + (tid & 31);
        float *of = g.out_f32 ? g.out_f32 + (size_t)blockIdx.z * (size_t)g.M * (size_t)g.ldo : nullptr;
#pragma unroll 1
        for (int cb = 0; cb < MM_BN; cb += 32) {
            uint32_t v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            if (r < g.M) {
                const int nb = n0 + cb;
#pragma unroll
                for (int q = 0; q < 32; q += 8) {
                    if (nb + q >= g.N) break;
                    float x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        float y = __uint_as_float(v[q + u]);
                        if (g.bias) y += g.bias[nb + q + u];
                        if (g.relu) y = fmaxf(y, 0.0f);
                        if (g.residual) y += g.residual[(int64_t)r * g.ldr + nb + q + u];
                        x[u] = y;
                    }
                    if (of) {
                        float4 *p = (float4 *)(of + (int64_t)r * g.ldo + nb + q);
                        p[0] = make_float4(x[0], x[1], x[2], x[3]);
                        p[1] = make_float4(x[4], x[5], x[6], x[7]);
                    }
                    if (g.out_bf16) {
                        uint4 w;
                        __nv_bfloat162 h0 = __floats2bfloat162_rn(x[0], x[1]), h1 = __floats2bfloat162_rn(x[2], x[3]);
                        __nv_bfloat162 h2 = __floats2bfloat162_rn(x[4], x[5]), h3 = __floats2bfloat162_rn(x[6], x[7]);
                        w.x = *(uint32_t *)&h0;
                        w.y = *(uint32_t *)&h1;
                        w.z = *(uint32_t *)&h2;
                        w.w = *(uint32_t *)&h3;
                        *(uint4 *)(g.out_bf16 + (int64_t)r * g.ldo + nb + q) = w;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u));
}

// ---------------------------------------------------------------------------
// k_gemm_bf16_pers: the same product for K <= 512 as a persistent,
// warp-specialised kernel.  Each CTA keeps its 128 x K slice of B resident in
// shared memory and walks M tiles:
//   warps 0-1   producers: gather the A chunks of its tiles (64 rows each)
//               into a ring of as many 16 KB stages as shared memory holds
//               next to B (cp.async, completion tracked by the stage's
//               mbarrier)
//   warp 2      MMA: one lane issues tcgen05.mma per chunk into one of two
//               TMEM accumulators and commits to the stage's "empty" and
//               the accumulator's "full" barriers
//   warps 3-10  epilogue: drain the other accumulator (tcgen05.ld; two
//               warps per TMEM lane quarter, 64 columns each), release it,
//               and store with bias / ReLU / residual
// so loads, tensor-core work and the epilogue of consecutive tiles overlap.
constexpr int PG_PROD_WARPS = 2, PG_EPI_WARPS = 8, PG_THREADS = 32 * (PG_PROD_WARPS + 1 + PG_EPI_WARPS);
constexpr int PG_MAX_STAGES = 8, PG_MAX_K = 512, PG_SMEM_LIMIT = 227 * 1024;

// Source rows of the four tile rows (lane, lane + 32, ...) a producer lane
// copies, per segment; -1 past the end.  Loaded once per tile so the chunk
// copies do not wait on index loads.
struct TileRows {
    int64_t r[3][2];
};

// Producer warp pw copies tile rows 64 * pw + lane and 64 * pw + 32 + lane.
__device__ __forceinline__ TileRows tile_rows(const GemmArgs &g, int m0, int pw, int lane) {
    TileRows t;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int r = m0 + 64 * pw + lane + 32 * j;
            int64_t v = -1;
            if (s < g.n_seg && r < g.M) v = g.a[s].idx ? (int64_t)g.a[s].idx[r] : (int64_t)r;
            t.r[s][j] = v;
        }
    }
    return t;
}

// Copy one 64-wide A chunk of a tile with the 32 threads of one warp: each
// copy instruction moves four whole 128-byte row pieces (lane l: row
// 4 i + l / 8, 16-byte piece l % 8), so every L2 sector is fetched once and
// whole; a row's source index comes from the lane that loaded it.
__device__ __forceinline__ void warp_load_chunk_a(const GemmArgs &g, const TileRows &tr, int chunk, uint32_t sdst,
                                                  int pw, int lane) {
    int seg = 0, kin = chunk * MM_BK;
    while (seg + 1 < g.n_seg && kin >= g.a[seg].width) {
        kin -= g.a[seg].width;
        ++seg;
    }
    const GemmSeg s = g.a[seg];
    const int64_t own0 = seg == 0 ? tr.r[0][0] : (seg == 1 ? tr.r[1][0] : tr.r[2][0]);
    const int64_t own1 = seg == 0 ? tr.r[0][1] : (seg == 1 ? tr.r[1][1] : tr.r[2][1]);
    const int c = lane & 7;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int rr = 4 * i + (lane >> 3);  // row within this warp's 64 (rows rr < 32 are owned as j = 0)
        const int64_t row = __shfl_sync(0xffffffffu, i < 8 ? own0 : own1, rr & 31);
        const int R = 64 * pw + rr;
        const uint32_t dst = sdst + (uint32_t)(R * 128) + (uint32_t)((c ^ (R & 7)) << 4);
        if (row >= 0)
            cp_async16(dst, s.base + row * s.ld + kin + c * 8);
        else
            asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(dst), "r"(0u) : "memory");
    }
}

// 32-byte global accesses (8 x 32 bits; the address is 32-byte aligned).
__device__ __forceinline__ void ld8f(const float *p, float *d) {
    asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3]), "=f"(d[4]), "=f"(d[5]), "=f"(d[6]), "=f"(d[7])
                 : "l"(p));
}
__device__ __forceinline__ void st8f(float *p, const float *s) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(s[0]), "f"(s[1]), "f"(s[2]),
                 "f"(s[3]), "f"(s[4]), "f"(s[5]), "f"(s[6]), "f"(s[7])
                 : "memory");
}
__device__ __forceinline__ void st8u(void *p, const uint32_t *s) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(s[0]), "r"(s[1]), "r"(s[2]),
                 "r"(s[3]), "r"(s[4]), "r"(s[5]), "r"(s[6]), "r"(s[7])
                 : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *(uint32_t *)&h;
}

// The epilogue of one row's 32 columns [nb, nb + 32).  With g.wide, 16
// columns at a time through 32-byte loads and stores (a bf16 row piece of 16
// columns is one 32-byte store, an fp32 piece two): half the store
// instructions of the 16-byte path and whole 32-byte sectors.  Otherwise
// bias and residual are read 8 columns (two 16-byte loads) at a time: N,
// ldr and the column offsets are multiples of 8, the tensors 16-byte aligned.
__device__ __forceinline__ void epilogue_store(const GemmArgs &g, int r, int nb, const uint32_t (&v)[32]) {
    if (r >= g.M) return;
    if (g.wide) {
#pragma unroll
        for (int q = 0; q < 32; q += 16) {
            if (nb + q >= g.N) break;
            const bool hi = nb + q + 8 < g.N;  // the upper 8 columns exist (N is a multiple of 8)
            float bs[16], rs[16], x[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) bs[u] = rs[u] = 0.0f;
            if (g.bias) {
                ld8f(g.bias + nb + q, bs);
                if (hi) ld8f(g.bias + nb + q + 8, bs + 8);
            }
            if (g.residual) {
                const float *rp = g.residual + (int64_t)r * g.ldr + nb + q;
                ld8f(rp, rs);
                if (hi) ld8f(rp + 8, rs + 8);
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                float y = __uint_as_float(v[q + u]);
                if (g.bias) y += bs[u];
                if (g.relu) y = fmaxf(y, 0.0f);
                if (g.residual) y += rs[u];
                x[u] = y;
            }
            if (g.out_f32) {
                float *p = g.out_f32 + (int64_t)r * g.ldo + nb + q;
                st8f(p, x);
                if (hi) st8f(p + 8, x + 8);
            }
            if (g.out_bf16) {
                uint32_t w[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) w[u] = pack_bf16x2(x[2 * u], x[2 * u + 1]);
                __nv_bfloat16 *p = g.out_bf16 + (int64_t)r * g.ldo + nb + q;
                if (hi) st8u(p, w);
                else *(uint4 *)p = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < 32; q += 8) {
        if (nb + q >= g.N) break;
        float bs[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, rs[8];
        if (g.bias) {
            const float4 b0 = *(const float4 *)(g.bias + nb + q), b1 = *(const float4 *)(g.bias + nb + q + 4);
            bs[0] = b0.x; bs[1] = b0.y; bs[2] = b0.z; bs[3] = b0.w;
            bs[4] = b1.x; bs[5] = b1.y; bs[6] = b1.z; bs[7] = b1.w;
        }
        if (g.residual) {
            const float *rp = g.residual + (int64_t)r * g.ldr + nb + q;
            const float4 r0 = *(const float4 *)rp, r1 = *(const float4 *)(rp + 4);
            rs[0] = r0.x; rs[1] = r0.y; rs[2] = r0.z; rs[3] = r0.w;
            rs[4] = r1.x; rs[5] = r1.y; rs[6] = r1.z; rs[7] = r1.w;
        }
        float x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float y = __uint_as_float(v[q + u]);
            if (g.bias) y += bs[u];
            if (g.relu) y = fmaxf(y, 0.0f);
            if (g.residual) y += rs[u];
            x[u] = y;
        }
        if (g.out_f32) {
            float4 *p = (float4 *)(g.out_f32 + (int64_t)r * g.ldo + nb + q);
            p[0] = make_float4(x[0], x[1], x[2], x[3]);
            p[1] = make_float4(x[4], x[5], x[6], x[7]);
        }
        if (g.out_bf16) {
            uint4 w;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(x[0], x[1]), h1 = __floats2bfloat162_rn(x[2], x[3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(x[4], x[5]), h3 = __floats2bfloat162_rn(x[6], x[7]);
            w.x = *(uint32_t *)&h0;
            w.y = *(uint32_t *)&h1;
            w.z = *(uint32_t *)&h2;
            w.w = *(uint32_t *)&h3;
            *(uint4 *)(g.out_bf16 + (int64_t)r * g.ldo + nb + q) = w;
        }
    }
}

__global__ void __launch_bounds__(PG_THREADS, 1) k_gemm_bf16_pers(const __grid_constant__ GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int nK = g.K / MM_BK;
    const int S = g.stages;  // A ring depth
    const uint32_t sB = smem_addr(smem);
    const uint32_t sA = sB + nK * MM_CHUNK_BYTES;
    uint64_t *bars = (uint64_t *)(smem + (nK + S) * MM_CHUNK_BYTES);
    uint64_t *full = bars, *empty = bars + PG_MAX_STAGES, *accf = bars + 2 * PG_MAX_STAGES, *acce = accf + 2;
    uint64_t *drain = acce + 2;
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.y * MM_BN;
    const int tiles = (g.M + MM_BM - 1) / MM_BM;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_addr(&full[s]), 32 * PG_PROD_WARPS);
            mbar_init(smem_addr(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_addr(&accf[b]), 1);
            mbar_init(smem_addr(&acce[b]), PG_EPI_WARPS);
        }
        mbar_init(smem_addr(drain), 1);
        mbar_fence_init();
    }
    if (warp == PG_PROD_WARPS) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(256u));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // B slice resident for the whole kernel
    for (int c = 0; c < nK; ++c) {
        for (int p = tid; p < MM_BN * 8; p += PG_THREADS) {
            const int R = p >> 3, cc = p & 7;
            const uint32_t dst = sB + (uint32_t)(c * MM_CHUNK_BYTES + R * 128 + ((cc ^ (R & 7)) << 4));
            const int n = n0 + R;
            if (n < g.N) cp_async16(dst, g.b + (int64_t)n * g.ldb + c * MM_BK + cc * 8);
            else asm volatile("st.shared.v4.u32 [%0], {%1, %1, %1, %1};" ::"r"(dst), "r"(0u) : "memory");
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool bad = false;

    if (warp < PG_PROD_WARPS) {
        // producers
        int q = 0;
        for (int t = blockIdx.x; t < tiles && !bad; t += gridDim.x) {
            const TileRows tr = tile_rows(g, t * MM_BM, warp, lane);
            for (int c = 0; c < nK && !bad; ++c, ++q) {
                const int s = q % S, u = q / S;
                if (u > 0 && !mbar_wait_bounded(smem_addr(&empty[s]), (u - 1) & 1, MM_WAIT_NS)) {
                    bad = true;
                    break;
                }
                warp_load_chunk_a(g, tr, c, sA + s * MM_CHUNK_BYTES, warp, lane);
                cp_async_arrive_noinc(smem_addr(&full[s]));
            }
        }
        cp_async_wait_all();
    } else if (warp == PG_PROD_WARPS) {
        // MMA issue (one lane)
        if (lane == 0) {
            const uint32_t idesc = umma_idesc_bf16_128x128();
            int q = 0, i = 0;
            for (int t = blockIdx.x; t < tiles && !bad; t += gridDim.x, ++i) {
                const int b = i & 1, v = i >> 1;
                if (v > 0 && !mbar_wait_bounded(smem_addr(&acce[b]), (v - 1) & 1, MM_WAIT_NS)) {
                    bad = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int c = 0; c < nK; ++c, ++q) {
                    const int s = q % S;
                    if (!mbar_wait_bounded(smem_addr(&full[s]), (q / S) & 1, MM_WAIT_NS)) {
                        bad = true;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a0 = sA + s * MM_CHUNK_BYTES, b0 = sB + c * MM_CHUNK_BYTES;
#pragma unroll
                    for (int k = 0; k < MM_BK / 16; ++k)
                        umma_bf16(tmem + (uint32_t)(b * MM_BN), umma_desc_sw128(a0 + k * 32),
                                  umma_desc_sw128(b0 + k * 32), idesc, (c > 0 || k > 0) ? 1u : 0u);
                    umma_commit(smem_addr(&empty[s]));
                }
                if (bad) break;
                umma_commit(smem_addr(&accf[b]));
            }
            // every MMA issued so far has completed before TMEM is released
            umma_commit(smem_addr(drain));
            (void)mbar_wait_bounded(smem_addr(drain), 0, MM_WAIT_NS);
        }
        __syncwarp();
    } else {
        // epilogue: warp w reads TMEM lanes 32 * (w % 4) .., columns 64 * ((w - 3) / 4) ..
        const int quad = warp & 3, half = (warp - PG_PROD_WARPS - 1) >> 2;
        int i = 0;
        for (int t = blockIdx.x; t < tiles && !bad; t += gridDim.x, ++i) {
            const int b = i & 1, v = i >> 1;
            if (!mbar_wait_bounded(smem_addr(&accf[b]), v & 1, MM_WAIT_NS)) {
                bad = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int r = t * MM_BM + quad * 32 + lane;
            const uint32_t base = tmem + (uint32_t)(b * MM_BN + half * 64) + ((uint32_t)(quad * 32) << 16);
            uint32_t v0[32], v1[32];
            tmem_ld32(base, v0);
            tmem_ld32(base + 32, v1);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&acce[b]));
            epilogue_store(g, r, n0 + half * 64, v0);
            epilogue_store(g, r, n0 + half * 64 + 32, v1);
        }
    }
    if (bad) atomicCAS(g.error, 0, FL_E_TIMEOUT);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == PG_PROD_WARPS) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u));
}

constexpr int MM_SMEM_BYTES = 2 * MM_STAGES * MM_CHUNK_BYTES + 1024 + 128;

// A ring depth that fits next to the resident B slice.
int pers_stages(int K) {
    const int free_bytes = PG_SMEM_LIMIT - 1024 - 512 - (K / MM_BK) * MM_CHUNK_BYTES;
    return std::max(2, std::min(PG_MAX_STAGES, free_bytes / MM_CHUNK_BYTES));
}

int pers_smem_bytes(int K) { return (K / MM_BK + pers_stages(K)) * MM_CHUNK_BYTES + 1024 + 512; }

cudaError_t launch_gemm_bf16_pers(const GemmArgs &g, cudaStream_t stream) {
    static int configured_bytes = 0;
    const int bytes = PG_SMEM_LIMIT;
    if (configured_bytes != bytes) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16_pers, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        configured_bytes = bytes;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int gy = (g.N + MM_BN - 1) / MM_BN;
    const int tiles = (g.M + MM_BM - 1) / MM_BM;
    const int gx = std::max(1, std::min(tiles, std::max(1, sms / gy)));
    GemmArgs a = g;
    a.stages = pers_stages(g.K);
    // 32-byte accesses: 32-byte aligned tensors; a bf16 row piece of 16
    // columns must start on a 32-byte boundary (ldo a multiple of 16)
    a.wide = ((((uintptr_t)g.bias | (uintptr_t)g.residual | (uintptr_t)g.out_f32 | (uintptr_t)g.out_bf16) % 32) == 0 &&
              (!g.residual || g.ldr % 8 == 0) && (!(g.out_f32 || g.out_bf16) || g.ldo % 8 == 0) &&
              (!g.out_bf16 || g.ldo % 16 == 0))
                 ? 1
                 : 0;
    k_gemm_bf16_pers<<<dim3(gx, gy, 1), PG_THREADS, pers_smem_bytes(g.K), stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gemm_bf16(const GemmArgs &g, int splits, cudaStream_t stream) {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, MM_SMEM_BYTES);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((g.M + MM_BM - 1) / MM_BM, (g.N + MM_BN - 1) / MM_BN, splits);
    k_gemm_bf16<<<grid, MM_THREADS, MM_SMEM_BYTES, stream>>>(g);
    return cudaGetLastError();
}

}  // namespace fl

// ------------------------------------------------------------------ C ABI
#include <mutex>

namespace fl {

int set_error(int code, const char *fmt, ...);
void add_launches(int64_t n);

// Per-device error flag of the GEMM kernel's bounded waits.
static int gemm_error_flag(int32_t **out) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static int32_t *flag[MAX_DEVICES] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return set_error(FL_E_NO_DEVICE, "no usable CUDA device");
    std::lock_guard<std::mutex> lock(mu);
    if (!flag[dev]) {
        cudaError_t e = cudaMalloc(&flag[dev], sizeof(int32_t));
        if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
        e = cudaMemset(flag[dev], 0, sizeof(int32_t));
        if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
    }
    *out = flag[dev];
    return FL_OK;
}

}  // namespace fl

extern "C" FL_API int fl_gemm_bf16(const FlGemmDesc *d, void *stream) {
    using namespace fl;
    if (!d) return set_error(FL_E_INVALID, "fl_gemm_bf16: NULL descriptor");
    if (d->m < 1 || d->n < 1 || d->n_seg < 1 || d->n_seg > 3 || !d->b)
        return set_error(FL_E_INVALID, "fl_gemm_bf16: bad sizes or NULL B");
    if (!d->out_f32 && !d->out_bf16) return set_error(FL_E_INVALID, "fl_gemm_bf16: no output");
    if (d->ldb % 8 || (d->out_f32 || d->out_bf16 ? d->ldo % 8 : 0) || d->ldo < d->n ||
        (d->residual && (d->ldr < d->n || d->ldr % 8)))
        return set_error(FL_E_INVALID, "fl_gemm_bf16: leading dimensions must be multiples of 8 and cover n");
    if (d->n % 8) return set_error(FL_E_INVALID, "fl_gemm_bf16: n must be a multiple of 8");
    if (((uintptr_t)d->bias | (uintptr_t)d->residual | (uintptr_t)d->out_f32 | (uintptr_t)d->out_bf16) % 16)
        return set_error(FL_E_INVALID, "fl_gemm_bf16: bias, residual and outputs must be 16-byte aligned");
    GemmArgs g{};
    int32_t K = 0;
    for (int s = 0; s < d->n_seg; ++s) {
        const FlGemmSegment &a = d->a[s];
        if (!a.base || a.width < 64 || a.width % 64 || a.ld % 8 || a.ld < a.width)
            return set_error(FL_E_INVALID, "fl_gemm_bf16: segment %d needs a base, a width that is a multiple of 64 "
                                           "and a leading dimension that is a multiple of 8", s);
        g.a[s].base = (const __nv_bfloat16 *)a.base;
        g.a[s].idx = a.rows;
        g.a[s].ld = a.ld;
        g.a[s].width = a.width;
        K += a.width;
    }
    if (d->ldb < K) return set_error(FL_E_INVALID, "fl_gemm_bf16: ldb %lld < K %d", (long long)d->ldb, K);
    const int chunks = K / MM_BK;
    const int splits = d->k_splits > 1 ? d->k_splits : 1;
    if (splits > 1 && (d->out_bf16 || d->bias || d->residual || d->relu || !d->out_f32))
        return set_error(FL_E_INVALID, "fl_gemm_bf16: split-K writes plain fp32 partials only");
    const int per = (chunks + splits - 1) / splits;
    if ((splits - 1) * per >= chunks) return set_error(FL_E_INVALID, "fl_gemm_bf16: more K splits than chunks");
    g.n_seg = d->n_seg;
    g.M = d->m;
    g.N = d->n;
    g.K = K;
    g.b = (const __nv_bfloat16 *)d->b;
    g.ldb = d->ldb;
    g.bias = d->bias;
    g.residual = d->residual;
    g.ldr = d->ldr;
    g.out_f32 = d->out_f32;
    g.out_bf16 = (__nv_bfloat16 *)d->out_bf16;
    g.ldo = d->ldo;
    g.relu = d->relu;
    g.k_chunks_per_split = per;
    int rc = gemm_error_flag(&g.error);
    if (rc) return rc;
    // K <= 512 without split: the persistent kernel with B resident
    cudaError_t e = (splits == 1 && K <= PG_MAX_K && !d->force_tiled) ? launch_gemm_bf16_pers(g, (cudaStream_t)stream)
                                                                       : launch_gemm_bf16(g, splits, (cudaStream_t)stream);
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "k_gemm_bf16 launch: %s", cudaGetErrorString(e));
    add_launches(1);
    return FL_OK;
}

extern "C" FL_API int fl_gemm_status(void *stream) {
    using namespace fl;
    int32_t *flag = nullptr;
    int rc = gemm_error_flag(&flag);
    if (rc) return rc;
    int32_t v = 0;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&v, flag, sizeof(v), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "fl_gemm_status: %s", cudaGetErrorString(e));
    if (v) {
        cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
        return set_error(v, "a tensor-core GEMM wait gave up (device error %d)", v);
    }
    return FL_OK;
}
