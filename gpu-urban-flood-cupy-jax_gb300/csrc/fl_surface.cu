// Surface kernels for sm_103a.
//
// k_surface: a persistent, warp-specialised kernel.  Each CTA walks its tiles
// (256 consecutive Hilbert-ordered cells each) through a two-stage
// shared-memory pipeline: a producer warp has the bulk-copy (TMA) engine
// bring a tile's contiguous blocks -- states, cell info, Horton fields, wet
// time, the edge entries and the halo cell list -- into a stage and then
// gathers its halo states with cp.async, while eight compute warps work on
// the other stage, so DRAM latency overlaps the arithmetic.  Per tile:
//   phase 2  every edge entry of the tile once -- ghost state, hydrostatic
//            reconstruction, HLL (reference triangular_swe_cuda_kernels.py
//            :22-203, equations.py:20-152, triangular_backend.py:1067-1178,
//            1294-1327) -- each cell's share written to its (cell, slot)
//            place in shared memory (one writer per place: no atomics);
//   phase 3  each thread sums its cell's slots in the reference's order and
//            does the cell update with Manning damping (:206-252), rainfall
//            and infiltration (triangular_backend.py:1330-1379), the velocity
//            clamp (solver/stabilizers.py:8-27), external inflow, wet time,
//            snapshot writes and the ledger.  (The inlet requests of inlet
//            cells are evaluated by k_nodes from this kernel's output.)
// An edge between two tiles is evaluated in each (same code, same inputs),
// so its two cells always apply the same mass flux: the scheme is exactly
// conservative and bitwise reproducible.  The last CTA of the grid only plans
// the next step (a single thread of float64 control arithmetic that would
// otherwise delay one CTA's tiles).
//
// The flux arithmetic uses reciprocal-based division and fast exp/log (it is
// instruction-bound); values stay within a few ulp of the reference's
// correctly rounded float32 operations.  The velocity clamp and the CFL dt use
// correctly rounded, uncontracted operations and match the reference
// bit-for-bit.
//
// k_dt: the global CFL minimum (equations.py:155-178) as a warp-shuffle and
// single-pass grid reduction; the last block to finish plans the step.
#include <algorithm>

#include "fl_device.cuh"

namespace fl {

int surface_smem_layout(SurfArgs &a, int kind);

constexpr uint64_t COPY_WAIT_NS = 1000000000ull;  // 1 s per wait on a tile copy

struct TileStage {
    float4 *st;         // [TILE + h_cap] own states then halo states
    float4 *ci;         // [TILE]
    float4 *hz;         // [TILE] (kind 1)
    float *wt;          // [TILE] (kind 1)
    float4 *en;         // [e_cap]
    int32_t *hs;        // [h_cap]
};

__device__ __forceinline__ TileStage stage_at(const SurfArgs &a, unsigned char *smem, int s) {
    unsigned char *b = smem + a.off_stage + s * a.stage_bytes;
    TileStage t;
    t.st = (float4 *)b;
    t.ci = (float4 *)(b + a.so_ci);
    t.hz = (float4 *)(b + a.so_hz);
    t.wt = (float *)(b + a.so_wt);
    t.en = (float4 *)(b + a.so_en);
    t.hs = (int32_t *)(b + a.so_hs);
    return t;
}

// Issue the bulk copies of tile t into a stage (one thread).  The byte count
// the barrier expects is the sum of exactly the copies issued here.
template <int KIND>
__device__ __forceinline__ void issue_tile(const SurfArgs &a, const float4 *in, const TileStage &S, int4 *info_slot,
                                           uint32_t bar, int t) {
    const int4 ti = a.tile_info[t];
    *info_slot = ti;
    const uint32_t ent_bytes = (uint32_t)ti.y * 16u;
    const uint32_t halo_bytes = (uint32_t)((ti.w + 3) & ~3) * 4u;
    uint32_t bytes = TILE * 16u * 2u + ent_bytes + halo_bytes;
    if (KIND == 1) bytes += TILE * 16u + TILE * 4u;
    mbar_arrive_expect_tx(bar, bytes);
    const size_t c0 = (size_t)t * TILE;
    bulk_copy_g2s(smem_addr(S.st), in + c0, TILE * 16u, bar);
    bulk_copy_g2s(smem_addr(S.ci), a.cinfo + c0, TILE * 16u, bar);
    if (KIND == 1) {
        bulk_copy_g2s(smem_addr(S.hz), a.horton + c0, TILE * 16u, bar);
        bulk_copy_g2s(smem_addr(S.wt), a.wet + c0, TILE * 4u, bar);
    }
    if (ent_bytes) bulk_copy_g2s(smem_addr(S.en), a.ent + ti.x, ent_bytes, bar);
    if (halo_bytes) bulk_copy_g2s(smem_addr(S.hs), a.halo_src + ti.z, halo_bytes, bar);
}

// Named barrier and barrier-reduction among the compute warps only (id 1).
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(TILE) : "memory"); }

__device__ __forceinline__ bool compute_all(bool p) {
    uint32_t r;
    asm volatile(
        "{\n"
        ".reg .pred pi, po;\n"
        "setp.ne.u32 pi, %1, 0;\n"
        "bar.red.and.pred po, 1, %2, pi;\n"
        "selp.u32 %0, 1, 0, po;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)p), "n"(TILE)
        : "memory");
    return r != 0;
}

// Warp-specialised persistent surface kernel: 8 compute warps (one thread
// per cell of a 256-cell tile) and one producer warp.  The producer fills the
// two stages: bulk copies (TMA engine) of a tile's states, cell info, Horton
// fields, wet time, edge entries and halo list onto stage barrier full[s],
// then, once they land, the halo state gathers (cp.async, one arrive per lane
// on halo[s] when they land).  The compute warps wait on full[s] and halo[s],
// run phase 2 (each edge entry once: flux into per-(cell, slot) places) and
// phase 3 (the cell update), and release the stage on empty[s].  Loads of
// the next tile therefore overlap both compute phases of the current one.
// Every wait is bounded (1 s): a timeout records FL_E_TIMEOUT and the CTA
// leaves after its copies in flight have landed (or a second bounded wait).
template <int KIND>
__global__ void __launch_bounds__(SURF_THREADS, 4) k_surface(const __grid_constant__ SurfArgs a, int slot, int plan_next) {
    extern __shared__ __align__(128) unsigned char smem[];
    float4 *s_flux = (float4 *)smem;  // [TILE * 3] per (cell, slot): {mass, x-mom, y-mom} x len
    uint64_t *s_bar = (uint64_t *)(smem + a.off_bar);  // full[2], halo[2], empty[2]
    int4 *s_info = (int4 *)(smem + a.off_bar + 48);
    const int tid = threadIdx.x;
    const int ncta = (int)gridDim.x - 1;  // the last CTA plans
    if ((int)blockIdx.x == ncta) {
        pdl_wait();
        if (plan_next && tid == 0) plan_step(a.run, a.snap_t, a.hy, &a.ctrl[slot ^ 1], false, 0.0f, FL_PHASE_ALL);
        return;
    }
    // barrier addresses: full(s) = base + 8 s, halo(s) = base + 16 + 8 s, empty(s) = base + 32 + 8 s
    const uint32_t bar_base = smem_addr(s_bar);
    const TileStage S0 = stage_at(a, smem, 0), S1 = stage_at(a, smem, 1);
    if (tid < TILE) {
#pragma unroll
        for (int k = 0; k < 3; ++k) s_flux[tid * 3 + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (tid == 0) {
        for (int k = 0; k < 2; ++k) {
            mbar_init(bar_base + 8u * k, 1);
            mbar_init(bar_base + 16u + 8u * k, 32);
            mbar_init(bar_base + 32u + 8u * k, TILE / 32);  // one arrival per compute warp
        }
        mbar_fence_init();
    }
    __syncthreads();  // the last block-wide barrier: the roles split here
    // launched as a programmatic dependent of the step's previous kernel: the
    // set-up above overlaps its end; the step record, the states and the wet
    // time it (or an earlier kernel) wrote are read after this wait
    pdl_wait();
    const StepCtrl s = a.ctrl[slot];
    if (!s.active) return;  // (uniform over the grid)
    const float4 *__restrict__ in = s.parity ? a.state1 : a.state0;
    float4 *__restrict__ out = s.parity ? a.state0 : a.state1;

    if (tid >= TILE) {
        // ---------------------------------------------------------- producer
        const int lane = tid - TILE;
        bool failed = false;
        int i = 0;
        for (int t = blockIdx.x; t < a.n_tiles; t += ncta, ++i) {
            const int st = i & 1;
            const TileStage &S = st ? S1 : S0;
            if (i >= 2) {  // the compute warps released this stage's previous tile
                bool ok = true;
                if (lane == 0) ok = mbar_wait_bounded((bar_base + 32u + 8u * st), ((i >> 1) - 1) & 1u, COPY_WAIT_NS);
                if (!__shfl_sync(0xffffffffu, ok, 0)) {
                    failed = true;
                    break;
                }
            }
            if (lane == 0) issue_tile<KIND>(a, in, S, &s_info[st], (bar_base + 8u * st), t);
            // every lane waits: each then reads the landed halo list itself
            const bool ok = mbar_wait_bounded((bar_base + 8u * st), (i >> 1) & 1u, COPY_WAIT_NS);
            if (!__all_sync(0xffffffffu, ok)) {
                // a copy is late: one more bounded wait so none lands after the CTA leaves
                (void)mbar_wait_bounded((bar_base + 8u * st), (i >> 1) & 1u, COPY_WAIT_NS);
                failed = true;
                break;
            }
            const int hc = s_info[st].w;
            for (int j = lane; j < hc; j += 32) cp_async16(smem_addr(&S.st[TILE + j]), in + S.hs[j]);
            cp_async_arrive_noinc((bar_base + 16u + 8u * st));
        }
        cp_async_wait_all();
        if (failed && lane == 0) {
            if (atomicCAS(&a.run->error, 0, FL_E_TIMEOUT) == 0) a.run->error_step = s.step;
        }
        return;
    }

    // ------------------------------------------------------------- compute
    const float dt = s.dt_f;
    const float md = a.md;
    const bool do_surface = (s.phases & FL_PHASE_SURFACE) != 0;
    const bool drain_finishes = (s.phases & FL_PHASE_DRAINAGE) != 0;
    const bool recharge_finishes = (s.phases & FL_PHASE_RECHARGE) != 0;
    float led[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    int i = 0;
    for (int t = blockIdx.x; t < a.n_tiles; t += ncta, ++i) {
        const int st_i = i & 1;
        const TileStage &S = st_i ? S1 : S0;
        // one thread waits for the tile's copies and gathers; the barrier
        // reduction hands them to the other compute threads
        bool ok = true;
        if (tid == 0)
            ok = mbar_wait_bounded((bar_base + 8u * st_i), (i >> 1) & 1u, COPY_WAIT_NS) &&
                 mbar_wait_bounded((bar_base + 16u + 8u * st_i), (i >> 1) & 1u, COPY_WAIT_NS);
        if (!compute_all(ok)) {
            if (tid == 0 && atomicCAS(&a.run->error, 0, FL_E_TIMEOUT) == 0) a.run->error_step = s.step;
            break;  // the producer waits out its own copies
        }

        // phase 2: each edge entry of the tile once
        const int c0 = t * TILE;
        if (do_surface) {
            const int n_e = s_info[st_i].y;
#pragma unroll 1
            for (int e = tid; e < n_e; e += TILE)
                tile_entry(S.en[e], S.st, s_flux, a.g, a.half_g, md, a.stage, dt, led[2], led[3]);
        }
        compute_sync();  // phase 2's slots are complete

        // phase 3: the cell update
        const int c = c0 + tid;
        if (c < a.C) {
            const float4 st = S.st[tid];
            const float4 ci = S.ci[tid];
            const uint32_t info = __float_as_uint(ci.z);
            if (s.check_finite && !isfinite(st.x)) {
                if (atomicCAS(&a.run->error, 0, FL_E_NONFINITE) == 0) a.run->error_step = s.step;
            }
            float wt = 0.0f;
            float4 hz = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            if (KIND == 1) {
                wt = S.wt[tid];
                hz = S.hz[tid];
            }
            float hn = 0.0f, hun = 0.0f, hvn = 0.0f;
            if (!do_surface) {
                hn = st.x; hun = st.y; hvn = st.z;
            } else if (info & CELL_ACTIVE) {
                const float rain = KIND == 1 ? s.rain_f * hz.w : s.rain_f;
                const float infil = KIND == 1 ? hz.y + (hz.x - hz.y) * __expf(-hz.z * wt) : a.infil_scalar;
                const CellNew u = cell_update(st, ci, &s_flux[tid * 3], dt, s.dtg_f, md, rain, infil);
                hn = u.h; hun = u.hu; hvn = u.hv;
                led[0] += u.rd * ci.x;
                led[1] += u.id * ci.x;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) s_flux[tid * 3 + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (s.phases & FL_PHASE_CLAMP) clamp_velocity_exact(hn, hun, hvn, a.vmax);
            // external boundary inflow after the clamp (reference engine.py:263-273)
            if ((info & CELL_RECEIVER) && (s.phases & FL_PHASE_INFLOW)) hn = __fadd_rn(hn, a.ext_add[c]);
            out[c] = make_float4(hn, hun, hvn, st.w);
            const bool final_here = !(drain_finishes && (info & CELL_COUPLED)) &&
                                    !(recharge_finishes && (info & CELL_RECHARGE));
            if (KIND == 1 && do_surface && final_here) a.wet[c] = wt + dt * (float)(hn > md);
            if (s.snap_slot >= 0) {
                const size_t o = (size_t)s.snap_slot * (size_t)a.C + (size_t)c;
                if (final_here) a.snap_h[o] = hn;
                a.snap_hu[o] = hun;
                a.snap_hv[o] = hvn;
            }
        }
        // each compute warp releases the stage once its lanes are done with it;
        // the flux slots need no barrier here: the next tile's phase 2 writes
        // them only after its opening barrier reduction, which every compute
        // thread reaches after this phase 3
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive((bar_base + 32u + 8u * st_i));
    }
    warp_add_ledger_at<SURF_TERMS>(led, a.ledger, (int)blockIdx.x * (TILE / 32) + (tid >> 5));
}

template __global__ void k_surface<0>(const __grid_constant__ SurfArgs, int, int);
template __global__ void k_surface<1>(const __grid_constant__ SurfArgs, int, int);

// Global CFL minimum over all cells; the last block plans the step.
__global__ void __launch_bounds__(256) k_dt(const __grid_constant__ DtArgs a, int slot, int plan) {
    const float4 *__restrict__ st = a.run->parity ? a.state1 : a.state0;
    float best = CUDART_INF_F;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.C; c += gridDim.x * blockDim.x) {
        const float4 v = st[c];
        const float local = a.li ? cfl_local_li(v.x, a.char_len[c], a.cfl, a.g, a.md)
                                 : cfl_local(v.x, v.y, v.z, a.char_len[c], a.cfl, a.g, a.md);
        if (isfinite(local) && local < best) best = local;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_xor_sync(0xffffffffu, best, o));
    __shared__ float wmin[32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = wmin[0];
        for (int w = 1; w < (int)((blockDim.x + 31) >> 5); ++w) b = fminf(b, wmin[w]);
        a.partial[blockIdx.x] = b;
        __threadfence();
        const unsigned int done = atomicAdd(a.counter, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    float b = CUDART_INF_F;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) b = fminf(b, ((volatile float *)a.partial)[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = fminf(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = wmin[0];
        for (int w = 1; w < (int)((blockDim.x + 31) >> 5); ++w) m = fminf(m, wmin[w]);
        if (a.dt_out) *a.dt_out = (m < CUDART_INF_F) ? (double)m : -1.0;
        if (plan) plan_step(a.run, a.snap_t, a.hy, &a.ctrl[slot], true, m, FL_PHASE_ALL);
        *a.counter = 0u;
    }
}

// Re-plan a step after fl_run changed the stop time (single thread).
__global__ void k_replan(RunCtrl *run, double *snap_t, HyetoView hy, StepCtrl *ctrl, int slot) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && !ctrl[slot].active) {
        plan_step(run, snap_t, hy, &ctrl[slot], false, 0.0f, FL_PHASE_ALL);
    }
}

// Non-finite depth check of the latest state (the reference checks h).
__global__ void k_finite(const float4 *state0, const float4 *state1, RunCtrl *run, int32_t C) {
    const float4 *st = run->parity ? state1 : state0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        if (!isfinite(st[c].x)) {
            if (atomicCAS(&run->error, 0, FL_E_NONFINITE) == 0) run->error_step = run->step;
            return;
        }
    }
}

// ---------------------------------------------------------------- I/O
// state[new] <- reference-order arrays (perm[new] = reference index)
__global__ void k_load_state(float4 *state, const float *h, const float *hu, const float *hv,
                             const float *bed, const int32_t *perm, int32_t C, int mask) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        const int r = perm[c];
        float4 v = state[c];
        if (mask & 1) v.x = h[r];
        if (mask & 2) v.y = hu[r];
        if (mask & 4) v.z = hv[r];
        v.w = bed[c];
        state[c] = v;
    }
}

__global__ void k_store_state(const float4 *state, float *h, float *hu, float *hv, const int32_t *perm,
                              int32_t C) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        const int r = perm[c];
        const float4 v = state[c];
        if (h) h[r] = v.x;
        if (hu) hu[r] = v.y;
        if (hv) hv[r] = v.z;
    }
}

__global__ void k_permute_f32(const float *src, float *dst, const int32_t *perm, int32_t C, int to_reference) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        if (to_reference) dst[perm[c]] = src[c];
        else dst[c] = src[perm[c]];
    }
}

__global__ void k_f64_to_ff(const double *src, float2 *dst, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = src[i];
        const float hi = (float)v;
        dst[i] = make_float2(hi, (float)(v - (double)hi));
    }
}

__global__ void k_ff_to_f64(const float2 *src, double *dst, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dst[i] = (double)src[i].x + (double)src[i].y;
    }
}

__global__ void k_f64_to_ff_perm(const double *src, float2 *dst, const int32_t *perm, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = src[perm[i]];
        const float hi = (float)v;
        dst[i] = make_float2(hi, (float)(v - (double)hi));
    }
}

__global__ void k_ff_to_f64_perm(const float2 *src, double *dst, const int32_t *perm, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dst[perm[i]] = (double)src[i].x + (double)src[i].y;
    }
}

// Link flows between the reference's link order (host side) and the
// solver's (perm[new] = reference link).
__global__ void k_f64_to_f32_perm(const double *src, float *dst, const int32_t *perm, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (float)src[perm[i]];
}

__global__ void k_f32_to_f64_perm(const float *src, double *dst, const int32_t *perm, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[perm[i]] = (double)src[i];
}

// Current surface volume sum(h * area) and node volume (float64 partials).
// Each of the VOL_BLOCKS blocks covers a fixed set of cells and nodes and
// writes its partial pair; the host adds the pairs in block order, so the
// result does not depend on scheduling.
__global__ void __launch_bounds__(256) k_volumes(const float4 *state0, const float4 *state1, const float4 *cinfo,
                                                 const float2 *V, RunCtrl *run, int32_t C, int32_t N, double *part) {
    __shared__ double red[8][2];
    const float4 *st = run->parity ? state1 : state0;
    double vs = 0.0, vn = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x)
        vs += (double)(st[c].x * cinfo[c].x);
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
        vn += (double)V[n].x + (double)V[n].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vs += __shfl_down_sync(0xffffffffu, vs, o);
        vn += __shfl_down_sync(0xffffffffu, vn, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5][0] = vs;
        red[threadIdx.x >> 5][1] = vn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; ++w) {
            a += red[w][0];
            b += red[w][1];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

}  // namespace fl

// Host launch wrappers (C++ linkage, used by fl_solver.cpp).
namespace fl {

// Launched as a programmatic dependent of the previous kernel in the stream
// (the drainage kernel before it triggers at its start), so its CTAs are
// scheduled and set up while that kernel finishes.
cudaError_t launch_surface(const SurfArgs &a, int kind, int slot, int plan_next, int grid, int smem_bytes,
                           cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(SURF_THREADS);
    cfg.dynamicSmemBytes = (size_t)smem_bytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return kind ? cudaLaunchKernelEx(&cfg, k_surface<1>, a, slot, plan_next)
                : cudaLaunchKernelEx(&cfg, k_surface<0>, a, slot, plan_next);
}

// The persistent grid of k_surface: every CTA slot of the device (never more
// CTAs than tiles), the last one the planner.  Tile t goes to CTA t mod
// (slots - 1), so the first CTAs take one tile more than the rest; CTAs are
// dispatched breadth-first over the SMs, so every SM carries the same number
// of tiles to within one CTA's share.  (Fewer CTAs with equal tile counts
// leave some SMs a CTA short: those SMs idle while the fully loaded ones
// finish.)  The assignment is the same on every launch, so each per-warp
// ledger slot sums the same values in the same order.
cudaError_t plan_surface_launch(SurfArgs &a, int kind, int device, int *grid, int *smem_bytes) {
    *smem_bytes = surface_smem_layout(a, kind);
    const void *fn = kind ? (const void *)k_surface<1> : (const void *)k_surface<0>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, *smem_bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SURF_THREADS, (size_t)*smem_bytes);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int slots = std::max(1, per_sm * sms - 1);
    const int ctas = std::max(1, std::min(slots, a.n_tiles));
    *grid = ctas + 1;
    return cudaSuccess;
}

int surface_warps(int grid) { return grid * (TILE / 32); }

cudaError_t launch_dt(const DtArgs &a, int blocks, int slot, int plan, cudaStream_t stream) {
    k_dt<<<blocks, 256, 0, stream>>>(a, slot, plan);
    return cudaGetLastError();
}

cudaError_t launch_replan(RunCtrl *run, double *snap_t, HyetoView hy, StepCtrl *ctrl, int slot, cudaStream_t stream) {
    k_replan<<<1, 32, 0, stream>>>(run, snap_t, hy, ctrl, slot);
    return cudaGetLastError();
}

// Grid of the grid-stride helper kernels below: enough 256-thread blocks for
// n elements, at most `per_sm` blocks per SM of the current device.
static int helper_grid(int64_t n, int per_sm) {
    static int sms[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    if (sms[dev] == 0 && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms[dev] = 1;
    const int64_t want = std::max<int64_t>(1, (n + 255) / 256);
    return (int)std::min<int64_t>(want, (int64_t)std::max(sms[dev], 1) * per_sm);
}

cudaError_t launch_finite(const float4 *s0, const float4 *s1, RunCtrl *run, int32_t C, cudaStream_t stream) {
    k_finite<<<helper_grid(C, 4), 256, 0, stream>>>(s0, s1, run, C);
    return cudaGetLastError();
}

cudaError_t launch_load_state(float4 *state, const float *h, const float *hu, const float *hv, const float *bed,
                              const int32_t *perm, int32_t C, int mask, cudaStream_t stream) {
    k_load_state<<<helper_grid(C, 4), 256, 0, stream>>>(state, h, hu, hv, bed, perm, C, mask);
    return cudaGetLastError();
}

cudaError_t launch_store_state(const float4 *state, float *h, float *hu, float *hv, const int32_t *perm, int32_t C,
                               cudaStream_t stream) {
    k_store_state<<<helper_grid(C, 4), 256, 0, stream>>>(state, h, hu, hv, perm, C);
    return cudaGetLastError();
}

cudaError_t launch_permute_f32(const float *src, float *dst, const int32_t *perm, int32_t C, int to_reference,
                               cudaStream_t stream) {
    k_permute_f32<<<helper_grid(C, 4), 256, 0, stream>>>(src, dst, perm, C, to_reference);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_ff(const double *src, float2 *dst, int32_t n, cudaStream_t stream) {
    k_f64_to_ff<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_ff_to_f64(const float2 *src, double *dst, int32_t n, cudaStream_t stream) {
    k_ff_to_f64<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_ff_perm(const double *src, float2 *dst, const int32_t *perm, int32_t n, cudaStream_t stream) {
    k_f64_to_ff_perm<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, perm, n);
    return cudaGetLastError();
}

cudaError_t launch_ff_to_f64_perm(const float2 *src, double *dst, const int32_t *perm, int32_t n, cudaStream_t stream) {
    k_ff_to_f64_perm<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, perm, n);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32_perm(const double *src, float *dst, const int32_t *perm, int32_t n, cudaStream_t stream) {
    k_f64_to_f32_perm<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, perm, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64_perm(const float *src, double *dst, const int32_t *perm, int32_t n, cudaStream_t stream) {
    k_f32_to_f64_perm<<<helper_grid(n, 2), 256, 0, stream>>>(src, dst, perm, n);
    return cudaGetLastError();
}

cudaError_t launch_volumes(const float4 *s0, const float4 *s1, const float4 *cinfo, const float2 *V, RunCtrl *run,
                           int32_t C, int32_t N, double *out2, cudaStream_t stream) {
    k_volumes<<<VOL_BLOCKS, 256, 0, stream>>>(s0, s1, cinfo, V, run, C, N, out2);
    return cudaGetLastError();
}

}  // namespace fl
