// Batched-ensemble kernels for sm_103a.
//
// k_surface_batch: the persistent surface kernel of k_surface (fl_surface.cu)
// over the tiles of every active scenario of a batch.  The planner's list
// maps a virtual tile index to (scenario, tile); each CTA walks virtual tiles
// through the same two-stage pipeline (bulk async copies of the tile's states,
// cell info, Horton fields, wet time, running maximum depth, edge entries and
// halo list; cp.async gathers of the halo states) and evaluates them with the
// same tile_entry / cell_update / clamp code as the single-scenario kernel,
// with the scenario's own dt, rain and flags.  Per tile it stores the step's
// ledger terms and, when the scenario's next step evaluates the CFL dt, the
// minimum local dt of the tile's output state -- plain stores, reduced per
// scenario by the planner.
//
// k_plan_batch: one CTA per scenario reduces its tiles' ledger terms and CFL
// minima and plans its next step with plan_step (the single-scenario
// planner); the last CTA to finish rebuilds the list of active scenarios.
//
// k_cfl_batch: the CFL minima of every tile's initial state (before step 0).
#include "fl_batch.cuh"
#include "fl_device.cuh"

namespace fl {

constexpr uint64_t BATCH_WAIT_NS = 1000000000ull;  // 1 s per wait on a tile copy

__device__ __forceinline__ int find_entry(const int32_t *prefix, int n, int v) {
    int lo = 0, hi = n;  // prefix[lo] <= v < prefix[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

template <int T>
struct BStage {
    float4 *st;     // [T + h_cap]
    float4 *ci;     // [T]
    float4 *hz;     // [T] (kind 1)
    float *wt;      // [T] (kind 1)
    float *hm;      // [T]
    float4 *en;     // [e_cap]
    int32_t *hs;    // [h_cap]
};

template <int T>
__device__ __forceinline__ BStage<T> bstage_at(const BatchArgs &a, unsigned char *smem, int s) {
    unsigned char *b = smem + a.off_stage + s * a.stage_bytes;
    BStage<T> t;
    t.st = (float4 *)b;
    t.ci = (float4 *)(b + a.so_ci);
    t.hz = (float4 *)(b + a.so_hz);
    t.wt = (float *)(b + a.so_wt);
    t.hm = (float *)(b + a.so_hm);
    t.en = (float4 *)(b + a.so_en);
    t.hs = (int32_t *)(b + a.so_hs);
    return t;
}

// Issue the bulk copies of virtual tile v into a stage (one thread); the
// expected byte count is the sum of exactly the copies issued.
template <int KIND, int T>
__device__ __forceinline__ void issue_btile(const BatchArgs &a, const int32_t *prefix, const BatchEntry *ent, int n,
                                            int v, const BStage<T> &S, int4 *info_slot, int *kt_slot, uint32_t bar) {
    const int k = find_entry(prefix, n, v);
    const BatchEntry &E = ent[k];
    const int t = E.tile0 + (v - prefix[k]);
    kt_slot[0] = k;
    kt_slot[1] = t;
    const int4 ti = a.tile_info[t];
    *info_slot = ti;
    const float4 *in = (E.flags & BF_PARITY) ? a.state1 : a.state0;
    const uint32_t ent_bytes = (uint32_t)ti.y * 16u;
    const uint32_t halo_bytes = (uint32_t)((ti.w + 3) & ~3) * 4u;
    uint32_t bytes = T * 16u * 2u + T * 4u + ent_bytes + halo_bytes;
    if (KIND == 1) bytes += T * 16u + T * 4u;
    mbar_arrive_expect_tx(bar, bytes);
    const size_t c0 = (size_t)t * T;
    bulk_copy_g2s(smem_addr(S.st), in + c0, T * 16u, bar);
    bulk_copy_g2s(smem_addr(S.ci), a.cinfo + c0, T * 16u, bar);
    bulk_copy_g2s(smem_addr(S.hm), a.hmax + c0, T * 4u, bar);
    if (KIND == 1) {
        bulk_copy_g2s(smem_addr(S.hz), a.horton + c0, T * 16u, bar);
        bulk_copy_g2s(smem_addr(S.wt), a.wet + c0, T * 4u, bar);
    }
    if (ent_bytes) bulk_copy_g2s(smem_addr(S.en), a.ent + ti.x, ent_bytes, bar);
    if (halo_bytes) bulk_copy_g2s(smem_addr(S.hs), a.halo_src + ti.z, halo_bytes, bar);
}

template <int T>
__device__ __forceinline__ void gather_bhalo(const BatchArgs &a, const BatchEntry &E, const BStage<T> &S, int count) {
    const float4 *in = (E.flags & BF_PARITY) ? a.state1 : a.state0;
    for (int j = threadIdx.x; j < count; j += T) cp_async16(smem_addr(&S.st[T + j]), in + S.hs[j]);
    cp_async_commit();
}

template <int KIND, int T>
__global__ void __launch_bounds__(T, 1024 / T) k_surface_batch(const __grid_constant__ BatchArgs a) {
    constexpr int W = T / 32;
    extern __shared__ __align__(128) unsigned char smem[];
    float4 *s_flux = (float4 *)smem;  // [T * 3]
    uint64_t *s_bar = (uint64_t *)(smem + a.off_bar);
    int4 *s_info = (int4 *)(smem + a.off_bar + 16);
    int *s_kt = (int *)(smem + a.off_bar + 48);         // [2][2] list entry and tile of each stage
    float *s_red = (float *)(smem + a.off_bar + 64);    // [W][5] warp partials
    int32_t *s_prefix = (int32_t *)(smem + a.off_list);
    const int tid = threadIdx.x;
    const int n = a.list->n;
    BatchEntry *s_ent = (BatchEntry *)(smem + a.off_list + MAX_SCEN * 4 + 16);
    for (int i = tid; i <= n; i += T) s_prefix[i] = a.list->prefix[i];
    for (int i = tid; i < n; i += T) s_ent[i] = a.list->e[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) s_flux[tid * 3 + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t bar0 = smem_addr(&s_bar[0]), bar1 = smem_addr(&s_bar[1]);
    if (tid == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar1, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int total = n > 0 ? s_prefix[n] : 0;
    int v = blockIdx.x;
    if (v >= total) return;
    const BStage<T> S0 = bstage_at<T>(a, smem, 0), S1 = bstage_at<T>(a, smem, 1);
    const int G = gridDim.x;
    const float md = a.md;
    uint32_t wpar = 0u, pending = 0u;
    if (tid == 0) {
        issue_btile<KIND, T>(a, s_prefix, s_ent, n, v, S0, &s_info[0], &s_kt[0], bar0);
        pending = 1u;
    }
    bool timed_out = !mbar_wait_bounded(bar0, 0, BATCH_WAIT_NS);
    wpar ^= 1u;
    if (__syncthreads_or(timed_out)) goto abort;
    pending = 0u;
    gather_bhalo<T>(a, s_ent[s_kt[0]], S0, s_info[0].w);

    for (int i = 0; v < total; ++i, v += G) {
        const int si = i & 1;
        const BStage<T> &S = si ? S1 : S0;
        const BStage<T> &SN = si ? S0 : S1;
        const uint32_t barN = si ? bar0 : bar1;
        const int vn = v + G;
        if (tid == 0 && vn < total) {
            issue_btile<KIND, T>(a, s_prefix, s_ent, n, vn, SN, &s_info[si ^ 1], &s_kt[(si ^ 1) * 2], barN);
            pending |= 1u << (si ^ 1);
        }
        cp_async_wait_all();
        __syncthreads();  // this tile's halo states are in place

        const BatchEntry E = s_ent[s_kt[si * 2]];
        const int t = s_kt[si * 2 + 1];
        const float dt = E.dt;
        const int phases = (E.flags >> BF_PHASE_SHIFT) & 7;
        const bool do_surface = (phases & FL_PHASE_SURFACE) != 0;
        float led[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (do_surface) {
            const int n_e = s_info[si].y;
#pragma unroll 1
            for (int e = tid; e < n_e; e += T) tile_entry(S.en[e], S.st, s_flux, a.g, a.half_g, md, a.stage, dt, led[2], led[3]);
        }
        bool bad = false;
        if (vn < total) {
            bad = !mbar_wait_bounded(barN, (wpar >> (si ^ 1)) & 1u, BATCH_WAIT_NS);
            wpar ^= 1u << (si ^ 1);
        }
        if (__syncthreads_or(bad)) goto abort;  // also: phase 2's slots are complete
        pending = 0u;
        if (vn < total) gather_bhalo<T>(a, s_ent[s_kt[(si ^ 1) * 2]], SN, s_info[si ^ 1].w);

        // phase 3: the cell update
        const int c_local = (t - E.tile0) * T + tid;
        const size_t c = (size_t)t * T + tid;
        float cmin = CUDART_INF_F;
        if (c_local < E.cells) {
            const float4 st = S.st[tid];
            const float4 ci = S.ci[tid];
            const uint32_t info = __float_as_uint(ci.z);
            if ((E.flags & BF_FINITE) && !isfinite(st.x)) {
                if (atomicCAS(&a.run[E.scen].error, 0, FL_E_NONFINITE) == 0) a.run[E.scen].error_step = a.run[E.scen].step - 1;
            }
            float wt = 0.0f;
            float4 hz = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            if (KIND == 1) {
                wt = S.wt[tid];
                hz = S.hz[tid];
            }
            float hn = st.x, hun = st.y, hvn = st.z;
            if (do_surface) {
                if (info & CELL_ACTIVE) {
                    const float rain = KIND == 1 ? E.rain * hz.w : E.rain;
                    const float infil = KIND == 1 ? hz.y + (hz.x - hz.y) * __expf(-hz.z * wt) : E.infil;
                    const CellNew u = cell_update(st, ci, &s_flux[tid * 3], dt, E.dtg, md, rain, infil);
                    hn = u.h; hun = u.hu; hvn = u.hv;
                    led[0] += u.rd * ci.x;
                    led[1] += u.id * ci.x;
                } else {
                    hn = 0.0f; hun = 0.0f; hvn = 0.0f;
                }
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) s_flux[tid * 3 + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (phases & FL_PHASE_CLAMP) clamp_velocity_exact(hn, hun, hvn, a.vmax);
            (E.flags & BF_PARITY ? a.state0 : a.state1)[c] = make_float4(hn, hun, hvn, st.w);
            if (KIND == 1 && do_surface) a.wet[c] = wt + dt * (float)(hn > md);
            const float hm = fmax32(S.hm[tid], hn);
            const int snap = (E.flags >> BF_SNAP_SHIFT) - 1;
            if (snap >= 0) {
                const size_t o = (size_t)a.snap_base[E.scen] + (size_t)snap * (size_t)E.cells + (size_t)c_local;
                a.snap_h[o] = hn;
                a.snap_hmax[o] = hm;
                a.snap_hu[o] = hun;
                a.snap_hv[o] = hvn;
                a.hmax[c] = 0.0f;
            } else {
                a.hmax[c] = hm;
            }
            if (E.flags & BF_CFL) {
                const float local = cfl_local(hn, hun, hvn, a.char_len[c], a.cfl, a.g, md);
                if (isfinite(local)) cmin = local;
            }
        }
        // the tile's ledger terms and CFL minimum: warp partials, then thread 0
#pragma unroll
        for (int j = 0; j < SURF_TERMS; ++j) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) led[j] += __shfl_down_sync(0xffffffffu, led[j], o);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cmin = fminf(cmin, __shfl_down_sync(0xffffffffu, cmin, o));
        if ((tid & 31) == 0) {
#pragma unroll
            for (int j = 0; j < SURF_TERMS; ++j) s_red[(tid >> 5) * 5 + j] = led[j];
            s_red[(tid >> 5) * 5 + 4] = cmin;
        }
        __syncthreads();  // this stage, the flux slots and the partials are complete
        if (tid == 0) {
#pragma unroll
            for (int j = 0; j < SURF_TERMS; ++j) {
                float sum = 0.0f;
#pragma unroll
                for (int w = 0; w < W; ++w) sum += s_red[w * 5 + j];
                a.tile_led[(size_t)t * SURF_TERMS + j] = sum;
            }
            if (E.flags & BF_CFL) {
                float m = CUDART_INF_F;
#pragma unroll
                for (int w = 0; w < W; ++w) m = fminf(m, s_red[w * 5 + 4]);
                a.tile_min[t] = m;
            }
        }
    }
    return;

abort:
    if (tid == 0) {
        for (int k = 0; k < n; ++k)
            if (atomicCAS(&a.run[s_ent[k].scen].error, 0, FL_E_TIMEOUT) == 0) a.run[s_ent[k].scen].error_step = a.run[s_ent[k].scen].step - 1;
        if (pending & 1u) (void)mbar_wait_bounded(bar0, (wpar & 1u) ^ 1u, BATCH_WAIT_NS);
        if (pending & 2u) (void)mbar_wait_bounded(bar1, ((wpar >> 1) & 1u) ^ 1u, BATCH_WAIT_NS);
    }
    cp_async_wait_all();
    __syncthreads();
}

// CFL minima of every tile's state before the first step (all scenarios'
// states in state0).
template <int T>
__global__ void __launch_bounds__(T) k_cfl_batch(const float4 *state0, const float *char_len, const int32_t *tile_valid,
                                                 float *tile_min, float cfl, float g, float md) {
    const int t = blockIdx.x;
    const int tid = threadIdx.x;
    float m = CUDART_INF_F;
    if (tid < tile_valid[t]) {
        const size_t c = (size_t)t * T + tid;
        const float4 v = state0[c];
        const float local = cfl_local(v.x, v.y, v.z, char_len[c], cfl, g, md);
        if (isfinite(local)) m = local;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wmin[T / 32];
    if ((tid & 31) == 0) wmin[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
        float b = wmin[0];
#pragma unroll
        for (int w = 1; w < T / 32; ++w) b = fminf(b, wmin[w]);
        tile_min[t] = b;
    }
}

// One CTA per scenario: fold the step's tile terms into the scenario's
// ledger, plan its next step, and (last CTA) rebuild the active list.
__global__ void __launch_bounds__(128) k_plan_batch(const __grid_constant__ PlanArgs a, int slot, int init) {
    const int b = blockIdx.x;
    const int tid = threadIdx.x;
    RunCtrl *run = &a.run[b];
    const StepCtrl cur = a.ctrl[2 * b + slot];
    const int cfl_interval = run->cfl_interval;
    const bool had_step = !init && cur.active;
    const bool cfl_done = init || (had_step && ((cur.step + 1) % cfl_interval == 0));
    const int t0 = a.scen_tile0[b], t1 = a.scen_tile0[b + 1];
    float m = CUDART_INF_F;
    float l[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int t = t0 + tid; t < t1; t += 128) {
        if (cfl_done) m = fminf(m, a.tile_min[t]);
        if (had_step) {
#pragma unroll
            for (int j = 0; j < SURF_TERMS; ++j) l[j] += a.tile_led[(size_t)t * SURF_TERMS + j];
        }
    }
    __shared__ float red[4][SURF_TERMS + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
#pragma unroll
        for (int j = 0; j < SURF_TERMS; ++j) l[j] += __shfl_xor_sync(0xffffffffu, l[j], o);
    }
    if ((tid & 31) == 0) {
#pragma unroll
        for (int j = 0; j < SURF_TERMS; ++j) red[tid >> 5][j] = l[j];
        red[tid >> 5][SURF_TERMS] = m;
    }
    __syncthreads();
    __shared__ bool last;
    if (tid == 0) {
        float mm = red[0][SURF_TERMS];
        for (int w = 1; w < 4; ++w) mm = fminf(mm, red[w][SURF_TERMS]);
        if (had_step) {
            for (int j = 0; j < SURF_TERMS; ++j)
                ff_accumulate(&a.ledger[b * SURF_TERMS + j], red[0][j] + red[1][j] + red[2][j] + red[3][j]);
        }
        const bool eval = (run->step % cfl_interval) == 0;
        plan_step(run, a.snap_t + (size_t)b * a.max_snaps, a.hy[b], &a.ctrl[2 * b + (slot ^ 1)], eval, mm,
                  FL_PHASE_SURFACE | FL_PHASE_CLAMP);
        __threadfence();
        last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last CTA: list of the scenarios active in the next step, in order
    __shared__ int32_t cnt[MAX_SCEN];
    __shared__ int32_t pos[MAX_SCEN + 1];
    for (int s = tid; s < a.n; s += 128) {
        const volatile StepCtrl *nx = &a.ctrl[2 * s + (slot ^ 1)];
        cnt[s] = nx->active ? (a.scen_tile0[s + 1] - a.scen_tile0[s]) : -1;
    }
    __syncthreads();
    if (tid == 0) {
        int k = 0, acc = 0;
        for (int s = 0; s < a.n; ++s) {
            if (cnt[s] >= 0) {
                pos[s] = k;
                a.list->prefix[k] = acc;
                acc += cnt[s];
                ++k;
            } else {
                pos[s] = -1;
            }
        }
        a.list->prefix[k] = acc;
        a.list->n = k;
        *a.counter = 0u;
    }
    __syncthreads();
    for (int s = tid; s < a.n; s += 128) {
        if (pos[s] < 0) continue;
        const volatile StepCtrl *nx = &a.ctrl[2 * s + (slot ^ 1)];
        BatchEntry e;
        e.dt = nx->dt_f;
        e.dtg = nx->dtg_f;
        e.rain = nx->rain_f;
        e.infil = a.scen_infil[s];
        e.scen = s;
        const bool cfl_next = ((nx->step + 1) % a.run[s].cfl_interval) == 0;
        e.flags = (nx->parity ? BF_PARITY : 0) | (cfl_next ? BF_CFL : 0) | (nx->check_finite ? BF_FINITE : 0) |
                  (nx->phases << BF_PHASE_SHIFT) | ((nx->snap_slot + 1) << BF_SNAP_SHIFT);
        e.tile0 = a.scen_tile0[s];
        e.cells = a.scen_cells[s];
        a.list->e[pos[s]] = e;
    }
}

template __global__ void k_surface_batch<0, 128>(const __grid_constant__ BatchArgs);
template __global__ void k_surface_batch<0, 256>(const __grid_constant__ BatchArgs);
template __global__ void k_surface_batch<1, 128>(const __grid_constant__ BatchArgs);
template __global__ void k_surface_batch<1, 256>(const __grid_constant__ BatchArgs);

static const void *surface_batch_fn(int kind, int tile) {
    if (kind) return tile == 128 ? (const void *)k_surface_batch<1, 128> : (const void *)k_surface_batch<1, 256>;
    return tile == 128 ? (const void *)k_surface_batch<0, 128> : (const void *)k_surface_batch<0, 256>;
}

cudaError_t batch_configure(int kind, int tile, int smem_bytes, int *per_sm) {
    const void *fn = surface_batch_fn(kind, tile);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fn, tile, (size_t)smem_bytes);
}

cudaError_t launch_surface_batch(const BatchArgs &a, int kind, int grid, int smem_bytes, cudaStream_t stream) {
    if (a.tile == 128) {
        if (kind) k_surface_batch<1, 128><<<grid, 128, (size_t)smem_bytes, stream>>>(a);
        else k_surface_batch<0, 128><<<grid, 128, (size_t)smem_bytes, stream>>>(a);
    } else {
        if (kind) k_surface_batch<1, 256><<<grid, 256, (size_t)smem_bytes, stream>>>(a);
        else k_surface_batch<0, 256><<<grid, 256, (size_t)smem_bytes, stream>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_cfl_batch(const float4 *state0, const float *char_len, const int32_t *tile_valid, float *tile_min,
                             int tiles, int tile, float cfl, float g, float md, cudaStream_t stream) {
    if (tile == 128) k_cfl_batch<128><<<tiles, 128, 0, stream>>>(state0, char_len, tile_valid, tile_min, cfl, g, md);
    else k_cfl_batch<256><<<tiles, 256, 0, stream>>>(state0, char_len, tile_valid, tile_min, cfl, g, md);
    return cudaGetLastError();
}

cudaError_t launch_plan_batch(const PlanArgs &a, int slot, int init, cudaStream_t stream) {
    k_plan_batch<<<a.n, 128, 0, stream>>>(a, slot, init);
    return cudaGetLastError();
}

}  // namespace fl
