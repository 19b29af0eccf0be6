// Surface kernels for sm_103a.
//
// k_surface: one CTA per tile of 256 consecutive (Hilbert-ordered) cells.
//   phase 1  the tile's states go to shared memory;
//   phase 2  the tile's edge entries are evaluated once each -- ghost state,
//            hydrostatic reconstruction, HLL (reference
//            triangular_swe_cuda_kernels.py:22-203, equations.py:20-152,
//            triangular_backend.py:1067-1178,1294-1327) -- and each cell's
//            share is written to its (cell, slot) place in shared memory (one
//            writer per place: no atomics);
//   phase 3  each thread sums its cell's slots in the reference's order and
//            does the cell update with Manning damping (:206-252), rainfall
//            and infiltration (triangular_backend.py:1330-1379), the velocity
//            clamp (solver/stabilizers.py:8-27), wet time, snapshot writes,
//            the inlet requests of its cell and the ledger.
// An interior edge inside a tile is evaluated once; an edge between two tiles
// once in each (same code), so the two cells always apply the same mass flux:
// the scheme is exactly conservative and bitwise reproducible.
//
// The flux arithmetic uses reciprocal-based division and fast exp/log (it is
// instruction-bound); values stay within a few ulp of the reference's
// correctly rounded float32 operations.  The velocity clamp and the CFL dt use
// correctly rounded, uncontracted operations and match the reference
// bit-for-bit.
//
// k_dt: the global CFL minimum (equations.py:155-178) as a warp-shuffle and
// single-pass grid reduction; the last block to finish plans the step.
#include "fl_device.cuh"

namespace fl {

template <int KIND>
__global__ void __launch_bounds__(TILE, 4) k_surface(const __grid_constant__ SurfArgs a, int slot, int plan_next) {
    __shared__ float4 s_state[TILE];       // the tile's cell states
    __shared__ float s_flux[TILE * 3 * 3];  // per (cell, slot): the edge's contribution x len
    wait_for_previous_grid();
    const StepCtrl s = a.ctrl[slot];
    if (plan_next && blockIdx.x == 0 && threadIdx.x == 0) {
        plan_step(a.run, a.snap_t, a.hy, &a.ctrl[slot ^ 1], false, 0.0f, FL_PHASE_ALL);
    }
    if (!s.active) return;
    allow_next_grid();
    const float4 *__restrict__ in = s.parity ? a.state1 : a.state0;
    float4 *__restrict__ out = s.parity ? a.state0 : a.state1;
    const int c0 = blockIdx.x * TILE;
    const int tid = threadIdx.x;
    const int c = c0 + tid;
    const bool valid = c < a.C;
    const float dt = s.dt_f;
    const float md = a.md;
    const bool do_surface = (s.phases & FL_PHASE_SURFACE) != 0;
    const bool drain_finishes = (s.phases & FL_PHASE_DRAINAGE) != 0;
    float led[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};

    // phase 1: the tile's states into shared memory, contributions zeroed
    float4 st = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 ci = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    float4 hz = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    float wt = 0.0f;
    if (valid) {
        st = in[c];
        ci = a.cinfo[c];
        if (KIND == 1) {
            hz = a.horton[c];
            wt = a.wet[c];
        }
        if (s.check_finite && !isfinite(st.x)) {
            if (atomicCAS(&a.run->error, 0, FL_E_NONFINITE) == 0) a.run->error_step = s.step;
        }
    }
    s_state[tid] = st;
#pragma unroll
    for (int j = 0; j < 9; ++j) s_flux[tid * 9 + j] = 0.0f;
    __syncthreads();

    // phase 2: each edge entry of the tile once; both cells of an edge get the
    // flux of one evaluation in the edge's own (left, right) orientation, and
    // an edge shared with another tile is evaluated there by the same code
    // (single call site), so the mass flux always matches bit-for-bit.
    if (do_surface) {
        const int e1 = a.tile_start[blockIdx.x + 1];
#pragma unroll 1
        for (int e = a.tile_start[blockIdx.x] + tid; e < e1; e += TILE) {
            const int2 lr = a.ent_lr[e];
            const float4 gg = a.ent_g[e];
            const uint32_t f = __float_as_uint(gg.w);
            const bool lp = (f & EF_LPRESENT) != 0, rp = (f & EF_RPRESENT) != 0;
            const bool ai = (f & EF_AI) != 0, interior = (f & EF_INTERIOR) != 0;
            const int code = (int)((f >> EF_CODE_SHIFT) & 7u) - 1;
            float4 Ls = lp ? s_state[lr.x - c0] : in[lr.x];
            if (!(f & EF_LACTIVE)) Ls = make_float4(0.0f, 0.0f, 0.0f, Ls.w);
            const float4 Rs = ai ? (rp ? s_state[lr.y - c0] : in[lr.y])
                                 : ghost_state(Ls.x, Ls.y, Ls.z, Ls.w, gg.x, gg.y, code, a.stage);
            EdgeFlux fl = hr_flux(Ls.x, Ls.y, Ls.z, Ls.w, Rs.x, Rs.y, Rs.z, Rs.w, gg.x, gg.y, a.g, a.half_g, md);
            const float len = gg.z;
            if (lp) {
                if (!interior && code == 4 && fl.h < 0.0f) {
                    fl.h = 0.0f; fl.huL = 0.0f; fl.hvL = 0.0f;
                }
                const int o = ((lr.x - c0) * 3 + (int)((f >> EF_LSLOT_SHIFT) & 3u)) * 3;
                s_flux[o] = (-fl.h) * len;
                s_flux[o + 1] = (-fl.huL) * len;
                s_flux[o + 2] = (-fl.hvL) * len;
                if (!ai) {
                    const float b = fl.h * len * dt;
                    led[2] += fmax32(-b, 0.0f);
                    led[3] += fmax32(b, 0.0f);
                }
            }
            if (rp) {
                const int o = ((lr.y - c0) * 3 + (int)((f >> EF_RSLOT_SHIFT) & 3u)) * 3;
                s_flux[o] = fl.h * len;
                s_flux[o + 1] = fl.huR * len;
                s_flux[o + 2] = fl.hvR * len;
            }
        }
    }
    __syncthreads();

    // phase 3: the cell update
    if (valid) {
        const uint32_t info = __float_as_uint(ci.z);
        float hn = 0.0f, hun = 0.0f, hvn = 0.0f;
        if (!do_surface) {
            hn = st.x; hun = st.y; hvn = st.z;
        } else if (info & CELL_ACTIVE) {
            // the reference's scatter order: left-side contributions, then right-side ones
            float L0 = 0.0f, L1 = 0.0f, L2 = 0.0f, R0 = 0.0f, R1 = 0.0f, R2 = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float x = s_flux[tid * 9 + k * 3], y = s_flux[tid * 9 + k * 3 + 1], z = s_flux[tid * 9 + k * 3 + 2];
                if (info & (1u << (CELL_RIGHT_SHIFT + k))) {
                    R0 = R0 + x; R1 = R1 + y; R2 = R2 + z;
                } else {
                    L0 = L0 + x; L1 = L1 + y; L2 = L2 + z;
                }
            }
            const float d0 = L0 + R0, d1 = L1 + R1, d2 = L2 + R2;
            const float area = ci.x;
            const float ia = rcp(area);
            hn = fmax32(st.x + dt * d0 * ia, 0.0f);
            hun = st.y + dt * d1 * ia;
            hvn = st.z + dt * d2 * ia;
            // semi-implicit Manning damping 1 + dt g n^2 |u| / h^(4/3)
            const bool wet = hn > md;
            const float hs = fmax32(hn, md);
            const float ih = rcp(hs);
            const float uu = hun * ih, vv = hvn * ih;
            const float speed = fsqrt(uu * uu + vv * vv);
            const float n = ci.y;
            const float h43 = __expf(1.3333334f * __logf(hs));
            const float damping = 1.0f + s.dtg_f * (n * n) * speed * rcp(h43);
            const float idamp = rcp(damping);
            hun = wet ? hun * idamp : 0.0f;
            hvn = wet ? hvn * idamp : 0.0f;
            // rainfall, infiltration, momentum rescale, dry zeroing
            float rain, infil;
            if (KIND == 1) {
                rain = s.rain_f * hz.w;
                infil = hz.y + (hz.x - hz.y) * __expf(-hz.z * wt);
            } else {
                rain = s.rain_f;
                infil = a.infil_scalar;
            }
            const float rd = fmax32(rain, 0.0f) * dt;
            const float h1 = hn + rd;
            const float id = fmin32(h1, fmax32(infil, 0.0f) * dt);
            const float h2 = h1 - id;
            const float scale = (h1 > md) ? h2 * rcp(fmax32(h1, md)) : 0.0f;
            const bool wet2 = h2 > md;
            hn = h2;
            hun = wet2 ? hun * scale : 0.0f;
            hvn = wet2 ? hvn * scale : 0.0f;
            led[0] = rd * area;
            led[1] = id * area;
        }
        if (s.phases & FL_PHASE_CLAMP) {
            // velocity clamp, rounded exactly as the reference computes it
            const float speed = xdiv(xsqrt(xadd(xmul(hun, hun), xmul(hvn, hvn))), fmax32(hn, 1.0e-8f));
            const float scale = fmin32(1.0f, xdiv(a.vmax, fmax32(speed, 1.0e-12f)));
            hun = xmul(hun, scale);
            hvn = xmul(hvn, scale);
        }
        out[c] = make_float4(hn, hun, hvn, st.w);
        // requested inlet capture / surcharge of this cell's inlets, from the
        // depth the drainage step starts with
        const uint32_t kc = __float_as_uint(ci.w);
        if (kc && drain_finishes && a.has_inlets) {
            const InletReqView &v = a.inl;
            for (int i = v.kcell_start[kc - 1]; i < v.kcell_start[kc]; ++i) {
                const int nn = v.in_node[i];
                v.req[i] = inlet_request(v, i, hn, ff_clamp0(v.Va[nn]), v.node_area[nn], dt);
            }
        }
        const bool final_here = !(drain_finishes && (info & CELL_COUPLED));
        if (KIND == 1 && do_surface && final_here) a.wet[c] = wt + dt * (float)(hn > md);
        if (s.snap_slot >= 0) {
            const size_t o = (size_t)s.snap_slot * (size_t)a.C + (size_t)c;
            if (final_here) a.snap_h[o] = hn;
            a.snap_hu[o] = hun;
            a.snap_hv[o] = hvn;
        }
    }
    warp_add_ledger<SURF_TERMS>(led, a.ledger);
}

template __global__ void k_surface<0>(const __grid_constant__ SurfArgs, int, int);
template __global__ void k_surface<1>(const __grid_constant__ SurfArgs, int, int);

// Global CFL minimum over all cells; the last block plans the step.
__global__ void __launch_bounds__(256) k_dt(const __grid_constant__ DtArgs a, int slot, int plan) {
    wait_for_previous_grid();
    const float4 *__restrict__ st = a.run->parity ? a.state1 : a.state0;
    float best = CUDART_INF_F;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.C; c += gridDim.x * blockDim.x) {
        // rounded exactly as the reference's float32 expression
        const float4 v = st[c];
        const float hs = fmax32(v.x, a.md);
        const float u = xdiv(v.y, hs), w = xdiv(v.z, hs);
        const float speed = xadd(xsqrt(xadd(xmul(u, u), xmul(w, w))), xsqrt(xmul(a.g, hs)));
        const float local = xdiv(xmul(a.cfl, a.char_len[c]), fmax32(speed, 1.0e-12f));
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

__global__ void k_f64_to_f32(const double *src, float *dst, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (float)src[i];
}

__global__ void k_f32_to_f64(const float *src, double *dst, int32_t n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (double)src[i];
}

// Current surface volume sum(h * area) and node volume (float64 partials).
__global__ void k_volumes(const float4 *state0, const float4 *state1, const float4 *cinfo, const float2 *V,
                          RunCtrl *run, int32_t C, int32_t N, double *out2) {
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
        atomicAdd(&out2[0], vs);
        atomicAdd(&out2[1], vn);
    }
}

}  // namespace fl

// Host launch wrappers (C++ linkage, used by fl_solver.cpp).
namespace fl {

static cudaError_t launch_pdl(const void *func, dim3 grid, dim3 block, void **args, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, func, args);
}

cudaError_t launch_surface(const SurfArgs &a, int kind, int slot, int plan_next, cudaStream_t stream) {
    const int nb = (a.C + TILE - 1) / TILE;
    void *args[] = {(void *)&a, (void *)&slot, (void *)&plan_next};
    const void *fn = kind ? (const void *)k_surface<1> : (const void *)k_surface<0>;
    return launch_pdl(fn, dim3(nb > 0 ? nb : 1), dim3(TILE), args, stream);
}

int surface_blocks(int32_t C) { return (C + TILE - 1) / TILE > 0 ? (C + TILE - 1) / TILE : 1; }

cudaError_t launch_dt(const DtArgs &a, int blocks, int slot, int plan, cudaStream_t stream) {
    void *args[] = {(void *)&a, (void *)&slot, (void *)&plan};
    return launch_pdl((const void *)k_dt, dim3(blocks), dim3(256), args, stream);
}

cudaError_t launch_replan(RunCtrl *run, double *snap_t, HyetoView hy, StepCtrl *ctrl, int slot, cudaStream_t stream) {
    k_replan<<<1, 32, 0, stream>>>(run, snap_t, hy, ctrl, slot);
    return cudaGetLastError();
}

cudaError_t launch_finite(const float4 *s0, const float4 *s1, RunCtrl *run, int32_t C, cudaStream_t stream) {
    k_finite<<<608, 256, 0, stream>>>(s0, s1, run, C);
    return cudaGetLastError();
}

cudaError_t launch_load_state(float4 *state, const float *h, const float *hu, const float *hv, const float *bed,
                              const int32_t *perm, int32_t C, int mask, cudaStream_t stream) {
    k_load_state<<<608, 256, 0, stream>>>(state, h, hu, hv, bed, perm, C, mask);
    return cudaGetLastError();
}

cudaError_t launch_store_state(const float4 *state, float *h, float *hu, float *hv, const int32_t *perm, int32_t C,
                               cudaStream_t stream) {
    k_store_state<<<608, 256, 0, stream>>>(state, h, hu, hv, perm, C);
    return cudaGetLastError();
}

cudaError_t launch_permute_f32(const float *src, float *dst, const int32_t *perm, int32_t C, int to_reference,
                               cudaStream_t stream) {
    k_permute_f32<<<608, 256, 0, stream>>>(src, dst, perm, C, to_reference);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_ff(const double *src, float2 *dst, int32_t n, cudaStream_t stream) {
    k_f64_to_ff<<<304, 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_ff_to_f64(const float2 *src, double *dst, int32_t n, cudaStream_t stream) {
    k_ff_to_f64<<<304, 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double *src, float *dst, int32_t n, cudaStream_t stream) {
    k_f64_to_f32<<<304, 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float *src, double *dst, int32_t n, cudaStream_t stream) {
    k_f32_to_f64<<<304, 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_volumes(const float4 *s0, const float4 *s1, const float4 *cinfo, const float2 *V, RunCtrl *run,
                           int32_t C, int32_t N, double *out2, cudaStream_t stream) {
    k_volumes<<<608, 256, 0, stream>>>(s0, s1, cinfo, V, run, C, N, out2);
    return cudaGetLastError();
}

}  // namespace fl
