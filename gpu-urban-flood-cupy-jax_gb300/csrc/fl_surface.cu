// Surface kernels for sm_103a.
//
// k_surface: one thread per (renumbered) cell.  The thread gathers the
// fluxes of the cell's three edges itself -- the cell-centric replacement of
// the reference's per-edge flux kernel with float atomicAdd scatters
// (gurugram_flood/kernels/triangular_swe_cuda_kernels.py:22-203) -- then does
// the cell update with Manning damping (:206-252), rainfall and infiltration
// (triangular_backend.py:1330-1379), and the velocity clamp
// (solver/stabilizers.py:8-27), all in one pass over the state.  Both cells of
// an interior edge evaluate the same flux with the edge's own left/right
// orientation, so the mass flux they apply is bit-identical and the scheme
// stays exactly conservative without atomics; summation order per cell is
// fixed, so runs are bitwise reproducible.
//
// The flux arithmetic uses reciprocal-based division and fast exp/log (the
// kernel is instruction-bound); values stay within a few ulp of the
// reference's correctly rounded float32 operations.  The velocity clamp and
// the CFL dt use correctly rounded, uncontracted operations and match the
// reference bit-for-bit.
//
// k_dt: the global CFL minimum (equations.py:155-178) as a warp-shuffle and
// single-pass grid reduction; the last block to finish plans the step.
#include "fl_device.cuh"

namespace fl {

template <int KIND>
__global__ void __launch_bounds__(256, 4) k_surface(const __grid_constant__ SurfArgs a, int slot, int plan_next) {
    wait_for_previous_grid();
    const StepCtrl s = a.ctrl[slot];
    if (plan_next && blockIdx.x == 0 && threadIdx.x == 0) {
        plan_step(a.run, a.snap_t, a.hy, &a.ctrl[slot ^ 1], false, 0.0f, FL_PHASE_ALL);
    }
    if (!s.active) return;
    allow_next_grid();
    const float4 *__restrict__ in = s.parity ? a.state1 : a.state0;
    float4 *__restrict__ out = s.parity ? a.state0 : a.state1;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    float led[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bool do_surface = (s.phases & FL_PHASE_SURFACE) != 0;
    const bool drain_finishes = (s.phases & FL_PHASE_DRAINAGE) != 0;
    if (c < a.C) {
        const float4 st = in[c];
        const uint4 tp = a.topo[c];
        if (s.check_finite && !isfinite(st.x)) {
            if (atomicCAS(&a.run->error, 0, FL_E_NONFINITE) == 0) a.run->error_step = s.step;
        }
        const float dt = s.dt_f;
        const float md = a.md;
        float hn = 0.0f, hun = 0.0f, hvn = 0.0f;
        const bool act = (tp.w & CELL_ACTIVE) != 0;
        if (!do_surface) {
            hn = st.x; hun = st.y; hvn = st.z;
        } else if (act || (tp.w & CELL_STAGE_LEDGER)) {
            // An inactive cell only evaluates its exterior stage edges: the
            // reference counts their flux in the boundary ledger and then
            // zeroes the cell.
            const float4 own = act ? st : make_float4(0.0f, 0.0f, 0.0f, st.w);
            float L0 = 0.0f, L1 = 0.0f, L2 = 0.0f, R0 = 0.0f, R1 = 0.0f, R2 = 0.0f;
            float bin = 0.0f, bout = 0.0f;
            const float4 g0 = a.g0[c], g1 = a.g1[c], g2 = a.g2[c];
            // the three neighbour states, gathered together up front
            const auto nb = [&](uint32_t w) {
                const uint32_t o = w & IDX_MASK;
                return (w != SLOT_NONE && o != NO_CELL && (w & OTHER_ACTIVE_BIT)) ? in[o] : own;
            };
            const float4 n0 = nb(tp.x), n1 = nb(tp.y), n2 = nb(tp.z);
            // one flux code path for all three edges (not unrolled): both cells
            // of an edge run the identical instruction sequence
#pragma unroll 1
            for (int k = 0; k < 3; ++k) {
                const uint32_t w = k == 0 ? tp.x : (k == 1 ? tp.y : tp.z);
                const float4 gk = k == 0 ? g0 : (k == 1 ? g1 : g2);
                const float4 nbk = k == 0 ? n0 : (k == 1 ? n1 : n2);
                if (w == SLOT_NONE) continue;
                const uint32_t other = w & IDX_MASK;
                const bool interior = other != NO_CELL;
                const bool oact = (w & OTHER_ACTIVE_BIT) != 0;
                const bool is_right = (w & RIGHT_BIT) != 0;
                const int raw = (int)((w >> CODE_SHIFT) & 7u) - 1;
                const bool ai = interior && oact;
                if (is_right && !ai) continue;  // the reference adds nothing here
                if (!act && (is_right || interior || raw != 3)) continue;
                const int code = (interior && !oact) ? 0 : raw;
                const float nx = gk.x, ny = gk.y, len = gk.z;
                // the edge's left and right states in the reference's orientation
                const float4 o = ai ? nbk : ghost_state(own.x, own.y, own.z, own.w, nx, ny, code, a.stage);
                const float4 L = is_right ? o : own;
                const float4 R = is_right ? own : o;
                EdgeFlux f = hr_flux(L.x, L.y, L.z, L.w, R.x, R.y, R.z, R.w, nx, ny, a.g, a.half_g, md);
                if (!is_right) {
                    if (!interior && code == 4 && f.h < 0.0f) {
                        f.h = 0.0f; f.huL = 0.0f; f.hvL = 0.0f;
                    }
                    L0 = L0 + (-f.h) * len;
                    L1 = L1 + (-f.huL) * len;
                    L2 = L2 + (-f.hvL) * len;
                    if (!ai) {
                        const float b = f.h * len * dt;
                        bin += fmax32(-b, 0.0f);
                        bout += fmax32(b, 0.0f);
                    }
                } else {
                    R0 = R0 + f.h * len;
                    R1 = R1 + f.huR * len;
                    R2 = R2 + f.hvR * len;
                }
            }
            led[2] = bin;
            led[3] = bout;
            if (act) {
                const float d0 = L0 + R0, d1 = L1 + R1, d2 = L2 + R2;
                const float area = g1.w;
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
                const float n = g0.w;
                const float h43 = __expf(1.3333334f * __logf(hs));
                const float damping = 1.0f + s.dtg_f * (n * n) * speed * rcp(h43);
                const float idamp = rcp(damping);
                hun = wet ? hun * idamp : 0.0f;
                hvn = wet ? hvn * idamp : 0.0f;
                // rainfall, infiltration, momentum rescale, dry zeroing
                float rain, infil;
                if (KIND == 1) {
                    const float4 hz = a.horton[c];
                    rain = s.rain_f * hz.w;
                    infil = hz.y + (hz.x - hz.y) * __expf(-hz.z * a.wet[c]);
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
        const uint32_t kc = tp.w >> CELL_KCELL_SHIFT;
        if (kc && drain_finishes && a.has_inlets) {
            const InletReqView &v = a.inl;
            for (int i = v.kcell_start[kc - 1]; i < v.kcell_start[kc]; ++i) {
                const int n = v.in_node[i];
                v.req[i] = inlet_request(v, i, hn, ff_clamp0(v.Va[n]), v.node_area[n], dt);
            }
        }
        const bool final_here = !(drain_finishes && (tp.w & CELL_COUPLED));
        if (KIND == 1 && do_surface && final_here) a.wet[c] = a.wet[c] + dt * (float)(hn > md);
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
__global__ void k_volumes(const float4 *state0, const float4 *state1, const float4 *g1, const float2 *V,
                          RunCtrl *run, int32_t C, int32_t N, double *out2) {
    const float4 *st = run->parity ? state1 : state0;
    double vs = 0.0, vn = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x)
        vs += (double)(st[c].x * g1[c].w);
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
    const int nb = (a.C + 255) / 256;
    void *args[] = {(void *)&a, (void *)&slot, (void *)&plan_next};
    const void *fn = kind ? (const void *)k_surface<1> : (const void *)k_surface<0>;
    return launch_pdl(fn, dim3(nb > 0 ? nb : 1), dim3(256), args, stream);
}

int surface_blocks(int32_t C) { return (C + 255) / 256 > 0 ? (C + 255) / 256 : 1; }

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

cudaError_t launch_volumes(const float4 *s0, const float4 *s1, const float4 *g1, const float2 *V, RunCtrl *run,
                           int32_t C, int32_t N, double *out2, cudaStream_t stream) {
    k_volumes<<<608, 256, 0, stream>>>(s0, s1, g1, V, run, C, N, out2);
    return cudaGetLastError();
}

}  // namespace fl
