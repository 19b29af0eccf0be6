// Device helpers: Riemann flux, float-float volume arithmetic, the step
// planner and warp reductions.  The drainage translation unit is compiled
// with -fmad=false so that a request or transfer evaluated at several call
// sites (both ends of a coupling, both ends of a link) is bit-identical.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "../../include/floodgb.h"
#include "fl_internal.h"

namespace fl {

__device__ __forceinline__ float fmax32(float a, float b) { return a >= b ? a : b; }
__device__ __forceinline__ float fmin32(float a, float b) { return a <= b ? a : b; }

struct EdgeFlux {
    float h;          // mass flux (same for both cells)
    float huL, hvL;   // momentum flux seen by the left cell
    float huR, hvR;   // momentum flux seen by the right cell
};

// Approximate reciprocal (MUFU) and square root: the surface kernel's flux
// arithmetic is instruction-bound, and these keep it within a few ulp of the
// correctly rounded operations the reference uses.
__device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float fsqrt(float x) {  // x >= 0; one approximate-square-root instruction
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Hydrostatic-reconstruction flux pair with the HLL Riemann solver on the
// reconstructed states (reference equations.py:20-152), times the face
// length len.  Same algebra as the reference with rewrites that do not
// change the value beyond rounding: a velocity is a product with one
// reciprocal of the depth; the HLL velocity of a reconstructed state
// (hu* / h* with hu* = u h*) is u itself; the three HLL cases are one
// formula with clamped wave speeds; maxima and minima are the hardware's
// single-instruction fmaxf / fminf (np.maximum / np.minimum on these finite
// values, up to the sign of zero).  Both cells of an edge call this with the
// edge's own (left, right) order at a single call site, so they get
// bit-identical results.
__device__ __forceinline__ EdgeFlux hr_flux(float hL, float huL, float hvL, float zL, float hR,
                                            float huR, float hvR, float zR, float nx, float ny, float len,
                                            float g, float half_g, float md) {
    const float h_l = fmaxf(hL, 0.0f), h_r = fmaxf(hR, 0.0f);
    const float zs = fmaxf(zL, zR);
    const float hls = fmaxf(h_l + zL - zs, 0.0f), hrs = fmaxf(h_r + zR - zs, 0.0f);
    const float il = h_l > md ? rcp(h_l) : 0.0f;
    const float ir = h_r > md ? rcp(h_r) : 0.0f;
    const float u_l = huL * il, v_l = hvL * il, u_r = huR * ir, v_r = hvR * ir;
    const bool wl = hls > md, wr = hrs > md;
    const float un_l = wl ? u_l * nx + v_l * ny : 0.0f;
    const float un_r = wr ? u_r * nx + v_r * ny : 0.0f;
    const float c_l = fsqrt(g * hls), c_r = fsqrt(g * hrs);
    const float p_l = half_g * hls * hls, p_r = half_g * hrs * hrs;
    const float hul = u_l * hls, hvl = v_l * hls, hur = u_r * hrs, hvr = v_r * hrs;
    const float fhl = hls * un_l, fhul = hul * un_l + p_l * nx, fhvl = hvl * un_l + p_l * ny;
    const float fhr = hrs * un_r, fhur = hur * un_r + p_r * nx, fhvr = hvr * un_r + p_r * ny;
    // HLL with the wave speeds clamped to sl <= 0 <= sr: one formula gives
    // the left flux when sl >= 0 (sl -> 0: sr FL / sr), the right one when
    // sr <= 0, and the star-region flux otherwise (the reference selects the
    // three cases; here they agree to rounding, without the selects)
    const float sl = fminf(fminf(un_l - c_l, un_r - c_r), 0.0f);
    const float sr = fmaxf(fmaxf(un_l + c_l, un_r + c_r), 0.0f);
    const float d = sr - sl;
    // both speeds ~0 (still water) or both sides dry: no HLL flux (the
    // products below are finite, so a zero factor zeroes them)
    const float inv = (d > 1.0e-12f && (wl || wr)) ? rcp(d) * len : 0.0f;
    const float slsr = sl * sr;
    const float fh = (sr * fhl - sl * fhr + slsr * (hrs - hls)) * inv;
    const float fhu = (sr * fhul - sl * fhur + slsr * (hur - hul)) * inv;
    const float fhv = (sr * fhvl - sl * fhvr + slsr * (hvr - hvl)) * inv;
    const float pcl = half_g * (h_l * h_l - hls * hls);
    const float pcr = half_g * (h_r * h_r - hrs * hrs);
    const float nxl = nx * len, nyl = ny * len;
    EdgeFlux f;
    f.h = fh;
    f.huL = fhu + pcl * nxl;
    f.hvL = fhv + pcl * nyl;
    f.huR = fhu + pcr * nxl;
    f.hvR = fhv + pcr * nyl;
    return f;
}

// Correctly rounded, never-contracted float32 operations for the parts whose
// results are compared bit-for-bit with the reference (CFL dt, velocity clamp).
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }

// Ghost right state of a non-active-interior edge (reference
// triangular_backend.py:1294-1327): reflective for codes 0/2, fixed stage
// with zero momentum for code 3, a copy of the left state otherwise.
__device__ __forceinline__ float4 ghost_state(float hL, float huL, float hvL, float zL, float nx,
                                              float ny, int code, float stage) {
    const float nm = huL * nx + hvL * ny;
    if (code == 3) return make_float4(fmax32(stage - zL, 0.0f), 0.0f, 0.0f, zL);
    if (code == 0 || code == 2) {
        return make_float4(hL, huL - 2.0f * nm * nx, hvL - 2.0f * nm * ny, zL);
    }
    return make_float4(hL, huL, hvL, zL);
}

// --------------------------------------------------------------- float-float
__device__ __forceinline__ float ff_val(float2 a) { return a.x + a.y; }

// a + b with the error of the leading sum kept in the low word (TwoSum).
__device__ __forceinline__ float2 ff_add(float2 a, float b) {
    const float s = a.x + b;
    if (!isfinite(s)) return make_float2(s, 0.0f);
    const float bb = s - a.x;
    const float err = (a.x - (s - bb)) + (b - bb);
    const float lo = a.y + err;
    const float hi = s + lo;
    return make_float2(hi, lo - (hi - s));
}

__device__ __forceinline__ float2 ff_clamp0(float2 a) {
    return (a.x + a.y < 0.0f) ? make_float2(0.0f, 0.0f) : a;
}

// --------------------------------------------------------------- tile steps
// Phase 2 of a surface tile: one edge entry {nx, ny, len, bits} over the
// staged states st[] (own cells, then halo), written into the per-(cell, slot)
// places of s_flux; boundary in/outflow volume of exterior entries goes to
// led_in / led_out.
__device__ __forceinline__ void tile_entry(const float4 en, const float4 *st, float4 *s_flux, float g, float half_g,
                                           float md, float stage, float dt, float &led_in, float &led_out) {
    const uint32_t f = __float_as_uint(en.w);
    const uint32_t li = f & EB_IDX_MASK, ri = (f >> EB_RIGHT_SHIFT) & EB_IDX_MASK;
    const bool ai = (f & EB_AI) != 0;
    const int code = (int)(f >> EB_CODE_SHIFT) - 1;
    float4 Ls = st[li], Rs;
    if (ai) {  // both cells active (entries are grouped by kind: warp-uniform)
        Rs = st[ri];
    } else {
        if (!(f & EB_LACTIVE)) Ls = make_float4(0.0f, 0.0f, 0.0f, Ls.w);
        Rs = ghost_state(Ls.x, Ls.y, Ls.z, Ls.w, en.x, en.y, code, stage);
    }
    // fluxes times the face length
    EdgeFlux fl = hr_flux(Ls.x, Ls.y, Ls.z, Ls.w, Rs.x, Rs.y, Rs.z, Rs.w, en.x, en.y, en.z, g, half_g, md);
    if (ai) {  // an interior face: no outflow-only rule, no boundary volume
        if (f & EB_LPRESENT) s_flux[li * 3 + ((f >> EB_LSLOT_SHIFT) & 3u)] = make_float4(-fl.h, -fl.huL, -fl.hvL, 0.0f);
        if (f & EB_RPRESENT) s_flux[ri * 3 + ((f >> EB_RSLOT_SHIFT) & 3u)] = make_float4(fl.h, fl.huR, fl.hvR, 0.0f);
        return;
    }
    if (f & EB_LPRESENT) {  // (a non-active-interior face is present on its left side only)
        if (!(f & EB_INTERIOR) && code == 4 && fl.h < 0.0f) {
            fl.h = 0.0f; fl.huL = 0.0f; fl.hvL = 0.0f;
        }
        s_flux[li * 3 + ((f >> EB_LSLOT_SHIFT) & 3u)] = make_float4(-fl.h, -fl.huL, -fl.hvL, 0.0f);
        const float b = fl.h * dt;
        led_in += fmax32(-b, 0.0f);
        led_out += fmax32(b, 0.0f);
    }
}

// Phase 3 of a surface tile for one active cell: the sum of its slot
// contributions in the reference's scatter order (left-side slots, then
// right-side ones), the update with semi-implicit Manning damping, rainfall,
// infiltration, momentum rescale and dry zeroing.  rd / id: the cell's rain
// and infiltration depth of the step.
struct CellNew {
    float h, hu, hv, rd, id;
};

__device__ __forceinline__ CellNew cell_update(const float4 st, const float4 ci, const float4 *slots, float dt, float dtg,
                                              float md, float rain, float infil) {
    const uint32_t info = __float_as_uint(ci.z);
    float L0 = 0.0f, L1 = 0.0f, L2 = 0.0f, R0 = 0.0f, R1 = 0.0f, R2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 v = slots[k];
        if (info & (1u << (CELL_RIGHT_SHIFT + k))) {
            R0 = R0 + v.x; R1 = R1 + v.y; R2 = R2 + v.z;
        } else {
            L0 = L0 + v.x; L1 = L1 + v.y; L2 = L2 + v.z;
        }
    }
    const float d0 = L0 + R0, d1 = L1 + R1, d2 = L2 + R2;
    const float ia = ci.w;  // 1 / area, formed on the host
    float hn = fmaxf(st.x + dt * d0 * ia, 0.0f);
    float hun = st.y + dt * d1 * ia;
    float hvn = st.z + dt * d2 * ia;
    // semi-implicit Manning damping 1 + dt g n^2 |u| / h^(4/3), with
    // |u| / h^(4/3) = |hu| h^(-7/3)
    const bool wet = hn > md;
    const float hs = fmaxf(hn, md);
    const float q = fsqrt(hun * hun + hvn * hvn);
    const float n = ci.y;
    const float hpow = __expf(-2.3333333f * __logf(hs));
    const float damping = 1.0f + dtg * (n * n) * q * hpow;
    const float idamp = rcp(damping);
    hun = wet ? hun * idamp : 0.0f;
    hvn = wet ? hvn * idamp : 0.0f;
    // rainfall, infiltration, momentum rescale, dry zeroing
    const float rd = fmaxf(rain, 0.0f) * dt;
    const float h1 = hn + rd;
    const float id = fminf(h1, fmaxf(infil, 0.0f) * dt);
    const float h2 = h1 - id;
    const float scale = (h1 > md) ? h2 * rcp(h1) : 0.0f;
    const bool wet2 = h2 > md;
    CellNew r;
    r.h = h2;
    r.hu = wet2 ? hun * scale : 0.0f;
    r.hv = wet2 ? hvn * scale : 0.0f;
    r.rd = rd;
    r.id = id;
    return r;
}

// Velocity clamp (solver/stabilizers.py:8-27), rounded exactly as the
// reference computes it.  When |q|^2 < 0.9999 (vmax max(h, 1e-8))^2 the exact
// speed is below vmax, the exact scale is 1 and the momenta are unchanged.
__device__ __forceinline__ void clamp_velocity_exact(float h, float &hu, float &hv, float vmax) {
    const float hm = fmaxf(h, 1.0e-8f);  // = max(h, 1e-8) for every h, NaN included
    const float lim = vmax * hm;
    if (!(hu * hu + hv * hv < 0.9999f * (lim * lim))) {
        const float speed = xdiv(xsqrt(xadd(xmul(hu, hu), xmul(hv, hv))), hm);
        const float scale = fmin32(1.0f, xdiv(vmax, fmax32(speed, 1.0e-12f)));
        hu = xmul(hu, scale);
        hv = xmul(hv, scale);
    }
}

// CFL local timestep of one cell (equations.py:155-178), correctly rounded
// and uncontracted: the reference's float32 expression bit-for-bit.
// NumPy's maximum passes a NaN through (fmax32 would return its second
// argument); the CFL expressions use this one, so a NaN depth or momentum
// gives a NaN local dt that the caller's isfinite test drops, as in the
// reference.  (The solver's own state never holds a NaN depth: the cell
// update clips it to zero.)
__device__ __forceinline__ float nanmax32(float a, float b) { return isnan(a) ? a : fmax32(a, b); }

__device__ __forceinline__ float cfl_local(float h, float hu, float hv, float char_len, float cfl, float g, float md) {
    const float hs = nanmax32(h, md);
    const float u = xdiv(hu, hs), w = xdiv(hv, hs);
    const float speed = xadd(xsqrt(xadd(xmul(u, u), xmul(w, w))), xsqrt(xmul(g, hs)));
    return xdiv(xmul(cfl, char_len), nanmax32(speed, 1.0e-12f));
}

// Local-inertial CFL of one cell (reference equations.py:181-210): gravity-
// wave speed only, correctly rounded as the reference's float32 arrays.
__device__ __forceinline__ float cfl_local_li(float h, float char_len, float cfl, float g, float md) {
    const float c = xsqrt(xmul(g, nanmax32(h, md)));
    return xdiv(xmul(cfl, char_len), nanmax32(c, 1.0e-12f));
}

// --------------------------------------------------------------- inlets
// Requested capture and surcharge volume of inlet i for one step (reference
// inlet_exchange_request_kernel, triangular_inlet_exchange_cuda_kernels.py:52-131).
// The head difference is (bed - invert) + h - V/A: a static datum offset plus
// two small depths, exact in float32 at any elevation.
__device__ __forceinline__ float2 inlet_request(const InletReqView &v, int i, float h_cell, float2 Vn, float dt) {
    const float4 p = v.in_par[i];
    const float dn = fmax32(ff_val(Vn), 0.0f) / fmax32(p.w, 1.0e-12f);
    const float dh = p.x + h_cell - dn;
    const float capc = p.y * dt;
    const float surc = p.z * dt;
    float cap, sur;
    if (v.rule == FL_CAPTURE_CAPACITY) {
        cap = capc;
        sur = 0.0f;
    } else if (v.rule == FL_CAPTURE_HEAD_LIMITED) {
        cap = dh > 0.0f ? capc : 0.0f;
        sur = dh < 0.0f ? surc : 0.0f;
    } else {
        const float sgn = (float)((dh > 0.0f) - (dh < 0.0f));
        const float q = v.coef_area * sqrtf(v.g2 * fabsf(dh)) * sgn;
        float qc = fmax32(q, 0.0f);
        if (v.rule == FL_CAPTURE_WEIR_ORIFICE) {
            const float dep = fmax32(h_cell, 0.0f);
            const float wq = v.weir_coef_perim * dep * sqrtf(v.g2 * dep);
            qc = fmin32(qc, wq);
        }
        cap = fmin32(qc * dt, capc);
        sur = fmin32(fmax32(-q, 0.0f) * dt, surc);
    }
    return make_float2(fmax32(cap, 0.0f), fmax32(sur, 0.0f));
}

// --------------------------------------------------------------- planning
__device__ __forceinline__ double hyeto_rate(const HyetoView &hy, double t) {
    int lo = 0, hi = hy.n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (hy.end_s[mid] <= t) lo = mid + 1; else hi = mid;
    }
    if (lo >= hy.n || t < hy.start_s[lo]) return 0.0;
    return hy.rate[lo];
}

// Plan the next step from the run state (single thread).  This is the
// host-side control of the reference loop (engine.py:220-232, 306-313):
// CFL dt evaluated every cfl_interval steps and reused x safety otherwise,
// dt = max(min(dt, max_dt, T - t), 1e-3), snapshot when t + dt crosses the
// next snapshot time or the end, finite check after every finite_interval
// steps.
static __device__ __noinline__ void plan_step(RunCtrl *run, double *snap_t, const HyetoView &hy,
                                       StepCtrl *out, bool eval, float dt_eval, int phases) {
    StepCtrl s;
    s.t0 = run->t;
    s.dt = 0.0;
    s.dt_f = 0.0f;
    s.dtg_f = 0.0f;
    s.rain_f = 0.0f;
    s.pad0 = 0.0f;
    s.active = 0;
    s.parity = run->parity;
    s.snap_slot = -1;
    s.check_finite = 0;
    s.phases = phases;
    s.pad1 = 0;
    s.step = run->step;
    const double t = run->t;
    const bool go = run->error == 0 && t < run->final_t && t < run->stop_t && run->step < run->max_step;
    if (!go) {
        *out = s;
        return;
    }
    double dt;
    if (eval || run->cached_dt < 0.0) {
        if (!(dt_eval < CUDART_INF_F)) {
            atomicCAS(&run->error, 0, FL_E_INVALID);
            run->error_step = run->step;
            *out = s;
            return;
        }
        dt = (double)dt_eval;
        run->cached_dt = dt;
        run->cfl_evals += 1;
    } else {
        dt = run->cached_dt * run->safety;
        run->cfl_reused += 1;
    }
    dt = fmin(dt, fmin(run->max_dt, run->final_t - t));
    dt = fmax(dt, 1.0e-3);
    const double te = t + dt;
    if (te >= run->next_snap_t || te >= run->final_t) {
        if (run->snap_count >= run->max_snaps) {
            atomicCAS(&run->error, 0, FL_E_SNAPSHOTS);
            run->error_step = run->step;
            *out = s;
            return;
        }
        s.snap_slot = run->snap_count;
        snap_t[run->snap_count] = te;
        run->snap_count += 1;
        run->next_snap_t += run->snap_interval;
    }
    s.active = 1;
    s.dt = dt;
    s.dt_f = (float)dt;
    s.dtg_f = (float)(dt * run->g);
    s.rain_f = (float)hyeto_rate(hy, t);
    s.check_finite = (run->finite_interval > 0 && run->step > 0 && run->step % run->finite_interval == 0);
    run->t = te;
    run->step += 1;
    run->parity ^= 1;
    run->last_dt = dt;
    *out = s;
}

// --------------------------------------------------------------- reductions
// Float-float running sum: (hi, lo) += x with TwoSum (Knuth), so per-slot
// totals over thousands of steps keep about 48 bits without FP64 (whose
// pipe is a small fraction of the FP32 rate on this part).
__device__ __forceinline__ void ff_accumulate(float2 *slot, float x) {
    const float2 v = *slot;
    const float s = __fadd_rn(v.x, x);
    const float bp = __fsub_rn(s, v.x);
    const float e = __fadd_rn(__fsub_rn(v.x, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    const float lo = __fadd_rn(v.y, e);
    const float hi = __fadd_rn(s, lo);
    *slot = make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// Per-warp running ledger: lane 0 adds the warp's float32 sums into the
// warp's own float-float slots (no block barrier; slot = global warp index).
template <int NT>
__device__ __forceinline__ void warp_add_ledger(const float (&v)[NT], float2 *ledger) {
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        float x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) ff_accumulate(&ledger[(size_t)warp * NT + j], x);
    }
}

// The same with an explicit warp index (kernels whose warps do not all add).
template <int NT>
__device__ __forceinline__ void warp_add_ledger_at(const float (&v)[NT], float2 *ledger, int warp) {
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        float x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) ff_accumulate(&ledger[(size_t)warp * NT + j], x);
    }
}

// --------------------------------------------------------------- programmatic dependent launch
// launch_dependents lets a grid launched as a programmatic dependent of this
// one start; wait blocks until every prerequisite grid has completed and its
// writes are visible (a no-op in a grid launched without the attribute).
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// --------------------------------------------------------------- async copies
// Bulk (TMA engine) copies global -> shared completing on an mbarrier, and
// 16-byte cp.async gathers.  Every wait on an mbarrier is bounded in time.
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// One arrive on the barrier when all of this thread's earlier cp.async
// copies have landed (the barrier's expected count includes it).
__device__ __forceinline__ void cp_async_arrive_noinc(uint32_t bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity to complete; false after limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// dst (shared) and src (global) 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace fl
