// Device helpers: Riemann flux, float-float volume arithmetic, the step
// planner and block reductions.  The translation units that include this
// header are compiled with -fmad=false so every float32 expression rounds
// exactly as written (and as the reference's elementwise NumPy/CuPy
// operations round), and so that a flux evaluated by both cells of an edge,
// or a request evaluated by both ends of a coupling, is bit-identical.
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

// HLL normal flux of the shallow-water equations on the reconstructed
// states (reference equations.py:20-81).
__device__ __forceinline__ void hll(float h_left, float hu_left, float hv_left, float h_right,
                                    float hu_right, float hv_right, float nx, float ny, float g,
                                    float half_g, float md, float &fh, float &fhu, float &fhv) {
    const float h_l = fmax32(h_left, 0.0f), h_r = fmax32(h_right, 0.0f);
    const bool wet_l = h_l > md, wet_r = h_r > md;
    const float u_l = wet_l ? hu_left / fmax32(h_l, md) : 0.0f;
    const float v_l = wet_l ? hv_left / fmax32(h_l, md) : 0.0f;
    const float u_r = wet_r ? hu_right / fmax32(h_r, md) : 0.0f;
    const float v_r = wet_r ? hv_right / fmax32(h_r, md) : 0.0f;
    const float un_l = u_l * nx + v_l * ny;
    const float un_r = u_r * nx + v_r * ny;
    const float c_l = sqrtf(g * h_l), c_r = sqrtf(g * h_r);
    const float p_l = half_g * h_l * h_l, p_r = half_g * h_r * h_r;
    const float fhl = h_l * un_l, fhul = hu_left * un_l + p_l * nx, fhvl = hv_left * un_l + p_l * ny;
    const float fhr = h_r * un_r, fhur = hu_right * un_r + p_r * nx, fhvr = hv_right * un_r + p_r * ny;
    const float sl = fmin32(un_l - c_l, un_r - c_r);
    const float sr = fmax32(un_l + c_l, un_r + c_r);
    if (!(wet_l || wet_r)) {
        fh = 0.0f; fhu = 0.0f; fhv = 0.0f;
        return;
    }
    if (sl >= 0.0f) {
        fh = fhl; fhu = fhul; fhv = fhvl;
    } else if (sr <= 0.0f) {
        fh = fhr; fhu = fhur; fhv = fhvr;
    } else {
        const float denom = (fabsf(sr - sl) > 1.0e-12f) ? (sr - sl) : 1.0f;
        const float slsr = sl * sr;
        fh = (sr * fhl - sl * fhr + slsr * (h_r - h_l)) / denom;
        fhu = (sr * fhul - sl * fhur + slsr * (hu_right - hu_left)) / denom;
        fhv = (sr * fhvl - sl * fhvr + slsr * (hv_right - hv_left)) / denom;
    }
}

// Hydrostatic-reconstruction flux pair (reference equations.py:84-152):
// both cells of an edge call this with the same (left, right) arguments and
// get bit-identical results.
__device__ __forceinline__ EdgeFlux hr_flux(float hL, float huL, float hvL, float zL, float hR,
                                            float huR, float hvR, float zR, float nx, float ny,
                                            float g, float half_g, float md) {
    const float h_l = fmax32(hL, 0.0f), h_r = fmax32(hR, 0.0f);
    const float eta_l = h_l + zL, eta_r = h_r + zR;
    const float zs = fmax32(zL, zR);
    const float hls = fmax32(eta_l - zs, 0.0f), hrs = fmax32(eta_r - zs, 0.0f);
    const bool wl = h_l > md, wr = h_r > md;
    const float u_l = wl ? huL / fmax32(h_l, md) : 0.0f;
    const float v_l = wl ? hvL / fmax32(h_l, md) : 0.0f;
    const float u_r = wr ? huR / fmax32(h_r, md) : 0.0f;
    const float v_r = wr ? hvR / fmax32(h_r, md) : 0.0f;
    float fh, fhu, fhv;
    hll(hls, u_l * hls, v_l * hls, hrs, u_r * hrs, v_r * hrs, nx, ny, g, half_g, md, fh, fhu, fhv);
    const float pcl = half_g * (h_l * h_l - hls * hls);
    const float pcr = half_g * (h_r * h_r - hrs * hrs);
    EdgeFlux f;
    f.h = fh;
    f.huL = fhu + pcl * nx;
    f.hvL = fhv + pcl * ny;
    f.huR = fhu + pcr * nx;
    f.hvR = fhv + pcr * ny;
    return f;
}

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
template <int NT>
__device__ __forceinline__ void block_add_ledger(const float (&v)[NT], double *ledger) {
    __shared__ float red[32][NT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float x[NT];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        x[j] = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[j] += __shfl_down_sync(0xffffffffu, x[j], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NT; ++j) red[warp][j] = x[j];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            double acc = 0.0;
            for (int w = 0; w < nw; ++w) acc += (double)red[w][j];
            ledger[(size_t)blockIdx.x * NT + j] += acc;
        }
    }
}

// Programmatic dependent launch: wait for the previous kernel's writes.
__device__ __forceinline__ void wait_for_previous_grid() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

__device__ __forceinline__ void allow_next_grid() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

}  // namespace fl
