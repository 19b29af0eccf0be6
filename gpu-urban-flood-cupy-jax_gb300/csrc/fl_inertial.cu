// Local-inertial surface step for sm_103a (solver.surface_step_mode =
// "local_inertial"): the reference's fast routing mode
// (gurugram_flood/kernels/triangular_local_inertial_cuda_kernels.py:59-262,
// triangular_backend.py:531-590, local_inertial.py:20-49) as two launches:
//   k_li_edges  one thread per edge: the LISFLOOD-style discharge update from
//               the water-surface slope (face distance and Manning n are
//               static per edge), written into the (cell, slot) place of
//               each of its cells                                   [:59-167]
//   k_li_cells  one thread per cell: the donor limit factors (a cell's volume
//               over the summed outgoing requests of its edges, in slot
//               order; the reference adds them with atomicAdd) of the cell
//               and of each neighbour that donates to it [:172-189], the
//               volume change, momentum from the face discharges, then the
//               same sources, clamp, external inflow, wet time and snapshots
//               as the full-SWE surface kernel; its last block plans the next
//               step                                                [:194-262]
// The cell kernel reads its cell's discharges and slot tables (flags, the
// other cell, the face normals) contiguously and gathers a donating
// neighbour's slots, depth and area.
// Compiled with -fmad=false: the discharge arithmetic is rounded as written.
#include <cuda_runtime.h>

#include "fl_device.cuh"

namespace fl {

__global__ void __launch_bounds__(256) k_li_edges(const __grid_constant__ LiArgs a, int slot) {
    pdl_launch_dependents();  // the cell kernel may launch and wait meanwhile
    pdl_wait();               // the previous step's kernels
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_SURFACE)) return;
    const float4 *__restrict__ in = s.parity ? a.state1 : a.state0;
    const float dt = s.dt_f, g = a.g;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.E; e += gridDim.x * blockDim.x) {
        const int2 lr = a.e_lr[e];
        const float4 geo = a.e_geo[e];
        const uint32_t f = __float_as_uint(geo.w);
        const int L = lr.x, R = (f & LI_INTERIOR) ? lr.y : lr.x;
        const bool la = (f & LI_LACTIVE) != 0, ra = (f & LI_RACTIVE) != 0, ai = (f & LI_AI) != 0;
        const bool bedge = (f & LI_BEDGE) != 0;
        const float4 sl = in[L], sr = in[R];
        const float hl = la ? sl.x : 0.0f, hul = la ? sl.y : 0.0f, hvl = la ? sl.z : 0.0f;
        const float hr = ra ? sr.x : 0.0f, hur = ra ? sr.y : 0.0f, hvr = ra ? sr.z : 0.0f;
        const float bl = sl.w, br = sr.w;
        const float etal = bl + hl;
        const float etar = ai ? br + hr : bl;
        const float bstar = ai ? fmax32(bl, br) : bl;
        const float hflow = fmax32(fmax32(etal, etar) - bstar, 0.0f);
        const float2 dm = a.e_dm[e];  // {max(0.5 (l_L + l_R), 1e-6), face n}, formed on the host in float32
        const float slope = (etar - etal) / dm.x;
        const float nx = geo.x, ny = geo.y, len = geo.z;
        const float nl = hul * nx + hvl * ny, nr = hur * nx + hvr * ny;
        const float qold = (ai ? 0.5f * (nl + nr) : nl) * len;
        const float mn = dm.y;
        const float area = fmax32(hflow * len, 1.0e-8f);
        const float radius = fmax32(hflow, 1.0e-6f);
        const float r43 = radius * cbrtf(radius);
        const float numer = qold - g * area * dt * slope;
        const float fric = 1.0f + g * dt * mn * mn * fabsf(qold) / (r43 * area);
        float q = numer / fric;
        if (!(ai || bedge)) q = 0.0f;
        if (bedge) q = fmax32(q, 0.0f);
        float *qs = reinterpret_cast<float *>(a.Qs);
        qs[(size_t)L * 4 + ((f >> LI_SLOTL_SHIFT) & 3u)] = q;
        if (f & LI_INTERIOR) qs[(size_t)lr.y * 4 + ((f >> LI_SLOTR_SHIFT) & 3u)] = q;
    }
}

// Donor limit factor of a cell (reference :172-189): its volume over the
// summed outgoing requests of its active interior edges, in slot order (the
// reference adds them with atomicAdd).  sb, q4: the cell's slot bits and
// discharges; h, area: its depth at the step start and its area.  The cell
// kernel evaluates it for a cell and for each neighbour that donates to it;
// every evaluation of one cell reads the same values, so all agree
// bit-for-bit (this file is compiled without contraction).
__device__ __forceinline__ float li_donor_scale(uint32_t sb, float4 q4, float h, float area, float dt) {
    const float qk[3] = {q4.x, q4.y, q4.z};
    float req = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t b = sb >> (4 * k);
        if (!(b & LIS_PRESENT) || !(b & LIS_AI)) continue;
        const float q = qk[k];
        if (q == 0.0f) continue;
        // the donor is the left cell for q >= 0, else the right one
        if ((q >= 0.0f) == ((b & LIS_LEFT) != 0)) req += fabsf(q) * dt;
    }
    const float vol = fmax32(h, 0.0f) * area;
    return req > 1.0e-12f ? fmin32(1.0f, vol / req) : 1.0f;
}

template <int KIND>
__global__ void __launch_bounds__(256) k_li_cells(const __grid_constant__ LiArgs a, int slot, int plan_next) {
    pdl_wait();  // the discharges of k_li_edges (and every earlier kernel's writes)
    if ((int)blockIdx.x == (int)gridDim.x - 1) {  // the last block plans the next step
        if (plan_next && threadIdx.x == 0) plan_step(a.run, a.snap_t, a.hy, &a.ctrl[slot ^ 1], false, 0.0f, FL_PHASE_ALL);
        return;
    }
    const StepCtrl s = a.ctrl[slot];
    if (!s.active) return;
    const float4 *__restrict__ in = s.parity ? a.state1 : a.state0;
    float4 *__restrict__ out = s.parity ? a.state0 : a.state1;
    const float dt = s.dt_f, md = a.md;
    const bool do_surface = (s.phases & FL_PHASE_SURFACE) != 0;
    const bool drain_finishes = (s.phases & FL_PHASE_DRAINAGE) != 0;
    const bool recharge_finishes = (s.phases & FL_PHASE_RECHARGE) != 0;
    float led[SURF_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.C) {
        const float4 st = in[c];
        const float4 ci = a.cinfo[c];
        const uint32_t info = __float_as_uint(ci.z);
        if (s.check_finite && !isfinite(st.x)) {
            if (atomicCAS(&a.run->error, 0, FL_E_NONFINITE) == 0) a.run->error_step = s.step;
        }
        float wt = 0.0f;
        float4 hz = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        if (KIND == 1) {
            wt = a.wet[c];
            hz = a.horton[c];
        }
        float hn = 0.0f, hun = 0.0f, hvn = 0.0f;
        if (!do_surface) {
            hn = st.x; hun = st.y; hvn = st.z;
        } else if (info & CELL_ACTIVE) {
            // the cell's face discharges in slot order
            const uint32_t sb = a.c_bits[c];
            const float4 q4 = a.Qs[c];
            const int4 oc = a.c_other[c];
            const float qk[3] = {q4.x, q4.y, q4.z};
            const int ok[3] = {oc.x, oc.y, oc.z};
            const float own_scale = li_donor_scale(sb, q4, st.x, ci.x, dt);
            float hd = 0.0f, qx = 0.0f, qy = 0.0f, bf = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t b = sb >> (4 * k);
                if (!(b & LIS_PRESENT)) continue;
                const float q = qk[k];
                if (q == 0.0f) continue;
                const float2 nrm = a.c_nrm[(size_t)k * (size_t)a.C + (size_t)c];
                if (b & LIS_INTERIOR) {
                    const bool left = (b & LIS_LEFT) != 0;
                    float sd = own_scale;
                    if ((q >= 0.0f) != left) {  // the neighbour donates: its factor from its own slots
                        const int m = ok[k];
                        sd = li_donor_scale(a.c_bits[m], a.Qs[m], in[m].x, a.cinfo[m].x, dt);
                    }
                    const float lim = q * sd * dt;
                    hd += left ? -lim : lim;
                } else {
                    const float bq = q * dt;
                    hd -= bq;
                    bf += bq;
                }
                qx += q * nrm.x;
                qy += q * nrm.y;
            }
            const float area = ci.x;
            const float h0 = fmax32(st.x + hd / area, 0.0f);
            const float per = 2.0f * area / fmax32(a.char_len[c], 1.0e-12f);
            const bool wet0 = h0 > md;
            const float hu0 = wet0 ? qx / fmax32(per, 1.0e-12f) : 0.0f;
            const float hv0 = wet0 ? qy / fmax32(per, 1.0e-12f) : 0.0f;
            // _apply_sources (reference triangular_backend.py:1330-1379)
            const float rain = KIND == 1 ? s.rain_f * hz.w : s.rain_f;
            const float infil = KIND == 1 ? hz.y + (hz.x - hz.y) * __expf(-hz.z * wt) : a.infil_scalar;
            const float rd = fmax32(rain, 0.0f) * dt;
            const float h1 = h0 + rd;
            const float id = fmin32(h1, fmax32(infil, 0.0f) * dt);
            const float h2 = h1 - id;
            const float sc = (h1 > md) ? h2 / fmax32(h1, md) : 0.0f;
            const bool wet2 = h2 > md;
            hn = h2;
            hun = wet2 ? hu0 * sc : 0.0f;
            hvn = wet2 ? hv0 * sc : 0.0f;
            led[0] += rd * area;
            led[1] += id * area;
            led[3] += bf;
        }
        if (s.phases & FL_PHASE_CLAMP) clamp_velocity_exact(hn, hun, hvn, a.vmax);
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
    warp_add_ledger<SURF_TERMS>(led, a.ledger);
}

int li_edge_blocks(int32_t E, int sms) { return std::max(1, std::min(sms * 8, (E + 255) / 256)); }
int li_cell_blocks(int32_t C) { return (C + 255) / 256 + 1; }  // + the planner block

// Both launched as programmatic dependents of the kernel before them, so
// each one's launch overlaps the end of the previous one.
cudaError_t launch_li(const LiArgs &a, int kind, int slot, int plan_next, int sms, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((unsigned)li_edge_blocks(a.E, sms));
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_li_edges, a, slot);
    if (e != cudaSuccess) return e;
    cfg.gridDim = dim3((unsigned)li_cell_blocks(a.C));
    return kind == 1 ? cudaLaunchKernelEx(&cfg, k_li_cells<1>, a, slot, plan_next)
                     : cudaLaunchKernelEx(&cfg, k_li_cells<0>, a, slot, plan_next);
}

}  // namespace fl
