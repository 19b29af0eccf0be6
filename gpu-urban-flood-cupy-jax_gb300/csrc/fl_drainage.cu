// Drainage kernels for sm_103a: the coupled 1D network of the reference
// (gurugram_flood/kernels/triangular_inlet_exchange_cuda_kernels.py and
// triangular_pipe_network_cuda_kernels.py), restated without atomics.
//
// The reference does each many-to-one sum (requests per cell, per node, per
// donor node; volume deltas per node; depth deltas per cell) with float64
// atomicAdd.  Here every sum is a gather over a precomputed list in a fixed
// order, so runs are reproducible, and every exchanged quantity is computed
// once and read by both sides, so volume is conserved exactly as in the
// reference.  Per step, after k_surface (which evaluates the inlet requests of
// its inlet cells and their capture limit factor, reference :52-177):
//   k_nodes   one thread per node: captures limited by their cells, the
//             surcharge limit by the node's volume, the node volume after
//             the exchange                                [reference :133-177]
//   k_links   one thread per link: the semi-implicit link update from the two
//             end volumes                              [pipe network :39-139]
//   k_donor   one thread per node: its donor limit factor, its volume over
//             the transfers it gives                   [pipe network :141-175]
//   k_network one thread per group = a surface cell with the nodes that
//             overflow into it (nodes are numbered so a group's nodes are
//             consecutive), or a node without a cell: limited transfers, node
//             continuity, outfall, overflow return, and the cell's final
//             depth                    [pipe network :141-211, overflow :179-207]
//
// Heads are carried as depth relative to a static per-link / per-inlet datum
// offset (bed - invert, invert_from - invert_to, ...), so float32 keeps
// millimetre-scale head differences exact at 200 m elevations; node storage
// volume is a float-float pair so small exchanges are not lost against large
// stored volumes.  No FP64 arithmetic is used on this path.
#include "fl_device.cuh"

namespace fl {

// Semi-implicit Saint-Venant link update with circular/Preissmann or
// rectangular geometry (reference pipe_link_flow_kernel :39-139); returns the
// signed transfer volume of the step.  Heads enter as end depths plus the
// link's static datum offsets.
__device__ __forceinline__ float link_transfer(float4 k0, float4 k1, float4 k2, float df, float dtn, float q,
                                               float g, float wave_speed, float dt) {
    const float depth = fmax32(0.5f * (df + dtn) + k0.z, 0.0f);
    const int flags = (int)k2.w;
    float area, radius;
    if (flags & 1) {
        const float dia = fmax32(k1.x, 1.0e-12f);
        const float rg = 0.5f * dia;
        const float od = fmin32(depth, dia);
        const float ratio = fmax32(fmin32((rg - od) / rg, 1.0f), -1.0f);
        const float theta = 2.0f * acosf(ratio);
        const float oa = 0.5f * rg * rg * (theta - sinf(theta));
        const float fa = 0.25f * 3.14159265358979323846f * dia * dia;
        const bool full = depth >= dia;
        const float ca = full ? fa : oa;
        const float cp = full ? 3.14159265358979323846f * dia : rg * theta;
        const float sw = g * fa / fmax32(wave_speed * wave_speed, 1.0e-12f);
        const float pd = fmax32(depth - dia, 0.0f);
        area = ca + sw * pd;
        radius = ca / fmax32(cp, 1.0e-12f);
    } else {
        area = k1.y;
        radius = k1.z;
    }
    if (flags & 2) {
        const float od = fmin32(fmax32(depth, 0.0f), fmax32(k2.z, 1.0e-6f));
        const float oa = fmax32(k2.y, 1.0e-6f) * od;
        const float op = fmax32(k2.y + 2.0f * od, 1.0e-12f);
        area = oa;
        radius = oa / op;
    }
    const float len = fmax32(k0.x, 1.0e-6f);
    const float sa = fmax32(area, 1.0e-12f);
    const float sr = fmax32(radius, 1.0e-12f);
    const float slope = (k0.y + (df - dtn)) / len;
    const float fric = g * k0.w * k0.w * fabsf(q) / (powf(sr, 4.0f / 3.0f) * sa);
    const float minor = k1.w * fabsf(q) / (2.0f * len * sa);
    const float num = q + g * sa * dt * slope;
    float up = num / (1.0f + dt * (fric + minor));
    up = fmin32(fmax32(up, -k2.x), k2.x);
    return up * dt;
}

__device__ __forceinline__ float node_depth(float2 V, float A) {
    return fmax32(ff_val(ff_clamp0(V)), 0.0f) / fmax32(A, 1.0e-12f);
}

// One thread per node: the inlet exchange of its volume.
__global__ void __launch_bounds__(128) k_nodes(const __grid_constant__ NodeArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    float led[D1_TERMS] = {0.0f, 0.0f};
    if (n < a.N) {
        const float2 V = ff_clamp0(a.Va[n]);
        const int j0 = a.node_in_start[n], j1 = a.node_in_start[n + 1];
        if (j0 == j1) {
            a.Vb[n] = V;
        } else {
            float sum = 0.0f;
            for (int j = j0; j < j1; ++j) sum += a.req[a.in_qk[j].x].y;
            const float sf = fmin32(1.0f, fmax32(ff_val(V), 0.0f) / fmax32(sum, 1.0e-12f));
            float dv = 0.0f;
            for (int j = j0; j < j1; ++j) {
                const int2 qk = a.in_qk[j];
                const float2 r = a.req[qk.x];
                const float cap = r.x * a.capf[qk.y];
                const float sur = r.y * sf;
                a.capsur[qk.x] = make_float2(cap, sur);
                dv += cap - sur;
                led[0] += cap;
                led[1] += sur;
            }
            a.Vb[n] = ff_add(V, dv);
        }
    }
    warp_add_ledger<D1_TERMS>(led, a.ledger);
}

// One thread per link: the transfer volume from the end volumes after the
// inlet exchange.
__global__ void __launch_bounds__(128) k_links(const __grid_constant__ LinkArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= a.L) return;
    const int f = a.link_from[l], to = a.link_to[l];
    const float df = node_depth(a.Vb[f], a.node_area[f]);
    const float dtn = node_depth(a.Vb[to], a.node_area[to]);
    const float *Qin = s.parity ? a.Q1 : a.Q0;
    a.T[l] = link_transfer(a.lk0[l], a.lk1[l], a.lk2[l], df, dtn, Qin[l], a.g, a.wave_speed, s.dt_f);
}

// One thread per node: its donor factor min(1, V / sum of the transfers it
// gives), summed in ascending link order.
__global__ void __launch_bounds__(128) k_donor(const __grid_constant__ DonorArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const int js = a.node_link_start[n], je = a.node_link_start[n + 1];
    float given = 0.0f;
    for (int j0 = js; j0 < je; j0 += 4) {
        int2 e[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) e[u] = (j0 + u < je) ? a.nl[j0 + u] : make_int2(-1, 0);
        float t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] = e[u].x >= 0 ? a.T[e[u].x] : 0.0f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (e[u].x < 0) continue;
            const uint32_t meta = (uint32_t)e[u].y;
            if (t[u] >= 0.0f ? (meta & NL_FROM) : (meta & NL_TO)) given += fabsf(t[u]);
        }
    }
    a.fac[n] = fmin32(1.0f, fmax32(ff_val(ff_clamp0(a.Vb[n])), 0.0f) / fmax32(given, 1.0e-12f));
}

__global__ void __launch_bounds__(128) k_network(const __grid_constant__ NetArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    float4 *hs = s.parity ? a.state0 : a.state1;  // written by k_surface this step
    float *Qout = s.parity ? a.Q0 : a.Q1;
    const float dt = s.dt_f;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    float led[D2_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (g < a.G) {
        const int4 gr = a.grp[g];
        const int c = gr.x, k = gr.y;
        float h = 0.0f, area = 1.0f;
        if (c >= 0) {
            h = hs[c].x;
            area = a.cinfo[c].x;
            if (k >= 0) {  // the cell's inlet exchange, in its inlets' order
                float dh = 0.0f;
                for (int q = a.kcell_start[k]; q < a.kcell_start[k + 1]; ++q) {
                    const float2 cs = a.capsur[q];
                    dh += (cs.y - cs.x) / area;
                }
                h = h + dh;
            }
        }
        float hd = 0.0f;
        for (int n = gr.z; n < gr.w; ++n) {
            const float2 Vp = ff_clamp0(a.Vb[n]);
            const float fn = a.fac[n];
            const int js = a.node_link_start[n], je = a.node_link_start[n + 1];
            float dv = 0.0f;
            for (int j0 = js; j0 < je; j0 += 4) {
                int2 e[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) e[u] = (j0 + u < je) ? a.nl[j0 + u] : make_int2(-1, 0);
                float t[4], fo[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (e[u].x >= 0) {
                        t[u] = a.T[e[u].x];
                        fo[u] = a.fac[(uint32_t)e[u].y & NL_NODE_MASK];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (e[u].x < 0) continue;
                    const uint32_t meta = (uint32_t)e[u].y;
                    const bool is_from = (meta & NL_FROM) != 0, is_to = (meta & NL_TO) != 0;
                    // donor = the from-node for t >= 0, else the to-node
                    const bool donor_is_from = t[u] >= 0.0f || (is_from && is_to);
                    const bool donor_here = donor_is_from ? is_from : is_to;
                    const float lim = fabsf(t[u]) * (donor_here ? fn : fo[u]);
                    const float sgn = donor_is_from ? lim : -lim;
                    if (is_from) {
                        dv -= sgn;
                        Qout[e[u].x] = sgn / fmax32(dt, 1.0e-12f);
                        led[3] += lim;
                    }
                    if (is_to) dv += sgn;
                }
            }
            float2 V = ff_clamp0(ff_add(Vp, dv));
            // outfall (reference pipe_outfall_kernel :176-211)
            const float4 nd = a.nd0[n];
            const float vol = fmax32(ff_val(V), 0.0f);
            if (nd.z > 0.0f) {
                const float dh = nd.y + vol / fmax32(nd.x, 1.0e-12f);
                const float sgn = (float)((dh > 0.0f) - (dh < 0.0f));
                float qo = nd.z * sqrtf(2.0f * a.g * fabsf(dh)) * sgn;
                qo = fmin32(qo, nd.w);
                const float out = fmin32(vol, fmax32(qo, 0.0f) * dt);
                V = ff_add(V, -out);
                led[0] += out;
            }
            // overflow return (reference node_overflow_return_kernel :179-207)
            const float capv = a.nd_capv[n];
            const float ovf = fmax32(ff_val(V) - capv, 0.0f);
            if (c >= 0 && ovf > 0.0f) {
                V = ff_add(V, -ovf);
                hd += ovf / area;
                led[1] += ovf;
            }
            led[2] += fmax32(ff_val(V) - capv, 0.0f);
            a.Va[n] = V;
            if (s.snap_slot >= 0) a.snap_v[(size_t)s.snap_slot * (size_t)a.N + n] = ff_val(V);
        }
        if (c >= 0) {
            const float hf = h + hd;
            hs[c].x = hf;
            if ((s.phases & FL_PHASE_SURFACE) && a.forcing_kind == 1) a.wet[c] = a.wet[c] + dt * (float)(hf > a.md);
            if (s.snap_slot >= 0) a.snap_h[(size_t)s.snap_slot * (size_t)a.C + c] = hf;
        }
    }
    warp_add_ledger<D2_TERMS>(led, a.ledger);
}

int node_blocks(int32_t N) { return (N + 127) / 128 > 0 ? (N + 127) / 128 : 1; }
int network_blocks(int32_t G) { return (G + 127) / 128 > 0 ? (G + 127) / 128 : 1; }

cudaError_t launch_nodes(const NodeArgs &a, int slot, cudaStream_t stream) {
    k_nodes<<<node_blocks(a.N), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

int link_blocks(int32_t L) { return (L + 127) / 128 > 0 ? (L + 127) / 128 : 1; }

cudaError_t launch_links(const LinkArgs &a, int slot, cudaStream_t stream) {
    k_links<<<link_blocks(a.L), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

cudaError_t launch_donor(const DonorArgs &a, int slot, cudaStream_t stream) {
    k_donor<<<node_blocks(a.N), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

cudaError_t launch_network(const NetArgs &a, int slot, cudaStream_t stream) {
    k_network<<<network_blocks(a.G), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

}  // namespace fl
