// Drainage kernels for sm_103a: the coupled 1D network of the reference
// (gurugram_flood/kernels/triangular_inlet_exchange_cuda_kernels.py and
// triangular_pipe_network_cuda_kernels.py), restated without atomics.
//
// The reference does each many-to-one sum (requests per cell, per node, per
// donor node; volume deltas per node; depth deltas per cell) with float64
// atomicAdd.  Here every sum is a gather over a precomputed list in a fixed
// order, so runs are reproducible, and every exchanged quantity is computed
// once and read by both sides, so volume is conserved exactly as in the
// reference.  Per step, after k_surface:
//   k_nodes   one thread per node: the capture and surcharge requests of its
//             inlets from the depth the surface step left in their cells
//             [reference :52-131], captures limited by their cells' volume,
//             surcharges by the node's, the node volume after the exchange
//                                                         [reference :133-177]
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
#include <algorithm>

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

// The drainage step's four passes as per-item functions; each kernel below
// runs one pass with one thread per item.  Values one pass writes and a
// later one reads (Vb, capsur, T, fac) are read through L2 (ld.cg).  Each
// kernel issues the loads that do not depend on the step record (the
// item's static indices, the values earlier kernels wrote) before that
// record arrives, so its latency overlaps theirs instead of adding to the
// dependent-load chain.
//
// k_links, k_donor and k_network are launched as programmatic dependents of
// the kernel before them: each kernel lets its dependent launch as soon as
// its own blocks run (griddepcontrol.launch_dependents), and the dependent
// loads its static tables, then waits for the whole previous grid to finish
// and its writes to be visible (griddepcontrol.wait) before it reads them.
// The launch latency and the static loads of each kernel overlap the
// previous one.  k_nodes follows the surface kernel with an ordinary launch.


// Capture limit factor of an inlet cell at depth h: its volume over the
// summed capture requests of its inlets [q0, q1), in their order (reference
// :133-177).  `own` is the capture request of the calling inlet: a cell whose
// only inlet it is needs no other node's volume (the sum is 0 + own, as the
// loop would form it; this file is compiled without contraction, so the
// request is rounded identically either way).
__device__ __forceinline__ float cell_capture_factor(const InletReqView &v, int q0, int q1, float own, float h,
                                                     float area, float dt) {
    float sum = 0.0f;
    if (q1 - q0 == 1) {
        sum = sum + own;
    } else {
        for (int q = q0; q < q1; ++q) sum += inlet_request(v, q, h, ff_clamp0(v.Va[v.in_node[q]]), dt).x;
    }
    return fmin32(1.0f, (fmax32(h, 0.0f) * area) / fmax32(sum, 1.0e-12f));
}

// Node n: the requests of its inlets from the depth the surface step left in
// their cells (reference inlet_exchange_request_kernel :52-131), captures
// limited by each cell's volume, surcharges by the node's, and the node
// volume after the exchange.
// V = the clamped start volume Va[n]; [j0, j1) = the node's inlets.
__device__ __forceinline__ void node_item(const NodeArgs &a, const StepCtrl &s, int n, float2 V, int j0, int j1,
                                          float (&led)[D1_TERMS]) {
    if (j0 == j1) {
        a.Vb[n] = V;
        return;
    }
    const float4 *hs = s.parity ? a.state0 : a.state1;  // written by the surface step
    const float dt = s.dt_f;
    float sum = 0.0f;
    for (int j = j0; j < j1; ++j) {
        const int4 qk = a.in_qk[j];
        sum += inlet_request(a.inl, qk.x, hs[qk.y].x, V, dt).y;
    }
    const float sf = fmin32(1.0f, fmax32(ff_val(V), 0.0f) / fmax32(sum, 1.0e-12f));
    float dv = 0.0f;
    for (int j = j0; j < j1; ++j) {
        const int4 qk = a.in_qk[j];
        const int c = qk.y;
        const float h = hs[c].x;
        const float2 r = inlet_request(a.inl, qk.x, h, V, dt);
        const float cap = r.x * cell_capture_factor(a.inl, qk.z, qk.w, r.x, h, a.cinfo[c].x, dt);
        const float sur = r.y * sf;
        a.capsur[qk.x] = make_float2(cap, sur);
        dv += cap - sur;
        led[0] += cap;
        led[1] += sur;
    }
    a.Vb[n] = ff_add(V, dv);
}

// Node n: its donor factor min(1, V / sum of the transfers it gives), summed
// in ascending link order.
// [js, je) = the node's link slots.
__device__ __forceinline__ float donor_item(const DonorArgs &a, int n, int js, int je) {
    float given = 0.0f;
    for (int j0 = js; j0 < je; j0 += 4) {
        int2 e[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) e[u] = (j0 + u < je) ? a.nl[j0 + u] : make_int2(-1, 0);
        float t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] = e[u].x >= 0 ? __ldcg(&a.T[e[u].x]) : 0.0f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (e[u].x < 0) continue;
            const uint32_t meta = (uint32_t)e[u].y;
            if (t[u] >= 0.0f ? (meta & NL_FROM) : (meta & NL_TO)) given += fabsf(t[u]);
        }
    }
    return fmin32(1.0f, fmax32(ff_val(ff_clamp0(__ldcg(&a.Vb[n]))), 0.0f) / fmax32(given, 1.0e-12f));
}

// Group g: limited transfers, node continuity, outfall, overflow return and
// the group cell's final depth.
// gr = the group record grp[g]; ci = the cell info of its cell (if any).
__device__ __forceinline__ void group_item(const NetArgs &a, const StepCtrl &s, int4 gr, float4 ci,
                                           float (&led)[D2_TERMS]) {
    float4 *hs = s.parity ? a.state0 : a.state1;  // written by k_surface this step
    float *Qout = s.parity ? a.Q0 : a.Q1;
    const float dt = s.dt_f;
    const int c = gr.x, k = gr.y;
    float h = 0.0f, area = 1.0f;
    uint32_t cflags = 0u;
    if (c >= 0) {
        h = hs[c].x;
        area = ci.x;
        cflags = __float_as_uint(ci.z);
        if (k >= 0) {  // the cell's inlet exchange, in its inlets' order
            float dh = 0.0f;
            for (int q = a.kcell_start[k]; q < a.kcell_start[k + 1]; ++q) {
                const float2 cs = __ldcg(&a.capsur[q]);
                dh += (cs.y - cs.x) / area;
            }
            h = h + dh;
        }
    }
    float hd = 0.0f;
    double hd64 = 0.0;  // table mode: the fallback return depth in float64
    for (int n = gr.z; n < gr.w; ++n) {
        const float2 Vp = ff_clamp0(__ldcg(&a.Vb[n]));
        const float fn = __ldcg(&a.fac[n]);
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
                    t[u] = __ldcg(&a.T[e[u].x]);
                    fo[u] = __ldcg(&a.fac[(uint32_t)e[u].y & NL_NODE_MASK]);
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
        const float capv = a.nd_capv[n];
        if (a.table) {
            // weighted return (reference triangular_backend.py:1424-1474) in
            // float64: a node with table entries returns overflow x weight
            // through them (at most its overflow); the others fall back to
            // their cell
            const double ovf = fmax((double)V.x + (double)V.y - (double)capv, 0.0);
            const int e0 = a.node_tstart[n], e1 = a.node_tstart[n + 1];
            double r = 0.0;
            if (e1 > e0) {
                for (int e = e0; e < e1; ++e) r += ovf * (double)a.node_tw[e];
                r = fmin(r, ovf);
                a.ovf_node[n] = ovf;
            } else if (c >= 0) {
                r = ovf;
                hd64 += r / (double)area;
            }
            if (r > 0.0) {
                const float rh = (float)r;
                V = ff_add(ff_add(V, -rh), -(float)(r - (double)rh));
                led[1] += rh;
            }
        } else {
            // overflow return (reference node_overflow_return_kernel :179-207)
            const float ovf = fmax32(ff_val(V) - capv, 0.0f);
            if (c >= 0 && ovf > 0.0f) {
                V = ff_add(V, -ovf);
                hd += ovf / area;
                led[1] += ovf;
            }
        }
        led[2] += fmax32(ff_val(V) - capv, 0.0f);
        a.Va[n] = V;
        if (s.snap_slot >= 0) a.snap_v[(size_t)s.snap_slot * (size_t)a.N + n] = ff_val(V);
    }
    if (c >= 0 && a.table && (cflags & CELL_SURCHARGE)) {
        // k_surcharge adds the table's return first, then this fallback
        hs[c].x = h;
        int lo = 0, hi = a.U;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (a.tcell[mid] < c) lo = mid + 1; else hi = mid;
        }
        a.s2[lo] = hd64;
    } else if (c >= 0) {
        const float hf = a.table ? (float)((double)h + hd64) : h + hd;
        hs[c].x = hf;
        // a recharge cell is finished by k_recharge
        const bool fin = !(a.has_recharge && (s.phases & FL_PHASE_RECHARGE) && (cflags & CELL_RECHARGE));
        if (fin) {
            if ((s.phases & FL_PHASE_SURFACE) && a.forcing_kind == 1) a.wet[c] = a.wet[c] + dt * (float)(hf > a.md);
            if (s.snap_slot >= 0) a.snap_h[(size_t)s.snap_slot * (size_t)a.C + c] = hf;
        }
    }
}

// Ensemble members: a batched launch runs member blockIdx.y; these move the
// per-member pointers of the arguments to that member's arrays (the static
// tables are shared).  A single run uses the arguments as they are.
__device__ __forceinline__ NodeArgs member_args(NodeArgs a, int m) {
    const MemberStrides &z = a.ms;
    a.state0 += m * z.cells;
    a.state1 += m * z.cells;
    a.capsur += m * z.inlets;
    a.Va += m * z.nodes;
    a.Vb += m * z.nodes;
    a.inl.Va += m * z.nodes;
    a.ctrl += 2 * m;
    a.ledger += m * z.led1;
    return a;
}

__device__ __forceinline__ LinkArgs member_args(LinkArgs a, int m) {
    const MemberStrides &z = a.ms;
    a.Vb += m * z.nodes;
    a.Q0 += m * z.links;
    a.Q1 += m * z.links;
    a.T += m * z.links;
    a.ctrl += 2 * m;
    return a;
}

__device__ __forceinline__ DonorArgs member_args(DonorArgs a, int m) {
    const MemberStrides &z = a.ms;
    a.Vb += m * z.nodes;
    a.T += m * z.links;
    a.fac += m * z.nodes;
    a.ctrl += 2 * m;
    return a;
}

__device__ __forceinline__ NetArgs member_args(NetArgs a, int m) {
    const MemberStrides &z = a.ms;
    a.capsur += m * z.inlets;
    a.T += m * z.links;
    a.fac += m * z.nodes;
    a.state0 += m * z.cells;
    a.state1 += m * z.cells;
    a.Vb += m * z.nodes;
    a.Va += m * z.nodes;
    a.Q0 += m * z.links;
    a.Q1 += m * z.links;
    a.wet += m * z.cells;
    a.snap_h += m * z.snap_h;
    a.snap_v += m * z.snap_v;
    a.ctrl += 2 * m;
    a.ledger += m * z.led2;
    return a;
}

template <bool MEM>
__global__ void __launch_bounds__(128) k_nodes(const __grid_constant__ NodeArgs a0, int slot) {
    const NodeArgs a = MEM ? member_args(a0, (int)blockIdx.y) : a0;
    pdl_launch_dependents();
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = n < a.N;
    const float2 V = in ? ff_clamp0(a.Va[n]) : make_float2(0.0f, 0.0f);
    const int j0 = in ? a.node_in_start[n] : 0, j1 = in ? a.node_in_start[n + 1] : 0;
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    float led[D1_TERMS] = {0.0f, 0.0f};
    if (in) node_item(a, s, n, V, j0, j1, led);
    warp_add_ledger<D1_TERMS>(led, a.ledger);
}

// Link l: the transfer volume from the end volumes after the inlet exchange
// (all inputs loaded before the step record; the flow of the step's parity).
template <bool MEM>
__global__ void __launch_bounds__(128) k_links(const __grid_constant__ LinkArgs a0, int slot) {
    const LinkArgs a = MEM ? member_args(a0, (int)blockIdx.y) : a0;
    pdl_launch_dependents();
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = l < a.L;
    const int f = in ? a.link_from[l] : 0, to = in ? a.link_to[l] : 0;
    float4 k0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), k1 = k0, k2 = k0;
    float q0 = 0.0f, q1 = 0.0f, af = 1.0f, at = 1.0f;
    if (in) {  // static tables and the previous step's flow
        k0 = a.lk0[l];
        k1 = a.lk1[l];
        k2 = a.lk2[l];
        q0 = a.Q0[l];
        q1 = a.Q1[l];
        af = a.node_area[f];
        at = a.node_area[to];
    }
    pdl_wait();  // k_nodes' volumes
    float df = 0.0f, dtn = 0.0f;
    if (in) {
        df = node_depth(__ldcg(&a.Vb[f]), af);
        dtn = node_depth(__ldcg(&a.Vb[to]), at);
    }
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    if (in) a.T[l] = link_transfer(k0, k1, k2, df, dtn, s.parity ? q1 : q0, a.g, a.wave_speed, s.dt_f);
}

// The donor factor depends on nothing the step record selects: it is formed
// while the record loads and stored only on an active step.
template <bool MEM>
__global__ void __launch_bounds__(128) k_donor(const __grid_constant__ DonorArgs a0, int slot) {
    const DonorArgs a = MEM ? member_args(a0, (int)blockIdx.y) : a0;
    pdl_launch_dependents();
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const StepCtrl s = a.ctrl[slot];
    const int js = n < a.N ? a.node_link_start[n] : 0, je = n < a.N ? a.node_link_start[n + 1] : 0;
    pdl_wait();  // k_links' transfers
    if (n >= a.N) return;
    const float fac = donor_item(a, n, js, je);
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    a.fac[n] = fac;
}

template <bool MEM>
__global__ void __launch_bounds__(128) k_network(const __grid_constant__ NetArgs a0, int slot) {
    const NetArgs a = MEM ? member_args(a0, (int)blockIdx.y) : a0;
    pdl_launch_dependents();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int4 gr = g < a.G ? a.grp[g] : make_int4(-1, -1, 0, 0);
    const float4 ci = gr.x >= 0 ? a.cinfo[gr.x] : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    const StepCtrl s = a.ctrl[slot];
    pdl_wait();  // k_donor's factors (and, through it, every earlier kernel's writes)
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    float led[D2_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (g < a.G) group_item(a, s, gr, ci, led);
    warp_add_ledger<D2_TERMS>(led, a.ledger);
}

// Weighted surcharge return into the table cells (reference
// triangular_backend.py:1424-1474), after k_network: h = float32((h + sum
// over the cell's entries, in entry order, of overflow x weight / area) +
// the fallback return of the cell's own nodes), then the cell is finished.
__global__ void __launch_bounds__(128) k_surcharge(const __grid_constant__ SurchargeArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= a.U) return;
    float4 *hs = s.parity ? a.state0 : a.state1;
    const int c = a.cell[u];
    const double area = (double)a.cinfo[c].x;
    double s1 = 0.0;
    for (int k = a.start[u]; k < a.start[u + 1]; ++k) {
        const int2 e = a.ent[k];
        s1 += a.ovf_node[e.x] * (double)__int_as_float(e.y) / area;
    }
    const float hf = (float)(((double)hs[c].x + s1) + a.s2[u]);
    hs[c].x = hf;
    const bool fin = !(a.has_recharge && (s.phases & FL_PHASE_RECHARGE) &&
                       (__float_as_uint(a.cinfo[c].z) & CELL_RECHARGE));
    if (fin) {
        const float dt = s.dt_f;
        if ((s.phases & FL_PHASE_SURFACE) && a.forcing_kind == 1) a.wet[c] = a.wet[c] + dt * (float)(hf > a.md);
        if (s.snap_slot >= 0) a.snap_h[(size_t)s.snap_slot * (size_t)a.C + c] = hf;
    }
}

int surcharge_blocks(int32_t U) { return (U + 127) / 128 > 0 ? (U + 127) / 128 : 1; }

cudaError_t launch_surcharge(const SurchargeArgs &a, int slot, cudaStream_t stream) {
    k_surcharge<<<surcharge_blocks(a.U), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

// Receiver j's hydrograph at time t (reference production_event_support.py
// :169-178): the first / last value outside the table, else np.interp's
// linear interpolation in float64 (slope over the bracketing interval, the
// exact value at a table time, the other end's form if the first gives NaN),
// rounded to float32.
__device__ __forceinline__ float inflow_q(const InflowArgs &a, int j, int k, double t) {
    const size_t J = (size_t)a.J;
    if (k < 0) return a.q[j];
    if (k >= a.T - 1) return a.q[(size_t)(a.T - 1) * J + j];
    const double x0 = a.times[k], x1 = a.times[k + 1];
    const double y0 = (double)a.q[(size_t)k * J + j], y1 = (double)a.q[(size_t)(k + 1) * J + j];
    if (x0 == t) return (float)y0;
    const double slope = __ddiv_rn(__dsub_rn(y1, y0), __dsub_rn(x1, x0));
    double r = __dadd_rn(__dmul_rn(slope, __dsub_rn(t, x0)), y0);
    if (isnan(r)) {
        r = __dadd_rn(__dmul_rn(slope, __dsub_rn(t, x1)), y1);
        if (isnan(r) && y0 == y1) r = y0;
    }
    return (float)r;
}

// External boundary inflow of the step (reference production_event_support.py
// :181-196, applied at t + dt/2 after the clamp, engine.py:263-273): each
// receiver adds float32(q) * dt / area into its cell's sum (np.add.at on
// zeros, receivers in index order); the surface kernel then adds the sum to
// the cell's depth.  Each receiver's volume goes to its own ledger slot.
__global__ void __launch_bounds__(128) k_inflow(const __grid_constant__ InflowArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_INFLOW)) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= a.U) return;
    const double t = __dadd_rn(s.t0, __dmul_rn(0.5, s.dt));
    // k: -1 before the table, T - 1 at or after its end, else times[k] <= t < times[k + 1]
    int k;
    if (t <= a.times[0]) {
        k = -1;
    } else if (t >= a.times[a.T - 1]) {
        k = a.T - 1;
    } else {
        int lo = 0, hi = a.T - 1;  // times[lo] < t < times[hi]
        while (hi - lo > 1) {
            const int m = (lo + hi) >> 1;
            if (a.times[m] <= t) lo = m; else hi = m;
        }
        k = lo;
    }
    const int c = a.cell[u];
    const float area = a.cinfo[c].x;
    float sum = 0.0f;
    for (int e = a.start[u]; e < a.start[u + 1]; ++e) {
        const int j = a.recv[e];
        const float added = __fmul_rn(inflow_q(a, j, k, t), s.dt_f);
        sum = __fadd_rn(sum, __fdiv_rn(added, area));
        ff_accumulate(&a.led[j], added);
    }
    a.add[c] = sum;
}

int inflow_blocks(int32_t U) { return (U + 127) / 128 > 0 ? (U + 127) / 128 : 1; }

cudaError_t launch_inflow(const InflowArgs &a, int slot, cudaStream_t stream) {
    k_inflow<<<inflow_blocks(a.U), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

// Surface recharge (reference june5_production_drainage.py:543-572), after
// the drainage step: one thread per recharge cell runs the cell's rows in
// table order on the depth the step left (every row sees that depth), keeps
// the last row's capture for the cell's final depth (NumPy's assignment with
// repeated indices), and finishes the cell (wet time, depth snapshot).
__global__ void __launch_bounds__(128) k_recharge(const __grid_constant__ RechargeArgs a, int slot) {
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_RECHARGE)) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= a.U) return;
    float4 *hs = s.parity ? a.state0 : a.state1;
    const float dt = s.dt_f;
    const int c = a.cell[u];
    const float h = hs[c].x;
    const float area = fmax32(a.cinfo[c].x, 1.0e-6f);
    float hf = h;
    for (int k = a.row_start[u]; k < a.row_start[u + 1]; ++k) {
        const int r = a.rows[k];
        const float4 p = a.par[r];  // {storage capacity, capture capacity, recharge capacity, stop depth}
        const float available = __fmul_rn(fmax32(__fsub_rn(h, p.w), 0.0f), area);
        const float request = __fmul_rn(p.y, dt);
        float st = a.storage[r];
        const float remaining = fmax32(__fsub_rn(p.x, st), 0.0f);
        const float cap = fmin32(fmin32(available, request), remaining);
        hf = fmax32(__fsub_rn(h, __fdiv_rn(cap, area)), 0.0f);
        st = __fadd_rn(st, cap);
        const float loss = fmin32(st, __fmul_rn(p.z, dt));
        a.storage[r] = __fsub_rn(st, loss);
        ff_accumulate(&a.led[2 * r], cap);
        ff_accumulate(&a.led[2 * r + 1], loss);
    }
    hs[c].x = hf;
    if ((s.phases & FL_PHASE_SURFACE) && a.forcing_kind == 1) a.wet[c] = a.wet[c] + dt * (float)(hf > a.md);
    if (s.snap_slot >= 0) a.snap_h[(size_t)s.snap_slot * (size_t)a.C + c] = hf;
}

int recharge_blocks(int32_t U) { return (U + 127) / 128 > 0 ? (U + 127) / 128 : 1; }

cudaError_t launch_recharge(const RechargeArgs &a, int slot, cudaStream_t stream) {
    k_recharge<<<recharge_blocks(a.U), 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

int node_blocks(int32_t N) { return (N + 127) / 128 > 0 ? (N + 127) / 128 : 1; }
int network_blocks(int32_t G) { return (G + 127) / 128 > 0 ? (G + 127) / 128 : 1; }

cudaError_t launch_nodes(const NodeArgs &a, int slot, cudaStream_t stream) {
    const dim3 grid((unsigned)node_blocks(a.N), (unsigned)std::max(a.ms.n, 1));
    if (a.ms.n > 1) k_nodes<true><<<grid, 128, 0, stream>>>(a, slot);
    else k_nodes<false><<<grid, 128, 0, stream>>>(a, slot);
    return cudaGetLastError();
}

int link_blocks(int32_t L) { return (L + 127) / 128 > 0 ? (L + 127) / 128 : 1; }

// Launch as a programmatic dependent of the previous kernel in the stream.
template <class Args>
static cudaError_t launch_dependent(void (*kernel)(Args, int), int blocks, const Args &a, int slot,
                                    cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks, (unsigned)std::max(a.ms.n, 1));
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a, slot);
}

cudaError_t launch_links(const LinkArgs &a, int slot, cudaStream_t stream) {
    return launch_dependent(a.ms.n > 1 ? k_links<true> : k_links<false>, link_blocks(a.L), a, slot, stream);
}

cudaError_t launch_donor(const DonorArgs &a, int slot, cudaStream_t stream) {
    return launch_dependent(a.ms.n > 1 ? k_donor<true> : k_donor<false>, node_blocks(a.N), a, slot, stream);
}

cudaError_t launch_network(const NetArgs &a, int slot, cudaStream_t stream) {
    return launch_dependent(a.ms.n > 1 ? k_network<true> : k_network<false>, network_blocks(a.G), a, slot, stream);
}

}  // namespace fl
