// Drainage kernels for sm_103a: the coupled 1D network of the reference
// (gurugram_flood/kernels/triangular_inlet_exchange_cuda_kernels.py and
// triangular_pipe_network_cuda_kernels.py), restated without atomics.
//
// The reference does each many-to-one sum (requests per cell, per node, per
// donor node; volume deltas per node; depth deltas per cell) with float64
// atomicAdd.  Here every sum is a gather over a precomputed CSR list in a
// fixed order, and where a quantity of a neighbour is needed (the capture
// limit of an inlet's cell, the surcharge limit of its node, the donor limit
// of a link's other end) it is recomputed from the same inputs with the same
// code, so both sides of every exchange see bit-identical values: volume is
// conserved exactly as in the reference and runs are reproducible.
//
// The inlet requests (reference :52-131) are evaluated by k_surface, which
// holds each inlet cell's post-surface depth; then three launches per step:
//   k_inlets  one thread per inlet cell (depth after the exchange) and one per
//             node (volume after the exchange)              [reference :133-177]
//   k_links   one thread per link: the semi-implicit link update from the two
//             end volumes after the exchange              [pipe network :39-139]
//   k_network one thread per drainage group = a surface cell together with
//             the nodes that overflow into it (or an orphan node): donor
//             limiting of the link transfers, node continuity, outfall,
//             overflow return and the cell's final depth      [reference
//             pipe network :141-211, overflow :179-207]
//
// Heads are carried as depth relative to a static per-link / per-inlet datum
// offset (bed - invert, invert_from - invert_to, ...), so float32 keeps
// millimetre-scale head differences exact at 200 m elevations; node storage
// volume is a float-float pair so small exchanges are not lost against large
// stored volumes.  No FP64 arithmetic is used on this path.
#include "fl_device.cuh"

namespace fl {

// Capture limit factor of inlet cell k: surface volume over the summed
// requests of its inlets (reference inlet_exchange_apply_kernel :133-177).
__device__ __forceinline__ float cell_capture_factor(const D1Args &a, const float4 *hs, int k) {
    const int c = a.kcell_cell[k];
    float sum = 0.0f;
    for (int i = a.kcell_start[k]; i < a.kcell_start[k + 1]; ++i) sum += a.req[i].x;
    return fmin32(1.0f, (fmax32(hs[c].x, 0.0f) * a.cinfo[c].x) / fmax32(sum, 1.0e-12f));
}

// Surcharge limit factor of node n: stored volume over the summed requests.
__device__ __forceinline__ float node_surcharge_factor(const D1Args &a, int n) {
    float sum = 0.0f;
    for (int j = a.node_in_start[n]; j < a.node_in_start[n + 1]; ++j) sum += a.req[a.node_in_list[j]].y;
    return fmin32(1.0f, fmax32(ff_val(ff_clamp0(a.Va[n])), 0.0f) / fmax32(sum, 1.0e-12f));
}

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

// One thread per inlet cell (its depth after the exchange) and one per node
// (its volume after the exchange).  The requests were written by k_surface;
// each limit factor is a fixed-order sum over the same values in both the
// cell's and the node's thread, so capture and surcharge balance exactly.
__global__ void __launch_bounds__(128) k_inlets(const __grid_constant__ D1Args a, int slot) {
    wait_for_previous_grid();
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    allow_next_grid();
    const float4 *hs = s.parity ? a.state0 : a.state1;  // written by k_surface this step
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float led[D1_TERMS] = {0.0f, 0.0f};
    if (t < a.K) {
        const int k = t;
        const int c = a.kcell_cell[k];
        const float h = hs[c].x;
        const float area = a.cinfo[c].x;
        const float capf = cell_capture_factor(a, hs, k);
        float dh = 0.0f;
        for (int i = a.kcell_start[k]; i < a.kcell_start[k + 1]; ++i) {
            const float2 r = a.req[i];
            const float cap = r.x * capf;
            const float sur = r.y * node_surcharge_factor(a, a.in_node[i]);
            dh += (sur - cap) / area;
            led[0] += cap;
            led[1] += sur;
        }
        a.hc_out[k] = h + dh;
    } else if (t < a.K + a.N) {
        const int n = t - a.K;
        const float2 V = ff_clamp0(a.Va[n]);
        const int j0 = a.node_in_start[n], j1 = a.node_in_start[n + 1];
        if (j0 == j1) {
            a.Vb[n] = V;
        } else {
            const float surf = node_surcharge_factor(a, n);
            float dv = 0.0f;
            for (int j = j0; j < j1; ++j) {
                const int i = a.node_in_list[j];
                const float2 r = a.req[i];
                dv += r.x * cell_capture_factor(a, hs, a.in_kcell[i]) - r.y * surf;
            }
            a.Vb[n] = ff_add(V, dv);
        }
    }
    warp_add_ledger<D1_TERMS>(led, a.ledger);
}

// One thread per link: the transfer volume from the end volumes after the
// inlet exchange.
__global__ void __launch_bounds__(128) k_links(const __grid_constant__ LinkArgs a, int slot) {
    wait_for_previous_grid();
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    allow_next_grid();
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= a.L) return;
    const int f = a.link_from[l], to = a.link_to[l];
    const float df = node_depth(a.Vb[f], a.node_area[f]);
    const float dtn = node_depth(a.Vb[to], a.node_area[to]);
    const float *Qin = s.parity ? a.Q1 : a.Q0;
    a.T[l] = link_transfer(a.lk0[l], a.lk1[l], a.lk2[l], df, dtn, Qin[l], a.g, a.wave_speed, s.dt_f);
}

// Sum of |transfer| over the links whose donor is node d.
__device__ __forceinline__ float donor_request(const D2Args &a, int d) {
    float sum = 0.0f;
    for (int j = a.node_link_start[d]; j < a.node_link_start[d + 1]; ++j) {
        const int l = a.node_link_list[j];
        const float t = a.T[l];
        const int donor = t >= 0.0f ? a.link_from[l] : a.link_to[l];
        if (donor == d) sum += fabsf(t);
    }
    return sum;
}

__global__ void __launch_bounds__(128) k_network(const __grid_constant__ D2Args a, int slot) {
    wait_for_previous_grid();
    const StepCtrl s = a.ctrl[slot];
    if (!s.active || !(s.phases & FL_PHASE_DRAINAGE)) return;
    float4 *hs = s.parity ? a.state0 : a.state1;  // written by k_surface this step
    float *Qout = s.parity ? a.Q0 : a.Q1;
    const float dt = s.dt_f;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    float led[D2_TERMS] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (g < a.G) {
        const int c = a.grp_cell[g];
        const int k = a.grp_kcell[g];
        float h = 0.0f, area = 1.0f;
        if (c >= 0) {
            h = (k >= 0) ? a.hc_out[k] : hs[c].x;
            area = a.cinfo[c].x;
        }
        float hd = 0.0f;
        for (int gi = a.grp_start[g]; gi < a.grp_start[g + 1]; ++gi) {
            const int n = a.grp_nodes[gi];
            const float2 Vp = ff_clamp0(a.Vb[n]);
            const float Vpf = fmax32(ff_val(Vp), 0.0f);
            const int j0 = a.node_link_start[n], j1 = a.node_link_start[n + 1];
            const float own = donor_request(a, n);
            float dv = 0.0f;
            for (int j = j0; j < j1; ++j) {
                const int l = a.node_link_list[j];
                const float t = a.T[l];
                const int from = a.link_from[l], to = a.link_to[l];
                const int d = t >= 0.0f ? from : to;
                float factor;
                if (d == n) {
                    factor = fmin32(1.0f, Vpf / fmax32(own, 1.0e-12f));
                } else {
                    const float Vd = fmax32(ff_val(ff_clamp0(a.Vb[d])), 0.0f);
                    factor = fmin32(1.0f, Vd / fmax32(donor_request(a, d), 1.0e-12f));
                }
                const float lim = fabsf(t) * factor;
                const float sgn = (d == from) ? lim : -lim;
                if (from == n) {
                    dv -= sgn;
                    Qout[l] = sgn / fmax32(dt, 1.0e-12f);
                    led[3] += lim;
                }
                if (to == n) dv += sgn;
            }
            float2 V = ff_clamp0(ff_add(Vp, dv));
            // outfall (reference pipe_outfall_kernel :176-211)
            const float4 nd = a.nd0[n];
            const float vol = fmax32(ff_val(V), 0.0f);
            if (nd.z > 0.0f) {
                const float dh = nd.y + vol / fmax32(nd.x, 1.0e-12f);
                const float sgn = (float)((dh > 0.0f) - (dh < 0.0f));
                float q = nd.z * sqrtf(2.0f * a.g * fabsf(dh)) * sgn;
                q = fmin32(q, nd.w);
                const float out = fmin32(vol, fmax32(q, 0.0f) * dt);
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

static cudaError_t launch_pdl2(const void *func, dim3 grid, dim3 block, void **args, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, func, args);
}

int inlet_blocks(int32_t K, int32_t N) { return (K + N + 127) / 128 > 0 ? (K + N + 127) / 128 : 1; }
int link_blocks(int32_t L) { return (L + 127) / 128 > 0 ? (L + 127) / 128 : 1; }
int network_blocks(int32_t G) { return (G + 127) / 128 > 0 ? (G + 127) / 128 : 1; }

cudaError_t launch_inlets(const D1Args &a, int slot, cudaStream_t stream) {
    void *args[] = {(void *)&a, (void *)&slot};
    return launch_pdl2((const void *)k_inlets, dim3(inlet_blocks(a.K, a.N)), dim3(128), args, stream);
}

cudaError_t launch_links(const LinkArgs &a, int slot, cudaStream_t stream) {
    void *args[] = {(void *)&a, (void *)&slot};
    return launch_pdl2((const void *)k_links, dim3(link_blocks(a.L)), dim3(128), args, stream);
}

cudaError_t launch_network(const D2Args &a, int slot, cudaStream_t stream) {
    void *args[] = {(void *)&a, (void *)&slot};
    return launch_pdl2((const void *)k_network, dim3(network_blocks(a.G)), dim3(128), args, stream);
}

}  // namespace fl
