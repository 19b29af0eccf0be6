// Batched-ensemble runtime behind the fl_batch_* entry points of
// include/floodgb.h: per-scenario layouts built with the single-scenario
// planner and concatenated tile by tile, device memory, the lockstep step
// loop as CUDA-graph chunks (surface launch + planning launch per step), and
// state / snapshot / ledger readout per scenario.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/floodgb.h"
#include "fl_batch.cuh"

namespace fl {

int set_error(int code, const char *fmt, ...);
int build_mesh_layout(const FlMeshDesc &m, const FlDrainDesc *d, HostLayout &L);
cudaError_t batch_configure(int kind, int tile, int smem_bytes, int *per_sm);
cudaError_t launch_surface_batch(const BatchArgs &a, int kind, int grid, int smem_bytes, cudaStream_t stream);
cudaError_t launch_cfl_batch(const float4 *state0, const float *char_len, const int32_t *tile_valid, float *tile_min,
                             int tiles, int tile, float cfl, float g, float md, cudaStream_t stream);
cudaError_t launch_plan_batch(const PlanArgs &a, int slot, int init, cudaStream_t stream);
cudaError_t launch_permute_f32(const float *src, float *dst, const int32_t *perm, int32_t C, int to_reference,
                               cudaStream_t stream);
void add_launches(int64_t n);

}  // namespace fl

using namespace fl;

#define FB_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess) return set_error(FL_E_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

struct FlBatch {
    int device = 0;
    int32_t S = 0;
    int kind = 0;
    int tile = 256;
    int chunk = 32;
    int grid = 0, smem = 0;
    int64_t cells = 0;  // padded, all scenarios
    int32_t tiles = 0;
    std::vector<FlParams> params;
    std::vector<int32_t> cell0, cells_s, tile0;  // per scenario (cell0 = first padded cell)
    std::vector<int64_t> snap_base_h;
    std::vector<std::vector<float>> area;        // per scenario, renumbered order
    int32_t max_snaps = 1;
    std::vector<void *> allocs;
    // device
    float4 *state[2] = {nullptr, nullptr};
    float4 *init_state = nullptr;
    float *hmax = nullptr, *wet = nullptr;
    int32_t *perm = nullptr;     // [cells] renumbered -> reference cell of its scenario
    float *stage_f = nullptr;    // [largest scenario]
    int32_t *tile_valid = nullptr;
    RunCtrl *run = nullptr;
    StepCtrl *ctrl = nullptr;
    BatchList *list = nullptr;
    float2 *ledger = nullptr;
    BatchArgs ba{};
    PlanArgs pa{};
    // host
    BatchList *poll_h = nullptr;  // pinned, 2 slots (header only is read)
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};

    template <class T>
    int alloc(T **p, size_t count) {
        if (count == 0) count = 1;
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, sizeof(T) * count);
        if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
        allocs.push_back(q);
        *p = (T *)q;
        return FL_OK;
    }
    template <class T>
    int upload(T **p, const std::vector<T> &v) {
        int rc = alloc(p, v.size());
        if (rc) return rc;
        if (!v.empty()) FB_CUDA(cudaMemcpy(*p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
        return FL_OK;
    }
};

// Shared memory of k_surface_batch: flux places, barriers + stage records +
// warp partials, the active list, two stages.
static int batch_smem_layout(BatchArgs &a, int kind, int S) {
    auto up = [](int x, int m) { return (x + m - 1) / m * m; };
    const int T = a.tile;
    a.off_bar = T * 3 * 16;
    a.off_list = up(a.off_bar + 64 + (T / 32) * 5 * 4, 128);
    a.off_stage = up(a.off_list + MAX_SCEN * 4 + 16 + S * (int)sizeof(BatchEntry), 128);
    int o = (T + a.h_cap) * 16;
    a.so_ci = o;
    o += T * 16;
    a.so_hz = o;
    if (kind) o += T * 16;
    a.so_wt = o;
    if (kind) o += T * 4;
    a.so_hm = o;
    o += T * 4;
    a.so_en = o;
    o += a.e_cap * 16;
    a.so_hs = o;
    o += a.h_cap * 4;
    a.stage_bytes = up(o, 128);
    return a.off_stage + 2 * a.stage_bytes;
}

static int batch_create_impl(int32_t n, const FlMeshDesc *meshes, const FlForcingDesc *forcings, const FlParams *params,
                             const FlBatchShape *shape, int32_t device, FlBatch *b) {
    if (n < 1 || n > MAX_SCEN) return set_error(FL_E_INVALID, "a batch holds 1..%d scenarios, got %d", MAX_SCEN, n);
    if (!meshes || !forcings || !params) return set_error(FL_E_INVALID, "fl_batch_create needs meshes, forcings and params");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_error(FL_E_NO_DEVICE, "no CUDA device is visible; CPU fallback is disabled");
    if (device < 0 || device >= ndev) return set_error(FL_E_NO_DEVICE, "device %d is not visible (%d devices)", device, ndev);
    b->device = device;
    FB_CUDA(cudaSetDevice(device));
    b->S = n;
    b->tile = shape && shape->tile_cells ? shape->tile_cells : 256;
    if (b->tile != 128 && b->tile != 256) return set_error(FL_E_INVALID, "tile_cells must be 128 or 256");
    b->chunk = shape && shape->chunk_steps ? shape->chunk_steps : 32;
    if (b->chunk < 2 || b->chunk % 2) return set_error(FL_E_INVALID, "chunk_steps must be even and >= 2");
    const int want_ctas = shape ? shape->ctas_per_sm : 0;
    if (want_ctas < 0) return set_error(FL_E_INVALID, "ctas_per_sm must be >= 0");

    bool stage_set = false;
    float stage = 0.0f;
    b->kind = 0;
    for (int32_t s = 0; s < n; ++s) {
        const FlParams &p = params[s];
        if (!(p.cfl > 0.0 && p.cfl <= 1.0) || p.cfl_update_interval_steps < 1 || !(p.max_dt_s > 0.0) ||
            !(p.duration_s > 0.0) || !(p.snapshot_interval_s > 0.0) || p.max_snapshots < 1)
            return set_error(FL_E_INVALID, "scenario %d: invalid solver parameters", s);
        if (p.surface_step_mode != 0)
            return set_error(FL_E_UNSUPPORTED, "scenario %d: the batched ensemble runs the full-SWE surface step only", s);
        if (p.gravity_mps2 != params[0].gravity_mps2 || p.min_depth_m != params[0].min_depth_m ||
            p.cfl != params[0].cfl || p.max_speed_mps != params[0].max_speed_mps)
            return set_error(FL_E_INVALID, "scenario %d: gravity, min depth, cfl and max speed must match the batch", s);
        const FlForcingDesc &f = forcings[s];
        if (f.kind != 0 && f.kind != 1) return set_error(FL_E_INVALID, "scenario %d: forcing kind must be 0 or 1", s);
        if (f.kind == 1 && (!f.rain_multiplier || !f.horton_f0_mps || !f.horton_fc_mps || !f.horton_k_per_s))
            return set_error(FL_E_INVALID, "scenario %d: per-cell forcing needs rain_multiplier and Horton arrays", s);
        if (f.hyetograph_count < 0 || (f.hyetograph_count > 0 && (!f.hyeto_start_s || !f.hyeto_end_s || !f.hyeto_rate_mps)))
            return set_error(FL_E_INVALID, "scenario %d: hyetograph arrays are missing", s);
        if (f.kind == 1) b->kind = 1;
        if (meshes[s].has_stage_boundary) {
            if (stage_set && meshes[s].boundary_stage_m != stage)
                return set_error(FL_E_INVALID, "scenario %d: every stage boundary of a batch must use the same stage", s);
            stage_set = true;
            stage = meshes[s].boundary_stage_m;
        }
    }
    b->params.assign(params, params + n);

    // per-scenario layouts, concatenated tile by tile
    std::vector<float4> cinfo, ent, horton;
    std::vector<int4> tile_info;
    std::vector<int32_t> halo_src, perm, tile_valid;
    std::vector<float> char_len;
    std::vector<float4> st0;
    int32_t e_cap = 0, h_cap = 0;
    b->cell0.resize(n);
    b->cells_s.resize(n);
    b->tile0.resize(n + 1);
    b->area.resize(n);
    int64_t c_off = 0;
    int32_t t_off = 0;
    for (int32_t s = 0; s < n; ++s) {
        HostLayout L;
        L.tile = b->tile;
        int rc = build_mesh_layout(meshes[s], nullptr, L);
        if (rc) return set_error(rc, "scenario %d: %s", s, fl_last_error());
        if (c_off + L.Cp > (int64_t)0x7FFFFFFF) return set_error(FL_E_INVALID, "the batch has too many cells");
        b->cell0[s] = (int32_t)c_off;
        b->cells_s[s] = L.C;
        b->tile0[s] = t_off;
        const int32_t e_off = (int32_t)ent.size(), h_off = (int32_t)halo_src.size();
        for (const int4 &ti : L.tile_info) tile_info.push_back(make_int4(ti.x + e_off, ti.y, ti.z + h_off, ti.w));
        ent.insert(ent.end(), L.ent.begin(), L.ent.end());
        for (int32_t g : L.halo_src) halo_src.push_back((int32_t)(g + c_off));
        cinfo.insert(cinfo.end(), L.cinfo.begin(), L.cinfo.end());
        const int64_t ntile = (int64_t)L.tile_info.size();
        for (int64_t t = 0; t < ntile; ++t) tile_valid.push_back((int32_t)std::min<int64_t>(b->tile, (int64_t)L.C - t * b->tile));
        b->area[s].resize(L.C);
        for (int32_t i = 0; i < L.Cp; ++i) {
            const bool real = i < L.C;
            perm.push_back(real ? L.perm[i] : 0);
            char_len.push_back(real ? L.char_len[i] : 0.0f);
            st0.push_back(make_float4(0.0f, 0.0f, 0.0f, real ? L.bed[i] : 0.0f));
            if (real) b->area[s][i] = L.cinfo[i].x;
            const FlForcingDesc &f = forcings[s];
            if (!real) horton.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
            else if (f.kind == 1) {
                const int32_t r = L.perm[i];
                horton.push_back(make_float4(f.horton_f0_mps[r], f.horton_fc_mps[r], f.horton_k_per_s[r], f.rain_multiplier[r]));
            } else {
                // uniform forcing in the per-cell form: f0 = fc = the capacity, multiplier 1
                horton.push_back(make_float4(f.infiltration_mps, f.infiltration_mps, 0.0f, 1.0f));
            }
        }
        e_cap = std::max(e_cap, L.e_cap);
        h_cap = std::max(h_cap, L.h_cap);
        c_off += L.Cp;
        t_off += (int32_t)ntile;
    }
    b->tile0[n] = t_off;
    b->cells = c_off;
    b->tiles = t_off;
    const size_t Cp = (size_t)c_off;

    // device memory
    float4 *d_cinfo, *d_ent, *d_horton = nullptr;
    int4 *d_tile_info;
    int32_t *d_halo, *d_scen_tile0, *d_scen_cells;
    float *d_char_len, *d_scen_infil, *tile_min, *tile_led;
    int rc;
    if ((rc = b->upload(&d_cinfo, cinfo)) || (rc = b->upload(&d_ent, ent)) || (rc = b->upload(&d_tile_info, tile_info)) ||
        (rc = b->upload(&d_halo, halo_src)) || (rc = b->upload(&d_char_len, char_len)) || (rc = b->upload(&b->perm, perm)) ||
        (rc = b->upload(&b->tile_valid, tile_valid)) || (rc = b->upload(&b->init_state, st0)) ||
        (rc = b->upload(&d_scen_tile0, b->tile0)) || (rc = b->upload(&d_scen_cells, b->cells_s)))
        return rc;
    if (b->kind == 1 && (rc = b->upload(&d_horton, horton))) return rc;
    std::vector<float> infil(n);
    for (int32_t s = 0; s < n; ++s) infil[s] = forcings[s].kind == 0 ? forcings[s].infiltration_mps : 0.0f;
    if ((rc = b->upload(&d_scen_infil, infil))) return rc;
    for (int k = 0; k < 2; ++k)
        if ((rc = b->alloc(&b->state[k], Cp))) return rc;
    FB_CUDA(cudaMemcpy(b->state[0], st0.data(), sizeof(float4) * Cp, cudaMemcpyHostToDevice));
    FB_CUDA(cudaMemcpy(b->state[1], st0.data(), sizeof(float4) * Cp, cudaMemcpyHostToDevice));
    if ((rc = b->alloc(&b->hmax, Cp)) || (rc = b->alloc(&b->wet, Cp)) || (rc = b->alloc(&tile_min, (size_t)b->tiles)) ||
        (rc = b->alloc(&tile_led, (size_t)b->tiles * SURF_TERMS)) || (rc = b->alloc(&b->run, (size_t)n)) ||
        (rc = b->alloc(&b->ctrl, (size_t)n * 2)) || (rc = b->alloc(&b->list, 1)) ||
        (rc = b->alloc(&b->ledger, (size_t)n * SURF_TERMS)))
        return rc;
    FB_CUDA(cudaMemset(tile_led, 0, sizeof(float) * (size_t)b->tiles * SURF_TERMS));
    FB_CUDA(cudaMemset(b->list, 0, sizeof(BatchList)));
    int32_t largest = 1;
    for (int32_t s = 0; s < n; ++s) largest = std::max(largest, b->cells_s[s]);
    if ((rc = b->alloc(&b->stage_f, (size_t)largest))) return rc;
    // snapshots: per scenario max_snapshots rows of its cells
    b->max_snaps = 1;
    b->snap_base_h.resize(n);
    int64_t snap_total = 0;
    for (int32_t s = 0; s < n; ++s) {
        b->max_snaps = std::max(b->max_snaps, params[s].max_snapshots);
        b->snap_base_h[s] = snap_total;
        snap_total += (int64_t)params[s].max_snapshots * b->cells_s[s];
    }
    float *snap_h, *snap_hmax, *snap_hu, *snap_hv;
    double *snap_t;
    int64_t *d_snap_base;
    if ((rc = b->alloc(&snap_h, (size_t)snap_total)) || (rc = b->alloc(&snap_hmax, (size_t)snap_total)) ||
        (rc = b->alloc(&snap_hu, (size_t)snap_total)) || (rc = b->alloc(&snap_hv, (size_t)snap_total)) ||
        (rc = b->alloc(&snap_t, (size_t)n * b->max_snaps)) || (rc = b->upload(&d_snap_base, b->snap_base_h)))
        return rc;
    // hyetographs
    std::vector<HyetoView> hv(n);
    for (int32_t s = 0; s < n; ++s) {
        const int nh = forcings[s].hyetograph_count;
        double *hy = nullptr;
        if ((rc = b->alloc(&hy, 3 * (size_t)(nh > 0 ? nh : 1)))) return rc;
        if (nh > 0) {
            FB_CUDA(cudaMemcpy(hy, forcings[s].hyeto_start_s, sizeof(double) * nh, cudaMemcpyHostToDevice));
            FB_CUDA(cudaMemcpy(hy + nh, forcings[s].hyeto_end_s, sizeof(double) * nh, cudaMemcpyHostToDevice));
            FB_CUDA(cudaMemcpy(hy + 2 * nh, forcings[s].hyeto_rate_mps, sizeof(double) * nh, cudaMemcpyHostToDevice));
        }
        hv[s].start_s = hy;
        hv[s].end_s = hy + nh;
        hv[s].rate = hy + 2 * nh;
        hv[s].n = nh;
    }
    HyetoView *d_hy;
    if ((rc = b->upload(&d_hy, hv))) return rc;
    unsigned int *counter = nullptr;
    if ((rc = b->alloc(&counter, 1))) return rc;
    FB_CUDA(cudaMemset(counter, 0, sizeof(unsigned int)));

    // kernel arguments and launch shape
    BatchArgs &a = b->ba;
    a.cinfo = d_cinfo;
    a.tile_info = d_tile_info;
    a.ent = d_ent;
    a.halo_src = d_halo;
    a.horton = d_horton;
    a.wet = b->wet;
    a.state0 = b->state[0];
    a.state1 = b->state[1];
    a.hmax = b->hmax;
    a.char_len = d_char_len;
    a.list = b->list;
    a.tile_min = tile_min;
    a.tile_led = tile_led;
    a.snap_h = snap_h;
    a.snap_hmax = snap_hmax;
    a.snap_hu = snap_hu;
    a.snap_hv = snap_hv;
    a.snap_base = d_snap_base;
    a.run = b->run;
    a.n_tiles = b->tiles;
    a.tile = b->tile;
    a.e_cap = e_cap;
    a.h_cap = h_cap;
    a.forcing_kind = b->kind;
    a.g = (float)params[0].gravity_mps2;
    a.half_g = (float)(0.5 * params[0].gravity_mps2);
    a.md = (float)params[0].min_depth_m;
    a.vmax = (float)params[0].max_speed_mps;
    a.stage = stage;
    a.cfl = (float)params[0].cfl;
    b->smem = batch_smem_layout(a, b->kind, n);
    int per_sm = 0, sms = 0;
    FB_CUDA(batch_configure(b->kind, b->tile, b->smem, &per_sm));
    FB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    if (per_sm < 1) return set_error(FL_E_UNSUPPORTED, "the batch's largest tile needs %d bytes of shared memory", b->smem);
    const int ctas = want_ctas > 0 ? std::min(want_ctas, per_sm) : per_sm;
    b->grid = std::max(1, std::min(ctas * sms, b->tiles));
    PlanArgs &pa = b->pa;
    pa.run = b->run;
    pa.ctrl = b->ctrl;
    pa.snap_t = snap_t;
    pa.hy = d_hy;
    pa.scen_tile0 = d_scen_tile0;
    pa.scen_cells = d_scen_cells;
    pa.scen_infil = d_scen_infil;
    pa.tile_min = tile_min;
    pa.tile_led = tile_led;
    pa.ledger = b->ledger;
    pa.list = b->list;
    pa.counter = counter;
    pa.n = n;
    pa.max_snaps = b->max_snaps;

    FB_CUDA(cudaMallocHost((void **)&b->poll_h, sizeof(BatchList) * 2));
    FB_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    for (auto &e : b->ev) FB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return FL_OK;
}

static int batch_reset(FlBatch *b, int64_t max_steps, cudaStream_t st) {
    std::vector<RunCtrl> r(b->S);
    for (int32_t s = 0; s < b->S; ++s) {
        const FlParams &p = b->params[s];
        RunCtrl &x = r[s];
        memset(&x, 0, sizeof(x));
        x.t = 0.0;
        x.cached_dt = -1.0;
        x.next_snap_t = 0.0;
        x.final_t = p.duration_s;
        x.stop_t = p.duration_s;
        x.max_dt = p.max_dt_s;
        x.safety = p.cfl_reuse_safety_factor;
        x.snap_interval = p.snapshot_interval_s;
        x.g = p.gravity_mps2;
        x.step = 0;
        x.max_step = max_steps > 0 ? max_steps : std::numeric_limits<int64_t>::max();
        x.parity = 0;
        x.max_snaps = p.max_snapshots;
        x.cfl_interval = p.cfl_update_interval_steps;
        x.finite_interval = p.finite_check_interval_steps;
        x.hyeto_n = 0;
    }
    FB_CUDA(cudaMemcpyAsync(b->run, r.data(), sizeof(RunCtrl) * b->S, cudaMemcpyHostToDevice, st));
    FB_CUDA(cudaMemsetAsync(b->ctrl, 0, sizeof(StepCtrl) * 2 * b->S, st));
    FB_CUDA(cudaMemcpyAsync(b->state[0], b->init_state, sizeof(float4) * (size_t)b->cells, cudaMemcpyDeviceToDevice, st));
    FB_CUDA(cudaMemsetAsync(b->hmax, 0, sizeof(float) * (size_t)b->cells, st));
    FB_CUDA(cudaMemsetAsync(b->wet, 0, sizeof(float) * (size_t)b->cells, st));
    FB_CUDA(cudaMemsetAsync(b->ledger, 0, sizeof(float2) * (size_t)b->S * SURF_TERMS, st));
    return FL_OK;
}

static int batch_capture(FlBatch *b) {
    if (b->graph) return FL_OK;
    cudaGraph_t g = nullptr;
    FB_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < b->chunk && e == cudaSuccess; ++j) {
        e = launch_surface_batch(b->ba, b->kind, b->grid, b->smem, b->cap_stream);
        if (e == cudaSuccess) e = launch_plan_batch(b->pa, j & 1, 0, b->cap_stream);
    }
    cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return set_error(FL_E_CUDA, "batch graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    return FL_OK;
}

extern "C" {

FL_API int fl_batch_create(int32_t n, const FlMeshDesc *meshes, const FlForcingDesc *forcings, const FlParams *params,
                           const FlBatchShape *shape, int32_t device, FlBatch **out) {
    if (!out) return set_error(FL_E_INVALID, "out is NULL");
    *out = nullptr;
    FlBatch *b = new (std::nothrow) FlBatch();
    if (!b) return set_error(FL_E_NOMEM, "out of host memory");
    int rc = batch_create_impl(n, meshes, forcings, params, shape, device, b);
    if (rc != FL_OK) {
        std::string msg = fl_last_error();
        fl_batch_destroy(b);
        set_error(rc, "%s", msg.c_str());
        return rc;
    }
    *out = b;
    return FL_OK;
}

FL_API void fl_batch_destroy(FlBatch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto &e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (void *p : b->allocs) cudaFree(p);
    if (b->poll_h) cudaFreeHost(b->poll_h);
    delete b;
}

FL_API int fl_batch_set_state(FlBatch *b, int32_t scen, const float *h, const float *hu, const float *hv, int32_t mem,
                              void *stream) {
    if (!b || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch or scenario");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    const int32_t C = b->cells_s[scen];
    std::vector<float4> v(C);
    FB_CUDA(cudaMemcpy(v.data(), b->init_state + b->cell0[scen], sizeof(float4) * C, cudaMemcpyDeviceToHost));
    std::vector<int32_t> perm(C);
    FB_CUDA(cudaMemcpy(perm.data(), b->perm + b->cell0[scen], sizeof(int32_t) * C, cudaMemcpyDeviceToHost));
    std::vector<float> src[3];
    const float *in[3] = {h, hu, hv};
    for (int k = 0; k < 3; ++k) {
        if (!in[k]) continue;
        src[k].resize(C);
        if (mem == FL_MEM_DEVICE) FB_CUDA(cudaMemcpy(src[k].data(), in[k], sizeof(float) * C, cudaMemcpyDeviceToHost));
        else memcpy(src[k].data(), in[k], sizeof(float) * C);
    }
    for (int32_t i = 0; i < C; ++i) {
        const int32_t r = perm[i];
        if (h) v[i].x = src[0][r];
        if (hu) v[i].y = src[1][r];
        if (hv) v[i].z = src[2][r];
    }
    FB_CUDA(cudaMemcpyAsync(b->init_state + b->cell0[scen], v.data(), sizeof(float4) * C, cudaMemcpyHostToDevice, st));
    FB_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_batch_run(FlBatch *b, int64_t max_steps, void *stream) {
    if (!b) return set_error(FL_E_INVALID, "batch is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    int rc = batch_reset(b, max_steps, st);
    if (rc) return rc;
    // CFL minima of the initial states, then plan step 0 of every scenario
    FB_CUDA(launch_cfl_batch(b->state[0], b->ba.char_len, b->tile_valid, b->ba.tile_min, b->tiles, b->tile, b->ba.cfl,
                             b->ba.g, b->ba.md, st));
    FB_CUDA(launch_plan_batch(b->pa, 1, 1, st));
    add_launches(2);
    if ((rc = batch_capture(b))) return rc;
    int64_t launched = 0;
    while (true) {
        FB_CUDA(cudaGraphLaunch(b->graph, st));
        add_launches(2 * (int64_t)b->chunk);
        FB_CUDA(cudaMemcpyAsync(&b->poll_h[launched & 1], b->list, 16, cudaMemcpyDeviceToHost, st));
        FB_CUDA(cudaEventRecord(b->ev[launched & 1], st));
        ++launched;
        if (launched >= 2) {
            FB_CUDA(cudaEventSynchronize(b->ev[launched & 1]));
            if (b->poll_h[launched & 1].n == 0) break;
        }
    }
    FB_CUDA(cudaStreamSynchronize(st));
    std::vector<RunCtrl> r(b->S);
    FB_CUDA(cudaMemcpy(r.data(), b->run, sizeof(RunCtrl) * b->S, cudaMemcpyDeviceToHost));
    for (int32_t s = 0; s < b->S; ++s) {
        if (r[s].error == FL_E_NONFINITE)
            return set_error(FL_E_NONFINITE, "scenario %d: non-finite depth detected at step %lld", s, (long long)r[s].error_step);
        if (r[s].error) return set_error(r[s].error, "scenario %d: device error %d at step %lld", s, r[s].error, (long long)r[s].error_step);
    }
    return FL_OK;
}

FL_API int fl_batch_progress(FlBatch *b, int32_t scen, FlProgress *out, void *stream) {
    if (!b || !out || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch, scenario or output");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    RunCtrl r;
    FB_CUDA(cudaMemcpyAsync(&r, b->run + scen, sizeof(RunCtrl), cudaMemcpyDeviceToHost, st));
    FB_CUDA(cudaStreamSynchronize(st));
    out->t_s = r.t;
    out->step_count = r.step;
    out->cfl_eval_count = r.cfl_evals;
    out->cfl_reused_count = r.cfl_reused;
    out->snapshot_count = r.snap_count;
    out->error = r.error;
    out->error_step = r.error_step;
    out->last_dt_s = r.last_dt;
    return FL_OK;
}

// Scenario rows (renumbered order) -> reference order, written to dst.
static int scen_to_reference(FlBatch *b, int32_t scen, const float *src, float *dst, int32_t mem, cudaStream_t st) {
    const int32_t C = b->cells_s[scen];
    FB_CUDA(launch_permute_f32(src, b->stage_f, b->perm + b->cell0[scen], C, 1, st));
    FB_CUDA(cudaMemcpyAsync(dst, b->stage_f, sizeof(float) * C,
                            mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    FB_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_batch_get_state(FlBatch *b, int32_t scen, float *h, float *hu, float *hv, int32_t mem, void *stream) {
    if (!b || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch or scenario");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    RunCtrl r;
    FB_CUDA(cudaMemcpy(&r, b->run + scen, sizeof(RunCtrl), cudaMemcpyDeviceToHost));
    const int32_t C = b->cells_s[scen];
    std::vector<float4> v(C);
    FB_CUDA(cudaMemcpy(v.data(), b->state[r.parity] + b->cell0[scen], sizeof(float4) * C, cudaMemcpyDeviceToHost));
    std::vector<int32_t> perm(C);
    FB_CUDA(cudaMemcpy(perm.data(), b->perm + b->cell0[scen], sizeof(int32_t) * C, cudaMemcpyDeviceToHost));
    std::vector<float> o[3];
    for (int k = 0; k < 3; ++k) o[k].resize(C);
    for (int32_t i = 0; i < C; ++i) {
        o[0][perm[i]] = v[i].x;
        o[1][perm[i]] = v[i].y;
        o[2][perm[i]] = v[i].z;
    }
    float *dst[3] = {h, hu, hv};
    for (int k = 0; k < 3; ++k) {
        if (!dst[k]) continue;
        if (mem == FL_MEM_DEVICE) FB_CUDA(cudaMemcpyAsync(dst[k], o[k].data(), sizeof(float) * C, cudaMemcpyHostToDevice, st));
        else memcpy(dst[k], o[k].data(), sizeof(float) * C);
    }
    FB_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_batch_get_snapshots(FlBatch *b, int32_t scen, int32_t first, int32_t count, double *times_s, float *h,
                                  float *hmax, int32_t mem, void *stream) {
    if (!b || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch or scenario");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    RunCtrl r;
    FB_CUDA(cudaMemcpy(&r, b->run + scen, sizeof(RunCtrl), cudaMemcpyDeviceToHost));
    if (first < 0 || count < 0 || first + count > r.snap_count)
        return set_error(FL_E_INVALID, "snapshots [%d, %d) requested, %d available", first, first + count, r.snap_count);
    if (times_s && count > 0)
        FB_CUDA(cudaMemcpy(times_s, b->pa.snap_t + (size_t)scen * b->max_snaps + first, sizeof(double) * count,
                           cudaMemcpyDeviceToHost));
    const size_t C = (size_t)b->cells_s[scen];
    for (int32_t i = 0; i < count; ++i) {
        const size_t o = (size_t)b->snap_base_h[scen] + (size_t)(first + i) * C;
        int rc;
        if (h && (rc = scen_to_reference(b, scen, b->ba.snap_h + o, h + (size_t)i * C, mem, st))) return rc;
        if (hmax && (rc = scen_to_reference(b, scen, b->ba.snap_hmax + o, hmax + (size_t)i * C, mem, st))) return rc;
    }
    add_launches((int64_t)count * ((h ? 1 : 0) + (hmax ? 1 : 0)));
    return FL_OK;
}

FL_API int fl_batch_get_snapshot_momentum(FlBatch *b, int32_t scen, int32_t first, int32_t count, float *hu,
                                          float *hv, int32_t mem, void *stream) {
    if (!b || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch or scenario");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    RunCtrl r;
    FB_CUDA(cudaMemcpy(&r, b->run + scen, sizeof(RunCtrl), cudaMemcpyDeviceToHost));
    if (first < 0 || count < 0 || first + count > r.snap_count)
        return set_error(FL_E_INVALID, "snapshots [%d, %d) requested, %d available", first, first + count, r.snap_count);
    const size_t C = (size_t)b->cells_s[scen];
    for (int32_t i = 0; i < count; ++i) {
        const size_t o = (size_t)b->snap_base_h[scen] + (size_t)(first + i) * C;
        int rc;
        if (hu && (rc = scen_to_reference(b, scen, b->ba.snap_hu + o, hu + (size_t)i * C, mem, st))) return rc;
        if (hv && (rc = scen_to_reference(b, scen, b->ba.snap_hv + o, hv + (size_t)i * C, mem, st))) return rc;
    }
    add_launches((int64_t)count * ((hu ? 1 : 0) + (hv ? 1 : 0)));
    return FL_OK;
}

FL_API int fl_batch_read_ledger(FlBatch *b, int32_t scen, double *out, int32_t n, void *stream) {
    if (!b || !out || scen < 0 || scen >= b->S) return set_error(FL_E_INVALID, "bad batch, scenario or output");
    cudaStream_t st = (cudaStream_t)stream;
    FB_CUDA(cudaSetDevice(b->device));
    double all[FL_LEDGER_COUNT] = {0};
    float2 v[SURF_TERMS];
    FB_CUDA(cudaMemcpyAsync(v, b->ledger + (size_t)scen * SURF_TERMS, sizeof(v), cudaMemcpyDeviceToHost, st));
    FB_CUDA(cudaStreamSynchronize(st));
    for (int j = 0; j < SURF_TERMS; ++j) all[FL_LEDGER_RAINFALL + j] = (double)v[j].x + (double)v[j].y;
    RunCtrl r;
    FB_CUDA(cudaMemcpy(&r, b->run + scen, sizeof(RunCtrl), cudaMemcpyDeviceToHost));
    const int32_t C = b->cells_s[scen];
    std::vector<float4> s(C);
    FB_CUDA(cudaMemcpy(s.data(), b->state[r.parity] + b->cell0[scen], sizeof(float4) * C, cudaMemcpyDeviceToHost));
    double vol = 0.0;
    for (int32_t i = 0; i < C; ++i) vol += (double)(s[i].x * b->area[scen][i]);
    all[FL_LEDGER_SURFACE_VOLUME] = vol;
    for (int i = 0; i < n && i < FL_LEDGER_COUNT; ++i) out[i] = all[i];
    return FL_OK;
}

FL_API int fl_batch_info(FlBatch *b, FlBatchShape *shape, int64_t *cells, int64_t *tiles, int32_t *grid) {
    if (!b) return set_error(FL_E_INVALID, "batch is NULL");
    if (shape) {
        shape->tile_cells = b->tile;
        shape->ctas_per_sm = 0;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) == cudaSuccess && sms > 0)
            shape->ctas_per_sm = (b->grid + sms - 1) / sms;
        shape->chunk_steps = b->chunk;
        shape->reserved = b->smem;
    }
    if (cells) *cells = b->cells;
    if (tiles) *tiles = b->tiles;
    if (grid) *grid = b->grid;
    return FL_OK;
}

}  // extern "C"
