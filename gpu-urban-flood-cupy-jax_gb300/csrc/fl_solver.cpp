// Solver runtime behind the C ABI (include/floodgb.h): device memory, the
// device-resident adaptive step loop as captured CUDA-graph chunks, state and
// snapshot transfer, the ledger, and error reporting.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/floodgb.h"
#include "fl_internal.h"

namespace fl {

// ---------------------------------------------------------------- errors
static thread_local std::string g_error;
static std::atomic<int64_t> g_launches{0};

int set_error(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

void add_launches(int64_t n) { g_launches += n; }

int build_mesh_layout(const FlMeshDesc &m, const FlDrainDesc *d, HostLayout &L);
int build_drain_layout(const FlMeshDesc &m, const FlDrainDesc &d, HostLayout &L);
int surface_smem_layout(SurfArgs &a, int kind);

// kernel launchers (fl_surface.cu / fl_drainage.cu)
cudaError_t launch_surface(const SurfArgs &a, int kind, int slot, int plan_next, int grid, int smem_bytes,
                           cudaStream_t stream);
cudaError_t plan_surface_launch(SurfArgs &a, int kind, int device, int *grid, int *smem_bytes);
int surface_warps(int grid);
cudaError_t launch_dt(const DtArgs &a, int blocks, int slot, int plan, cudaStream_t stream);
cudaError_t launch_replan(RunCtrl *run, double *snap_t, HyetoView hy, StepCtrl *ctrl, int slot, cudaStream_t stream);
cudaError_t launch_finite(const float4 *s0, const float4 *s1, RunCtrl *run, int32_t C, cudaStream_t stream);
cudaError_t launch_load_state(float4 *state, const float *h, const float *hu, const float *hv, const float *bed,
                              const int32_t *perm, int32_t C, int mask, cudaStream_t stream);
cudaError_t launch_store_state(const float4 *state, float *h, float *hu, float *hv, const int32_t *perm, int32_t C,
                               cudaStream_t stream);
cudaError_t launch_permute_f32(const float *src, float *dst, const int32_t *perm, int32_t C, int to_reference,
                               cudaStream_t stream);
cudaError_t launch_f64_to_ff(const double *src, float2 *dst, int32_t n, cudaStream_t stream);
cudaError_t launch_ff_to_f64(const float2 *src, double *dst, int32_t n, cudaStream_t stream);
cudaError_t launch_f64_to_f32_perm(const double *src, float *dst, const int32_t *perm, int32_t n, cudaStream_t stream);
cudaError_t launch_f32_to_f64_perm(const float *src, double *dst, const int32_t *perm, int32_t n, cudaStream_t stream);
cudaError_t launch_volumes(const float4 *s0, const float4 *s1, const float4 *g1, const float2 *V, RunCtrl *run,
                           int32_t C, int32_t N, double *out2, cudaStream_t stream);
cudaError_t launch_nodes(const NodeArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_links(const LinkArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_donor(const DonorArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_network(const NetArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_recharge(const RechargeArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_inflow(const InflowArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_surcharge(const SurchargeArgs &a, int slot, cudaStream_t stream);
cudaError_t launch_li(const LiArgs &a, int kind, int slot, int plan_next, int sms, cudaStream_t stream);
int li_cell_blocks(int32_t C);
int node_blocks(int32_t N);
int network_blocks(int32_t G);
cudaError_t launch_f64_to_ff_perm(const double *src, float2 *dst, const int32_t *perm, int32_t n, cudaStream_t stream);
cudaError_t launch_ff_to_f64_perm(const float2 *src, double *dst, const int32_t *perm, int32_t n, cudaStream_t stream);

}  // namespace fl

using namespace fl;

#define FL_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess) return set_error(FL_E_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

struct FlSolver {
    int device = 0;
    int32_t C = 0, N = 0, NL = 0, I = 0, K = 0, G = 0;
    int kind = 0;
    FlParams params{};
    int32_t Cp = 0;  // cells padded to whole tiles
    int dt_blocks = 0, surf_grid = 0, surf_smem = 0, d1_blocks = 0, d2_blocks = 0;
    int chunk = 32;
    std::vector<void *> allocs;
    // device
    int32_t *perm = nullptr;
    std::vector<int32_t> perm_h;
    float *bed = nullptr;
    float4 *state[2] = {nullptr, nullptr};
    float2 *Va = nullptr, *Vb = nullptr;
    float *Q[2] = {nullptr, nullptr};
    float *wet = nullptr;
    StepCtrl *ctrl = nullptr;
    RunCtrl *run = nullptr;
    double *snap_t = nullptr;
    float *snap_h = nullptr, *snap_hu = nullptr, *snap_hv = nullptr, *snap_v = nullptr;
    float2 *led_s = nullptr, *led_1 = nullptr, *led_2 = nullptr;  // float-float running sums
    size_t n_led_s = 0, n_led_1 = 0, n_led_2 = 0;
    double *dt_out = nullptr, *vol_out = nullptr;
    float *stage_f[3] = {nullptr, nullptr, nullptr};
    double *stage_d = nullptr;
    SurfArgs sa{};
    DtArgs da{};
    NodeArgs nd{};
    LinkArgs lk{};
    DonorArgs dn{};
    NetArgs nw{};
    int32_t *node_perm = nullptr;  // node_perm[new] = reference node
    int32_t *link_perm = nullptr;  // link_perm[new] = reference link
    float *stage_n = nullptr;      // [N] node-order staging
    char *drain_base = nullptr;    // the drainage arena (L2 access-policy window)
    size_t drain_bytes = 0;
    bool l2_persist = false;
    HyetoView hy{};
    // host
    RunCtrl *run_h = nullptr;   // pinned mirror
    RunCtrl *poll_h = nullptr;  // pinned, 2 slots
    int slot = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // cell info: the host copy keeps the flag bits that inflow / recharge set
    std::vector<float4> cinfo_h;
    float4 *cinfo_d = nullptr;
    void *ext_mem = nullptr;  // external inflow tables (one allocation)
    void *rch_mem = nullptr;  // recharge tables (one allocation)
    InflowArgs ext{};
    LiArgs li{};
    bool li_mode = false;     // surface_step_mode = local_inertial
    int sms = 1;
    SurchargeArgs sur{};
    RechargeArgs rch{};
    int32_t R = 0;            // recharge rows
    bool has_drain() const { return N > 0; }
    bool has_inflow() const { return ext.U > 0; }
    bool has_table() const { return sur.U > 0; }
    bool has_recharge() const { return rch.U > 0; }
    int launches_per_step() const {
        return (li_mode ? 2 : 1) * members + (has_drain() ? 4 : 0) + (has_table() ? 1 : 0) + (has_inflow() ? 1 : 0) +
               (has_recharge() ? 1 : 0);
    }

    // Ensemble members (fl_create_members; 1 for fl_create): every per-member
    // array is allocated member after member, starting at the pointers in
    // `mb`; the fields above (state, wet, ctrl, run, run_h, snapshots,
    // ledgers, dt_out, vol_out, Va, Vb, Q, hy) address the selected member.
    int32_t members = 1, cur = 0;
    struct MemberBase {
        float4 *state[2] = {nullptr, nullptr};
        float *wet = nullptr;
        StepCtrl *ctrl = nullptr;
        RunCtrl *run = nullptr, *run_h = nullptr;
        double *snap_t = nullptr;
        float *snap_h = nullptr, *snap_hu = nullptr, *snap_hv = nullptr, *snap_v = nullptr;
        float2 *led_s = nullptr, *led_1 = nullptr, *led_2 = nullptr;
        double *dt_out = nullptr, *vol_out = nullptr;
        float2 *Va = nullptr, *Vb = nullptr;
        float *Q[2] = {nullptr, nullptr};
    } mb;
    std::vector<HyetoView> hys;  // [members]
    size_t snap_stride_h() const { return (size_t)params.max_snapshots * (size_t)C; }
    size_t snap_stride_v() const { return (size_t)params.max_snapshots * (size_t)(N > 0 ? N : 1); }
    void select(int32_t m) {
        cur = m;
        for (int b = 0; b < 2; ++b) {
            state[b] = mb.state[b] + (size_t)m * Cp;
            Q[b] = mb.Q[b] ? mb.Q[b] + (size_t)m * NL : nullptr;
        }
        wet = mb.wet + (size_t)m * Cp;
        ctrl = mb.ctrl + 2 * (size_t)m;
        run = mb.run + m;
        run_h = mb.run_h + m;
        snap_t = mb.snap_t + (size_t)m * params.max_snapshots;
        snap_h = mb.snap_h + m * snap_stride_h();
        snap_hu = mb.snap_hu + m * snap_stride_h();
        snap_hv = mb.snap_hv + m * snap_stride_h();
        snap_v = mb.snap_v + m * snap_stride_v();
        led_s = mb.led_s + (size_t)m * n_led_s;
        led_1 = mb.led_1 ? mb.led_1 + (size_t)m * n_led_1 : nullptr;
        led_2 = mb.led_2 ? mb.led_2 + (size_t)m * n_led_2 : nullptr;
        dt_out = mb.dt_out + m;
        vol_out = mb.vol_out + 2 * (size_t)VOL_BLOCKS * (size_t)m;
        Va = mb.Va ? mb.Va + (size_t)m * N : nullptr;
        Vb = mb.Vb ? mb.Vb + (size_t)m * N : nullptr;
        hy = hys[m];
    }

    // Drainage tables live in one arena so one L2 access-policy window can
    // keep them resident across the surface kernel's stream of cell data.
    char *arena = nullptr;
    size_t arena_size = 0, arena_used = 0;

    template <class T>
    int alloc(T **p, size_t count) {
        if (count == 0) count = 1;
        const size_t bytes = sizeof(T) * count;
        if (arena) {
            const size_t at = (arena_used + 255) & ~(size_t)255;
            if (at + bytes > arena_size) return set_error(FL_E_NOMEM, "internal: drainage arena too small");
            *p = (T *)(arena + at);
            arena_used = at + bytes;
            return FL_OK;
        }
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes);
        if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        allocs.push_back(q);
        *p = (T *)q;
        return FL_OK;
    }
    template <class T>
    int upload(T **p, const std::vector<T> &v) {
        int rc = alloc(p, v.size());
        if (rc) return rc;
        if (!v.empty()) FL_CUDA(cudaMemcpy(*p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
        return FL_OK;
    }
};

static int sync_run(FlSolver *s, cudaStream_t st) {
    FL_CUDA(cudaMemcpyAsync(s->run_h, s->run, sizeof(RunCtrl), cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

static int push_run(FlSolver *s, cudaStream_t st) {
    FL_CUDA(cudaMemcpyAsync(s->run, s->run_h, sizeof(RunCtrl), cudaMemcpyHostToDevice, st));
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

// The surface / CFL kernel arguments of member m: the solver's arguments
// (the shared tables and settings) with that member's arrays.
static SurfArgs surf_args(const FlSolver *s, int m) {
    SurfArgs a = s->sa;
    a.state0 = s->mb.state[0] + (size_t)m * s->Cp;
    a.state1 = s->mb.state[1] + (size_t)m * s->Cp;
    a.wet = s->mb.wet + (size_t)m * s->Cp;
    a.ctrl = s->mb.ctrl + 2 * (size_t)m;
    a.run = s->mb.run + m;
    a.hy = s->hys[m];
    a.ledger = s->mb.led_s + (size_t)m * s->n_led_s;
    a.snap_h = s->mb.snap_h + m * s->snap_stride_h();
    a.snap_hu = s->mb.snap_hu + m * s->snap_stride_h();
    a.snap_hv = s->mb.snap_hv + m * s->snap_stride_h();
    a.snap_t = s->mb.snap_t + (size_t)m * s->params.max_snapshots;
    return a;
}

static DtArgs dt_args(const FlSolver *s, int m) {
    DtArgs d = s->da;
    d.state0 = s->mb.state[0] + (size_t)m * s->Cp;
    d.state1 = s->mb.state[1] + (size_t)m * s->Cp;
    d.ctrl = s->mb.ctrl + 2 * (size_t)m;
    d.run = s->mb.run + m;
    d.hy = s->hys[m];
    d.snap_t = s->mb.snap_t + (size_t)m * s->params.max_snapshots;
    return d;
}

// One step: [CFL reduction + plan] surface [inlets network], the CFL and
// surface launches once per member, each drainage kernel once for all
// members.
static int launch_step(FlSolver *s, int slot, bool eval, bool plan_next, cudaStream_t st) {
    if (eval) {
        for (int m = 0; m < s->members; ++m) FL_CUDA(launch_dt(dt_args(s, m), s->dt_blocks, slot, 1, st));
        g_launches += s->members;
    }
    if (s->has_inflow()) {
        FL_CUDA(launch_inflow(s->ext, slot, st));
        g_launches++;
    }
    if (s->li_mode) {
        FL_CUDA(launch_li(s->li, s->kind, slot, plan_next ? 1 : 0, s->sms, st));
        g_launches += 2;
    } else {
        for (int m = 0; m < s->members; ++m)
            FL_CUDA(launch_surface(surf_args(s, m), s->kind, slot, plan_next ? 1 : 0, s->surf_grid, s->surf_smem, st));
        g_launches += s->members;
    }
    if (s->has_drain()) {
        FL_CUDA(launch_nodes(s->nd, slot, st));
        FL_CUDA(launch_links(s->lk, slot, st));
        FL_CUDA(launch_donor(s->dn, slot, st));
        FL_CUDA(launch_network(s->nw, slot, st));
        g_launches += 4;
    }
    if (s->has_table()) {
        FL_CUDA(launch_surcharge(s->sur, slot, st));
        g_launches++;
    }
    if (s->has_recharge()) {
        FL_CUDA(launch_recharge(s->rch, slot, st));
        g_launches++;
    }
    return FL_OK;
}

// Keep the drainage tables in L2: a persisting set-aside for this context
// (released with it) and an access-policy window over the drainage arena on
// every kernel of the step graph.  Best effort: without it the loop is only
// slower.
static void setup_l2_persistence(FlSolver *s) {
    if (!s->drain_base || !s->drain_bytes) return;
    int max_persist = 0, max_window = 0;
    if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, s->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, s->device) != cudaSuccess ||
        max_persist <= 0 || max_window <= 0) {
        cudaGetLastError();
        return;
    }
    const size_t want = std::min(s->drain_bytes, (size_t)std::min(max_persist, max_window));
    size_t cur = 0;
    cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
    if (cur < want && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    s->l2_persist = true;
}

static void set_drain_window(FlSolver *s, cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return;
    }
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    int max_window = 0;
    cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, s->device);
    size_t persist = 0;
    cudaDeviceGetLimit(&persist, cudaLimitPersistingL2CacheSize);
    cudaKernelNodeAttrValue v = {};
    v.accessPolicyWindow.base_ptr = s->drain_base;
    v.accessPolicyWindow.num_bytes = std::min(s->drain_bytes, (size_t)max_window);
    v.accessPolicyWindow.hitRatio = std::min(1.0f, (float)persist / (float)std::max<size_t>(v.accessPolicyWindow.num_bytes, 1));
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
            cudaGraphKernelNodeSetAttribute(nd, cudaKernelNodeAttributeAccessPolicyWindow, &v);
    }
    cudaGetLastError();
}

static int capture_graph(FlSolver *s) {
    if (s->graph) return FL_OK;
    cudaGraph_t g = nullptr;
    FL_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int interval = s->params.cfl_update_interval_steps;
    int rc = FL_OK;
    for (int j = 0; j < s->chunk && rc == FL_OK; ++j) {
        const bool eval = (j % interval) == 0;
        const bool next_eval = ((j + 1) % interval) == 0;
        rc = launch_step(s, j & 1, eval, !next_eval, s->cap_stream);
    }
    cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
    if (rc != FL_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    if (s->l2_persist) set_drain_window(s, g);
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    // the launches above were captured, not executed
    g_launches -= (int64_t)s->chunk * s->launches_per_step() + (int64_t)s->members * ((s->chunk + interval - 1) / interval);
    return FL_OK;
}

static int error_code_message(FlSolver *s) {
    const RunCtrl &r = *s->run_h;
    if (r.error == FL_E_NONFINITE)
        return set_error(FL_E_NONFINITE,
                         "Non-finite depth detected at step %lld (t=%.1f min). Lower solver.cfl_update_interval_steps "
                         "or solver.cfl_reuse_safety_factor.",
                         (long long)r.error_step, r.t / 60.0);
    if (r.error == FL_E_SNAPSHOTS) return set_error(FL_E_SNAPSHOTS, "more than %d snapshots requested", r.max_snaps);
    if (r.error == FL_E_INVALID) return set_error(FL_E_INVALID, "No finite cells are available for timestep calculation.");
    if (r.error == FL_E_TIMEOUT)
        return set_error(FL_E_TIMEOUT,
                         "a tile copy of the surface kernel did not complete within its time limit at step %lld",
                         (long long)r.error_step);
    if (r.error) return set_error(r.error, "device error %d at step %lld", r.error, (long long)r.error_step);
    return FL_OK;
}

extern "C" {

FL_API int fl_abi_version(void) { return FLOODGB_ABI_VERSION; }

FL_API const char *fl_last_error(void) { return g_error.c_str(); }

FL_API int64_t fl_launch_count(void) { return g_launches.load(); }

FL_API int fl_device_count(int32_t *count) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0;
    if (count) *count = n;
    return FL_OK;
}

FL_API int fl_plan_check(const FlMeshDesc *mesh, const FlDrainDesc *drain, int64_t *stats, int32_t *perm_out) {
    if (!mesh) return set_error(FL_E_INVALID, "mesh descriptor is NULL");
    HostLayout L;
    int rc = build_mesh_layout(*mesh, drain, L);
    if (rc) return rc;
    if (drain) {
        rc = build_drain_layout(*mesh, *drain, L);
        if (rc) return rc;
    }
    if (stats) {
        stats[0] = L.C;
        stats[1] = L.E;
        stats[2] = L.slots_used;
        stats[3] = L.K;
        stats[4] = L.N;
        stats[5] = L.L;
        stats[6] = L.G;
        stats[7] = L.max_inlets_per_cell;
    }
    if (perm_out) memcpy(perm_out, L.perm.data(), sizeof(int32_t) * L.perm.size());
    return FL_OK;
}

FL_API int fl_plan_tiles(const FlMeshDesc *mesh, int64_t *tiles) {
    if (!mesh || !tiles) return set_error(FL_E_INVALID, "mesh descriptor or output is NULL");
    HostLayout L;
    int rc = build_mesh_layout(*mesh, nullptr, L);
    if (rc) return rc;
    int64_t halo = 0;
    for (const int4 &t : L.tile_info) halo += t.w;
    SurfArgs a{};
    a.e_cap = L.e_cap;
    a.h_cap = L.h_cap;
    tiles[0] = (int64_t)L.tile_info.size();
    tiles[1] = (int64_t)L.ent.size();
    tiles[2] = halo;
    tiles[3] = L.e_cap;
    tiles[4] = L.h_cap;
    tiles[5] = surface_smem_layout(a, 1);
    return FL_OK;
}

FL_API void fl_destroy(FlSolver *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    for (auto &e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    if (s->l2_persist) cudaCtxResetPersistingL2Cache();
    for (void *p : s->allocs) cudaFree(p);
    if (s->ext_mem) cudaFree(s->ext_mem);
    if (s->rch_mem) cudaFree(s->rch_mem);
    // the pinned run records start at member 0's (run_h addresses the selected member)
    RunCtrl *run_h = s->mb.run_h ? s->mb.run_h : s->run_h;
    if (run_h) cudaFreeHost(run_h);
    if (s->poll_h) cudaFreeHost(s->poll_h);
    delete s;
}

// forcings: M entries (the members' rainfall); the per-cell fields come from
// forcings[0].
static int create_impl(const FlMeshDesc *mesh, const FlDrainDesc *drain, const FlForcingDesc *forcings, int32_t M,
                       const FlParams *params, int32_t device, FlSolver *s) {
    const FlForcingDesc *forcing = forcings;
    if (!mesh || !forcing || !params) return set_error(FL_E_INVALID, "fl_create needs mesh, forcing and params");
    if (M < 1 || M > 1024) return set_error(FL_E_INVALID, "members must be in [1, 1024], got %d", M);
    s->members = M;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_error(FL_E_NO_DEVICE, "no CUDA device is visible; CPU fallback is disabled");
    if (device < 0 || device >= ndev) return set_error(FL_E_NO_DEVICE, "device %d is not visible (%d devices)", device, ndev);
    const FlParams &p = *params;
    if (!(p.cfl > 0.0 && p.cfl <= 1.0)) return set_error(FL_E_INVALID, "solver.cfl must be in (0, 1]");
    if (p.cfl_update_interval_steps < 1) return set_error(FL_E_INVALID, "cfl_update_interval_steps must be >= 1");
    if (!(p.max_dt_s > 0.0)) return set_error(FL_E_INVALID, "max_dt_s must be positive");
    if (!(p.duration_s > 0.0)) return set_error(FL_E_INVALID, "Simulation duration must be positive");
    if (!(p.snapshot_interval_s > 0.0)) return set_error(FL_E_INVALID, "snapshot_interval_s must be positive");
    if (p.max_snapshots < 1) return set_error(FL_E_INVALID, "max_snapshots must be >= 1");
    if (forcing->kind != 0 && forcing->kind != 1) return set_error(FL_E_INVALID, "forcing kind must be 0 or 1");
    if (forcing->kind == 1 && (!forcing->rain_multiplier || !forcing->horton_f0_mps || !forcing->horton_fc_mps ||
                               !forcing->horton_k_per_s))
        return set_error(FL_E_INVALID, "per-cell forcing needs rain_multiplier and Horton f0/fc/k arrays");
    for (int32_t m = 0; m < M; ++m) {
        const FlForcingDesc &f = forcings[m];
        if (f.hyetograph_count < 0 || (f.hyetograph_count > 0 && (!f.hyeto_start_s || !f.hyeto_end_s || !f.hyeto_rate_mps)))
            return set_error(FL_E_INVALID, "hyetograph arrays of member %d are missing", m);
    }
    if (M > 1 && p.surface_step_mode != 0)
        return set_error(FL_E_UNSUPPORTED, "ensemble members run the full_swe surface step only");
    if (M > 1 && drain && drain->surcharge_entry_count > 0)
        return set_error(FL_E_UNSUPPORTED, "ensemble members do not support the weighted surcharge table");
    s->device = device;
    FL_CUDA(cudaSetDevice(device));
    s->params = p;
    s->kind = forcing->kind;

    HostLayout L;
    int rc = build_mesh_layout(*mesh, drain, L);
    if (rc) return rc;
    const bool with_drain = drain && drain->node_count > 0;
    if (with_drain) {
        rc = build_drain_layout(*mesh, *drain, L);  // also flags the surcharge-table cells in cinfo
        if (rc) return rc;
    }
    s->C = L.C;
    s->perm_h = L.perm;
    s->N = L.N;
    s->NL = L.L;
    s->I = L.I;
    s->K = L.K;
    s->G = L.G;
    s->Cp = L.Cp;
    const int32_t C = s->C, Cp = s->Cp;

    // static surface layout (per-cell arrays padded to whole tiles)
    float4 *cinfo, *ent;
    int4 *tile_info;
    int32_t *halo_src;
    float *char_len;
    if ((rc = s->upload(&cinfo, L.cinfo)) || (rc = s->upload(&tile_info, L.tile_info)) ||
        (rc = s->upload(&ent, L.ent)) || (rc = s->upload(&halo_src, L.halo_src)) ||
        (rc = s->upload(&char_len, L.char_len)) || (rc = s->upload(&s->bed, L.bed)) ||
        (rc = s->upload(&s->perm, L.perm)))
        return rc;
    float4 *horton = nullptr;
    if (s->kind == 1) {
        std::vector<float4> hz(Cp, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        for (int32_t i = 0; i < C; ++i) {
            const int32_t r = L.perm[i];
            hz[i] = make_float4(forcing->horton_f0_mps[r], forcing->horton_fc_mps[r], forcing->horton_k_per_s[r],
                                forcing->rain_multiplier[r]);
        }
        if ((rc = s->upload(&horton, hz))) return rc;
    }
    // per-member arrays (member after member)
    const size_t Mz = (size_t)M;
    if ((rc = s->alloc(&s->wet, Mz * Cp))) return rc;
    FL_CUDA(cudaMemset(s->wet, 0, sizeof(float) * Mz * Cp));
    for (int b = 0; b < 2; ++b) {
        if ((rc = s->alloc(&s->state[b], Mz * Cp))) return rc;
    }
    {
        std::vector<float4> st0(Cp, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        for (int32_t i = 0; i < C; ++i) st0[i] = make_float4(0.0f, 0.0f, 0.0f, L.bed[i]);
        for (size_t m = 0; m < Mz; ++m)
            for (int b = 0; b < 2; ++b)
                FL_CUDA(cudaMemcpy(s->state[b] + m * Cp, st0.data(), sizeof(float4) * Cp, cudaMemcpyHostToDevice));
    }
    if ((rc = s->alloc(&s->ctrl, 2 * Mz)) || (rc = s->alloc(&s->run, Mz)) ||
        (rc = s->alloc(&s->snap_t, Mz * p.max_snapshots)))
        return rc;
    FL_CUDA(cudaMemset(s->ctrl, 0, sizeof(StepCtrl) * 2 * Mz));
    const size_t snap_cells = (size_t)p.max_snapshots * (size_t)C;
    const size_t snap_nodes = (size_t)p.max_snapshots * (s->N > 0 ? s->N : 1);
    if ((rc = s->alloc(&s->snap_h, Mz * snap_cells)) || (rc = s->alloc(&s->snap_hu, Mz * snap_cells)) ||
        (rc = s->alloc(&s->snap_hv, Mz * snap_cells)) || (rc = s->alloc(&s->snap_v, Mz * snap_nodes)))
        return rc;
    // hyetographs, one per member
    s->hys.resize(M);
    for (int32_t m = 0; m < M; ++m) {
        const int nh = forcings[m].hyetograph_count;
        double *hy = nullptr;
        if ((rc = s->alloc(&hy, 3 * (size_t)(nh > 0 ? nh : 1)))) return rc;
        if (nh > 0) {
            FL_CUDA(cudaMemcpy(hy, forcings[m].hyeto_start_s, sizeof(double) * nh, cudaMemcpyHostToDevice));
            FL_CUDA(cudaMemcpy(hy + nh, forcings[m].hyeto_end_s, sizeof(double) * nh, cudaMemcpyHostToDevice));
            FL_CUDA(cudaMemcpy(hy + 2 * nh, forcings[m].hyeto_rate_mps, sizeof(double) * nh, cudaMemcpyHostToDevice));
        }
        s->hys[m].start_s = hy;
        s->hys[m].end_s = hy + nh;
        s->hys[m].rate = hy + 2 * nh;
        s->hys[m].n = nh;
    }
    s->hy = s->hys[0];
    // scratch
    s->sa.n_tiles = (int32_t)L.tile_info.size();
    s->sa.e_cap = L.e_cap;
    s->sa.h_cap = L.h_cap;
    FL_CUDA(plan_surface_launch(s->sa, s->kind, device, &s->surf_grid, &s->surf_smem));
    int sms = 0;
    FL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    s->sms = sms;
    if (p.surface_step_mode != 0 && p.surface_step_mode != 1)
        return set_error(FL_E_INVALID, "solver.surface_step_mode must be 'full_swe' or 'local_inertial'");
    s->li_mode = p.surface_step_mode == 1;
    // the surface ledger: per warp of the surface kernel (or of the local-inertial cell kernel)
    s->n_led_s = (size_t)std::max(surface_warps(s->surf_grid), s->li_mode ? li_cell_blocks(C) * 8 : 0) * SURF_TERMS;
    s->dt_blocks = std::max(1, std::min(sms * 4, (C + 255) / 256));
    float *dt_partial = nullptr;
    unsigned int *counter = nullptr;
    if ((rc = s->alloc(&dt_partial, s->dt_blocks)) || (rc = s->alloc(&counter, 1)) || (rc = s->alloc(&s->dt_out, Mz)) ||
        (rc = s->alloc(&s->vol_out, 2 * (size_t)VOL_BLOCKS * Mz)) || (rc = s->alloc(&s->led_s, Mz * s->n_led_s)))
        return rc;
    FL_CUDA(cudaMemset(counter, 0, sizeof(unsigned int)));
    for (int b = 0; b < 3; ++b)
        if ((rc = s->alloc(&s->stage_f[b], C))) return rc;
    const size_t nd = std::max<size_t>((size_t)std::max(s->N, s->NL), 1);
    if ((rc = s->alloc(&s->stage_d, nd))) return rc;

    // drainage
    if (with_drain) {
        {
            // arena for every drainage table (256-byte aligned pieces)
            const size_t I = (size_t)std::max(s->I, 1), N = (size_t)std::max(s->N, 1), NL = (size_t)std::max(s->NL, 1);
            const size_t K = (size_t)std::max(s->K, 1), G = (size_t)std::max(s->G, 1), S = L.nl.size() + 1;
            const size_t bytes = I * (4 + 8 + 16 + 8 + 8) + (K + 1) * 4 + K * 4 + (N + 1) * 4 * 2 + N * (4 + 16 + 4) +
                                 G * 16 + S * 8 + NL * (4 * 3 + 16 * 3 + 4 * 3) + N * (8 * 2 + 4 + 4 + 4) +
                                 (size_t)(node_blocks(s->N) * 4 * D1_TERMS + network_blocks(s->G) * 4 * D2_TERMS) * 8 +
                                 (L.node_tstart.size() + L.node_tw.size()) * 4 + N * 8 +
                                 (L.tcell.size() + L.tcell_start.size()) * 4 + L.tcell_ent.size() * 8 +
                                 L.tcell.size() * 8 + 80 * 256 +
                                 // the other members' node / link / inlet arrays and ledgers
                                 (Mz - 1) * (N * (8 * 2 + 4) + NL * (4 * 3) + I * 8 +
                                             (size_t)(node_blocks(s->N) * 4 * D1_TERMS + network_blocks(s->G) * 4 * D2_TERMS) * 8);
            void *q = nullptr;
            cudaError_t e = cudaMalloc(&q, bytes);
            if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
            s->allocs.push_back(q);
            s->arena = (char *)q;
            s->arena_size = bytes;
            s->arena_used = 0;
        }
        int32_t *in_node, *kcell_start, *node_in_start, *nls, *lf, *lt;
        float4 *in_par, *nd0, *lk0, *lk1, *lk2;
        float *node_area, *nd_capv;
        int4 *grp, *in_qk;
        int2 *nl;
        if ((rc = s->upload(&in_node, L.in_node)) || (rc = s->upload(&in_qk, L.in_qk)) ||
            (rc = s->upload(&lf, L.link_from)) || (rc = s->upload(&lt, L.link_to)) ||
            (rc = s->upload(&in_par, L.in_par)) || (rc = s->upload(&kcell_start, L.kcell_start)) ||
            (rc = s->upload(&node_in_start, L.node_in_start)) || (rc = s->upload(&node_area, L.node_area)) ||
            (rc = s->upload(&nd0, L.nd0)) || (rc = s->upload(&nd_capv, L.nd_capv)) || (rc = s->upload(&grp, L.grp)) ||
            (rc = s->upload(&nls, L.node_link_start)) || (rc = s->upload(&nl, L.nl)) ||
            (rc = s->upload(&lk0, L.lk0)) || (rc = s->upload(&lk1, L.lk1)) || (rc = s->upload(&lk2, L.lk2)) ||
            (rc = s->upload(&s->node_perm, L.node_perm)) || (rc = s->upload(&s->link_perm, L.link_perm)))
            return rc;
        const size_t MN = Mz * (size_t)s->N, ML = Mz * (size_t)std::max(s->NL, 1);
        if ((rc = s->alloc(&s->Va, MN)) || (rc = s->alloc(&s->Vb, MN)) || (rc = s->alloc(&s->Q[0], ML)) ||
            (rc = s->alloc(&s->Q[1], ML)) || (rc = s->alloc(&s->stage_n, s->N)))
            return rc;
        FL_CUDA(cudaMemset(s->Va, 0, sizeof(float2) * MN));
        FL_CUDA(cudaMemset(s->Vb, 0, sizeof(float2) * MN));
        FL_CUDA(cudaMemset(s->Q[0], 0, sizeof(float) * ML));
        FL_CUDA(cudaMemset(s->Q[1], 0, sizeof(float) * ML));
        s->d1_blocks = node_blocks(s->N);
        s->d2_blocks = network_blocks(s->G);
        s->n_led_1 = (size_t)s->d1_blocks * 4 * D1_TERMS;
        s->n_led_2 = (size_t)s->d2_blocks * 4 * D2_TERMS;
        float *T, *fac;
        float2 *capsur;
        if ((rc = s->alloc(&s->led_1, Mz * s->n_led_1)) || (rc = s->alloc(&s->led_2, Mz * s->n_led_2)) ||
            (rc = s->alloc(&T, ML)) || (rc = s->alloc(&fac, MN)) || (rc = s->alloc(&capsur, Mz * std::max(s->I, 1))))
            return rc;
        FL_CUDA(cudaMemset(capsur, 0, sizeof(float2) * Mz * std::max(s->I, 1)));
        MemberStrides ms{};
        ms.n = M;
        ms.cells = Cp;
        ms.nodes = s->N;
        ms.links = s->NL;
        ms.inlets = s->I;
        ms.led1 = (int64_t)s->n_led_1;
        ms.led2 = (int64_t)s->n_led_2;
        ms.snap_h = (int64_t)snap_cells;
        ms.snap_v = (int64_t)snap_nodes;
        InletReqView &v = s->nd.inl;
        v.in_node = in_node;
        v.in_par = in_par;
        v.Va = s->Va;
        v.rule = drain->inlet_capture_rule;
        v.coef_area = drain->inlet_orifice_coefficient * drain->inlet_orifice_area_m2;
        const float eq = sqrtf(4.0f * 3.14159265358979323846f * std::max(drain->inlet_orifice_area_m2, 0.0f));
        const float perim = drain->inlet_weir_perimeter_m > 0.0f ? drain->inlet_weir_perimeter_m : eq;
        v.weir_coef_perim = drain->inlet_weir_coefficient * std::max(perim, 0.0f);
        v.g2 = (float)(2.0 * (double)(float)p.gravity_mps2);
        NodeArgs &a = s->nd;
        a.node_in_start = node_in_start;
        a.in_qk = in_qk;
        a.cinfo = cinfo;
        a.state0 = s->state[0];
        a.state1 = s->state[1];
        a.capsur = capsur;
        a.Va = s->Va;
        a.Vb = s->Vb;
        a.ctrl = s->ctrl;
        a.ledger = s->led_1;
        a.N = s->N;
        a.ms = ms;
        LinkArgs &la = s->lk;
        la.link_from = lf;
        la.link_to = lt;
        la.lk0 = lk0;
        la.lk1 = lk1;
        la.lk2 = lk2;
        la.node_area = node_area;
        la.Vb = s->Vb;
        la.Q0 = s->Q[0];
        la.Q1 = s->Q[1];
        la.T = T;
        la.ctrl = s->ctrl;
        la.L = s->NL;
        la.g = (float)p.gravity_mps2;
        la.wave_speed = drain->pressurized_wave_speed_mps;
        la.ms = ms;
        DonorArgs &dn = s->dn;
        dn.node_link_start = nls;
        dn.nl = nl;
        dn.Vb = s->Vb;
        dn.T = T;
        dn.fac = fac;
        dn.ctrl = s->ctrl;
        dn.N = s->N;
        dn.ms = ms;
        NetArgs &b = s->nw;
        b.grp = grp;
        b.kcell_start = kcell_start;
        b.capsur = capsur;
        b.node_link_start = nls;
        b.nl = nl;
        b.T = T;
        b.fac = fac;
        b.nd0 = nd0;
        b.nd_capv = nd_capv;
        b.cinfo = cinfo;
        b.state0 = s->state[0];
        b.state1 = s->state[1];
        b.Vb = s->Vb;
        b.Va = s->Va;
        b.Q0 = s->Q[0];
        b.Q1 = s->Q[1];
        b.wet = s->wet;
        b.snap_h = s->snap_h;
        b.snap_v = s->snap_v;
        b.ctrl = s->ctrl;
        b.ledger = s->led_2;
        b.G = s->G;
        b.C = C;
        b.N = s->N;
        b.forcing_kind = s->kind;
        b.g = (float)p.gravity_mps2;
        b.md = (float)p.min_depth_m;
        b.has_recharge = 0;
        b.table = 0;
        b.U = 0;
        b.ms = ms;
        if (!L.node_tstart.empty()) {
            int32_t *tstart, *tcell, *tcs;
            float *tw;
            int2 *tent;
            double *ovf, *s2;
            const size_t U = L.tcell.size();
            if ((rc = s->upload(&tstart, L.node_tstart)) || (rc = s->upload(&tw, L.node_tw)) ||
                (rc = s->upload(&tcell, L.tcell)) || (rc = s->upload(&tcs, L.tcell_start)) ||
                (rc = s->upload(&tent, L.tcell_ent)) || (rc = s->alloc(&ovf, (size_t)s->N)) || (rc = s->alloc(&s2, U)))
                return rc;
            FL_CUDA(cudaMemset(ovf, 0, sizeof(double) * s->N));
            FL_CUDA(cudaMemset(s2, 0, sizeof(double) * std::max<size_t>(U, 1)));
            b.table = 1;
            b.node_tstart = tstart;
            b.node_tw = tw;
            b.ovf_node = ovf;
            b.tcell = tcell;
            b.s2 = s2;
            b.U = (int32_t)U;
            SurchargeArgs &sg = s->sur;
            sg.cell = tcell;
            sg.start = tcs;
            sg.ent = tent;
            sg.ovf_node = ovf;
            sg.s2 = s2;
            sg.cinfo = cinfo;
            sg.state0 = s->state[0];
            sg.state1 = s->state[1];
            sg.wet = s->wet;
            sg.snap_h = s->snap_h;
            sg.ctrl = s->ctrl;
            sg.U = (int32_t)U;
            sg.C = C;
            sg.forcing_kind = s->kind;
            sg.md = (float)p.min_depth_m;
            sg.has_recharge = 0;
        }
        s->drain_base = s->arena;
        s->drain_bytes = s->arena_used;
        s->arena = nullptr;  // later allocations are separate
    }
    setup_l2_persistence(s);
    SurfArgs &a = s->sa;
    a.cinfo = cinfo;
    s->cinfo_d = cinfo;
    s->cinfo_h = L.cinfo;
    a.tile_info = tile_info;
    a.ent = ent;
    a.halo_src = halo_src;
    a.horton = horton;
    a.wet = s->wet;
    a.state0 = s->state[0];
    a.state1 = s->state[1];
    a.ctrl = s->ctrl;
    a.run = s->run;
    a.hy = s->hy;
    a.ledger = s->led_s;
    a.snap_h = s->snap_h;
    a.snap_hu = s->snap_hu;
    a.snap_hv = s->snap_hv;
    a.snap_t = s->snap_t;
    a.C = C;
    a.forcing_kind = s->kind;
    a.infil_scalar = forcing->infiltration_mps;
    a.g = (float)p.gravity_mps2;
    a.half_g = (float)(0.5 * p.gravity_mps2);
    a.md = (float)p.min_depth_m;
    a.vmax = (float)p.max_speed_mps;
    a.stage = mesh->has_stage_boundary ? mesh->boundary_stage_m : 0.0f;
    a.has_stage = mesh->has_stage_boundary;
    DtArgs &d = s->da;
    d.state0 = s->state[0];
    d.state1 = s->state[1];
    d.char_len = char_len;
    d.ctrl = s->ctrl;
    d.run = s->run;
    d.hy = s->hy;
    d.partial = dt_partial;
    d.counter = counter;
    d.snap_t = s->snap_t;
    d.C = C;
    d.cfl = (float)p.cfl;
    d.g = (float)p.gravity_mps2;
    d.md = (float)p.min_depth_m;
    d.dt_out = nullptr;
    d.li = s->li_mode ? 1 : 0;
    if (s->li_mode) {
        // local-inertial tables: edges renumbered by their left cell (new
        // order), each cell's edges in the reference's slot order
        const int32_t E = mesh->edge_count;
        std::vector<int32_t> eord(E), enew(E);
        std::iota(eord.begin(), eord.end(), 0);
        std::stable_sort(eord.begin(), eord.end(), [&](int32_t x, int32_t y) {
            return L.inv[mesh->edge_left_cell[x]] < L.inv[mesh->edge_left_cell[y]];
        });
        for (int32_t k = 0; k < E; ++k) enew[eord[k]] = k;
        auto act = [&](int32_t c) { return mesh->active_mask ? mesh->active_mask[c] > 0.5f : true; };
        std::vector<int2> lr(E);
        std::vector<float4> geo(E);
        for (int32_t k = 0; k < E; ++k) {
            const int32_t e = eord[k], l = mesh->edge_left_cell[e], r = mesh->edge_right_cell[e];
            const bool interior = r >= 0, la = act(l), ra = interior ? act(r) : la;
            const int32_t code = (interior && la && !ra) ? 0 : mesh->boundary_code[e];
            uint32_t f = 0;
            if (interior) f |= LI_INTERIOR;
            if (interior && la && ra) f |= LI_AI;
            if (!interior && la && (code == 1 || code == 4)) f |= LI_BEDGE;
            if (la) f |= LI_LACTIVE;
            if (ra) f |= LI_RACTIVE;
            float fb;
            memcpy(&fb, &f, 4);
            lr[k] = make_int2(L.inv[l], interior ? L.inv[r] : -1);
            geo[k] = make_float4(mesh->edge_normal_x[e], mesh->edge_normal_y[e], mesh->edge_length_m[e], fb);
        }
        // per cell: the slot bits, the other cell and the normal of each slot's
        // edge; per edge: its slot in each of its cells, the face distance
        // max(0.5 (l_L + l_R), 1e-6) and the face Manning n (the mean over
        // the two cells of an active interior edge), in float32 as the
        // reference forms them
        std::vector<uint32_t> cbits(Cp, 0u);
        std::vector<int4> coth(Cp, make_int4(-1, -1, -1, -1));
        std::vector<float2> cnrm((size_t)3 * C, make_float2(0.0f, 0.0f));
        std::vector<uint32_t> eslot(E, 0u);
        for (int32_t i = 0; i < C; ++i) {
            const int32_t c = L.perm[i];
            int32_t ov[3] = {-1, -1, -1};
            for (int j = 0; j < 3; ++j) {
                const int32_t eo = L.inc[(size_t)c * 3 + j];
                if (eo < 0) continue;
                const int32_t k = enew[eo];
                uint32_t f;
                memcpy(&f, &geo[k].w, 4);
                const bool left = lr[k].x == i;
                uint32_t b = LIS_PRESENT;
                if (left) b |= LIS_LEFT;
                if (f & LI_AI) b |= LIS_AI;
                if (f & LI_INTERIOR) {
                    b |= LIS_INTERIOR;
                    ov[j] = left ? lr[k].y : lr[k].x;
                }
                cbits[i] |= b << (4 * j);
                eslot[k] |= (uint32_t)j << (left ? LI_SLOTL_SHIFT : LI_SLOTR_SHIFT);
                cnrm[(size_t)j * C + i] = make_float2(geo[k].x, geo[k].y);
            }
            coth[i] = make_int4(ov[0], ov[1], ov[2], -1);
        }
        std::vector<float2> edm(E);
        for (int32_t k = 0; k < E; ++k) {
            uint32_t f;
            memcpy(&f, &geo[k].w, 4);
            f |= eslot[k];
            memcpy(&geo[k].w, &f, 4);
            const int32_t l = lr[k].x, r = (f & LI_INTERIOR) ? lr[k].y : lr[k].x;
            const float hl = 0.5f * (L.char_len[l] + L.char_len[r]);
            const float dist = hl >= 1.0e-6f ? hl : 1.0e-6f;
            const float mn = (f & LI_AI) ? 0.5f * (L.cinfo[l].y + L.cinfo[r].y) : L.cinfo[l].y;
            edm[k] = make_float2(dist, mn);
        }
        int2 *d_lr;
        float4 *d_geo, *d_qs;
        float2 *d_dm, *d_nrm;
        uint32_t *d_bits;
        int4 *d_oth;
        if ((rc = s->upload(&d_lr, lr)) || (rc = s->upload(&d_geo, geo)) || (rc = s->upload(&d_dm, edm)) ||
            (rc = s->upload(&d_bits, cbits)) || (rc = s->upload(&d_oth, coth)) || (rc = s->upload(&d_nrm, cnrm)) ||
            (rc = s->alloc(&d_qs, (size_t)Cp)))
            return rc;
        LiArgs &q = s->li;
        q.e_lr = d_lr;
        q.e_geo = d_geo;
        q.e_dm = d_dm;
        q.c_bits = d_bits;
        q.c_other = d_oth;
        q.c_nrm = d_nrm;
        q.cinfo = cinfo;
        q.char_len = char_len;
        q.horton = horton;
        q.wet = s->wet;
        q.state0 = s->state[0];
        q.state1 = s->state[1];
        q.Qs = d_qs;
        q.ctrl = s->ctrl;
        q.run = s->run;
        q.hy = s->hy;
        q.snap_t = s->snap_t;
        q.ledger = s->led_s;
        q.snap_h = s->snap_h;
        q.snap_hu = s->snap_hu;
        q.snap_hv = s->snap_hv;
        q.ext_add = nullptr;
        q.E = E;
        q.C = C;
        q.forcing_kind = s->kind;
        q.infil_scalar = forcing->infiltration_mps;
        q.g = (float)p.gravity_mps2;
        q.md = (float)p.min_depth_m;
        q.vmax = (float)p.max_speed_mps;
    }

    // host side
    FL_CUDA(cudaHostAlloc((void **)&s->run_h, Mz * sizeof(RunCtrl), cudaHostAllocDefault));
    FL_CUDA(cudaHostAlloc((void **)&s->poll_h, 2 * Mz * sizeof(RunCtrl), cudaHostAllocDefault));
    memset(s->run_h, 0, Mz * sizeof(RunCtrl));
    FL_CUDA(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
    FL_CUDA(cudaEventCreateWithFlags(&s->ev[0], cudaEventDisableTiming));
    FL_CUDA(cudaEventCreateWithFlags(&s->ev[1], cudaEventDisableTiming));
    const int interval = p.cfl_update_interval_steps;
    s->chunk = interval % 2 == 0 ? interval : 2 * interval;
    while (s->chunk < 16) s->chunk *= 2;  // short CFL cycles: several per graph
    // member 0's arrays start every per-member allocation
    FlSolver::MemberBase &b0 = s->mb;
    b0.state[0] = s->state[0];
    b0.state[1] = s->state[1];
    b0.wet = s->wet;
    b0.ctrl = s->ctrl;
    b0.run = s->run;
    b0.run_h = s->run_h;
    b0.snap_t = s->snap_t;
    b0.snap_h = s->snap_h;
    b0.snap_hu = s->snap_hu;
    b0.snap_hv = s->snap_hv;
    b0.snap_v = s->snap_v;
    b0.led_s = s->led_s;
    b0.led_1 = s->led_1;
    b0.led_2 = s->led_2;
    b0.dt_out = s->dt_out;
    b0.vol_out = s->vol_out;
    b0.Va = s->Va;
    b0.Vb = s->Vb;
    b0.Q[0] = s->Q[0];
    b0.Q[1] = s->Q[1];
    s->select(0);
    FL_CUDA(cudaDeviceSynchronize());
    return fl_reset_clock(s, nullptr);
}

FL_API int fl_create(const FlMeshDesc *mesh, const FlDrainDesc *drain, const FlForcingDesc *forcing,
                     const FlParams *params, int32_t device, FlSolver **out) {
    return fl_create_members(mesh, drain, forcing, 1, params, device, out);
}

FL_API int fl_create_members(const FlMeshDesc *mesh, const FlDrainDesc *drain, const FlForcingDesc *forcings,
                             int32_t n_members, const FlParams *params, int32_t device, FlSolver **out) {
    if (!out) return set_error(FL_E_INVALID, "out is NULL");
    *out = nullptr;
    FlSolver *s = new (std::nothrow) FlSolver();
    if (!s) return set_error(FL_E_NOMEM, "out of host memory");
    int rc = create_impl(mesh, drain, forcings, n_members, params, device, s);
    if (rc != FL_OK) {
        std::string msg = g_error;
        fl_destroy(s);
        g_error = msg;
        return rc;
    }
    *out = s;
    return FL_OK;
}

FL_API int fl_member_select(FlSolver *s, int32_t member) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    if (member < 0 || member >= s->members)
        return set_error(FL_E_INVALID, "member %d is out of range (%d members)", member, s->members);
    s->select(member);
    return FL_OK;
}

FL_API int fl_member_count(FlSolver *s, int32_t *members) {
    if (!s || !members) return set_error(FL_E_INVALID, "solver or output is NULL");
    *members = s->members;
    return FL_OK;
}

static int reset_member_clock(FlSolver *s, cudaStream_t st);

FL_API int fl_reset_clock(FlSolver *s, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    const int32_t keep = s->cur;
    for (int32_t m = 0; m < s->members; ++m) {
        s->select(m);
        const int rc = reset_member_clock(s, st);
        if (rc) {
            s->select(keep);
            return rc;
        }
    }
    s->select(keep);
    s->slot = 0;
    return FL_OK;
}

// The clock reset of the selected member.
static int reset_member_clock(FlSolver *s, cudaStream_t st) {
    const int32_t parity = s->run_h ? s->run_h->parity : 0;
    RunCtrl r;
    memset(&r, 0, sizeof(r));
    r.t = 0.0;
    r.cached_dt = -1.0;
    r.next_snap_t = 0.0;
    r.final_t = s->params.duration_s;
    r.stop_t = 0.0;
    r.max_dt = s->params.max_dt_s;
    r.safety = s->params.cfl_reuse_safety_factor;
    r.snap_interval = s->params.snapshot_interval_s;
    r.g = s->params.gravity_mps2;
    r.last_dt = 0.0;
    r.step = 0;
    r.max_step = std::numeric_limits<int64_t>::max();
    r.parity = parity;
    r.snap_count = 0;
    r.max_snaps = s->params.max_snapshots;
    r.error = 0;
    r.cfl_interval = s->params.cfl_update_interval_steps;
    r.finite_interval = s->params.finite_check_interval_steps;
    r.hyeto_n = s->hy.n;
    *s->run_h = r;
    FL_CUDA(cudaMemcpyAsync(s->run, s->run_h, sizeof(RunCtrl), cudaMemcpyHostToDevice, st));
    FL_CUDA(cudaMemsetAsync(s->ctrl, 0, sizeof(StepCtrl) * 2, st));
    FL_CUDA(cudaMemsetAsync(s->wet, 0, sizeof(float) * (size_t)s->C, st));
    FL_CUDA(cudaMemsetAsync(s->led_s, 0, sizeof(float2) * s->n_led_s, st));
    if (s->has_drain()) {
        FL_CUDA(cudaMemsetAsync(s->led_1, 0, sizeof(float2) * s->n_led_1, st));
        FL_CUDA(cudaMemsetAsync(s->led_2, 0, sizeof(float2) * s->n_led_2, st));
    }
    if (s->has_inflow()) FL_CUDA(cudaMemsetAsync(s->ext.led, 0, sizeof(float2) * s->ext.J, st));
    if (s->has_recharge()) {
        FL_CUDA(cudaMemsetAsync(s->rch.storage, 0, sizeof(float) * s->R, st));
        FL_CUDA(cudaMemsetAsync(s->rch.led, 0, sizeof(float2) * 2 * (size_t)s->R, st));
    }
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_set_state(FlSolver *s, const float *h, const float *hu, const float *hv, const double *node_volume,
                        const double *link_flow, const float *wet_time, int32_t mem, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    const int32_t C = s->C;
    const cudaMemcpyKind k = mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const float *src[3] = {h, hu, hv};
    int mask = 0;
    for (int b = 0; b < 3; ++b) {
        if (!src[b]) continue;
        FL_CUDA(cudaMemcpyAsync(s->stage_f[b], src[b], sizeof(float) * C, k, st));
        mask |= 1 << b;
    }
    if (mask) {
        FL_CUDA(launch_load_state(s->state[s->run_h->parity], s->stage_f[0], s->stage_f[1], s->stage_f[2], s->bed,
                                  s->perm, C, mask, st));
    }
    if (wet_time) {
        FL_CUDA(cudaMemcpyAsync(s->stage_f[0], wet_time, sizeof(float) * C, k, st));
        FL_CUDA(launch_permute_f32(s->stage_f[0], s->wet, s->perm, C, 0, st));
    }
    if (node_volume && s->N > 0) {
        FL_CUDA(cudaMemcpyAsync(s->stage_d, node_volume, sizeof(double) * s->N, k, st));
        FL_CUDA(launch_f64_to_ff_perm(s->stage_d, s->Va, s->node_perm, s->N, st));
    }
    if (link_flow && s->NL > 0) {
        FL_CUDA(cudaStreamSynchronize(st));
        FL_CUDA(cudaMemcpyAsync(s->stage_d, link_flow, sizeof(double) * s->NL, k, st));
        FL_CUDA(launch_f64_to_f32_perm(s->stage_d, s->Q[s->run_h->parity], s->link_perm, s->NL, st));
    }
    g_launches += (mask ? 1 : 0) + (wet_time ? 1 : 0) + (node_volume && s->N ? 1 : 0) + (link_flow && s->NL ? 1 : 0);
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_get_state(FlSolver *s, float *h, float *hu, float *hv, double *node_volume, double *link_flow,
                        float *wet_time, int32_t mem, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    const int32_t C = s->C;
    const cudaMemcpyKind k = mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (h || hu || hv) {
        FL_CUDA(launch_store_state(s->state[s->run_h->parity], h ? s->stage_f[0] : nullptr, hu ? s->stage_f[1] : nullptr,
                                   hv ? s->stage_f[2] : nullptr, s->perm, C, st));
        if (h) FL_CUDA(cudaMemcpyAsync(h, s->stage_f[0], sizeof(float) * C, k, st));
        if (hu) FL_CUDA(cudaMemcpyAsync(hu, s->stage_f[1], sizeof(float) * C, k, st));
        if (hv) FL_CUDA(cudaMemcpyAsync(hv, s->stage_f[2], sizeof(float) * C, k, st));
        FL_CUDA(cudaStreamSynchronize(st));
    }
    if (wet_time) {
        FL_CUDA(launch_permute_f32(s->wet, s->stage_f[0], s->perm, C, 1, st));
        FL_CUDA(cudaMemcpyAsync(wet_time, s->stage_f[0], sizeof(float) * C, k, st));
        FL_CUDA(cudaStreamSynchronize(st));
    }
    if (node_volume && s->N > 0) {
        FL_CUDA(launch_ff_to_f64_perm(s->Va, s->stage_d, s->node_perm, s->N, st));
        FL_CUDA(cudaMemcpyAsync(node_volume, s->stage_d, sizeof(double) * s->N, k, st));
        FL_CUDA(cudaStreamSynchronize(st));
    }
    if (link_flow && s->NL > 0) {
        FL_CUDA(launch_f32_to_f64_perm(s->Q[s->run_h->parity], s->stage_d, s->link_perm, s->NL, st));
        FL_CUDA(cudaMemcpyAsync(link_flow, s->stage_d, sizeof(double) * s->NL, k, st));
        FL_CUDA(cudaStreamSynchronize(st));
    }
    return FL_OK;
}

// fl_run with several members: every member runs to the end of the run, all
// of them stepping together (each with its own dt) until the last one ends.
static int run_members(FlSolver *s, double t_target_s, int64_t max_steps, cudaStream_t st) {
    const int32_t M = s->members, keep = s->cur;
    if (max_steps > 0 || t_target_s < s->params.duration_s)
        return set_error(FL_E_UNSUPPORTED, "with several members fl_run runs every member to the end of the run "
                                           "(t_target >= duration, no step cap)");
    FL_CUDA(cudaMemcpyAsync(s->mb.run_h, s->mb.run, sizeof(RunCtrl) * M, cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    int64_t step0 = -1;
    for (int32_t m = 0; m < M; ++m) {
        RunCtrl &r = s->mb.run_h[m];
        if (r.error) {
            s->select(m);
            const int rc = error_code_message(s);
            s->select(keep);
            return rc;
        }
        if (r.t < r.final_t) {
            if (step0 < 0) step0 = r.step;
            else if (r.step != step0) return set_error(FL_E_UNSUPPORTED, "members are at different steps");
        }
        r.stop_t = r.final_t;
        r.max_step = std::numeric_limits<int64_t>::max();
    }
    if (step0 < 0) return FL_OK;  // every member has ended
    const int interval = s->params.cfl_update_interval_steps;
    if (step0 % interval != 0)
        return set_error(FL_E_UNSUPPORTED, "members resume at step %lld, not a multiple of the CFL interval",
                         (long long)step0);
    FL_CUDA(cudaMemcpyAsync(s->mb.run, s->mb.run_h, sizeof(RunCtrl) * M, cudaMemcpyHostToDevice, st));
    // the first launch (a CFL step) plans every member's step from its run state
    for (int32_t m = 0; m < M; ++m)
        FL_CUDA(cudaMemsetAsync(&s->mb.ctrl[2 * m + s->slot], 0, sizeof(StepCtrl), st));
    int rc = capture_graph(s);
    if (rc) return rc;
    int64_t launched = 0, last_total = -1;
    int stalled = 0;
    const int per_chunk = s->chunk * s->launches_per_step() + M * ((s->chunk + interval - 1) / interval);
    while (true) {
        FL_CUDA(cudaGraphLaunch(s->graph, st));
        g_launches += per_chunk;
        FL_CUDA(cudaMemcpyAsync(&s->poll_h[(launched & 1) * M], s->mb.run, sizeof(RunCtrl) * M,
                                cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaEventRecord(s->ev[launched & 1], st));
        ++launched;
        if (launched >= 2) {
            FL_CUDA(cudaEventSynchronize(s->ev[launched & 1]));
            const RunCtrl *p = &s->poll_h[(launched & 1) * M];
            bool done = true, failed = false;
            int64_t total = 0;
            for (int32_t m = 0; m < M; ++m) {
                failed = failed || p[m].error != 0;
                if (p[m].t < p[m].stop_t) done = false;
                total += p[m].step;
            }
            if (failed || done) break;
            stalled = (total == last_total) ? stalled + 1 : 0;
            last_total = total;
            if (stalled >= 3) {
                FL_CUDA(cudaStreamSynchronize(st));
                return set_error(FL_E_CUDA, "device loop stopped advancing at %lld member steps", (long long)total);
            }
        }
    }
    s->slot = 0;
    FL_CUDA(cudaMemcpyAsync(s->mb.run_h, s->mb.run, sizeof(RunCtrl) * M, cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    for (int32_t m = 0; m < M; ++m) {
        s->select(m);
        const RunCtrl &e = *s->run_h;
        if (!e.error && e.finite_interval > 0 && e.step > 0 && e.step % e.finite_interval == 0) {
            FL_CUDA(launch_finite(s->state[0], s->state[1], s->run, s->C, st));
            g_launches++;
            if ((rc = sync_run(s, st))) break;
        }
        if (s->run_h->error) {
            rc = error_code_message(s);
            break;
        }
    }
    s->select(keep);
    return rc;
}

FL_API int fl_run(FlSolver *s, double t_target_s, int64_t max_steps, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    if (s->members > 1) return run_members(s, t_target_s, max_steps, st);
    int rc = sync_run(s, st);
    if (rc) return rc;
    if (s->run_h->error) return error_code_message(s);
    RunCtrl &r = *s->run_h;
    const double stop = std::min(t_target_s, r.final_t);
    const int64_t start_step = r.step;
    r.stop_t = stop;
    r.max_step = max_steps > 0 ? start_step + max_steps : std::numeric_limits<int64_t>::max();
    if ((rc = push_run(s, st))) return rc;
    if (!(r.t < stop)) return FL_OK;
    const int interval = s->params.cfl_update_interval_steps;
    // the next launch re-plans from the run state
    FL_CUDA(cudaMemsetAsync(&s->ctrl[s->slot], 0, sizeof(StepCtrl), st));
    int64_t hs = start_step;
    if (hs % interval != 0) {
        FL_CUDA(launch_replan(s->run, s->snap_t, s->hy, s->ctrl, s->slot, st));
        g_launches++;
    }
    while (hs % interval != 0) {  // unaligned prefix: single steps
        const bool next_eval = (hs + 1) % interval == 0;
        if ((rc = launch_step(s, s->slot, false, !next_eval, st))) return rc;
        s->slot ^= 1;
        ++hs;
    }
    if ((rc = capture_graph(s))) return rc;
    // graph chunks, polling progress one chunk behind
    int64_t launched = 0;
    int64_t last_step = -1;
    int stalled = 0;
    const int per_chunk = s->chunk * s->launches_per_step() + s->members * ((s->chunk + interval - 1) / interval);
    while (true) {
        FL_CUDA(cudaGraphLaunch(s->graph, st));
        g_launches += per_chunk;
        FL_CUDA(cudaMemcpyAsync(&s->poll_h[launched & 1], s->run, sizeof(RunCtrl), cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaEventRecord(s->ev[launched & 1], st));
        ++launched;
        if (launched >= 2) {
            FL_CUDA(cudaEventSynchronize(s->ev[launched & 1]));
            const RunCtrl &p = s->poll_h[launched & 1];
            if (p.error || !(p.t < stop) || p.step >= r.max_step) break;
            // every chunk of an unfinished run advances the step count
            stalled = (p.step == last_step) ? stalled + 1 : 0;
            last_step = p.step;
            if (stalled >= 3) {
                FL_CUDA(cudaStreamSynchronize(st));
                return set_error(FL_E_CUDA, "device loop stopped advancing at step %lld (t=%.3f s)",
                                 (long long)p.step, p.t);
            }
        }
    }
    s->slot = 0;
    if ((rc = sync_run(s, st))) return rc;
    const RunCtrl &e = *s->run_h;
    if (!e.error && e.finite_interval > 0 && e.step > 0 && e.step % e.finite_interval == 0) {
        FL_CUDA(launch_finite(s->state[0], s->state[1], s->run, s->C, st));
        g_launches++;
        if ((rc = sync_run(s, st))) return rc;
    }
    if (s->run_h->error) return error_code_message(s);
    if (s->run_h->t < stop) return set_error(FL_E_STEP_CAP, "step cap reached at t=%.3f s (target %.3f s)", s->run_h->t, stop);
    return FL_OK;
}

FL_API int fl_step(FlSolver *s, double dt_s, int32_t phases, double rain_rate_mps, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    if (s->members > 1) return set_error(FL_E_UNSUPPORTED, "fl_step runs a single-member solver");
    if (!(dt_s > 0.0)) return set_error(FL_E_INVALID, "timestep_s must be positive.");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    RunCtrl &r = *s->run_h;
    StepCtrl c;
    memset(&c, 0, sizeof(c));
    c.t0 = r.t;
    c.dt = dt_s;
    c.dt_f = (float)dt_s;
    c.dtg_f = (float)(dt_s * s->params.gravity_mps2);
    c.rain_f = (float)rain_rate_mps;
    c.active = 1;
    c.parity = r.parity;
    c.snap_slot = -1;
    c.check_finite = 0;
    c.phases = phases;
    c.step = r.step;
    r.t += dt_s;
    r.step += 1;
    r.parity ^= 1;
    r.last_dt = dt_s;
    FL_CUDA(cudaMemcpyAsync(&s->ctrl[s->slot], &c, sizeof(StepCtrl), cudaMemcpyHostToDevice, st));
    FL_CUDA(cudaMemcpyAsync(s->run, s->run_h, sizeof(RunCtrl), cudaMemcpyHostToDevice, st));
    if (s->has_inflow() && (phases & FL_PHASE_INFLOW)) {
        FL_CUDA(launch_inflow(s->ext, s->slot, st));
        g_launches++;
    }
    if (s->li_mode) {
        FL_CUDA(launch_li(s->li, s->kind, s->slot, 0, s->sms, st));
        g_launches += 2;
    } else {
        FL_CUDA(launch_surface(s->sa, s->kind, s->slot, 0, s->surf_grid, s->surf_smem, st));
        g_launches++;
    }
    if (s->has_drain() && (phases & FL_PHASE_DRAINAGE)) {
        FL_CUDA(launch_nodes(s->nd, s->slot, st));
        FL_CUDA(launch_links(s->lk, s->slot, st));
        FL_CUDA(launch_donor(s->dn, s->slot, st));
        FL_CUDA(launch_network(s->nw, s->slot, st));
        g_launches += 4;
        if (s->has_table()) {
            FL_CUDA(launch_surcharge(s->sur, s->slot, st));
            g_launches++;
        }
    } else if (s->has_drain()) {
        // no drainage this step: carry link flow to the other parity buffer
        FL_CUDA(cudaMemcpyAsync(s->Q[r.parity], s->Q[c.parity], sizeof(float) * std::max(s->NL, 1),
                                cudaMemcpyDeviceToDevice, st));
    }
    if (s->has_recharge() && (phases & FL_PHASE_RECHARGE)) {
        FL_CUDA(launch_recharge(s->rch, s->slot, st));
        g_launches++;
    }
    s->slot ^= 1;
    FL_CUDA(cudaStreamSynchronize(st));
    FL_CUDA(cudaGetLastError());
    return FL_OK;
}

FL_API int fl_time_kernel(FlSolver *s, int32_t kernel, int32_t reps, void *stream, double *ms_per_launch) {
    if (!s || !ms_per_launch || reps < 1) return set_error(FL_E_INVALID, "bad fl_time_kernel arguments");
    if (s->members > 1) return set_error(FL_E_UNSUPPORTED, "fl_time_kernel times a single-member solver");
    if ((kernel == 1 || kernel == 2 || kernel == 4 || kernel == 5) && !s->has_drain())
        return set_error(FL_E_INVALID, "solver has no drainage");
    if (kernel < 0 || kernel > 5) return set_error(FL_E_INVALID, "kernel must be 0..5");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    const RunCtrl &r = *s->run_h;
    StepCtrl c;
    memset(&c, 0, sizeof(c));
    const double dt = r.last_dt > 0.0 ? r.last_dt : 0.1;
    c.t0 = r.t;
    c.dt = dt;
    c.dt_f = (float)dt;
    c.dtg_f = (float)(dt * s->params.gravity_mps2);
    c.active = 1;
    c.parity = r.parity;
    c.snap_slot = -1;
    c.phases = FL_PHASE_ALL;
    c.step = r.step;
    FL_CUDA(cudaMemcpyAsync(&s->ctrl[0], &c, sizeof(StepCtrl), cudaMemcpyHostToDevice, st));
    auto launch = [&](cudaStream_t ls) -> cudaError_t {
        switch (kernel) {
            case 0:
                return s->li_mode ? launch_li(s->li, s->kind, 0, 0, s->sms, ls)
                                  : launch_surface(s->sa, s->kind, 0, 0, s->surf_grid, s->surf_smem, ls);
            case 1: return launch_nodes(s->nd, 0, ls);
            case 2: return launch_network(s->nw, 0, ls);
            case 4: return launch_links(s->lk, 0, ls);
            case 5: return launch_donor(s->dn, 0, ls);
            default: {
                DtArgs a = s->da;
                a.dt_out = s->dt_out;
                return launch_dt(a, s->dt_blocks, 0, 0, ls);
            }
        }
    };
    const int per = (kernel == 0 && s->li_mode) ? 2 : 1;  // kernels per launch
    // A chain of launches captured as one graph and replayed, as in the step
    // loop: the time is the kernels' own, not the host's launch rate or a
    // graph launch's.
    const int chain = std::min(reps, 32);
    const int replays = (reps + chain - 1) / chain;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    FL_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int i = 0; i < chain && le == cudaSuccess; ++i) le = launch(s->cap_stream);
    const cudaError_t ce = cudaStreamEndCapture(s->cap_stream, &g);
    cudaError_t err = le != cudaSuccess ? le : ce;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err == cudaSuccess) err = cudaGraphLaunch(ge, st);  // warm-up
    if (err == cudaSuccess) err = cudaEventRecord(e0, st);
    for (int i = 0; i < replays && err == cudaSuccess; ++i) err = cudaGraphLaunch(ge, st);
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ge) cudaGraphExecDestroy(ge);
    if (err != cudaSuccess) return set_error(FL_E_CUDA, "fl_time_kernel: %s", cudaGetErrorString(err));
    g_launches += (int64_t)per * chain * (replays + 1);
    *ms_per_launch = (double)ms / ((double)replays * chain);
    return FL_OK;
}

FL_API int fl_stable_timestep(FlSolver *s, double *dt_s, void *stream) {
    if (!s || !dt_s) return set_error(FL_E_INVALID, "solver or output is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    DtArgs a = dt_args(s, s->cur);
    a.dt_out = s->dt_out;
    FL_CUDA(launch_dt(a, s->dt_blocks, 0, 0, st));
    g_launches++;
    double v = -1.0;
    FL_CUDA(cudaMemcpyAsync(&v, s->dt_out, sizeof(double), cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    if (!(v > 0.0)) return set_error(FL_E_INVALID, "No finite cells are available for timestep calculation.");
    *dt_s = v;
    return FL_OK;
}

FL_API int fl_update_forcing(FlSolver *s, const float *rain_multiplier, const float *f0, const float *fc,
                             const float *k, float infiltration_mps) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    FL_CUDA(cudaSetDevice(s->device));
    if (s->kind == 0) {
        if (s->sa.infil_scalar != infiltration_mps) {
            s->sa.infil_scalar = infiltration_mps;
            s->li.infil_scalar = infiltration_mps;
            if (s->graph) {  // the graph holds the kernel arguments by value
                cudaGraphExecDestroy(s->graph);
                s->graph = nullptr;
            }
        }
        return FL_OK;
    }
    const int32_t C = s->C;
    std::vector<float4> hz(C);
    FL_CUDA(cudaMemcpy(hz.data(), s->sa.horton, sizeof(float4) * C, cudaMemcpyDeviceToHost));
    for (int32_t i = 0; i < C; ++i) {
        const int32_t r = s->perm_h[i];
        if (f0) hz[i].x = f0[r];
        if (fc) hz[i].y = fc[r];
        if (k) hz[i].z = k[r];
        if (rain_multiplier) hz[i].w = rain_multiplier[r];
    }
    FL_CUDA(cudaMemcpy((void *)s->sa.horton, hz.data(), sizeof(float4) * C, cudaMemcpyHostToDevice));
    return FL_OK;
}

FL_API int fl_get_progress(FlSolver *s, FlProgress *out, void *stream) {
    if (!s || !out) return set_error(FL_E_INVALID, "solver or output is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    const RunCtrl &r = *s->run_h;
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

static void sum_blocks(const std::vector<float2> &v, int terms, double *out) {
    for (int j = 0; j < terms; ++j) out[j] = 0.0;
    const size_t blocks = v.size() / terms;
    for (size_t b = 0; b < blocks; ++b)
        for (int j = 0; j < terms; ++j) out[j] += (double)v[b * terms + j].x + (double)v[b * terms + j].y;
}

FL_API int fl_read_ledger(FlSolver *s, double *out, int32_t n, void *stream) {
    if (!s || !out) return set_error(FL_E_INVALID, "solver or output is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    double all[FL_LEDGER_COUNT] = {0};
    std::vector<float2> v(s->n_led_s);
    FL_CUDA(cudaMemcpyAsync(v.data(), s->led_s, sizeof(float2) * v.size(), cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    sum_blocks(v, SURF_TERMS, all + FL_LEDGER_RAINFALL);
    if (s->has_drain()) {
        std::vector<float2> v1(s->n_led_1), v2(s->n_led_2);
        FL_CUDA(cudaMemcpyAsync(v1.data(), s->led_1, sizeof(float2) * v1.size(), cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaMemcpyAsync(v2.data(), s->led_2, sizeof(float2) * v2.size(), cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaStreamSynchronize(st));
        sum_blocks(v1, D1_TERMS, all + FL_LEDGER_CAPTURE);
        sum_blocks(v2, D2_TERMS, all + FL_LEDGER_OUTFALL);
    }
    if (s->has_inflow()) {
        std::vector<float2> ve(s->ext.J);
        FL_CUDA(cudaMemcpyAsync(ve.data(), s->ext.led, sizeof(float2) * ve.size(), cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaStreamSynchronize(st));
        sum_blocks(ve, 1, all + FL_LEDGER_EXTERNAL_INFLOW);
    }
    if (s->has_recharge()) {
        std::vector<float2> vr(2 * (size_t)s->R);
        FL_CUDA(cudaMemcpyAsync(vr.data(), s->rch.led, sizeof(float2) * vr.size(), cudaMemcpyDeviceToHost, st));
        FL_CUDA(cudaStreamSynchronize(st));
        sum_blocks(vr, 2, all + FL_LEDGER_RECHARGE_CAPTURE);
    }
    FL_CUDA(launch_volumes(s->state[0], s->state[1], s->sa.cinfo, s->Va, s->run, s->C, s->N, s->vol_out, st));
    g_launches++;
    std::vector<double> vp(2 * (size_t)VOL_BLOCKS);
    FL_CUDA(cudaMemcpyAsync(vp.data(), s->vol_out, sizeof(double) * vp.size(), cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    all[FL_LEDGER_SURFACE_VOLUME] = 0.0;
    all[FL_LEDGER_SURFACE_VOLUME + 1] = 0.0;
    for (int b = 0; b < VOL_BLOCKS; ++b) {  // block order: the same sum on every call
        all[FL_LEDGER_SURFACE_VOLUME] += vp[2 * b];
        all[FL_LEDGER_SURFACE_VOLUME + 1] += vp[2 * b + 1];
    }
    for (int i = 0; i < n && i < FL_LEDGER_COUNT; ++i) out[i] = all[i];
    return FL_OK;
}

FL_API int fl_get_snapshots(FlSolver *s, int32_t first, int32_t count, double *times_s, float *h, float *hu,
                            float *hv, float *node_volume, int32_t mem, void *stream) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    int rc = sync_run(s, st);
    if (rc) return rc;
    if (first < 0 || count < 0 || first + count > s->run_h->snap_count)
        return set_error(FL_E_INVALID, "snapshots [%d, %d) requested, %d available", first, first + count,
                         s->run_h->snap_count);
    const cudaMemcpyKind k = mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t C = (size_t)s->C;
    if (times_s) {
        FL_CUDA(cudaMemcpyAsync(times_s, s->snap_t + first, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
    }
    float *src[3] = {s->snap_h, s->snap_hu, s->snap_hv};
    float *dst[3] = {h, hu, hv};
    for (int b = 0; b < 3; ++b) {
        if (!dst[b]) continue;
        for (int32_t i = 0; i < count; ++i) {
            FL_CUDA(launch_permute_f32(src[b] + (size_t)(first + i) * C, s->stage_f[0], s->perm, s->C, 1, st));
            FL_CUDA(cudaMemcpyAsync(dst[b] + (size_t)i * C, s->stage_f[0], sizeof(float) * C, k, st));
            FL_CUDA(cudaStreamSynchronize(st));
        }
    }
    if (node_volume && s->N > 0 && count > 0) {
        for (int32_t i = 0; i < count; ++i) {
            FL_CUDA(launch_permute_f32(s->snap_v + (size_t)(first + i) * s->N, s->stage_n, s->node_perm, s->N, 1, st));
            FL_CUDA(cudaMemcpyAsync(node_volume + (size_t)i * s->N, s->stage_n, sizeof(float) * s->N, k, st));
            FL_CUDA(cudaStreamSynchronize(st));
        }
    }
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

// ------------------------------------------------- inflow and recharge tables
static uint32_t cell_flags(const float4 &ci) {
    uint32_t f;
    memcpy(&f, &ci.z, 4);
    return f;
}

static void set_cell_flags(float4 &ci, uint32_t f) { memcpy(&ci.z, &f, 4); }

// Replace one flag bit on the given cells (new order) and upload the cell info.
static int put_flag(FlSolver *s, uint32_t bit, const std::vector<int32_t> &cells) {
    for (float4 &ci : s->cinfo_h) set_cell_flags(ci, cell_flags(ci) & ~bit);
    for (int32_t c : cells) set_cell_flags(s->cinfo_h[c], cell_flags(s->cinfo_h[c]) | bit);
    FL_CUDA(cudaMemcpy(s->cinfo_d, s->cinfo_h.data(), sizeof(float4) * s->cinfo_h.size(), cudaMemcpyHostToDevice));
    return FL_OK;
}

// Drop the captured step graph (it holds kernel arguments by value).
static void drop_graph(FlSolver *s) {
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
}

static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

FL_API int fl_set_boundary_inflow(FlSolver *s, int32_t J, const int32_t *cells, int32_t T, const double *times,
                                  const float *q) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    if (s->members > 1 && J > 0) return set_error(FL_E_UNSUPPORTED, "external inflow needs a single-member solver");
    if (J < 0) return set_error(FL_E_INVALID, "receiver_count must be >= 0");
    if (J > 0 && (!cells || !times || !q || T < 1))
        return set_error(FL_E_INVALID, "external inflow needs receiver cells, at least one time and the flow table");
    std::vector<int32_t> inv(s->C);
    for (int32_t i = 0; i < s->C; ++i) inv[s->perm_h[i]] = i;
    // receivers grouped by cell (cells in new order, receivers ascending)
    std::vector<std::pair<int32_t, int32_t>> byc(J);
    for (int32_t j = 0; j < J; ++j) {
        const int32_t c = cells[j];
        if (c < 0 || c >= s->C) return set_error(FL_E_INVALID, "External boundary inflow cell_index is outside mesh range.");
        if (!(cell_flags(s->cinfo_h[inv[c]]) & CELL_ACTIVE))
            return set_error(FL_E_INVALID, "External boundary inflow cell_index contains inactive cells.");
        byc[j] = {inv[c], j};
    }
    for (int32_t k = 0; k < T && J > 0; ++k) {
        if (!std::isfinite(times[k]) || (k > 0 && !(times[k] > times[k - 1])))
            return set_error(FL_E_INVALID, "external inflow times must be finite and strictly increasing");
    }
    std::sort(byc.begin(), byc.end());
    std::vector<int32_t> ucell, start, recv(J);
    for (int32_t k = 0; k < J; ++k) {
        if (k == 0 || byc[k].first != byc[k - 1].first) {
            ucell.push_back(byc[k].first);
            start.push_back(k);
        }
        recv[k] = byc[k].second;
    }
    start.push_back(J);
    const int32_t U = (int32_t)ucell.size();
    FL_CUDA(cudaSetDevice(s->device));
    FL_CUDA(cudaDeviceSynchronize());  // no launch in flight still reads the old tables
    drop_graph(s);
    if (s->ext_mem) {
        cudaFree(s->ext_mem);
        s->ext_mem = nullptr;
    }
    s->ext = InflowArgs{};
    s->sa.ext_add = nullptr;
    s->li.ext_add = nullptr;
    int rc = put_flag(s, CELL_RECEIVER, ucell);
    if (rc || J == 0) return rc;
    const size_t o_s = up256(sizeof(int32_t) * U), o_r = o_s + up256(sizeof(int32_t) * (U + 1)),
                 o_t = o_r + up256(sizeof(int32_t) * J), o_q = o_t + up256(sizeof(double) * T),
                 o_l = o_q + up256(sizeof(float) * (size_t)T * J), o_a = o_l + up256(sizeof(float2) * J),
                 bytes = o_a + sizeof(float) * (size_t)s->Cp;
    void *m = nullptr;
    cudaError_t e = cudaMalloc(&m, bytes);
    if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    s->ext_mem = m;
    char *b = (char *)m;
    FL_CUDA(cudaMemcpy(b, ucell.data(), sizeof(int32_t) * U, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_s, start.data(), sizeof(int32_t) * (U + 1), cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_r, recv.data(), sizeof(int32_t) * J, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_t, times, sizeof(double) * T, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_q, q, sizeof(float) * (size_t)T * J, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemset(b + o_l, 0, sizeof(float2) * J));
    FL_CUDA(cudaMemset(b + o_a, 0, sizeof(float) * (size_t)s->Cp));
    InflowArgs &x = s->ext;
    x.cell = (const int32_t *)b;
    x.start = (const int32_t *)(b + o_s);
    x.recv = (const int32_t *)(b + o_r);
    x.times = (const double *)(b + o_t);
    x.q = (const float *)(b + o_q);
    x.led = (float2 *)(b + o_l);
    x.add = (float *)(b + o_a);
    x.cinfo = s->cinfo_d;
    x.ctrl = s->ctrl;
    x.U = U;
    x.J = J;
    x.T = T;
    s->sa.ext_add = x.add;
    s->li.ext_add = x.add;
    return FL_OK;
}

FL_API int fl_set_recharge(FlSolver *s, int32_t R, const int32_t *cells, const float *storage_cap,
                           const float *capture_cap, const float *recharge_cap, const float *stop_depth) {
    if (!s) return set_error(FL_E_INVALID, "solver is NULL");
    if (s->members > 1 && R > 0) return set_error(FL_E_UNSUPPORTED, "surface recharge needs a single-member solver");
    if (R < 0) return set_error(FL_E_INVALID, "row_count must be >= 0");
    if (R > 0 && (!cells || !storage_cap || !capture_cap || !recharge_cap || !stop_depth))
        return set_error(FL_E_INVALID, "recharge needs cells and the four per-row arrays");
    std::vector<int32_t> inv(s->C);
    for (int32_t i = 0; i < s->C; ++i) inv[s->perm_h[i]] = i;
    // rows grouped by cell (cells in new order, rows in table order)
    std::vector<std::pair<int32_t, int32_t>> byc(R);
    for (int32_t r = 0; r < R; ++r) {
        if (cells[r] < 0 || cells[r] >= s->C) return set_error(FL_E_INVALID, "recharge source_cell_index is outside mesh range");
        byc[r] = {inv[cells[r]], r};
    }
    std::sort(byc.begin(), byc.end());
    std::vector<int32_t> ucell, start, rows(R);
    std::vector<float4> par(R);
    for (int32_t k = 0; k < R; ++k) {
        if (k == 0 || byc[k].first != byc[k - 1].first) {
            ucell.push_back(byc[k].first);
            start.push_back(k);
        }
        rows[k] = byc[k].second;
    }
    start.push_back(R);
    for (int32_t r = 0; r < R; ++r) par[r] = make_float4(storage_cap[r], capture_cap[r], recharge_cap[r], stop_depth[r]);
    const int32_t U = (int32_t)ucell.size();
    FL_CUDA(cudaSetDevice(s->device));
    FL_CUDA(cudaDeviceSynchronize());
    drop_graph(s);
    if (s->rch_mem) {
        cudaFree(s->rch_mem);
        s->rch_mem = nullptr;
    }
    s->rch = RechargeArgs{};
    s->R = 0;
    s->nw.has_recharge = 0;
    s->sur.has_recharge = 0;
    int rc = put_flag(s, CELL_RECHARGE, ucell);
    if (rc || R == 0) return rc;
    const size_t o_s = up256(sizeof(int32_t) * U), o_r = o_s + up256(sizeof(int32_t) * (U + 1)),
                 o_p = o_r + up256(sizeof(int32_t) * R), o_st = o_p + up256(sizeof(float4) * R),
                 o_l = o_st + up256(sizeof(float) * R), bytes = o_l + sizeof(float2) * 2 * (size_t)R;
    void *m = nullptr;
    cudaError_t e = cudaMalloc(&m, bytes);
    if (e != cudaSuccess) return set_error(FL_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    s->rch_mem = m;
    char *b = (char *)m;
    FL_CUDA(cudaMemcpy(b, ucell.data(), sizeof(int32_t) * U, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_s, start.data(), sizeof(int32_t) * (U + 1), cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_r, rows.data(), sizeof(int32_t) * R, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemcpy(b + o_p, par.data(), sizeof(float4) * R, cudaMemcpyHostToDevice));
    FL_CUDA(cudaMemset(b + o_st, 0, sizeof(float) * R));
    FL_CUDA(cudaMemset(b + o_l, 0, sizeof(float2) * 2 * (size_t)R));
    RechargeArgs &a = s->rch;
    a.cell = (const int32_t *)b;
    a.row_start = (const int32_t *)(b + o_s);
    a.rows = (const int32_t *)(b + o_r);
    a.par = (const float4 *)(b + o_p);
    a.storage = (float *)(b + o_st);
    a.led = (float2 *)(b + o_l);
    a.cinfo = s->cinfo_d;
    a.state0 = s->state[0];
    a.state1 = s->state[1];
    a.wet = s->wet;
    a.snap_h = s->snap_h;
    a.ctrl = s->ctrl;
    a.U = U;
    a.C = s->C;
    a.forcing_kind = s->kind;
    a.md = (float)s->params.min_depth_m;
    s->R = R;
    s->nw.has_recharge = 1;
    s->sur.has_recharge = 1;
    return FL_OK;
}

FL_API int fl_get_recharge_storage(FlSolver *s, float *out, int32_t n, int32_t mem, void *stream) {
    if (!s || !out) return set_error(FL_E_INVALID, "solver or output is NULL");
    if (n != s->R) return set_error(FL_E_INVALID, "recharge storage has %d rows, %d requested", s->R, n);
    if (n == 0) return FL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    FL_CUDA(cudaMemcpyAsync(out, s->rch.storage, sizeof(float) * n,
                            mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

FL_API int fl_set_recharge_storage(FlSolver *s, const float *in, int32_t n, int32_t mem, void *stream) {
    if (!s || !in) return set_error(FL_E_INVALID, "solver or input is NULL");
    if (n != s->R) return set_error(FL_E_INVALID, "recharge storage has %d rows, %d given", s->R, n);
    if (n == 0) return FL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    FL_CUDA(cudaSetDevice(s->device));
    FL_CUDA(cudaMemcpyAsync(s->rch.storage, in, sizeof(float) * n,
                            mem == FL_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    FL_CUDA(cudaStreamSynchronize(st));
    return FL_OK;
}

}  // extern "C"
