/*
 * CPU oracle for the flood step -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates the reference's algorithm for the hot path so the
 * GPU implementation can be checked against it.  It is used by the tests,
 * by __graft_entry__.smoke() as a checker, and by bench.py's CPU-baseline
 * leg; the product path (libfloodgb) never links or calls it.
 *
 * Semantics follow the reference (arsanjeevk/gpu-urban-flood-cupy-jax):
 *   surface step   gurugram_flood/kernels/triangular_backend.py:1067-1178
 *                  (_advance_triangular_swe), equations.py:20-152 (HLL,
 *                  hydrostatic reconstruction), triangular_backend.py:1294-1327
 *                  (_right_edge_state), :1330-1379 (_apply_sources)
 *   velocity clamp gurugram_flood/solver/stabilizers.py:8-27
 *   timestep       equations.py:155-178, engine.py:220-232
 *   drainage       triangular_inlet_exchange_cuda_kernels.py:52-207,255-443,
 *                  triangular_pipe_network_cuda_kernels.py:39-211,263-421,
 *                  triangular_backend.py:665-830,1399-1485,1758-1764
 *   forcing        production_infiltration_support.py:96-138,
 *                  real_gurugram_domain.py:374-388
 *   run loop       gurugram_flood/solver/engine.py:219-386
 *   local inertial triangular_local_inertial_cuda_kernels.py:59-262,
 *                  triangular_backend.py:531-590, equations.py:181-210
 *   inflow         gurugram_flood/domain/production_event_support.py:169-196
 *   recharge       gurugram_flood/domain/june5_production_drainage.py:543-572
 * Surface arithmetic is float32 in the reference's operation order (build
 * with -ffp-contract=off); drainage volumes, heads and flows are float64 as
 * in the reference's CuPy kernels.
 */
#ifndef FLOOD_ORACLE_H
#define FLOOD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t cell_count, edge_count;
    const float *bed, *manning, *area, *char_len, *active; /* active may be NULL */
    const int32_t *left, *right, *bcode;
    const float *nx, *ny, *len;
    const int32_t *cell_edges; /* C x 3, reference cell_edge_indices order */
    int32_t has_stage;
    float stage;
} OrcMesh;

typedef struct {
    int32_t node_count, link_count, inlet_count;
    const int32_t *inlet_cell, *inlet_node, *node_cell;
    const float *node_invert, *node_area, *node_maxdepth;
    const float *cap_capacity, *sur_capacity;            /* nullable */
    const int32_t *link_from, *link_to;
    const float *link_len, *link_area, *link_radius, *link_n;
    const float *link_capacity, *link_invert, *link_diam, *link_minor; /* nullable */
    const int32_t *link_geom;                             /* nullable (with rect w/h) */
    const float *link_rect_w, *link_rect_h;
    const float *out_area, *out_coef, *out_tail, *out_capacity; /* out_capacity nullable */
    float wave_speed;
    int32_t capture_rule; /* 0 capacity, 1 head_limited_capacity, 2 orifice, 3 weir_orifice */
    float orifice_area, orifice_coef, weir_perimeter, weir_coef;
    /* weighted surcharge-return table (triangular_backend.py:1424-1474); sur_count 0: none */
    int32_t sur_count;
    const int32_t *sur_cell, *sur_node;
    const float *sur_weight;
    int32_t sur_normalized;
} OrcDrain;

/* Forcing for one step.  rain_kind/infil_kind: 0 scalar, 1 per-cell array. */
typedef struct {
    int32_t rain_kind;
    float rain_scalar;
    const float *rain_cell;
    int32_t infil_kind;
    float infil_scalar;
    const float *infil_cell;
} OrcForcing;

/* diag[0..5]: rain_m3, infil_m3, boundary_net, boundary_in, boundary_out, final_surface_volume */
int orc_surface_step(const OrcMesh *m, const float *h, const float *hu, const float *hv,
                     const OrcForcing *f, double dt, double g, float min_depth,
                     float *h_out, float *hu_out, float *hv_out, double *diag);

void orc_clamp_velocity(int32_t n, const float *h, float *hu, float *hv, float max_speed);

/* Local-inertial surface step (triangular_local_inertial_cuda_kernels.py:59-262
 * + _apply_sources); diag as orc_surface_step. */
int orc_li_step(const OrcMesh *m, const float *h, const float *hu, const float *hv, const OrcForcing *f,
                double dt, double g, float min_depth, float *h_out, float *hu_out, float *hv_out, double *diag);

/* stable_local_inertial_timestep_s (equations.py:181-210); < 0 if no finite cell */
double orc_li_stable_dt(int32_t n, const float *char_len, const float *h, float cfl, float g, float min_depth);

/* returns the global min of the float32 local CFL dt, as a double; <0 if none finite */
double orc_stable_dt(int32_t n, const float *char_len, const float *h, const float *hu,
                     const float *hv, float cfl, float g, float min_depth);

/* diag[0..6]: capture, surcharge, link_abs, outfall, overflow, unreturned, final_node_volume */
int orc_pipe_step(const OrcMesh *m, const OrcDrain *d, float *h, double *node_volume,
                  double *link_flow, double dt, float g, double *diag);

/* External boundary inflow (production_event_support.py:24-29, 169-196). */
typedef struct {
    int32_t receiver_count, time_count;
    const int32_t *receiver_cell;
    const double *times_s;   /* strictly increasing */
    const float *q_m3ps;     /* time_count x receiver_count, row-major */
} OrcInflow;

/* Receiver j's flow at time t: the first / last value outside the table,
 * else np.interp in float64 rounded to float32. */
float orc_inflow_q(const OrcInflow *x, int32_t j, double t);

/* apply_external_boundary_inflow_depth: h += per-cell sum (in receiver order)
 * of float32(q_j) * float32(dt) / area; returns the added volume (float32
 * terms summed in float64). */
double orc_external_inflow(int32_t C, const float *area, const OrcInflow *x, double time_s, double dt, float *h);

/* Surface recharge rows (june5_production_drainage.py:99-111). */
typedef struct {
    int32_t row_count;
    const int32_t *source_cell;
    const float *storage_capacity, *capture_capacity, *recharge_capacity, *stop_depth;
} OrcRecharge;

/* apply_june5_surface_recharge (:543-572), float32 throughout; storage is
 * updated in place; diag[0] capture, diag[1] recharge loss (float64 sums). */
void orc_recharge(const OrcRecharge *r, const float *area, double dt, float *h, float *storage, double *diag);

typedef struct {
    double cfl, safety, max_dt, max_speed, duration_s, snapshot_interval_s;
    int32_t cfl_interval, finite_interval;
    double g;
    float min_depth;
    int32_t horton;              /* 1: per-cell Horton + rain multiplier */
    const float *rain_mult, *f0, *fc, *k; /* Horton fields (horton == 1) */
    int32_t infil_kind;          /* horton == 0: 0 scalar, 1 per-cell constant */
    float infil_scalar;
    const float *infil_cell;
    int32_t hyeto_n;
    const double *hyeto_start_s, *hyeto_end_s, *hyeto_rate;
    int32_t has_drainage;
    int64_t max_steps;           /* <=0: unlimited */
    int32_t max_snapshots;
    const OrcInflow *inflow;     /* nullable: applied after the clamp at t + dt/2 */
    const OrcRecharge *recharge; /* nullable: applied after the drainage step */
    float *recharge_storage;     /* [row_count], in/out (with recharge) */
    int32_t local_inertial;      /* 1: surface_step_mode = local_inertial */
    /* resume point (all zero for a run from t = 0): simulated time and step
     * count reached, the cached CFL dt of that point (< 0: none) and the
     * time of the next snapshot.  A run resumed from the values an earlier
     * run returned continues it step for step. */
    double t_start_s;
    int64_t step_start;
    double cached_dt_s;
    double next_snapshot_s;
} OrcRunParams;

typedef struct {
    int64_t step_count, cfl_evals, cfl_reused;
    int32_t snapshot_count, error; /* error: 0 ok, 1 non-finite depth, 2 snapshot overflow */
    int64_t error_step;
    double t_end;
    double ledger[12]; /* rain, infil, bnet, outfall, overflow, unreturned, capture, surcharge, link_abs,
                          external inflow, recharge capture, recharge loss */
    double cached_dt_s;     /* the CFL dt the next reuse step scales (< 0: none) */
    double next_snapshot_s; /* the snapshot time the loop waits for next */
} OrcRunResult;

/* state arrays are updated in place; snapshots: max_snapshots x C (h, hu, hv) and x N (volume f32) */
int orc_run(const OrcMesh *m, const OrcDrain *d, const OrcRunParams *p, float *h, float *hu,
            float *hv, double *node_volume, double *link_flow, float *wet_time,
            double *snap_t, float *snap_h, float *snap_hu, float *snap_hv, float *snap_v,
            OrcRunResult *out);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
