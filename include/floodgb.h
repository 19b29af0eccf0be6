/*
 * floodgb -- C ABI of the GB300 (sm_103a) flood step library (libfloodgb.so).
 *
 * The library replaces the reference's CuPy fused-kernel dispatch for the
 * explicit finite-volume flood step (arsanjeevk/gpu-urban-flood-cupy-jax,
 * package gurugram_flood).  Each entry point below names the reference
 * interface it stands in for.  All signatures use plain pointers and sizes;
 * arrays are given in the reference's layout and cell order (the library
 * renumbers internally and converts back on output).
 *
 * Return codes: FL_OK (0) or a negative FL_E_* code; fl_last_error() gives
 * the message of the most recent failure on the calling thread.
 *
 * Threading: a solver is used from one host thread at a time; every call
 * takes the CUDA stream it runs on (NULL = the legacy default stream).
 */
#ifndef FLOODGB_H
#define FLOODGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_API __attribute__((visibility("default")))

#define FLOODGB_ABI_VERSION 1

enum {
    FL_OK = 0,
    FL_E_INVALID = -1,     /* bad argument, shape or index (reference: ValueError) */
    FL_E_CUDA = -2,        /* CUDA runtime failure */
    FL_E_NO_DEVICE = -3,   /* no usable CUDA device (reference: BackendUnavailableError) */
    FL_E_NONFINITE = -4,   /* non-finite depth at a check step (reference: SimulationError) */
    FL_E_STEP_CAP = -5,    /* the step cap ended fl_run before the target time */
    FL_E_NOMEM = -6,       /* host or device allocation failed */
    FL_E_UNSUPPORTED = -7, /* input uses a reference feature this library does not implement */
    FL_E_SNAPSHOTS = -8,   /* more snapshots than FlParams.max_snapshots */
    FL_E_TIMEOUT = -9      /* a device-side wait gave up after its time limit (the run stops) */
};

/* Step phases for fl_step (a bit set). */
enum {
    FL_PHASE_SURFACE = 1,  /* fluxes, cell update + Manning, rain and infiltration */
    FL_PHASE_CLAMP = 2,    /* velocity clamp */
    FL_PHASE_DRAINAGE = 4, /* inlet exchange, links, outfalls, overflow return */
    FL_PHASE_INFLOW = 8,   /* external boundary inflow (after the clamp) */
    FL_PHASE_RECHARGE = 16, /* surface recharge capture (after the drainage) */
    FL_PHASE_ALL = 31
};

/* Memory kind of caller buffers in state / snapshot transfers. */
enum { FL_MEM_HOST = 0, FL_MEM_DEVICE = 1 };

/* Inlet capture rules (reference: inlet_capture_rule strings). */
enum { FL_CAPTURE_CAPACITY = 0, FL_CAPTURE_HEAD_LIMITED = 1, FL_CAPTURE_ORIFICE = 2, FL_CAPTURE_WEIR_ORIFICE = 3 };

/* Surface mesh: the fields of TriangularSurfaceTopology
 * (gurugram_flood/kernels/triangular_backend.py:58-90), host pointers. */
typedef struct {
    int32_t cell_count, edge_count;
    const float *bed_elevation_m, *manning_n, *cell_area_m2, *characteristic_length_m;
    const float *active_mask; /* NULL: every cell active; values must be 0 or 1 */
    const int32_t *edge_left_cell, *edge_right_cell, *boundary_code;
    const float *edge_normal_x, *edge_normal_y, *edge_length_m;
    const float *centroid_x, *centroid_y; /* optional: enable space-filling-curve renumbering */
    int32_t has_stage_boundary;
    float boundary_stage_m;
} FlMeshDesc;

/* Drainage: TriangularNodeCouplingTopology (:130-154) and
 * TriangularPipeNetworkTopology (:172-200), host pointers; optional arrays
 * may be NULL exactly where the reference allows None. */
typedef struct {
    int32_t node_count, link_count, inlet_count;
    const int32_t *inlet_cell_index, *inlet_node_index, *node_surface_cell_index;
    const float *node_invert_elevation_m, *node_storage_area_m2, *node_max_depth_m;
    const float *inlet_capture_capacity_m3ps, *inlet_surcharge_capacity_m3ps;
    const int32_t *link_from_node_index, *link_to_node_index;
    const float *link_length_m, *link_area_m2, *link_hydraulic_radius_m, *link_manning_n;
    const float *link_flow_capacity_m3ps, *link_invert_elevation_m, *link_diameter_m;
    const float *link_minor_loss_coefficient;
    const int32_t *link_geometry_code;
    const float *link_rect_width_m, *link_rect_height_m;
    const float *outfall_area_m2, *outfall_coefficient, *outfall_tailwater_head_m;
    const float *outfall_flow_capacity_m3ps;
    float pressurized_wave_speed_mps;
    int32_t inlet_capture_rule;
    float inlet_orifice_area_m2, inlet_orifice_coefficient, inlet_weir_perimeter_m, inlet_weir_coefficient;
    /* Weighted surcharge-return table (surcharge_cell_index / _node_index /
     * _return_weight / _return_weight_is_normalized, used when all three
     * arrays are given: triangular_backend.py:1424-1474).  Entries with a
     * negative node or cell are ignored; entry_count 0 = the per-node return
     * to node_surface_cell_index. */
    int32_t surcharge_entry_count;
    const int32_t *surcharge_cell_index, *surcharge_node_index;
    const float *surcharge_return_weight;
    int32_t surcharge_return_weight_is_normalized;
} FlDrainDesc;

/* Forcing: kind 0 = uniform (scalar rain from the hyetograph, scalar
 * infiltration capacity); kind 1 = per cell (rain = rate x multiplier,
 * Horton capacity fc + (f0 - fc) exp(-k wet_time)); reference
 * production_infiltration_support.py:96-138. */
typedef struct {
    int32_t kind;
    const float *rain_multiplier, *horton_f0_mps, *horton_fc_mps, *horton_k_per_s;
    float infiltration_mps;
    int32_t hyetograph_count;
    const double *hyeto_start_s, *hyeto_end_s, *hyeto_rate_mps;
} FlForcingDesc;

/* Solver knobs: SolverConfig (gurugram_flood/config.py:84-100). */
typedef struct {
    double gravity_mps2, min_depth_m;
    double cfl;
    int32_t cfl_update_interval_steps;
    double cfl_reuse_safety_factor;
    double max_dt_s, max_speed_mps;
    int32_t finite_check_interval_steps;
    double duration_s, snapshot_interval_s;
    int32_t max_snapshots;
    /* 0: full_swe (step_triangular_surface); 1: local_inertial
     * (step_triangular_surface_local_inertial, triangular_backend.py:531-590,
     * with stable_local_inertial_triangular_timestep_s, :975-994). */
    int32_t surface_step_mode;
} FlParams;

typedef struct {
    double t_s;
    int64_t step_count, cfl_eval_count, cfl_reused_count;
    int32_t snapshot_count;
    int32_t error;      /* 0 or an FL_E_* code */
    int64_t error_step; /* step count at the failed check */
    double last_dt_s;
} FlProgress;

/* Ledger terms (cumulative m^3, float64): the keys of engine.py's `cum`
 * (engine.py:197-207) plus the diagnostics the pipe step returns. */
enum {
    FL_LEDGER_RAINFALL = 0,
    FL_LEDGER_INFILTRATION,
    FL_LEDGER_BOUNDARY_IN,
    FL_LEDGER_BOUNDARY_OUT,
    FL_LEDGER_CAPTURE,
    FL_LEDGER_SURCHARGE,
    FL_LEDGER_OUTFALL,
    FL_LEDGER_OVERFLOW,
    FL_LEDGER_UNRETURNED,
    FL_LEDGER_LINK_ABS,
    FL_LEDGER_SURFACE_VOLUME, /* current sum(h * area) */
    FL_LEDGER_NODE_VOLUME,    /* current sum(node volume) */
    FL_LEDGER_EXTERNAL_INFLOW,  /* external_boundary_inflow_m3 */
    FL_LEDGER_RECHARGE_CAPTURE, /* surface_recharge_capture_m3 */
    FL_LEDGER_RECHARGE_LOSS,    /* surface_recharge_loss_m3 */
    FL_LEDGER_COUNT
};

typedef struct FlSolver FlSolver;

/* Library version and last error message (thread-local). */
FL_API int fl_abi_version(void);
FL_API const char *fl_last_error(void);

/* Number of visible CUDA devices (0 on a machine without a GPU). */
FL_API int fl_device_count(int32_t *count);

/* Build the device layout and upload the static inputs.  Replaces the
 * upload + cell_edge_indices build of triangular_topology_to_backend,
 * triangular_node_coupling_to_backend and triangular_pipe_network_to_backend
 * (triangular_backend.py:329-475) and the per-run setup of run_simulation
 * (gurugram_flood/solver/engine.py:137-161).  drain may be NULL. */
FL_API int fl_create(const FlMeshDesc *mesh, const FlDrainDesc *drain, const FlForcingDesc *forcing,
                     const FlParams *params, int32_t device, FlSolver **out);
FL_API void fl_destroy(FlSolver *solver);

/* Ensemble members on one mesh.  No counterpart in the reference, which runs
 * one scenario per process.  n_members runs of the same mesh, drainage
 * network and parameters that differ in their rainfall: member m takes the
 * hyetograph of forcings[m], and the per-cell fields (Horton f0 / fc / k,
 * rain multiplier, scalar infiltration) of forcings[0] apply to every
 * member.  Each member has its own state, adaptive dt, snapshots and
 * ledger and follows exactly the single-instance step of fl_run; per step
 * the surface kernel runs once per member and each drainage kernel once for
 * all members (the members share the static tables).  The calls that take a
 * solver address the selected member (fl_member_select; member 0 after
 * creation), except fl_run, which runs every member to the end of the run
 * (t_target >= the duration, no step cap), and fl_reset_clock, which resets
 * every member.  Not available with several members: the local-inertial
 * step, external inflow, surface recharge, the weighted surcharge table,
 * fl_step and fl_time_kernel (FL_E_UNSUPPORTED).  fl_create is
 * fl_create_members with one member. */
FL_API int fl_create_members(const FlMeshDesc *mesh, const FlDrainDesc *drain, const FlForcingDesc *forcings,
                             int32_t n_members, const FlParams *params, int32_t device, FlSolver **out);
FL_API int fl_member_select(FlSolver *solver, int32_t member);
FL_API int fl_member_count(FlSolver *solver, int32_t *members);

/* State transfer in reference order: TriangularSurfaceState,
 * TriangularPipeNetworkState (:49-55, :203-208) and the Horton wet time.
 * Any pointer may be NULL to leave that field unchanged / unread. */
FL_API int fl_set_state(FlSolver *solver, const float *h, const float *hu, const float *hv,
                        const double *node_volume, const double *link_flow, const float *wet_time,
                        int32_t mem, void *stream);
FL_API int fl_get_state(FlSolver *solver, float *h, float *hu, float *hv, double *node_volume,
                        double *link_flow, float *wet_time, int32_t mem, void *stream);

/* Rewind the clock: t = 0, no cached CFL dt, ledger, snapshots, Horton wet
 * time and recharge storage cleared (the start of run_simulation's loop,
 * engine.py:165-215). */
FL_API int fl_reset_clock(FlSolver *solver, void *stream);

/* Advance the adaptive loop of run_simulation (engine.py:219-344) until the
 * simulated time reaches min(t_target_s, duration) or max_steps more steps
 * ran (FL_E_STEP_CAP).  The loop runs on the device as CUDA-graph chunks of
 * cfl_update_interval_steps steps; the host only polls progress. */
FL_API int fl_run(FlSolver *solver, double t_target_s, int64_t max_steps, void *stream);

/* One step with an explicit dt and a phase set: step_triangular_surface
 * (triangular_backend.py:478-528) for FL_PHASE_SURFACE, clamp_velocity
 * (stabilizers.py:8-27) for FL_PHASE_CLAMP, step_triangular_dynamic_pipe_network
 * (triangular_backend.py:665-830) for FL_PHASE_DRAINAGE, the external
 * boundary inflow at the step's mid time for FL_PHASE_INFLOW and the surface
 * recharge for FL_PHASE_RECHARGE (engine.py:263-289).  rain_rate_mps is
 * the base rainfall rate for the step (multiplied per cell in kind 1). */
FL_API int fl_step(FlSolver *solver, double dt_s, int32_t phases, double rain_rate_mps, void *stream);

/* stable_triangular_timestep_s (triangular_backend.py:955-972) on the current
 * state, with the configured cfl. */
FL_API int fl_stable_timestep(FlSolver *solver, double *dt_s, void *stream);

/* Replace the per-cell forcing fields (kind 1: reference-order arrays, any
 * may be NULL to keep it) or the scalar infiltration capacity (kind 0).
 * The reference passes forcing per step (TriangularSurfaceForcing,
 * triangular_backend.py:93-101); the run loop derives it from these fields. */
FL_API int fl_update_forcing(FlSolver *solver, const float *rain_multiplier, const float *horton_f0_mps,
                             const float *horton_fc_mps, const float *horton_k_per_s, float infiltration_mps);

FL_API int fl_get_progress(FlSolver *solver, FlProgress *out, void *stream);

/* Cumulative ledger, FL_LEDGER_COUNT doubles (n may be smaller). */
FL_API int fl_read_ledger(FlSolver *solver, double *out, int32_t n, void *stream);

/* External boundary inflow: ExternalBoundaryInflowSurface
 * (gurugram_flood/domain/production_event_support.py:24-29), applied every
 * step after the velocity clamp as apply_external_boundary_inflow_depth
 * (:169-196): q_j at t + dt/2 by linear interpolation of the hydrograph
 * (held at the first / last value outside it), h += sum_j float32(q_j) * dt
 * / area over the receivers of each cell.  receiver_cell_index: reference
 * cell order, active cells only; times_s strictly increasing; q_m3ps is
 * [time_count x receiver_count] row-major.  receiver_count 0 removes it.
 * Host pointers; takes effect from the next step. */
FL_API int fl_set_boundary_inflow(FlSolver *solver, int32_t receiver_count, const int32_t *receiver_cell_index,
                                  int32_t time_count, const double *times_s, const float *q_m3ps);

/* Surface recharge: June5RechargeTopology
 * (gurugram_flood/domain/june5_production_drainage.py:99-111), applied every
 * step after the drainage step as apply_june5_surface_recharge (:543-572):
 * capture = min(removable depth above stop_depth x area, capture capacity x
 * dt, remaining storage), then a recharge loss of min(storage, recharge
 * capacity x dt).  Rows sharing a cell all see the same depth and the last
 * row's capture sets it (the reference's NumPy assignment).  row_count 0
 * removes it.  Host pointers; the stored volumes start at zero. */
FL_API int fl_set_recharge(FlSolver *solver, int32_t row_count, const int32_t *source_cell_index,
                           const float *storage_capacity_m3, const float *capture_capacity_m3ps,
                           const float *recharge_capacity_m3ps, const float *stop_depth_m);

/* Stored recharge volume per row (float32, row order), read or replaced. */
FL_API int fl_get_recharge_storage(FlSolver *solver, float *storage_m3, int32_t n, int32_t mem, void *stream);
FL_API int fl_set_recharge_storage(FlSolver *solver, const float *storage_m3, int32_t n, int32_t mem, void *stream);

/* Snapshots [first, first+count) of depth, hu, hv (count x cell_count, reference
 * order) and node volume (count x node_count, float32 as engine.py:321 stores
 * it); times in seconds.  Any output pointer may be NULL. */
FL_API int fl_get_snapshots(FlSolver *solver, int32_t first, int32_t count, double *times_s, float *h,
                            float *hu, float *hv, float *node_volume, int32_t mem, void *stream);

/* Host-only layout check (no GPU needed): builds the renumbered layout and
 * reports its sizes.  stats[0..7] = cells, edges, slots used, inlet cells,
 * nodes, links, drainage groups, max inlets per cell. */
FL_API int fl_plan_check(const FlMeshDesc *mesh, const FlDrainDesc *drain, int64_t *stats, int32_t *perm_out);

/* Host-only surface tiling report (no GPU needed; no reference counterpart).
 * tiles[0..5] = tiles, edge entries, halo cells (sum over tiles), largest
 * entry count of a tile, largest padded halo of a tile, and the shared memory
 * the surface kernel needs per CTA with per-cell forcing (bytes). */
FL_API int fl_plan_tiles(const FlMeshDesc *mesh, int64_t *tiles);

/* Time `reps` back-to-back launches of one kernel of a step (0 surface (the
 * two local-inertial launches in that mode), 1 node inlet exchange, 2 pipe
 * network, 3 CFL reduction, 4 link update, 5 donor factors) between CUDA
 * events on `stream`, at the solver's current state and last dt.  The
 * launches are captured in chains of up to 32 per CUDA graph, each launched
 * as in the step loop (the surface, link, donor and network kernels as
 * programmatic dependents of the launch before them), so the time per launch
 * is the kernel's own in-loop cost, not a graph launch's.  The clock is not
 * advanced but the state buffers are overwritten (reset before the next run).
 * No reference counterpart: it is the measurement hook for the roofline. */
FL_API int fl_time_kernel(FlSolver *solver, int32_t kernel, int32_t reps, void *stream, double *ms_per_launch);

/* Allocation-free CFL timestep.  It has no counterpart in the reference.  It
 * is for callers that may not allocate device memory at this point: a plugin
 * limited to its host application's memory pool, code running while another
 * library captures the stream into a CUDA graph, a service that forbids
 * allocation after start-up.  Over caller-owned device arrays in any cell
 * order it computes the minimum over cells of
 *   cfl * char_len / max(|(hu, hv)| / max(h, min_depth) + sqrt(g * max(h, min_depth)), 1e-12)
 * in float32 with correctly rounded operations (the same reduction as
 * fl_stable_timestep; cells whose value is not finite, e.g. a NaN depth, are
 * skipped), writing it to the device double *dt_out (-1.0 when no cell gives
 * a finite value), asynchronously on `stream`.  It allocates nothing: its
 * scratch is a 16 KB static device array that every GPU loading the library
 * keeps until exit.  The first call on a device looks up that array's
 * address and caches it (make that call before any stream capture; a
 * cudaDeviceReset after it is not supported, as the cached address would then
 * be stale).  At most 8,388,608 cells per call (FL_E_INVALID beyond).  All
 * calls share the one array, so calls that overlap on the GPU race; calls
 * ordered on one stream are safe. */
FL_API int fl_stable_timestep_noalloc(const float *char_len, const float *h, const float *hu, const float *hv,
                                      int32_t n, double cfl, double gravity_mps2, double min_depth_m,
                                      double *dt_out, void *stream);

/* ------------------------------------------------------------------ batch
 * Batched ensemble (no counterpart in the reference, which runs one scenario
 * per process): n surface-only scenarios -- meshes of any sizes, each with
 * its own forcing, hyetograph, duration and adaptive dt -- advanced together
 * by one persistent surface launch per step over all active scenarios' tiles
 * and one planning launch, captured in CUDA graphs.  Each scenario follows
 * exactly the single-instance step of fl_run (same fluxes, dt rule, clamp,
 * snapshot rule and ledger).  Besides the hourly depth snapshots, each
 * snapshot also stores the per-cell maximum depth since the previous one.
 * The surface kernel's tile size and CTAs per SM come from FlBatchShape
 * (floodgb.autotune picks them by timing). */
typedef struct FlBatch FlBatch;

typedef struct {
    int32_t tile_cells;   /* cells per tile: 128 or 256 (0: 256) */
    int32_t ctas_per_sm;  /* persistent CTAs per SM (0: as many as fit) */
    int32_t chunk_steps;  /* steps per CUDA-graph chunk (0: 32) */
    int32_t reserved;
} FlBatchShape;

/* meshes/forcings/params: n entries each (no drainage; every mesh's stage
 * boundary, if any, must use the same stage; at most 256 scenarios). */
FL_API int fl_batch_create(int32_t n, const FlMeshDesc *meshes, const FlForcingDesc *forcings,
                           const FlParams *params, const FlBatchShape *shape, int32_t device, FlBatch **out);
FL_API void fl_batch_destroy(FlBatch *batch);
/* Initial state of one scenario (reference cell order); default: dry. */
FL_API int fl_batch_set_state(FlBatch *batch, int32_t scen, const float *h, const float *hu, const float *hv,
                              int32_t mem, void *stream);
/* Run every scenario from t = 0 to its own duration (or until max_steps
 * lockstep steps, if > 0); restarts from the state last set. */
FL_API int fl_batch_run(FlBatch *batch, int64_t max_steps, void *stream);
FL_API int fl_batch_progress(FlBatch *batch, int32_t scen, FlProgress *out, void *stream);
FL_API int fl_batch_get_state(FlBatch *batch, int32_t scen, float *h, float *hu, float *hv, int32_t mem,
                              void *stream);
/* Snapshots [first, first+count) of depth and of the maximum depth since the
 * previous snapshot (count x cells each, reference order); times in s. */
FL_API int fl_batch_get_snapshots(FlBatch *batch, int32_t scen, int32_t first, int32_t count, double *times_s,
                                  float *h, float *hmax, int32_t mem, void *stream);
/* The momentum (hu, hv) at the same snapshots (count x cells each, reference
 * order; either pointer may be NULL).  No counterpart in the reference: the
 * surrogate's training data. */
FL_API int fl_batch_get_snapshot_momentum(FlBatch *batch, int32_t scen, int32_t first, int32_t count, float *hu,
                                          float *hv, int32_t mem, void *stream);
/* Cumulative ledger of one scenario (FL_LEDGER_RAINFALL..BOUNDARY_OUT and
 * FL_LEDGER_SURFACE_VOLUME are filled). */
FL_API int fl_batch_read_ledger(FlBatch *batch, int32_t scen, double *out, int32_t n, void *stream);
/* Shape in use, total cells (padded), tiles, and the persistent grid. */
FL_API int fl_batch_info(FlBatch *batch, FlBatchShape *shape, int64_t *cells, int64_t *tiles, int32_t *grid);

/* ------------------------------------------------------------ surrogate
 * Dense layers of the learned surrogate (no counterpart in the reference,
 * whose AI code is not shipped): C[m, n] = act(A[m, K] . B[n, K]^T + bias)
 * (+ residual) on the tensor cores, bf16 operands, fp32 accumulation.  A is
 * the concatenation along K of up to three bf16 segments; row r of segment s
 * is base_s + rows_s[r] * ld_s (rows_s NULL: row r), so gathered inputs need
 * no copy.  Widths are multiples of 64; leading dimensions multiples of 8.
 * k_splits > 1 splits K into that many slices, each writing a plain fp32
 * partial [m, ldo] tile at out_f32 + slice * m * ldo. */
typedef struct {
    const void *base;     /* bf16 */
    const int32_t *rows;  /* row map or NULL */
    int64_t ld;
    int32_t width;
} FlGemmSegment;

typedef struct {
    FlGemmSegment a[3];
    int32_t n_seg;
    int32_t m, n;
    const void *b;        /* bf16 [n, ldb], K contiguous */
    int64_t ldb;
    const float *bias;    /* [n] or NULL */
    const float *residual; /* fp32 [m, ldr] or NULL */
    int64_t ldr;
    float *out_f32;       /* [m, ldo] or NULL */
    void *out_bf16;       /* bf16 [m, ldo] or NULL */
    int64_t ldo;
    int32_t relu;
    int32_t k_splits;
    int32_t force_tiled;  /* 1: one-tile-per-CTA kernel even when K <= 512 (tests) */
} FlGemmDesc;

FL_API int fl_gemm_bf16(const FlGemmDesc *desc, void *stream);
/* Synchronises `stream`; FL_E_TIMEOUT if a GEMM's device wait gave up since
 * the last call (the flag is then cleared). */
FL_API int fl_gemm_status(void *stream);

/* Memory-bound companions of fl_gemm_bf16 for message passing and training
 * (fixed-order sums: reproducible).
 * fl_transpose_bf16: dst[k, r] = A[r, k] for the segment concatenation A
 *   (as fl_gemm_bf16's A), columns m..ldd-1 of dst set to 0.
 * fl_segment_sum: dst[i, :width] (+)= sum over p in [start[i], start[i+1]) of
 *   src[order ? order[p] : p, col0 : col0+width]; optional bf16 copy (with
 *   the bf16 copy and no accumulation, dst may be NULL: bf16 only).
 * fl_relu_bwd: out = dx * (z > 0) (z NULL: no mask), bf16 (+ fp32).
 * fl_colsum: out[c] (+)= sum_r x[r, c]; scratch holds 256 x n floats.
 * fl_adam: Adam step on fp32 w[rows, cols]; refreshes w_bf16 and its
 *   transpose wt_bf16[cols, ldt] when given.
 * fl_cast_bf16: dst = bf16(src). */
FL_API int fl_transpose_bf16(const FlGemmSegment *segs, int32_t n_seg, int32_t m, void *dst, int64_t ldd,
                             void *stream);
FL_API int fl_segment_sum(const float *src, int64_t lds, int32_t col0, const int32_t *start, const int32_t *order,
                          int32_t n_out, int32_t width, float *dst, int64_t ldd, void *dst_bf16, int64_t ldb,
                          int32_t accumulate, void *stream);
FL_API int fl_relu_bwd(const float *dx, int64_t ldx, const void *z_bf16, int64_t ldz, int32_t m, int32_t n,
                       void *out_bf16, int64_t ldo, float *out_f32, int64_t ldf, void *stream);
FL_API int fl_colsum(const float *x, int64_t ldx, int32_t m, int32_t n, float *scratch, float *out, int32_t accumulate,
                     void *stream);
FL_API int fl_adam(float *w, float *m1, float *m2, const float *g, int32_t rows, int32_t cols, float lr, float b1,
                   float b2, float eps, int32_t step, float weight_decay, void *w_bf16, void *wt_bf16, int64_t ldt,
                   void *stream);
FL_API int fl_cast_bf16(const float *src, int64_t lds, int32_t m, int32_t n, void *dst, int64_t ldd, void *stream);

/* Self-test of the bounded device waits (no reference counterpart): one
 * warp waits on an mbarrier that nothing arrives on; *status receives
 * FL_E_TIMEOUT once the wait gives up after limit_s (at most 5 s), and the
 * device stays usable. */
FL_API int fl_wait_selftest(double limit_s, int32_t *status, double *elapsed_s);

/* Number of kernel launches the library has issued in this process. */
FL_API int64_t fl_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
