// Batched ensemble: layout and argument structures shared by the batch
// kernels (fl_batch_kernels.cu) and the batch runtime (fl_batch.cpp).
#pragma once

#include "fl_internal.h"

namespace fl {

constexpr int MAX_SCEN = 256;

// Flags of an active scenario's step.
constexpr int32_t BF_PARITY = 1;       // input state in state1
constexpr int32_t BF_CFL = 2;          // compute the CFL minima of the output (the next step evaluates)
constexpr int32_t BF_FINITE = 4;       // check the input depth for non-finite values
constexpr int BF_PHASE_SHIFT = 4;      // bits 4-6: FL_PHASE_* bits
constexpr int BF_SNAP_SHIFT = 8;       // bits 8-31: snapshot slot + 1 (0: none)

// One active scenario of a step, written by the planner.
struct BatchEntry {
    float dt, dtg, rain, infil;
    int32_t scen, flags, tile0, cells;
};

// The step's active scenarios; tiles of entry k are virtual tiles
// [prefix[k], prefix[k + 1]).
struct BatchList {
    int32_t n;
    int32_t pad[3];
    int32_t prefix[MAX_SCEN + 1];
    int32_t pad2[3];
    BatchEntry e[MAX_SCEN];
};

struct BatchArgs {
    const float4 *cinfo;          // [cells] {area, manning, flags, 0}
    const int4 *tile_info;        // [tiles] {first entry, entry count, first halo index, halo count}
    const float4 *ent;
    const int32_t *halo_src;      // global (concatenated) cell indices
    const float4 *horton;         // kind 1
    float *wet;                   // kind 1
    float4 *state0, *state1;
    float *hmax;                  // running maximum depth since the last snapshot
    const float *char_len;
    const BatchList *list;
    float *tile_min;              // [tiles] CFL minimum of the tile's output (flagged steps)
    float *tile_led;              // [tiles * SURF_TERMS] the tile's ledger terms of the step
    float *snap_h, *snap_hmax;
    float *snap_hu, *snap_hv;     // momentum at each snapshot (same layout)
    const int64_t *snap_base;     // [n] first snapshot element of each scenario
    RunCtrl *run;                 // [n]
    int32_t n_tiles, tile, e_cap, h_cap;
    int32_t off_bar, off_list, off_stage, stage_bytes;
    int32_t so_ci, so_hz, so_wt, so_hm, so_en, so_hs;
    int32_t forcing_kind;
    float g, half_g, md, vmax, stage, cfl;
};

struct PlanArgs {
    RunCtrl *run;                 // [n]
    StepCtrl *ctrl;               // [n * 2]
    double *snap_t;               // [n * max_snaps]
    const HyetoView *hy;          // [n]
    const int32_t *scen_tile0;    // [n + 1]
    const int32_t *scen_cells;    // [n]
    const float *scen_infil;      // [n] uniform infiltration capacity (kind 0)
    const float *tile_min;
    const float *tile_led;
    float2 *ledger;               // [n * SURF_TERMS] float-float running sums
    BatchList *list;
    unsigned int *counter;
    int32_t n, max_snaps;
};

}  // namespace fl
