// Internal layout and control structures shared by the host runtime
// (fl_solver.cpp, fl_plan.cpp) and the kernels (fl_surface.cu, fl_drainage.cu).
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace fl {

// ---------------------------------------------------------------------------
// Surface layout.  Cells are renumbered along a Hilbert curve and grouped in
// tiles of TILE consecutive cells; per-cell arrays are padded to a whole
// number of tiles so every tile is one contiguous, 16-byte aligned block.  A
// cell's (up to three) edges are its "slots", in the reference's
// cell_edge_indices order: edges it is the left cell of (ascending), then
// edges it is the right cell of (ascending).
//
// Each tile has a list of edge entries (every edge with an endpoint in the
// tile that contributes to it, once per tile: an edge inside the tile is one
// entry serving both cells, an edge between two tiles has an entry in each)
// and a halo: the cells outside the tile whose state its entries read,
// ascending.  Entries address cells by tile-local index: 0..TILE-1 for the
// tile's own cells, TILE + j for halo cell j.  An entry is one float4
// {nx, ny, len, bits}:
// ---------------------------------------------------------------------------
constexpr int TILE = 256;
constexpr int SURF_THREADS = TILE + 32;  // surface kernel: 8 compute warps + 1 producer warp
constexpr uint32_t EB_IDX_MASK = 1023u;    // bits 0-9: left local index
constexpr int EB_RIGHT_SHIFT = 10;         // bits 10-19: right local index
constexpr int EB_LSLOT_SHIFT = 20;         // bits 20-21: the edge's slot in the left cell
constexpr uint32_t EB_LPRESENT = 1u << 22; // the left cell is in this tile and takes -F_L
constexpr int EB_RSLOT_SHIFT = 23;         // bits 23-24: the edge's slot in the right cell
constexpr uint32_t EB_RPRESENT = 1u << 25; // the right cell is in this tile and takes +F_R
constexpr uint32_t EB_LACTIVE = 1u << 26;  // left cell active
constexpr uint32_t EB_AI = 1u << 27;       // active interior edge
constexpr uint32_t EB_INTERIOR = 1u << 28; // the edge has a right cell
constexpr int EB_CODE_SHIFT = 29;          // bits 29-31: effective boundary code + 1
// tile_info[t] = {first entry, entry count, first halo index (multiple of 4), halo count}
constexpr int64_t MAX_CELLS = 0x7FFFFFFE;

// cinfo[c] = {area, manning, flags (bits), 1 / area}
constexpr uint32_t CELL_ACTIVE = 1u;
constexpr uint32_t CELL_COUPLED = 2u;       // drainage writes this cell's final depth
constexpr uint32_t CELL_SURCHARGE = 4u;     // a weighted surcharge-return cell (k_surcharge finishes it)
constexpr int CELL_RIGHT_SHIFT = 3;         // bits 3-5: slot k is a right-side slot
constexpr uint32_t CELL_RECEIVER = 1u << 6; // an external boundary inflow receiver
constexpr uint32_t CELL_RECHARGE = 1u << 7; // the recharge step writes this cell's final depth

// Per-step control, double-buffered by launch slot.  Written by the planner
// (one thread) of the previous launch, read by every kernel of the step.
struct StepCtrl {
    double t0;        // simulated time at the start of the step
    double dt;        // float64 step length (the reference's Python float dt)
    float dt_f;       // float32(dt): what the kernels multiply by
    float dtg_f;      // float32(dt * g): the Manning term's Python-float product
    float rain_f;     // float32(base rainfall rate at t0)
    float pad0;
    int32_t active;   // 0: the step is a no-op
    int32_t parity;   // state buffer holding the input state
    int32_t snap_slot;     // >= 0: the step's end state is snapshot slot k
    int32_t check_finite;  // check the input depth for non-finite values
    int32_t phases;
    int32_t pad1;
    int64_t step;     // index of this step (0-based)
};

// Run control: advanced only by the planner.
struct RunCtrl {
    double t;             // time at the start of the next step to plan
    double cached_dt;     // float64 of the last CFL minimum; < 0 before the first
    double next_snap_t;
    double final_t;
    double stop_t;        // fl_run pause target
    double max_dt, safety, snap_interval, g;
    double last_dt;
    int64_t step;         // steps planned (active)
    int64_t max_step;     // planner stops at this step count
    int64_t cfl_evals, cfl_reused;
    int64_t error_step;
    int32_t parity;       // buffer holding the latest state
    int32_t snap_count, max_snaps;
    int32_t error;        // sticky FL_E_* code (written with atomicCAS)
    int32_t cfl_interval, finite_interval;
    int32_t hyeto_n;
    int32_t pad;
};

struct HyetoView {
    const double *start_s, *end_s, *rate;
    int32_t n;
};

// Ledger slots of the per-warp running sums (float-float pairs).
constexpr int SURF_TERMS = 4;   // rain, infil, boundary in, boundary out
constexpr int VOL_BLOCKS = 304;  // blocks of the volume reduction (each writes one partial pair)
constexpr int D1_TERMS = 2;     // capture, surcharge
constexpr int D2_TERMS = 4;     // outfall, overflow, unreturned, link |transfer|

// ---------------------------------------------------------------------------
// Drainage layout.  Nodes are renumbered so that the nodes overflowing into
// one surface cell are consecutive ("groups", in cell order; nodes without a
// surface cell last).  Inlets are in cell order (q); each node lists its
// inlets (node order j) as in_qk[j] = {q, its cell, the cell's inlet range
// [q0, q1) in cell order}.  Each node lists its incident links as slots
// {link, meta}: meta = the other end node | NL_FROM if the node is the link's
// from-node | NL_TO if it is its to-node (a self-loop has both).
// ---------------------------------------------------------------------------
constexpr uint32_t NL_NODE_MASK = 0x3FFFFFFFu;
constexpr uint32_t NL_FROM = 1u << 30;
constexpr uint32_t NL_TO = 1u << 31;

// Ensemble members on one mesh: every per-member array is laid out member
// after member with these strides (elements); a batched drainage launch runs
// member blockIdx.y.  A single run has n = 1 and uses none of them.
struct MemberStrides {
    int32_t n;                    // members (the launch's gridDim.y)
    int64_t cells;                // state / wet: Cp
    int64_t nodes;                // Va, Vb, fac
    int64_t links;                // Q, T
    int64_t inlets;               // capsur
    int64_t led1, led2;           // drainage ledger slots
    int64_t snap_h, snap_v;       // snapshot arrays: max_snapshots x C, max_snapshots x N
};

// What k_nodes needs to evaluate the inlet requests of a node's inlets.
struct InletReqView {
    const int32_t *in_node;       // [I] cell order
    const float4 *in_par;         // [I] {bed - invert, capture capacity, surcharge capacity, node storage area}
    const float2 *Va;             // node volume (float-float) at the start of the drainage step
    int32_t rule;
    float coef_area;              // float32(Cd * A_orifice)
    float weir_coef_perim;        // float32(Cw * perimeter) for weir_orifice
    float g2;                     // 2 g (float32)
};

// External boundary inflow: one thread per receiver cell sums its receivers'
// depths for the step into add[cell], which the surface kernel adds after
// the clamp.
struct InflowArgs {
    const int32_t *cell;          // [U] receiver cells (new order)
    const int32_t *start;         // [U + 1] receivers of cell u: recv[start[u] .. start[u + 1])
    const int32_t *recv;          // receiver indices grouped by cell, ascending within a cell
    const double *times;          // [T] strictly increasing
    const float *q;               // [T * J] row-major
    float2 *led;                  // [J] float-float volume added by each receiver
    float *add;                   // [Cp] the step's added depth of receiver cells
    const float4 *cinfo;
    StepCtrl *ctrl;
    int32_t U, J, T;
};

struct SurfArgs {
    const float4 *cinfo;          // [Cp] {area, manning, flags, 1 / area}
    const int4 *tile_info;        // [tiles]
    const float4 *ent;            // entries {nx, ny, len, bits}
    const int32_t *halo_src;      // halo cells of each tile (padded to 4 per tile)
    const float4 *horton;         // [Cp] {f0, fc, k, rain multiplier} (kind 1)
    float *wet;                   // [Cp] wet time (kind 1)
    float4 *state0, *state1;      // [Cp] {h, hu, hv, bed}
    StepCtrl *ctrl;
    RunCtrl *run;
    HyetoView hy;
    float2 *ledger;               // [grid * 8 * SURF_TERMS] float-float running sums
    int32_t n_tiles;
    int32_t e_cap, h_cap;         // largest entry / padded halo count of a tile
    // dynamic shared memory layout (bytes): flux slots, barriers, two stages
    int32_t off_bar, off_stage, stage_bytes;
    int32_t so_ci, so_hz, so_wt, so_en, so_hs;  // offsets inside a stage (states at 0)
    float *snap_h, *snap_hu, *snap_hv;
    double *snap_t;
    int32_t C;
    int32_t forcing_kind;
    float infil_scalar;
    float g, half_g, md, vmax, stage;
    int32_t has_stage;
    const float *ext_add;         // [Cp] external inflow depth of receiver cells this step
};

// Local-inertial surface step (two launches: edge discharge, cell update with
// the donor limit factors).  Edges are renumbered by their first cell (new
// order).  The edge kernel writes each discharge into its cells' (cell, slot)
// places, so the cell kernel reads a cell's three discharges and static slot
// tables contiguously.
constexpr uint32_t LI_INTERIOR = 1u;  // the edge has a right cell
constexpr uint32_t LI_AI = 2u;        // active interior (both cells active)
constexpr uint32_t LI_BEDGE = 4u;     // routable boundary edge (left active, outflow / transmissive)
constexpr uint32_t LI_LACTIVE = 8u;
constexpr uint32_t LI_RACTIVE = 16u;
constexpr int LI_SLOTL_SHIFT = 8;     // bits 8-9: the edge's slot in its left cell
constexpr int LI_SLOTR_SHIFT = 10;    // bits 10-11: its slot in its right cell
// per-cell slot bits, 4 per slot k at bit 4k
constexpr uint32_t LIS_PRESENT = 1u;  // the slot has an edge
constexpr uint32_t LIS_LEFT = 2u;     // the cell is the edge's left cell
constexpr uint32_t LIS_AI = 4u;       // active interior edge
constexpr uint32_t LIS_INTERIOR = 8u; // the edge has a right cell

struct LiArgs {
    const int2 *e_lr;             // [E] {left, right or -1}
    const float4 *e_geo;          // [E] {nx, ny, length, flags | slots (bits)}
    const float2 *e_dm;           // [E] {face distance, face Manning n}
    const uint32_t *c_bits;       // [Cp] LIS_* of slot k at bit 4k
    const int4 *c_other;          // [Cp] the other cell of each slot's interior edge, -1 = none
    const float2 *c_nrm;          // [3 * Cp] slot-major: the normal of slot k's edge
    const float4 *cinfo;
    const float *char_len;
    const float4 *horton;         // kind 1
    float *wet;
    float4 *state0, *state1;
    float4 *Qs;                   // [Cp] the discharges of the cell's slot edges this step (w unused)
    StepCtrl *ctrl;
    RunCtrl *run;
    HyetoView hy;
    double *snap_t;
    float2 *ledger;               // [warps * SURF_TERMS] of the cell kernel
    float *snap_h, *snap_hu, *snap_hv;
    const float *ext_add;
    int32_t E, C;
    int32_t forcing_kind;
    float infil_scalar, g, md, vmax;
};

struct DtArgs {
    const float4 *state0, *state1;
    const float *char_len;
    StepCtrl *ctrl;
    RunCtrl *run;
    HyetoView hy;
    float *partial;               // [gridDim.x]
    unsigned int *counter;
    double *snap_t;
    int32_t C;
    float cfl, g, md;
    double *dt_out;               // optional: fl_stable_timestep result
    int32_t li;                   // local-inertial CFL (gravity-wave speed only)
};

// k_nodes: one thread per node, the inlet exchange of its volume.
struct NodeArgs {
    const int32_t *node_in_start; // [N + 1] inlet range (node order)
    const int4 *in_qk;            // [I] node order: {inlet in cell order, its cell, the cell's inlets [q0, q1)}
    InletReqView inl;             // inlet parameters
    const float4 *cinfo;
    const float4 *state0, *state1;  // the surface step's output holds the inlet cells' depth
    float2 *capsur;               // [I] cell order: granted {capture, surcharge}
    const float2 *Va;             // node volume before the exchange
    float2 *Vb;                   // after
    StepCtrl *ctrl;
    float2 *ledger;               // [warps * D1_TERMS] float-float running sums
    int32_t N;
    MemberStrides ms;
};

// k_links: one thread per link, its transfer volume from the end volumes.
struct LinkArgs {
    const int32_t *link_from, *link_to;
    const float4 *lk0, *lk1, *lk2;
    const float *node_area;
    const float2 *Vb;
    const float *Q0, *Q1;         // link flow, ping-pong with the state parity
    float *T;
    StepCtrl *ctrl;
    int32_t L;
    float g, wave_speed;
    MemberStrides ms;
};

// k_donor: one thread per node, its donor limit factor.
struct DonorArgs {
    const int32_t *node_link_start;  // [N + 1]
    const int2 *nl;               // link slots {link, meta}
    const float2 *Vb;
    const float *T;
    float *fac;
    StepCtrl *ctrl;
    int32_t N;
    MemberStrides ms;
};

// k_network: one thread per group (a surface cell with the nodes that overflow
// into it, or a node without a surface cell).
struct NetArgs {
    const int4 *grp;              // {cell or -1, inlet cell or -1, first node, end node}
    const int32_t *kcell_start;
    const float2 *capsur;         // cell order granted {capture, surcharge}
    const int32_t *node_link_start;
    const int2 *nl;
    const float *T, *fac;
    const float4 *nd0;            // {storage area, outfall head offset, Cd*A outfall, outfall capacity}
    const float *nd_capv;         // storage area * max(max depth, 0)
    const float4 *cinfo;
    float4 *state0, *state1;
    const float2 *Vb;             // after the inlet exchange
    float2 *Va;                   // final
    float *Q0, *Q1;
    float *wet;
    float *snap_h, *snap_v;
    StepCtrl *ctrl;
    float2 *ledger;               // [warps * D2_TERMS] float-float running sums
    int32_t G, C, N;
    int32_t forcing_kind;
    float g, md;
    int32_t has_recharge;         // recharge cells are finished by k_recharge
    // weighted surcharge-return table (table != 0): nodes with entries return
    // through it, the others fall back to their cell; float64 as the reference
    int32_t table;
    const int32_t *node_tstart;   // [N + 1] valid entries of each node, entry order
    const float *node_tw;         // their normalized weights
    double *ovf_node;             // [N] overflow of nodes with entries (for k_surcharge)
    const int32_t *tcell;         // [U] table cells (new order, ascending)
    double *s2;                   // [U] fallback return depth of table cells that are group cells
    int32_t U;
    MemberStrides ms;
};

// Weighted surcharge return into the table cells, after k_network:
// h = float32((h + sum over entries of overflow x weight / area) + fallback).
struct SurchargeArgs {
    const int32_t *cell;          // [U] table cells (new order)
    const int32_t *start;         // [U + 1]
    const int2 *ent;              // {node (new order), weight bits} in entry order per cell
    const double *ovf_node;
    const double *s2;
    const float4 *cinfo;
    float4 *state0, *state1;
    float *wet;
    float *snap_h;
    StepCtrl *ctrl;
    int32_t U, C;
    int32_t forcing_kind;
    float md;
    int32_t has_recharge;
};

// Surface recharge: one thread per recharge cell, its rows in table order.
struct RechargeArgs {
    const int32_t *cell;          // [U] recharge cells (new order)
    const int32_t *row_start;     // [U + 1] rows of cell u: rows[row_start[u] .. row_start[u + 1])
    const int32_t *rows;          // table rows grouped by cell, in table order within a cell
    const float4 *par;            // [R] {storage capacity, capture capacity, recharge capacity, stop depth}
    float *storage;               // [R] stored volume (table order)
    float2 *led;                  // [2R] float-float capture, recharge loss per row
    const float4 *cinfo;
    float4 *state0, *state1;
    float *wet;
    float *snap_h;
    StepCtrl *ctrl;
    int32_t U, C;
    int32_t forcing_kind;
    float md;
};

// Host-side renumbered layout (fl_plan.cpp).
struct HostLayout {
    int32_t C = 0, E = 0, N = 0, L = 0, I = 0, K = 0, G = 0;
    int32_t tile = TILE;              // cells per tile (multiple of 32, at most TILE)
    std::vector<int32_t> perm;        // perm[new] = reference cell
    std::vector<int32_t> inv;         // inv[reference] = new
    int32_t Cp = 0;                   // C rounded up to whole tiles
    std::vector<float4> cinfo;        // [Cp]
    std::vector<int32_t> inc;         // [C * 3] reference cell -> its edges in slot order (-1 none)
    // weighted surcharge-return table (empty without one)
    std::vector<int32_t> node_tstart; // [N + 1]
    std::vector<float> node_tw;
    std::vector<int32_t> tcell, tcell_start;
    std::vector<int2> tcell_ent;
    std::vector<int4> tile_info;
    std::vector<float4> ent;
    std::vector<int32_t> halo_src;
    int32_t e_cap = 0, h_cap = 0;
    std::vector<float> char_len;
    std::vector<float> bed;
    int64_t slots_used = 0;
    // drainage
    std::vector<int32_t> in_cell, in_node, in_kcell, in_order; // cell order; in_order[q] = reference inlet
    std::vector<int4> in_qk;          // node order: {inlet in cell order, its cell, the cell's inlets [q0, q1)}
    std::vector<float4> in_par;
    std::vector<int32_t> kcell_cell, kcell_start;
    std::vector<int32_t> node_in_start;
    std::vector<int32_t> node_perm, node_inv;  // node_perm[new] = reference node
    std::vector<int32_t> link_perm, link_inv;  // link_perm[new] = reference link
    std::vector<float> node_area, nd_capv;
    std::vector<float4> nd0;
    std::vector<int4> grp;
    std::vector<int32_t> node_link_start;
    std::vector<int2> nl;
    std::vector<int32_t> link_from, link_to;   // renumbered nodes
    std::vector<float4> lk0, lk1, lk2;
    int32_t max_inlets_per_cell = 0;
};

}  // namespace fl
