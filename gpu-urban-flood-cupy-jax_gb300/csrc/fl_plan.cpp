// Host-side layout builder: validates the reference-layout inputs, renumbers
// cells along a Hilbert curve of their centroids, builds each tile's edge
// entry list and the per-cell info words, and the CSR tables the drainage
// kernels gather over.  Pure C++ (no CUDA calls), so it also runs
// through fl_plan_check on machines without a GPU.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>

#include "../../include/floodgb.h"
#include "fl_internal.h"

namespace fl {

int set_error(int code, const char *fmt, ...);

namespace {

// Hilbert index of (x, y) on a 2^16 x 2^16 grid.
uint64_t hilbert_d(uint32_t x, uint32_t y) {
    const uint32_t n = 1u << 16;
    uint64_t d = 0;
    for (uint32_t s = n / 2; s > 0; s /= 2) {
        const uint32_t rx = (x & s) > 0;
        const uint32_t ry = (y & s) > 0;
        d += (uint64_t)s * (uint64_t)s * ((3 * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - x;
                y = s - 1 - y;
            }
            std::swap(x, y);
        }
    }
    return d;
}

float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

}  // namespace

// Bounds check of the tile tables against the buffers the surface kernel
// copies and indexes: every entry's local indices inside its tile's own cells
// plus halo, every halo cell a real cell, every copy 16-byte sized.
static int validate_tiles(const HostLayout &L) {
    const int64_t TL = L.tile, MAXH = 3 * L.tile;
    const int64_t tiles = (int64_t)L.tile_info.size();
    for (int64_t t = 0; t < tiles; ++t) {
        const int4 ti = L.tile_info[t];
        const int64_t own = std::min<int64_t>(TL, (int64_t)L.C - t * TL);
        if (ti.x < 0 || ti.y < 0 || (int64_t)ti.x + ti.y > (int64_t)L.ent.size() || ti.y > L.e_cap ||
            ti.z < 0 || ti.z % 4 != 0 || ti.w < 0 || ti.w > MAXH || (int64_t)ti.z + ((ti.w + 3) & ~3) > (int64_t)L.halo_src.size() ||
            ((ti.w + 3) & ~3) > L.h_cap)
            return set_error(FL_E_INVALID, "internal: tile %lld table out of range", (long long)t);
        for (int32_t j = 0; j < ti.w; ++j) {
            const int32_t g = L.halo_src[ti.z + j];
            if (g < 0 || g >= L.C || (g >= t * TL && g < t * TL + own))
                return set_error(FL_E_INVALID, "internal: tile %lld halo cell %d out of range", (long long)t, g);
        }
        for (int32_t j = 0; j < ti.y; ++j) {
            uint32_t bits;
            memcpy(&bits, &L.ent[ti.x + j].w, 4);
            const uint32_t li = bits & EB_IDX_MASK, ri = (bits >> EB_RIGHT_SHIFT) & EB_IDX_MASK;
            const bool lin = li < (uint32_t)own, rin = ri < (uint32_t)own;
            const bool lok = lin || (li >= (uint32_t)TL && li < (uint32_t)(TL + ti.w));
            const bool rok = !(bits & EB_AI) || rin || (ri >= (uint32_t)TL && ri < (uint32_t)(TL + ti.w));
            const uint32_t ls = (bits >> EB_LSLOT_SHIFT) & 3u, rs = (bits >> EB_RSLOT_SHIFT) & 3u;
            if (!lok || !rok || ((bits & EB_LPRESENT) && (!lin || ls > 2u)) ||
                ((bits & EB_RPRESENT) && (!(bits & EB_AI) || !rin || rs > 2u)))
                return set_error(FL_E_INVALID, "internal: tile %lld entry %d has an out-of-range cell index", (long long)t, j);
        }
    }
    return FL_OK;
}

int build_mesh_layout(const FlMeshDesc &m, const FlDrainDesc *d, HostLayout &L) {
    const int64_t C = m.cell_count, E = m.edge_count;
    if (C <= 0 || E <= 0) return set_error(FL_E_INVALID, "mesh needs cell_count > 0 and edge_count > 0");
    if (C > MAX_CELLS) return set_error(FL_E_INVALID, "mesh has %lld cells; the limit is %lld", (long long)C, (long long)MAX_CELLS);
    if (!m.bed_elevation_m || !m.manning_n || !m.cell_area_m2 || !m.characteristic_length_m || !m.edge_left_cell ||
        !m.edge_right_cell || !m.boundary_code || !m.edge_normal_x || !m.edge_normal_y || !m.edge_length_m)
        return set_error(FL_E_INVALID, "mesh descriptor has a NULL required array");
    L.C = (int32_t)C;
    L.E = (int32_t)E;
    std::vector<uint8_t> active(C, 1);
    if (m.active_mask) {
        for (int64_t c = 0; c < C; ++c) {
            const float a = m.active_mask[c];
            if (a != 0.0f && a != 1.0f)
                return set_error(FL_E_UNSUPPORTED, "active_mask must hold 0/1 values (cell %lld has %g)", (long long)c, (double)a);
            active[c] = a > 0.5f;
        }
    }
    // incidences: left ones (ascending edge), then right ones (ascending edge)
    std::vector<uint8_t> count(C, 0);
    std::vector<int32_t> inc(C * 3, -1);
    std::vector<uint8_t> inc_right(C * 3, 0);
    for (int pass = 0; pass < 2; ++pass) {
        for (int64_t e = 0; e < E; ++e) {
            const int32_t l = m.edge_left_cell[e], r = m.edge_right_cell[e];
            if (pass == 0) {
                if (l < 0 || l >= C) return set_error(FL_E_INVALID, "edge_left_cell[%lld] = %d is out of range", (long long)e, l);
                if (r < -1 || r >= C) return set_error(FL_E_INVALID, "edge_right_cell[%lld] = %d is out of range", (long long)e, r);
                if (r == l) return set_error(FL_E_INVALID, "edge %lld has the same left and right cell", (long long)e);
                const int32_t code = m.boundary_code[e];
                if (code < -1 || code > 4) return set_error(FL_E_INVALID, "Unsupported triangular boundary code %d on edge %lld.", code, (long long)e);
                if (!(m.edge_length_m[e] > 0.0f)) return set_error(FL_E_INVALID, "edge %lld has a non-positive length", (long long)e);
            }
            const int32_t c = pass == 0 ? l : r;
            if (c < 0) continue;
            if (count[c] >= 3)
                return set_error(FL_E_INVALID, "triangular topology contains a cell with more than three edges (cell %d)", c);
            inc[c * 3 + count[c]] = (int32_t)e;
            inc_right[c * 3 + count[c]] = (uint8_t)pass;
            count[c]++;
        }
    }
    for (int64_t c = 0; c < C; ++c) {
        if (!(m.cell_area_m2[c] > 0.0f)) return set_error(FL_E_INVALID, "cell %lld has a non-positive area", (long long)c);
    }
    L.inc = inc;

    // renumbering
    L.perm.resize(C);
    std::iota(L.perm.begin(), L.perm.end(), 0);
    if (m.centroid_x && m.centroid_y) {
        double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
        for (int64_t c = 0; c < C; ++c) {
            xmin = std::min(xmin, (double)m.centroid_x[c]);
            xmax = std::max(xmax, (double)m.centroid_x[c]);
            ymin = std::min(ymin, (double)m.centroid_y[c]);
            ymax = std::max(ymax, (double)m.centroid_y[c]);
        }
        const double span = std::max(std::max(xmax - xmin, ymax - ymin), 1e-9);
        std::vector<uint64_t> key(C);
        for (int64_t c = 0; c < C; ++c) {
            const double fx = (m.centroid_x[c] - xmin) / span, fy = (m.centroid_y[c] - ymin) / span;
            const uint32_t qx = (uint32_t)std::min(65535.0, std::max(0.0, fx * 65535.0));
            const uint32_t qy = (uint32_t)std::min(65535.0, std::max(0.0, fy * 65535.0));
            key[c] = hilbert_d(qx, qy);
        }
        std::stable_sort(L.perm.begin(), L.perm.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
    }
    L.inv.resize(C);
    for (int64_t i = 0; i < C; ++i) L.inv[L.perm[i]] = (int32_t)i;

    // coupled cells (drainage finishes their depth)
    std::vector<uint8_t> coupled(C, 0);
    if (d) {
        for (int32_t i = 0; i < d->inlet_count; ++i) {
            const int32_t c = d->inlet_cell_index[i];
            if (c >= 0 && c < C) coupled[c] = 1;
        }
        for (int32_t n = 0; n < d->node_count; ++n) {
            const int32_t c = d->node_surface_cell_index[n];
            if (c >= 0 && c < C) coupled[c] = 1;
        }
    }

    L.cinfo.resize(C);
    L.char_len.resize(C);
    L.bed.resize(C);
    L.slots_used = 0;
    // slot of each edge in its left / right cell
    std::vector<int8_t> lslot(E, -1), rslot(E, -1);
    for (int64_t c = 0; c < C; ++c) {
        for (int k = 0; k < count[c]; ++k) {
            const int32_t e = inc[c * 3 + k];
            if (inc_right[c * 3 + k]) rslot[e] = (int8_t)k; else lslot[e] = (int8_t)k;
            L.slots_used++;
        }
    }
    for (int64_t i = 0; i < C; ++i) {
        const int32_t c = L.perm[i];
        uint32_t info = 0;
        if (active[c]) info |= CELL_ACTIVE;
        if (coupled[c]) info |= CELL_COUPLED;
        for (int k = 0; k < count[c]; ++k)
            if (inc_right[c * 3 + k]) info |= 1u << (CELL_RIGHT_SHIFT + k);
        float fi;
        memcpy(&fi, &info, 4);
        L.cinfo[i] = f4(m.cell_area_m2[c], m.manning_n[c], fi, 1.0f / m.cell_area_m2[c]);
        L.char_len[i] = m.characteristic_length_m[c];
        L.bed[i] = m.bed_elevation_m[c];
    }

    // tile entry lists and halos
    const int64_t TL = L.tile, MAXH = 3 * L.tile;
    if (TL < 32 || TL > TILE || TL % 32 != 0) return set_error(FL_E_INVALID, "tile size %lld is not a multiple of 32 in [32, %d]", (long long)TL, TILE);
    const int64_t tiles = (C + TL - 1) / TL;
    L.Cp = (int32_t)(tiles * TL);
    {
        uint32_t none = 0;
        float fz;
        memcpy(&fz, &none, 4);
        L.cinfo.resize((size_t)L.Cp, f4(1.0f, 0.0f, fz, 1.0f));  // padding cells: inactive, never referenced
    }
    L.tile_info.assign((size_t)tiles, make_int4(0, 0, 0, 0));
    L.ent.clear();
    L.halo_src.clear();
    L.ent.reserve((size_t)(C * 17 / 10));
    L.e_cap = 0;
    L.h_cap = 0;
    std::vector<int32_t> entry_of(E, -1);  // entry of edge e in the current tile
    std::vector<int64_t> entry_tile(E, -1);
    std::vector<int32_t> ent_left, ent_right;  // global (renumbered) cells of the tile's entries
    std::vector<uint32_t> ent_bits;
    std::vector<int32_t> halo;
    for (int64_t t = 0; t < tiles; ++t) {
        const int64_t c0 = t * TL, c1 = std::min<int64_t>(C, c0 + TL);
        const size_t first = L.ent.size();
        ent_left.clear();
        ent_right.clear();
        ent_bits.clear();
        for (int64_t i = c0; i < c1; ++i) {
            const int32_t c = L.perm[i];
            for (int k = 0; k < count[c]; ++k) {
                const int32_t e = inc[c * 3 + k];
                const bool is_right = inc_right[c * 3 + k] != 0;
                const int32_t lref = m.edge_left_cell[e], rref = m.edge_right_cell[e];
                const bool interior = rref >= 0;
                const bool la = active[lref] != 0;
                const bool ra = interior ? active[rref] != 0 : la;
                const bool ai = interior && la && ra;
                const int32_t raw = m.boundary_code[e];
                const int32_t code = (interior && la && !ra) ? 0 : raw;
                // does this side take a contribution?
                bool contributes;
                if (is_right) contributes = ai;
                else contributes = la || (!interior && code == 3 && m.has_stage_boundary);
                if (!contributes) continue;
                int32_t idx = entry_tile[e] == t ? entry_of[e] : -1;
                if (idx < 0) {
                    idx = (int32_t)ent_bits.size();
                    entry_of[e] = idx;
                    entry_tile[e] = t;
                    uint32_t bits = 0;
                    if (la) bits |= EB_LACTIVE;
                    if (ai) bits |= EB_AI;
                    if (interior) bits |= EB_INTERIOR;
                    bits |= (uint32_t)(code + 1) << EB_CODE_SHIFT;
                    ent_bits.push_back(bits);
                    ent_left.push_back(L.inv[lref]);
                    ent_right.push_back(ai ? L.inv[rref] : -1);  // the right state is read only on active interior edges
                    L.ent.push_back(f4(m.edge_normal_x[e], m.edge_normal_y[e], m.edge_length_m[e], 0.0f));
                }
                if (is_right) ent_bits[idx] |= EB_RPRESENT | ((uint32_t)rslot[e] << EB_RSLOT_SHIFT);
                else ent_bits[idx] |= EB_LPRESENT | ((uint32_t)lslot[e] << EB_LSLOT_SHIFT);
            }
        }
        // entries grouped by kind so a warp's entries take the same path:
        // active interior with both cells in the tile, active interior with
        // one, then boundary / inactive-neighbour entries (stable; the order
        // does not change any cell's result: each entry writes its own
        // (cell, slot) places and a cell sums its slots in slot order)
        {
            const size_t n = ent_bits.size();
            auto kind = [&](size_t j) {
                const uint32_t b = ent_bits[j];
                if (!(b & EB_AI)) return 2;
                return ((b & EB_LPRESENT) && (b & EB_RPRESENT)) ? 0 : 1;
            };
            std::vector<size_t> order(n);
            std::iota(order.begin(), order.end(), (size_t)0);
            std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return kind(x) < kind(y); });
            std::vector<int32_t> nl(n), nr(n);
            std::vector<uint32_t> nb(n);
            std::vector<float4> ne(n);
            for (size_t k = 0; k < n; ++k) {
                nl[k] = ent_left[order[k]];
                nr[k] = ent_right[order[k]];
                nb[k] = ent_bits[order[k]];
                ne[k] = L.ent[first + order[k]];
            }
            ent_left.swap(nl);
            ent_right.swap(nr);
            ent_bits.swap(nb);
            std::copy(ne.begin(), ne.end(), L.ent.begin() + (std::ptrdiff_t)first);
        }
        // halo: cells outside the tile that an entry reads, ascending
        halo.clear();
        for (size_t j = 0; j < ent_bits.size(); ++j) {
            if (ent_left[j] < c0 || ent_left[j] >= c1) halo.push_back(ent_left[j]);
            if (ent_right[j] >= 0 && (ent_right[j] < c0 || ent_right[j] >= c1)) halo.push_back(ent_right[j]);
        }
        std::sort(halo.begin(), halo.end());
        halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
        if ((int64_t)halo.size() > MAXH)
            return set_error(FL_E_INVALID, "tile %lld reads %zu outside cells (limit %lld)", (long long)t, halo.size(), (long long)MAXH);
        auto local = [&](int32_t g) -> uint32_t {
            if (g >= c0 && g < c1) return (uint32_t)(g - c0);
            return (uint32_t)(TL + (std::lower_bound(halo.begin(), halo.end(), g) - halo.begin()));
        };
        for (size_t j = 0; j < ent_bits.size(); ++j) {
            uint32_t bits = ent_bits[j] | local(ent_left[j]);
            if (ent_right[j] >= 0) bits |= local(ent_right[j]) << EB_RIGHT_SHIFT;
            memcpy(&L.ent[first + j].w, &bits, 4);
        }
        const int32_t hstart = (int32_t)L.halo_src.size();
        L.halo_src.insert(L.halo_src.end(), halo.begin(), halo.end());
        while (L.halo_src.size() % 4) L.halo_src.push_back(halo.empty() ? 0 : halo.back());
        const int32_t hpad = (int32_t)L.halo_src.size() - hstart;
        L.tile_info[t] = make_int4((int32_t)first, (int32_t)ent_bits.size(), hstart, (int32_t)halo.size());
        L.e_cap = std::max(L.e_cap, (int32_t)ent_bits.size());
        L.h_cap = std::max(L.h_cap, hpad);
        if (L.ent.size() > (size_t)INT32_MAX) return set_error(FL_E_INVALID, "mesh has too many edge entries");
    }
    return validate_tiles(L);
}

// Dynamic shared memory of k_surface for the layout's largest tile: the
// per-(cell, slot) flux places, two mbarriers + two tile records, and two
// stages of {own + halo states, cell info, [Horton, wet time], entries, halo
// list}.  Returns the total bytes and fills the offsets in `a`.
int surface_smem_layout(SurfArgs &a, int kind) {
    auto up = [](int x, int m) { return (x + m - 1) / m * m; };
    const int flux = TILE * 3 * 16;
    a.off_bar = flux;
    a.off_stage = up(flux + 128, 128);  // barriers (6 x 8 B) and the two tile records (2 x 16 B)
    int o = (TILE + a.h_cap) * 16;
    a.so_ci = o;
    o += TILE * 16;
    a.so_hz = o;
    if (kind) o += TILE * 16;
    a.so_wt = o;
    if (kind) o += TILE * 4;
    a.so_en = o;
    o += a.e_cap * 16;
    a.so_hs = o;
    o += a.h_cap * 4;
    a.stage_bytes = up(o, 128);
    return a.off_stage + 2 * a.stage_bytes;
}

// Bounds check of the drainage tables against the arrays the kernels index.
static int validate_drain(const HostLayout &L) {
    const int32_t N = L.N, I = L.I, K = L.K, NL = L.L, C = L.C;
    if ((int32_t)L.node_in_start.size() != N + 1 || L.node_in_start[0] != 0 || L.node_in_start[N] != I ||
        (int32_t)L.node_link_start.size() != N + 1 || L.node_link_start[0] != 0 ||
        L.node_link_start[N] != (int32_t)L.nl.size() || (int32_t)L.kcell_start.size() != K + 1 ||
        L.kcell_start[0] != 0 || L.kcell_start[K] != I)
        return set_error(FL_E_INVALID, "internal: drainage table sizes");
    for (int32_t n = 0; n < N; ++n)
        if (L.node_in_start[n + 1] < L.node_in_start[n] || L.node_link_start[n + 1] < L.node_link_start[n])
            return set_error(FL_E_INVALID, "internal: drainage CSR not monotone at node %d", n);
    for (int32_t k = 0; k < K; ++k)
        if (L.kcell_start[k + 1] <= L.kcell_start[k] || L.kcell_cell[k] < 0 || L.kcell_cell[k] >= C)
            return set_error(FL_E_INVALID, "internal: inlet cell %d", k);
    for (int32_t q = 0; q < I; ++q)
        if (L.in_node[q] < 0 || L.in_node[q] >= N || L.in_kcell[q] < 0 || L.in_kcell[q] >= K)
            return set_error(FL_E_INVALID, "internal: inlet %d tables", q);
    for (int32_t n = 0; n < N; ++n)
        for (int32_t j = L.node_in_start[n]; j < L.node_in_start[n + 1]; ++j)
            if (L.in_qk[j].x < 0 || L.in_qk[j].x >= I || L.in_node[L.in_qk[j].x] != n ||
                L.in_qk[j].y != L.kcell_cell[L.in_kcell[L.in_qk[j].x]] || L.in_qk[j].z != L.kcell_start[L.in_kcell[L.in_qk[j].x]] ||
                L.in_qk[j].w != L.kcell_start[L.in_kcell[L.in_qk[j].x] + 1])
                return set_error(FL_E_INVALID, "internal: node %d inlet list", n);
    for (const int2 &e : L.nl)
        if (e.x < 0 || e.x >= NL || (int32_t)((uint32_t)e.y & NL_NODE_MASK) >= N || !((uint32_t)e.y & (NL_FROM | NL_TO)))
            return set_error(FL_E_INVALID, "internal: link slot out of range");
    int32_t prev = 0;
    for (const int4 &g : L.grp) {
        if (g.x < -1 || g.x >= C || g.y < -1 || g.y >= K || g.z != prev || g.w < g.z || g.w > N)
            return set_error(FL_E_INVALID, "internal: drainage group out of range");
        prev = g.w;
    }
    if (prev != N) return set_error(FL_E_INVALID, "internal: drainage groups do not cover the nodes");
    if (!L.node_tstart.empty()) {
        const int32_t U = (int32_t)L.tcell.size();
        if ((int32_t)L.node_tstart.size() != N + 1 || L.node_tstart[0] != 0 ||
            L.node_tstart[N] != (int32_t)L.node_tw.size() || (int32_t)L.tcell_start.size() != U + 1 ||
            L.tcell_start[0] != 0 || L.tcell_start[U] != (int32_t)L.tcell_ent.size() ||
            L.tcell_ent.size() != L.node_tw.size())
            return set_error(FL_E_INVALID, "internal: surcharge table sizes");
        for (int32_t n = 0; n < N; ++n)
            if (L.node_tstart[n + 1] < L.node_tstart[n]) return set_error(FL_E_INVALID, "internal: surcharge CSR");
        for (int32_t u = 0; u < U; ++u)
            if (L.tcell[u] < 0 || L.tcell[u] >= C || (u > 0 && L.tcell[u] <= L.tcell[u - 1]) ||
                L.tcell_start[u + 1] <= L.tcell_start[u])
                return set_error(FL_E_INVALID, "internal: surcharge cell %d", u);
        for (const int2 &e : L.tcell_ent)
            if (e.x < 0 || e.x >= N) return set_error(FL_E_INVALID, "internal: surcharge entry node");
    }
    return FL_OK;
}

int build_drain_layout(const FlMeshDesc &m, const FlDrainDesc &d, HostLayout &L) {
    const int32_t N = d.node_count, NL = d.link_count, I = d.inlet_count, C = L.C;
    if (N < 0 || NL < 0 || I < 0) return set_error(FL_E_INVALID, "negative drainage counts");
    if (N == 0 && (NL > 0 || I > 0)) return set_error(FL_E_INVALID, "links or inlets need nodes");
    L.N = N;
    L.L = NL;
    L.I = I;
    if (N == 0) return FL_OK;
    if (!d.node_surface_cell_index || !d.node_invert_elevation_m || !d.node_storage_area_m2 || !d.node_max_depth_m)
        return set_error(FL_E_INVALID, "drainage descriptor has a NULL required node array");
    if (I > 0 && (!d.inlet_cell_index || !d.inlet_node_index))
        return set_error(FL_E_INVALID, "drainage descriptor has a NULL inlet index array");
    if (NL > 0 && (!d.link_from_node_index || !d.link_to_node_index || !d.link_length_m || !d.link_area_m2 ||
                   !d.link_hydraulic_radius_m || !d.link_manning_n))
        return set_error(FL_E_INVALID, "drainage descriptor has a NULL required link array");
    if (d.inlet_capture_rule < 0 || d.inlet_capture_rule > 3)
        return set_error(FL_E_INVALID, "inlet_capture_rule must be 'orifice', 'weir_orifice', 'capacity', or 'head_limited_capacity'.");
    for (int32_t n = 0; n < N; ++n) {
        const int32_t c = d.node_surface_cell_index[n];
        if (c >= C) return set_error(FL_E_INVALID, "node_surface_cell_index[%d] = %d is out of range", n, c);
    }
    const float INF = std::numeric_limits<float>::infinity();

    if ((uint32_t)N > NL_NODE_MASK) return set_error(FL_E_INVALID, "too many drainage nodes");
    // drainage groups: each coupled cell (a cell with inlets or with nodes that
    // overflow into it) with its nodes, in cell order, then the nodes without a
    // surface cell.  Nodes are renumbered in group order.
    for (int32_t i = 0; i < I; ++i) {
        const int32_t c = d.inlet_cell_index[i], n = d.inlet_node_index[i];
        if (c < 0 || c >= C) return set_error(FL_E_INVALID, "inlet_cell_index[%d] = %d is out of range", i, c);
        if (n < 0 || n >= N) return set_error(FL_E_INVALID, "inlet_node_index[%d] = %d is out of range", i, n);
    }
    std::vector<int32_t> node_cell_new(N, -1);
    for (int32_t n = 0; n < N; ++n) {
        const int32_t c = d.node_surface_cell_index[n];
        node_cell_new[n] = c >= 0 ? L.inv[c] : -1;
    }
    L.node_perm.resize(N);
    std::iota(L.node_perm.begin(), L.node_perm.end(), 0);
    std::stable_sort(L.node_perm.begin(), L.node_perm.end(), [&](int32_t a, int32_t b) {
        const int32_t ca = node_cell_new[a] < 0 ? std::numeric_limits<int32_t>::max() : node_cell_new[a];
        const int32_t cb = node_cell_new[b] < 0 ? std::numeric_limits<int32_t>::max() : node_cell_new[b];
        return ca < cb;
    });
    L.node_inv.assign(N, 0);
    for (int32_t k = 0; k < N; ++k) L.node_inv[L.node_perm[k]] = k;

    // inlets in cell order (stable in reference order)
    std::vector<int32_t> order(I);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return L.inv[d.inlet_cell_index[a]] < L.inv[d.inlet_cell_index[b]];
    });
    L.in_order = order;
    L.in_cell.resize(I);
    L.in_node.resize(I);
    L.in_kcell.resize(I);
    L.in_par.resize(I);
    L.kcell_cell.clear();
    L.kcell_start.clear();
    L.max_inlets_per_cell = 0;
    for (int32_t q = 0; q < I; ++q) {
        const int32_t i = order[q];
        const int32_t cref = d.inlet_cell_index[i], nref = d.inlet_node_index[i];
        const int32_t c = L.inv[cref];
        if (L.kcell_cell.empty() || L.kcell_cell.back() != c) {
            L.kcell_cell.push_back(c);
            L.kcell_start.push_back(q);
        }
        L.in_cell[q] = c;
        L.in_node[q] = L.node_inv[nref];
        L.in_kcell[q] = (int32_t)L.kcell_cell.size() - 1;
        const double off = (double)m.bed_elevation_m[cref] - (double)d.node_invert_elevation_m[nref];
        const float capc = d.inlet_capture_capacity_m3ps ? std::max(d.inlet_capture_capacity_m3ps[i], 0.0f) : INF;
        const float surc = d.inlet_surcharge_capacity_m3ps ? std::max(d.inlet_surcharge_capacity_m3ps[i], 0.0f) : INF;
        L.in_par[q] = f4((float)off, capc, surc, d.node_storage_area_m2[nref]);
    }
    L.kcell_start.push_back(I);
    L.K = (int32_t)L.kcell_cell.size();
    for (int32_t k = 0; k < L.K; ++k)
        L.max_inlets_per_cell = std::max(L.max_inlets_per_cell, L.kcell_start[k + 1] - L.kcell_start[k]);

    // inlets in node order (stable in cell order)
    L.node_in_start.assign(N + 1, 0);
    for (int32_t q = 0; q < I; ++q) L.node_in_start[L.in_node[q] + 1]++;
    for (int32_t n = 0; n < N; ++n) L.node_in_start[n + 1] += L.node_in_start[n];
    L.in_qk.assign(I, make_int4(0, 0, 0, 0));
    {
        std::vector<int32_t> fill(L.node_in_start.begin(), L.node_in_start.end() - 1);
        for (int32_t q = 0; q < I; ++q) {
            const int32_t k = L.in_kcell[q];
            L.in_qk[fill[L.in_node[q]]++] = make_int4(q, L.in_cell[q], L.kcell_start[k], L.kcell_start[k + 1]);
        }
    }

    // node parameters (renumbered)
    const bool has_outfall = d.outfall_area_m2 && d.outfall_coefficient && d.outfall_tailwater_head_m;
    L.node_area.resize(N);
    L.nd0.resize(N);
    L.nd_capv.resize(N);
    for (int32_t k = 0; k < N; ++k) {
        const int32_t n = L.node_perm[k];
        const float A = d.node_storage_area_m2[n];
        L.node_area[k] = A;
        float off = 0.0f, ca = 0.0f, cap = INF;
        if (has_outfall) {
            off = (float)((double)d.node_invert_elevation_m[n] - (double)d.outfall_tailwater_head_m[n]);
            ca = d.outfall_coefficient[n] * d.outfall_area_m2[n];
            if (d.outfall_flow_capacity_m3ps) cap = std::max(d.outfall_flow_capacity_m3ps[n], 0.0f);
        }
        L.nd0[k] = f4(A, off, ca, cap);
        L.nd_capv[k] = (float)((double)A * (double)std::max(d.node_max_depth_m[n], 0.0f));
    }

    // groups over the renumbered nodes
    L.grp.clear();
    int32_t ni = 0;  // next renumbered node
    size_t ki = 0;   // cursor into kcell_cell (sorted)
    while (true) {
        const int32_t next_node_cell = ni < N && node_cell_new[L.node_perm[ni]] >= 0 ? node_cell_new[L.node_perm[ni]]
                                                                                      : std::numeric_limits<int32_t>::max();
        const int32_t next_k_cell = ki < L.kcell_cell.size() ? L.kcell_cell[ki] : std::numeric_limits<int32_t>::max();
        const int32_t c = std::min(next_node_cell, next_k_cell);
        if (c == std::numeric_limits<int32_t>::max()) break;
        const int32_t kc = next_k_cell == c ? (int32_t)ki : -1;
        if (next_k_cell == c) ++ki;
        const int32_t first = ni;
        while (ni < N && node_cell_new[L.node_perm[ni]] == c) ++ni;
        L.grp.push_back(make_int4(c, kc, first, ni));
    }
    for (; ni < N; ++ni) L.grp.push_back(make_int4(-1, -1, ni, ni + 1));  // nodes without a surface cell
    L.G = (int32_t)L.grp.size();

    // links in the order of their renumbered (from, to) nodes, so a node's
    // links and a link's end nodes lie close together; each node's slot list
    // keeps the reference link order, so every per-node sum runs in the same
    // order as with links in reference order
    L.link_from.resize(NL);
    L.link_to.resize(NL);
    L.lk0.resize(NL);
    L.lk1.resize(NL);
    L.lk2.resize(NL);
    L.node_link_start.assign(N + 1, 0);
    std::vector<int32_t> lfn(NL), ltn(NL);
    for (int32_t l = 0; l < NL; ++l) {
        const int32_t f = d.link_from_node_index[l], t = d.link_to_node_index[l];
        if (f < 0 || f >= N || t < 0 || t >= N)
            return set_error(FL_E_INVALID, "link %d has a node index out of range", l);
        lfn[l] = L.node_inv[f];
        ltn[l] = L.node_inv[t];
    }
    L.link_perm.resize(NL);
    std::iota(L.link_perm.begin(), L.link_perm.end(), 0);
    std::stable_sort(L.link_perm.begin(), L.link_perm.end(), [&](int32_t a, int32_t b) {
        return lfn[a] != lfn[b] ? lfn[a] < lfn[b] : ltn[a] < ltn[b];
    });
    L.link_inv.assign(NL, 0);
    for (int32_t k = 0; k < NL; ++k) L.link_inv[L.link_perm[k]] = k;
    const bool rect = d.link_geometry_code && d.link_rect_width_m && d.link_rect_height_m;
    for (int32_t k = 0; k < NL; ++k) {
        const int32_t l = L.link_perm[k];
        const int32_t f = d.link_from_node_index[l], t = d.link_to_node_index[l];
        const int32_t fn = lfn[l], tn = ltn[l];
        L.link_from[k] = fn;
        L.link_to[k] = tn;
        const double invf = d.node_invert_elevation_m[f], invt = d.node_invert_elevation_m[t];
        const double inv = d.link_invert_elevation_m ? (double)d.link_invert_elevation_m[l] : std::min(invf, invt);
        L.lk0[k] = f4(d.link_length_m[l], (float)(invf - invt), (float)(0.5 * (invf + invt) - inv),
                      std::max(d.link_manning_n[l], 0.0f));
        const float km = d.link_minor_loss_coefficient ? std::max(d.link_minor_loss_coefficient[l], 0.0f) : 0.0f;
        L.lk1[k] = f4(d.link_diameter_m ? d.link_diameter_m[l] : 0.0f, d.link_area_m2[l], d.link_hydraulic_radius_m[l], km);
        int flags = 0;
        if (d.link_diameter_m) flags |= 1;
        float W = 0.0f, H = 0.0f;
        if (rect && d.link_geometry_code[l] == 2) {
            flags |= 2;
            W = d.link_rect_width_m[l];
            H = d.link_rect_height_m[l];
        }
        const float capq = d.link_flow_capacity_m3ps ? std::max(d.link_flow_capacity_m3ps[l], 0.0f) : INF;
        L.lk2[k] = f4(capq, W, H, (float)flags);
        L.node_link_start[fn + 1]++;
        if (tn != fn) L.node_link_start[tn + 1]++;
    }
    for (int32_t n = 0; n < N; ++n) L.node_link_start[n + 1] += L.node_link_start[n];
    L.nl.assign(L.node_link_start[N], make_int2(0, 0));
    {
        std::vector<int32_t> fill(L.node_link_start.begin(), L.node_link_start.end() - 1);
        for (int32_t l = 0; l < NL; ++l) {  // reference link order in every node's list
            const int32_t k = L.link_inv[l];
            const int32_t f = L.link_from[k], t = L.link_to[k];
            if (t == f) {
                L.nl[fill[f]++] = make_int2(k, (int32_t)((uint32_t)f | NL_FROM | NL_TO));
            } else {
                L.nl[fill[f]++] = make_int2(k, (int32_t)((uint32_t)t | NL_FROM));
                L.nl[fill[t]++] = make_int2(k, (int32_t)((uint32_t)f | NL_TO));
            }
        }
    }
    // weighted surcharge-return table: normalized weights (float32, the
    // per-node sum in entry order), each node's valid entries and each table
    // cell's entries, both in entry order
    L.node_tstart.clear();
    L.node_tw.clear();
    L.tcell.clear();
    L.tcell_start.clear();
    L.tcell_ent.clear();
    const int32_t E = d.surcharge_entry_count;
    if (E < 0) return set_error(FL_E_INVALID, "surcharge_entry_count must be >= 0");
    if (E > 0) {
        if (!d.surcharge_cell_index || !d.surcharge_node_index || !d.surcharge_return_weight)
            return set_error(FL_E_INVALID, "the surcharge table needs cell, node and weight arrays");
        std::vector<float> wsum(N, 0.0f), w(E, 0.0f);
        std::vector<uint8_t> valid(E, 0);
        for (int32_t e = 0; e < E; ++e) {
            const int32_t n = d.surcharge_node_index[e], c = d.surcharge_cell_index[e];
            if (n >= N || c >= C) return set_error(FL_E_INVALID, "surcharge entry %d is out of range", e);
            valid[e] = n >= 0 && c >= 0;
            if (valid[e]) {
                w[e] = std::max(d.surcharge_return_weight[e], 0.0f);
                wsum[n] += w[e];
            }
        }
        if (!d.surcharge_return_weight_is_normalized)
            for (int32_t e = 0; e < E; ++e)
                if (valid[e]) w[e] = w[e] / std::max(wsum[d.surcharge_node_index[e]], 1.0e-12f);
        L.node_tstart.assign(N + 1, 0);
        for (int32_t e = 0; e < E; ++e)
            if (valid[e]) L.node_tstart[L.node_inv[d.surcharge_node_index[e]] + 1]++;
        for (int32_t n = 0; n < N; ++n) L.node_tstart[n + 1] += L.node_tstart[n];
        L.node_tw.assign(L.node_tstart[N], 0.0f);
        std::vector<int32_t> fill(L.node_tstart.begin(), L.node_tstart.end() - 1);
        std::vector<std::pair<int32_t, int32_t>> byc;  // (cell new, entry)
        for (int32_t e = 0; e < E; ++e) {
            if (!valid[e]) continue;
            L.node_tw[fill[L.node_inv[d.surcharge_node_index[e]]]++] = w[e];
            byc.push_back({L.inv[d.surcharge_cell_index[e]], e});
        }
        std::sort(byc.begin(), byc.end());
        for (size_t k = 0; k < byc.size(); ++k) {
            const int32_t c = byc[k].first, e = byc[k].second;
            if (L.tcell.empty() || L.tcell.back() != c) {
                L.tcell.push_back(c);
                L.tcell_start.push_back((int32_t)k);
                uint32_t f;
                memcpy(&f, &L.cinfo[c].z, 4);
                f |= CELL_COUPLED | CELL_SURCHARGE;
                memcpy(&L.cinfo[c].z, &f, 4);
            }
            int32_t wb;
            memcpy(&wb, &w[e], 4);
            L.tcell_ent.push_back(make_int2(L.node_inv[d.surcharge_node_index[e]], wb));
        }
        L.tcell_start.push_back((int32_t)byc.size());
    }
    return validate_drain(L);
}

}  // namespace fl
