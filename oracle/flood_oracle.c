/*
 * CPU oracle for the flood step -- TEST INFRASTRUCTURE ONLY (see flood_oracle.h).
 * Compiled with -ffp-contract=off so float32 expressions round exactly as the
 * reference's NumPy/CuPy elementwise operations do.
 */
#include "flood_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline float fmax32(float a, float b) { return a >= b ? a : b; }
static inline float fmin32(float a, float b) { return a <= b ? a : b; }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* HLL normal flux, equations.py:20-81 (hll_shallow_water_normal_flux). */
static void hll_flux(float h_left, float hu_left, float hv_left, float h_right, float hu_right,
                     float hv_right, float nx, float ny, float g, float half_g, float md,
                     float *fh, float *fhu, float *fhv) {
    float h_l = fmax32(h_left, 0.0f), h_r = fmax32(h_right, 0.0f);
    int wet_l = h_l > md, wet_r = h_r > md;
    float u_l = wet_l ? hu_left / fmax32(h_l, md) : 0.0f;
    float v_l = wet_l ? hv_left / fmax32(h_l, md) : 0.0f;
    float u_r = wet_r ? hu_right / fmax32(h_r, md) : 0.0f;
    float v_r = wet_r ? hv_right / fmax32(h_r, md) : 0.0f;
    float un_l = u_l * nx + v_l * ny;
    float un_r = u_r * nx + v_r * ny;
    float c_l = sqrtf(g * h_l), c_r = sqrtf(g * h_r);
    float p_l = half_g * h_l * h_l, p_r = half_g * h_r * h_r;
    float fhl = h_l * un_l, fhul = hu_left * un_l + p_l * nx, fhvl = hv_left * un_l + p_l * ny;
    float fhr = h_r * un_r, fhur = hu_right * un_r + p_r * nx, fhvr = hv_right * un_r + p_r * ny;
    float sl = fmin32(un_l - c_l, un_r - c_r);
    float sr = fmax32(un_l + c_l, un_r + c_r);
    float denom = (fabsf(sr - sl) > 1.0e-12f) ? (sr - sl) : 1.0f;
    float hh = (sr * fhl - sl * fhr + sl * sr * (h_r - h_l)) / denom;
    float hhu = (sr * fhul - sl * fhur + sl * sr * (hu_right - hu_left)) / denom;
    float hhv = (sr * fhvl - sl * fhvr + sl * sr * (hv_right - hv_left)) / denom;
    float a, b, c;
    if (sl >= 0.0f) { a = fhl; b = fhul; c = fhvl; }
    else if (sr <= 0.0f) { a = fhr; b = fhur; c = fhvr; }
    else { a = hh; b = hhu; c = hhv; }
    if (!(wet_l || wet_r)) { a = 0.0f; b = 0.0f; c = 0.0f; }
    *fh = a; *fhu = b; *fhv = c;
}

/* Per-edge fluxes of _advance_triangular_swe (triangular_backend.py:1067-1150):
 * masked states, ghost right state, hydrostatic reconstruction pair,
 * outflow-only inflow block.  fl/fr hold the left and right flux triples. */
static void edge_flux(const OrcMesh *m, const float *h, const float *hu, const float *hv, int e,
                      float g, float half_g, float md, float *fl, float *fr, int *active_interior,
                      int *interior_out) {
    int left = m->left[e], right = m->right[e];
    int interior = right >= 0;
    int safe_right = interior ? right : left;
    int la = 1, ra = 1;
    if (m->active) { la = m->active[left] > 0.5f; ra = m->active[safe_right] > 0.5f; }
    int ai = interior && la && ra;
    int inactive_right_boundary = interior && la && !ra;
    float hL = la ? h[left] : 0.0f, huL = la ? hu[left] : 0.0f, hvL = la ? hv[left] : 0.0f;
    float zL = m->bed[left];
    float hRb = ra ? h[safe_right] : 0.0f, huRb = ra ? hu[safe_right] : 0.0f;
    float hvRb = ra ? hv[safe_right] : 0.0f, zRb = m->bed[safe_right];
    int code = inactive_right_boundary ? 0 : m->bcode[e];
    float nx = m->nx[e], ny = m->ny[e];

    /* _right_edge_state (:1294-1327) */
    float nm = huL * nx + hvL * ny;
    float hu_ref = huL - 2.0f * nm * nx;
    float hv_ref = hvL - 2.0f * nm * ny;
    float stage = m->has_stage ? m->stage : 0.0f;
    float h_stage = fmax32(stage - zL, 0.0f);
    int reflective = code == 0 || code == 2;
    int stage_b = code == 3;
    float hb = stage_b ? h_stage : hL;
    float hub = stage_b ? 0.0f : (reflective ? hu_ref : huL);
    float hvb = stage_b ? 0.0f : (reflective ? hv_ref : hvL);
    float hR = ai ? hRb : hb, huR = ai ? huRb : hub, hvR = ai ? hvRb : hvb;
    float zR = ai ? zRb : zL;

    /* hydrostatic_reconstruction_flux_pair (equations.py:84-152) */
    float h_l = fmax32(hL, 0.0f), h_r = fmax32(hR, 0.0f);
    float eta_l = h_l + zL, eta_r = h_r + zR;
    float zs = fmax32(zL, zR);
    float hls = fmax32(eta_l - zs, 0.0f), hrs = fmax32(eta_r - zs, 0.0f);
    int wl = h_l > md, wr = h_r > md;
    float u_l = wl ? huL / fmax32(h_l, md) : 0.0f;
    float v_l = wl ? hvL / fmax32(h_l, md) : 0.0f;
    float u_r = wr ? huR / fmax32(h_r, md) : 0.0f;
    float v_r = wr ? hvR / fmax32(h_r, md) : 0.0f;
    float fh, fhu, fhv;
    hll_flux(hls, u_l * hls, v_l * hls, hrs, u_r * hrs, v_r * hrs, nx, ny, g, half_g, md, &fh, &fhu, &fhv);
    float pcl = half_g * (h_l * h_l - hls * hls);
    float pcr = half_g * (h_r * h_r - hrs * hrs);
    fl[0] = fh; fl[1] = fhu + pcl * nx; fl[2] = fhv + pcl * ny;
    fr[0] = fh; fr[1] = fhu + pcr * nx; fr[2] = fhv + pcr * ny;
    if (!interior && code == 4 && fl[0] < 0.0f) { fl[0] = 0.0f; fl[1] = 0.0f; fl[2] = 0.0f; }
    *active_interior = ai;
    *interior_out = interior;
}

int orc_surface_step(const OrcMesh *m, const float *h, const float *hu, const float *hv,
                     const OrcForcing *f, double dt, double g_d, float md, float *h_out,
                     float *hu_out, float *hv_out, double *diag) {
    const int C = m->cell_count, E = m->edge_count;
    const float dtf = (float)dt;
    const float g = (float)g_d;
    const float dtg = (float)(dt * g_d);     /* timestep_s * gravity: Python-float product */
    const float half_g = (float)(0.5 * g_d); /* 0.5 * gravity: Python-float product */
    float *flux = (float *)malloc(sizeof(float) * 6 * (size_t)(E > 0 ? E : 1));
    unsigned char *flags = (unsigned char *)malloc((size_t)(E > 0 ? E : 1));
    if (!flux || !flags) { free(flux); free(flags); return -1; }
    double bin = 0.0, bout = 0.0;

#pragma omp parallel for schedule(static) reduction(+ : bin, bout)
    for (int e = 0; e < E; ++e) {
        int ai, interior;
        edge_flux(m, h, hu, hv, e, g, half_g, md, flux + 6 * (size_t)e, flux + 6 * (size_t)e + 3, &ai, &interior);
        flags[e] = (unsigned char)(ai | (interior << 1));
        if (!ai) {
            float b = flux[6 * (size_t)e] * m->len[e] * dtf;
            bin += (double)fmax32(-b, 0.0f);
            bout += (double)fmax32(b, 0.0f);
        }
    }

    double rain_m3 = 0.0, infil_m3 = 0.0, vol = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rain_m3, infil_m3, vol)
    for (int c = 0; c < C; ++c) {
        /* scatter_add_1d of the left contributions, then of the right ones,
         * each in ascending edge order (np.add.at order), then summed. */
        float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f, r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
        for (int s = 0; s < 3; ++s) {
            int e = m->cell_edges[3 * (size_t)c + s];
            if (e < 0) continue;
            const float *fe = flux + 6 * (size_t)e;
            float len = m->len[e];
            if (m->left[e] == c) {
                l0 = l0 + (-fe[0]) * len;
                l1 = l1 + (-fe[1]) * len;
                l2 = l2 + (-fe[2]) * len;
            }
            if (m->right[e] == c && (flags[e] & 2)) {
                float a = (flags[e] & 1) ? fe[3] * len : 0.0f;
                float b = (flags[e] & 1) ? fe[4] * len : 0.0f;
                float cc = (flags[e] & 1) ? fe[5] * len : 0.0f;
                r0 = r0 + a; r1 = r1 + b; r2 = r2 + cc;
            }
        }
        float d0 = l0 + r0, d1 = l1 + r1, d2 = l2 + r2;
        int act = m->active ? (m->active[c] > 0.5f) : 1;
        float area = m->area[c];
        float hn = act ? fmax32(h[c] + dtf * d0 / area, 0.0f) : 0.0f;
        float hun = act ? hu[c] + dtf * d1 / area : 0.0f;
        float hvn = act ? hv[c] + dtf * d2 / area : 0.0f;
        /* Manning damping (triangular_backend.py:1160-1171) */
        int wet = hn > md;
        float hs = fmax32(hn, md);
        float uu = hun / hs, vv = hvn / hs;
        float speed = sqrtf(uu * uu + vv * vv);
        float n = m->manning[c];
        float damping = 1.0f + dtg * (n * n) * speed / powf(hs, 4.0f / 3.0f);
        hun = wet ? hun / damping : 0.0f;
        hvn = wet ? hvn / damping : 0.0f;

        /* _apply_sources (triangular_backend.py:1354-1379) */
        float av = m->active ? m->active[c] : 1.0f;
        float rain = f->rain_kind ? f->rain_cell[c] : f->rain_scalar;
        float infc = f->infil_kind ? f->infil_cell[c] : f->infil_scalar;
        float rd = fmax32(rain, 0.0f) * dtf * av;
        float h1 = hn + rd;
        float id = fmin32(h1, fmax32(infc, 0.0f) * dtf * av);
        float h2 = h1 - id;
        float scale = (h1 > md) ? h2 / fmax32(h1, md) : 0.0f;
        hun = hun * scale;
        hvn = hvn * scale;
        int wet2 = h2 > md;
        h_out[c] = h2;
        hu_out[c] = wet2 ? hun : 0.0f;
        hv_out[c] = wet2 ? hvn : 0.0f;
        rain_m3 += (double)(rd * area);
        infil_m3 += (double)(id * area);
        vol += (double)(h2 * area);
    }
    free(flux);
    free(flags);
    if (diag) {
        diag[0] = rain_m3; diag[1] = infil_m3; diag[2] = bin - bout;
        diag[3] = bin; diag[4] = bout; diag[5] = vol;
    }
    return 0;
}

/* Local-inertial surface step: the reference's fused CUDA path
 * (triangular_local_inertial_cuda_kernels.py:59-262: edge discharge, donor
 * scale, cell gather) then _apply_sources (triangular_backend.py:1330-1379).
 * The donor request of a cell is summed over its cell_edges slots in order
 * (the reference adds them with atomicAdd in an unspecified order). */
int orc_li_step(const OrcMesh *m, const float *h, const float *hu, const float *hv, const OrcForcing *f, double dt,
                double g_d, float md, float *h_out, float *hu_out, float *hv_out, double *diag) {
    const int C = m->cell_count, E = m->edge_count;
    const float dtf = (float)dt, g = (float)g_d;
    float *Q = (float *)malloc(sizeof(float) * (size_t)(E > 0 ? E : 1));
    float *scale = (float *)malloc(sizeof(float) * (size_t)(C > 0 ? C : 1));
    if (!Q || !scale) { free(Q); free(scale); return -1; }
#pragma omp parallel for schedule(static)
    for (int e = 0; e < E; ++e) {
        const int L = m->left[e], R0 = m->right[e];
        const int interior = R0 >= 0, R = interior ? R0 : L;
        const int la = m->active ? m->active[L] > 0.5f : 1, ra = m->active ? m->active[R] > 0.5f : 1;
        const int ai = interior && la && ra;
        const int code = (interior && la && !ra) ? 0 : m->bcode[e];
        const float hl = la ? h[L] : 0.0f, hul = la ? hu[L] : 0.0f, hvl = la ? hv[L] : 0.0f;
        const float hr = ra ? h[R] : 0.0f, hur = ra ? hu[R] : 0.0f, hvr = ra ? hv[R] : 0.0f;
        const float bl = m->bed[L], br = m->bed[R];
        const float etal = bl + hl;
        const float etar = ai ? br + hr : bl;
        const float bstar = ai ? fmax32(bl, br) : bl;
        const float hflow = fmax32(fmax32(etal, etar) - bstar, 0.0f);
        const float dist = fmax32(0.5f * (m->char_len[L] + m->char_len[R]), 1.0e-6f);
        const float slope = (etar - etal) / dist;
        const float nx = m->nx[e], ny = m->ny[e], len = m->len[e];
        const float nl = hul * nx + hvl * ny, nr = hur * nx + hvr * ny;
        const float qold = (ai ? 0.5f * (nl + nr) : nl) * len;
        const float mn = ai ? 0.5f * (m->manning[L] + m->manning[R]) : m->manning[L];
        const int bedge = !interior && la && (code == 1 || code == 4);
        const float area = fmax32(hflow * len, 1.0e-8f);
        const float radius = fmax32(hflow, 1.0e-6f);
        const float r43 = radius * cbrtf(radius);
        const float numer = qold - g * area * dtf * slope;
        const float fric = 1.0f + g * dtf * mn * mn * fabsf(qold) / (r43 * area);
        float q = numer / fric;
        if (!(ai || bedge)) q = 0.0f;
        if (bedge) q = fmax32(q, 0.0f);
        Q[e] = q;
    }
#pragma omp parallel for schedule(static)
    for (int c = 0; c < C; ++c) {
        float req = 0.0f;
        for (int s = 0; s < 3; ++s) {
            const int e = m->cell_edges[3 * (size_t)c + s];
            if (e < 0 || m->right[e] < 0) continue;
            const int L = m->left[e], R = m->right[e];
            const int ai = m->active ? (m->active[L] > 0.5f && m->active[R] > 0.5f) : 1;
            const float q = Q[e];
            if (!ai || q == 0.0f) continue;
            if ((q >= 0.0f ? L : R) == c) req += fabsf(q) * dtf;
        }
        const float vol = fmax32(h[c], 0.0f) * m->area[c];
        scale[c] = req > 1.0e-12f ? fmin32(1.0f, vol / req) : 1.0f;
    }
    double rain_m3 = 0.0, infil_m3 = 0.0, bout = 0.0, vtot = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rain_m3, infil_m3, bout, vtot)
    for (int c = 0; c < C; ++c) {
        const int act = m->active ? m->active[c] > 0.5f : 1;
        if (!act) { h_out[c] = hu_out[c] = hv_out[c] = 0.0f; continue; }
        float hd = 0.0f, hs = 0.0f, vs = 0.0f, bf = 0.0f;
        for (int s = 0; s < 3; ++s) {
            const int e = m->cell_edges[3 * (size_t)c + s];
            if (e < 0) continue;
            const float q = Q[e];
            if (q == 0.0f) continue;
            if (m->right[e] >= 0) {
                const int donor = q >= 0.0f ? m->left[e] : m->right[e];
                const float lim = q * scale[donor] * dtf;
                hd += (c == m->left[e]) ? -lim : lim;
            } else {
                const float b = q * dtf;
                hd -= b;
                bf += b;
            }
            hs += q * m->nx[e];
            vs += q * m->ny[e];
        }
        const float area = m->area[c];
        const float hn = fmax32(h[c] + hd / area, 0.0f);
        const float per = 2.0f * area / fmax32(m->char_len[c], 1.0e-12f);
        const int wet = hn > md;
        float hun = wet ? hs / fmax32(per, 1.0e-12f) : 0.0f;
        float hvn = wet ? vs / fmax32(per, 1.0e-12f) : 0.0f;
        /* _apply_sources */
        const float rain = f->rain_kind ? f->rain_cell[c] : f->rain_scalar;
        const float infc = f->infil_kind ? f->infil_cell[c] : f->infil_scalar;
        const float rd = fmax32(rain, 0.0f) * dtf;
        const float h1 = hn + rd;
        const float id = fmin32(h1, fmax32(infc, 0.0f) * dtf);
        const float h2 = h1 - id;
        const float sc = (h1 > md) ? h2 / fmax32(h1, md) : 0.0f;
        hun = hun * sc;
        hvn = hvn * sc;
        const int wet2 = h2 > md;
        h_out[c] = h2;
        hu_out[c] = wet2 ? hun : 0.0f;
        hv_out[c] = wet2 ? hvn : 0.0f;
        rain_m3 += (double)(rd * area);
        infil_m3 += (double)(id * area);
        bout += (double)bf;
        vtot += (double)(h2 * area);
    }
    free(Q);
    free(scale);
    if (diag) {
        diag[0] = rain_m3; diag[1] = infil_m3; diag[2] = -bout;
        diag[3] = 0.0; diag[4] = bout; diag[5] = vtot;
    }
    return 0;
}

/* stable_local_inertial_timestep_s (equations.py:181-210): gravity-wave
 * speed only, float32 per cell; the global min as a double, < 0 if none. */
double orc_li_stable_dt(int32_t n, const float *cl, const float *h, float cfl, float g, float md) {
    float best = INFINITY;
    for (int i = 0; i < n; ++i) {
        const float c = sqrtf(g * fmax32(h[i], md));
        const float d = cfl * cl[i] / fmax32(c, 1.0e-12f);
        if (isfinite(d) && d < best) best = d;
    }
    return isfinite(best) ? (double)best : -1.0;
}

void orc_clamp_velocity(int32_t n, const float *h, float *hu, float *hv, float vmax) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        float speed = sqrtf(hu[i] * hu[i] + hv[i] * hv[i]) / fmax32(h[i], 1.0e-8f);
        float scale = fmin32(1.0f, vmax / fmax32(speed, 1.0e-12f));
        hu[i] = hu[i] * scale;
        hv[i] = hv[i] * scale;
    }
}

double orc_stable_dt(int32_t n, const float *cl, const float *h, const float *hu, const float *hv,
                     float cfl, float g, float md) {
    float best = INFINITY;
#pragma omp parallel for schedule(static) reduction(min : best)
    for (int i = 0; i < n; ++i) {
        float hs = fmax32(h[i], md);
        float a = hu[i] / hs, b = hv[i] / hs;
        float speed = sqrtf(a * a + b * b) + sqrtf(g * hs);
        float local = cfl * cl[i] / fmax32(speed, 1.0e-12f);
        if (isfinite(local) && local < best) best = local;
    }
    return isfinite(best) ? (double)best : -1.0;
}

/* ---------------------------------------------------------------- drainage */

static inline double dsign(double x) { return (double)((x > 0.0) - (x < 0.0)); }

/* Weighted surcharge return (triangular_backend.py:1424-1474), the NumPy
 * path's float64 arithmetic: overflow above the float32 capacity product;
 * each valid entry (node >= 0, cell >= 0) returns overflow x weight (weights
 * clipped at 0 and, unless already normalized, divided by their float32
 * per-node sum in entry order) to its cell; a node returns at most its
 * overflow; nodes without a valid entry return their residual overflow to
 * their node_surface_cell.  h = float32((h + sum over entries) + sum over
 * fallbacks), the per-cell sums formed in entry / node order first.
 * Returns the returned volume. */
static double weighted_overflow_return(const OrcMesh *m, const OrcDrain *d, float *h, double *V) {
    const int N = d->node_count, C = m->cell_count, E = d->sur_count;
    double *ovf = (double *)calloc((size_t)N, sizeof(double));
    double *cap = (double *)calloc((size_t)N, sizeof(double));
    double *by_node = (double *)calloc((size_t)N, sizeof(double));
    double *s1 = (double *)calloc((size_t)C, sizeof(double));
    double *s2 = (double *)calloc((size_t)C, sizeof(double));
    float *wsum = (float *)calloc((size_t)N, sizeof(float));
    char *expl = (char *)calloc((size_t)N, 1);
    if (!ovf || !cap || !by_node || !s1 || !s2 || !wsum || !expl) return 0.0;
    for (int n = 0; n < N; ++n) {
        cap[n] = (double)(d->node_area[n] * fmax32(d->node_maxdepth[n], 0.0f));
        ovf[n] = fmax(V[n] - cap[n], 0.0);
    }
    for (int e = 0; e < E; ++e) {
        const int n = d->sur_node[e], c = d->sur_cell[e];
        const int valid = n >= 0 && c >= 0;
        const float raw = valid ? fmax32(d->sur_weight[e], 0.0f) : 0.0f;
        wsum[valid ? n : 0] += raw;
        if (valid) expl[n] = 1;
    }
    for (int e = 0; e < E; ++e) {
        const int n = d->sur_node[e], c = d->sur_cell[e];
        const int valid = n >= 0 && c >= 0;
        const int sn = valid ? n : 0, sc = valid ? c : 0;
        const float raw = valid ? fmax32(d->sur_weight[e], 0.0f) : 0.0f;
        const float w = d->sur_normalized ? raw : (valid ? raw / fmax32(wsum[sn], 1.0e-12f) : 0.0f);
        const double ret = ovf[sn] * (double)w;
        s1[sc] += ret / (double)m->area[sc];
        by_node[sn] += ret;
    }
    double total = 0.0;
    for (int n = 0; n < N; ++n) {
        const double r = fmin(by_node[n], ovf[n]);
        V[n] = V[n] - r;
        total += r;
    }
    for (int n = 0; n < N; ++n) {
        const int c = d->node_cell[n];
        const int fb = !expl[n] && c >= 0;
        const double r = fb ? fmax(V[n] - cap[n], 0.0) : 0.0;
        s2[fb ? c : 0] += r / (double)m->area[fb ? c : 0];
        V[n] = V[n] - r;
        total += r;
    }
    for (int c = 0; c < C; ++c) h[c] = (float)(((double)h[c] + s1[c]) + s2[c]);
    free(ovf); free(cap); free(by_node); free(s1); free(s2); free(wsum); free(expl);
    return total;
}

int orc_pipe_step(const OrcMesh *m, const OrcDrain *d, float *h, double *V, double *Q, double dt,
                  float g, double *diag) {
    const int N = d->node_count, L = d->link_count, I = d->inlet_count, C = m->cell_count;
    const float dtf = (float)dt;
    const double dtd = (double)dtf; /* the CUDA kernels take timestep as float32 */
    double cap_sum = 0, sur_sum = 0, link_abs = 0, out_sum = 0, ovf_sum = 0, unret = 0, vfin = 0;
    for (int n = 0; n < N; ++n) V[n] = fmax(V[n], 0.0);

    /* inlet exchange: inlet_exchange_cuda (triangular_inlet_exchange_cuda_kernels.py:255-397) */
    if (I > 0) {
        double *rc = (double *)calloc((size_t)I, sizeof(double));
        double *rs = (double *)calloc((size_t)I, sizeof(double));
        double *by_cell = (double *)calloc((size_t)C, sizeof(double));
        double *by_node = (double *)calloc((size_t)(N > 0 ? N : 1), sizeof(double));
        float *hd = (float *)calloc((size_t)C, sizeof(float));
        double *vd = (double *)calloc((size_t)(N > 0 ? N : 1), sizeof(double));
        if (!rc || !rs || !by_cell || !by_node || !hd || !vd) return -1;
        for (int i = 0; i < I; ++i) {
            int c = d->inlet_cell[i], n = d->inlet_node[i];
            double sh = (double)(m->bed[c] + h[c]);
            double nh = (double)d->node_invert[n] + fmax(V[n], 0.0) / fmax((double)d->node_area[n], 1.0e-12);
            double dh = sh - nh;
            double capc = d->cap_capacity ? fmax((double)d->cap_capacity[i], 0.0) * dtd : 1.0e300;
            double surc = d->sur_capacity ? fmax((double)d->sur_capacity[i], 0.0) * dtd : 1.0e300;
            double a = 0.0, b = 0.0;
            if (d->capture_rule == 0) {
                a = capc; b = 0.0;
            } else if (d->capture_rule == 1) {
                a = dh > 0.0 ? capc : 0.0;
                b = dh < 0.0 ? surc : 0.0;
            } else if (d->capture_rule == 2) {
                double q = (double)(d->orifice_coef * d->orifice_area) * sqrt(2.0 * (double)g * fabs(dh)) * dsign(dh);
                a = fmin(fmax(q, 0.0) * dtd, capc);
                b = fmin(fmax(-q, 0.0) * dtd, surc);
            } else {
                double q = (double)(d->orifice_coef * d->orifice_area) * sqrt(2.0 * (double)g * fabs(dh)) * dsign(dh);
                float eq = sqrtf(4.0f * 3.14159265358979323846f * fmax32(d->orifice_area, 0.0f));
                float per = d->weir_perimeter > 0.0f ? d->weir_perimeter : eq;
                float dep = fmax32(h[c], 0.0f);
                double wq = (double)(d->weir_coef * fmax32(per, 0.0f) * dep) * sqrt(2.0 * (double)g * (double)dep);
                a = fmin(fmin(fmax(q, 0.0), wq) * dtd, capc);
                b = fmin(fmax(-q, 0.0) * dtd, surc);
            }
            rc[i] = fmax(a, 0.0);
            rs[i] = fmax(b, 0.0);
            by_cell[c] += rc[i];
            by_node[n] += rs[i];
        }
        for (int i = 0; i < I; ++i) {
            int c = d->inlet_cell[i], n = d->inlet_node[i];
            double avail = (double)fmax32(h[c], 0.0f) * (double)m->area[c];
            double capf = fmin(1.0, avail / fmax(by_cell[c], 1.0e-12));
            double cap = rc[i] * capf;
            double surf = fmin(1.0, fmax(V[n], 0.0) / fmax(by_node[n], 1.0e-12));
            double sur = rs[i] * surf;
            cap_sum += cap;
            sur_sum += sur;
            hd[c] += (float)((sur - cap) / (double)m->area[c]);
            vd[n] += cap - sur;
        }
        for (int c = 0; c < C; ++c) h[c] = h[c] + hd[c];
        for (int n = 0; n < N; ++n) V[n] = V[n] + vd[n];
        free(rc); free(rs); free(by_cell); free(by_node); free(hd); free(vd);
    }

    /* links: step_triangular_pipe_links_and_outfalls_cuda (triangular_pipe_network_cuda_kernels.py:263-421) */
    for (int n = 0; n < N; ++n) V[n] = fmax(V[n], 0.0);
    if (L > 0) {
        double *head = (double *)malloc(sizeof(double) * (size_t)N);
        double *tr = (double *)malloc(sizeof(double) * (size_t)L);
        double *ra = (double *)malloc(sizeof(double) * (size_t)L);
        int *donor = (int *)malloc(sizeof(int) * (size_t)L);
        double *by_donor = (double *)calloc((size_t)N, sizeof(double));
        double *vd = (double *)calloc((size_t)N, sizeof(double));
        if (!head || !tr || !ra || !donor || !by_donor || !vd) return -1;
        for (int n = 0; n < N; ++n) {
            float amax = fmax32(d->node_area[n], 1.0e-12f);
            head[n] = (double)d->node_invert[n] + fmax(V[n], 0.0) / (double)amax;
        }
        for (int l = 0; l < L; ++l) {
            int fn = d->link_from[l], tn = d->link_to[l];
            double fh = head[fn], th = head[tn];
            double inv = d->link_invert ? (double)d->link_invert[l]
                                        : fmin((double)d->node_invert[fn], (double)d->node_invert[tn]);
            double depth = fmax(0.5 * (fh + th) - inv, 0.0);
            float area, radius;
            if (d->link_diam) {
                float dia = fmax32(d->link_diam[l], 1.0e-12f);
                float rg = 0.5f * dia;
                float od = fmin32((float)depth, dia);
                float ratio = fmax32(fmin32((rg - od) / rg, 1.0f), -1.0f);
                float theta = 2.0f * acosf(ratio);
                float oa = 0.5f * rg * rg * (theta - sinf(theta));
                float fa = 0.25f * 3.14159265358979323846f * dia * dia;
                float ca = ((float)depth >= dia) ? fa : oa;
                float fp = 3.14159265358979323846f * dia;
                float cp = ((float)depth >= dia) ? fp : (rg * theta);
                float sw = g * fa / fmax32(d->wave_speed * d->wave_speed, 1.0e-12f);
                float pd = fmax32((float)depth - dia, 0.0f);
                area = ca + sw * pd;
                radius = ca / fmax32(cp, 1.0e-12f);
            } else {
                area = d->link_area[l];
                radius = d->link_radius[l];
            }
            if (d->link_geom && d->link_rect_w && d->link_rect_h && d->link_geom[l] == 2) {
                float od = fmin32(fmax32((float)depth, 0.0f), fmax32(d->link_rect_h[l], 1.0e-6f));
                float oa = fmax32(d->link_rect_w[l], 1.0e-6f) * od;
                float op = fmax32(d->link_rect_w[l] + 2.0f * od, 1.0e-12f);
                area = oa;
                radius = oa / op;
            }
            double len = fmax((double)d->link_len[l], 1.0e-6);
            double sa = fmax((double)area, 1.0e-12);
            double sr = fmax((double)radius, 1.0e-12);
            double flow = Q[l];
            double slope = (fh - th) / len;
            double mn = fmax((double)d->link_n[l], 0.0);
            double fric = (double)g * mn * mn * fabs(flow) / (pow(sr, 4.0 / 3.0) * sa);
            double mk = d->link_minor ? fmax((double)d->link_minor[l], 0.0) : 0.0;
            double minor = mk * fabs(flow) / (2.0 * len * sa);
            double num = flow + (double)g * sa * dtd * slope;
            double up = num / (1.0 + dtd * (fric + minor));
            if (d->link_capacity) {
                double capq = fmax((double)d->link_capacity[l], 0.0);
                up = fmin(fmax(up, -capq), capq);
            }
            double t = up * dtd;
            tr[l] = t;
            donor[l] = t >= 0.0 ? fn : tn;
            ra[l] = fabs(t);
            by_donor[donor[l]] += ra[l];
        }
        for (int l = 0; l < L; ++l) {
            int dn = donor[l], fn = d->link_from[l], tn = d->link_to[l];
            double factor = fmin(1.0, fmax(V[dn], 0.0) / fmax(by_donor[dn], 1.0e-12));
            double lim = ra[l] * factor;
            double sgn = (dn == fn) ? lim : -lim;
            vd[fn] += -sgn;
            vd[tn] += sgn;
            Q[l] = sgn / fmax(dtd, 1.0e-12);
            link_abs += lim;
        }
        for (int n = 0; n < N; ++n) V[n] = fmax(V[n] + vd[n], 0.0);
        free(head); free(tr); free(ra); free(donor); free(by_donor); free(vd);
    }

    /* outfalls (pipe_outfall_kernel) and overflow return (node_overflow_return_kernel) */
    if (N > 0) {
        float *hd = (float *)calloc((size_t)C, sizeof(float));
        if (!hd) return -1;
        for (int n = 0; n < N; ++n) {
            double vol = fmax(V[n], 0.0);
            double hh = (double)d->node_invert[n] + vol / fmax((double)d->node_area[n], 1.0e-12);
            double dh = hh - (double)d->out_tail[n];
            double q = (double)(d->out_coef[n] * d->out_area[n]) * sqrt(2.0 * (double)g * fabs(dh)) * dsign(dh);
            if (d->out_capacity) q = fmin(q, fmax((double)d->out_capacity[n], 0.0));
            double out = fmin(vol, fmax(q, 0.0) * dtd);
            V[n] = vol - out;
            out_sum += out;
        }
        if (d->sur_count > 0) {
            ovf_sum = weighted_overflow_return(m, d, h, V);
        } else {
            for (int n = 0; n < N; ++n) {
                double capv = (double)d->node_area[n] * (double)fmax32(d->node_maxdepth[n], 0.0f);
                double ovf = fmax(V[n] - capv, 0.0);
                int c = d->node_cell[n];
                double ret = c >= 0 ? ovf : 0.0;
                if (c >= 0) hd[c] += (float)(ret / (double)m->area[c]);
                V[n] = V[n] - ret;
                ovf_sum += ret;
            }
            for (int c = 0; c < C; ++c) h[c] = h[c] + hd[c];
        }
        free(hd);
        for (int n = 0; n < N; ++n) {
            float capf = d->node_area[n] * fmax32(d->node_maxdepth[n], 0.0f);
            unret += fmax(V[n] - (double)capf, 0.0);
            vfin += V[n];
        }
    }
    if (diag) {
        diag[0] = cap_sum; diag[1] = sur_sum; diag[2] = link_abs; diag[3] = out_sum;
        diag[4] = ovf_sum; diag[5] = unret; diag[6] = vfin;
    }
    return 0;
}

/* ---------------------------------------------------------------- run loop */

float orc_inflow_q(const OrcInflow *x, int32_t j, double t) {
    const int T = x->time_count, J = x->receiver_count;
    if (t <= x->times_s[0]) return x->q_m3ps[j];
    if (t >= x->times_s[T - 1]) return x->q_m3ps[(size_t)(T - 1) * J + j];
    int lo = 0, hi = T - 1; /* times[lo] < t < times[hi] */
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x->times_s[mid] <= t) lo = mid; else hi = mid;
    }
    const double x0 = x->times_s[lo], x1 = x->times_s[lo + 1];
    const double y0 = x->q_m3ps[(size_t)lo * J + j], y1 = x->q_m3ps[(size_t)(lo + 1) * J + j];
    if (x0 == t) return (float)y0;
    /* np.interp: slope over the interval, the other end's form on NaN */
    const double slope = (y1 - y0) / (x1 - x0);
    double r = slope * (t - x0) + y0;
    if (isnan(r)) {
        r = slope * (t - x1) + y1;
        if (isnan(r) && y0 == y1) r = y0;
    }
    return (float)r;
}

double orc_external_inflow(int32_t C, const float *area, const OrcInflow *x, double time_s, double dt, float *h) {
    float *add = (float *)calloc((size_t)C, sizeof(float));
    if (!add) return 0.0;
    const float dtf = (float)dt;
    double total = 0.0;
    for (int j = 0; j < x->receiver_count; ++j) {
        const int c = x->receiver_cell[j];
        const float added = orc_inflow_q(x, j, time_s) * dtf;
        add[c] = add[c] + added / area[c];
        total += (double)added;
    }
    for (int c = 0; c < C; ++c) h[c] = h[c] + add[c];
    free(add);
    return total;
}

void orc_recharge(const OrcRecharge *r, const float *area_all, double dt, float *h, float *storage, double *diag) {
    const int R = r->row_count;
    const float dtf = (float)dt;
    float *hin = (float *)malloc(sizeof(float) * (size_t)(R > 0 ? R : 1));
    if (!hin) return;
    for (int k = 0; k < R; ++k) hin[k] = h[r->source_cell[k]]; /* every row sees the incoming depth */
    diag[0] = diag[1] = 0.0;
    for (int k = 0; k < R; ++k) {
        const int c = r->source_cell[k];
        const float area = fmax32(area_all[c], 1.0e-6f);
        const float removable = fmax32(hin[k] - r->stop_depth[k], 0.0f);
        const float available = removable * area;
        const float request = r->capture_capacity[k] * dtf;
        const float remaining = fmax32(r->storage_capacity[k] - storage[k], 0.0f);
        const float capture = fmin32(fmin32(available, request), remaining);
        h[c] = fmax32(hin[k] - capture / area, 0.0f); /* the last row of a cell sets it */
        float st = storage[k] + capture;
        const float loss = fmin32(st, r->recharge_capacity[k] * dtf);
        storage[k] = st - loss;
        diag[0] += (double)capture;
        diag[1] += (double)loss;
    }
    free(hin);
}

static double hyeto_rate(const OrcRunParams *p, double t) {
    /* idx = searchsorted(end_s, t, side="right") */
    int lo = 0, hi = p->hyeto_n;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (p->hyeto_end_s[mid] <= t) lo = mid + 1; else hi = mid;
    }
    if (lo >= p->hyeto_n || t < p->hyeto_start_s[lo]) return 0.0;
    return p->hyeto_rate[lo];
}

int orc_run(const OrcMesh *m, const OrcDrain *d, const OrcRunParams *p, float *h, float *hu,
            float *hv, double *V, double *Q, float *wt, double *snap_t, float *snap_h,
            float *snap_hu, float *snap_hv, float *snap_v, OrcRunResult *out) {
    const int C = m->cell_count;
    const int N = d ? d->node_count : 0;
    float *h2 = (float *)malloc(sizeof(float) * (size_t)C);
    float *hu2 = (float *)malloc(sizeof(float) * (size_t)C);
    float *hv2 = (float *)malloc(sizeof(float) * (size_t)C);
    float *rain = (float *)malloc(sizeof(float) * (size_t)C);
    float *infil = (float *)malloc(sizeof(float) * (size_t)C);
    if (!h2 || !hu2 || !hv2 || !rain || !infil) return -1;
    memset(out, 0, sizeof(*out));
    double t = p->t_start_s, cached = p->step_start > 0 ? p->cached_dt_s : -1.0;
    double next_snap = p->next_snapshot_s;
    int64_t step = p->step_start;
    const double T = p->duration_s;
    int rc = 0;
    while (t < T) {
        if (p->max_steps > 0 && step >= p->max_steps) break;
        double dt;
        if (cached < 0.0 || step % p->cfl_interval == 0) {
            dt = p->local_inertial ? orc_li_stable_dt(C, m->char_len, h, (float)p->cfl, (float)p->g, p->min_depth)
                                   : orc_stable_dt(C, m->char_len, h, hu, hv, (float)p->cfl, (float)p->g, p->min_depth);
            if (dt < 0.0) { rc = 3; break; }
            cached = dt;
            out->cfl_evals++;
        } else {
            dt = cached * p->safety;
            out->cfl_reused++;
        }
        dt = fmin(dt, fmin(p->max_dt, T - t));
        dt = fmax(dt, 1.0e-3);
        double base = hyeto_rate(p, t);
        OrcForcing f;
        memset(&f, 0, sizeof(f));
        if (p->horton) {
            float b = (float)base;
#pragma omp parallel for schedule(static)
            for (int c = 0; c < C; ++c) {
                rain[c] = b * p->rain_mult[c];
                infil[c] = p->fc[c] + (p->f0[c] - p->fc[c]) * expf(-p->k[c] * wt[c]);
            }
            f.rain_kind = 1; f.rain_cell = rain;
            f.infil_kind = 1; f.infil_cell = infil;
        } else {
            f.rain_kind = 0; f.rain_scalar = (float)base;
            f.infil_kind = p->infil_kind; f.infil_scalar = p->infil_scalar; f.infil_cell = p->infil_cell;
        }
        double sd[6], pd[7] = {0, 0, 0, 0, 0, 0, 0};
        if (p->local_inertial)
            orc_li_step(m, h, hu, hv, &f, dt, p->g, p->min_depth, h2, hu2, hv2, sd);
        else
            orc_surface_step(m, h, hu, hv, &f, dt, p->g, p->min_depth, h2, hu2, hv2, sd);
        memcpy(h, h2, sizeof(float) * (size_t)C);
        memcpy(hu, hu2, sizeof(float) * (size_t)C);
        memcpy(hv, hv2, sizeof(float) * (size_t)C);
        orc_clamp_velocity(C, h, hu, hv, (float)p->max_speed);
        double ext = 0.0, rd[2] = {0.0, 0.0};
        if (p->inflow && p->inflow->receiver_count > 0)
            ext = orc_external_inflow(C, m->area, p->inflow, t + 0.5 * dt, dt, h);
        if (p->has_drainage && d) orc_pipe_step(m, d, h, V, Q, dt, (float)p->g, pd);
        if (p->recharge && p->recharge->row_count > 0) orc_recharge(p->recharge, m->area, dt, h, p->recharge_storage, rd);
        const float dtw = (float)dt;
#pragma omp parallel for schedule(static)
        for (int c = 0; c < C; ++c) wt[c] = wt[c] + dtw * (float)(h[c] > p->min_depth);
        out->ledger[0] += sd[0]; out->ledger[1] += sd[1]; out->ledger[2] += sd[2];
        out->ledger[3] += pd[3]; out->ledger[4] += pd[4]; out->ledger[5] += pd[5];
        out->ledger[6] += pd[0]; out->ledger[7] += pd[1]; out->ledger[8] += pd[2];
        out->ledger[9] += ext; out->ledger[10] += rd[0]; out->ledger[11] += rd[1];
        t += dt;
        step += 1;
        if (p->finite_interval > 0 && step % p->finite_interval == 0) {
            int bad = 0;
            for (int c = 0; c < C; ++c) if (!isfinite(h[c])) { bad = 1; break; }
            if (bad) { out->error = 1; out->error_step = step; rc = 1; break; }
        }
        if (t >= next_snap || t >= T) {
            int k = out->snapshot_count;
            if (k >= p->max_snapshots) { out->error = 2; rc = 2; break; }
            snap_t[k] = t;
            memcpy(snap_h + (size_t)k * C, h, sizeof(float) * (size_t)C);
            memcpy(snap_hu + (size_t)k * C, hu, sizeof(float) * (size_t)C);
            memcpy(snap_hv + (size_t)k * C, hv, sizeof(float) * (size_t)C);
            for (int n = 0; n < N; ++n) snap_v[(size_t)k * N + n] = (float)V[n];
            out->snapshot_count = k + 1;
            next_snap += p->snapshot_interval_s;
        }
    }
    out->step_count = step - p->step_start;
    out->t_end = t;
    out->cached_dt_s = cached;
    out->next_snapshot_s = next_snap;
    free(h2); free(hu2); free(hv2); free(rain); free(infil);
    return rc;
}
