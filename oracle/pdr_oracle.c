/*
 * CPU oracle for the photara_drender raster / texture / bake / refine path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never linked into it.
 * Compile with -O2 -ffp-contract=off (no fused multiply-add, no fast-math) so that every
 * fp32 expression rounds exactly once per operation, in the order the reference's
 * HLSL source and host C++ write it. Citations are paths inside the reference
 * (fenghuayumo/photara_drender v0.4.0).
 *
 * Conventions chosen where the reference leaves behaviour to the platform:
 *  - float -> int conversions saturate (NaN -> 0), as CUDA's cvt does.
 *  - HLSL clamp/min/max follow IEEE maxNum/minNum (fmaxf/fminf): NaN yields the other operand.
 *  - HLSL round() is round-half-to-even (rintf).
 *  - HLSL lerp(x, y, s) is x*(1-s) + y*s (the GLSL FMix definition DXC lowers to).
 *  - HLSL normalize(v) is v / sqrt(dot(v, v)).
 */
#include "pdr_oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define TILE 16u

/* ---- scalar helpers ------------------------------------------------------------------ */

static int32_t f2i_sat(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

static int32_t d2i_sat(double f) {
    if (f != f) return 0;
    if (f >= 2147483648.0) return INT32_MAX;
    if (f < -2147483648.0) return INT32_MIN;
    return (int32_t)f;
}

static uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)f;
}

/* (uint)round(x) as the shaders write it for triangle ids */
static uint32_t rid(float x) { return f2u_sat(rintf(x)); }

static float clampf_hlsl(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

static int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }

static float cross2(float ax, float ay, float bx, float by) { return ax * by - ay * bx; }
static double cross2d(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

static float lerpf_hlsl(float x, float y, float s) { return x * (1.0f - s) + y * s; }

/* texture_forward.hlsl:16-35 / rasterizer.cpp:164-179 */
static int32_t positive_modulo(int32_t value, int32_t divisor) {
    const int32_t r = value % divisor;
    return r < 0 ? r + divisor : r;
}

static int32_t address_coordinate(int32_t c, uint32_t size, uint32_t mode) {
    if (mode == 0) return clampi(c, 0, (int32_t)size - 1);
    if (mode == 1) return positive_modulo(c, (int32_t)size);
    const int32_t period = (int32_t)size * 2;
    const int32_t m = positive_modulo(c, period);
    return m < (int32_t)size ? m : period - 1 - m;
}

/* wrapping int add (HLSL int arithmetic wraps) */
static int32_t add1(int32_t x) { return (int32_t)((uint32_t)x + 1u); }

static float sample_ndc(uint32_t p, float v0, float vsize) {
    /* rasterize_forward.hlsl:55-57: ((float(p) - v0 + 0.5) * 2 / vsize) - 1 */
    return ((float)p - v0 + 0.5f) * 2.0f / vsize - 1.0f;
}

/* ---- tile binning: src/rasterizer.cpp:61-138 ----------------------------------------- */

int64_t ora_bin_tiles(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                      uint32_t width, uint32_t height, const float vp[4],
                      uint32_t* offsets, uint32_t* list, int64_t cap) {
    const uint32_t tcx = (width + TILE - 1) / TILE;
    const uint32_t tcy = (height + TILE - 1) / TILE;
    const uint64_t tiles = (uint64_t)tcx * tcy;
    (void)V;
    memset(offsets, 0, (tiles + 1) * sizeof(uint32_t));
    for (int pass = 0; pass < 2; ++pass) {
        uint32_t* cursor = NULL;
        if (pass == 1) {
            if (!list) break;
            cursor = (uint32_t*)malloc(tiles * sizeof(uint32_t));
            memcpy(cursor, offsets, tiles * sizeof(uint32_t));
        }
        for (uint32_t t = 0; t < T; ++t) {
            float min_x = INFINITY, min_y = INFINITY, max_x = -INFINITY, max_y = -INFINITY;
            int valid = 1;
            for (uint32_t c = 0; c < 3; ++c) {
                const uint32_t vi = idx[t * 3 + c];
                const float w = pos[(uint64_t)vi * 4 + 3];
                if (!(w > 1e-8f) || !isfinite(w)) { valid = 0; break; }
                const float x = pos[(uint64_t)vi * 4 + 0] / w;
                const float y = pos[(uint64_t)vi * 4 + 1] / w;
                if (!isfinite(x) || !isfinite(y)) { valid = 0; break; }
                /* std::min/std::max on finite values */
                min_x = x < min_x ? x : min_x;
                min_y = y < min_y ? y : min_y;
                max_x = max_x < x ? x : max_x;
                max_y = max_y < y ? y : max_y;
            }
            if (!valid || max_x < -1.0f || min_x > 1.0f || max_y < -1.0f || min_y > 1.0f) continue;
            const int64_t px0 = f2i_sat(floorf((min_x * 0.5f + 0.5f) * vp[2] + vp[0]));
            const int64_t px1 = (int64_t)f2i_sat(ceilf((max_x * 0.5f + 0.5f) * vp[2] + vp[0])) - 1;
            const int64_t py0 = f2i_sat(floorf((min_y * 0.5f + 0.5f) * vp[3] + vp[1]));
            const int64_t py1 = (int64_t)f2i_sat(ceilf((max_y * 0.5f + 0.5f) * vp[3] + vp[1])) - 1;
            const uint32_t x0 = (uint32_t)(px0 < 0 ? 0 : (px0 > (int64_t)width - 1 ? (int64_t)width - 1 : px0));
            const uint32_t x1 = (uint32_t)(px1 < 0 ? 0 : (px1 > (int64_t)width - 1 ? (int64_t)width - 1 : px1));
            const uint32_t y0 = (uint32_t)(py0 < 0 ? 0 : (py0 > (int64_t)height - 1 ? (int64_t)height - 1 : py0));
            const uint32_t y1 = (uint32_t)(py1 < 0 ? 0 : (py1 > (int64_t)height - 1 ? (int64_t)height - 1 : py1));
            for (uint32_t ty = y0 / TILE; ty <= y1 / TILE; ++ty) {
                for (uint32_t tx = x0 / TILE; tx <= x1 / TILE; ++tx) {
                    const uint64_t tile = (uint64_t)ty * tcx + tx;
                    if (pass == 0) {
                        offsets[tile + 1] += 1;
                    } else {
                        const uint32_t slot = cursor[tile]++;
                        if ((int64_t)slot < cap) list[slot] = t;
                    }
                }
            }
        }
        if (pass == 0) {
            uint64_t acc = 0;
            for (uint64_t i = 1; i <= tiles; ++i) {
                acc += offsets[i];
                if (acc > UINT32_MAX) return ORA_OVERFLOW;
                offsets[i] = (uint32_t)acc;
            }
        } else {
            free(cursor);
        }
    }
    return (int64_t)offsets[tiles];
}

/* ---- rasterize forward: shaders/rasterize_forward.hlsl:45-175 ------------------------ */

static int validate_mesh(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T) {
    (void)pos;
    if (V == 0) return ORA_INVALID;
    if (T == 0) return ORA_INVALID;
    for (uint64_t i = 0; i < (uint64_t)T * 3; ++i)
        if (idx[i] >= V) return ORA_RANGE;
    return ORA_OK;
}

/* ties (optional, one byte per pixel): ORA_TIE_DEPTH when another covering triangle had the winner's
 * depth, so the lowest-id rule decided the pixel; ORA_TIE_EDGE when the winner passed one of its edge
 * tests only on the edge or inside the 1e-7 tolerance (e * sign <= 0). */
static int raster_forward_impl(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                               uint32_t W, uint32_t H, uint32_t cull_mode, int out_deriv,
                               const float vp[4], float* raster, float* deriv, uint8_t* ties) {
    int rc = validate_mesh(pos, V, idx, T);
    if (rc) return rc;
    if (W == 0 || H == 0) return ORA_INVALID;
    if (!isfinite(vp[0]) || !isfinite(vp[1]) || !isfinite(vp[2]) || !isfinite(vp[3]) ||
        vp[2] <= 0.0f || vp[3] <= 0.0f)
        return ORA_INVALID;
    const uint32_t tcx = (W + TILE - 1) / TILE, tcy = (H + TILE - 1) / TILE;
    uint32_t* offsets = (uint32_t*)malloc(((uint64_t)tcx * tcy + 1) * sizeof(uint32_t));
    int64_t n = ora_bin_tiles(pos, V, idx, T, W, H, vp, offsets, NULL, 0);
    if (n < 0) { free(offsets); return (int)n; }
    uint32_t* list = (uint32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint32_t));
    ora_bin_tiles(pos, V, idx, T, W, H, vp, offsets, list, n);

#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t py = 0; py < (int64_t)H; ++py) {
        for (uint32_t px = 0; px < W; ++px) {
            const uint64_t pixel = (uint64_t)py * W + px;
            const float sx = sample_ndc(px, vp[0], vp[2]);
            const float sy = sample_ndc((uint32_t)py, vp[1], vp[3]);
            float best_depth = 3.402823466e+38f;
            uint32_t best_tri = 0;
            int depth_tie = 0, edge_tie = 0;
            float bb0 = 0.0f, bb1 = 0.0f;
            float bd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            const uint64_t tile = ((uint64_t)py / TILE) * tcx + px / TILE;
            for (uint32_t e = offsets[tile]; e < offsets[tile + 1]; ++e) {
                const uint32_t t = list[e];
                const uint32_t i0 = idx[t * 3 + 0], i1 = idx[t * 3 + 1], i2 = idx[t * 3 + 2];
                if (i0 >= V || i1 >= V || i2 >= V) continue;
                const float* p0 = pos + (uint64_t)i0 * 4;
                const float* p1 = pos + (uint64_t)i1 * 4;
                const float* p2 = pos + (uint64_t)i2 * 4;
                if (p0[3] <= 1e-8f || p1[3] <= 1e-8f || p2[3] <= 1e-8f) continue;
                const float s0x = p0[0] / p0[3], s0y = p0[1] / p0[3];
                const float s1x = p1[0] / p1[3], s1y = p1[1] / p1[3];
                const float s2x = p2[0] / p2[3], s2y = p2[1] / p2[3];
                const float screen_area = cross2(s1x - s0x, s1y - s0y, s2x - s0x, s2y - s0y);
                if (fabsf(screen_area) <= 1e-12f) continue;
                if ((cull_mode == 1 && screen_area <= 0.0f) || (cull_mode == 2 && screen_area >= 0.0f)) continue;
                const float e0 = cross2(s1x - sx, s1y - sy, s2x - sx, s2y - sy);
                const float e1 = cross2(s2x - sx, s2y - sy, s0x - sx, s0y - sy);
                const float e2 = cross2(s0x - sx, s0y - sy, s1x - sx, s1y - sy);
                const float sign = screen_area > 0.0f ? 1.0f : -1.0f;
                const float ceps = -1e-7f;
                if (e0 * sign < ceps || e1 * sign < ceps || e2 * sign < ceps) continue;
                const float q0x = p0[0] - sx * p0[3], q0y = p0[1] - sy * p0[3];
                const float q1x = p1[0] - sx * p1[3], q1y = p1[1] - sy * p1[3];
                const float q2x = p2[0] - sx * p2[3], q2y = p2[1] - sy * p2[3];
                const float a0 = cross2(q1x, q1y, q2x, q2y);
                const float a1 = cross2(q2x, q2y, q0x, q0y);
                const float a2 = cross2(q0x, q0y, q1x, q1y);
                const float ha = a0 + a1 + a2;
                if (fabsf(ha) <= 1e-12f) continue;
                const float inv = 1.0f / ha;
                const float b0 = clampf_hlsl(a0 * inv, 0.0f, 1.0f);
                const float b1 = clampf_hlsl(a1 * inv, 0.0f, 1.0f);
                const float iz = p0[2] * a0 + p1[2] * a1 + p2[2] * a2;
                const float iw = p0[3] * a0 + p1[3] * a1 + p2[3] * a2;
                if (fabsf(iw) <= 1e-12f) continue;
                const float depth = clampf_hlsl(iz / iw, -1.0f, 1.0f);
                const int same_depth = depth == best_depth && best_tri != 0;
                if (depth > best_depth || (same_depth && t + 1 >= best_tri)) {
                    depth_tie |= same_depth;
                    continue;
                }
                depth_tie = same_depth;
                edge_tie = e0 * sign <= 0.0f || e1 * sign <= 0.0f || e2 * sign <= 0.0f;
                best_depth = depth;
                best_tri = t + 1;
                bb0 = b0;
                bb1 = b1;
                if (out_deriv) {
                    const float da0_dx = -p1[3] * p2[1] + p2[3] * p1[1];
                    const float da0_dy = -p1[0] * p2[3] + p1[3] * p2[0];
                    const float da1_dx = -p2[3] * p0[1] + p2[1] * p0[3];
                    const float da1_dy = -p2[0] * p0[3] + p2[3] * p0[0];
                    const float da2_dx = -p0[3] * p1[1] + p0[1] * p1[3];
                    const float da2_dy = -p0[0] * p1[3] + p0[3] * p1[0];
                    const float dadx = da0_dx + da1_dx + da2_dx;
                    const float dady = da0_dy + da1_dy + da2_dy;
                    bd[0] = (da0_dx - b0 * dadx) * inv * 2.0f / vp[2];
                    bd[2] = (da1_dx - b1 * dadx) * inv * 2.0f / vp[2];
                    bd[1] = (da0_dy - b0 * dady) * inv * 2.0f / vp[3];
                    bd[3] = (da1_dy - b1 * dady) * inv * 2.0f / vp[3];
                }
            }
            if (ties) ties[pixel] = (uint8_t)(best_tri != 0 ? (depth_tie ? ORA_TIE_DEPTH : 0) | (edge_tie ? ORA_TIE_EDGE : 0) : 0);
            float* r = raster + pixel * 4;
            if (best_tri == 0) {
                r[0] = r[1] = r[2] = r[3] = 0.0f;
                if (deriv) deriv[pixel * 4 + 0] = deriv[pixel * 4 + 1] = deriv[pixel * 4 + 2] = deriv[pixel * 4 + 3] = 0.0f;
            } else {
                r[0] = bb0;
                r[1] = bb1;
                r[2] = best_depth;
                r[3] = (float)best_tri;
                if (deriv) {
                    deriv[pixel * 4 + 0] = bd[0];
                    deriv[pixel * 4 + 1] = bd[1];
                    deriv[pixel * 4 + 2] = bd[2];
                    deriv[pixel * 4 + 3] = bd[3];
                }
            }
        }
    }
    free(list);
    free(offsets);
    return ORA_OK;
}

int ora_rasterize_forward(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                          uint32_t W, uint32_t H, uint32_t cull_mode, int out_deriv,
                          const float vp[4], float* raster, float* deriv) {
    return raster_forward_impl(pos, V, idx, T, W, H, cull_mode, out_deriv, vp, raster, deriv, NULL);
}

int ora_rasterize_forward_ties(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                               uint32_t W, uint32_t H, uint32_t cull_mode, const float vp[4], float* raster,
                               uint8_t* ties) {
    return raster_forward_impl(pos, V, idx, T, W, H, cull_mode, 0, vp, raster, NULL, ties);
}

/* FP64 twin: same formulas in double for the triangle the fp32 pass selected. */
int ora_rasterize_forward_f64(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                              uint32_t W, uint32_t H, const float vp[4], const float* raster,
                              double* r64, double* d64) {
    (void)V;
    for (uint64_t pixel = 0; pixel < (uint64_t)W * H; ++pixel) {
        const uint32_t px = (uint32_t)(pixel % W), py = (uint32_t)(pixel / W);
        const uint32_t id = rid(raster[pixel * 4 + 3]);
        double* r = r64 + pixel * 4;
        double* d = d64 + pixel * 4;
        r[0] = r[1] = r[2] = r[3] = 0.0;
        d[0] = d[1] = d[2] = d[3] = 0.0;
        if (id == 0 || id > T) continue;
        const uint32_t t = id - 1;
        const float* p0 = pos + (uint64_t)idx[t * 3 + 0] * 4;
        const float* p1 = pos + (uint64_t)idx[t * 3 + 1] * 4;
        const float* p2 = pos + (uint64_t)idx[t * 3 + 2] * 4;
        const double sx = ((double)px - vp[0] + 0.5) * 2.0 / vp[2] - 1.0;
        const double sy = ((double)py - vp[1] + 0.5) * 2.0 / vp[3] - 1.0;
        const double q0x = p0[0] - sx * p0[3], q0y = p0[1] - sy * p0[3];
        const double q1x = p1[0] - sx * p1[3], q1y = p1[1] - sy * p1[3];
        const double q2x = p2[0] - sx * p2[3], q2y = p2[1] - sy * p2[3];
        const double a0 = cross2d(q1x, q1y, q2x, q2y);
        const double a1 = cross2d(q2x, q2y, q0x, q0y);
        const double a2 = cross2d(q0x, q0y, q1x, q1y);
        const double inv = 1.0 / (a0 + a1 + a2);
        const double b0 = fmin(fmax(a0 * inv, 0.0), 1.0), b1 = fmin(fmax(a1 * inv, 0.0), 1.0);
        const double iz = (double)p0[2] * a0 + (double)p1[2] * a1 + (double)p2[2] * a2;
        const double iw = (double)p0[3] * a0 + (double)p1[3] * a1 + (double)p2[3] * a2;
        r[0] = b0;
        r[1] = b1;
        r[2] = fmin(fmax(iz / iw, -1.0), 1.0);
        r[3] = (double)id;
        const double da0_dx = -(double)p1[3] * p2[1] + (double)p2[3] * p1[1];
        const double da0_dy = -(double)p1[0] * p2[3] + (double)p1[3] * p2[0];
        const double da1_dx = -(double)p2[3] * p0[1] + (double)p2[1] * p0[3];
        const double da1_dy = -(double)p2[0] * p0[3] + (double)p2[3] * p0[0];
        const double da2_dx = -(double)p0[3] * p1[1] + (double)p0[1] * p1[3];
        const double da2_dy = -(double)p0[0] * p1[3] + (double)p0[3] * p1[0];
        const double dadx = da0_dx + da1_dx + da2_dx, dady = da0_dy + da1_dy + da2_dy;
        d[0] = (da0_dx - b0 * dadx) * inv * 2.0 / vp[2];
        d[2] = (da1_dx - b1 * dadx) * inv * 2.0 / vp[2];
        d[1] = (da0_dy - b0 * dady) * inv * 2.0 / vp[3];
        d[3] = (da1_dy - b1 * dady) * inv * 2.0 / vp[3];
    }
    return ORA_OK;
}

/* ---- rasterize backward: rasterize_backward.hlsl:36-158, reduce_vertex_gradients.hlsl,
 *      rasterizer.cpp:145-162 (vertex CSR over corners, ascending corner order) ---------- */

/* ACC(x) is the identity, or |x| in the FP64 twins' abs_terms mode (sum of absolute terms,
 * the scale against which summation-order error is stated). */
#define RB_BODY(REAL, CROSS, EPS_AREA, SAMPLE)                                                       \
    _Pragma("omp parallel for schedule(dynamic, 256)")                                               \
    for (uint32_t t = 0; t < T; ++t) {                                                               \
        REAL g[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};                                  \
        const uint32_t vi[3] = {idx[t * 3 + 0], idx[t * 3 + 1], idx[t * 3 + 2]};                     \
        if (vi[0] < V && vi[1] < V && vi[2] < V) {                                                   \
            const float* p[3] = {pos + (uint64_t)vi[0] * 4, pos + (uint64_t)vi[1] * 4,               \
                                 pos + (uint64_t)vi[2] * 4};                                          \
            if (!(p[0][3] <= 1e-8f || p[1][3] <= 1e-8f || p[2][3] <= 1e-8f)) {                        \
                const float s0x = p[0][0] / p[0][3], s0y = p[0][1] / p[0][3];                        \
                const float s1x = p[1][0] / p[1][3], s1y = p[1][1] / p[1][3];                        \
                const float s2x = p[2][0] / p[2][3], s2y = p[2][1] / p[2][3];                        \
                const float mnx = fminf(s0x, fminf(s1x, s2x)), mny = fminf(s0y, fminf(s1y, s2y));    \
                const float mxx = fmaxf(s0x, fmaxf(s1x, s2x)), mxy = fmaxf(s0y, fmaxf(s1y, s2y));    \
                const int32_t x0 = clampi(f2i_sat(floorf((mnx * 0.5f + 0.5f) * vp[2] + vp[0])), 0, (int32_t)W); \
                const int32_t x1 = clampi(f2i_sat(ceilf((mxx * 0.5f + 0.5f) * vp[2] + vp[0])), 0, (int32_t)W);  \
                const int32_t y0 = clampi(f2i_sat(floorf((mny * 0.5f + 0.5f) * vp[3] + vp[1])), 0, (int32_t)H); \
                const int32_t y1 = clampi(f2i_sat(ceilf((mxy * 0.5f + 0.5f) * vp[3] + vp[1])), 0, (int32_t)H);  \
                for (int32_t y = y0; y < y1; ++y) {                                                  \
                    for (int32_t x = x0; x < x1; ++x) {                                              \
                        const uint64_t pix = (uint64_t)y * W + (uint64_t)x;                          \
                        if (rid(raster[pix * 4 + 3]) != t + 1) continue;                             \
                        const float lgx = grad_raster[pix * 4 + 0], lgy = grad_raster[pix * 4 + 1];  \
                        if (lgx == 0.0f && lgy == 0.0f) continue;                                    \
                        REAL sx, sy;                                                                 \
                        SAMPLE;                                                                      \
                        const REAL q0x = p[0][0] - sx * p[0][3], q0y = p[0][1] - sy * p[0][3];       \
                        const REAL q1x = p[1][0] - sx * p[1][3], q1y = p[1][1] - sy * p[1][3];       \
                        const REAL q2x = p[2][0] - sx * p[2][3], q2y = p[2][1] - sy * p[2][3];       \
                        const REAL area = CROSS(q1x, q1y, q2x, q2y) + CROSS(q2x, q2y, q0x, q0y) +    \
                                          CROSS(q0x, q0y, q1x, q1y);                                 \
                        if (fabs((double)area) <= (double)1e-12f) continue;                          \
                        const REAL eps = area >= 0 ? (REAL)EPS_AREA : -(REAL)EPS_AREA;               \
                        const REAL inv = (REAL)1 / (area + eps);                                     \
                        const REAL a0 = CROSS(q1x, q1y, q2x, q2y);                                   \
                        const REAL a1 = CROSS(q2x, q2y, q0x, q0y);                                   \
                        const REAL b0 = a0 * inv, b1 = a1 * inv;                                     \
                        const REAL gb0 = lgx * inv, gb1 = lgy * inv;                                 \
                        const REAL gc = gb0 * b0 + gb1 * b1;                                         \
                        const REAL g0x = gc * (q2y - q1y) - gb1 * q2y;                               \
                        const REAL g1x = gc * (q0y - q2y) + gb0 * q2y;                               \
                        const REAL g2x = gc * (q1y - q0y) - gb0 * q1y + gb1 * q0y;                   \
                        const REAL g0y = gc * (q1x - q2x) + gb1 * q2x;                               \
                        const REAL g1y = gc * (q2x - q0x) - gb0 * q2x;                               \
                        const REAL g2y = gc * (q0x - q1x) + gb0 * q1x - gb1 * q0x;                   \
                        g[0][0] += ACC(g0x); g[0][1] += ACC(g0y); g[0][2] += (REAL)0; g[0][3] += ACC(-sx * g0x - sy * g0y); \
                        g[1][0] += ACC(g1x); g[1][1] += ACC(g1y); g[1][2] += (REAL)0; g[1][3] += ACC(-sx * g1x - sy * g1y); \
                        g[2][0] += ACC(g2x); g[2][1] += ACC(g2y); g[2][2] += (REAL)0; g[2][3] += ACC(-sx * g2x - sy * g2y); \
                    }                                                                                \
                }                                                                                    \
            }                                                                                        \
        }                                                                                            \
        for (int k = 0; k < 3; ++k)                                                                  \
            for (int c = 0; c < 4; ++c) corner[((uint64_t)t * 3 + k) * 4 + c] = g[k][c];             \
    }

static void vertex_csr(const uint32_t* idx, uint32_t T, uint32_t V, uint32_t** off_out, uint32_t** corners_out) {
    uint32_t* off = (uint32_t*)calloc((size_t)V + 1, sizeof(uint32_t));
    for (uint64_t c = 0; c < (uint64_t)T * 3; ++c) off[idx[c] + 1]++;
    for (uint32_t v = 1; v <= V; ++v) off[v] += off[v - 1];
    uint32_t* cur = (uint32_t*)malloc(((size_t)V + 1) * sizeof(uint32_t));
    memcpy(cur, off, ((size_t)V + 1) * sizeof(uint32_t));
    uint32_t* corners = (uint32_t*)malloc((size_t)T * 3 * sizeof(uint32_t));
    for (uint32_t c = 0; c < T * 3; ++c) corners[cur[idx[c]]++] = c;
    free(cur);
    *off_out = off;
    *corners_out = corners;
}

int ora_rasterize_backward(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                           uint32_t W, uint32_t H, const float vp[4], const float* raster,
                           const float* grad_raster, float* grad_pos) {
    int rc = validate_mesh(pos, V, idx, T);
    if (rc) return rc;
    float* corner = (float*)malloc((size_t)T * 12 * sizeof(float));
#define SAMPLE_F sx = sample_ndc((uint32_t)x, vp[0], vp[2]); sy = sample_ndc((uint32_t)y, vp[1], vp[3])
#define ACC(x) (x)
    RB_BODY(float, cross2, 1e-6f, SAMPLE_F)
#undef ACC
    uint32_t *off, *corners;
    vertex_csr(idx, T, V, &off, &corners);
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; ++v) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t a = off[v]; a < off[v + 1]; ++a)
            for (int c = 0; c < 4; ++c) acc[c] += corner[(uint64_t)corners[a] * 4 + c];
        for (int c = 0; c < 4; ++c) grad_pos[(uint64_t)v * 4 + c] = acc[c];
    }
    free(off);
    free(corners);
    free(corner);
    return ORA_OK;
}

int ora_rasterize_backward_f64(const float* pos, uint32_t V, const uint32_t* idx, uint32_t T,
                               uint32_t W, uint32_t H, const float vp[4], const float* raster,
                               const float* grad_raster, double* grad_pos, int abs_terms) {
    int rc = validate_mesh(pos, V, idx, T);
    if (rc) return rc;
    double* corner = (double*)malloc((size_t)T * 12 * sizeof(double));
#define SAMPLE_D sx = ((double)x - vp[0] + 0.5) * 2.0 / vp[2] - 1.0; sy = ((double)y - vp[1] + 0.5) * 2.0 / vp[3] - 1.0
#define ACC(x) (abs_terms ? fabs(x) : (x))
    RB_BODY(double, cross2d, 1e-6f, SAMPLE_D)
#undef ACC
    uint32_t *off, *corners;
    vertex_csr(idx, T, V, &off, &corners);
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; ++v) {
        double acc[4] = {0, 0, 0, 0};
        for (uint32_t a = off[v]; a < off[v + 1]; ++a)
            for (int c = 0; c < 4; ++c) acc[c] += corner[(uint64_t)corners[a] * 4 + c];
        for (int c = 0; c < 4; ++c) grad_pos[(uint64_t)v * 4 + c] = acc[c];
    }
    free(off);
    free(corners);
    free(corner);
    return ORA_OK;
}

/* ---- interpolation: interpolate_forward.hlsl:15-54 ---------------------------------- */

int ora_interpolate_forward(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                            uint32_t T, const float* raster, uint64_t P, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)P; ++p) {
        const uint32_t id = rid(raster[p * 4 + 3]);
        int ok = id != 0 && id <= T;
        uint32_t i0 = 0, i1 = 0, i2 = 0;
        if (ok) {
            i0 = idx[(id - 1) * 3 + 0];
            i1 = idx[(id - 1) * 3 + 1];
            i2 = idx[(id - 1) * 3 + 2];
            ok = i0 < V && i1 < V && i2 < V;
        }
        for (uint32_t a = 0; a < A; ++a) {
            if (!ok) { out[p * A + a] = 0.0f; continue; }
            const float u = raster[p * 4 + 0], v = raster[p * 4 + 1];
            const float w = 1.0f - u - v;
            const float a0 = attr[(uint64_t)i0 * A + a], a1 = attr[(uint64_t)i1 * A + a], a2 = attr[(uint64_t)i2 * A + a];
            out[p * A + a] = u * a0 + v * a1 + w * a2;
        }
    }
    return ORA_OK;
}

/* interpolate_grad_attributes.hlsl:15-58 sums, per (vertex, attribute), weight * grad over all
 * pixels in ascending order; adding zero-weight terms leaves a finite sum unchanged, so the
 * per-pixel scatter below accumulates every vertex in the same order. interpolate_grad_raster.hlsl
 * gives the raster gradient. */
/* Threaded without changing any sum: the raster gradient is per pixel; for the attribute gradient
 * each thread owns a range of vertices and scans all pixels in order, so every vertex's sum keeps the
 * sequential (pixel) order and the result is bit-identical for any thread count. */
#define IB_BODY(REAL)                                                                                \
    _Pragma("omp parallel for schedule(static)")                                                     \
    for (uint64_t p = 0; p < P; ++p) {                                                               \
        const uint32_t id = rid(raster[p * 4 + 3]);                                                  \
        REAL* gr = grad_raster + p * 4;                                                              \
        gr[0] = gr[1] = gr[2] = gr[3] = 0;                                                           \
        if (id == 0 || id > T) continue;                                                             \
        const uint32_t i0 = idx[(id - 1) * 3 + 0], i1 = idx[(id - 1) * 3 + 1], i2 = idx[(id - 1) * 3 + 2]; \
        if (i0 < V && i1 < V && i2 < V) {                                                            \
            REAL gx = 0, gy = 0;                                                                     \
            for (uint32_t a = 0; a < A; ++a) {                                                       \
                const REAL a0 = attr[(uint64_t)i0 * A + a], a1 = attr[(uint64_t)i1 * A + a];        \
                const REAL a2 = attr[(uint64_t)i2 * A + a];                                          \
                const REAL g = grad_out[p * A + a];                                                  \
                gx += g * (a0 - a2);                                                                 \
                gy += g * (a1 - a2);                                                                 \
            }                                                                                        \
            gr[0] = gx;                                                                              \
            gr[1] = gy;                                                                              \
        }                                                                                            \
    }                                                                                                \
    _Pragma("omp parallel")                                                                          \
    {                                                                                                \
        const uint32_t nt = (uint32_t)omp_get_num_threads(), tid = (uint32_t)omp_get_thread_num();   \
        const uint32_t v_lo = (uint32_t)((uint64_t)V * tid / nt), v_hi = (uint32_t)((uint64_t)V * (tid + 1) / nt); \
        memset(grad_attr + (uint64_t)v_lo * A, 0, (size_t)(v_hi - v_lo) * A * sizeof(REAL));        \
        for (uint64_t p = 0; p < P && v_lo < v_hi; ++p) {                                            \
            const uint32_t id = rid(raster[p * 4 + 3]);                                              \
            if (id == 0 || id > T) continue;                                                         \
            const uint32_t i0 = idx[(id - 1) * 3 + 0], i1 = idx[(id - 1) * 3 + 1], i2 = idx[(id - 1) * 3 + 2]; \
            const uint32_t vs[3] = {i0, i1, i2};                                                     \
            const float u = raster[p * 4 + 0], v = raster[p * 4 + 1];                                \
            for (int k = 0; k < 3; ++k) {                                                            \
                const uint32_t vx = vs[k];                                                           \
                if (vx < v_lo || vx >= v_hi) continue;                                               \
                int first = 1;                                                                       \
                for (int j = 0; j < k; ++j) if (vs[j] == vx) first = 0;                              \
                if (!first) continue;                                                                \
                REAL wgt = 0;                                                                        \
                if (i0 == vx) wgt += (REAL)u;                                                        \
                if (i1 == vx) wgt += (REAL)v;                                                        \
                if (i2 == vx) wgt += (REAL)1 - (REAL)u - (REAL)v;                                    \
                for (uint32_t a = 0; a < A; ++a) grad_attr[(uint64_t)vx * A + a] += ACC(wgt * (REAL)grad_out[p * A + a]); \
            }                                                                                        \
        }                                                                                            \
    }

int ora_interpolate_backward(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                             uint32_t T, const float* raster, uint64_t P, const float* grad_out,
                             float* grad_attr, float* grad_raster) {
#define ACC(x) (x)
    IB_BODY(float)
#undef ACC
    return ORA_OK;
}

int ora_interpolate_backward_f64(const float* attr, uint32_t V, uint32_t A, const uint32_t* idx,
                                 uint32_t T, const float* raster, uint64_t P, const float* grad_out,
                                 double* grad_attr, double* grad_raster, int abs_terms) {
#define ACC(x) (abs_terms ? fabs(x) : (x))
    IB_BODY(double)
#undef ACC
    return ORA_OK;
}

/* ---- texture: texture_forward.hlsl:37-79 --------------------------------------------- */

int ora_texture_forward(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                        const float* uv, const float* raster, uint64_t P, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)P; ++p) {
        if (rid(raster[p * 4 + 3]) == 0) {
            for (uint32_t c = 0; c < C; ++c) out[p * C + c] = 0.0f;
            continue;
        }
        const float tx = uv[p * 2 + 0] * (float)tw - 0.5f;
        const float ty = uv[p * 2 + 1] * (float)th - 0.5f;
        const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
        const float fx = tx - floorf(tx), fy = ty - floorf(ty);
        const int32_t x0 = address_coordinate(bx, tw, mode), x1 = address_coordinate(add1(bx), tw, mode);
        const int32_t y0 = address_coordinate(by, th, mode), y1 = address_coordinate(add1(by), th, mode);
        const float w0 = (1.0f - fx) * (1.0f - fy), w1 = fx * (1.0f - fy);
        const float w2 = (1.0f - fx) * fy, w3 = fx * fy;
        for (uint32_t c = 0; c < C; ++c) {
            const float t0 = tex[((uint64_t)(uint32_t)y0 * tw + (uint32_t)x0) * C + c];
            const float t1 = tex[((uint64_t)(uint32_t)y0 * tw + (uint32_t)x1) * C + c];
            const float t2 = tex[((uint64_t)(uint32_t)y1 * tw + (uint32_t)x0) * C + c];
            const float t3 = tex[((uint64_t)(uint32_t)y1 * tw + (uint32_t)x1) * C + c];
            out[p * C + c] = t0 * w0 + t1 * w1 + t2 * w2 + t3 * w3;
        }
    }
    return ORA_OK;
}

/* rasterizer.cpp:187-258: the texel->sample table uses double texel positions and float
 * weights; texture_grad_texture.hlsl:15-38 sums each texel's entries in ascending order,
 * which the ascending-entry scatter below reproduces. texture_grad_uv.hlsl:38-80 for uv. */
#define TB_BODY(REAL)                                                                                \
    const uint64_t texels = (uint64_t)tw * th;                                                       \
    for (uint64_t p = 0; p < P; ++p) { /* the reference throws at the first bad pixel, in order */ \
        if (raster[p * 4 + 3] == 0.0f) continue;                                                     \
        const float u = uv[p * 2 + 0], v = uv[p * 2 + 1];                                            \
        if (!isfinite(u) || !isfinite(v)) return ORA_INVALID;                                        \
        if (fabs((double)u * tw - 0.5) > 1.0e9 || fabs((double)v * th - 0.5) > 1.0e9) return ORA_RANGE; \
    }                                                                                                \
    /* each thread owns a band of texel rows and scans all pixels in order: every texel's sum keeps \
     * the sequential order, bit-identical for any thread count */                                 \
    _Pragma("omp parallel")                                                                          \
    {                                                                                                \
        const uint32_t nt = (uint32_t)omp_get_num_threads(), tid = (uint32_t)omp_get_thread_num();   \
        const uint32_t y_lo = (uint32_t)((uint64_t)th * tid / nt), y_hi = (uint32_t)((uint64_t)th * (tid + 1) / nt); \
        memset(grad_tex + (uint64_t)y_lo * tw * C, 0, (size_t)(y_hi - y_lo) * tw * C * sizeof(REAL)); \
        for (uint64_t p = 0; p < P && y_lo < y_hi; ++p) {                                            \
            if (raster[p * 4 + 3] == 0.0f) continue;                                                 \
            const float u = uv[p * 2 + 0], v = uv[p * 2 + 1];                                        \
            const double tx = (double)u * tw - 0.5, ty = (double)v * th - 0.5;                       \
            const int32_t by = d2i_sat(floor(ty));                                                   \
            const int32_t ys[2] = {address_coordinate(by, th, mode), address_coordinate(by + 1, th, mode)}; \
            const int in0 = (uint32_t)ys[0] >= y_lo && (uint32_t)ys[0] < y_hi;                       \
            const int in1 = (uint32_t)ys[1] >= y_lo && (uint32_t)ys[1] < y_hi;                       \
            if (!in0 && !in1) continue;                                                              \
            const int32_t bx = d2i_sat(floor(tx));                                                   \
            const REAL fx = (REAL)(tx - floor(tx)), fy = (REAL)(ty - floor(ty));                     \
            const int32_t xs[2] = {address_coordinate(bx, tw, mode), address_coordinate(bx + 1, tw, mode)}; \
            const REAL w[4] = {((REAL)1 - fx) * ((REAL)1 - fy), fx * ((REAL)1 - fy), ((REAL)1 - fx) * fy, fx * fy}; \
            const uint64_t tx4[4] = {(uint64_t)ys[0] * tw + xs[0], (uint64_t)ys[0] * tw + xs[1],    \
                                     (uint64_t)ys[1] * tw + xs[0], (uint64_t)ys[1] * tw + xs[1]};    \
            for (int k = 0; k < 4; ++k) {                                                            \
                if (!(k < 2 ? in0 : in1)) continue;                                                  \
                for (uint32_t c = 0; c < C; ++c) grad_tex[tx4[k] * C + c] += ACC(w[k] * (REAL)grad[p * C + c]); \
            }                                                                                        \
        }                                                                                            \
    }                                                                                                \
    (void)texels;                                                                                    \
    if (grad_uv) {                                                                                   \
        _Pragma("omp parallel for schedule(static)")                                                 \
        for (uint64_t p = 0; p < P; ++p) {                                                           \
            if (rid(raster[p * 4 + 3]) == 0) { grad_uv[p * 2] = grad_uv[p * 2 + 1] = 0; continue; } \
            REAL tx, ty, fx, fy; int32_t bx, by;                                                     \
            UVPOS;                                                                                   \
            const int32_t x0 = address_coordinate(bx, tw, mode), x1 = address_coordinate(add1(bx), tw, mode); \
            const int32_t y0 = address_coordinate(by, th, mode), y1 = address_coordinate(add1(by), th, mode); \
            REAL gx = 0, gy = 0;                                                                     \
            for (uint32_t c = 0; c < C; ++c) {                                                       \
                const REAL c00 = tex[((uint64_t)(uint32_t)y0 * tw + (uint32_t)x0) * C + c];          \
                const REAL c10 = tex[((uint64_t)(uint32_t)y0 * tw + (uint32_t)x1) * C + c];          \
                const REAL c01 = tex[((uint64_t)(uint32_t)y1 * tw + (uint32_t)x0) * C + c];          \
                const REAL c11 = tex[((uint64_t)(uint32_t)y1 * tw + (uint32_t)x1) * C + c];          \
                const REAL g = grad[p * C + c];                                                      \
                const REAL dx = ((REAL)1 - fy) * (c10 - c00) + fy * (c11 - c01);                     \
                const REAL dy = ((REAL)1 - fx) * (c01 - c00) + fx * (c11 - c10);                     \
                gx += g * (dx * (REAL)tw);                                                           \
                gy += g * (dy * (REAL)th);                                                           \
            }                                                                                        \
            grad_uv[p * 2] = gx;                                                                     \
            grad_uv[p * 2 + 1] = gy;                                                                 \
        }                                                                                            \
    }

static int texture_validate(uint32_t tw, uint32_t th, uint32_t C) {
    if (tw == 0 || th == 0 || C == 0) return ORA_INVALID;
    if (tw > 1073741823u || th > 1073741823u) return ORA_RANGE;
    return ORA_OK;
}

int ora_texture_backward(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                         const float* uv, const float* raster, uint64_t P, const float* grad,
                         float* grad_tex, float* grad_uv) {
    int rc = texture_validate(tw, th, C);
    if (rc) return rc;
#define UVPOS tx = uv[p * 2] * (float)tw - 0.5f; ty = uv[p * 2 + 1] * (float)th - 0.5f; \
    bx = f2i_sat(floorf(tx)); by = f2i_sat(floorf(ty)); fx = tx - floorf(tx); fy = ty - floorf(ty)
#define ACC(x) (x)
    TB_BODY(float)
#undef ACC
#undef UVPOS
    return ORA_OK;
}

int ora_texture_backward_f64(const float* tex, uint32_t tw, uint32_t th, uint32_t C, uint32_t mode,
                             const float* uv, const float* raster, uint64_t P, const float* grad,
                             double* grad_tex, double* grad_uv, int abs_terms) {
    int rc = texture_validate(tw, th, C);
    if (rc) return rc;
#define UVPOS tx = (double)uv[p * 2] * tw - 0.5; ty = (double)uv[p * 2 + 1] * th - 0.5; \
    bx = d2i_sat(floor(tx)); by = d2i_sat(floor(ty)); fx = tx - floor(tx); fy = ty - floor(ty)
#define ACC(x) (abs_terms ? fabs(x) : (x))
    TB_BODY(double)
#undef ACC
#undef UVPOS
    return ORA_OK;
}

/* Host threads the oracle's parallel loops use (0: all); results do not depend on it. */
void ora_set_threads(int threads) {
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
}

int ora_get_threads(void) { return omp_get_max_threads(); }

/* ---- transforms and softmax scale ---------------------------------------------------- */

void ora_transform_positions(const float* pos3, uint32_t V, const float m[16], float* clip4) {
    for (uint64_t v = 0; v < V; ++v) {
        const float x = pos3[v * 3], y = pos3[v * 3 + 1], z = pos3[v * 3 + 2];
        for (int r = 0; r < 4; ++r)
            clip4[v * 4 + r] = m[r * 4] * x + m[r * 4 + 1] * y + m[r * 4 + 2] * z + m[r * 4 + 3];
    }
}

float ora_suggest_softmax_scale(const float* pos, uint32_t V, const float* cams, uint32_t ncam) {
    if (V == 0 || ncam == 0) return 0.0f;
    const uint64_t stride = V / 10000 > 1 ? V / 10000 : 1;
    double best = INFINITY;
    for (uint64_t v = 0; v < V; v += stride) {
        const double x = pos[v * 3], y = pos[v * 3 + 1], z = pos[v * 3 + 2];
        if (!isfinite(x) || !isfinite(y) || !isfinite(z)) continue;
        for (uint32_t c = 0; c < ncam; ++c) {
            const double dx = cams[c * 3] - x, dy = cams[c * 3 + 1] - y, dz = cams[c * 3 + 2] - z;
            const double sq = dx * dx + dy * dy + dz * dz;
            best = sq < best ? sq : best;
        }
    }
    if (!isfinite(best) || best <= 0.0) return 0.0f;
    return (float)(20.0 * best);
}

/* ---- projection: shaders/project_texture.hlsl:26-247 --------------------------------- */

static float load_channel(const ora_project_params* pp, const float* photo, int32_t cx, int32_t cy, uint32_t ch) {
    const int32_t w = (int32_t)pp->image_width, h = (int32_t)pp->image_height;
    cx = clampi(cx, 0, w - 1);
    cy = clampi(cy, 0, h - 1);
    return photo[((uint64_t)(uint32_t)cy * pp->image_width + (uint32_t)cx) * pp->channel_count + ch];
}

static float sample_photo(const ora_project_params* pp, const float* photo, float ppx, float ppy, uint32_t ch) {
    const float tx = ppx - 0.5f, ty = ppy - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const float v00 = load_channel(pp, photo, bx, by, ch);
    const float v10 = load_channel(pp, photo, add1(bx), by, ch);
    const float v01 = load_channel(pp, photo, bx, add1(by), ch);
    const float v11 = load_channel(pp, photo, add1(bx), add1(by), ch);
    return lerpf_hlsl(lerpf_hlsl(v00, v10, fx), lerpf_hlsl(v01, v11, fx), fy);
}

static float sample_mask(const ora_project_params* pp, const float* mask, float ppx, float ppy) {
    const int32_t w = (int32_t)pp->image_width, h = (int32_t)pp->image_height;
    const float tx = ppx - 0.5f, ty = ppy - 0.5f;
    const int32_t bx = f2i_sat(floorf(tx)), by = f2i_sat(floorf(ty));
    const float fx = tx - floorf(tx), fy = ty - floorf(ty);
    const int32_t x0 = clampi(bx, 0, w - 1), x1 = clampi(add1(bx), 0, w - 1);
    const int32_t y0 = clampi(by, 0, h - 1), y1 = clampi(add1(by), 0, h - 1);
    const float v00 = mask[(uint64_t)y0 * pp->image_width + x0];
    const float v10 = mask[(uint64_t)y0 * pp->image_width + x1];
    const float v01 = mask[(uint64_t)y1 * pp->image_width + x0];
    const float v11 = mask[(uint64_t)y1 * pp->image_width + x1];
    return lerpf_hlsl(lerpf_hlsl(v00, v10, fx), lerpf_hlsl(v01, v11, fx), fy);
}

static float shadow_visibility(const ora_project_params* pp, const float* shadow, float ppx, float ppy,
                               float depth) {
    const int32_t w = (int32_t)pp->image_width, h = (int32_t)pp->image_height;
    const int32_t cx = f2i_sat(floorf(ppx)), cy = f2i_sat(floorf(ppy));
    const int32_t r = (int32_t)pp->pcf_radius;
    float visible = 0.0f, count = 0.0f;
    for (int32_t y = -r; y <= r; ++y) {
        for (int32_t x = -r; x <= r; ++x) {
            const int32_t X = cx + x, Y = cy + y;
            if (X < 0 || Y < 0 || X >= w || Y >= h) continue;
            const uint64_t off = ((uint64_t)Y * pp->image_width + (uint64_t)X) * 4;
            if (rid(shadow[off + 3]) != 0) {
                visible += depth <= shadow[off + 2] + pp->depth_bias ? 1.0f : 0.0f;
                count += 1.0f;
            }
        }
    }
    return count > 0.0f ? visible / count : 0.0f;
}

void ora_project_texture(const ora_project_params* pp, const float* apos, const float* anrm,
                         const float* araster, const float* shadow, const float* photo,
                         const float* mask, const float* rayvis, float* acc_color, float* acc_weight,
                         float* best_conf, uint32_t* source_view) {
    const uint64_t N = (uint64_t)pp->atlas_width * pp->atlas_height;
    const float* M = pp->world_to_clip;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        if (rid(araster[i * 4 + 3]) == 0) continue;
        const float px = apos[i * 3], py = apos[i * 3 + 1], pz = apos[i * 3 + 2];
        const float nx0 = anrm[i * 3], ny0 = anrm[i * 3 + 1], nz0 = anrm[i * 3 + 2];
        const float nl = sqrtf(nx0 * nx0 + ny0 * ny0 + nz0 * nz0);
        const float nx = nx0 / nl, ny = ny0 / nl, nz = nz0 / nl;
        const float cx = M[0] * px + M[1] * py + M[2] * pz + M[3] * 1.0f;
        const float cy = M[4] * px + M[5] * py + M[6] * pz + M[7] * 1.0f;
        const float cz = M[8] * px + M[9] * py + M[10] * pz + M[11] * 1.0f;
        const float cw = M[12] * px + M[13] * py + M[14] * pz + M[15] * 1.0f;
        if (cw <= 1e-8f) continue;
        const float ndx = cx / cw, ndy = cy / cw, ndz = cz / cw;
        if (ndx < -1.0f || ndy < -1.0f || ndx > 1.0f || ndy > 1.0f || ndz < -1.0f || ndz > 1.0f) continue;
        const float ppx = pp->viewport[0] + (ndx * 0.5f + 0.5f) * pp->viewport[2];
        const float ppy = pp->viewport[1] + (ndy * 0.5f + 0.5f) * pp->viewport[3];
        if (ppx < pp->viewport[0] || ppy < pp->viewport[1] || ppx >= pp->viewport[0] + pp->viewport[2] ||
            ppy >= pp->viewport[1] + pp->viewport[3])
            continue;
        float vis = rayvis[i];
        if (pp->visibility_mode == 0) vis = shadow_visibility(pp, shadow, ppx, ppy, ndz);
        else if (pp->visibility_mode == 1) vis *= shadow_visibility(pp, shadow, ppx, ppy, ndz);
        if (pp->has_mask) vis *= clampf_hlsl(sample_mask(pp, mask, ppx, ppy), 0.0f, 1.0f);
        const float vx0 = pp->camera_position[0] - px, vy0 = pp->camera_position[1] - py, vz0 = pp->camera_position[2] - pz;
        const float vl = sqrtf(vx0 * vx0 + vy0 * vy0 + vz0 * vz0);
        const float vx = vx0 / vl, vy = vy0 / vl, vz = vz0 / vl;
        const float cosv = nx * vx + ny * vy + nz * vz;
        if (cosv < pp->min_view_cosine || vis <= 0.0f) continue;
        const float c0 = sample_photo(pp, photo, ppx, ppy, 0);
        const float c1 = sample_photo(pp, photo, ppx, ppy, 1);
        const float c2 = sample_photo(pp, photo, ppx, ppy, 2);
        const float alpha = pp->channel_count == 4 ? sample_photo(pp, photo, ppx, ppy, 3) : 1.0f;
        if (pp->blend_mode == 2) {
            const float dist = fmaxf(sqrtf(vx0 * vx0 + vy0 * vy0 + vz0 * vz0), 1e-6f);
            const float footprint = cosv / (dist * dist);
            const float ex = clampf_hlsl(vis * alpha * footprint * pp->view_weight, 0.0f, 64.0f);
            const float prev = best_conf[i];
            const float cur = fmaxf(prev, ex);
            if (cur > prev) {
                const float rs = expf(prev - cur);
                acc_color[i * 3] *= rs;
                acc_color[i * 3 + 1] *= rs;
                acc_color[i * 3 + 2] *= rs;
                acc_weight[i] *= rs;
                best_conf[i] = cur;
            }
            if (ex >= prev) source_view[i] = pp->view_index;
            const float sw = expf(ex - cur);
            if (sw <= 0.0f) continue;
            acc_color[i * 3] += c0 * sw;
            acc_color[i * 3 + 1] += c1 * sw;
            acc_color[i * 3 + 2] += c2 * sw;
            acc_weight[i] += sw;
            continue;
        }
        const float conf = vis * alpha * cosv * pp->view_weight;
        if (conf <= 0.0f) continue;
        if (conf > best_conf[i]) {
            best_conf[i] = conf;
            source_view[i] = pp->view_index;
        }
        if (pp->blend_mode == 0) {
            if (conf >= acc_weight[i]) {
                acc_color[i * 3] = c0;
                acc_color[i * 3 + 1] = c1;
                acc_color[i * 3 + 2] = c2;
                acc_weight[i] = conf;
            }
        } else {
            acc_color[i * 3] += c0 * conf;
            acc_color[i * 3 + 1] += c1 * conf;
            acc_color[i * 3 + 2] += c2 * conf;
            acc_weight[i] += conf;
        }
    }
}

/* ---- bake host: src/texture_baker.cpp:156-361 (shadow-map visibility) ----------------- */

int ora_bake(const float* pos3, const float* nrm3, const float* uv2, uint32_t V, const uint32_t* idx,
             uint32_t T, const ora_view* views, uint32_t nviews, uint32_t aw, uint32_t ah,
             uint32_t blend_mode, uint32_t pcf_radius, float mask_floor, float softmax_scale,
             float* color4, float* confidence, uint32_t* source_view, float* valid_mask,
             float* coverage_mask, uint32_t* face_ids) {
    return ora_bake_ex(pos3, nrm3, uv2, V, idx, T, views, nviews, aw, ah, blend_mode, pcf_radius, mask_floor,
                       softmax_scale, 0, NULL, color4, confidence, source_view, valid_mask, coverage_mask, face_ids);
}

int ora_bake_ex(const float* pos3, const float* nrm3, const float* uv2, uint32_t V, const uint32_t* idx,
                uint32_t T, const ora_view* views, uint32_t nviews, uint32_t aw, uint32_t ah,
                uint32_t blend_mode, uint32_t pcf_radius, float mask_floor, float softmax_scale,
                uint32_t visibility_mode, const uint32_t* ray_bits,
                float* color4, float* confidence, uint32_t* source_view, float* valid_mask,
                float* coverage_mask, uint32_t* face_ids) {
    if (V == 0 || T == 0 || nviews == 0) return ORA_INVALID;
    for (uint64_t i = 0; i < (uint64_t)T * 3; ++i) if (idx[i] >= V) return ORA_RANGE;
    if (aw == 0 || ah == 0 || pcf_radius > 4 || !isfinite(mask_floor) || mask_floor < 0.0f || mask_floor > 1.0f)
        return ORA_INVALID;
    const uint64_t N = (uint64_t)aw * ah;
    float* aclip = (float*)malloc((size_t)V * 4 * sizeof(float));
    for (uint64_t v = 0; v < V; ++v) {
        aclip[v * 4 + 0] = uv2[v * 2 + 0] * 2.0f - 1.0f;
        aclip[v * 4 + 1] = uv2[v * 2 + 1] * 2.0f - 1.0f;
        aclip[v * 4 + 2] = 0.0f;
        aclip[v * 4 + 3] = 1.0f;
    }
    const float avp[4] = {0.0f, 0.0f, (float)aw, (float)ah};
    float* araster = (float*)malloc(N * 4 * sizeof(float));
    int rc = ora_rasterize_forward(aclip, V, idx, T, aw, ah, 0, 0, avp, araster, NULL);
    if (rc) { free(aclip); free(araster); return rc; }
    float* apos = (float*)malloc(N * 3 * sizeof(float));
    float* anrm = (float*)malloc(N * 3 * sizeof(float));
    ora_interpolate_forward(pos3, V, 3, idx, T, araster, N, apos);
    ora_interpolate_forward(nrm3, V, 3, idx, T, araster, N, anrm);
    for (uint64_t i = 0; i < N; ++i) {
        const float r = roundf(araster[i * 4 + 3]); /* std::round */
        coverage_mask[i] = r != 0.0f ? 1.0f : 0.0f;
        face_ids[i] = coverage_mask[i] > 0.5f ? (uint32_t)r - 1u : UINT32_MAX;
    }
    float scale = softmax_scale;
    if (blend_mode == 2 && (!(scale > 0.0f) || !isfinite(scale))) {
        float* cams = (float*)malloc((size_t)nviews * 3 * sizeof(float));
        for (uint32_t k = 0; k < nviews; ++k) memcpy(cams + k * 3, views[k].camera_position, 3 * sizeof(float));
        scale = ora_suggest_softmax_scale(pos3, V, cams, nviews);
        free(cams);
        if (!(scale > 0.0f) || !isfinite(scale)) scale = 1.0f;
    }
    float* acc = (float*)calloc(N * 3, sizeof(float));
    float* accw = (float*)calloc(N, sizeof(float));
    float* best = (float*)calloc(N, sizeof(float));
    float* rayvis = (float*)malloc(N * sizeof(float));
    for (uint64_t i = 0; i < N; ++i) { rayvis[i] = 1.0f; source_view[i] = UINT32_MAX; }
    float* clip = (float*)malloc((size_t)V * 4 * sizeof(float));
    for (uint32_t k = 0; k < nviews && rc == 0; ++k) {
        const ora_view* vw = &views[k];
        if (vw->width == 0 || vw->height == 0 || (vw->channel_count != 3 && vw->channel_count != 4)) { rc = ORA_INVALID; break; }
        if (!isfinite(vw->weight) || vw->weight < 0.0f || !isfinite(vw->depth_bias) || vw->depth_bias < 0.0f ||
            !isfinite(vw->min_view_cosine) || vw->min_view_cosine < -1.0f || vw->min_view_cosine > 1.0f) { rc = ORA_INVALID; break; }
        const float vvp[4] = {vw->has_viewport ? vw->viewport[0] : 0.0f, vw->has_viewport ? vw->viewport[1] : 0.0f,
                              vw->has_viewport ? vw->viewport[2] : (float)vw->width,
                              vw->has_viewport ? vw->viewport[3] : (float)vw->height};
        const uint64_t Pv = (uint64_t)vw->width * vw->height;
        ora_transform_positions(pos3, V, vw->world_to_clip, clip);
        float* shadow = (float*)malloc(Pv * 4 * sizeof(float));
        rc = ora_rasterize_forward(clip, V, idx, T, vw->width, vw->height, 0, 0, vvp, shadow, NULL);
        if (rc) { free(shadow); break; }
        float* floored = NULL;
        const float* mask = vw->visibility_mask;
        if (mask_floor > 0.0f && mask) {
            floored = (float*)malloc(Pv * sizeof(float));
            for (uint64_t i = 0; i < Pv; ++i) floored[i] = mask[i] < mask_floor ? mask_floor : mask[i];
            mask = floored;
        }
        ora_project_params pp;
        memcpy(pp.world_to_clip, vw->world_to_clip, sizeof(pp.world_to_clip));
        memcpy(pp.camera_position, vw->camera_position, sizeof(pp.camera_position));
        pp.view_weight = blend_mode == 2 ? vw->weight * scale : vw->weight;
        memcpy(pp.viewport, vvp, sizeof(vvp));
        pp.atlas_width = aw;
        pp.atlas_height = ah;
        pp.image_width = vw->width;
        pp.image_height = vw->height;
        pp.depth_bias = vw->depth_bias;
        pp.min_view_cosine = vw->min_view_cosine;
        pp.channel_count = vw->channel_count;
        pp.blend_mode = blend_mode;
        pp.pcf_radius = pcf_radius;
        pp.has_mask = vw->visibility_mask != NULL;
        pp.visibility_mode = ray_bits ? visibility_mode : 0;
        pp.view_index = k;
        if (ray_bits) {
            const uint32_t words = (nviews + 31) / 32;
            for (uint64_t i = 0; i < N; ++i) rayvis[i] = (float)((ray_bits[i * words + k / 32] >> (k % 32)) & 1u);
        }
        ora_project_texture(&pp, apos, anrm, araster, shadow, vw->image, mask, rayvis, acc, accw, best, source_view);
        free(floored);
        free(shadow);
    }
    if (rc == 0) {
        for (uint64_t i = 0; i < N; ++i) {
            const float w = accw[i];
            confidence[i] = w;
            valid_mask[i] = w > 0.0f ? 1.0f : 0.0f;
            const float div = blend_mode != 0 && w > 0.0f ? w : 1.0f;
            color4[i * 4 + 0] = acc[i * 3 + 0] / div;
            color4[i * 4 + 1] = acc[i * 3 + 1] / div;
            color4[i * 4 + 2] = acc[i * 3 + 2] / div;
            color4[i * 4 + 3] = valid_mask[i];
        }
    }
    free(clip); free(rayvis); free(best); free(accw); free(acc);
    free(apos); free(anrm); free(araster); free(aclip);
    return rc;
}

/* ---- atlas refinement kernels ------------------------------------------------------- */

static void clamp_layout(float u, float v, uint32_t tw, uint32_t th, uint32_t tx[4], float w[4]) {
    const float px = u * (float)tw - 0.5f, py = v * (float)th - 0.5f;
    const int32_t bx = f2i_sat(floorf(px)), by = f2i_sat(floorf(py));
    const float fx = px - floorf(px), fy = py - floorf(py);
    const uint32_t x0 = (uint32_t)clampi(bx, 0, (int32_t)tw - 1), x1 = (uint32_t)clampi(add1(bx), 0, (int32_t)tw - 1);
    const uint32_t y0 = (uint32_t)clampi(by, 0, (int32_t)th - 1), y1 = (uint32_t)clampi(add1(by), 0, (int32_t)th - 1);
    tx[0] = y0 * tw + x0;
    tx[1] = y0 * tw + x1;
    tx[2] = y1 * tw + x0;
    tx[3] = y1 * tw + x1;
    w[0] = (1.0f - fx) * (1.0f - fy);
    w[1] = fx * (1.0f - fy);
    w[2] = (1.0f - fx) * fy;
    w[3] = fx * fy;
}

/* Order in which the two refiner gradients visit pixels / seam pairs. The reference adds with
 * atomics, so on a GPU any order is one the reference may take; reversing it gives a second valid
 * accumulation order, and the two results bound the reference's own order noise. */
static int g_reverse_order = 0;
void ora_set_reverse_order(int reverse) { g_reverse_order = reverse != 0; }

/* atlas_photometric_gradient.hlsl:45-108: per-pixel math in pixel order; the loss is
 * reduced per 64-pixel group with the shader's tree, then groups in order. Threaded without changing
 * any sum: per-pixel loss terms in parallel, the gradient by texel-row owners that each visit all
 * pixels in order (every texel's sum keeps the sequential order), the loss tree sequentially. */
static void photometric_pixel(const float* tex, uint32_t tw, uint32_t th, const float* uv, const float* target,
                              uint32_t p, float eps, float m, float norm, uint32_t tx[4], float w[4], float og[3],
                              float* local) {
    clamp_layout(uv[(uint64_t)p * 2], uv[(uint64_t)p * 2 + 1], tw, th, tx, w);
    float l = 0.0f;
    for (uint32_t c = 0; c < 3; ++c) {
        float rendered = 0.0f;
        for (int k = 0; k < 4; ++k) rendered += tex[(uint64_t)tx[k] * 3 + c] * w[k];
        const float d = rendered - target[(uint64_t)p * 3 + c];
        const float robust = sqrtf(d * d + eps * eps);
        og[c] = d / robust * m * norm;
        l += robust * m * norm;
    }
    *local = l;
}

static float group_tree_sum(const float* local, uint64_t n) {
    float loss = 0.0f;
    float group[64];
    for (uint64_t g0 = 0; g0 < n; g0 += 64) {
        for (uint32_t gi = 0; gi < 64; ++gi) group[gi] = g0 + gi < n ? local[g0 + gi] : 0.0f;
        for (uint32_t stride = 32; stride > 0; stride >>= 1)
            for (uint32_t gi = 0; gi < stride; ++gi) group[gi] += group[gi + stride];
        if (group[0] != 0.0f) loss += group[0];
    }
    return loss;
}

float ora_photometric_gradient(const float* tex, uint32_t tw, uint32_t th, const float* uv,
                               const float* target, const float* mask, uint32_t P, float eps,
                               float norm, float* grad) {
    const int rev = g_reverse_order;
    float* local = (float*)malloc(((size_t)P + 1) * sizeof(float));  /* by visiting position */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)P; ++i) {
        const uint32_t p = rev ? P - 1 - (uint32_t)i : (uint32_t)i;
        local[i] = 0.0f;
        const float m = mask[p];
        if (m > 0.0f) {
            uint32_t tx[4];
            float w[4], og[3];
            photometric_pixel(tex, tw, th, uv, target, p, eps, m, norm, tx, w, og, &local[i]);
        }
    }
#pragma omp parallel
    {
        const uint32_t nt = (uint32_t)omp_get_num_threads(), tid = (uint32_t)omp_get_thread_num();
        const uint32_t y_lo = (uint32_t)((uint64_t)th * tid / nt), y_hi = (uint32_t)((uint64_t)th * (tid + 1) / nt);
        for (uint32_t i = 0; i < P && y_lo < y_hi; ++i) {
            const uint32_t p = rev ? P - 1 - i : i;
            const float m = mask[p];
            if (!(m > 0.0f)) continue;
            uint32_t tx[4];
            float w[4], og[3], l;
            clamp_layout(uv[(uint64_t)p * 2], uv[(uint64_t)p * 2 + 1], tw, th, tx, w);
            const uint32_t ya = tx[0] / tw, yb = tx[2] / tw;
            const int in0 = ya >= y_lo && ya < y_hi, in1 = yb >= y_lo && yb < y_hi;
            if (!in0 && !in1) continue;
            photometric_pixel(tex, tw, th, uv, target, p, eps, m, norm, tx, w, og, &l);
            for (uint32_t c = 0; c < 3; ++c)
                for (int k = 0; k < 4; ++k)
                    if (k < 2 ? in0 : in1) grad[(uint64_t)tx[k] * 3 + c] += og[c] * w[k];
        }
    }
    const float loss = group_tree_sum(local, P);
    free(local);
    return loss;
}

float ora_seam_gradient(const float* tex, uint32_t tw, uint32_t th, const float* pairs,
                        uint32_t npairs, float eps, float norm, float* grad) {
    const int rev = g_reverse_order;
    float* local = (float*)malloc(((size_t)npairs + 1) * sizeof(float));
    float* gs = (float*)malloc(((size_t)npairs * 3 + 1) * sizeof(float));
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)npairs; ++ii) {
        const uint32_t i = rev ? npairs - 1 - (uint32_t)ii : (uint32_t)ii;
        uint32_t t0[4], t1[4];
        float w0[4], w1[4];
        clamp_layout(pairs[(uint64_t)i * 4], pairs[(uint64_t)i * 4 + 1], tw, th, t0, w0);
        clamp_layout(pairs[(uint64_t)i * 4 + 2], pairs[(uint64_t)i * 4 + 3], tw, th, t1, w1);
        float l = 0.0f;
        for (uint32_t c = 0; c < 3; ++c) {
            float c0 = 0.0f, c1 = 0.0f;
            for (int k = 0; k < 4; ++k) {
                c0 += tex[(uint64_t)t0[k] * 3 + c] * w0[k];
                c1 += tex[(uint64_t)t1[k] * 3 + c] * w1[k];
            }
            const float d = c0 - c1;
            const float robust = sqrtf(d * d + eps * eps);
            gs[(uint64_t)i * 3 + c] = d / robust * norm;
            l += robust * norm;
        }
        local[ii] = l;
    }
#pragma omp parallel
    {
        const uint32_t nt = (uint32_t)omp_get_num_threads(), tid = (uint32_t)omp_get_thread_num();
        const uint32_t y_lo = (uint32_t)((uint64_t)th * tid / nt), y_hi = (uint32_t)((uint64_t)th * (tid + 1) / nt);
        for (uint32_t ii = 0; ii < npairs && y_lo < y_hi; ++ii) {
            const uint32_t i = rev ? npairs - 1 - ii : ii;
            uint32_t t0[4], t1[4];
            float w0[4], w1[4];
            clamp_layout(pairs[(uint64_t)i * 4], pairs[(uint64_t)i * 4 + 1], tw, th, t0, w0);
            clamp_layout(pairs[(uint64_t)i * 4 + 2], pairs[(uint64_t)i * 4 + 3], tw, th, t1, w1);
            for (uint32_t c = 0; c < 3; ++c) {
                const float g = gs[(uint64_t)i * 3 + c];
                for (int k = 0; k < 4; ++k) {
                    const uint32_t ya = t0[k] / tw, yb = t1[k] / tw;
                    if (ya >= y_lo && ya < y_hi) grad[(uint64_t)t0[k] * 3 + c] += g * w0[k];
                    if (yb >= y_lo && yb < y_hi) grad[(uint64_t)t1[k] * 3 + c] += -g * w1[k];
                }
            }
        }
    }
    const float loss = group_tree_sum(local, npairs);
    free(local);
    free(gs);
    return loss;
}

/* FP64 twins of the two refiner gradients: the same taps (texel positions and weights from the
 * fp32 uv, computed exactly in double), every product and sum in double. With abs_terms the gradient
 * accumulates |term| (the sum of absolute terms that bounds summation-order error). Return the loss. */
static void clamp_layout_f64(float u, float v, uint32_t tw, uint32_t th, uint32_t tx[4], double w[4]) {
    const double px = (double)u * tw - 0.5, py = (double)v * th - 0.5;
    const double flx = floor(px), fly = floor(py);
    const int32_t bx = d2i_sat(flx), by = d2i_sat(fly);
    const double fx = px - flx, fy = py - fly;
    const uint32_t x0 = (uint32_t)clampi(bx, 0, (int32_t)tw - 1), x1 = (uint32_t)clampi(add1(bx), 0, (int32_t)tw - 1);
    const uint32_t y0 = (uint32_t)clampi(by, 0, (int32_t)th - 1), y1 = (uint32_t)clampi(add1(by), 0, (int32_t)th - 1);
    tx[0] = y0 * tw + x0;
    tx[1] = y0 * tw + x1;
    tx[2] = y1 * tw + x0;
    tx[3] = y1 * tw + x1;
    w[0] = (1.0 - fx) * (1.0 - fy);
    w[1] = fx * (1.0 - fy);
    w[2] = (1.0 - fx) * fy;
    w[3] = fx * fy;
}

double ora_photometric_gradient_f64(const float* tex, uint32_t tw, uint32_t th, const float* uv,
                                    const float* target, const float* mask, uint32_t P, float eps,
                                    float norm, double* grad, int abs_terms) {
    double loss = 0.0;
    const double e = eps, n = norm;
    for (uint32_t p = 0; p < P; ++p) {
        const double m = mask[p];
        if (!(m > 0.0)) continue;
        uint32_t tx[4];
        double w[4];
        clamp_layout_f64(uv[(uint64_t)p * 2], uv[(uint64_t)p * 2 + 1], tw, th, tx, w);
        for (uint32_t c = 0; c < 3; ++c) {
            double rendered = 0.0;
            for (int k = 0; k < 4; ++k) rendered += (double)tex[(uint64_t)tx[k] * 3 + c] * w[k];
            const double d = rendered - target[(uint64_t)p * 3 + c];
            const double robust = sqrt(d * d + e * e);
            const double og = d / robust * m * n;
            loss += robust * m * n;
            for (int k = 0; k < 4; ++k) grad[(uint64_t)tx[k] * 3 + c] += abs_terms ? fabs(og * w[k]) : og * w[k];
        }
    }
    return loss;
}

double ora_seam_gradient_f64(const float* tex, uint32_t tw, uint32_t th, const float* pairs, uint32_t npairs,
                             float eps, float norm, double* grad, int abs_terms) {
    double loss = 0.0;
    const double e = eps, n = norm;
    for (uint32_t i = 0; i < npairs; ++i) {
        uint32_t t0[4], t1[4];
        double w0[4], w1[4];
        clamp_layout_f64(pairs[(uint64_t)i * 4], pairs[(uint64_t)i * 4 + 1], tw, th, t0, w0);
        clamp_layout_f64(pairs[(uint64_t)i * 4 + 2], pairs[(uint64_t)i * 4 + 3], tw, th, t1, w1);
        for (uint32_t c = 0; c < 3; ++c) {
            double c0 = 0.0, c1 = 0.0;
            for (int k = 0; k < 4; ++k) {
                c0 += (double)tex[(uint64_t)t0[k] * 3 + c] * w0[k];
                c1 += (double)tex[(uint64_t)t1[k] * 3 + c] * w1[k];
            }
            const double d = c0 - c1;
            const double robust = sqrt(d * d + e * e);
            const double g = d / robust * n;
            loss += robust * n;
            for (int k = 0; k < 4; ++k) {
                grad[(uint64_t)t0[k] * 3 + c] += abs_terms ? fabs(g * w0[k]) : g * w0[k];
                grad[(uint64_t)t1[k] * 3 + c] += abs_terms ? fabs(g * w1[k]) : -g * w1[k];
            }
        }
    }
    return loss;
}

/* atlas_adam_update.hlsl:20-43 */
void ora_adam_update(float* tex, float* grad, float* m, float* v, uint64_t n, float lr, float b1,
                     float b2, float eps, float bc1, float bc2, float cmin, float cmax) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float g = grad[i];
        const float m1 = b1 * m[i] + (1.0f - b1) * g;
        const float m2 = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = m1;
        v[i] = m2;
        const float c1 = m1 / bc1, c2 = m2 / bc2;
        tex[i] = clampf_hlsl(tex[i] - lr * c1 / (sqrtf(c2) + eps), cmin, cmax);
        grad[i] = 0.0f;
    }
}

/* texture_refiner.cpp:219-242 */
int ora_refine_view_cache(const float* pos3, const float* uv2, uint32_t V, const uint32_t* idx,
                          uint32_t T, const ora_view* vw, float* uv_out, float* target, float* mask,
                          double* valid_weight) {
    const uint64_t P = (uint64_t)vw->width * vw->height;
    const float vvp[4] = {vw->has_viewport ? vw->viewport[0] : 0.0f, vw->has_viewport ? vw->viewport[1] : 0.0f,
                          vw->has_viewport ? vw->viewport[2] : (float)vw->width,
                          vw->has_viewport ? vw->viewport[3] : (float)vw->height};
    float* clip = (float*)malloc((size_t)V * 4 * sizeof(float));
    ora_transform_positions(pos3, V, vw->world_to_clip, clip);
    float* raster = (float*)malloc(P * 4 * sizeof(float));
    int rc = ora_rasterize_forward(clip, V, idx, T, vw->width, vw->height, 0, 0, vvp, raster, NULL);
    if (rc) { free(clip); free(raster); return rc; }
    ora_interpolate_forward(uv2, V, 2, idx, T, raster, P, uv_out);
    double vwsum = 0.0;
    for (uint64_t p = 0; p < P; ++p) {
        target[p * 3] = vw->image[p * vw->channel_count];
        target[p * 3 + 1] = vw->image[p * vw->channel_count + 1];
        target[p * 3 + 2] = vw->image[p * vw->channel_count + 2];
        mask[p] = 0.0f;
        if (raster[p * 4 + 3] != 0.0f) {
            float ext = 1.0f;
            if (vw->visibility_mask) {
                const float m = vw->visibility_mask[p];
                ext = m < 0.0f ? 0.0f : (1.0f < m ? 1.0f : m); /* std::clamp */
            }
            mask[p] = ext;
            vwsum += ext;
        }
    }
    *valid_weight = vwsum;
    free(clip);
    free(raster);
    return ORA_OK;
}

int ora_refine(const float* init, const float* pos3, const float* uv2, uint32_t V, const uint32_t* idx,
               uint32_t T, const ora_view* views, uint32_t nviews, const float* pairs, uint32_t npairs,
               const ora_refine_options* o, float* out, float* loss_hist, float* seam_hist) {
    if (V == 0 || T == 0 || nviews == 0) return ORA_INVALID;
    for (uint64_t i = 0; i < (uint64_t)T * 3; ++i) if (idx[i] >= V) return ORA_INVALID;
    const uint64_t n = (uint64_t)o->width * o->height * 3;
    if (o->width == 0 || o->height == 0 || o->steps == 0 || o->batch_size == 0 ||
        !isfinite(o->learning_rate) || o->learning_rate <= 0.0f || !isfinite(o->minimum_learning_rate) ||
        o->minimum_learning_rate < 0.0f || o->minimum_learning_rate > o->learning_rate ||
        !isfinite(o->photometric_epsilon) || o->photometric_epsilon <= 0.0f ||
        !(o->adam_beta1 > 0.0f && o->adam_beta1 < 1.0f) || !(o->adam_beta2 > 0.0f && o->adam_beta2 < 1.0f) ||
        !(o->clamp_min < o->clamp_max) || !isfinite(o->seam_learning_rate) || o->seam_learning_rate <= 0.0f ||
        !isfinite(o->seam_epsilon) || o->seam_epsilon <= 0.0f)
        return ORA_INVALID;
    if (n > UINT32_MAX) return ORA_OVERFLOW;
    float** cuv = (float**)calloc(nviews, sizeof(float*));
    float** ctg = (float**)calloc(nviews, sizeof(float*));
    float** cmk = (float**)calloc(nviews, sizeof(float*));
    double* cvw = (double*)calloc(nviews, sizeof(double));
    int rc = ORA_OK;
    for (uint32_t k = 0; k < nviews && rc == 0; ++k) {
        const ora_view* vw = &views[k];
        if (vw->width == 0 || vw->height == 0 || (vw->channel_count != 3 && vw->channel_count != 4)) { rc = ORA_INVALID; break; }
        const uint64_t P = (uint64_t)vw->width * vw->height;
        cuv[k] = (float*)malloc(P * 2 * sizeof(float));
        ctg[k] = (float*)malloc(P * 3 * sizeof(float));
        cmk[k] = (float*)malloc(P * sizeof(float));
        rc = ora_refine_view_cache(pos3, uv2, V, idx, T, vw, cuv[k], ctg[k], cmk[k], &cvw[k]);
    }
    if (rc == 0) {
        memcpy(out, init, n * sizeof(float));
        float* g = (float*)calloc(n, sizeof(float));
        float* m = (float*)calloc(n, sizeof(float));
        float* v = (float*)calloc(n, sizeof(float));
        const float pi = acosf(-1.0f);
        for (uint32_t s = 0; s < o->steps; ++s) {
            double bvw = 0.0;
            for (uint32_t b = 0; b < o->batch_size; ++b) bvw += cvw[((uint64_t)s * o->batch_size + b) % nviews];
            const float norm = bvw > 0.0 ? (float)(1.0 / (bvw * 3.0)) : 0.0f;
            float loss = 0.0f;
            for (uint32_t b = 0; b < o->batch_size; ++b) {
                const uint32_t k = (uint32_t)(((uint64_t)s * o->batch_size + b) % nviews);
                loss += ora_photometric_gradient(out, o->width, o->height, cuv[k], ctg[k], cmk[k],
                                                 views[k].width * views[k].height, o->photometric_epsilon, norm, g);
            }
            loss_hist[s] = loss;
            const float phase = (float)s / (float)o->steps;
            const float lr = o->minimum_learning_rate +
                             0.5f * (o->learning_rate - o->minimum_learning_rate) * (1.0f + cosf(pi * phase));
            ora_adam_update(out, g, m, v, n, lr, o->adam_beta1, o->adam_beta2, o->adam_epsilon,
                            1.0f - powf(o->adam_beta1, (float)(s + 1)), 1.0f - powf(o->adam_beta2, (float)(s + 1)),
                            o->clamp_min, o->clamp_max);
        }
        const uint32_t seam_steps = npairs == 0 ? 0 : o->seam_polish_steps;
        if (seam_steps) {
            memset(g, 0, n * sizeof(float));
            memset(m, 0, n * sizeof(float));
            memset(v, 0, n * sizeof(float));
            for (uint32_t s = 0; s < seam_steps; ++s) {
                seam_hist[s] = ora_seam_gradient(out, o->width, o->height, pairs, npairs, o->seam_epsilon,
                                                 1.0f / (float)(npairs * 3u), g);
                ora_adam_update(out, g, m, v, n, o->seam_learning_rate, o->adam_beta1, o->adam_beta2, o->adam_epsilon,
                                1.0f - powf(o->adam_beta1, (float)(s + 1)), 1.0f - powf(o->adam_beta2, (float)(s + 1)),
                                o->clamp_min, o->clamp_max);
            }
        }
        free(g); free(m); free(v);
    }
    for (uint32_t k = 0; k < nviews; ++k) { free(cuv[k]); free(ctg[k]); free(cmk[k]); }
    free(cuv); free(ctg); free(cmk); free(cvw);
    return rc;
}

/* ---- chart-aware total variation: python/photara_drender/atlas.py:84-115 --------------- */

double ora_tv_gradient(const float* tex, uint32_t tw, uint32_t th, uint32_t C, const uint8_t* valid,
                       const int32_t* chart, float eps, float weight, float* grad) {
    uint64_t pairs = 0;
#pragma omp parallel for schedule(static) reduction(+ : pairs)
    for (uint32_t y = 0; y < th; ++y)
        for (uint32_t x = 0; x < tw; ++x) {
            const uint64_t i = (uint64_t)y * tw + x;
            if (x + 1 < tw && valid[i] && valid[i + 1] && (!chart || chart[i] == chart[i + 1])) pairs++;
            if (y + 1 < th && valid[i] && valid[i + tw] && (!chart || chart[i] == chart[i + tw])) pairs++;
        }
    const double denom = (double)(pairs > 0 ? pairs : 1) * C;
    const float scale = (float)((double)weight / denom);
    /* Texel-row owners: a thread owning rows [y_lo, y_hi) visits the pairs of rows y_lo - 1 .. y_hi - 1
     * in the sequential (row-major, right then down) order and updates only its own texels, so every
     * texel's sum keeps the sequential order. The loss (double) is summed per band, bands in order. */
    const uint32_t nbands = (uint32_t)omp_get_max_threads();
    double* band_loss = (double*)calloc(nbands, sizeof(double));
#pragma omp parallel num_threads(nbands)
    {
        const uint32_t nt = (uint32_t)omp_get_num_threads(), tid = (uint32_t)omp_get_thread_num();
        const uint32_t y_lo = (uint32_t)((uint64_t)th * tid / nt), y_hi = (uint32_t)((uint64_t)th * (tid + 1) / nt);
        double bl = 0.0;
        for (uint32_t y = y_lo > 0 ? y_lo - 1 : 0; y < y_hi; ++y)
            for (uint32_t x = 0; x < tw; ++x) {
                const uint64_t i = (uint64_t)y * tw + x;
                const int own_i = y >= y_lo;
                for (int dir = 0; dir < 2; ++dir) {
                    uint64_t j;
                    if (dir == 0) { if (x + 1 >= tw) continue; j = i + 1; }
                    else { if (y + 1 >= th) continue; j = i + tw; }
                    const int own_j = dir == 0 ? own_i : (y + 1 < y_hi);
                    if (!own_i && !own_j) continue;
                    if (!(valid[i] && valid[j] && (!chart || chart[i] == chart[j]))) continue;
                    for (uint32_t c = 0; c < C; ++c) {
                        const float d = tex[j * C + c] - tex[i * C + c];
                        const float r = sqrtf(d * d + eps * eps);
                        if (own_i) bl += r;
                        const float gg = d / r * scale;
                        if (own_j) grad[j * C + c] += gg;
                        if (own_i) grad[i * C + c] -= gg;
                    }
                }
            }
        band_loss[tid] = bl;
    }
    double loss = 0.0;
    for (uint32_t b = 0; b < nbands; ++b) loss += band_loss[b];
    free(band_loss);
    return loss * (double)weight / denom;
}

/* FP64 twin of ora_tv_gradient (abs_terms as above); returns the weighted loss. */
double ora_tv_gradient_f64(const float* tex, uint32_t tw, uint32_t th, uint32_t C, const uint8_t* valid,
                           const int32_t* chart, float eps, float weight, double* grad, int abs_terms) {
    uint64_t pairs = 0;
    for (uint32_t y = 0; y < th; ++y)
        for (uint32_t x = 0; x < tw; ++x) {
            const uint64_t i = (uint64_t)y * tw + x;
            if (x + 1 < tw && valid[i] && valid[i + 1] && (!chart || chart[i] == chart[i + 1])) pairs++;
            if (y + 1 < th && valid[i] && valid[i + tw] && (!chart || chart[i] == chart[i + tw])) pairs++;
        }
    const double scale = (double)weight / ((double)(pairs > 0 ? pairs : 1) * C);
    const double e = eps;
    double loss = 0.0;
    for (uint32_t y = 0; y < th; ++y)
        for (uint32_t x = 0; x < tw; ++x) {
            const uint64_t i = (uint64_t)y * tw + x;
            for (int dir = 0; dir < 2; ++dir) {
                uint64_t j;
                if (dir == 0) { if (x + 1 >= tw) continue; j = i + 1; }
                else { if (y + 1 >= th) continue; j = i + tw; }
                if (!(valid[i] && valid[j] && (!chart || chart[i] == chart[j]))) continue;
                for (uint32_t c = 0; c < C; ++c) {
                    const double d = (double)tex[j * C + c] - (double)tex[i * C + c];
                    const double r = sqrt(d * d + e * e);
                    loss += r * scale;
                    const double gg = d / r * scale;
                    grad[j * C + c] += abs_terms ? fabs(gg) : gg;
                    grad[i * C + c] += abs_terms ? fabs(gg) : -gg;
                }
            }
        }
    return loss;
}

/* ---- ray-query visibility ------------------------------------------------------------------ */

/* shaders/project_ray_visibility.hlsl:14-55 for one camera: the ray set-up in fp32 as the shader
 * writes it, then every triangle tested in double precision (Moller-Trumbore). State per texel: 1 when
 * the camera is visible, 0 when a triangle is hit with margin (barycentrics and t at least 1e-5 inside)
 * or the texel is not covered, -1 when a triangle lies within that margin of the ray without a clear
 * hit: a ray tracer may decide those texels either way. */
int ora_ray_visibility(const float* pos3, uint32_t V, const uint32_t* idx, uint32_t T, const float* apos,
                       const float* anrm, const float* araster, uint64_t N, const float camera[3], float bias,
                       int8_t* state) {
    if (!pos3 || !idx || !apos || !anrm || !araster || !camera || !state) return ORA_INVALID;
    for (uint64_t k = 0; k < (uint64_t)T * 3; ++k)
        if (idx[k] >= V) return ORA_RANGE;
    const double eps = 1e-5;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
        const uint64_t i = (uint64_t)ii;
        if (f2u_sat(rintf(araster[i * 4 + 3])) == 0) {
            state[i] = 0;
            continue;
        }
        const float px = apos[i * 3], py = apos[i * 3 + 1], pz = apos[i * 3 + 2];
        const float nx0 = anrm[i * 3], ny0 = anrm[i * 3 + 1], nz0 = anrm[i * 3 + 2];
        const float nl = sqrtf(nx0 * nx0 + ny0 * ny0 + nz0 * nz0);
        const float nx = nx0 / nl, ny = ny0 / nl, nz = nz0 / nl;
        const float vx = camera[0] - px, vy = camera[1] - py, vz = camera[2] - pz;
        const float dist = sqrtf(vx * vx + vy * vy + vz * vz);
        if (dist <= bias * 2.0f) {
            state[i] = 1;
            continue;
        }
        const float dxf = vx / dist, dyf = vy / dist, dzf = vz / dist;
        const float sgn = (nx * dxf + ny * dyf + nz * dzf) >= 0.0f ? 1.0f : -1.0f;
        const double ox = px + nx * (bias * sgn), oy = py + ny * (bias * sgn), oz = pz + nz * (bias * sgn);
        const double dx = dxf, dy = dyf, dz = dzf;
        const double t0 = bias;
        const double t1 = fmaxf(bias, dist - bias * 2.0f);
        int hit = 0, near = 0;
        for (uint32_t t = 0; t < T && !hit; ++t) {
            const float* a = pos3 + (size_t)idx[t * 3] * 3;
            const float* b = pos3 + (size_t)idx[t * 3 + 1] * 3;
            const float* c = pos3 + (size_t)idx[t * 3 + 2] * 3;
            const double e1x = (double)b[0] - a[0], e1y = (double)b[1] - a[1], e1z = (double)b[2] - a[2];
            const double e2x = (double)c[0] - a[0], e2y = (double)c[1] - a[1], e2z = (double)c[2] - a[2];
            const double qx0 = dy * e2z - dz * e2y, qy0 = dz * e2x - dx * e2z, qz0 = dx * e2y - dy * e2x;
            const double det = e1x * qx0 + e1y * qy0 + e1z * qz0;
            if (det == 0.0) continue;
            const double inv = 1.0 / det;
            const double sx = ox - a[0], sy = oy - a[1], sz = oz - a[2];
            const double u = (sx * qx0 + sy * qy0 + sz * qz0) * inv;
            const double rx = sy * e1z - sz * e1y, ry = sz * e1x - sx * e1z, rz = sx * e1y - sy * e1x;
            const double v = (dx * rx + dy * ry + dz * rz) * inv;
            const double tt = (e2x * rx + e2y * ry + e2z * rz) * inv;
            const double te = eps * (fabs(tt) > 1.0 ? fabs(tt) : 1.0);
            if (u > eps && v > eps && u + v < 1.0 - eps && tt > t0 + te && tt < t1 - te) hit = 1;
            else if (u > -eps && v > -eps && u + v < 1.0 + eps && tt > t0 - te && tt < t1 + te) near = 1;
        }
        state[i] = hit ? 0 : (near ? -1 : 1);
    }
    return 0;
}

/* ---- atlas padding and surface fill: src/texture_padding.cpp:37-351 --------------------- */

#define ORA_PAD_FAR 12000 /* texture_padding.cpp:20, offset of texels with no source yet */
#define ORA_PAD_MAX_SIDE 16384 /* texture_padding.cpp:18, offsets are clamped to +-this */

typedef struct {
    int32_t w, h;
    int16_t* ox;
    int16_t* oy;
} ora_field;

/* One relaxation step of texture_padding.cpp:54-78: adopt the neighbour's nearest source when it is
 * strictly closer (squared length of the offset; ties keep the current one). */
static void ora_relax(ora_field* f, int32_t x, int32_t y, int32_t nx, int32_t ny) {
    if (nx < 0 || ny < 0 || nx >= f->w || ny >= f->h) return;
    const uint64_t c = (uint64_t)y * (uint64_t)f->w + (uint64_t)x;
    const uint64_t n = (uint64_t)ny * (uint64_t)f->w + (uint64_t)nx;
    const int32_t cx = (int32_t)f->ox[n] + (nx - x), cy = (int32_t)f->oy[n] + (ny - y);
    const int64_t cand = (int64_t)cx * cx + (int64_t)cy * cy;
    const int64_t cur = (int64_t)f->ox[c] * f->ox[c] + (int64_t)f->oy[c] * f->oy[c];
    if (cand >= cur) return;
    f->ox[c] = (int16_t)clampi(cx, -ORA_PAD_MAX_SIDE, ORA_PAD_MAX_SIDE);
    f->oy[c] = (int16_t)clampi(cy, -ORA_PAD_MAX_SIDE, ORA_PAD_MAX_SIDE);
}

/* texture_padding.cpp:37-95: Danielsson 8SSEDT, one raster-order sweep and one reverse sweep. */
static void ora_nearest_field(ora_field* f, const float* source_mask, float threshold) {
    const uint64_t n = (uint64_t)f->w * (uint64_t)f->h;
    for (uint64_t i = 0; i < n; ++i) {
        const int src = source_mask[i] >= threshold;
        f->ox[i] = src ? 0 : ORA_PAD_FAR;
        f->oy[i] = src ? 0 : ORA_PAD_FAR;
    }
    for (int32_t y = 0; y < f->h; ++y)
        for (int32_t x = 0; x < f->w; ++x) {
            ora_relax(f, x, y, x - 1, y);
            ora_relax(f, x, y, x, y - 1);
            ora_relax(f, x, y, x - 1, y - 1);
            ora_relax(f, x, y, x + 1, y - 1);
        }
    for (int32_t y = f->h - 1; y >= 0; --y)
        for (int32_t x = f->w - 1; x >= 0; --x) {
            ora_relax(f, x, y, x + 1, y);
            ora_relax(f, x, y, x, y + 1);
            ora_relax(f, x, y, x + 1, y + 1);
            ora_relax(f, x, y, x - 1, y + 1);
        }
}

int ora_nearest_field_offsets(const float* source_mask, uint32_t width, uint32_t height, float threshold,
                              int16_t* offset_x, int16_t* offset_y) {
    if (width == 0 || height == 0 || width > ORA_PAD_MAX_SIDE || height > ORA_PAD_MAX_SIDE) return ORA_INVALID;
    ora_field f = {(int32_t)width, (int32_t)height, offset_x, offset_y};
    ora_nearest_field(&f, source_mask, threshold);
    return ORA_OK;
}

int ora_pad_texture_atlas(float* color, uint32_t channels, const float* valid, const float* coverage, float* filled,
                          uint32_t width, uint32_t height, uint32_t margin, int fill_unobserved,
                          uint32_t maximum_fill_distance, float threshold, uint64_t stats[5], int* reason) {
    /* texture_padding.cpp:226-351; stats = valid, gutter, unobserved, remaining_unobserved, filled */
    *reason = 0;
    for (int k = 0; k < 5; ++k) stats[k] = 0;
    if (width == 0 || height == 0) { *reason = 1; return ORA_INVALID; }
    if (width > ORA_PAD_MAX_SIDE || height > ORA_PAD_MAX_SIDE) { *reason = 2; return ORA_INVALID; }
    if (channels != 3 && channels != 4) { *reason = 4; return ORA_INVALID; }
    if (!isfinite(threshold) || threshold <= 0.0f || threshold > 1.0f) { *reason = 6; return ORA_INVALID; }
    const uint64_t n = (uint64_t)width * height;
    float* source = (float*)malloc(n * sizeof(float));
    memcpy(source, valid, n * sizeof(float));
    for (uint64_t i = 0; i < n; ++i) {
        if (valid[i] >= threshold) {
            ++stats[0];
        } else if (filled[i] > 0.5f && coverage && coverage[i] > 0.5f) {
            source[i] = 1.0f;
            ++stats[2];
            ++stats[4];
        } else {
            filled[i] = 0.0f;
        }
    }
    if (stats[0] == 0 && stats[4] == 0) { free(source); return ORA_OK; }
    ora_field f = {(int32_t)width, (int32_t)height, (int16_t*)malloc(n * 2), (int16_t*)malloc(n * 2)};
    ora_nearest_field(&f, source, threshold);
    const int64_t margin2 = (int64_t)margin * margin;
    const int64_t limit2 = maximum_fill_distance == 0 ? INT64_MAX
                                                       : (int64_t)maximum_fill_distance * maximum_fill_distance;
    const int64_t none2 = 2LL * ORA_PAD_FAR * ORA_PAD_FAR;
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) {
            const uint64_t p = (uint64_t)y * width + x;
            if (source[p] >= threshold) continue;
            const int32_t ox = f.ox[p], oy = f.oy[p];
            const int64_t d2 = (int64_t)ox * ox + (int64_t)oy * oy;
            if (d2 >= none2) continue;
            const int32_t sx = (int32_t)x + ox, sy = (int32_t)y + oy;
            if (sx < 0 || sy < 0 || sx >= (int32_t)width || sy >= (int32_t)height) continue;
            const uint64_t s = (uint64_t)sy * width + (uint32_t)sx;
            const int covered = coverage && coverage[p] > 0.5f;
            int fill = 0;
            if (!covered) fill = margin > 0 && d2 <= margin2;
            else if (fill_unobserved) fill = d2 <= limit2;
            if (!fill) {
                if (covered) ++stats[3];
                continue;
            }
            for (uint32_t c = 0; c < channels; ++c) color[p * channels + c] = color[s * channels + c];
            if (channels == 4) color[p * 4 + 3] = 1.0f;
            filled[p] = 1.0f;
            ++stats[4];
            ++stats[covered ? 2 : 1];
        }
    free(f.ox);
    free(f.oy);
    free(source);
    return ORA_OK;
}

typedef struct {
    uint64_t key;
    uint32_t face, slot;
} ora_edge;

static int ora_edge_cmp(const void* a, const void* b) {
    const uint64_t x = ((const ora_edge*)a)->key, y = ((const ora_edge*)b)->key;
    return x < y ? -1 : x > y;
}

int ora_fill_texture_on_surface(float* color, uint32_t channels, const float* valid, const uint32_t* face_ids,
                                float* filled, uint32_t width, uint32_t height, const uint32_t* indices,
                                uint32_t triangle_count, uint64_t stats[4], int* reason) {
    /* texture_padding.cpp:100-184; stats = filled, remaining, measured faces, propagated faces */
    const uint32_t none = 0xFFFFFFFFu;
    const uint64_t n = (uint64_t)width * height;
    *reason = 0;
    for (int k = 0; k < 4; ++k) stats[k] = 0;
    if (n == 0 || triangle_count == 0) { *reason = 1; return ORA_INVALID; }
    if (channels != 3 && channels != 4) { *reason = 2; return ORA_INVALID; }
    if (triangle_count >= none) { *reason = 3; return ORA_INVALID; }
    const uint32_t faces = triangle_count;
    double* means = (double*)calloc((size_t)faces * 3, sizeof(double));
    uint32_t* counts = (uint32_t*)calloc(faces, sizeof(uint32_t));
    for (uint64_t p = 0; p < n; ++p) {
        const uint32_t f = face_ids[p];
        if (f == none) continue;
        if (f >= faces) { *reason = 4; free(means); free(counts); return ORA_INVALID; }
        if (valid[p] < 0.5f) continue;
        ++counts[f];
        for (int c = 0; c < 3; ++c) means[(uint64_t)f * 3 + c] += color[p * channels + c];
    }
    ora_edge* edges = (ora_edge*)malloc((size_t)faces * 3 * sizeof(ora_edge));
    for (uint32_t f = 0; f < faces; ++f)
        for (uint32_t e = 0; e < 3; ++e) {
            const uint32_t a = indices[(uint64_t)f * 3 + e], b = indices[(uint64_t)f * 3 + (e + 1) % 3];
            if (a == b) { *reason = 5; free(means); free(counts); free(edges); return ORA_INVALID; }
            const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            edges[(uint64_t)f * 3 + e] = (ora_edge){((uint64_t)lo << 32) | hi, f, e};
        }
    qsort(edges, (size_t)faces * 3, sizeof(ora_edge), ora_edge_cmp);
    uint32_t* nb = (uint32_t*)malloc((size_t)faces * 3 * sizeof(uint32_t));
    for (uint64_t i = 0; i < (uint64_t)faces * 3; ++i) nb[i] = none;
    for (uint64_t b = 0; b < (uint64_t)faces * 3;) {
        uint64_t e = b + 1;
        while (e < (uint64_t)faces * 3 && edges[e].key == edges[b].key) ++e;
        if (e - b > 2) { *reason = 6; free(means); free(counts); free(edges); free(nb); return ORA_INVALID; }
        if (e - b == 2) {
            nb[(uint64_t)edges[b].face * 3 + edges[b].slot] = edges[b + 1].face;
            nb[(uint64_t)edges[b + 1].face * 3 + edges[b + 1].slot] = edges[b].face;
        }
        b = e;
    }
    free(edges);
    uint32_t* sources = (uint32_t*)malloc((size_t)faces * sizeof(uint32_t));
    uint32_t* queue = (uint32_t*)malloc((size_t)faces * sizeof(uint32_t));
    uint64_t tail = 0;
    for (uint32_t f = 0; f < faces; ++f) {
        sources[f] = none;
        if (counts[f] == 0) continue;
        for (int c = 0; c < 3; ++c) means[(uint64_t)f * 3 + c] /= counts[f];
        sources[f] = f;
        queue[tail++] = f;
        ++stats[2];
    }
    for (uint64_t head = 0; head < tail; ++head) {
        const uint32_t f = queue[head];
        for (int s = 0; s < 3; ++s) {
            const uint32_t g = nb[(uint64_t)f * 3 + s];
            if (g == none || sources[g] != none) continue;
            sources[g] = sources[f];
            queue[tail++] = g;
            ++stats[3];
        }
    }
    for (uint64_t p = 0; p < n; ++p) {
        const uint32_t f = face_ids[p];
        if (f == none || valid[p] >= 0.5f) continue;
        const uint32_t s = sources[f];
        if (s == none) { ++stats[1]; continue; }
        for (int c = 0; c < 3; ++c) color[p * channels + c] = (float)means[(uint64_t)s * 3 + c];
        if (channels == 4) color[p * 4 + 3] = 1.0f;
        filled[p] = 1.0f;
        ++stats[0];
    }
    free(means); free(counts); free(nb); free(sources); free(queue);
    return ORA_OK;
}
