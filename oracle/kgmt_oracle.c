/*
 * kgmt_oracle.c -- CPU restatement of the KGMT planning loop (test
 * infrastructure only; see kgmt_oracle.h).  Build with -ffp-contract=off:
 * the FP32 mirror depends on every multiply and add being rounded on its own.
 *
 * Semantics fixed relative to the reference (each is a documented decision):
 *  - sampling: counter-based Philox4x32-10 (Salmon et al., SC'11) keyed by the
 *    query seed, counter (slot or node, iteration, domain, block); replaces the
 *    wall-clock-seeded curand XORWOW of Planner.cu:37-50 / KGMT.cu:80-81;
 *  - uniforms in (0,1] like curand_uniform: u = ((x >> 8) + 1) * 2^-24;
 *  - fine-cell first visits are tested against the marks as they stood at the
 *    start of the iteration (the reference races, KGMT.cu:254-255);
 *  - every expanded frontier node leaves the frontier (kernel1 semantics,
 *    KGMT.cu:232; kernel2 clears the wrong flags at KGMT.cu:271);
 *  - all regions are scored, the total is summed in a fixed order
 *    (KO_SCORE_LANES strided lanes then a halving tree), reset every
 *    iteration (Graph.cu:314 skips the last region, Graph.cu:266/285 lose
 *    partial sums);
 *  - the goal node is the smallest new tree index within the goal radius
 *    (KGMT.cu:342-361 lets every such thread race);
 *  - re-activation draws are fresh each iteration (KGMT.cu:371-372 reuses one);
 *  - the fine cell is located relative to the exact coarse-cell corner
 *    (Graph.cu:85-95 overwrites neighbouring corners for the 6-D model);
 *  - capacity: samples per entry S' = min(S, free / R); when that is 0 the
 *    first `free` entries get one sample each; a full tree stops the query
 *    (KGMT.cu:183-193 overflows instead);
 *  - steps k = min_steps + (int)(u * (max_steps - min_steps + 1)) clamped to
 *    max_steps (statePropagator.cu:81 can give MAX+1 when u == 1).
 */
#include "kgmt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As   */
/* Easy as 1, 2, 3", SC'11.  Multipliers and Weyl key increments from the   */
/* paper.                                                                    */
/* ------------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void ko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for(int round = 0; round < 10; ++round)
        {
            uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
            uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
            uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
            uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
            uint32_t n0 = hi1 ^ c1 ^ k0;
            uint32_t n2 = hi0 ^ c3 ^ k1;
            c0 = n0;
            c1 = lo1;
            c2 = n2;
            c3 = lo0;
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

float ko_u01(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1.0p-24f; }

void ko_sample_uniforms(uint64_t seed, uint32_t slot, uint32_t itr, float u[8])
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t out[4];
    for(uint32_t blk = 0; blk < 2; ++blk)
        {
            uint32_t ctr[4] = {slot, itr, 0u, blk};
            ko_philox4x32_10(ctr, key, out);
            for(int i = 0; i < 4; ++i) u[blk * 4 + i] = ko_u01(out[i]);
        }
}

float ko_react_uniform(uint64_t seed, uint32_t node, uint32_t itr)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {node, itr, 1u, 0u};
    uint32_t out[4];
    ko_philox4x32_10(ctr, key, out);
    return ko_u01(out[0]);
}

/* ------------------------------------------------------------------------ */
/* Portable single-precision sine/cosine.  Cody & Waite argument reduction   */
/* by pi/2 split in three parts (first two short enough that n*P1 and n*P2   */
/* are exact for |n| < 2^13), then minimax polynomials on |r| <= pi/4 in     */
/* Horner form: sin r = r + r^3 (S1 + S2 r^2 + S3 r^4) and                   */
/* cos r = 1 - r^2/2 + r^4 (C2 + C3 r^2 + C4 r^4), fitted by Lawson's        */
/* iteratively reweighted least squares (fit_sincos.py) and rounded to      */
/* float.  Same operations, same order on CPU and GPU, so both round        */
/* identically.                                                              */
/* ------------------------------------------------------------------------ */
#define KO_TWO_OVER_PI 0x1.45f306p-1f
#define KO_PIO2_1 0x1.92p+0f
#define KO_PIO2_2 0x1.fb4p-12f
#define KO_PIO2_3 0x1.4442d2p-24f
#define KO_S1 (-0x1.555546p-3f)
#define KO_S2 0x1.11073ap-7f
#define KO_S3 (-0x1.9943ep-13f)
#define KO_C1 (-0x1.0p-1f)
#define KO_C2 0x1.55554ap-5f
#define KO_C3 (-0x1.6c0c34p-10f)
#define KO_C4 0x1.99eba6p-16f

void ko_sincosf(float x, float* s_out, float* c_out)
{
    /* fused multiply-adds (fmaf, one rounding each) in the same places as the
     * CUDA kernels */
    /* n = nearest integer to x * 2/pi by adding 1.5 * 2^23 (the sum rounds to
     * an integer as rintf does while |x * 2/pi| < 2^22; beyond, the same
     * value as the kernels); the sum's two lowest bits are n mod 4 */
    float t = x * KO_TWO_OVER_PI;
    t = t + 0x1.8p23f;
    float n = t - 0x1.8p23f;
    uint32_t tb;
    memcpy(&tb, &t, sizeof tb);
    int q = (int)(tb & 3u);
    float r = fmaf(-n, KO_PIO2_1, x);
    r = fmaf(-n, KO_PIO2_2, r);
    r = fmaf(-n, KO_PIO2_3, r);
    float r2 = r * r;
    float ps = fmaf(r2, KO_S3, KO_S2);
    ps = fmaf(r2, ps, KO_S1);
    float sp = fmaf(r * r2, ps, r);
    float pc = fmaf(r2, KO_C4, KO_C3);
    pc = fmaf(r2, pc, KO_C2);
    pc = fmaf(r2, pc, KO_C1);
    float cp = fmaf(r2, pc, 1.0f);
    float s, c;
    switch(q)
        {
            case 0: s = sp, c = cp; break;
            case 1: s = cp, c = -sp; break;
            case 2: s = -sp, c = -cp; break;
            default: s = -cp, c = sp; break;
        }
    *s_out = s;
    *c_out = c;
}

/* Checks, over every float of the binades [1, 2) and (-2, -1], that
 * RN(c_hi * x + RN(c_lo * x)) (one fused multiply-add) equals the IEEE
 * quotient x / 6, with c_hi = RN(1/6), c_lo = RN(1/6 - c_hi): the division
 * replacement the CUDA kernels use.  The identity is invariant under scaling
 * by powers of two while c_lo * x stays normal, so one binade proves it for
 * all finite |x| > 2^-98.  Returns the number of mismatches. */
long ko_check_div6(void)
{
    const float ch = 0x1.555556p-3f, cl = -0x1.555556p-28f;
    long bad = 0;
    for(uint32_t m = 0; m < (1u << 23); ++m)
        {
            uint32_t bits = 0x3f800000u | m;
            float x;
            memcpy(&x, &bits, 4);
            for(int sg = 0; sg < 2; ++sg)
                {
                    float xx = sg ? -x : x;
                    if(fmaf(ch, xx, cl * xx) != xx / 6.0f) ++bad;
                }
        }
    return bad;
}

/* SAMPLE_DIM / STATE_DIM per model (statePropagator.cu rows x1[...]) */
int ko_sample_dim(int32_t model) { return model == KO_MODEL_QUADROTOR ? 17 : model == KO_MODEL_UNICYCLE ? 7 : 10; }
int ko_state_dim(int32_t model) { return model == KO_MODEL_QUADROTOR ? 12 : model == KO_MODEL_UNICYCLE ? 4 : 6; }
int ko_ws_dims(int32_t model) { return model == KO_MODEL_UNICYCLE ? 2 : 3; }

/* ------------------------------------------------------------------------ */
/* Regions (workspace-only grids).  Graph.cu:99-153 (getRegion: z least     */
/* significant) and Graph.cu:155-205 (getSubRegion).                        */
/* ------------------------------------------------------------------------ */
static inline int cell_index(float t, int len)
{
    if(!(t >= 0.0f)) return 0; /* negative or NaN */
    if(t >= (float)len) return len - 1;
    int i = (int)t;
    return i > len - 1 ? len - 1 : i;
}

/* W workspace digits, x most significant: r1 = ix*L + iy (W = 2) or
 * (ix*L + iy)*L + iz (W = 3), Graph.cu:105-113 */
static void coarse_idx(const ko_config* c, const float* x, int idx[3])
{
    float range = c->ws_max - c->ws_min;
    float L = (float)c->coarse_len;
    int w = ko_ws_dims(c->model);
    for(int d = 0; d < w; ++d)
        {
            float t = (L * (x[d] - c->ws_min)) / range;
            idx[d] = cell_index(t, (int)c->coarse_len);
        }
}

int ko_region(const ko_config* c, const float* x)
{
    int idx[3];
    coarse_idx(c, x, idx);
    int L = (int)c->coarse_len;
    if(ko_ws_dims(c->model) == 2) return idx[0] * L + idx[1];
    return (idx[0] * L + idx[1]) * L + idx[2];
}

int ko_subregion(const ko_config* c, const float* x, int r1)
{
    int L = (int)c->coarse_len;
    int w = ko_ws_dims(c->model);
    int idx[3];
    if(w == 2) idx[0] = r1 / L, idx[1] = r1 % L;
    else idx[0] = r1 / (L * L), idx[1] = (r1 / L) % L, idx[2] = r1 % L;
    float size1 = (c->ws_max - c->ws_min) / (float)c->coarse_len;
    float L2 = (float)c->fine_len;
    int j[3];
    for(int d = 0; d < w; ++d)
        {
            float minr = c->ws_min + (float)idx[d] * size1;
            float t = (L2 * (x[d] - minr)) / size1;
            j[d] = cell_index(t, (int)c->fine_len);
        }
    int F = (int)c->fine_len;
    if(w == 2) return j[0] * F + j[1];
    return (j[0] * F + j[1]) * F + j[2];
}

/* helper.cuh:138-152 over the first w components */
float ko_distance_w(const float* a, const float* b, int w)
{
    float dx = a[0] - b[0], dy = a[1] - b[1];
    float s = dx * dx + dy * dy;
    if(w == 3)
        {
            float dz = a[2] - b[2];
            s = s + dz * dz;
        }
    return sqrtf(s);
}

float ko_distance(const float* a, const float* b) { return ko_distance_w(a, b, 3); }

/* ------------------------------------------------------------------------ */
/* Collision: collisionCheck.cu:3-10 (separated iff bbMax <= obsMin or      */
/* obsMax <= bbMin on some axis; touching counts as free) and 49-61.        */
/* ------------------------------------------------------------------------ */
/* w: workspace dimension; boxes are rows of 2w floats */
static int motion_valid_f(const float* p0, const float* p1, const float* obs, uint32_t n_obs, int w)
{
    float bmin[3], bmax[3];
    for(int d = 0; d < w; ++d)
        {
            if(p0[d] > p1[d]) bmin[d] = p1[d], bmax[d] = p0[d];
            else bmin[d] = p0[d], bmax[d] = p1[d];
        }
    for(uint32_t o = 0; o < n_obs; ++o)
        {
            const float* b = obs + 2 * w * (size_t)o;
            int sep = 0;
            for(int d = 0; d < w; ++d)
                if(bmax[d] <= b[d] || b[w + d] <= bmin[d]) sep = 1;
            if(!sep) return 0;
        }
    return 1;
}

int ko_segment_valid(const float* p0, const float* p1, const float* obstacles, uint32_t n_obs)
{
    return motion_valid_f(p0, p1, obstacles, n_obs, 3);
}

static int motion_valid_d(const double* p0, const double* p1, const float* obs, uint32_t n_obs, int w)
{
    double bmin[3], bmax[3];
    for(int d = 0; d < w; ++d)
        {
            if(p0[d] > p1[d]) bmin[d] = p1[d], bmax[d] = p0[d];
            else bmin[d] = p0[d], bmax[d] = p1[d];
        }
    for(uint32_t o = 0; o < n_obs; ++o)
        {
            const float* b = obs + 2 * w * (size_t)o;
            int sep = 0;
            for(int d = 0; d < w; ++d)
                if(bmax[d] <= (double)b[d] || (double)b[w + d] <= bmin[d]) sep = 1;
            if(!sep) return 0;
        }
    return 1;
}

/* distance of a state to the velocity and workspace thresholds */
static double bound_margin_d(const ko_config* c, const double* pos, const double* vel)
{
    double m = 1e30;
    for(int d = 0; d < 3; ++d)
        {
            double t[4] = {fabs(vel[d] - c->v_min), fabs(vel[d] - c->v_max), fabs(pos[d] - c->ws_min), fabs(pos[d] - c->ws_max)};
            for(int i = 0; i < 4; ++i)
                if(t[i] < m) m = t[i];
        }
    return m;
}

/* distance of a value to a closed interval's two ends */
static double end_margin_d(double x, double lo, double hi)
{
    double a = fabs(x - lo), b = fabs(x - hi);
    return a < b ? a : b;
}

static double face_margin_d(const double* p0, const double* p1, const float* obs, uint32_t n_obs, int w)
{
    double bmin[3], bmax[3], m = 1e30;
    for(int d = 0; d < w; ++d)
        {
            if(p0[d] > p1[d]) bmin[d] = p1[d], bmax[d] = p0[d];
            else bmin[d] = p0[d], bmax[d] = p1[d];
        }
    /* signed separation of the step box from a box: max over axes of
     * max(obsMin - bbMax, bbMin - obsMax); the verdict for that box flips
     * only when it crosses zero */
    for(uint32_t o = 0; o < n_obs; ++o)
        {
            const float* b = obs + 2 * w * (size_t)o;
            double sep = -1e30;
            for(int d = 0; d < w; ++d)
                {
                    double a1 = (double)b[d] - bmax[d];
                    double a2 = bmin[d] - (double)b[w + d];
                    double s = a1 > a2 ? a1 : a2;
                    if(s > sep) sep = s;
                }
            if(fabs(sep) < m) m = fabs(sep);
        }
    return m;
}

/* ------------------------------------------------------------------------ */
/* Controls and step count (statePropagator.cu:78-81, 248-253).             */
/* ------------------------------------------------------------------------ */
static int ctrl_count(const ko_config* c) { return c->model == KO_MODEL_QUADROTOR ? 4 : 3; }

static void draw_controls(const ko_config* c, const float* u, float* ctrl, int* steps)
{
    int nc = ctrl_count(c);
    for(int i = 0; i < nc; ++i) ctrl[i] = c->u_min[i] + u[i] * (c->u_max[i] - c->u_min[i]);
    uint32_t span = c->max_steps - c->min_steps + 1u;
    int k = (int)c->min_steps + (int)(u[nc] * (float)span);
    if(k > (int)c->max_steps) k = (int)c->max_steps;
    *steps = k;
}

/* ------------------------------------------------------------------------ */
/* Double integrator, FP32 (statePropagator.cu:76-142).                      */
/* ------------------------------------------------------------------------ */
static int prop_di_f(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, float* x1)
{
    float a[3];
    int k;
    draw_controls(c, u, a, &k);
    float p[3] = {x0[0], x0[1], x0[2]};
    float v[3] = {x0[3], x0[4], x0[5]};
    const float h = c->step_size;
    int ok = 1;
    for(int i = 0; i < k; ++i)
        {
            float p0[3] = {p[0], p[1], p[2]};
            for(int d = 0; d < 3; ++d)
                {
                    float half = v[d] + (a[d] * h) / 2.0f;
                    float full = v[d] + a[d] * h;
                    float sum;
                    if(c->di_rule == KO_DI_RULE_REFERENCE) sum = v[d] + ((v[d] + 2.0f * half) + full);
                    else sum = ((v[d] + 2.0f * half) + 2.0f * half) + full;
                    p[d] = p[d] + (sum * h) / 6.0f;
                }
            for(int d = 0; d < 3; ++d) v[d] = v[d] + ((((a[d] + 2.0f * a[d]) + 2.0f * a[d]) + a[d]) * h) / 6.0f;
            if(v[0] < c->v_min || v[0] > c->v_max || v[1] < c->v_min || v[1] > c->v_max || v[2] < c->v_min || v[2] > c->v_max)
                {
                    ok = 0;
                    break;
                }
            if(p[0] < c->ws_min || p[0] > c->ws_max || p[1] < c->ws_min || p[1] > c->ws_max || p[2] < c->ws_min || p[2] > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            if(!motion_valid_f(p0, p, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    x1[0] = p[0], x1[1] = p[1], x1[2] = p[2];
    x1[3] = v[0], x1[4] = v[1], x1[5] = v[2];
    x1[6] = a[0], x1[7] = a[1], x1[8] = a[2];
    x1[9] = h * (float)k;
    return ok;
}

static int prop_di_d(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, double* x1, double* margin)
{
    float af[3];
    int k;
    draw_controls(c, u, af, &k);
    double a[3] = {af[0], af[1], af[2]};
    double p[3] = {x0[0], x0[1], x0[2]};
    double v[3] = {x0[3], x0[4], x0[5]};
    const double h = (double)c->step_size;
    int ok = 1;
    double m = 1e30;
    for(int i = 0; i < k; ++i)
        {
            double p0[3] = {p[0], p[1], p[2]};
            for(int d = 0; d < 3; ++d)
                {
                    double half = v[d] + (a[d] * h) / 2.0;
                    double full = v[d] + a[d] * h;
                    double sum;
                    if(c->di_rule == KO_DI_RULE_REFERENCE) sum = v[d] + ((v[d] + 2.0 * half) + full);
                    else sum = ((v[d] + 2.0 * half) + 2.0 * half) + full;
                    p[d] = p[d] + (sum * h) / 6.0;
                }
            for(int d = 0; d < 3; ++d) v[d] = v[d] + a[d] * h;
            double bm = bound_margin_d(c, p, v);
            if(bm < m) m = bm;
            if(v[0] < c->v_min || v[0] > c->v_max || v[1] < c->v_min || v[1] > c->v_max || v[2] < c->v_min || v[2] > c->v_max)
                {
                    ok = 0;
                    break;
                }
            if(p[0] < c->ws_min || p[0] > c->ws_max || p[1] < c->ws_min || p[1] > c->ws_max || p[2] < c->ws_min || p[2] > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            double fm = face_margin_d(p0, p, obs, n_obs, 3);
            if(fm < m) m = fm;
            if(!motion_valid_d(p0, p, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    for(int d = 0; d < 3; ++d) x1[d] = p[d], x1[3 + d] = v[d], x1[6 + d] = a[d];
    x1[9] = h * (double)k;
    if(margin) *margin = m;
    return ok;
}

/* ------------------------------------------------------------------------ */
/* 12-D quadrotor, FP32 mirror (statePropagator.cu:246-323, ode 325-370).   */
/* ------------------------------------------------------------------------ */
typedef struct {
    float zc, lc, mc, nc;
} quad_ctrl_f;

static void quad_ode_f(const ko_config* c, const float* s, const quad_ctrl_f* u, float* d)
{
    float phi = s[3], theta = s[4], psi = s[5];
    float uu = s[6], vv = s[7], ww = s[8];
    float p = s[9], q = s[10], r = s[11];
    float sphi, cphi, sth, cth, spsi, cpsi;
    ko_sincosf(phi, &sphi, &cphi);
    ko_sincosf(theta, &sth, &cth);
    ko_sincosf(psi, &spsi, &cpsi);
    /* the two terms over cos(theta) share one division, as on the device */
    const float icth = 1.0f / cth;
    float tth = sth * icth;
    const float g = c->gravity;
    const float sps = sphi * sth, cps = cphi * sth;
    d[0] = fmaf(fmaf(cps, cpsi, sphi * spsi), ww, fmaf(fmaf(sps, cpsi, -(cphi * spsi)), vv, (cth * cpsi) * uu));
    d[1] = fmaf(fmaf(cps, spsi, -(sphi * cpsi)), ww, fmaf(fmaf(sps, spsi, cphi * cpsi), vv, (cth * spsi) * uu));
    d[2] = fmaf(cphi * cth, ww, fmaf(sphi * cth, vv, (-sth) * uu));
    float qr = fmaf(q, sphi, r * cphi);
    d[3] = fmaf(qr, tth, p);
    d[4] = fmaf(q, cphi, -(r * sphi));
    d[5] = qr * icth;
    float xyz = (-c->nu) * sqrtf(fmaf(ww, ww, fmaf(vv, vv, uu * uu)));
    float mx = c->mass_inv * xyz;
    d[6] = fmaf(mx, uu, fmaf(-g, sth, fmaf(r, vv, -(q * ww))));
    d[7] = fmaf(mx, vv, fmaf(g * cth, sphi, fmaf(p, ww, -(r * uu))));
    d[8] = fmaf(c->mass_inv, u->zc, fmaf(mx, ww, fmaf(g * cth, cphi, fmaf(q, uu, -(p * vv)))));
    float lmn = (-c->mu) * sqrtf(fmaf(r, r, fmaf(q, q, p * p)));
    float iix = 1.0f / c->ix, iiy = 1.0f / c->iy, iiz = 1.0f / c->iz;
    float jx = (c->iy - c->iz) / c->ix, jy = (c->iz - c->ix) / c->iy, jz = (c->ix - c->iy) / c->iz;
    d[9] = fmaf(iix, u->lc, fmaf(iix * lmn, p, (jx * q) * r));
    d[10] = fmaf(iiy, u->mc, fmaf(iiy * lmn, q, (jy * p) * r));
    d[11] = fmaf(iiz, u->nc, fmaf(iiz * lmn, r, (jz * p) * q));
}

static int prop_quad_f(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, float* x1)
{
    float ctrl[4];
    int k;
    draw_controls(c, u, ctrl, &k);
    quad_ctrl_f qc = {ctrl[0], ctrl[1], ctrl[2], ctrl[3]};
    const float h = c->step_size;
    const float hh = 0.5f * h;
    const float h6 = h / 6.0f;
    float s[12], k1[12], k2[12], k3[12], k4[12], t[12];
    for(int j = 0; j < 12; ++j) s[j] = x0[j];
    int ok = 1;
    for(int i = 0; i < k; ++i)
        {
            float p0[3] = {s[0], s[1], s[2]};
            quad_ode_f(c, s, &qc, k1);
            for(int j = 0; j < 12; ++j) t[j] = fmaf(hh, k1[j], s[j]);
            quad_ode_f(c, t, &qc, k2);
            for(int j = 0; j < 12; ++j) t[j] = fmaf(hh, k2[j], s[j]);
            quad_ode_f(c, t, &qc, k3);
            for(int j = 0; j < 12; ++j) t[j] = fmaf(h, k3[j], s[j]);
            quad_ode_f(c, t, &qc, k4);
            for(int j = 0; j < 12; ++j) s[j] = fmaf(h6, fmaf(2.0f, k3[j], fmaf(2.0f, k2[j], k1[j])) + k4[j], s[j]);
            if(s[6] < c->v_min || s[6] > c->v_max || s[7] < c->v_min || s[7] > c->v_max || s[8] < c->v_min || s[8] > c->v_max)
                {
                    ok = 0;
                    break;
                }
            if(s[0] < c->ws_min || s[0] > c->ws_max || s[1] < c->ws_min || s[1] > c->ws_max || s[2] < c->ws_min || s[2] > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            if(!motion_valid_f(p0, s, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    for(int j = 0; j < 12; ++j) x1[j] = s[j];
    x1[12] = ctrl[0], x1[13] = ctrl[1], x1[14] = ctrl[2], x1[15] = ctrl[3];
    x1[16] = h * (float)k;
    return ok;
}

static void quad_ode_d(const ko_config* c, const double* s, const double* u, double* d)
{
    double phi = s[3], theta = s[4], psi = s[5];
    double uu = s[6], vv = s[7], ww = s[8];
    double p = s[9], q = s[10], r = s[11];
    double sphi = sin(phi), cphi = cos(phi), sth = sin(theta), cth = cos(theta), spsi = sin(psi), cpsi = cos(psi);
    double tth = tan(theta);
    double nu = c->nu, mu = c->mu, g = c->gravity, mi = c->mass_inv, ix = c->ix, iy = c->iy, iz = c->iz;
    d[0] = cth * cpsi * uu + (sphi * sth * cpsi - cphi * spsi) * vv + (cphi * sth * cpsi + sphi * spsi) * ww;
    d[1] = cth * spsi * uu + (sphi * sth * spsi + cphi * cpsi) * vv + (cphi * sth * spsi - sphi * cpsi) * ww;
    d[2] = -sth * uu + sphi * cth * vv + cphi * cth * ww;
    d[3] = p + (q * sphi + r * cphi) * tth;
    d[4] = q * cphi - r * sphi;
    d[5] = (q * sphi + r * cphi) / cth;
    double xyz = -nu * sqrt(uu * uu + vv * vv + ww * ww);
    d[6] = (r * vv - q * ww) - g * sth + mi * xyz * uu;
    d[7] = (p * ww - r * uu) + g * cth * sphi + mi * xyz * vv;
    d[8] = (q * uu - p * vv) + g * cth * cphi + mi * xyz * ww + mi * u[0];
    double lmn = -mu * sqrt(p * p + q * q + r * r);
    d[9] = (iy - iz) / ix * q * r + (1.0 / ix) * lmn * p + (1.0 / ix) * u[1];
    d[10] = (iz - ix) / iy * p * r + (1.0 / iy) * lmn * q + (1.0 / iy) * u[2];
    d[11] = (ix - iy) / iz * p * q + (1.0 / iz) * lmn * r + (1.0 / iz) * u[3];
}

static int prop_quad_d(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, double* x1,
                       double* margin)
{
    float ctrlf[4];
    int k;
    draw_controls(c, u, ctrlf, &k);
    double ctrl[4] = {ctrlf[0], ctrlf[1], ctrlf[2], ctrlf[3]};
    const double h = (double)c->step_size;
    double s[12], k1[12], k2[12], k3[12], k4[12], t[12];
    for(int j = 0; j < 12; ++j) s[j] = x0[j];
    int ok = 1;
    double m = 1e30;
    for(int i = 0; i < k; ++i)
        {
            double p0[3] = {s[0], s[1], s[2]};
            quad_ode_d(c, s, ctrl, k1);
            for(int j = 0; j < 12; ++j) t[j] = s[j] + 0.5 * h * k1[j];
            quad_ode_d(c, t, ctrl, k2);
            for(int j = 0; j < 12; ++j) t[j] = s[j] + 0.5 * h * k2[j];
            quad_ode_d(c, t, ctrl, k3);
            for(int j = 0; j < 12; ++j) t[j] = s[j] + h * k3[j];
            quad_ode_d(c, t, ctrl, k4);
            for(int j = 0; j < 12; ++j) s[j] += h / 6.0 * (k1[j] + 2.0 * k2[j] + 2.0 * k3[j] + k4[j]);
            double bm = bound_margin_d(c, s, s + 6);
            if(bm < m) m = bm;
            if(s[6] < c->v_min || s[6] > c->v_max || s[7] < c->v_min || s[7] > c->v_max || s[8] < c->v_min || s[8] > c->v_max)
                {
                    ok = 0;
                    break;
                }
            if(s[0] < c->ws_min || s[0] > c->ws_max || s[1] < c->ws_min || s[1] > c->ws_max || s[2] < c->ws_min || s[2] > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            double fm = face_margin_d(p0, s, obs, n_obs, 3);
            if(fm < m) m = fm;
            if(!motion_valid_d(p0, s, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    for(int j = 0; j < 12; ++j) x1[j] = s[j];
    for(int j = 0; j < 4; ++j) x1[12 + j] = ctrl[j];
    x1[16] = h * (double)k;
    if(margin) *margin = m;
    return ok;
}

/* ------------------------------------------------------------------------ */
/* Dubins airplane (statePropagator.cu:147-244).  State x y z yaw pitch v;   */
/* draws a, yaw rate, pitch rate, steps; row [state | yr pr a | k*h].  The   */
/* attitude is linear in time within a step, so the RK4 stages are the       */
/* closed forms at t, t + h/2, t + h, summed in the reference's order        */
/* (v cos p) cos y + 2 (A + A) + B, weighted by h/6.  Checks: speed, pitch,  */
/* workspace, obstacles.  FP32 mirror: the end-stage attitude sine/cosine is */
/* the next step's start pair, exactly as the CUDA kernel carries it.        */
/* ------------------------------------------------------------------------ */
static int prop_dubins_f(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, float* x1)
{
    float ctrl[3];
    int k;
    draw_controls(c, u, ctrl, &k);
    const float a = ctrl[0], yr = ctrl[1], pr = ctrl[2];
    const float h = c->step_size, hh = 0.5f * h, h6 = h / 6.0f;
    float x = x0[0], y = x0[1], z = x0[2], yaw = x0[3], pitch = x0[4], v = x0[5];
    const float dvm = hh * a, dve = h * a;
    const float dpm = hh * pr, dym = hh * yr;
    const float dpe = h * pr, dye = h * yr;
    const float dv = h6 * ((a + 2.0f * (a + a)) + a);
    float sp, cp, sy, cy;
    ko_sincosf(pitch, &sp, &cp);
    ko_sincosf(yaw, &sy, &cy);
    int ok = 1;
    for(int i = 0; i < k; ++i)
        {
            float p0[3] = {x, y, z};
            float spm, cpm, sym, cym, spe, cpe, sye, cye;
            ko_sincosf(pitch + dpm, &spm, &cpm);
            ko_sincosf(yaw + dym, &sym, &cym);
            ko_sincosf(pitch + dpe, &spe, &cpe);
            ko_sincosf(yaw + dye, &sye, &cye);
            const float vm = v + dvm, ve = v + dve;
            const float ax = (vm * cpm) * cym, bx = (ve * cpe) * cye;
            const float ay = (vm * cpm) * sym, by = (ve * cpe) * sye;
            const float az = vm * spm, bz = ve * spe;
            x = x + h6 * ((((v * cp) * cy) + 2.0f * (ax + ax)) + bx);
            y = y + h6 * ((((v * cp) * sy) + 2.0f * (ay + ay)) + by);
            z = z + h6 * (((v * sp) + 2.0f * (az + az)) + bz);
            yaw = yaw + dye;
            pitch = pitch + dpe;
            v = v + dv;
            sp = spe, cp = cpe, sy = sye, cy = cye;
            if(v < c->v_min || v > c->v_max || pitch < c->pitch_min || pitch > c->pitch_max || x < c->ws_min || x > c->ws_max ||
               y < c->ws_min || y > c->ws_max || z < c->ws_min || z > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            float p1[3] = {x, y, z};
            if(!motion_valid_f(p0, p1, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = z, x1[3] = yaw, x1[4] = pitch, x1[5] = v;
    x1[6] = yr, x1[7] = pr, x1[8] = a;
    x1[9] = h * (float)k;
    return ok;
}

static int prop_dubins_d(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, double* x1, double* margin)
{
    float cf[3];
    int k;
    draw_controls(c, u, cf, &k);
    const double a = cf[0], yr = cf[1], pr = cf[2];
    const double h = (double)c->step_size;
    double x = x0[0], y = x0[1], z = x0[2], yaw = x0[3], pitch = x0[4], v = x0[5];
    int ok = 1;
    double m = 1e30;
    for(int i = 0; i < k; ++i)
        {
            double p0[3] = {x, y, z};
            /* classic RK4 of x' = v cos p cos y, y' = v cos p sin y, z' = v sin p
             * with p, y, v linear in time */
            double pm = pitch + 0.5 * h * pr, ym = yaw + 0.5 * h * yr, pe = pitch + h * pr, ye = yaw + h * yr;
            double vm = v + 0.5 * h * a, ve = v + h * a;
            x += h / 6.0 * (v * cos(pitch) * cos(yaw) + 4.0 * vm * cos(pm) * cos(ym) + ve * cos(pe) * cos(ye));
            y += h / 6.0 * (v * cos(pitch) * sin(yaw) + 4.0 * vm * cos(pm) * sin(ym) + ve * cos(pe) * sin(ye));
            z += h / 6.0 * (v * sin(pitch) + 4.0 * vm * sin(pm) + ve * sin(pe));
            yaw = ye;
            pitch = pe;
            v = ve;
            double pos[3] = {x, y, z};
            double bm = end_margin_d(v, c->v_min, c->v_max);
            double t = end_margin_d(pitch, c->pitch_min, c->pitch_max);
            if(t < bm) bm = t;
            for(int d = 0; d < 3; ++d)
                {
                    t = end_margin_d(pos[d], c->ws_min, c->ws_max);
                    if(t < bm) bm = t;
                }
            if(bm < m) m = bm;
            if(v < c->v_min || v > c->v_max || pitch < c->pitch_min || pitch > c->pitch_max || x < c->ws_min || x > c->ws_max ||
               y < c->ws_min || y > c->ws_max || z < c->ws_min || z > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            double fm = face_margin_d(p0, pos, obs, n_obs, 3);
            if(fm < m) m = fm;
            if(!motion_valid_d(p0, pos, obs, n_obs, 3))
                {
                    ok = 0;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = z, x1[3] = yaw, x1[4] = pitch, x1[5] = v;
    x1[6] = yr, x1[7] = pr, x1[8] = a;
    x1[9] = h * (double)k;
    if(margin) *margin = m;
    return ok;
}

/* ------------------------------------------------------------------------ */
/* Unicycle (statePropagator.cu:13-74), planar.  State x y theta v; draws a, */
/* steering, dt, steps; row [state | a steering dt].  Explicit Euler in the  */
/* reference's order; tan(steering), the same every step, is taken as the    */
/* portable sin/cos ratio.  Checks: workspace (x, y), then the boxes in the  */
/* plane; the reference has no speed check.                                  */
/* ------------------------------------------------------------------------ */
static int prop_uni_f(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, float* x1)
{
    float ctrl[3];
    int k;
    draw_controls(c, u, ctrl, &k);
    const float a = ctrl[0], steer = ctrl[1], dt = ctrl[2];
    const float h = c->step_size;
    float x = x0[0], y = x0[1], th = x0[2], v = x0[3];
    float ss, cs;
    ko_sincosf(steer, &ss, &cs);
    const float tan_steer = ss / cs;
    int ok = 1;
    for(int i = 0; i < k; ++i)
        {
            float p0[2] = {x, y};
            float st, ct;
            ko_sincosf(th, &st, &ct);
            x = x + (v * ct) * h;
            y = y + (v * st) * h;
            th = th + ((v / c->wheelbase) * tan_steer) * h;
            v = v + a * h;
            if(x < c->ws_min || x > c->ws_max || y < c->ws_min || y > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            float p1[2] = {x, y};
            if(!motion_valid_f(p0, p1, obs, n_obs, 2))
                {
                    ok = 0;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = th, x1[3] = v;
    x1[4] = a, x1[5] = steer, x1[6] = dt;
    return ok;
}

static int prop_uni_d(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, double* x1, double* margin)
{
    float cf[3];
    int k;
    draw_controls(c, u, cf, &k);
    const double a = cf[0], steer = cf[1], dt = cf[2];
    const double h = (double)c->step_size, tan_steer = tan(steer);
    double x = x0[0], y = x0[1], th = x0[2], v = x0[3];
    int ok = 1;
    double m = 1e30;
    for(int i = 0; i < k; ++i)
        {
            double p0[2] = {x, y};
            double ct = cos(th), st = sin(th);
            x += v * ct * h;
            y += v * st * h;
            th += (v / (double)c->wheelbase) * tan_steer * h;
            v += a * h;
            double bm = end_margin_d(x, c->ws_min, c->ws_max), t = end_margin_d(y, c->ws_min, c->ws_max);
            if(t < bm) bm = t;
            if(bm < m) m = bm;
            if(x < c->ws_min || x > c->ws_max || y < c->ws_min || y > c->ws_max)
                {
                    ok = 0;
                    break;
                }
            double p1[2] = {x, y};
            double fm = face_margin_d(p0, p1, obs, n_obs, 2);
            if(fm < m) m = fm;
            if(!motion_valid_d(p0, p1, obs, n_obs, 2))
                {
                    ok = 0;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = th, x1[3] = v;
    x1[4] = a, x1[5] = steer, x1[6] = dt;
    if(margin) *margin = m;
    return ok;
}

static int propagate_one_f(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, float* x1)
{
    switch(c->model)
        {
            case KO_MODEL_QUADROTOR: return prop_quad_f(c, x0, u, obs, n_obs, x1);
            case KO_MODEL_DUBINS_AIRPLANE: return prop_dubins_f(c, x0, u, obs, n_obs, x1);
            case KO_MODEL_UNICYCLE: return prop_uni_f(c, x0, u, obs, n_obs, x1);
            default: return prop_di_f(c, x0, u, obs, n_obs, x1);
        }
}

static int propagate_one_d(const ko_config* c, const float* x0, const float* u, const float* obs, uint32_t n_obs, double* x1, double* m)
{
    switch(c->model)
        {
            case KO_MODEL_QUADROTOR: return prop_quad_d(c, x0, u, obs, n_obs, x1, m);
            case KO_MODEL_DUBINS_AIRPLANE: return prop_dubins_d(c, x0, u, obs, n_obs, x1, m);
            case KO_MODEL_UNICYCLE: return prop_uni_d(c, x0, u, obs, n_obs, x1, m);
            default: return prop_di_d(c, x0, u, obs, n_obs, x1, m);
        }
}

void ko_propagate_f32(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs, uint32_t n,
                      float* x1, uint8_t* valid, int32_t* r1, int32_t* r2)
{
    int D = ko_sample_dim(c->model);
    for(uint32_t i = 0; i < n; ++i)
        {
            float* y = x1 + (size_t)i * D;
            valid[i] = (uint8_t)propagate_one_f(c, x0 + (size_t)i * D, u + (size_t)i * 8, obstacles, n_obs, y);
            int a = ko_region(c, y);
            if(r1) r1[i] = a;
            if(r2) r2[i] = ko_subregion(c, y, a);
        }
}

void ko_propagate_f64(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs, uint32_t n,
                      double* x1, uint8_t* valid)
{
    int D = ko_sample_dim(c->model);
    for(uint32_t i = 0; i < n; ++i)
        {
            const float* a = x0 + (size_t)i * D;
            const float* w = u + (size_t)i * 8;
            double* y = x1 + (size_t)i * D;
            valid[i] = (uint8_t)propagate_one_d(c, a, w, obstacles, n_obs, y, NULL);
        }
}

double ko_verdict_margin_f64(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs)
{
    double y[KO_MAX_SAMPLE_DIM], m = 1e30;
    propagate_one_d(c, x0, u, obstacles, n_obs, y, &m);
    return m;
}

/* ------------------------------------------------------------------------ */
/* Region scores.  Graph.cu:311-358: freeVol = (eps+valid)/(eps+valid+      */
/* invalid) * cellVolume; score = freeVol^4 / ((1+coverage)(1+count^2));    */
/* normalised eps + score/total; regions without valid samples get 1.       */
/* ------------------------------------------------------------------------ */
void ko_score_update(const ko_config* c, const int32_t* counter, const int32_t* valid, uint64_t* marks, uint64_t* newmarks,
                     float* score, float* total_out)
{
    uint32_t L = c->coarse_len, F = c->fine_len;
    const int planar = ko_ws_dims(c->model) == 2;
    uint32_t R1 = planar ? L * L : L * L * L;
    float F2 = (float)(planar ? F * F : F * F * F);
    float size1 = (c->ws_max - c->ws_min) / (float)L;
    float area = size1 * size1;
    float vol = planar ? area : area * size1; /* W_R1_VOL in the workspace dimension */
    float lanes[KO_SCORE_LANES];
    for(int l = 0; l < KO_SCORE_LANES; ++l) lanes[l] = 0.0f;
    for(uint32_t r = 0; r < R1; ++r)
        {
            uint64_t m = marks[r] | newmarks[r];
            marks[r] = m;
            newmarks[r] = 0;
            float raw = 0.0f;
            int32_t nv = valid[r];
            if(nv > 0)
                {
                    int32_t n = counter[r];
                    float cov = (float)__builtin_popcountll(m) / F2;
                    float a = c->epsilon + (float)nv;
                    float b = a + (float)(n - nv);
                    float fv = (a / b) * vol;
                    float f2 = fv * fv;
                    float f4 = f2 * f2;
                    float nf = (float)n;
                    float den = (1.0f + cov) * (1.0f + nf * nf);
                    raw = f4 / den;
                }
            score[r] = raw;
            lanes[r % KO_SCORE_LANES] += raw;
        }
    for(int stride = KO_SCORE_LANES / 2; stride >= 1; stride /= 2)
        for(int l = 0; l < stride; ++l) lanes[l] += lanes[l + stride];
    float total = lanes[0];
    for(uint32_t r = 0; r < R1; ++r)
        {
            if(valid[r] == 0) score[r] = 1.0f;
            else score[r] = total > 0.0f ? c->epsilon + score[r] / total : c->epsilon;
        }
    if(total_out) *total_out = total;
}

/* KGMT.cu:387-388 */
float ko_f_accept(uint32_t itr, float eps, uint32_t tree_size, uint32_t n_next, uint32_t capacity)
{
    float ta = 1.0f - (float)(tree_size + n_next) / (float)capacity;
    float ie = (float)itr * eps;
    double t = (double)ta;
    double t5 = ((t * t) * (t * t)) * t;
    return (float)((double)ie * t5);
}

/* ------------------------------------------------------------------------ */
/* Whole plan (KGMT.cu:41-105 / 167-211 / 305-403).                         */
/* ------------------------------------------------------------------------ */
int ko_plan(const ko_config* c, const float* init, const float* goal, const float* obstacles, uint32_t n_obs, ko_result* res,
            float* samples, int32_t* parents, float* costs, float* path, ko_iter_trace* trace)
{
    return ko_plan_hooked(c, init, goal, obstacles, n_obs, res, samples, parents, costs, path, trace, NULL, NULL);
}

int ko_plan_hooked(const ko_config* c, const float* init, const float* goal, const float* obstacles, uint32_t n_obs, ko_result* res,
                   float* samples, int32_t* parents, float* costs, float* path, ko_iter_trace* trace, ko_iter_hook hook, void* user)
{
    const int D = ko_sample_dim(c->model);
    const uint32_t T = c->tree_capacity;
    const uint32_t S = c->samples_per_node;
    const uint32_t L = c->coarse_len;
    const int W = ko_ws_dims(c->model);
    const uint32_t R1 = W == 2 ? L * L : L * L * L;
    const uint32_t FC = W == 2 ? c->fine_len * c->fine_len : c->fine_len * c->fine_len * c->fine_len;
    if(T < 2 || S < 1 || L < 1 || c->fine_len < 1 || FC > 64) return -1;

    int32_t* node_r1 = (int32_t*)calloc(T, sizeof(int32_t));
    uint32_t* rep_old = (uint32_t*)malloc(sizeof(uint32_t) * T);
    uint32_t* rep_new = (uint32_t*)malloc(sizeof(uint32_t) * T); /* entries past T are never read */
    float* us = (float*)malloc(sizeof(float) * (size_t)T * D);
    int32_t* up = (int32_t*)malloc(sizeof(int32_t) * T);
    int32_t* ur1 = (int32_t*)malloc(sizeof(int32_t) * T);
    uint8_t* uflag = (uint8_t*)malloc(T);
    int32_t* counter = (int32_t*)calloc(R1, sizeof(int32_t));
    int32_t* validc = (int32_t*)calloc(R1, sizeof(int32_t));
    float* score = (float*)calloc(R1, sizeof(float));
    uint64_t* marks = (uint64_t*)calloc(R1, sizeof(uint64_t));
    uint64_t* newmarks = (uint64_t*)calloc(R1, sizeof(uint64_t));
    int fail = !node_r1 || !rep_old || !rep_new || !us || !up || !ur1 || !uflag || !counter || !validc || !score || !marks || !newmarks;
    if(fail)
        {
            free(node_r1), free(rep_old), free(rep_new), free(us), free(up), free(ur1), free(uflag);
            free(counter), free(validc), free(score), free(marks), free(newmarks);
            return -2;
        }

    /* plan() initialisation, KGMT.cu:50-78 */
    memset(samples, 0, sizeof(float) * (size_t)T * D);
    for(uint32_t i = 0; i < T; ++i) parents[i] = -1;
    memset(costs, 0, sizeof(float) * T);
    for(int j = 0; j < D; ++j) samples[j] = init[j];
    node_r1[0] = ko_region(c, init);
    uint32_t tree_size = 1;
    uint32_t n_react = 0, w_new = KO_ROOT_REPEAT;
    for(uint32_t j = 0; j < KO_ROOT_REPEAT; ++j) rep_new[j] = 0;
    int status = KO_STATUS_RUNNING;
    int32_t goal_idx = -1;
    uint32_t itr = 0, drawn = 0;
    uint32_t new_nodes = 1; /* nodes appended by the last iteration (the root before the first) */

    while(status == KO_STATUS_RUNNING)
        {
            ++itr;
            /* --- propagateFrontier (KGMT.cu:167-211, 218-259) --- */
            uint32_t R = n_react + w_new;
            uint32_t free_slots = T - tree_size;
            uint32_t Sp = 0, Ruse = R;
            if(R > 0)
                {
                    Sp = free_slots / R;
                    if(Sp > S) Sp = S;
                    if(Sp == 0)
                        {
                            Sp = 1;
                            Ruse = free_slots;
                        }
                }
            uint32_t N = Ruse * Sp;
            uint32_t n_next = 0;
            for(uint32_t s = 0; s < N; ++s)
                {
                    uint32_t e = s / Sp;
                    uint32_t par = e < n_react ? rep_old[e] : rep_new[e - n_react];
                    float u[8];
                    ko_sample_uniforms(c->seed, s, itr, u);
                    float* y = us + (size_t)s * D;
                    int ok = propagate_one_f(c, samples + (size_t)par * D, u, obstacles, n_obs, y);
                    int a = ko_region(c, y);
                    int b = ko_subregion(c, y, a);
                    up[s] = (int32_t)par;
                    ur1[s] = a;
                    counter[a] += 1;
                    uint8_t acc = 0;
                    if(ok)
                        {
                            validc[a] += 1;
                            float ua = u[ctrl_count(c) + 1];
                            int fresh = !((marks[a] >> b) & 1ull);
                            acc = (uint8_t)((ua < score[a]) || fresh);
                            newmarks[a] |= 1ull << b;
                        }
                    uflag[s] = acc;
                    n_next += acc;
                }
            drawn += N;

            /* --- Graph::updateVertices (Graph.cu:207-358) --- */
            float total = 0.0f;
            ko_score_update(c, counter, validc, marks, newmarks, score, &total);

            /* --- updateFrontier (KGMT.cu:380-403, 305-378) --- */
            float fa = ko_f_accept(itr, c->epsilon, tree_size, n_next, T);
            uint32_t nr = 0;
            for(uint32_t i = 0; i < tree_size; ++i)
                {
                    float ur = ko_react_uniform(c->seed, i, itr);
                    if(ur <= score[node_r1[i]] + fa) rep_old[nr++] = i;
                }
            uint32_t w = 0, t = 0;
            for(uint32_t s = 0; s < N; ++s)
                {
                    if(!uflag[s]) continue;
                    uint32_t idx = tree_size + t++;
                    const float* y = us + (size_t)s * D;
                    for(int j = 0; j < D; ++j) samples[(size_t)idx * D + j] = y[j];
                    parents[idx] = up[s];
                    float dist = ko_distance_w(y, goal, W);
                    costs[idx] = dist;
                    node_r1[idx] = ur1[s];
                    uint32_t rep = validc[ur1[s]] < KO_SPARSE_VALID_LIMIT ? KO_NEW_NODE_REPEAT_SPARSE : KO_NEW_NODE_REPEAT_DENSE;
                    for(uint32_t j = 0; j < rep; ++j, ++w)
                        if(w < T) rep_new[w] = idx;
                    if(dist < c->goal_radius && goal_idx < 0) goal_idx = (int32_t)idx;
                }
            if(trace)
                {
                    ko_iter_trace* tr = &trace[itr - 1];
                    tr->itr = itr;
                    tr->tree_size_before = tree_size;
                    tr->n_samples = N;
                    tr->samples_per_entry = Sp;
                    tr->n_next = n_next;
                    tr->n_react = nr;
                    tr->repeat_total = nr + w;
                    tr->f_accept = fa;
                    tr->score_total = total;
                }
            if(hook)
                {
                    /* h_frontierSize_ (KGMT.cu:171-172): the distinct nodes this
                     * iteration expanded, re-activated ones and the last
                     * iteration's new ones */
                    ko_iter_view v;
                    v.itr = itr;
                    v.tree_size = tree_size + n_next;
                    v.frontier_size = n_react + new_nodes;
                    v.expanded = N;
                    v.n_react = nr;
                    v.n_rep_new = w < T ? w : T;
                    v.goal_index = goal_idx;
                    v.regions = R1;
                    v.rep_old = rep_old;
                    v.rep_new = rep_new;
                    v.counter = counter;
                    v.valid = validc;
                    v.score = score;
                    hook(&v, user);
                }
            new_nodes = n_next;
            tree_size += n_next;
            n_react = nr;
            w_new = w;
            if(goal_idx >= 0) status = KO_STATUS_SUCCESS;
            else if(itr >= c->max_iterations) status = KO_STATUS_ITER_LIMIT;
            else if(tree_size >= T) status = KO_STATUS_CAPACITY;
        }

    uint32_t plen = 0;
    if(goal_idx >= 0)
        {
            int32_t i = goal_idx;
            while(i >= 0)
                {
                    if(path)
                        for(int j = 0; j < D; ++j) path[(size_t)plen * D + j] = samples[(size_t)i * D + j];
                    ++plen;
                    i = parents[i];
                }
        }
    res->status = status;
    res->iterations = itr;
    res->tree_size = tree_size;
    res->goal_index = goal_idx;
    res->path_len = plen;
    res->samples_drawn = drawn;

    free(node_r1), free(rep_old), free(rep_new), free(us), free(up), free(ur1), free(uflag);
    free(counter), free(validc), free(score), free(marks), free(newmarks);
    return 0;
}

int ko_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ko_plan_batch(uint32_t nq, const ko_config* cfgs, const float* inits, const float* goals, const float* obstacles,
                  const uint32_t* obs_offset, const uint32_t* obs_count, ko_result* res, int threads)
{
    int err = 0;
#ifdef _OPENMP
    if(threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : err)
#endif
    for(int64_t q = 0; q < (int64_t)nq; ++q)
        {
            const ko_config* c = &cfgs[q];
            int D = ko_sample_dim(c->model);
            float* samples = (float*)malloc(sizeof(float) * (size_t)c->tree_capacity * D);
            int32_t* parents = (int32_t*)malloc(sizeof(int32_t) * c->tree_capacity);
            float* costs = (float*)malloc(sizeof(float) * c->tree_capacity);
            /* a planar query takes its boxes as rows of 4 (x, y extents) */
            const float* rows = obstacles + 6 * (size_t)obs_offset[q];
            float* rows2 = NULL;
            if(ko_ws_dims(c->model) == 2 && obs_count[q] > 0)
                {
                    rows2 = (float*)malloc(sizeof(float) * 4 * (size_t)obs_count[q]);
                    if(rows2)
                        for(uint32_t o = 0; o < obs_count[q]; ++o)
                            {
                                rows2[4 * o + 0] = rows[6 * o + 0], rows2[4 * o + 1] = rows[6 * o + 1];
                                rows2[4 * o + 2] = rows[6 * o + 3], rows2[4 * o + 3] = rows[6 * o + 4];
                            }
                    rows = rows2;
                }
            if(!samples || !parents || !costs || !rows)
                {
                    err |= 1;
                }
            else
                {
                    int rc = ko_plan(c, inits + (size_t)q * KO_MAX_SAMPLE_DIM, goals + (size_t)q * KO_MAX_SAMPLE_DIM, rows, obs_count[q],
                                     &res[q], samples, parents, costs, NULL, NULL);
                    if(rc) err |= 1;
                }
            free(samples), free(parents), free(costs), free(rows2);
        }
    return err ? -1 : 0;
}
