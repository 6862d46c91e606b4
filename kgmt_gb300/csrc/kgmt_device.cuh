// kgmt_device.cuh -- per-sample device math of the KGMT planning loop.
//
// Everything here is compiled with -fmad=false: every float multiply and add
// is rounded on its own, in the order written, so the region ids, collision
// verdicts, acceptance decisions and therefore the whole tree are
// reproducible bit for bit by a single-precision CPU restatement that keeps
// the same order (-ffp-contract=off).
//
// Reference counterparts (nipe1783/KGMT):
//   Philox sampling replaces curand XORWOW   src/planners/Planner.cu:37-50
//   double integrator                        src/statePropagator/statePropagator.cu:76-142
//   quadrotor RK4 + ode                      src/statePropagator/statePropagator.cu:246-370
//   swept AABB broad phase                   src/collisionCheck/collisionCheck.cu:3-10, 49-61
//   coarse / fine region ids                 src/graphs/Graph.cu:99-153, 155-205
//   goal distance                            include/helper/helper.cuh:138-152
#pragma once
#include <cstdint>

#include "kgmt_types.h"

namespace kgmt {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Counter (index, itr,
// domain, block), key = 64-bit query seed.
// ---------------------------------------------------------------------------
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for(int r = 0; r < 10; ++r)
        {
            uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
            uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
            uint32_t n0 = hi1 ^ c1 ^ k0;
            uint32_t n2 = hi0 ^ c3 ^ k1;
            c0 = n0;
            c1 = lo1;
            c2 = n2;
            c3 = lo0;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
    return {c0, c1, c2, c3};
}

// uniform in (0, 1], like curand_uniform
__device__ __forceinline__ float u01(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1.0p-24f; }

// ---------------------------------------------------------------------------
// Portable sine/cosine: Cody & Waite reduction by pi/2 (three-part split,
// n*P1 and n*P2 exact for |n| < 2^13) and minimax polynomials on |r| <= pi/4
// in Horner form: sin r = r + r^3 (s1 + s2 r^2 + s3 r^4), cos r = 1 - r^2/2
// + r^4 (c2 + c3 r^2 + c4 r^4), fitted by Lawson's iteratively reweighted
// least squares to relative errors 3.8e-9 and 1.2e-10 and rounded to float
// (oracle/fit_sincos.py).  Same operations as the CPU restatement, so both
// round identically; accuracy about one ulp for |x| < 1e4.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sincos_portable(float x, float& s, float& c)
{
    // explicit fused multiply-adds (one rounding each), placed exactly as in
    // the CPU restatement; nothing else is contracted (-fmad=false).
    // The nearest multiple n of pi/2 by adding 1.5 * 2^23: while
    // |x * 2/pi| < 2^22 the sum rounds to an integer exactly as rintf does
    // (to nearest, ties to even), subtracting the constant again gives n
    // exactly, and the sum's two lowest bits are n mod 4, the quadrant.
    // Beyond that range (where the reduction means nothing) both sides still
    // compute the same values.
    const float t = x * 0x1.45f306p-1f + 0x1.8p23f;
    const float n = t - 0x1.8p23f;
    const int q = __float_as_int(t) & 3;
    float r = fmaf(-n, 0x1.92p+0f, x);
    r = fmaf(-n, 0x1.fb4p-12f, r);
    r = fmaf(-n, 0x1.4442d2p-24f, r);
    float r2 = r * r;
    float ps = fmaf(r2, -0x1.9943ep-13f, 0x1.11073ap-7f);
    ps = fmaf(r2, ps, -0x1.555546p-3f);
    float sp = fmaf(r * r2, ps, r);
    float pc = fmaf(r2, 0x1.99eba6p-16f, -0x1.6c0c34p-10f);
    pc = fmaf(r2, pc, 0x1.55554ap-5f);
    pc = fmaf(r2, pc, -0x1.0p-1f);
    float cp = fmaf(r2, pc, 1.0f);
    float ss = (q & 1) ? cp : sp;
    float cc = (q & 1) ? sp : cp;
    // sine negative in quadrants 2 and 3, cosine in 1 and 2: sign-bit flips
    s = __int_as_float(__float_as_int(ss) ^ ((q & 2) << 30));
    c = __int_as_float(__float_as_int(cc) ^ (((q + 1) & 2) << 30));
}

// ---------------------------------------------------------------------------
// x / 6 rounded exactly as the IEEE division, as one multiply and one fused
// multiply-add: RN(c_hi * x + RN(c_lo * x)) with c_hi = RN(1/6), c_lo =
// RN(1/6 - c_hi) (Brisebarre & Muller, "Correctly rounded multiplication by
// arbitrary precision constants", IEEE TC 2008).  Checked exhaustively over a
// binade (tests/test_arith_cpu.py); the identity scales by powers of two, so
// it holds for every finite |x| > 2^-98.  Elsewhere the true division runs.
// A divergent branch costs about as much as the arithmetic it guards, so the
// hot loops evaluate div6_fast for several values, combine the div6_exact
// predicates and take one rarely-taken branch to redo them with the division.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float div6_fast(float x) { return fmaf(0x1.555556p-3f, x, -0x1.555556p-28f * x); }
__device__ __forceinline__ bool div6_exact(float x)
{
    const float ax = fabsf(x);
    return ax > 0x1p-98f && ax <= 0x1.fffffep127f;
}
__device__ __forceinline__ float div6(float x) { return div6_exact(x) ? div6_fast(x) : x / 6.0f; }

// x / d for a divisor that may be an exact power of two: then the product
// with the exact reciprocal is the same IEEE result, without a division
__device__ __forceinline__ float div_maybe_pow2(float x, float d, float inv_d, bool pow2) { return pow2 ? x * inv_d : x / d; }

// ---------------------------------------------------------------------------
// Regions on workspace-only grids.  r1 = (ix*L + iy)*L + iz (z least
// significant, Graph.cu:105-113); the fine cell is located relative to the
// exact corner ws_min + idx * cell_size.
// ---------------------------------------------------------------------------
// clamp(trunc(t), 0, len - 1), with NaN and negative t giving 0: the
// reference's `(int)t` then two clamps (Graph.cu:107-109) for every t in
// range.  Branch-free: fmaxf returns 0 for a NaN t, and truncating the
// clamped float equals clamping the truncated one (len - 1 < 2^24 is exact).
__device__ __forceinline__ int cell_index(float t, int len)
{
    return (int)fminf(fmaxf(t, 0.0f), (float)(len - 1));
}

struct CellIds {
    int r1;
    int r2;  // fine cell inside r1, [0, fine_len^3)
};

// t[i] / d for three values, one (query-uniform) branch for all three
__device__ __forceinline__ void div3_maybe_pow2(float* t, float d, float inv_d, bool pow2)
{
    if(pow2)
        {
#pragma unroll
            for(int i = 0; i < 3; ++i) t[i] = t[i] * inv_d;
        }
    else
        {
#pragma unroll
            for(int i = 0; i < 3; ++i) t[i] = t[i] / d;
        }
}

// Workspace position of a sample row: x y z, or x y and a z pinned to ws_min
// for the planar unicycle (whose third component is its heading).  Planar
// regions drop the z digit: r1 = ix*L + iy, fine cell jx*F + jy.
__device__ __forceinline__ float row_z(const QueryParams& P, const float* x) { return P.planar ? P.ws_min : x[2]; }

__device__ __forceinline__ CellIds cell_ids(const QueryParams& P, const float* row)
{
    const float x = row[0], y = row[1], z = row_z(P, row);
    const float Lf = (float)P.coarse_len;
    const int L = (int)P.coarse_len;
    float t[3] = {Lf * (x - P.ws_min), Lf * (y - P.ws_min), Lf * (z - P.ws_min)};
    div3_maybe_pow2(t, P.ws_range, P.inv_range, P.range_pow2 != 0);
    const int ix = cell_index(t[0], L), iy = cell_index(t[1], L), iz = cell_index(t[2], L);
    const float Ff = (float)P.fine_len;
    const int F = (int)P.fine_len;
    float mx = P.ws_min + (float)ix * P.cell_size;
    float my = P.ws_min + (float)iy * P.cell_size;
    float mz = P.ws_min + (float)iz * P.cell_size;
    float f[3] = {Ff * (x - mx), Ff * (y - my), Ff * (z - mz)};
    div3_maybe_pow2(f, P.cell_size, P.inv_cell, P.cell_pow2 != 0);
    const int jx = cell_index(f[0], F), jy = cell_index(f[1], F), jz = cell_index(f[2], F);
    if(P.planar) return {ix * L + iy, jx * F + jy};
    return {(ix * L + iy) * L + iz, (jx * F + jy) * F + jz};
}

__device__ __forceinline__ int region_of(const QueryParams& P, const float* row)
{
    const float Lf = (float)P.coarse_len;
    const int L = (int)P.coarse_len;
    float t[3] = {Lf * (row[0] - P.ws_min), Lf * (row[1] - P.ws_min), Lf * (row_z(P, row) - P.ws_min)};
    div3_maybe_pow2(t, P.ws_range, P.inv_range, P.range_pow2 != 0);
    const int ixy = cell_index(t[0], L) * L + cell_index(t[1], L);
    return P.planar ? ixy : ixy * L + cell_index(t[2], L);
}

// helper.cuh:138-152 (distance over the W workspace components)
__device__ __forceinline__ float goal_distance(const QueryParams& P, const float* row)
{
    float dx = row[0] - P.goal[0], dy = row[1] - P.goal[1];
    float s = dx * dx + dy * dy;
    if(!P.planar)
        {
            float dz = row[2] - P.goal[2];
            s = s + dz * dz;
        }
    return sqrtf(s);
}

// ---------------------------------------------------------------------------
// Swept-AABB broad phase against boxes stored as two float4 (min.xyz, max.xyz).
// Separated iff bbMax <= obsMin or obsMax <= bbMin on some axis; touching is
// free.  Returns true when the step box hits no obstacle.
// ---------------------------------------------------------------------------
struct PropCount {
    int steps = 0;       // RK4 steps executed
    uint32_t tests = 0;  // step-box x box tests
};

__device__ __forceinline__ bool box_hit(const float4* __restrict__ obs, uint32_t o, float lx, float ly, float lz, float hx, float hy,
                                        float hz)
{
    const float4 mn = obs[2 * o];
    const float4 mx = obs[2 * o + 1];
    const bool sep = (hx <= mn.x) | (mx.x <= lx) | (hy <= mn.y) | (mx.y <= ly) | (hz <= mn.z) | (mx.z <= lz);
    return !sep;
}

// planar workspace (W_DIM 2): the z extents play no part
__device__ __forceinline__ bool box_hit_xy(const float4* __restrict__ obs, uint32_t o, float lx, float ly, float hx, float hy)
{
    const float4 mn = obs[2 * o];
    const float4 mx = obs[2 * o + 1];
    const bool sep = (hx <= mn.x) | (mx.x <= lx) | (hy <= mn.y) | (mx.y <= ly);
    return !sep;
}

// Cell coordinate on the obstacle grid; monotone in x (a subtraction and a
// multiply by the positive grid_scale), and the grid is built with the same
// function, so a point inside both a box and the step box lies in a cell both
// cell ranges contain -- culling by cells never drops a hit.  (Region ids use
// the reference's division instead; the culling grid is internal.)
__device__ __forceinline__ int grid_cell(const QueryParams& P, float x)
{
    return cell_index((x - P.ws_min) * P.grid_scale, (int)P.grid_dim);
}

// Where the culling grid of the current query lives: its starts (and the
// first kSmemGridItems items) staged in shared memory by the propagate
// kernel, the rest of the items in global memory.  start == nullptr: no grid.
struct GridView {
    const uint16_t* start;
    const uint16_t* items_s;
    const uint16_t* items_g;
};

__device__ __forceinline__ uint32_t grid_item(const GridView& g, uint32_t j)
{
    return j < kSmemGridItems ? g.items_s[j] : __ldg(g.items_g + j);
}

// Consecutive step boxes of a trajectory share an end point, so the grid cell
// of each end point is computed once and carried into the next step.  Since
// grid_cell is monotone, the cell range of a step box [min(a, b), max(a, b)]
// is [min(cell(a), cell(b)), max(cell(a), cell(b))] per axis.
struct StepCells {
    int x, y, z;  // cell of the step's start point
    bool ok;      // the start point has no NaN coordinate
};

__device__ __forceinline__ StepCells start_cells(const QueryParams& P, float x, float y, float z)
{
    const bool ok = (x == x) & (y == y) & (z == z);
    return {grid_cell(P, x), grid_cell(P, y), grid_cell(P, z), ok};
}

// true when the step box [a, b] (per-axis min/max) hits no obstacle.  The grid
// path tests the boxes listed in the cells the step box overlaps, cell by cell
// (x, then y, then z); more than kGridMaxVisit cells, or a NaN end point, fall
// back to testing every box.  sc: cells of a on entry, of b on return.
// PLANAR: z is ignored (a and b carry z = ws_min, grid cell 0).
template <bool PLANAR = false>
__device__ __forceinline__ bool step_free(const QueryParams& P, const GridView& grid, const float4* __restrict__ obs, uint32_t n_obs,
                                          float ax, float ay, float az, float bx, float by, float bz, StepCells& sc, PropCount& cnt)
{
    if(n_obs == 0) return true;
    const float lx = ax > bx ? bx : ax, hx = ax > bx ? ax : bx;
    const float ly = ay > by ? by : ay, hy = ay > by ? ay : by;
    const float lz = az > bz ? bz : az, hz = az > bz ? az : bz;
    // loops stop at the first hit (a flag, not a return from inside them:
    // fewer divergent exits for the compiler to reconverge every step)
    bool hit = false;
    if(grid.start != nullptr)
        {
            const StepCells a = sc;
            sc = start_cells(P, bx, by, bz);
            const int x0 = min(a.x, sc.x), x1 = max(a.x, sc.x);
            const int y0 = min(a.y, sc.y), y1 = max(a.y, sc.y);
            const int z0 = min(a.z, sc.z), z1 = max(a.z, sc.z);
            const int G = (int)P.grid_dim;
            const bool cells_ok = a.ok & sc.ok;
            // the common case, both end points in one cell, runs its own short
            // loop only when it is every running lane's case: a warp whose
            // lanes differ takes the cell-range loop below (the same boxes in
            // the same order for a single cell) instead of running both
            if(__all_sync(__activemask(), cells_ok & (x0 == x1) & (y0 == y1) & (z0 == z1)))
                {
                    // cell coordinates are clamped to [0, G), so both loads stay in bounds
                    const int c0 = (x0 * G + y0) * G + z0;
                    const uint32_t e0 = grid.start[c0 + 1];
                    for(uint32_t j = grid.start[c0]; j < e0 && !hit; ++j)
                        {
                            ++cnt.tests;
                            hit = PLANAR ? box_hit_xy(obs, grid_item(grid, j), lx, ly, hx, hy) : box_hit(obs, grid_item(grid, j), lx, ly, lz, hx, hy, hz);
                        }
                    return !hit;
                }
            const uint32_t n_cells = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1));
            if(cells_ok & (n_cells <= kGridMaxVisit))
                {
                    // the cells in x, y, z order (z fastest) as one loop over
                    // the (x, y) columns: the item lists of a column's cells
                    // z0..z1 lie back to back, so each column is one range
                    // (lanes with different cell ranges part at one loop, not three)
                    const uint32_t n_cols = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1));
                    int cx = x0, cy = y0;
                    for(uint32_t ci = 0; ci < n_cols && !hit; ++ci)
                        {
                            const int c = (cx * G + cy) * G + z0;
                            const uint32_t e = grid.start[c + (z1 - z0) + 1];
                            for(uint32_t k = grid.start[c]; k < e && !hit; ++k)
                                {
                                    ++cnt.tests;
                                    hit = PLANAR ? box_hit_xy(obs, grid_item(grid, k), lx, ly, hx, hy) : box_hit(obs, grid_item(grid, k), lx, ly, lz, hx, hy, hz);
                                }
                            const bool wy = cy < y1;
                            cy = wy ? cy + 1 : y0;
                            cx = wy ? cx : cx + 1;
                        }
                    return !hit;
                }
        }
    for(uint32_t o = 0; o < n_obs; ++o) hit |= PLANAR ? box_hit_xy(obs, o, lx, ly, hx, hy) : box_hit(obs, o, lx, ly, lz, hx, hy, hz);
    cnt.tests += n_obs;
    return !hit;
}

// ---------------------------------------------------------------------------
// Controls and step count (statePropagator.cu:78-81 / 248-253).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int draw_steps(const QueryParams& P, float u)
{
    int k = (int)P.min_steps + (int)(u * P.step_span);
    return k > (int)P.max_steps ? (int)P.max_steps : k;
}

// ---------------------------------------------------------------------------
// Double integrator.  `rule` selects the classic RK4 position update or the
// reference's own formula (statePropagator.cu:97-99, (5v + 2ah) h / 6).
// x0/x1 are sample rows [x y z vx vy vz ax ay az duration].
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool propagate_di(const QueryParams& P, const GridView& grid, const float* x0, const float* u, const float4* obs, uint32_t n_obs,
                                             float* x1, PropCount& cnt)
{
    const float a0 = P.u_min[0] + u[0] * P.u_span[0];
    const float a1 = P.u_min[1] + u[1] * P.u_span[1];
    const float a2 = P.u_min[2] + u[2] * P.u_span[2];
    const int k = draw_steps(P, u[3]);
    const float h = P.step_size;
    float p[3] = {x0[0], x0[1], x0[2]};
    float v[3] = {x0[3], x0[4], x0[5]};
    const float a[3] = {a0, a1, a2};
    const bool ref_rule = P.di_rule == KGMT_DI_RULE_REFERENCE;
    // the velocity increment is the same every step: ((a + 2a) + 2a + a) h / 6
    float dv[3];
#pragma unroll
    for(int d = 0; d < 3; ++d) dv[d] = div6((((a[d] + 2.0f * a[d]) + 2.0f * a[d]) + a[d]) * h);
    StepCells sc = start_cells(P, p[0], p[1], p[2]);
    bool ok = true;
    int done = 0;
    for(int i = 0; i < k; ++i)
        {
            ++done;
            const float q0 = p[0], q1 = p[1], q2 = p[2];
            float x[3];
#pragma unroll
            for(int d = 0; d < 3; ++d)
                {
                    float half = v[d] + (a[d] * h) / 2.0f;
                    float full = v[d] + a[d] * h;
                    float sum = ref_rule ? v[d] + ((v[d] + 2.0f * half) + full) : ((v[d] + 2.0f * half) + 2.0f * half) + full;
                    x[d] = sum * h;
                }
            // one rarely-taken branch per step covers both the exact-division
            // fallback and the bound checks
            const bool exact = div6_exact(x[0]) & div6_exact(x[1]) & div6_exact(x[2]);
            float pn[3];
#pragma unroll
            for(int d = 0; d < 3; ++d) pn[d] = p[d] + div6_fast(x[d]);
#pragma unroll
            for(int d = 0; d < 3; ++d) v[d] = v[d] + dv[d];
            // velocity bound, then workspace bound: either ends the sample here
            bool out = (v[0] < P.v_min) | (v[0] > P.v_max) | (v[1] < P.v_min) | (v[1] > P.v_max) | (v[2] < P.v_min) | (v[2] > P.v_max) |
                       (pn[0] < P.ws_min) | (pn[0] > P.ws_max) | (pn[1] < P.ws_min) | (pn[1] > P.ws_max) | (pn[2] < P.ws_min) |
                       (pn[2] > P.ws_max);
            if(!exact | out)
                {
                    if(!exact)
                        {
#pragma unroll
                            for(int d = 0; d < 3; ++d) pn[d] = p[d] + x[d] / 6.0f;
                            out = (v[0] < P.v_min) | (v[0] > P.v_max) | (v[1] < P.v_min) | (v[1] > P.v_max) | (v[2] < P.v_min) |
                                  (v[2] > P.v_max) | (pn[0] < P.ws_min) | (pn[0] > P.ws_max) | (pn[1] < P.ws_min) | (pn[1] > P.ws_max) |
                                  (pn[2] < P.ws_min) | (pn[2] > P.ws_max);
                        }
                    if(out)
                        {
#pragma unroll
                            for(int d = 0; d < 3; ++d) p[d] = pn[d];
                            ok = false;
                            break;
                        }
                }
#pragma unroll
            for(int d = 0; d < 3; ++d) p[d] = pn[d];
            if(!step_free(P, grid, obs, n_obs, q0, q1, q2, p[0], p[1], p[2], sc, cnt))
                {
                    ok = false;
                    break;
                }
        }
    x1[0] = p[0], x1[1] = p[1], x1[2] = p[2];
    x1[3] = v[0], x1[4] = v[1], x1[5] = v[2];
    x1[6] = a0, x1[7] = a1, x1[8] = a2;
    x1[9] = h * (float)k;
    cnt.steps = done;
    return ok;
}

// ---------------------------------------------------------------------------
// Dubins airplane (statePropagator.cu:147-244): state [x y z yaw pitch v],
// controls drawn as a, yaw rate, pitch rate; row [x y z yaw pitch v | yr pr
// a | k*h].  Yaw and pitch are linear in time within a step and v is linear,
// so the RK4 stages are closed-form: with A the midpoint term,
//   x += (h/6) * ((v cos p) cos y + 2 (A + A) + B)
// in the reference's order (the midpoint stages k2 = k3 coincide).  The end
// stage's attitude is the next step's start attitude (same float operation),
// so its sine and cosine are carried over.  Checks in the reference's order:
// speed, pitch, workspace, obstacles.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool propagate_dubins(const QueryParams& P, const GridView& grid, const float* x0, const float* u, const float4* obs,
                                                 uint32_t n_obs, float* x1, PropCount& cnt)
{
    const float a = P.u_min[0] + u[0] * P.u_span[0];
    const float yr = P.u_min[1] + u[1] * P.u_span[1];
    const float pr = P.u_min[2] + u[2] * P.u_span[2];
    const int k = draw_steps(P, u[3]);
    const float h = P.step_size, hh = P.half_step, h6 = P.sixth_step;
    float x = x0[0], y = x0[1], z = x0[2], yaw = x0[3], pitch = x0[4], v = x0[5];
    const float dvm = hh * a, dve = h * a;               // 0.5 h a, h a
    const float dpm = hh * pr, dym = hh * yr;            // midpoint attitude offsets
    const float dpe = h * pr, dye = h * yr;              // end attitude offsets
    const float dv = h6 * ((a + 2.0f * (a + a)) + a);    // (h/6)(a + 2(a + a) + a)
    float sp, cp, sy, cy;
    sincos_portable(pitch, sp, cp);
    sincos_portable(yaw, sy, cy);
    StepCells sc = start_cells(P, x, y, z);
    bool ok = true;
    int done = 0;
    for(int i = 0; i < k; ++i)
        {
            ++done;
            const float q0 = x, q1 = y, q2 = z;
            float spm, cpm, sym, cym, spe, cpe, sye, cye;
            sincos_portable(pitch + dpm, spm, cpm);
            sincos_portable(yaw + dym, sym, cym);
            sincos_portable(pitch + dpe, spe, cpe);
            sincos_portable(yaw + dye, sye, cye);
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
            const bool out = (v < P.v_min) | (v > P.v_max) | (pitch < P.pitch_min) | (pitch > P.pitch_max) | (x < P.ws_min) | (x > P.ws_max) |
                             (y < P.ws_min) | (y > P.ws_max) | (z < P.ws_min) | (z > P.ws_max);
            if(out)
                {
                    ok = false;
                    break;
                }
            if(!step_free(P, grid, obs, n_obs, q0, q1, q2, x, y, z, sc, cnt))
                {
                    ok = false;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = z, x1[3] = yaw, x1[4] = pitch, x1[5] = v;
    x1[6] = yr, x1[7] = pr, x1[8] = a;
    x1[9] = h * (float)k;
    cnt.steps = done;
    return ok;
}

// ---------------------------------------------------------------------------
// Unicycle (statePropagator.cu:13-74), planar: state [x y theta v], controls
// drawn as a, steering, dt; row [x y theta v | a steering dt].  Explicit Euler
// in the reference's order; tan(steering) is the same every step and is taken
// as sin/cos of the portable pair.  Checks: workspace (x, y), then obstacles
// in the plane (there is no speed check in the reference).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool propagate_unicycle(const QueryParams& P, const GridView& grid, const float* x0, const float* u, const float4* obs,
                                                   uint32_t n_obs, float* x1, PropCount& cnt)
{
    const float a = P.u_min[0] + u[0] * P.u_span[0];
    const float steer = P.u_min[1] + u[1] * P.u_span[1];
    const float dt = P.u_min[2] + u[2] * P.u_span[2];
    const int k = draw_steps(P, u[3]);
    const float h = P.step_size, zw = P.ws_min;
    float x = x0[0], y = x0[1], th = x0[2], v = x0[3];
    float ss, cs;
    sincos_portable(steer, ss, cs);
    const float tan_steer = ss / cs;
    StepCells sc = start_cells(P, x, y, zw);
    bool ok = true;
    int done = 0;
    for(int i = 0; i < k; ++i)
        {
            ++done;
            const float q0 = x, q1 = y;
            float st, ct;
            sincos_portable(th, st, ct);
            x = x + (v * ct) * h;
            y = y + (v * st) * h;
            th = th + ((v / P.wheelbase) * tan_steer) * h;
            v = v + a * h;
            if((x < P.ws_min) | (x > P.ws_max) | (y < P.ws_min) | (y > P.ws_max))
                {
                    ok = false;
                    break;
                }
            if(!step_free<true>(P, grid, obs, n_obs, q0, q1, zw, x, y, zw, sc, cnt))
                {
                    ok = false;
                    break;
                }
        }
    x1[0] = x, x1[1] = y, x1[2] = th, x1[3] = v;
    x1[4] = a, x1[5] = steer, x1[6] = dt;
    cnt.steps = done;
    return ok;
}

// ---------------------------------------------------------------------------
// 12-D quadrotor: state [x y z phi theta psi u v w p q r], controls
// [Zc Lc Mc Nc], classic RK4 over the rigid-body ode of
// statePropagator.cu:325-370 (Euler-angle kinematics, drag -nu|v|, -mu|w|).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void quad_ode(const QueryParams& P, const float* s, float zc, float lc, float mc, float nc, float* d)
{
    const float phi = s[3], theta = s[4], psi = s[5];
    const float uu = s[6], vv = s[7], ww = s[8];
    const float p = s[9], q = s[10], r = s[11];
    float sphi, cphi, sth, cth, spsi, cpsi;
    sincos_portable(phi, sphi, cphi);
    sincos_portable(theta, sth, cth);
    sincos_portable(psi, spsi, cpsi);
    // the two terms over cos(theta) share one division
    const float icth = 1.0f / cth;
    const float tth = sth * icth;
    const float g = P.gravity;
    const float sps = sphi * sth, cps = cphi * sth;
    d[0] = fmaf(fmaf(cps, cpsi, sphi * spsi), ww, fmaf(fmaf(sps, cpsi, -(cphi * spsi)), vv, (cth * cpsi) * uu));
    d[1] = fmaf(fmaf(cps, spsi, -(sphi * cpsi)), ww, fmaf(fmaf(sps, spsi, cphi * cpsi), vv, (cth * spsi) * uu));
    d[2] = fmaf(cphi * cth, ww, fmaf(sphi * cth, vv, (-sth) * uu));
    const float qr = fmaf(q, sphi, r * cphi);
    d[3] = fmaf(qr, tth, p);
    d[4] = fmaf(q, cphi, -(r * sphi));
    d[5] = qr * icth;
    const float xyz = (-P.nu) * sqrtf(fmaf(ww, ww, fmaf(vv, vv, uu * uu)));
    const float mx = P.mass_inv * xyz;
    d[6] = fmaf(mx, uu, fmaf(-g, sth, fmaf(r, vv, -(q * ww))));
    d[7] = fmaf(mx, vv, fmaf(g * cth, sphi, fmaf(p, ww, -(r * uu))));
    d[8] = fmaf(P.mass_inv, zc, fmaf(mx, ww, fmaf(g * cth, cphi, fmaf(q, uu, -(p * vv)))));
    const float lmn = (-P.mu) * sqrtf(fmaf(r, r, fmaf(q, q, p * p)));
    d[9] = fmaf(P.iix, lc, fmaf(P.iix * lmn, p, (P.jx * q) * r));
    d[10] = fmaf(P.iiy, mc, fmaf(P.iiy * lmn, q, (P.jy * p) * r));
    d[11] = fmaf(P.iiz, nc, fmaf(P.iiz * lmn, r, (P.jz * p) * q));
}

__device__ __forceinline__ bool propagate_quad(const QueryParams& P, const GridView& grid, const float* x0, const float* u, const float4* obs, uint32_t n_obs,
                                               float* x1, PropCount& cnt)
{
    const float zc = P.u_min[0] + u[0] * P.u_span[0];
    const float lc = P.u_min[1] + u[1] * P.u_span[1];
    const float mc = P.u_min[2] + u[2] * P.u_span[2];
    const float nc = P.u_min[3] + u[3] * P.u_span[3];
    const int k_steps = draw_steps(P, u[4]);
    const float h = P.step_size, hh = P.half_step, h6 = P.sixth_step;
    // RK4 with the stage sum accumulated as each derivative arrives:
    // acc = k1; acc = fma(2, k2, acc); acc = fma(2, k3, acc); acc += k4 is
    // exactly fma(2, k3, fma(2, k2, k1)) + k4, with one derivative live at a time
    float s[12], k[12], t[12], acc[12];
#pragma unroll
    for(int j = 0; j < 12; ++j) s[j] = x0[j];
    StepCells sc = start_cells(P, s[0], s[1], s[2]);
    bool ok = true;
    int done = 0;
    for(int i = 0; i < k_steps; ++i)
        {
            ++done;
            const float q0 = s[0], q1 = s[1], q2 = s[2];
            quad_ode(P, s, zc, lc, mc, nc, k);
#pragma unroll
            for(int j = 0; j < 12; ++j) acc[j] = k[j], t[j] = fmaf(hh, k[j], s[j]);
            quad_ode(P, t, zc, lc, mc, nc, k);
#pragma unroll
            for(int j = 0; j < 12; ++j) acc[j] = fmaf(2.0f, k[j], acc[j]), t[j] = fmaf(hh, k[j], s[j]);
            quad_ode(P, t, zc, lc, mc, nc, k);
#pragma unroll
            for(int j = 0; j < 12; ++j) acc[j] = fmaf(2.0f, k[j], acc[j]), t[j] = fmaf(h, k[j], s[j]);
            quad_ode(P, t, zc, lc, mc, nc, k);
#pragma unroll
            for(int j = 0; j < 12; ++j) s[j] = fmaf(h6, acc[j] + k[j], s[j]);
            const bool out = (s[6] < P.v_min) | (s[6] > P.v_max) | (s[7] < P.v_min) | (s[7] > P.v_max) | (s[8] < P.v_min) |
                             (s[8] > P.v_max) | (s[0] < P.ws_min) | (s[0] > P.ws_max) | (s[1] < P.ws_min) | (s[1] > P.ws_max) |
                             (s[2] < P.ws_min) | (s[2] > P.ws_max);
            if(out)
                {
                    ok = false;
                    break;
                }
            if(!step_free(P, grid, obs, n_obs, q0, q1, q2, s[0], s[1], s[2], sc, cnt))
                {
                    ok = false;
                    break;
                }
        }
#pragma unroll
    for(int j = 0; j < 12; ++j) x1[j] = s[j];
    x1[12] = zc, x1[13] = lc, x1[14] = mc, x1[15] = nc;
    x1[16] = h * (float)k_steps;
    cnt.steps = done;
    return ok;
}

}  // namespace kgmt
