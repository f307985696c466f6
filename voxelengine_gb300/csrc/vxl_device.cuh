// vxl_device.cuh — device-side building blocks of the voxel-lighting path.
//
// Every translation unit that includes this file is compiled with
// -fmad=false -prec-div=true -prec-sqrt=true -ftz=false, so each arithmetic
// operation below is one IEEE fp32 rounding: the same arithmetic the shaders
// specify (Sources/Shaders/lib/Light.frag) evaluated the way the reference's
// glm-based host code evaluates it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "vxl_internal.h"

namespace vxl {

// ------------------------------------------------------------------ grid
// Fine voxel (x,y,z) lives in the 4x4x4 brick word
//   word = (x>>2) + (y>>2)*bx + (z>>2)*bx*by       (bricks in x-fastest order)
// at bit (x&3) + (y&3)*4 + (z&3)*16. One zero brick pads the + side of every
// axis, so cells up to n+1 (the reference DDA's inclusive upper bound) address
// valid, empty memory. A separate bitmap holds one bit per 8^3 tile
// (tile (x>>3) + (y>>3)*tx + (z>>3)*tx*ty), set when any voxel of it is set.
struct GridView {
    const uint64_t* __restrict__ words;
    const uint32_t* __restrict__ tmask;
    int nx, ny, nz;
    int bx;        // bricks along x (padding included)
    uint32_t bxy;  // bricks per z slice
    int tx;        // tiles along x
    uint32_t txy;  // tiles per z slice
    uint32_t ux, uy, uz;  // nx + 1, ny + 1, nz + 1: the DDA's inclusive bounds (Light.frag:53-55)
};

inline GridView view_of(const vxl_grid* g) {
    GridView v;
    v.words = g->words;
    v.tmask = g->tmask;
    v.nx = g->nx;
    v.ny = g->ny;
    v.nz = g->nz;
    v.bx = g->bx;
    v.bxy = (uint32_t)g->bx * (uint32_t)g->by;
    v.tx = g->tx;
    v.txy = (uint32_t)g->tx * (uint32_t)g->ty;
    v.ux = (uint32_t)g->nx + 1u;
    v.uy = (uint32_t)g->ny + 1u;
    v.uz = (uint32_t)g->nz + 1u;
    return v;
}

__device__ __forceinline__ uint32_t word_index(const GridView& g, int x, int y, int z) {
    return (uint32_t)(x >> 2) + (uint32_t)(y >> 2) * (uint32_t)g.bx + (uint32_t)(z >> 2) * g.bxy;
}
__device__ __forceinline__ uint32_t bit_index(int x, int y, int z) {
    return (uint32_t)((x & 3) | ((y & 3) << 2) | ((z & 3) << 4));
}
// occupancy of a fine voxel; cells outside [0,n) read as empty
__device__ __forceinline__ bool fine_at(const GridView& g, int x, int y, int z) {
    if ((unsigned)x >= (unsigned)g.nx || (unsigned)y >= (unsigned)g.ny || (unsigned)z >= (unsigned)g.nz) return false;
    uint64_t w = __ldg(g.words + word_index(g, x, y, z));
    return (w >> bit_index(x, y, z)) & 1ull;
}
// texelFetch(SHADOW_VOX_TEXTURE, b, 0).r != 0 for ShadowVox byte b, i.e. any
// voxel of the 2x2x2 block at 2*b (robust access: outside -> 0)
__device__ __forceinline__ bool block2_any(const GridView& g, int bx, int by, int bz) {
    int x = 2 * bx, y = 2 * by, z = 2 * bz;
    if ((unsigned)x >= (unsigned)g.nx || (unsigned)y >= (unsigned)g.ny || (unsigned)z >= (unsigned)g.nz) return false;
    uint64_t w = __ldg(g.words + word_index(g, x, y, z));
    uint32_t sh = bit_index(x, y, z);  // x,y,z even: block bits are sh + {0,1,4,5,16,17,20,21}
    return ((w >> sh) & 0x0000000000330033ull) != 0ull;
}

// ---------------------------------------------------------- trace layout
// The grid as the occlusion traversal reads it (see vxl_grid_desc): cell x at
// x' = x + 4, brick (x'>>2, y'>>2, z'>>2) at word (x'>>2) + ((y'>>2) << lbx) +
// ((z'>>2) << (lbx + lby)), bit (x'&3) + 4(y'&3) + 16(z'&3); the cells with a
// coordinate equal to -1 or n+2 (and all three in [-1, n+2]) are set.
struct TraceLayout {
    uint64_t* words;
    int lbx, lby, bz;
    int nx, ny, nz;
};

// The bit address of a cell splits into one term per axis,
//   A = ax(x') + ay(y') + az(z'),
//   ax = (x'&3)      | (x'>>2) << 6
//   ay = (y'&3) << 2 | (y'>>2) << (6 + lbx)
//   az = (z'&3) << 4 | (z'>>2) << (6 + lbx + lby),
// whose bit fields do not overlap. A step of one cell along an axis is an add
// and a mask on that axis's term: the add carries across the bits the other
// axes use (the gap), the mask clears them again. Masks and increments per
// axis (index 0 = x, 1 = y, 2 = z):
struct AxisCode {
    uint32_t field;  // the bits of A this axis owns
    uint32_t keep;   // ~gap: the mask applied after each step
    uint32_t inc;    // increment of a +1 step (gap + unit); a -1 step adds -unit
    uint32_t unit;
    int lo_shift;    // position of the axis's two low bits
    int hi_shift;    // position of its brick index
};
__host__ __device__ inline AxisCode axis_code(int axis, int lbx, int lby) {
    AxisCode c;
    c.lo_shift = 2 * axis;
    c.hi_shift = axis == 0 ? 6 : (axis == 1 ? 6 + lbx : 6 + lbx + lby);
    const uint32_t lo_bits = 3u << c.lo_shift;
    const uint32_t hi_bits = axis == 2 ? ~((1u << c.hi_shift) - 1u)
                                       : (((1u << (axis == 0 ? lbx : lby)) - 1u) << c.hi_shift);
    c.field = lo_bits | hi_bits;
    const uint32_t gap = ((1u << c.hi_shift) - 1u) & ~((4u << c.lo_shift) - 1u);
    c.keep = ~gap;
    c.unit = 1u << c.lo_shift;
    c.inc = gap + c.unit;
    return c;
}
// the axis term of shifted coordinate v (v >= 0)
__host__ __device__ inline uint32_t axis_term(const AxisCode& c, int v) {
    return ((uint32_t)(v & 3) << c.lo_shift) | ((uint32_t)(v >> 2) << c.hi_shift);
}

// ------------------------------------------------------------------ math
struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(f3 a, f3 b) {
    float t = a.x * b.x + a.y * b.y;
    return t + a.z * b.z;
}
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float glsl_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float glsl_step(float e, float x) { return x < e ? 0.0f : 1.0f; }
// mod(x, 0.5) exactly: x/0.5 = 2x, 0.5*floor(2x) and the difference are exact
__device__ __forceinline__ float mod_half(float x) { return x - 0.5f * floorf(x * 2.0f); }
// glm::normalize: v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ f3 normalize(f3 v) {
    float r = 1.0f / sqrtf(dot(v, v));
    return mul(v, r);
}
__device__ __forceinline__ f3 mix(f3 a, f3 b, float t) {
    float u = 1.0f - t;
    return add(mul(a, u), mul(b, t));
}
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ f3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float* p, f3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// sin/cos of this library: Cody-Waite reduction by pi/2 split in three parts
// (P1 = 201/128 exact, P2 with 12 significant bits, P3 the float remainder),
// Taylor polynomials through r^9 (sin) and r^10 (cos), Horner without FMA.
// Accurate to ~1 ulp on [0, 2*pi]; identical bits to the oracle's.
__device__ __forceinline__ void sincos_own(float x, float* s, float* c) {
    float kf = rintf(x * 0.6366197466850281f);
    int k = (int)kf;
    float r = x - kf * 1.5703125f;
    r = r - kf * 0.0004838705062866211f;
    r = r - kf * -4.371138828673793e-08f;
    float r2 = r * r;
    float ps = -1.9841270113829523e-04f + r2 * 2.7557318844628753e-06f;
    ps = 8.333333767950535e-03f + r2 * ps;
    ps = -1.666666716337204e-01f + r2 * ps;
    float sn = r + (r * r2) * ps;
    float pc = 2.4801587642286904e-05f + r2 * -2.755731998149713e-07f;
    pc = -1.3888889225199819e-03f + r2 * pc;
    pc = 4.16666679084301e-02f + r2 * pc;
    pc = -0.5f + r2 * pc;
    float cs = 1.0f + r2 * pc;
    switch (k & 3) {
        case 0: *s = sn; *c = cs; break;
        case 1: *s = cs; *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

// PCG hash (Jarzynski & Olano, JCGT 2020)
__host__ __device__ __forceinline__ uint32_t pcg(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float rand01(uint32_t seed_h, uint32_t pixel, uint32_t sample) {
    // seed_h = pcg(seed), hoisted by callers
    return u01(pcg(pcg(seed_h + pixel) + sample));
}

// cosineSampleHemisphere, Sources/Shaders/LightAmbient.frag:81-87
__device__ __forceinline__ f3 cosine_sample(float u1, float u2) {
    float r = sqrtf(u1);
    float theta = 6.283f * u2;
    float s, c;
    sincos_own(theta, &s, &c);
    float z1 = 1.0f - u1;
    return mk(r * c, r * s, sqrtf(z1 > 0.0f ? z1 : 0.0f));
}
// tangent frame of calculateAmbientIrradiance, LightAmbient.frag:112-113
__device__ __forceinline__ void tangent_frame(f3 n, f3* t, f3* b) {
    *t = fabsf(n.z) > 0.5f ? mk(0.0f, -n.z, n.y) : mk(-n.y, n.x, 0.0f);
    *b = cross(n, *t);
}
__device__ __forceinline__ f3 frame_dir(f3 t, f3 b, f3 n, f3 l) {
    return add(add(mul(t, l.x), mul(b, l.y)), mul(n, l.z));
}

// --------------------------------------------------------------- records
struct Hit {
    int vx, vy, vz;
    float t;
    int steps;
    int flags;
};
__device__ __forceinline__ void store_record(vxl_ray_record* r, const Hit& h) {
    int4 a = make_int4(h.vx, h.vy, h.vz, __float_as_int(h.t));
    int2 b = make_int2(h.steps, h.flags);
    // records are 24 bytes: write as 3 x int2 to keep 8-byte alignment
    int2* p = reinterpret_cast<int2*>(r);
    p[0] = make_int2(a.x, a.y);
    p[1] = make_int2(a.z, a.w);
    p[2] = b;
}

__device__ __forceinline__ bool ray_domain_ok(f3 o, f3 d) {
    const float lim = 1073741824.0f;  // 2^30: floor(o) must fit an int
    return isfinite(o.x) && isfinite(o.y) && isfinite(o.z) && isfinite(d.x) && isfinite(d.y) && isfinite(d.z) &&
           fabsf(o.x) < lim && fabsf(o.y) < lim && fabsf(o.z) < lim;
}

// ---------------------------------------------------------------- DDA
// raycastShadowVolume, Sources/Shaders/lib/Light.frag:29-81. The outer
// `++i < 4` loop re-runs an identical pass (mip stays 0), so one pass is the
// whole result.
//
// Literal form: float select vector and products exactly as written, with
// IEEE inf/NaN behaviour; used for directions with a zero or tiny component.
static __device__ __noinline__ Hit dda_literal(const GridView& g, f3 o, f3 d, float maxt) {
    Hit r{0, 0, 0, 0.0f, 0, 0};
    f3 ss = mk(glsl_sign(d.x), glsl_sign(d.y), glsl_sign(d.z));
    f3 td = mk(1.0f / (d.x * ss.x), 1.0f / (d.y * ss.y), 1.0f / (d.z * ss.z));
    int cx = (int)floorf(o.x), cy = (int)floorf(o.y), cz = (int)floorf(o.z);
    f3 nb = mk((float)cx + (ss.x * 0.5f + 0.5f), (float)cy + (ss.y * 0.5f + 0.5f), (float)cz + (ss.z * 0.5f + 0.5f));
    f3 tm = mk((nb.x - o.x) / d.x, (nb.y - o.y) / d.y, (nb.z - o.z) / d.z);
    const int ux = g.nx + 1, uy = g.ny + 1, uz = g.nz + 1;
    int n = 0;
    float totalt = 0.0f;
    do {
        float selx = glsl_step(tm.x, tm.z) * glsl_step(tm.x, tm.y);
        float sely = glsl_step(tm.y, tm.x) * glsl_step(tm.y, tm.z);
        float selz = glsl_step(tm.z, tm.y) * glsl_step(tm.z, tm.x);
        r.vx = cx;
        r.vy = cy;
        r.vz = cz;
        if (cx < 0 || cy < 0 || cz < 0 || cx > ux || cy > uy || cz > uz) {
            r.flags |= VXL_RF_EXIT_BOUNDS;
            r.t = totalt;
            return r;
        }
        r.steps++;
        bool voxel = fine_at(g, cx, cy, cz);
        float best_t = tm.x * selx + tm.y * sely;
        best_t = best_t + tm.z * selz;
        if (voxel) {
            r.t = best_t;
            r.flags = VXL_RF_HIT | (selx != 0.0f ? VXL_RF_SELX : 0) | (sely != 0.0f ? VXL_RF_SELY : 0) |
                      (selz != 0.0f ? VXL_RF_SELZ : 0);
            return r;
        }
        cx += (int)(selx * ss.x);
        cy += (int)(sely * ss.y);
        cz += (int)(selz * ss.z);
        tm.x += td.x * selx;
        tm.y += td.y * sely;
        tm.z += td.z * selz;
        totalt = best_t;
    } while (++n < 256 && totalt < maxt);
    r.flags |= (n >= 256) ? VXL_RF_EXIT_STEPS : VXL_RF_EXIT_MAXT;
    r.t = totalt;
    return r;
}

// Fast form, exact for directions whose components all have |d| >= 1e-30:
// then every t_max stays finite (|t| <= 1e30 + 256e30), the select vector is
// "components equal to the minimum" (ties select several axes, as step()
// does), and the reference's dot(t_max, select) and t_max += t_delta*select
// reduce to sums of the selected components (unselected components are > 0,
// so their products are +0). The 4^3 brick word of the current cell is kept
// in a register and reloaded only when the cell leaves it.
struct DState {
    int cx, cy, cz;
    float tx, ty, tz;
    float tdx, tdy, tdz;
    int sx, sy, sz;   // step signs, +1 / -1
    float maxt;
    float tot;        // totalt: best_t of the previous step
    int n;            // the reference's n; also the number of fetches made
    bool leap;        // empty bricks may be crossed in one go (see dda_leap)
    uint32_t wcur;
    uint64_t word;
};

// state after `vec3 stepSign = sign(direction) ... t_max = ...` (Light.frag:32-46)
__device__ __forceinline__ void dda_init(DState& s, f3 o, f3 d, float maxt) {
    s.sx = d.x > 0.0f ? 1 : -1;
    s.sy = d.y > 0.0f ? 1 : -1;
    s.sz = d.z > 0.0f ? 1 : -1;
    // 1/|d|: the correctly rounded reciprocal, which is what the IEEE division 1/|d| gives
    s.tdx = __frcp_rn(fabsf(d.x));
    s.tdy = __frcp_rn(fabsf(d.y));
    s.tdz = __frcp_rn(fabsf(d.z));
    s.cx = (int)floorf(o.x);
    s.cy = (int)floorf(o.y);
    s.cz = (int)floorf(o.z);
    s.tx = (((float)s.cx + (s.sx > 0 ? 1.0f : 0.0f)) - o.x) / d.x;
    s.ty = (((float)s.cy + (s.sy > 0 ? 1.0f : 0.0f)) - o.y) / d.y;
    s.tz = (((float)s.cz + (s.sz > 0 ? 1.0f : 0.0f)) - o.z) / d.z;
    s.maxt = maxt;
    s.tot = 0.0f;
    s.n = 0;
    s.leap = false;
    s.wcur = 0xffffffffu;
    s.word = 0;
}

// Whether a ray may leap: the 256-iteration cap of Light.frag:75 can never be
// reached before totalt >= maxt. Axis i crosses at most maxt*|d_i| + 2 cell
// faces before time maxt, so with maxt*|d|_1 < 240 the loop always ends by
// maxt, a hit or the bounds, and n no longer affects the result.
__device__ __forceinline__ bool leap_allowed(f3 d, float maxt) {
    return maxt * (fabsf(d.x) + fabsf(d.y) + fabsf(d.z)) < 240.0f;
}

// Cross the empty 4^3 brick holding the current cell in one go. Inside an
// empty brick every test misses, so the iterations until the cell leaves the
// brick only move the per-axis state: axis i crosses its faces at the times
// T_i(0) = t_i, T_i(j+1) = T_i(j) + td_i (the same float adds the stepping
// does), the brick is left at X = min_i T_i(e_i - 1) (e_i = cells to the brick
// face), and every crossing at a time <= X is taken, ties included. Exact when
// no iteration before the exit can stop the loop: totalt of an iteration is
// at most 3*time, so fl(3X) < maxt suffices (the cap is excluded by
// leap_allowed). totalt after the exit iteration is the sum of the t_max
// components equal to X. Returns false (state untouched) if the condition fails.
__device__ __forceinline__ bool dda_leap(DState& s) {
    const int lx = s.cx & 3, ly = s.cy & 3, lz = s.cz & 3;
    const int ex = s.sx > 0 ? 4 - lx : lx + 1;
    const int ey = s.sy > 0 ? 4 - ly : ly + 1;
    const int ez = s.sz > 0 ? 4 - lz : lz + 1;
    float xx = s.tx, xy = s.ty, xz = s.tz;
    for (int j = 1; j < ex; j++) xx = xx + s.tdx;
    for (int j = 1; j < ey; j++) xy = xy + s.tdy;
    for (int j = 1; j < ez; j++) xz = xz + s.tdz;
    const float X = fminf(fminf(xx, xy), xz);
    if (!(3.0f * X < s.maxt)) return false;
    int kx = 0, ky = 0, kz = 0;
    float px = s.tx, py = s.ty, pz = s.tz;  // last crossing time taken per axis
    for (; kx < ex && s.tx <= X; kx++) { px = s.tx; s.tx = s.tx + s.tdx; }
    for (; ky < ey && s.ty <= X; ky++) { py = s.ty; s.ty = s.ty + s.tdy; }
    for (; kz < ez && s.tz <= X; kz++) { pz = s.tz; s.tz = s.tz + s.tdz; }
    s.cx += s.sx * kx;
    s.cy += s.sy * ky;
    s.cz += s.sz * kz;
    s.n += kx + ky + kz;
    // the exit iteration selects the axes whose crossing time equals X
    const bool ax = kx > 0 && px == X, ay = ky > 0 && py == X, az = kz > 0 && pz == X;
    float best = (ax ? X : 0.0f) + (ay ? X : 0.0f);
    s.tot = best + (az ? X : 0.0f);
    return true;
}

// Up to `budget` iterations of the inner do-while of Light.frag:50-75.
// Returns 0 while the ray goes on; otherwise the record flags, r filled in.
// After a leap (s.leap) a miss may report an approximate cell, t and count;
// hits are always found by exact stepping.
// CACHE: keep the current brick word in registers (one load per brick
// entered); otherwise read it at every step, which is faster while the grid
// stays in L2 (fewer live registers) and slower for grids that do not.
// ONE_COUNT: the step budget and the 256-step cap share one limit, so a step
// tests one counter (faster in the single-scene pool, slower in the batched
// one, whose register allocation differs).
template <bool LEAP, bool CACHE, bool ONE_COUNT>
__device__ __forceinline__ int dda_steps(const GridView& g, DState& s, Hit& r, int budget) {
    const int lim = ONE_COUNT ? min(s.n + budget, 256) : 256;
    for (int it = 0; ONE_COUNT || it < budget; it++) {
        if ((unsigned)s.cx > g.ux || (unsigned)s.cy > g.uy || (unsigned)s.cz > g.uz) {
            r = Hit{s.cx, s.cy, s.cz, s.tot, s.n, VXL_RF_EXIT_BOUNDS};
            return VXL_RF_EXIT_BOUNDS;
        }
        uint64_t word;
        if (CACHE) {
            const uint32_t wi = word_index(g, s.cx, s.cy, s.cz);
            if (wi != s.wcur) {
                s.wcur = wi;
                s.word = __ldg(g.words + wi);
            }
            word = s.word;
        } else {
            word = __ldg(g.words + word_index(g, s.cx, s.cy, s.cz));
        }
        if (LEAP && s.leap && word == 0ull && dda_leap(s)) {
            if (!(s.tot < s.maxt)) {
                r = Hit{s.cx, s.cy, s.cz, s.tot, s.n, VXL_RF_EXIT_MAXT};
                return VXL_RF_EXIT_MAXT;
            }
            continue;
        }
        const float m = fminf(fminf(s.tx, s.ty), s.tz);
        const bool bx = s.tx == m, by = s.ty == m, bz = s.tz == m;
        // dot(t_max, select): the minimum itself unless several axes tie
        // (+0.0f turns a -0 minimum into the +0 the dot product gives)
        float best = m + 0.0f;
        if ((bx && (by || bz)) || (by && bz)) {
            best = (bx ? s.tx : 0.0f) + (by ? s.ty : 0.0f);
            best = best + (bz ? s.tz : 0.0f);
        }
        if ((word >> bit_index(s.cx, s.cy, s.cz)) & 1ull) {
            const int f = VXL_RF_HIT | (bx ? VXL_RF_SELX : 0) | (by ? VXL_RF_SELY : 0) | (bz ? VXL_RF_SELZ : 0);
            r = Hit{s.cx, s.cy, s.cz, best, s.n + 1, f};
            return f;
        }
        const int px = s.cx, py = s.cy, pz = s.cz;
        if (bx) { s.cx += s.sx; s.tx = s.tx + s.tdx; }
        if (by) { s.cy += s.sy; s.ty = s.ty + s.tdy; }
        if (bz) { s.cz += s.sz; s.tz = s.tz + s.tdz; }
        s.tot = best;
        if (!(++s.n < lim && best < s.maxt)) {
            if (ONE_COUNT && s.n < 256 && best < s.maxt) return 0;  // budget spent; the ray goes on
            // the record reports the last cell tested, not the advanced one
            const int f = s.n >= 256 ? VXL_RF_EXIT_STEPS : VXL_RF_EXIT_MAXT;
            r = Hit{px, py, pz, best, s.n, f};
            return f;
        }
    }
    return 0;
}

// `budget` iterations that can meet neither the bounds nor the 256-step cap
// (the caller has checked both for the whole budget): only a hit or
// totalt >= maxt ends the ray early, the step count follows the iteration
// index, and with a compile-time budget the loop unrolls without a counter.
template <bool CACHE>
__device__ __forceinline__ int dda_steps_clear(const GridView& g, DState& s, Hit& r, int budget) {
#pragma unroll
    for (int it = 0; it < budget; it++) {
        uint64_t word;
        if (CACHE) {
            const uint32_t wi = word_index(g, s.cx, s.cy, s.cz);
            if (wi != s.wcur) {
                s.wcur = wi;
                s.word = __ldg(g.words + wi);
            }
            word = s.word;
        } else {
            word = __ldg(g.words + word_index(g, s.cx, s.cy, s.cz));
        }
        const float m = fminf(fminf(s.tx, s.ty), s.tz);
        const bool bx = s.tx == m, by = s.ty == m, bz = s.tz == m;
        float best = m + 0.0f;
        if ((bx && (by || bz)) || (by && bz)) {
            best = (bx ? s.tx : 0.0f) + (by ? s.ty : 0.0f);
            best = best + (bz ? s.tz : 0.0f);
        }
        if ((word >> bit_index(s.cx, s.cy, s.cz)) & 1ull) {
            const int f = VXL_RF_HIT | (bx ? VXL_RF_SELX : 0) | (by ? VXL_RF_SELY : 0) | (bz ? VXL_RF_SELZ : 0);
            r = Hit{s.cx, s.cy, s.cz, best, s.n + it + 1, f};
            return f;
        }
        const int px = s.cx, py = s.cy, pz = s.cz;
        if (bx) { s.cx += s.sx; s.tx = s.tx + s.tdx; }
        if (by) { s.cy += s.sy; s.ty = s.ty + s.tdy; }
        if (bz) { s.cz += s.sz; s.tz = s.tz + s.tdz; }
        s.tot = best;
        if (!(best < s.maxt)) {
            s.n += it + 1;
            r = Hit{px, py, pz, best, s.n, VXL_RF_EXIT_MAXT};
            return VXL_RF_EXIT_MAXT;
        }
    }
    s.n += budget;
    return 0;
}

// Without the leap an iteration moves the cell by at most one along each
// axis, so from a cell within the bounds the next m + 1 iterations, m the
// fewest cells to the bound along any axis's step direction, test cells within
// the bounds too. With SKIP_BOUNDS, when that covers the budget for every
// active lane of the warp and no lane can reach the 256-step cap in it, the
// warp runs the budget without the bounds test and the step counter;
// otherwise it keeps both at every iteration (a per-lane choice would run both
// loops one after the other). Faster in the single-scene pool, slower in the
// batched kernel (-10%), which keeps the tests.
template <bool LEAP = false, bool CACHE = true, bool ONE_COUNT = false, bool SKIP_BOUNDS = false>
__device__ __forceinline__ int dda_run(const GridView& g, DState& s, Hit& r, int budget) {
    if (SKIP_BOUNDS && !LEAP) {
        const int mx = s.sx > 0 ? (int)g.ux - s.cx : s.cx;
        const int my = s.sy > 0 ? (int)g.uy - s.cy : s.cy;
        const int mz = s.sz > 0 ? (int)g.uz - s.cz : s.cz;
        const bool inside = (unsigned)s.cx <= g.ux && (unsigned)s.cy <= g.uy && (unsigned)s.cz <= g.uz;
        const bool clear = inside && min(min(mx, my), mz) >= budget - 1 && s.n + budget < 256;
        if (__all_sync(__activemask(), clear)) return dda_steps_clear<CACHE>(g, s, r, budget);
    }
    return dda_steps<LEAP, CACHE, ONE_COUNT>(g, s, r, budget);
}

__device__ __forceinline__ Hit dda_fast(const GridView& g, f3 o, f3 d, float maxt) {
    DState s;
    dda_init(s, o, d, maxt);
    Hit r;
    while (dda_run(g, s, r, 1 << 20) == 0) {
    }
    return r;
}

__device__ __forceinline__ bool dir_fast_ok(f3 d) {
    return fabsf(d.x) >= 1e-30f && fabsf(d.y) >= 1e-30f && fabsf(d.z) >= 1e-30f;
}

__device__ __forceinline__ Hit dda(const GridView& g, f3 o, f3 d, float maxt) {
    if (!ray_domain_ok(o, d)) {
        Hit r{0, 0, 0, 0.0f, 0, VXL_RF_EXIT_BOUNDS};
        return r;
    }
    if (dir_fast_ok(d)) return dda_fast(g, o, d, maxt);
    return dda_literal(g, o, d, maxt);
}

// ------------------------------------------------------------ marchers
// raycastShadowVolumeSparse (step0 = 0.5) / SuperSparse (step0 = 2.5),
// Sources/Shaders/lib/Light.frag:131-173 / :175-217.
__device__ __forceinline__ Hit march(const GridView& g, f3 origin, f3 dir, float dist, float step0) {
    Hit r{0, 0, 0, dist, 0, 0};
    if (!ray_domain_ok(origin, dir)) return r;
    float stepFactor = step0;
    f3 stepDir = mul(dir, stepFactor);
    f3 pos = origin;
    float d = stepFactor;
    const int sx = g.nx >> 1, sy = g.ny >> 1, sz = g.nz >> 1;
    while (d < 16.0f) {
        // texelFetch(ivec3(pos/2)) with the mod(pos,0.5) > 0.25 bit quirk (:142-148)
        int bx = (int)(pos.x * 0.5f), by = (int)(pos.y * 0.5f), bz = (int)(pos.z * 0.5f);
        int qx = mod_half(pos.x) > 0.25f, qy = mod_half(pos.y) > 0.25f, qz = mod_half(pos.z) > 0.25f;
        r.steps++;
        r.vx = bx * 2 + qx;
        r.vy = by * 2 + qy;
        r.vz = bz * 2 + qz;
        bool inb = (unsigned)bx < (unsigned)sx && (unsigned)by < (unsigned)sy && (unsigned)bz < (unsigned)sz;
        if (inb && fine_at(g, r.vx, r.vy, r.vz)) {
            r.t = d;
            r.flags = VXL_RF_HIT;
            return r;
        }
        pos = add(pos, stepDir);
        d += stepFactor;
    }
    stepFactor *= 2.0f;
    stepDir = mul(stepDir, 2.0f);
    float lod1MaxT = dist < 164.0f ? dist : 164.0f;
    while (d < lod1MaxT) {
        // getVolumeAt(ivec3(pos), 1): byte ivec3(pos)/2 (truncating) != 0
        int ix = (int)pos.x, iy = (int)pos.y, iz = (int)pos.z;
        int bx = ix / 2, by = iy / 2, bz = iz / 2;
        r.steps++;
        r.vx = bx * 2;
        r.vy = by * 2;
        r.vz = bz * 2;
        if (block2_any(g, bx, by, bz)) {
            r.t = d;
            r.flags = VXL_RF_HIT | VXL_RF_COARSE;
            return r;
        }
        pos = add(pos, stepDir);
        d += stepFactor;
    }
    r.t = dist;
    return r;
}

}  // namespace vxl
