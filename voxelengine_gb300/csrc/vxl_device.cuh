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
//   tile = (x>>3) + (y>>3)*tx + (z>>3)*tx*ty,  word = tile*8 + ((x>>2)&1) + ((y>>2)&1)*2 + ((z>>2)&1)*4
// at bit (x&3) + (y&3)*4 + (z&3)*16. Each tile (8^3 voxels) is 64 bytes.
// One zero tile pads the + side of every axis, so cells up to n+1 (the
// reference DDA's inclusive upper bound) address valid, empty memory.
struct GridView {
    const uint64_t* __restrict__ words;
    const uint32_t* __restrict__ tmask;
    int nx, ny, nz;
    int tx, ty, tz;
    uint32_t txy;
};

__device__ __forceinline__ uint32_t word_index(const GridView& g, int x, int y, int z) {
    uint32_t tile = (uint32_t)(x >> 3) + (uint32_t)(y >> 3) * (uint32_t)g.tx + (uint32_t)(z >> 3) * g.txy;
    return tile * 8u + (uint32_t)(((x >> 2) & 1) | (((y >> 2) & 1) << 1) | (((z >> 2) & 1) << 2));
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
__device__ __forceinline__ Hit dda_fast(const GridView& g, f3 o, f3 d, float maxt) {
    Hit r{0, 0, 0, 0.0f, 0, 0};
    const int stx = d.x > 0.0f ? 1 : -1, sty = d.y > 0.0f ? 1 : -1, stz = d.z > 0.0f ? 1 : -1;
    const float tdx = 1.0f / fabsf(d.x), tdy = 1.0f / fabsf(d.y), tdz = 1.0f / fabsf(d.z);
    int cx = (int)floorf(o.x), cy = (int)floorf(o.y), cz = (int)floorf(o.z);
    float tx = (((float)cx + (stx > 0 ? 1.0f : 0.0f)) - o.x) / d.x;
    float ty = (((float)cy + (sty > 0 ? 1.0f : 0.0f)) - o.y) / d.y;
    float tz = (((float)cz + (stz > 0 ? 1.0f : 0.0f)) - o.z) / d.z;
    const unsigned ux = (unsigned)g.nx + 1u, uy = (unsigned)g.ny + 1u, uz = (unsigned)g.nz + 1u;
    uint32_t wcur = 0xffffffffu;
    uint64_t word = 0;
    int n = 0;
    int steps = 0;
    float best = 0.0f, totalt = 0.0f;
    bool bx, by, bz;
    for (;;) {
        float m = fminf(fminf(tx, ty), tz);
        bx = tx == m;
        by = ty == m;
        bz = tz == m;
        if ((unsigned)cx > ux || (unsigned)cy > uy || (unsigned)cz > uz) {
            r.flags = VXL_RF_EXIT_BOUNDS;
            best = totalt;
            break;
        }
        steps++;
        uint32_t wi = word_index(g, cx, cy, cz);
        if (wi != wcur) {
            wcur = wi;
            word = __ldg(g.words + wi);
        }
        best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
        best = best + (bz ? tz : 0.0f);
        if ((word >> bit_index(cx, cy, cz)) & 1ull) {
            r.flags = VXL_RF_HIT | (bx ? VXL_RF_SELX : 0) | (by ? VXL_RF_SELY : 0) | (bz ? VXL_RF_SELZ : 0);
            break;
        }
        if (bx) { cx += stx; tx = tx + tdx; }
        if (by) { cy += sty; ty = ty + tdy; }
        if (bz) { cz += stz; tz = tz + tdz; }
        totalt = best;
        if (!(++n < 256 && totalt < maxt)) {
            r.flags = n >= 256 ? VXL_RF_EXIT_STEPS : VXL_RF_EXIT_MAXT;
            // the record reports the last cell tested, not the advanced one
            if (bx) cx -= stx;
            if (by) cy -= sty;
            if (bz) cz -= stz;
            break;
        }
    }
    r.vx = cx;
    r.vy = cy;
    r.vz = cz;
    r.t = best;
    r.steps = steps;
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
