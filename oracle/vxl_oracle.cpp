// vxl_oracle.cpp — CPU restatement of VoxelEngine's voxel-lighting path.
//
// TEST INFRASTRUCTURE ONLY: the parity checker and timed CPU baseline for the
// CUDA path in voxelengine_gb300/. Nothing in the product links or calls this.
//
// Every function cites the reference lines it restates (paths relative to the
// VoxelEngine source tree). Compiled with -ffp-contract=off so each GLSL/glm
// operation is one IEEE fp32 rounding, like the CUDA path (built -fmad=false).
//
// GLSL built-ins used by the shaders are restated with GLSL semantics:
//   sign(x)   = x>0 ? 1 : x<0 ? -1 : 0           (+0.0 for +-0 and NaN)
//   step(e,x) = x<e ? 0 : 1                       (NaN compares give 1)
//   mod(x,y)  = x - y*floor(x/y)
//   mix(x,y,a)= x*(1-a) + y*a
//   int(x)    = truncation toward zero;  ivec / int = truncation toward zero
//   normalize(v) = v * (1 / sqrt(dot(v,v))), dot = (x*x + y*y) + z*z  (glm's form)
//   out-of-range texelFetch returns 0 (robust image access)
// sin/cos are this project's own (Cody-Waite reduction by pi/2 split in three,
// Taylor polynomials through x^9 / x^10, Horner, no FMA), identical in the CUDA
// path; they are not the shaders' driver sin/cos.
#include "vxl_oracle.h"

#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float dot(V3 a, V3 b) {
    float t = a.x * b.x + a.y * b.y;
    return t + a.z * b.z;
}
inline V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float glsl_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float glsl_step(float e, float x) { return x < e ? 0.0f : 1.0f; }
inline float glsl_mod(float x, float y) { return x - y * std::floor(x / y); }
// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
inline V3 normalize(V3 v) {
    float r = 1.0f / std::sqrt(dot(v, v));
    return mul(v, r);
}
inline V3 mix(V3 a, V3 b, float t) {
    float u = 1.0f - t;
    return add(mul(a, u), mul(b, t));
}
inline float smoothstep(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}
inline V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }

// Inputs outside the shader's defined domain (non-finite, or coordinates that
// do not fit an int) give a miss with zero fetches, here and in the CUDA path.
inline bool ray_domain_ok(V3 o, V3 d) {
    const float lim = 1073741824.0f;  // 2^30
    return std::isfinite(o.x) && std::isfinite(o.y) && std::isfinite(o.z) && std::isfinite(d.x) &&
           std::isfinite(d.y) && std::isfinite(d.z) && std::fabs(o.x) < lim && std::fabs(o.y) < lim &&
           std::fabs(o.z) < lim;
}

struct Grid {
    const uint8_t* g;
    int sx, sy, sz;
    // texelFetch(SHADOW_VOX_TEXTURE, pos, 0).r with robust out-of-range = 0
    inline uint32_t texel(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= sx || y >= sy || z >= sz) return 0u;
        return g[(size_t)x + (size_t)y * sx + (size_t)z * sx * sy];
    }
    // getVolumeAt, Sources/Shaders/lib/Light.frag:14-27
    inline bool volume_at(int x, int y, int z, int mip) const {
        int bit = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
        int mask = 1 << bit;
        x /= 2;
        y /= 2;
        z /= 2;
        uint32_t voxel = texel(x, y, z);  // realMip = mip/2 = 0: ShadowVox has one mip
        if (mip % 2 == 1) return voxel != 0u;
        return (voxel & (uint32_t)mask) != 0u;
    }
};

template <typename F>
void parallel_for(int n, int threads, F&& f) {
    if (threads <= 1 || n < 256) {
        for (int i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int> next{0};
    const int chunk = 64;
    auto worker = [&]() {
        for (;;) {
            int s = next.fetch_add(chunk);
            if (s >= n) break;
            int e = s + chunk < n ? s + chunk : n;
            for (int i = s; i < e; i++) f(i);
        }
    };
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
}

// ---------------------------------------------------------------------------
// raycastShadowVolume, Sources/Shaders/lib/Light.frag:29-81 (mip 0 only: the
// outer `++i < 4` loop re-runs an identical pass, see vo_dda_literal).
// `occ(x, y, z)` is the occupancy test of the visited cell; sx,sy,sz are the
// ShadowVox byte dims (fine dims / 2).
template <class Occ>
int dda_t(int gsx, int gsy, int gsz, V3 o, V3 d, float maxt, vo_rec* r, Occ&& occ) {
    vo_rec rec{0, 0, 0, 0.0f, 0, 0};
    if (!ray_domain_ok(o, d)) {
        rec.flags = VO_F_EXIT_BOUNDS;
        if (r) *r = rec;
        return 0;
    }
    V3 ss = v3(glsl_sign(d.x), glsl_sign(d.y), glsl_sign(d.z));
    V3 td = v3(1.0f / (d.x * ss.x), 1.0f / (d.y * ss.y), 1.0f / (d.z * ss.z));
    int cx = (int)std::floor(o.x), cy = (int)std::floor(o.y), cz = (int)std::floor(o.z);
    V3 nb = v3((float)cx + (ss.x * 0.5f + 0.5f), (float)cy + (ss.y * 0.5f + 0.5f),
               (float)cz + (ss.z * 0.5f + 0.5f));
    V3 tm = v3((nb.x - o.x) / d.x, (nb.y - o.y) / d.y, (nb.z - o.z) / d.z);
    // clamp(current_voxel, ivec3(0), ivec3(u_VolumeDimension/mipSize)*2+1)
    const int ux = gsx * 2 + 1, uy = gsy * 2 + 1, uz = gsz * 2 + 1;
    int n = 0;
    float totalt = 0.0f;
    do {
        float selx = glsl_step(tm.x, tm.z) * glsl_step(tm.x, tm.y);
        float sely = glsl_step(tm.y, tm.x) * glsl_step(tm.y, tm.z);
        float selz = glsl_step(tm.z, tm.y) * glsl_step(tm.z, tm.x);
        rec.vx = cx;
        rec.vy = cy;
        rec.vz = cz;
        if (cx < 0 || cy < 0 || cz < 0 || cx > ux || cy > uy || cz > uz) {
            rec.flags |= VO_F_EXIT_BOUNDS;
            rec.t = totalt;
            if (r) *r = rec;
            return 0;
        }
        rec.steps++;
        bool voxel = occ(cx, cy, cz);
        float best_t = tm.x * selx + tm.y * sely;
        best_t = best_t + tm.z * selz;
        if (voxel) {
            rec.t = best_t;
            rec.flags = VO_F_HIT | (selx != 0.0f ? VO_F_SELX : 0) | (sely != 0.0f ? VO_F_SELY : 0) |
                        (selz != 0.0f ? VO_F_SELZ : 0);
            if (r) *r = rec;
            return 1;
        }
        cx += (int)(selx * ss.x);
        cy += (int)(sely * ss.y);
        cz += (int)(selz * ss.z);
        tm.x += td.x * selx;
        tm.y += td.y * sely;
        tm.z += td.z * selz;
        totalt = best_t;
    } while (++n < 256 && totalt < maxt);
    rec.flags |= (n >= 256) ? VO_F_EXIT_STEPS : VO_F_EXIT_MAXT;
    rec.t = totalt;
    if (r) *r = rec;
    return 0;
}

int dda(const Grid& G, V3 o, V3 d, float maxt, vo_rec* r) {
    return dda_t(G.sx, G.sy, G.sz, o, d, maxt, r, [&](int x, int y, int z) { return G.volume_at(x, y, z, 0); });
}

// Shared body of raycastShadowVolumeSparse / SuperSparse,
// Sources/Shaders/lib/Light.frag:131-173 and :175-217.
float march(const Grid& G, V3 origin, V3 dir, float dist, float step0, vo_rec* r) {
    vo_rec rec{0, 0, 0, dist, 0, 0};
    if (!ray_domain_ok(origin, dir)) {
        if (r) *r = rec;
        return dist;
    }
    float stepFactor = step0;
    V3 stepDir = mul(dir, stepFactor);
    V3 pos = origin;
    float d = stepFactor;
    while (d < 16.0f) {
        // texelFetch(SHADOW_VOX_TEXTURE, ivec3(pos/2), 0).r
        int bx = (int)(pos.x / 2.0f), by = (int)(pos.y / 2.0f), bz = (int)(pos.z / 2.0f);
        uint32_t vol = G.texel(bx, by, bz);
        uint32_t bit = 0u;
        int qx = glsl_mod(pos.x, 0.5f) > 0.25f, qy = glsl_mod(pos.y, 0.5f) > 0.25f,
            qz = glsl_mod(pos.z, 0.5f) > 0.25f;
        bit += qx ? 1u : 0u;
        bit += qy ? 2u : 0u;
        bit += qz ? 4u : 0u;
        uint32_t mask = 1u << bit;
        rec.steps++;
        rec.vx = bx * 2 + qx;
        rec.vy = by * 2 + qy;
        rec.vz = bz * 2 + qz;
        if ((mask & vol) != 0u) {
            rec.t = d;
            rec.flags = VO_F_HIT;
            if (r) *r = rec;
            return d;
        }
        pos = add(pos, stepDir);
        d += stepFactor;
    }
    stepFactor *= 2.0f;
    stepDir = mul(stepDir, 2.0f);
    float lod1MaxT = dist < 164.0f ? dist : 164.0f;
    while (d < lod1MaxT) {
        // getVolumeAt(ivec3(pos), 1)
        int ix = (int)pos.x, iy = (int)pos.y, iz = (int)pos.z;
        rec.steps++;
        rec.vx = (ix / 2) * 2;
        rec.vy = (iy / 2) * 2;
        rec.vz = (iz / 2) * 2;
        if (G.volume_at(ix, iy, iz, 1)) {
            rec.t = d;
            rec.flags = VO_F_HIT | VO_F_COARSE;
            if (r) *r = rec;
            return d;
        }
        pos = add(pos, stepDir);
        d += stepFactor;
    }
    if (r) *r = rec;
    return dist;
}

// ---------------------------------------------------------------------------
// sin/cos: own implementation (see file header)
const float kTwoOverPi = 0.6366197466850281f;
const float kP1 = 1.5703125f;
const float kP2 = 0.0004838705062866211f;
const float kP3 = -4.371138828673793e-08f;

void sincos_own(float x, float* s, float* c) {
    float kf = std::rint(x * kTwoOverPi);
    int k = (int)kf;
    float r = x - kf * kP1;
    r = r - kf * kP2;
    r = r - kf * kP3;
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

// PCG hash (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020)
inline uint32_t pcg(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
inline float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }
inline float rand01(uint32_t seed, uint32_t pixel, uint32_t sample) {
    return u01(pcg(pcg(pcg(seed) + pixel) + sample));
}

// cosineSampleHemisphere, Sources/Shaders/LightAmbient.frag:81-87
inline V3 cosine_sample(float u1, float u2) {
    float r = std::sqrt(u1);
    float theta = 6.283f * u2;
    float s, c;
    sincos_own(theta, &s, &c);
    float x = r * c;
    float y = r * s;
    float z1 = 1.0f - u1;
    return v3(x, y, std::sqrt(z1 > 0.0f ? z1 : 0.0f));
}

// tangent frame of calculateAmbientIrradiance, Sources/Shaders/LightAmbient.frag:112-113
inline void tangent_frame(V3 n, V3* t, V3* b) {
    *t = std::fabs(n.z) > 0.5f ? v3(0.0f, -n.z, n.y) : v3(-n.y, n.x, 0.0f);
    *b = cross(n, *t);
}
inline V3 frame_dir(V3 t, V3 b, V3 n, V3 l) { return add(add(mul(t, l.x), mul(b, l.y)), mul(n, l.z)); }

// ---------------------------------------------------------------------------
// DDA-mode per-pixel occlusion (this library's ray generator over the
// reference DDA). Sample ids: spec j -> (2j, 2j+1), AO k -> (64+2k, 65+2k).
void occlusion_pixel(const Grid& G, const float* pos, const float* nrm, const float* rough, int i,
                     const vo_params& p, float* shadow, float* ao, float* ao_vis, float* spec,
                     float* spec_t, vo_rec* recs) {
    const int R = p.n_shadow + p.n_ao + p.n_spec;
    V3 P = load3(pos + 3 * (size_t)i), N = load3(nrm + 3 * (size_t)i);
    if (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f) {  // sky pixel: nothing traced
        if (shadow) shadow[i] = 1.0f;
        if (ao) ao[i] = 1.0f;
        if (ao_vis) ao_vis[i] = 1.0f;
        if (spec) spec[i] = 1.0f;
        if (spec_t) spec_t[i] = p.spec_len;
        if (recs)
            for (int k = 0; k < R; k++) recs[(size_t)i * R + k] = vo_rec{0, 0, 0, 0.0f, 0, 0};
        return;
    }
    V3 O = add(P, mul(N, p.bias));
    int slot = 0;
    float sh = 1.0f;
    if (p.n_shadow > 0) {
        vo_rec rr;
        int h = dda(G, O, load3(p.light_dir), p.shadow_len, &rr);
        sh = h ? 0.0f : 1.0f;
        if (recs) recs[(size_t)i * R + slot] = rr;
        slot++;
    }
    V3 T, B;
    tangent_frame(N, &T, &B);
    float acc = 0.0f, vis = 0.0f;
    for (int k = 0; k < p.n_ao; k++) {
        float u1 = rand01(p.seed, (uint32_t)i, 64u + 2u * k);
        float u2 = rand01(p.seed, (uint32_t)i, 65u + 2u * k);
        V3 l = cosine_sample(u1, u2);
        V3 d = frame_dir(T, B, N, l);
        vo_rec rr;
        int h = dda(G, O, d, p.ao_len, &rr);
        float tt = h ? (rr.t < p.ao_len ? rr.t : p.ao_len) : p.ao_len;
        float q = tt / p.ao_len;
        acc += q * q;
        vis += h ? 0.0f : 1.0f;
        if (recs) recs[(size_t)i * R + slot] = rr;
        slot++;
    }
    float sp = 0.0f, st = 0.0f;
    if (p.n_spec > 0) {
        float ro = rough ? rough[i] : p.default_rough;
        float a = ro * ro;
        float a2 = a * a;
        V3 V = normalize(sub(load3(p.cam_pos), P));
        for (int j = 0; j < p.n_spec; j++) {
            float u1 = rand01(p.seed, (uint32_t)i, 2u * j);
            float u2 = rand01(p.seed, (uint32_t)i, 2u * j + 1u);
            float ct = std::sqrt((1.0f - u1) / (1.0f + (a2 - 1.0f) * u1));
            float st2 = 1.0f - ct * ct;
            float sn = std::sqrt(st2 > 0.0f ? st2 : 0.0f);
            float s, c;
            sincos_own(6.2831855f * u2, &s, &c);
            V3 H = frame_dir(T, B, N, v3(sn * c, sn * s, ct));
            float vh = dot(V, H);
            V3 Rf = sub(mul(H, 2.0f * vh), V);
            V3 d = normalize(Rf);
            vo_rec rr;
            int h = dda(G, O, d, p.spec_len, &rr);
            sp += h ? 0.0f : 1.0f;
            st += h ? rr.t : p.spec_len;
            if (recs) recs[(size_t)i * R + slot] = rr;
            slot++;
        }
    }
    if (shadow) shadow[i] = sh;
    if (ao) ao[i] = p.n_ao > 0 ? acc / (float)p.n_ao : 1.0f;
    if (ao_vis) ao_vis[i] = p.n_ao > 0 ? vis / (float)p.n_ao : 1.0f;
    if (spec) spec[i] = p.n_spec > 0 ? sp / (float)p.n_spec : 1.0f;
    if (spec_t) spec_t[i] = p.n_spec > 0 ? st / (float)p.n_spec : p.spec_len;
}

// value noise with a PCG lattice, smoothstep-weighted trilinear
inline float lattice(int ix, int iy, int iz, uint32_t seed) {
    return u01(pcg((uint32_t)ix + pcg((uint32_t)iy + pcg((uint32_t)iz + seed))));
}
float value_noise3(float x, float y, float z, uint32_t seed) {
    float fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
    int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    float fx = x - fx0, fy = y - fy0, fz = z - fz0;
    float wx = fx * fx * (3.0f - 2.0f * fx);
    float wy = fy * fy * (3.0f - 2.0f * fy);
    float wz = fz * fz * (3.0f - 2.0f * fz);
    float c000 = lattice(ix, iy, iz, seed), c100 = lattice(ix + 1, iy, iz, seed);
    float c010 = lattice(ix, iy + 1, iz, seed), c110 = lattice(ix + 1, iy + 1, iz, seed);
    float c001 = lattice(ix, iy, iz + 1, seed), c101 = lattice(ix + 1, iy, iz + 1, seed);
    float c011 = lattice(ix, iy + 1, iz + 1, seed), c111 = lattice(ix + 1, iy + 1, iz + 1, seed);
    float x00 = c000 + (c100 - c000) * wx;
    float x10 = c010 + (c110 - c010) * wx;
    float x01 = c001 + (c101 - c001) * wx;
    float x11 = c011 + (c111 - c011) * wx;
    float y0 = x00 + (x10 - x00) * wy;
    float y1 = x01 + (x11 - x01) * wy;
    return y0 + (y1 - y0) * wz;
}
// octave sum convention of Sources/Util/Noise.cpp:108-122 (amplitude x0.5,
// frequency x2, normalised by the amplitude sum); octave i uses seed + i*0x9E3779B9
float noise_octaves(float x, float y, float z, uint32_t seed, float freq, int octaves) {
    float total = 0.0f, frequency = freq, amplitude = 1.0f, maxValue = 0.0f;
    for (int i = 0; i < octaves; i++) {
        total += value_noise3(x * frequency, y * frequency, z * frequency, seed + (uint32_t)i * 0x9E3779B9u) *
                 amplitude;
        maxValue += amplitude;
        amplitude *= 0.5f;
        frequency *= 2.0f;
    }
    return total / maxValue;
}

inline void set_fine(uint8_t* g, int sx, int sy, int x, int y, int z) {
    int bit = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    g[(size_t)(x >> 1) + (size_t)(y >> 1) * sx + (size_t)(z >> 1) * sx * sy] |= (uint8_t)(1u << bit);
}

// ShadowVoxSystem::SetVolumeAt, Sources/World/Systems/ShadowVoxSystem.cpp:82-94
inline void set_volume_at(uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int value) {
    if (x < 0 || y < 0 || z < 0 || x >= sx * 2 || y >= sy * 2 || z >= sz * 2) return;
    int bit = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    int mask = 1 << bit;
    x /= 2;
    y /= 2;
    z /= 2;
    uint8_t* data = g + ((size_t)x + ((size_t)y * (size_t)sx) + ((size_t)z * (size_t)sx * sy));
    *data = (uint8_t)((*data & ~mask) | (value << bit));
}

// inner loops of ShadowVoxSystem::OnUpdate, Sources/World/Systems/ShadowVoxSystem.cpp:137-155
// (and :159-177; :22-40 for OnVoxDestroyed). M is column-major 4x4.
void voxelize_model(uint8_t* g, int sx, int sy, int sz, const uint8_t* model, int msx, int msy, int msz,
                    const float* M, int value, int* aabb) {
    V3 o = v3(M[12], M[13], M[14]);
    V3 dx = v3(M[0] * 0.1f, M[1] * 0.1f, M[2] * 0.1f);
    V3 dy = v3(M[4] * 0.1f, M[5] * 0.1f, M[6] * 0.1f);
    V3 dz = v3(M[8] * 0.1f, M[9] * 0.1f, M[10] * 0.1f);
    for (int z = 0; z < msz; z++)
        for (int y = 0; y < msy; y++)
            for (int x = 0; x < msx; x++) {
                // VoxAsset::PixelAt, Sources/Asset/VoxAsset.h:52-56
                uint8_t v = model[(size_t)x + (size_t)y * msx + (size_t)z * msx * msy];
                if (v >= 16) {
                    V3 wp = add(add(add(o, mul(dx, (float)x)), mul(dy, (float)y)), mul(dz, (float)z));
                    int fx = (int)(wp.x * 10.0f), fy = (int)(wp.y * 10.0f), fz = (int)(wp.z * 10.0f);
                    if (aabb) {
                        if (fx < aabb[0]) aabb[0] = fx;
                        if (fy < aabb[1]) aabb[1] = fy;
                        if (fz < aabb[2]) aabb[2] = fz;
                        if (fx > aabb[3]) aabb[3] = fx;
                        if (fy > aabb[4]) aabb[4] = fy;
                        if (fz > aabb[5]) aabb[5] = fz;
                    }
                    set_volume_at(g, sx, sy, sz, fx, fy, fz, value);
                }
            }
}

// glm::translate(m, v): Result[3] = m[0]*v[0] + m[1]*v[1] + m[2]*v[2] + m[3]
void translate(const float* m, const float* v, float* out) {
    std::memcpy(out, m, 16 * sizeof(float));
    for (int r = 0; r < 4; r++) {
        float a = m[0 + r] * v[0] + m[4 + r] * v[1];
        a = a + m[8 + r] * v[2];
        out[12 + r] = a + m[12 + r];
    }
}

// dirty-region tail of OnUpdate, Sources/World/Systems/ShadowVoxSystem.cpp:180-190
void region_from_aabb(const int* aabb, int sx, int sy, int sz, int* region) {
    if (aabb[3] != 0 || aabb[4] != 0 || aabb[5] != 0) {
        int mn[3] = {aabb[0] / 2, aabb[1] / 2, aabb[2] / 2};
        int mx[3] = {aabb[3] / 2, aabb[4] / 2, aabb[5] / 2};
        int lim[3] = {sx - 1, sy - 1, sz - 1};
        for (int a = 0; a < 3; a++) {
            if (mn[a] < 0) mn[a] = 0;
            if (mx[a] > lim[a]) mx[a] = lim[a];
            region[a] = mn[a];
            region[3 + a] = mx[a] - mn[a] + 1;
        }
    } else {
        for (int a = 0; a < 6; a++) region[a] = -1;
    }
}

}  // namespace

// ===========================================================================
extern "C" {

int vo_version(void) { return 1; }

void vo_sincos(float x, float* s, float* c) { sincos_own(x, s, c); }
uint32_t vo_pcg(uint32_t v) { return pcg(v); }
float vo_rand01(uint32_t seed, uint32_t pixel, uint32_t sample) { return rand01(seed, pixel, sample); }

int vo_get_volume_at(const uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int mip) {
    Grid G{g, sx, sy, sz};
    return G.volume_at(x, y, z, mip) ? 1 : 0;
}

int vo_dda(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float maxt, vo_rec* r) {
    Grid G{g, sx, sy, sz};
    return dda(G, load3(o), load3(d), maxt, r);
}

// Literal restatement of Light.frag:29-81 including the outer `++i < 4` loop and
// the shared `totalt`; used only by tests to show it equals the single pass.
int vo_dda_literal(const uint8_t* g, int sx, int sy, int sz, const float* o_in, const float* d_in, float maxt,
                   float* hit, float* normal, int* fetches) {
    Grid G{g, sx, sy, sz};
    V3 origin = load3(o_in), direction = load3(d_in);
    int nf = 0;
    if (!ray_domain_ok(origin, direction)) {
        if (fetches) *fetches = 0;
        return 0;
    }
    V3 stepSign = v3(glsl_sign(direction.x), glsl_sign(direction.y), glsl_sign(direction.z));
    V3 t_delta = v3(1.0f / (direction.x * stepSign.x), 1.0f / (direction.y * stepSign.y),
                    1.0f / (direction.z * stepSign.z));
    int mip = 0;
    int i = 0;
    float totalt = 0.0f;
    do {
        float mipSize = (float)(1 << mip);
        origin = v3(origin.x / mipSize, origin.y / mipSize, origin.z / mipSize);
        int cx = (int)std::floor(origin.x), cy = (int)std::floor(origin.y), cz = (int)std::floor(origin.z);
        V3 nb = v3((float)cx + (stepSign.x * 0.5f + 0.5f), (float)cy + (stepSign.y * 0.5f + 0.5f),
                   (float)cz + (stepSign.z * 0.5f + 0.5f));
        V3 t_max = v3((nb.x - origin.x) / direction.x, (nb.y - origin.y) / direction.y,
                      (nb.z - origin.z) / direction.z);
        int ux = (int)((float)G.sx / mipSize) * 2 + 1, uy = (int)((float)G.sy / mipSize) * 2 + 1,
            uz = (int)((float)G.sz / mipSize) * 2 + 1;
        int n = 0;
        do {
            V3 sel = v3(glsl_step(t_max.x, t_max.z) * glsl_step(t_max.x, t_max.y),
                        glsl_step(t_max.y, t_max.x) * glsl_step(t_max.y, t_max.z),
                        glsl_step(t_max.z, t_max.y) * glsl_step(t_max.z, t_max.x));
            if (cx < 0 || cy < 0 || cz < 0 || cx > ux || cy > uy || cz > uz) {
                if (fetches) *fetches = nf;
                return 0;
            }
            nf++;
            bool voxel = G.volume_at(cx, cy, cz, mip);
            float best_t = dot(t_max, sel);
            if (voxel) {
                if (normal) {
                    normal[0] = -stepSign.x * sel.x;
                    normal[1] = -stepSign.y * sel.y;
                    normal[2] = -stepSign.z * sel.z;
                }
                if (hit) {
                    V3 h = mul(add(origin, mul(direction, best_t)), mipSize);
                    hit[0] = h.x;
                    hit[1] = h.y;
                    hit[2] = h.z;
                }
                if (fetches) *fetches = nf;
                return 1;
            }
            cx += (int)(sel.x * stepSign.x);
            cy += (int)(sel.y * stepSign.y);
            cz += (int)(sel.z * stepSign.z);
            t_max = add(t_max, mulv(t_delta, sel));
            totalt = best_t;
        } while (++n < 256 && totalt < maxt);
        origin = mul(origin, mipSize);
    } while (++i < 4);
    if (fetches) *fetches = nf;
    return 0;
}

float vo_sparse(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float dist, vo_rec* r) {
    Grid G{g, sx, sy, sz};
    return march(G, load3(o), load3(d), dist, 0.5f, r);
}
float vo_supersparse(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float dist,
                     vo_rec* r) {
    Grid G{g, sx, sy, sz};
    return march(G, load3(o), load3(d), dist, 2.5f, r);
}

void vo_cosine_sample(float u1, float u2, float* out3) {
    V3 v = cosine_sample(u1, u2);
    out3[0] = v.x;
    out3[1] = v.y;
    out3[2] = v.z;
}

void vo_trace_rays(const uint8_t* g, int sx, int sy, int sz, const float* rays, int n, int mode, vo_rec* recs,
                   int threads) {
    Grid G{g, sx, sy, sz};
    parallel_for(n, threads, [&](int i) {
        const float* q = rays + 7 * (size_t)i;
        V3 o = load3(q), d = load3(q + 3);
        if (mode == VO_MODE_DDA)
            dda(G, o, d, q[6], recs + i);
        else
            march(G, o, d, q[6], mode == VO_MODE_SPARSE ? 0.5f : 2.5f, recs + i);
    });
}

void vo_occlusion(const uint8_t* g, int sx, int sy, int sz, const float* pos, const float* nrm, const float* rough,
                  int npix, const vo_params* p, float* shadow, float* ao, float* ao_vis, float* spec, float* spec_t,
                  vo_rec* recs, int p0, int p1, int threads) {
    Grid G{g, sx, sy, sz};
    if (p0 < 0) p0 = 0;
    if (p1 > npix || p1 < 0) p1 = npix;
    parallel_for(p1 - p0, threads, [&](int k) {
        occlusion_pixel(G, pos, nrm, rough, p0 + k, *p, shadow, ao, ao_vis, spec, spec_t, recs);
    });
}

// LightAmbient.frag:141-175 from the world-space position already scaled to
// fine-voxel units (wcp of :150), the world normal, linear depth and the
// per-pixel blue-noise texel getNoise() (:49-52).
void vo_light_ambient(const uint8_t* g, int sx, int sy, int sz, const float* wcp_in, const float* nrm,
                      const float* depth, const float* noise, int npix, float* shadow, float* irradiance,
                      vo_rec* recs, int threads) {
    Grid G{g, sx, sy, sz};
    const V3 SUN_DIR = normalize(v3(0.3f, 0.4f, 0.5f));  // LightAmbient.frag:15
    parallel_for(npix, threads, [&](int i) {
        const float* nz = noise + 4 * (size_t)i;
        V3 normal = load3(nrm + 3 * (size_t)i);
        V3 wd = SUN_DIR;
        V3 wcp = load3(wcp_in + 3 * (size_t)i);
        V3 randomVec = mul(cosine_sample(nz[0], nz[1]), 0.1f);
        randomVec.z *= glsl_sign(nz[2] - 0.5f);
        wd = mix(wd, randomVec, 0.5f);
        wd = normalize(wd);
        wcp = add(wcp, mul(wd, nz[3] * 1.0f));
        wcp = add(wcp, mul(randomVec, 2.5f));
        float bias = smoothstep(0.0f, 0.2f, depth[i]) * 50.0f + 1.5f;
        V3 o = add(wcp, mul(normal, bias));
        vo_rec r0, r1;
        float t = march(G, o, wd, 128.0f, 0.5f, &r0);
        shadow[i] = (t != 128.0f) ? 0.0f : 1.0f;
        // calculateAmbientIrradiance, LightAmbient.frag:111-126
        V3 T, B;
        tangent_frame(normal, &T, &B);
        V3 rv = cosine_sample(nz[0], nz[1]);
        V3 dir = frame_dir(T, B, normal, rv);
        float dd = march(G, o, dir, 128.0f, 2.5f, &r1) / 128.0f;
        irradiance[i] = dd * dd * 0.05f;
        if (recs) {
            recs[2 * (size_t)i] = r0;
            recs[2 * (size_t)i + 1] = r1;
        }
    });
}

// LightReflection.frag:92-113: view_r is the world-space reflection vector
// (InverseView * vec4(R,0)).xyz before normalisation.
void vo_light_reflection(const uint8_t* g, int sx, int sy, int sz, const float* wcp_in, const float* nrm,
                         const float* view_r, const float* rough, const float* noise, int npix, float* t_out,
                         vo_rec* recs, int threads) {
    Grid G{g, sx, sy, sz};
    parallel_for(npix, threads, [&](int i) {
        const float* nz = noise + 4 * (size_t)i;
        V3 normal = load3(nrm + 3 * (size_t)i);
        V3 wd = normalize(load3(view_r + 3 * (size_t)i));
        V3 wcp = load3(wcp_in + 3 * (size_t)i);
        V3 randomVec = cosine_sample(nz[0], nz[1]);
        randomVec.z *= glsl_sign(nz[2] - 0.5f);
        wd = mix(wd, randomVec, rough[i] * 0.1f);
        wcp = add(wcp, mul(normal, nz[3]));
        wd = mul(wd, 1.0f + nz[3] * 0.5f);
        vo_rec r0;
        t_out[i] = march(G, add(wcp, normal), wd, 256.0f, 0.5f, &r0);
        if (recs) recs[i] = r0;
    });
}

// LightPoint.frag:234-267 (spot = 0) and LightSpot.frag:83-117 (spot = 1);
// wpos is the world position in world units. Pixels beyond the light's range
// are discarded by the shader: their output is left untouched.
void vo_light_point(const uint8_t* g, int sx, int sy, int sz, const float* wpos, const float* nrm, const float* noise,
                    int npix, const float* light_pos, float range, int spot, float* shadow, vo_rec* recs,
                    int threads) {
    Grid G{g, sx, sy, sz};
    V3 L = load3(light_pos);
    parallel_for(npix, threads, [&](int i) {
        const float* nz = noise + 4 * (size_t)i;
        V3 worldPos = load3(wpos + 3 * (size_t)i);
        V3 normal = load3(nrm + 3 * (size_t)i);
        V3 lightDir = sub(L, worldPos);
        float lightDistance = std::sqrt(dot(lightDir, lightDir));
        if (lightDistance > range) {
            if (recs) recs[i] = vo_rec{0, 0, 0, -1.0f, 0, 0};
            return;
        }
        V3 wd;
        float hitDist;
        if (spot) {
            wd = mul(normalize(lightDir), 10.0f);
            hitDist = lightDistance * 10.0f;
        } else {
            wd = lightDir;
            hitDist = lightDistance * 10.5f;
        }
        V3 wcp = mul(worldPos, 10.0f);
        V3 randomVec = mul(cosine_sample(nz[0], nz[1]), 0.1f);
        randomVec.z *= glsl_sign(nz[2] - 0.5f);
        wd = mix(wd, randomVec, 0.5f);
        wd = normalize(wd);
        wcp = add(wcp, mul(wd, nz[3] * 1.0f));
        wcp = add(wcp, mul(randomVec, 2.5f));
        vo_rec r0;
        float t = march(G, add(wcp, mul(normal, 0.5f)), wd, hitDist, spot ? 2.5f : 0.5f, &r0);
        shadow[i] = (t < hitDist) ? 0.0f : 1.0f;
        if (recs) recs[i] = r0;
    });
}

float vo_value_noise3(float x, float y, float z, uint32_t seed) { return value_noise3(x, y, z, seed); }
float vo_noise_octaves(float x, float y, float z, uint32_t seed, float freq, int octaves) {
    return noise_octaves(x, y, z, seed, freq, octaves);
}

// Seeded scene: fine voxel (x,y,z) is set where the 3-octave value noise at the
// voxel centre exceeds `thresh`, or where y < ground_y.
void vo_scene_noise(uint8_t* g, int sx, int sy, int sz, uint32_t seed, float thresh, float freq, int ground_y,
                    int threads) {
    const int nx = 2 * sx, ny = 2 * sy, nz = 2 * sz;
    std::memset(g, 0, (size_t)sx * sy * sz);
    // one task per byte-plane pair of z so that tasks write disjoint bytes
    parallel_for(sz, threads, [&](int bz) {
        for (int z = 2 * bz; z < 2 * bz + 2; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    bool on = y < ground_y;
                    if (!on) {
                        float v = noise_octaves((float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f, seed, freq, 3);
                        on = v > thresh;
                    }
                    if (on) set_fine(g, sx, sy, x, y, z);
                }
    });
}

// heightfield terrain (this library's synthetic scene; no reference counterpart):
// voxel (x, y, z) set where (float)y < base + amp * fbm(x + 0.5, 0.5, z + 0.5)
void vo_scene_terrain(uint8_t* g, int sx, int sy, int sz, uint32_t seed, float base, float amp, float freq,
                      int octaves, float* height, int threads) {
    const int nx = 2 * sx, ny = 2 * sy, nz = 2 * sz;
    std::vector<float> hv;
    if (!height) {
        hv.resize((size_t)nx * nz);
        height = hv.data();
    }
    parallel_for(nz, threads, [&](int z) {
        for (int x = 0; x < nx; x++) {
            const float v = noise_octaves((float)x + 0.5f, 0.5f, (float)z + 0.5f, seed, freq, octaves);
            const float m = amp * v;
            height[(size_t)z * nx + x] = base + m;
        }
    });
    // one task per byte-plane pair of z so that tasks write disjoint bytes
    parallel_for(sz, threads, [&](int bz) {
        for (int z = 2 * bz; z < 2 * bz + 2; z++)
            for (int x = 0; x < nx; x++) {
                const float h = height[(size_t)z * nx + x];
                for (int y = 0; y < ny && (float)y < h; y++) set_fine(g, sx, sy, x, y, z);
            }
    });
}

void vo_box_params(uint32_t seed, int i, int nx, int ny, int nz, int smin, int smax, int* out6) {
    uint32_t base = pcg(pcg(seed ^ 0x5bd1e995u) + (uint32_t)i);
    int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++) {
        uint32_t r1 = pcg(base + 2u * a), r2 = pcg(base + 2u * a + 1u);
        int s = smin + (int)(r1 % (uint32_t)(smax - smin + 1));
        if (s > n[a]) s = n[a];
        int p = (int)(r2 % (uint32_t)(n[a] - s + 1));
        out6[a] = p;
        out6[3 + a] = s;
    }
}

void vo_scene_boxes(uint8_t* g, int sx, int sy, int sz, uint32_t seed, int nboxes, int smin, int smax) {
    for (int i = 0; i < nboxes; i++) {
        int b[6];
        vo_box_params(seed, i, 2 * sx, 2 * sy, 2 * sz, smin, smax, b);
        for (int z = b[2]; z < b[2] + b[5]; z++)
            for (int y = b[1]; y < b[1] + b[4]; y++)
                for (int x = b[0]; x < b[0] + b[3]; x++) set_fine(g, sx, sy, x, y, z);
    }
}

// Primary visibility: pinhole camera at `cam` looking at `target` (up = +y),
// rays clipped to the grid box [0, 2*s) and walked with a plain entry-face DDA.
// pos = cam + dir * t_entry (fine-voxel units), nrm = entry face normal, sky
// pixels get pos = nrm = 0. rough = 0.05 + 0.95 * U(seed, pixel, 7777).
void vo_gbuffer(const uint8_t* g, int sx, int sy, int sz, const float* cam_in, const float* target,
                float tan_half_fov, int W, int H, uint32_t seed, float* pos, float* nrm, float* rough, int threads) {
    Grid G{g, sx, sy, sz};
    const int Nd[3] = {2 * sx, 2 * sy, 2 * sz};
    V3 cam = load3(cam_in);
    V3 fwd = normalize(sub(load3(target), cam));
    V3 right = normalize(cross(fwd, v3(0.0f, 1.0f, 0.0f)));
    V3 upv = cross(right, fwd);
    float aspect = (float)W / (float)H;
    parallel_for(W * H, threads, [&](int i) {
        int px = i % W, py = i / W;
        float u = (((float)px + 0.5f) * 2.0f / (float)W - 1.0f) * tan_half_fov * aspect;
        float v = (1.0f - ((float)py + 0.5f) * 2.0f / (float)H) * tan_half_fov;
        V3 d = normalize(add(add(fwd, mul(right, u)), mul(upv, v)));
        float dv[3] = {d.x, d.y, d.z}, cv[3] = {cam.x, cam.y, cam.z};
        for (int a = 0; a < 3; a++)
            if (dv[a] == 0.0f) dv[a] = 1e-20f;
        float inv[3], tn[3], tf[3];
        for (int a = 0; a < 3; a++) {
            inv[a] = 1.0f / dv[a];
            float t0 = (0.0f - cv[a]) * inv[a], t1 = ((float)Nd[a] - cv[a]) * inv[a];
            tn[a] = t0 < t1 ? t0 : t1;
            tf[a] = t0 < t1 ? t1 : t0;
        }
        int ax = 0;
        float tenter = tn[0];
        if (tn[1] > tenter) { tenter = tn[1]; ax = 1; }
        if (tn[2] > tenter) { tenter = tn[2]; ax = 2; }
        float texit = tf[0] < tf[1] ? tf[0] : tf[1];
        texit = texit < tf[2] ? texit : tf[2];
        float* po = pos + 3 * (size_t)i;
        float* no = nrm + 3 * (size_t)i;
        po[0] = po[1] = po[2] = 0.0f;
        no[0] = no[1] = no[2] = 0.0f;
        rough[i] = 0.05f + 0.95f * rand01(seed, (uint32_t)i, 7777u);
        if (tenter > texit || texit <= 0.0f) return;
        float tent = tenter > 0.0f ? tenter : 0.0f;
        int c[3], st[3];
        float tmax[3], tdel[3];
        for (int a = 0; a < 3; a++) {
            st[a] = dv[a] > 0.0f ? 1 : -1;
            if (a == ax && tenter > 0.0f) {
                c[a] = dv[a] > 0.0f ? 0 : Nd[a] - 1;
            } else {
                float pa = cv[a] + dv[a] * tent;
                int ci = (int)std::floor(pa);
                c[a] = ci < 0 ? 0 : (ci > Nd[a] - 1 ? Nd[a] - 1 : ci);
            }
            tmax[a] = ((float)(c[a] + (st[a] > 0 ? 1 : 0)) - cv[a]) * inv[a];
            tdel[a] = std::fabs(inv[a]);
        }
        int last = tenter > 0.0f ? ax : -1;
        for (int it = 0; it < Nd[0] + Nd[1] + Nd[2] + 3; it++) {
            if (G.volume_at(c[0], c[1], c[2], 0)) {
                if (last < 0) return;  // camera inside an occupied cell: no surface
                po[0] = cv[0] + dv[0] * tent;
                po[1] = cv[1] + dv[1] * tent;
                po[2] = cv[2] + dv[2] * tent;
                no[last] = (float)(-st[last]);
                return;
            }
            int a = (tmax[0] <= tmax[1] && tmax[0] <= tmax[2]) ? 0 : (tmax[1] <= tmax[2] ? 1 : 2);
            tent = tmax[a];
            c[a] += st[a];
            tmax[a] += tdel[a];
            last = a;
            if (c[a] < 0 || c[a] >= Nd[a]) return;
        }
    });
}

void vo_set_volume_at(uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int value) {
    set_volume_at(g, sx, sy, sz, x, y, z, value);
}
void vo_voxelize_model(uint8_t* g, int sx, int sy, int sz, const uint8_t* model, int msx, int msy, int msz,
                       const float* M, int value, int* aabb) {
    voxelize_model(g, sx, sy, sz, model, msx, msy, msz, M, value, aabb);
}
void vo_translate(const float* m, const float* v, float* out) { translate(m, v, out); }

// ShadowVoxSystem::OnUpdate, Sources/World/Systems/ShadowVoxSystem.cpp:116-191:
// entities in order; each clears its previous pose and sets its current pose
// (both with translate(-Pivot)); regions[6e..] = dirty byte region (x,y,z,w,h,d)
// or all -1 when the entity's aabbmax stayed at its start value.
void vo_shadowvox_update(uint8_t* g, int sx, int sy, int sz, int n, const uint8_t* const* models, const int* mdims,
                         const float* prev, const float* cur, const float* pivot, int* regions) {
    for (int e = 0; e < n; e++) {
        int aabb[6] = {sx - 1, sy - 1, sz - 1, 0, 0, 0};
        float np[3] = {-pivot[3 * e], -pivot[3 * e + 1], -pivot[3 * e + 2]};
        float M[16];
        translate(prev + 16 * (size_t)e, np, M);
        voxelize_model(g, sx, sy, sz, models[e], mdims[3 * e], mdims[3 * e + 1], mdims[3 * e + 2], M, 0, aabb);
        translate(cur + 16 * (size_t)e, np, M);
        voxelize_model(g, sx, sy, sz, models[e], mdims[3 * e], mdims[3 * e + 1], mdims[3 * e + 2], M, 1, aabb);
        if (regions) region_from_aabb(aabb, sx, sy, sz, regions + 6 * (size_t)e);
    }
}

// ShadowVoxSystem::OnVoxDestroyed, Sources/World/Systems/ShadowVoxSystem.cpp:7-53
// (uses WorldMatrix without the -Pivot translation, as the reference does).
void vo_vox_destroyed(uint8_t* g, int sx, int sy, int sz, const uint8_t* model, int msx, int msy, int msz,
                      const float* world, int* region) {
    int aabb[6] = {sx - 1, sy - 1, sz - 1, 0, 0, 0};
    voxelize_model(g, sx, sy, sz, model, msx, msy, msz, world, 0, aabb);
    if (region) region_from_aabb(aabb, sx, sy, sz, region);
}

// FNV-1a 64-bit over the bytes of s: the std::hash<std::string> of the MSVC
// toolchain the reference's .pf files were written with (Sources/Asset/Assets.h:207-210).
uint64_t vo_fnv1a64(const char* s) {
    uint64_t h = 14695981039346656037ull;
    for (const unsigned char* p = (const unsigned char*)s; *p; ++p) {
        h ^= (uint64_t)*p;
        h *= 1099511628211ull;
    }
    return h;
}

}  // extern "C"

// ===========================================================================
// Soft-opacity / albedo variant (this library's differentiable model; no
// reference counterpart). Every ray visits the cells the reference DDA
// (Light.frag:29-81) visits on an empty grid, up to maxt = len, and stops
// early once its transmittance falls below 2^-40. Opacity is clamped to
// [0, 1 - 2^-12]; the clamp's derivative is taken as 1 on the closed interval.
//   shadow ray:   T_sh = prod (1 - a_i)
//   AO ray k:     T_k  = prod (1 - a_i),  C_k = sum_i T_<i a_i rho_i  (rgb)
//   image:        I = rho_s * (k_sun T_sh + k_amb / K sum_k (T_k + C_k))
// rho_s is the albedo of the surface voxel floor(pos - 0.5 nrm). The adjoint
// uses prefix and suffix products (no division).
namespace {

const double kSoftAmax = 1.0 - 1.0 / 4096.0;
const double kSoftTmin = 1.0 / 1099511627776.0;  // 2^-40: a ray stops once its transmittance is below this

struct SoftRay {
    std::vector<int64_t> cells;  // voxel index, -1 for cells outside the data grid
};

void soft_pixel(const float* vox, int nx, int ny, int nz, const float* pos, const float* nrm, int i,
                const vo_soft_params& p, const float* grad_image, int64_t pv, double pdelta, double* image,
                double* gacc) {
    V3 P = load3(pos + 3 * (size_t)i), N = load3(nrm + 3 * (size_t)i);
    double* I = image + 3 * (size_t)i;
    I[0] = I[1] = I[2] = 0.0;
    if (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f) return;
    const int sxi = (int)std::floor(P.x - N.x * 0.5f), syi = (int)std::floor(P.y - N.y * 0.5f),
              szi = (int)std::floor(P.z - N.z * 0.5f);
    if (sxi < 0 || syi < 0 || szi < 0 || sxi >= nx || syi >= ny || szi >= nz) return;
    const int64_t s = (int64_t)sxi + (int64_t)syi * nx + (int64_t)szi * nx * ny;
    const double rs[3] = {vox[4 * s + 1], vox[4 * s + 2], vox[4 * s + 3]};
    auto alpha_raw = [&](int64_t v) { return (double)vox[4 * v] + (v == pv ? pdelta : 0.0); };
    auto alpha = [&](int64_t v) {
        double a = alpha_raw(v);
        return a < 0.0 ? 0.0 : (a > kSoftAmax ? kSoftAmax : a);
    };
    auto walk = [&](V3 o, V3 d, std::vector<int64_t>& cells) {
        cells.clear();
        dda_t(nx / 2, ny / 2, nz / 2, o, d, p.len, nullptr, [&](int x, int y, int z) {
            bool in = x >= 0 && y >= 0 && z >= 0 && x < nx && y < ny && z < nz;
            cells.push_back(in ? (int64_t)x + (int64_t)y * nx + (int64_t)z * nx * ny : -1);
            return false;
        });
    };
    V3 O = add(P, mul(N, p.bias));
    V3 T, B;
    tangent_frame(N, &T, &B);
    const int K = p.n_ao;
    std::vector<int64_t> cells;
    std::vector<double> pre, suf, sufc;
    // per ray: T and C (and the cells for the adjoint)
    double Tsh = 1.0, Tsum = 0.0, Csum[3] = {0, 0, 0};
    struct RayRes {
        std::vector<int64_t> cells;
        double T, C[3];
    };
    std::vector<RayRes> rays;
    auto trace = [&](V3 d) {
        RayRes rr;
        walk(O, d, rr.cells);
        double t = 1.0, c[3] = {0, 0, 0};
        for (size_t j = 0; j < rr.cells.size(); j++) {
            int64_t v = rr.cells[j];
            if (v < 0) continue;
            double a = alpha(v);
            for (int ch = 0; ch < 3; ch++) c[ch] += t * a * (double)vox[4 * v + 1 + ch];
            t *= 1.0 - a;
            if (t < kSoftTmin) {  // the walk ends here: later cells are not visited
                rr.cells.resize(j + 1);
                break;
            }
        }
        rr.T = t;
        for (int ch = 0; ch < 3; ch++) rr.C[ch] = c[ch];
        rays.push_back(rr);
    };
    if (p.n_shadow > 0) trace(load3(p.light_dir));
    for (int k = 0; k < K; k++) {
        float u1 = rand01(p.seed, (uint32_t)i, 64u + 2u * k);
        float u2 = rand01(p.seed, (uint32_t)i, 65u + 2u * k);
        trace(frame_dir(T, B, N, cosine_sample(u1, u2)));
    }
    int r0 = 0;
    if (p.n_shadow > 0) {
        Tsh = rays[0].T;
        r0 = 1;
    }
    for (int k = 0; k < K; k++) {
        Tsum += rays[r0 + k].T;
        for (int ch = 0; ch < 3; ch++) Csum[ch] += rays[r0 + k].C[ch];
    }
    const double ks = p.n_shadow > 0 ? (double)p.k_sun : 0.0;
    const double ka = K > 0 ? (double)p.k_amb / K : 0.0;
    double L[3];
    for (int ch = 0; ch < 3; ch++) {
        L[ch] = ks * Tsh + ka * (Tsum + Csum[ch]);
        I[ch] = rs[ch] * L[ch];
    }
    if (!grad_image || !gacc) return;
    const double gI[3] = {grad_image[3 * (size_t)i], grad_image[3 * (size_t)i + 1], grad_image[3 * (size_t)i + 2]};
    for (int ch = 0; ch < 3; ch++) gacc[4 * s + 1 + ch] += gI[ch] * L[ch];
    auto dclamp = [&](int64_t v) {
        double a = alpha_raw(v);
        return (a >= 0.0 && a <= kSoftAmax) ? 1.0 : 0.0;
    };
    for (size_t r = 0; r < rays.size(); r++) {
        const bool is_sh = p.n_shadow > 0 && r == 0;
        double w[3];
        for (int ch = 0; ch < 3; ch++) w[ch] = gI[ch] * rs[ch] * (is_sh ? ks : ka);
        const std::vector<int64_t>& cs = rays[r].cells;
        const size_t m = cs.size();
        pre.assign(m + 1, 1.0);
        for (size_t j = 0; j < m; j++) pre[j + 1] = pre[j] * (cs[j] < 0 ? 1.0 : 1.0 - alpha(cs[j]));
        suf.assign(m + 1, 1.0);     // suf[j] = prod_{l >= j} (1 - a_l)
        sufc.assign(3 * (m + 1), 0.0);  // sum_{l >= j} prod_{j <= q < l}(1 - a_q) a_l rho_l
        for (size_t j = m; j-- > 0;) {
            double a = cs[j] < 0 ? 0.0 : alpha(cs[j]);
            suf[j] = suf[j + 1] * (1.0 - a);
            for (int ch = 0; ch < 3; ch++) {
                double rho = cs[j] < 0 ? 0.0 : (double)vox[4 * cs[j] + 1 + ch];
                sufc[3 * j + ch] = a * rho + (1.0 - a) * sufc[3 * (j + 1) + ch];
            }
        }
        for (size_t j = 0; j < m; j++) {
            int64_t v = cs[j];
            if (v < 0) continue;
            double dT = -pre[j] * suf[j + 1];  // d T / d a_j
            double ga = 0.0;
            for (int ch = 0; ch < 3; ch++) {
                double dC = 0.0;
                if (!is_sh) {
                    double rho = (double)vox[4 * v + 1 + ch];
                    dC = pre[j] * rho - pre[j] * sufc[3 * (j + 1) + ch];
                    gacc[4 * v + 1 + ch] += w[ch] * pre[j] * alpha(v);
                }
                ga += w[ch] * (dT + dC);
            }
            gacc[4 * v] += ga * dclamp(v);
        }
    }
}

}  // namespace

extern "C" void vo_soft_render(const float* vox, int nx, int ny, int nz, const float* pos, const float* nrm, int npix,
                               const vo_soft_params* p, const float* grad_image, int64_t perturb_voxel,
                               double perturb_delta, double* image, double* grad_vox, int threads) {
    const size_t nv = (size_t)nx * ny * nz;
    if (!grad_image || !grad_vox) {
        parallel_for(npix, threads, [&](int i) {
            soft_pixel(vox, nx, ny, nz, pos, nrm, i, *p, nullptr, perturb_voxel, perturb_delta, image, nullptr);
        });
        return;
    }
    int T = threads < 1 ? 1 : (threads > 4 ? 4 : threads);
    std::vector<std::vector<double>> acc(T, std::vector<double>(4 * nv, 0.0));
    std::vector<std::thread> ts;
    for (int t = 0; t < T; t++)
        ts.emplace_back([&, t]() {
            for (int i = t; i < npix; i += T)
                soft_pixel(vox, nx, ny, nz, pos, nrm, i, *p, grad_image, perturb_voxel, perturb_delta, image,
                           acc[t].data());
        });
    for (auto& t : ts) t.join();
    for (size_t k = 0; k < 4 * nv; k++) {
        double s = 0.0;
        for (int t = 0; t < T; t++) s += acc[t][k];
        grad_vox[k] = s;
    }
}

// ===========================================================================
// Primary visibility: the G-buffer producer of GeometryVoxel.{vert,frag}.
namespace {

// VoxAsset::Upload, Sources/Asset/VoxAsset.cpp:3-63: a voxel of mip m+1 is the
// first non-zero of its children at mip m, probed in the order vi = 0..8
// (child (2x + (vi&1), 2y + (vi>>1&1), 2z + (vi>>2&1)); vi = 8 repeats vi = 0).
void mip_down(const uint8_t* parent, int psx, int psy, uint8_t* child, int csx, int csy, int csz) {
    for (int x = 0; x < csx; x++)
        for (int y = 0; y < csy; y++)
            for (int z = 0; z < csz; z++) {
                uint8_t vox = 0;
                for (int vi = 0; vi < 9; vi++) {
                    const uint8_t up = parent[(size_t)(2 * x + ((vi >> 0) & 1)) +
                                              (size_t)(2 * y + ((vi >> 1) & 1)) * psx +
                                              (size_t)(2 * z + ((vi >> 2) & 1)) * psx * psy];
                    if (up) {
                        vox = up;
                        break;
                    }
                }
                child[(size_t)x + (size_t)y * csx + (size_t)z * csx * csy] = vox;
            }
}
inline int mip_dim(int d) { return d > 1 ? d / 2 : 1; }

struct Volume {
    const uint8_t* m[3];
    int sx[3], sy[3], sz[3];
    // texelFetch(VOLUME_TEXTURE, p, mip).r with robust out-of-range = 0
    inline uint32_t texel(int mip, int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= sx[mip] || y >= sy[mip] || z >= sz[mip]) return 0u;
        return m[mip][(size_t)x + (size_t)y * sx[mip] + (size_t)z * sx[mip] * sy[mip]];
    }
};

// glm's scalar max / min: (x < y) ? y : x and (y < x) ? y : x
inline float gmax(float x, float y) { return (x < y) ? y : x; }
inline float gmin(float x, float y) { return (y < x) ? y : x; }

// clipToAABB, Sources/Shaders/GeometryVoxel.frag:50-61
V3 clip_to_aabb(V3 o, V3 d, V3 size) {
    const V3 c = v3(gmin(gmax(o.x, 0.0f), size.x), gmin(gmax(o.y, 0.0f), size.y), gmin(gmax(o.z, 0.0f), size.z));
    if (c.x == o.x && c.y == o.y && c.z == o.z) return o;
    const V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const V3 sgn = v3(glsl_step(d.x, 0.0f), glsl_step(d.y, 0.0f), glsl_step(d.z, 0.0f));
    const V3 t = mulv(sub(mulv(sgn, size), o), inv);
    const float tmin = gmax(gmax(t.x, t.y), t.z);
    return add(o, mul(d, tmin - 0.001f));
}

// intersectVolume, Sources/Shaders/GeometryVoxel.frag:63-125, with LOD 1,
// MIP_COUNT 2 and TRANSPARENCY 1. lcam = In.localCameraPos; (uvx, uvy) the
// fragment's UV, res = GetRes(), frame = GetFrame().
int intersect_volume(const Volume& V, V3 origin, V3 direction, V3 lcam, float uvx, float uvy, float resx, float resy,
                     int frame, V3* hit, V3* normal, uint32_t* material, int* fetches) {
    const V3 ss = v3(glsl_sign(direction.x), glsl_sign(direction.y), glsl_sign(direction.z));
    const V3 td = v3(1.0f / (direction.x * ss.x), 1.0f / (direction.y * ss.y), 1.0f / (direction.z * ss.z));
    int mip = 2;
    int i = 0;
    int nf = 0;
    do {
        const float mipSize = (float)(1 << mip);
        origin = v3(origin.x / mipSize, origin.y / mipSize, origin.z / mipSize);
        int cx = (int)std::floor(origin.x), cy = (int)std::floor(origin.y), cz = (int)std::floor(origin.z);
        const V3 nb = v3((float)cx + (ss.x * 0.5f + 0.5f), (float)cy + (ss.y * 0.5f + 0.5f),
                         (float)cz + (ss.z * 0.5f + 0.5f));
        V3 tm = v3((nb.x - origin.x) / direction.x, (nb.y - origin.y) / direction.y, (nb.z - origin.z) / direction.z);
        // clamp(current_voxel, ivec3(-1), ivec3(volumeDimension/mipSize)+1)
        const int ux = (int)((float)V.sx[0] / mipSize) + 1, uy = (int)((float)V.sy[0] / mipSize) + 1,
                  uz = (int)((float)V.sz[0] / mipSize) + 1;
        int n = 0;
        bool descended = false;
        do {
            const float selx = glsl_step(tm.x, tm.z) * glsl_step(tm.x, tm.y);
            const float sely = glsl_step(tm.y, tm.x) * glsl_step(tm.y, tm.z);
            const float selz = glsl_step(tm.z, tm.y) * glsl_step(tm.z, tm.x);
            cx += (int)(selx * ss.x);
            cy += (int)(sely * ss.y);
            cz += (int)(selz * ss.z);
            if (cx < -1 || cy < -1 || cz < -1 || cx > ux || cy > uy || cz > uz) {
                if (fetches) *fetches = nf;
                return 0;
            }
            const uint32_t voxel = V.texel(mip, cx, cy, cz);
            nf++;
            if (voxel != 0u) {
                float best_t = tm.x * selx + tm.y * sely;
                best_t = best_t + tm.z * selz;
                bool accept = mip == 0;
                if (!accept) {
                    const V3 p = mul(add(origin, mul(direction, best_t)), mipSize);
                    const V3 dd = sub(p, lcam);
                    accept = (float)mip < 0.001f * std::sqrt(dot(dd, dd));
                }
                if (accept) {
                    const float kx = std::round(uvx * resx * 0.5f), ky = std::round(uvy * resy * 0.5f);
                    const bool glass = voxel < 16u && glsl_mod(ky + kx, 2.0f) == (float)(frame % 2);
                    if (!glass) {
                        *normal = v3(-ss.x * selx, -ss.y * sely, -ss.z * selz);
                        *hit = mul(add(origin, mul(direction, best_t)), mipSize);
                        *material = voxel;
                        if (fetches) *fetches = nf;
                        return 1;
                    }
                } else {
                    mip--;
                    const V3 step = mul(direction, best_t);
                    origin = add(origin, v3(step.x / mipSize, step.y / mipSize, step.z / mipSize));
                    descended = true;
                    break;
                }
            }
            tm = v3(tm.x + td.x * selx, tm.y + td.y * sely, tm.z + td.z * selz);
        } while (++n < 512);
        (void)descended;
        origin = mul(origin, mipSize);
    } while (++i < 4);
    if (fetches) *fetches = nf;
    return 0;
}

// Inverse of the affine part of a column-major 4x4 (rows 0-2): R^-1 by the
// adjugate over the determinant, t' = -R^-1 t; fixed operation order (the
// CUDA path does the same operations).
void affine_inverse(const float* m, float* ri, float* ti) {
    const float a00 = m[0], a10 = m[1], a20 = m[2];
    const float a01 = m[4], a11 = m[5], a21 = m[6];
    const float a02 = m[8], a12 = m[9], a22 = m[10];
    const float c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
    const float c10 = a02 * a21 - a01 * a22, c11 = a00 * a22 - a02 * a20, c12 = a01 * a20 - a00 * a21;
    const float c20 = a01 * a12 - a02 * a11, c21 = a02 * a10 - a00 * a12, c22 = a00 * a11 - a01 * a10;
    float det = a00 * c00 + a01 * c01;
    det = det + a02 * c02;
    const float id = 1.0f / det;
    // ri row-major: ri[r*3 + c] = cofactor(c, r) / det
    ri[0] = c00 * id; ri[1] = c10 * id; ri[2] = c20 * id;
    ri[3] = c01 * id; ri[4] = c11 * id; ri[5] = c21 * id;
    ri[6] = c02 * id; ri[7] = c12 * id; ri[8] = c22 * id;
    for (int r = 0; r < 3; r++) {
        float v = ri[r * 3 + 0] * m[12] + ri[r * 3 + 1] * m[13];
        v = v + ri[r * 3 + 2] * m[14];
        ti[r] = -v;
    }
}
inline V3 rmul3(const float* r, V3 v) {  // row-major 3x3 times vector
    float x = r[0] * v.x + r[1] * v.y;
    float y = r[3] * v.x + r[4] * v.y;
    float z = r[6] * v.x + r[7] * v.y;
    return v3(x + r[2] * v.z, y + r[5] * v.z, z + r[8] * v.z);
}
inline V3 cmul3(const float* m, V3 v) {  // linear part of a column-major 4x4 times vector
    float x = m[0] * v.x + m[4] * v.y;
    float y = m[1] * v.x + m[5] * v.y;
    float z = m[2] * v.x + m[6] * v.y;
    return v3(x + m[8] * v.z, y + m[9] * v.z, z + m[10] * v.z);
}

}  // namespace

extern "C" {

void vo_volume_mips(const uint8_t* mip0, int sx, int sy, int sz, uint8_t* mip1, uint8_t* mip2) {
    const int x1 = mip_dim(sx), y1 = mip_dim(sy), z1 = mip_dim(sz);
    mip_down(mip0, sx, sy, mip1, x1, y1, z1);
    mip_down(mip1, x1, y1, mip2, mip_dim(x1), mip_dim(y1), mip_dim(z1));
}

int vo_clip_intersect(const uint8_t* mip0, const uint8_t* mip1, const uint8_t* mip2, int sx, int sy, int sz,
                      const float* origin, const float* dir, const float* lcam, float uvx, float uvy, float resx,
                      float resy, int frame, int clip, float* hit, float* normal, uint32_t* material, int* fetches) {
    Volume V;
    V.m[0] = mip0;
    V.m[1] = mip1;
    V.m[2] = mip2;
    V.sx[0] = sx; V.sy[0] = sy; V.sz[0] = sz;
    for (int k = 1; k < 3; k++) {
        V.sx[k] = mip_dim(V.sx[k - 1]);
        V.sy[k] = mip_dim(V.sy[k - 1]);
        V.sz[k] = mip_dim(V.sz[k - 1]);
    }
    V3 o = load3(origin), d = load3(dir);
    if (clip) o = clip_to_aabb(o, d, v3((float)sx, (float)sy, (float)sz));
    V3 h = v3(0, 0, 0), nrm = v3(0, 0, 0);
    uint32_t mat = 0;
    const int r = intersect_volume(V, o, d, load3(lcam), uvx, uvy, resx, resy, frame, &h, &nrm, &mat, fetches);
    hit[0] = h.x; hit[1] = h.y; hit[2] = h.z;
    normal[0] = nrm.x; normal[1] = nrm.y; normal[2] = nrm.z;
    *material = mat;
    return r;
}

void vo_affine_inverse(const float* m, float* ri, float* ti) { affine_inverse(m, ri, ti); }

// Per-pixel primary visibility over instances (GeometryVoxelPipeline::Use,
// GeometryVoxelPipeline.h:50-70, resolved by depth): the pixel ray of the
// vxl_scene_gbuffer camera, in world units, is moved into each instance's
// volume space (local = R^-1 (p - t) * 10, direction R^-1 d normalized),
// tested against the volume box [0, dims] and, where it enters, clipped
// (clipToAABB) and traced (intersectVolume); the nearest hit by view depth
// wins, ties to the lower instance index.
void vo_primary(const uint8_t* const* mip0s, const uint8_t* const* mip1s, const uint8_t* const* mip2s,
                const int* vdims, const float* worlds, const int* vol_of, int ninst, const float* cam_in,
                const float* target, float tan_half_fov, int W, int H, int frame, float* pos, float* nrm,
                float* depth, int32_t* material, int32_t* instance, int threads) {
    const V3 cam = load3(cam_in);
    const V3 fwd = normalize(sub(load3(target), cam));
    const V3 right = normalize(cross(fwd, v3(0.0f, 1.0f, 0.0f)));
    const V3 upv = cross(right, fwd);
    const float aspect = (float)W / (float)H;
    std::vector<float> rinv((size_t)ninst * 9), tinv((size_t)ninst * 3);
    for (int k = 0; k < ninst; k++) affine_inverse(worlds + 16 * (size_t)k, &rinv[9 * (size_t)k], &tinv[3 * (size_t)k]);
    parallel_for(W * H, threads, [&](int i) {
        const int px = i % W, py = i / W;
        const float uvx = ((float)px + 0.5f) * 2.0f / (float)W - 1.0f;
        const float uvy = ((float)py + 0.5f) * 2.0f / (float)H - 1.0f;
        const float u = uvx * tan_half_fov * aspect;
        const float v = (1.0f - ((float)py + 0.5f) * 2.0f / (float)H) * tan_half_fov;
        const V3 d = normalize(add(add(fwd, mul(right, u)), mul(upv, v)));
        float best = 0.0f;
        int bi = -1;
        V3 bp = v3(0, 0, 0), bn = v3(0, 0, 0);
        uint32_t bm = 0;
        for (int k = 0; k < ninst; k++) {
            const float* M = worlds + 16 * (size_t)k;
            const float* ri = &rinv[9 * (size_t)k];
            const float* ti = &tinv[3 * (size_t)k];
            const int vi = vol_of[k];
            const int sx = vdims[3 * vi], sy = vdims[3 * vi + 1], sz = vdims[3 * vi + 2];
            V3 lc = rmul3(ri, cam);
            lc = mul(add(lc, v3(ti[0], ti[1], ti[2])), 10.0f);
            const V3 ld = normalize(rmul3(ri, d));
            // the pixel's ray enters the volume box (what rasterizing its cube covers)
            const float dims[3] = {(float)sx, (float)sy, (float)sz};
            const float lo[3] = {lc.x, lc.y, lc.z}, dl[3] = {ld.x, ld.y, ld.z};
            float t0 = -INFINITY, t1 = INFINITY;
            for (int a = 0; a < 3; a++) {
                const float inv = 1.0f / dl[a];
                const float ta = (0.0f - lo[a]) * inv, tb = (dims[a] - lo[a]) * inv;
                t0 = std::fmax(t0, std::fmin(ta, tb));
                t1 = std::fmin(t1, std::fmax(ta, tb));
            }
            if (!(t0 <= t1 && t1 >= 0.0f)) continue;
            Volume V;
            V.m[0] = mip0s[vi];
            V.m[1] = mip1s[vi];
            V.m[2] = mip2s[vi];
            V.sx[0] = sx; V.sy[0] = sy; V.sz[0] = sz;
            for (int q = 1; q < 3; q++) {
                V.sx[q] = mip_dim(V.sx[q - 1]);
                V.sy[q] = mip_dim(V.sy[q - 1]);
                V.sz[q] = mip_dim(V.sz[q - 1]);
            }
            const V3 o = clip_to_aabb(lc, ld, v3(dims[0], dims[1], dims[2]));
            V3 h, nn;
            uint32_t mat;
            if (!intersect_volume(V, o, ld, lc, uvx, uvy, (float)W, (float)H, frame, &h, &nn, &mat, nullptr)) continue;
            // world position (world units) of the hit, its view depth
            const V3 wl = cmul3(M, mul(h, 0.1f));
            const V3 wp = v3(wl.x + M[12], wl.y + M[13], wl.z + M[14]);
            const float dep = dot(sub(wp, cam), fwd);
            if (bi < 0 || dep < best) {
                best = dep;
                bi = k;
                bp = wp;
                bn = normalize(cmul3(M, nn));
                bm = mat;
            }
        }
        float* po = pos + 3 * (size_t)i;
        float* no = nrm + 3 * (size_t)i;
        if (bi >= 0) {
            po[0] = bp.x * 10.0f; po[1] = bp.y * 10.0f; po[2] = bp.z * 10.0f;
            no[0] = bn.x; no[1] = bn.y; no[2] = bn.z;
            depth[i] = best;
        } else {
            po[0] = po[1] = po[2] = 0.0f;
            no[0] = no[1] = no[2] = 0.0f;
            depth[i] = 0.0f;
        }
        material[i] = (int32_t)bm;
        instance[i] = bi;
    });
}

}  // extern "C"

// ===========================================================================
// Temporal accumulation: LightTAA.frag:37-141 (main), luminance :30-35.
// Images are fp32 arrays, x fastest; texture() is this library's sampler:
// bilinear, clamp to edge, texel centres at (i + 0.5) / size:
//   x = u * W - 0.5, i0 = floor(x), a = x - i0 (same for y), taps clamped,
//   v = (t00 (1-a) + t10 a)(1-b) + (t01 (1-a) + t11 a) b.
// sin/cos are this library's own (sincos_own).
namespace {

struct Img {
    const float* p;
    int c;  // channels
};
struct TaaImgs {
    Img light, last, color, normal, material, depth, motion;
    int W, H;
};

void tex(const Img& im, int W, int H, float u, float v, float* out) {
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
    const float bx = 1.0f - ax, by = 1.0f - ay;
    for (int k = 0; k < im.c; k++) {
        const float t00 = im.p[((size_t)y0 * W + x0) * im.c + k], t10 = im.p[((size_t)y0 * W + x1) * im.c + k];
        const float t01 = im.p[((size_t)y1 * W + x0) * im.c + k], t11 = im.p[((size_t)y1 * W + x1) * im.c + k];
        const float top = t00 * bx + t10 * ax;
        const float bot = t01 * bx + t11 * ax;
        out[k] = top * by + bot * ay;
    }
    for (int k = im.c; k < 4; k++) out[k] = 0.0f;
}
inline float len2(float x, float y) { return std::sqrt(x * x + y * y); }
inline float len3(const float* a, const float* b) {
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float d = dx * dx + dy * dy;
    d = d + dz * dz;
    return std::sqrt(d);
}
inline float len4(const float* a, const float* b) {
    const float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2], d3 = a[3] - b[3];
    float d = d0 * d0 + d1 * d1;
    d = d + d2 * d2;
    d = d + d3 * d3;
    return std::sqrt(d);
}
inline float dot3(const float* a, const float* b) {
    float d = a[0] * b[0] + a[1] * b[1];
    return d + a[2] * b[2];
}
inline float clampf(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

void taa_pixel(const TaaImgs& I, const float* noise, int px, int py, float* out) {
    const int W = I.W, H = I.H;
    const float FAR = 4096.0f;
    const float GR = 2.118033988749895f;
    const float iResx = 1.0f / (float)W, iResy = 1.0f / (float)H;
    const float uvx = ((float)px + 0.5f) / (float)W, uvy = ((float)py + 0.5f) / (float)H;
    float motion[4], cl[4], cc[4], cm[4], cn[4], cd[4], ll[4];
    tex(I.motion, W, H, uvx, uvy, motion);
    const float oux = uvx + motion[0], ouy = uvy + motion[1];
    tex(I.light, W, H, uvx, uvy, cl);
    tex(I.color, W, H, uvx, uvy, cc);
    tex(I.material, W, H, uvx, uvy, cm);
    tex(I.normal, W, H, uvx, uvy, cn);
    tex(I.depth, W, H, uvx, uvy, cd);
    const float depth = cd[0];
    if (depth == 1.0f) {
        for (int k = 0; k < 4; k++) out[k] = cl[k];
        return;
    }
    tex(I.last, W, H, oux, ouy, ll);
    float lastVariance = ll[3];
    if (clampf(oux, 0.0f, 1.0f) != oux || clampf(ouy, 0.0f, 1.0f) != ouy) {
        float count = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (int x = -9; x <= 9; ++x)
            for (int y = -9; y <= 9; ++y) {
                const float ox = (float)x * iResx, oy = (float)y * iResy;
                const float u = clampf(uvx + ox, 0.001f, 0.999f), v = clampf(uvy + oy, 0.001f, 0.999f);
                float nmo[4], nco[4], nno[4], nma[4], nde[4], nli[4];
                tex(I.motion, W, H, u, v, nmo);
                tex(I.color, W, H, u, v, nco);
                tex(I.normal, W, H, u, v, nno);
                tex(I.material, W, H, u, v, nma);
                tex(I.depth, W, H, u, v, nde);
                float factor = gmax(dot3(cn, nno), 0.0f);
                factor *= glsl_step(0.8f, 1.0f - len4(cm, nma));
                factor *= 1.0f - clampf(std::fabs(depth - nde[0]) * FAR, 0.0f, 1.0f);
                factor *= 1.0f - clampf(len3(cc, nco), 0.0f, 1.0f);
                if (len2(motion[0] - nmo[0], motion[1] - nmo[1]) > 0.1f) factor = 0.0f;
                tex(I.light, W, H, u, v, nli);
                s0 += factor * nli[0];
                s1 += factor * nli[1];
                s2 += factor * nli[2];
                count += factor;
            }
        out[0] = s0 / count;
        out[1] = s1 / count;
        out[2] = s2 / count;
        out[3] = 1.0f;
        return;
    }
    float nmin[3] = {10000.0f, 10000.0f, 10000.0f}, nmax[3] = {0.0f, 0.0f, 0.0f};
    float ncol[3] = {0.0f, 0.0f, 0.0f};
    float diffSum = 1.0f, count = 0.0f;
    const float size = 12.0f;
    float radius = 1.0f;
    const float dscale = gmin(gmax(0.1f, 0.5f), 1.0f / depth);  // clamp(0.1, 0.5, 1.0/currentDepth)
    for (float angle = noise[0] * 3.1415f * GR; radius <= size; angle += 2.39f) {
        radius += 1.0f;
        float sn, cs;
        sincos_own(angle, &sn, &cs);
        const float rv = radius * (lastVariance + 1.0f);
        const float ox = cs * iResx * rv * dscale, oy = sn * iResy * rv * dscale;
        const float u = clampf(uvx + ox, 0.001f, 0.999f), v = clampf(uvy + oy, 0.001f, 0.999f);
        float nmo[4], nco[4], nno[4], nma[4], nde[4], nli[4];
        tex(I.motion, W, H, u, v, nmo);
        tex(I.color, W, H, u, v, nco);
        tex(I.normal, W, H, u, v, nno);
        tex(I.material, W, H, u, v, nma);
        tex(I.depth, W, H, u, v, nde);
        float factor = 1.212f - radius / size;
        factor *= glsl_step(0.8f, 1.0f - len4(cm, nma));
        factor *= gmax(dot3(cn, nno), 0.0f);
        factor *= 1.0f - clampf(std::fabs(depth - nde[0]) * FAR, 0.0f, 1.0f);
        factor *= 1.0f - clampf(len3(cc, nco) * 10000.0f, 0.0f, 1.0f);
        if (len2(motion[0] - nmo[0], motion[1] - nmo[1]) > 0.1f) factor = 0.0f;
        tex(I.light, W, H, u, v, nli);
        for (int k = 0; k < 3; k++) {
            nmin[k] = gmin(nmin[k], nli[k]);
            nmax[k] = gmax(nmax[k], nli[k]);
            ncol[k] += factor * nli[k];
        }
        count += factor;
        diffSum += len3(nli, cl) * factor;
    }
    for (int k = 0; k < 3; k++) {
        cl[k] += ncol[k];
        cl[k] /= count + 1.0f;
    }
    diffSum /= radius;
    for (int k = 0; k < 3; k++) ll[k] = gmin(gmax(ll[k], nmin[k]), nmax[k]);
    const float a0 = std::fabs(cl[0] - ll[0]), a1 = std::fabs(cl[1] - ll[1]), a2 = std::fabs(cl[2] - ll[2]);
    float lum = a0 * 0.2125f + a1 * 0.7154f;
    lum = lum + a2 * 0.0721f;
    const float variance = clampf(lum * 5.5f, 0.0f, 1.0f);
    lastVariance += variance;
    lastVariance -= diffSum * 0.08f;
    lastVariance += len2(motion[0], motion[1]) * 20.0f;
    const float t = clampf(1.0f - lastVariance, 0.3f, 0.9f);
    const float omt = 1.0f - t;
    for (int k = 0; k < 3; k++) out[k] = cl[k] * omt + ll[k] * t;
    out[3] = clampf(lastVariance * 0.7f, 0.0f, 1.0f);
}

}  // namespace

extern "C" void vo_taa(const float* light, const float* last, const float* color, const float* normal,
                       const float* material, const float* depth, const float* motion, const float* noise, int W,
                       int H, float* out, int threads) {
    TaaImgs I{{light, 4}, {last, 4}, {color, 3}, {normal, 3}, {material, 4}, {depth, 1}, {motion, 2}, W, H};
    parallel_for(W * H, threads, [&](int i) {
        taa_pixel(I, noise + 4 * (size_t)i, i % W, i / W, out + 4 * (size_t)i);
    });
}

// ------------------------------------------------------------ depth -> position
// LightAmbient.vert:32-36: FarVec = (InverseProjection * (Pos.xy, 1, 1)).xyz / w at
// the full-screen pass's vertices, interpolated; it is linear in Pos.xy (a
// perspective inverse has a constant w at z = 1), so it is evaluated here at
// the fragment's NDC. The pass samples the G-buffer at UV = (Pos.xy*0.5+0.5)
// with UV.y flipped (:40-41), so texel (i, j) -- row j from the start of the
// image -- is read by the fragment at NDC ((i+0.5)*2/W - 1, 1 - (j+0.5)*2/H).
// LightAmbient.frag:141: pos = FarVec * (depth * (1 + 1/FAR)), FAR = 4096;
// :150: wcp = (InverseView * (pos, 1)).xyz * 10. Sky: !(depth < 0.999) (:138).
// Matrix-vector products add the column terms in column order, fp32, no FMA.
static void mat4_vec(const float* m, float x, float y, float z, float w, float* o) {
    for (int r = 0; r < 4; r++) {
        float a = m[r] * x;
        a = a + m[4 + r] * y;
        a = a + m[8 + r] * z;
        a = a + m[12 + r] * w;
        o[r] = a;
    }
}

void vo_rebuild_from_depth(const float* depth, const float* nrm, int W, int H, const float* inv_view,
                           const float* inv_proj, float* wcp, float* nrm_out) {
    const float kFarScale = 1.0f + 1.0f / 4096.0f;
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            const size_t k = (size_t)j * W + i;
            const float d = depth[k];
            float* p = wcp + 3 * k;
            float* n = nrm_out + 3 * k;
            if (!(d < 0.999f)) {
                p[0] = p[1] = p[2] = 0.0f;
                n[0] = n[1] = n[2] = 0.0f;
                continue;
            }
            const float nx = ((float)i + 0.5f) * 2.0f / (float)W - 1.0f;
            const float ny = 1.0f - ((float)j + 0.5f) * 2.0f / (float)H;
            float v[4], q[4];
            mat4_vec(inv_proj, nx, ny, 1.0f, 1.0f, v);
            const float s = d * kFarScale;
            const float px = (v[0] / v[3]) * s, py = (v[1] / v[3]) * s, pz = (v[2] / v[3]) * s;
            mat4_vec(inv_view, px, py, pz, 1.0f, q);
            p[0] = q[0] * 10.0f;
            p[1] = q[1] * 10.0f;
            p[2] = q[2] * 10.0f;
            n[0] = nrm[3 * k];
            n[1] = nrm[3 * k + 1];
            n[2] = nrm[3 * k + 2];
        }
}

// ---------------------------------------------------------------------------
// RayVoxCast, Sources/World/Systems/PhysicsSystem.cpp:98-145: the engine's own
// CPU DDA, used for picking one placed model. It is a second meaning of
// "voxel DDA", next to raycastShadowVolume:
// * it steps before it tests, so the origin cell is never tested;
// * it leaves at the first cell outside [0, size-1];
// * it runs at most 257 iterations (`do ... while (i++ < 256)`);
// * it nudges zero direction components to 1e-8;
// * a hit reports the entry time of the hit cell, dot(tMax, select) * 0.1.
// Host C++ compiled against glm, so the arithmetic order is glm's: mat4 * vec4
// adds the column terms pairwise, (c0*x + c1*y) + (c2*z + c3*w), and dot adds
// left to right. inv_obb is glm::inverse(obb), column-major, supplied by the
// caller (the cofactor inverse is not restated here). The model is 1 byte per
// voxel, x fastest (VoxAsset::PixelAt, Sources/Asset/VoxAsset.h:52-56), and
// obbSize is the model size.
static void glm_mat4_vec(const float* m, float x, float y, float z, float w, float* o) {
    for (int r = 0; r < 4; r++) {
        const float a0 = m[r] * x + m[4 + r] * y;
        const float a1 = m[8 + r] * z + m[12 + r] * w;
        o[r] = a0 + a1;
    }
}

int vo_ray_vox_cast(const uint8_t* model, int msx, int msy, int msz, const float* inv_obb, const float* ray_pos,
                    const float* ray_dir, float* t_out, int* cell_out, int* iters_out) {
    float lp[4], ld[4], m[16];
    glm_mat4_vec(inv_obb, ray_pos[0], ray_pos[1], ray_pos[2], 1.0f, lp);
    const V3 localPos = v3(lp[0] * 10.0f, lp[1] * 10.0f, lp[2] * 10.0f);
    std::memcpy(m, inv_obb, sizeof(m));
    m[12] = 0.0f;  // invObb[3] = vec4(0, 0, 0, 1)
    m[13] = 0.0f;
    m[14] = 0.0f;
    m[15] = 1.0f;
    glm_mat4_vec(m, ray_dir[0], ray_dir[1], ray_dir[2], 0.0f, ld);
    V3 localDir = v3(ld[0], ld[1], ld[2]);
    if (localDir.x == 0.0f) localDir.x = 0.00000001f;
    if (localDir.y == 0.0f) localDir.y = 0.00000001f;
    if (localDir.z == 0.0f) localDir.z = 0.00000001f;
    const V3 stepSign = v3(glsl_sign(localDir.x), glsl_sign(localDir.y), glsl_sign(localDir.z));
    const V3 tDelta = v3(1.0f / (localDir.x * stepSign.x), 1.0f / (localDir.y * stepSign.y),
                         1.0f / (localDir.z * stepSign.z));
    int cx = (int)std::floor(localPos.x), cy = (int)std::floor(localPos.y), cz = (int)std::floor(localPos.z);
    const V3 nb = v3((float)cx + (stepSign.x * 0.5f + 0.5f), (float)cy + (stepSign.y * 0.5f + 0.5f),
                     (float)cz + (stepSign.z * 0.5f + 0.5f));
    V3 tMax = v3((nb.x - localPos.x) / localDir.x, (nb.y - localPos.y) / localDir.y,
                 (nb.z - localPos.z) / localDir.z);
    int i = 0;
    do {
        // step(tMax, tMax.zxy) * step(tMax, tMax.yzx)
        const float sx = glsl_step(tMax.x, tMax.z) * glsl_step(tMax.x, tMax.y);
        const float sy = glsl_step(tMax.y, tMax.x) * glsl_step(tMax.y, tMax.z);
        const float sz = glsl_step(tMax.z, tMax.y) * glsl_step(tMax.z, tMax.x);
        cx += (int)(sx * stepSign.x);
        cy += (int)(sy * stepSign.y);
        cz += (int)(sz * stepSign.z);
        if (iters_out) *iters_out = i + 1;
        if (cell_out) {
            cell_out[0] = cx;
            cell_out[1] = cy;
            cell_out[2] = cz;
        }
        if (cx < 0 || cy < 0 || cz < 0 || cx > msx - 1 || cy > msy - 1 || cz > msz - 1) return 0;
        const uint8_t voxel = model[(size_t)cx + (size_t)cy * msx + (size_t)cz * msx * msy];
        if (voxel != 0) {
            float d = tMax.x * sx + tMax.y * sy;
            d = d + tMax.z * sz;
            if (t_out) *t_out = d * 0.1f;
            return 1;
        }
        tMax.x += tDelta.x * sx;
        tMax.y += tDelta.y * sy;
        tMax.z += tDelta.z * sz;
    } while (i++ < 256);
    return 0;
}
