// occl_common.cuh — pieces shared by the warp-pooled occlusion kernels
// (occlusion.cu: exact stepping on the grid's words, with per-ray records;
// occl_lean.cu: stepping on the trace layout): the scene descriptor, the
// pool's ray slots and the ray generator.
#pragma once
#include "vxl_device.cuh"

namespace vxl {

struct TraceConstsP {
    f3 light;
    f3 cam;
    float bias, shadow_len, ao_len, spec_len, default_rough;
    int n_shadow, n_ao, n_spec, R;
    int spec_first;  // dispatch order: spec, shadow, AO (else shadow, AO, spec)
    uint32_t seed_h;
};

// The two-level map of empty space (vxl_grid clear1/clear2): level 1, one bit
// per 8^3 tile, set when the tile or a neighbour has a voxel; level 2, one bit
// per 64^3 cells (8^3 tiles), set when a level-1 bit in it is. NULL c1: none.
struct ClearMaps {
    const uint32_t* c1;
    const uint32_t* c2;
    int tx, ty, tz;  // tiles per axis
    int sx, sy;      // 64^3 regions per x row and per y column
};

// One scene of a launch: grid, G-buffer, outputs, tiling, ray parameters.
struct SceneDesc {
    GridView g;
    ClearMaps cm;
    const float* pos;
    const float* nrm;
    const float* rough;
    float* o_shadow;
    float* o_ao;
    float* o_vis;
    float* o_spec;
    float* o_spec_t;
    vxl_ray_record* rec;
    int64_t npix;
    int64_t tile_begin;  // first global tile of this scene (batched launches)
    int64_t ntiles;
    int width, height;   // image size, for block tiles
    int tile_w;          // pixels per tile row; TP = runs of TP pixels
    uint32_t pix_base;   // added to the pixel index that seeds the ray generator (a chunk of a larger frame)
    TraceConstsP c;
};

struct __align__(16) PSlot {
    int c01;     // cx (low 16 bits, signed) | cy << 16
    int c2m;     // cz (low 16 bits, signed) | meta << 16
    float a0, a1, a2;  // t_max (literal rays: origin)
    float b0, b1, b2;  // t_delta (literal rays: direction)
};
// meta: bit 0-2 negative step on x,y,z; bit 3 literal ray; bits 4-8 pixel in tile; bits 9-13 ray index k;
// bit 14 empty bricks may be leapt (leap_allowed and no per-ray records requested)
constexpr int kMetaLit = 1 << 3;
constexpr int kMetaLeap = 1 << 14;
constexpr int kPoolMaxR = 31;

// shared memory of one warp's pool: slots, result t per ray, hit mask per ray index
__host__ __device__ __forceinline__ size_t pool_bytes(int TP, int R) {
    size_t b = (size_t)TP * R * (sizeof(PSlot) + sizeof(float)) + (size_t)R * sizeof(uint32_t);
    return (b + 15) & ~(size_t)15;
}

__device__ __forceinline__ int lo16(int v) { return (v << 16) >> 16; }
__device__ __forceinline__ int hi16(int v) { return v >> 16; }

__device__ __forceinline__ float kind_maxt(const TraceConstsP& c, int k) {
    return k < c.n_shadow ? c.shadow_len : (k < c.n_shadow + c.n_ao ? c.ao_len : c.spec_len);
}

// ray k of a pixel (same generator as k_occlusion / the oracle's occlusion_pixel)
// hpix = pcg(seed_h + pixel): the per-pixel half of rand01, hoisted by callers
__device__ __forceinline__ f3 gen_dir(const TraceConstsP& c, int k, uint32_t hpix, f3 P, f3 N, f3 T, f3 B,
                                      float rough) {
    if (k < c.n_shadow) return c.light;
    if (k < c.n_shadow + c.n_ao) {
        uint32_t j = (uint32_t)(k - c.n_shadow);
        float u1 = u01(pcg(hpix + 64u + 2u * j));
        float u2 = u01(pcg(hpix + 65u + 2u * j));
        return frame_dir(T, B, N, cosine_sample(u1, u2));
    }
    uint32_t j = (uint32_t)(k - c.n_shadow - c.n_ao);
    float a = rough * rough;
    float a2 = a * a;
    f3 V = normalize(sub(c.cam, P));
    float u1 = u01(pcg(hpix + 2u * j));
    float u2 = u01(pcg(hpix + 2u * j + 1u));
    float ct = sqrtf((1.0f - u1) / (1.0f + (a2 - 1.0f) * u1));
    float st2 = 1.0f - ct * ct;
    float sn = sqrtf(st2 > 0.0f ? st2 : 0.0f);
    float s, cs;
    sincos_own(6.2831855f * u2, &s, &cs);
    f3 H = frame_dir(T, B, N, mk(sn * cs, sn * s, ct));
    float vh = dot(V, H);
    return normalize(sub(mul(H, 2.0f * vh), V));
}

// lanes below this one (read at each use rather than kept in a register)
__device__ __forceinline__ unsigned lanes_below() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// pixel index of position p of a scene-local tile; false outside the image
template <int TP>
__device__ __forceinline__ bool tile_pixel(const SceneDesc& S, int64_t tile, int p, int64_t* gpix) {
    if (S.tile_w >= TP || S.width <= 0) {
        *gpix = tile * TP + p;
        return *gpix < S.npix;
    }
    const int tw = S.tile_w, th = TP / tw;
    const int64_t tpr = (S.width + tw - 1) / tw;
    const int64_t ty = tile / tpr, tx = tile - ty * tpr;
    const int64_t x = tx * tw + p % tw, y = ty * th + p / tw;
    *gpix = y * S.width + x;
    return x < S.width && y < S.height;
}

__device__ __forceinline__ bool map_bit(const uint32_t* m, int x, int y, int z, int nx, int ny) {
    const uint32_t i = (uint32_t)x + (uint32_t)y * (uint32_t)nx + (uint32_t)z * (uint32_t)nx * (uint32_t)ny;
    return (__ldg(m + (i >> 5)) >> (i & 31)) & 1u;
}

// Whether no cell that the DDA state s can still test before its ray ends
// holds a voxel, proved on the two-level map: the ray is then a miss, whatever
// ends it (maxt, the bounds or the 256-iteration cap), and needs no more
// steps. The line is x(T) = fx + sx |d_x| (T - tx) (fx the face crossed at
// the next x crossing, time tx), and likewise for y and z. From the tile of
// the current cell, a march steps over clear regions: a whole 64^3 region
// when its level-2 bit is clear, else an 8^3 tile when its level-1 bit is,
// else the proof fails. The march covers the line up to time maxt plus two
// cells (every cell the DDA tests is entered before totalt reaches maxt) or
// until it leaves the grid's tiles (the DDA would stop at the bounds there).
// The DDA tests cells the line passes through, and the march's regions are
// placed from float positions accurate to far less than a tile: the
// one-tile dilation of level 1 covers both.
static __device__ __noinline__ bool path_clear(const ClearMaps& M, const DState& s) {
    const float fx = (float)(s.cx + (s.sx > 0 ? 1 : 0)), fy = (float)(s.cy + (s.sy > 0 ? 1 : 0)),
                fz = (float)(s.cz + (s.sz > 0 ? 1 : 0));
    const float vx = (float)s.sx * __frcp_rn(s.tdx), vy = (float)s.sy * __frcp_rn(s.tdy),
                vz = (float)s.sz * __frcp_rn(s.tdz);  // the direction
    const float tend = s.maxt + 2.0f * fmaxf(fmaxf(s.tdx, s.tdy), s.tdz);
    int qx = s.cx >> 3, qy = s.cy >> 3, qz = s.cz >> 3;
    for (int it = 0; it < 64; it++) {
        if ((unsigned)qx >= (unsigned)M.tx || (unsigned)qy >= (unsigned)M.ty || (unsigned)qz >= (unsigned)M.tz)
            return true;
        int L, x0, y0, z0;  // the clear region: edge in cells and low corner
        if (!map_bit(M.c2, qx >> 3, qy >> 3, qz >> 3, M.sx, M.sy)) {
            L = 64;
            x0 = (qx >> 3) * 64;
            y0 = (qy >> 3) * 64;
            z0 = (qz >> 3) * 64;
        } else if (!map_bit(M.c1, qx, qy, qz, M.tx, M.ty)) {
            L = 8;
            x0 = qx * 8;
            y0 = qy * 8;
            z0 = qz * 8;
        } else {
            return false;
        }
        // the times at which the line leaves the region through each far face
        const float ex = (float)(x0 + (s.sx > 0 ? L : 0)), ey = (float)(y0 + (s.sy > 0 ? L : 0)),
                    ez = (float)(z0 + (s.sz > 0 ? L : 0));
        const float Tx = s.tx + (ex - fx) * (float)s.sx * s.tdx;
        const float Ty = s.ty + (ey - fy) * (float)s.sy * s.tdy;
        const float Tz = s.tz + (ez - fz) * (float)s.sz * s.tdz;
        const float T = fminf(fminf(Tx, Ty), Tz);
        if (!(T == T)) return false;
        if (T >= tend) return true;
        // the tile the line enters at T: out of the region along the exit
        // axes, where the line is along the others
        qx = (T == Tx ? (s.sx > 0 ? x0 + L : x0 - 1) : __float2int_rd(fx + vx * (T - s.tx))) >> 3;
        qy = (T == Ty ? (s.sy > 0 ? y0 + L : y0 - 1) : __float2int_rd(fy + vy * (T - s.ty))) >> 3;
        qz = (T == Tz ? (s.sz > 0 ? z0 + L : z0 - 1) : __float2int_rd(fz + vz * (T - s.tz))) >> 3;
    }
    return false;
}

// host side (occlusion.cu): launch constants and the descriptor of one scene
TraceConstsP consts_of(const vxl_trace_params* p, const vxl_tuning& tune);
SceneDesc scene_of(const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p, const vxl_outputs* o,
                   const vxl_tuning& tune);

}  // namespace vxl
