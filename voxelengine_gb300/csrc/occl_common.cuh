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

// One scene of a launch: grid, G-buffer, outputs, tiling, ray parameters.
struct SceneDesc {
    GridView g;
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

// host side (occlusion.cu): launch constants and the descriptor of one scene
TraceConstsP consts_of(const vxl_trace_params* p, const vxl_tuning& tune);
SceneDesc scene_of(const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p, const vxl_outputs* o,
                   const vxl_tuning& tune);

}  // namespace vxl
