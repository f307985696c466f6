// taa.cu — temporal accumulation of the lighting buffer (the pass after the
// occlusion path): Sources/Shaders/LightTAA.frag:37-141, one thread per
// pixel, operation for operation. texture() is this library's sampler for the
// pass (bilinear, clamp to edge, texel centres at (i + 0.5) / size; the
// engine's light images use its default linear filter) and sin/cos are the
// library's own (sincos_own), as in the oracle.
#include "vxl_device.cuh"
#include "vxl_internal.h"

namespace vxl {
namespace {

struct TaaIn {
    const float* light;     // 4 channels
    const float* last;      // 4
    const float* color;     // 3
    const float* normal;    // 3
    const float* material;  // 4
    const float* depth;     // 1
    const float* motion;    // 2
    const float* noise;     // 4
    int W, H;
};

__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float clampg(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

template <int C>
__device__ __forceinline__ void tex(const float* __restrict__ p, int W, int H, float u, float v, float* out) {
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
    const float bx = 1.0f - ax, by = 1.0f - ay;
    const size_t i00 = ((size_t)y0 * W + x0) * C, i10 = ((size_t)y0 * W + x1) * C;
    const size_t i01 = ((size_t)y1 * W + x0) * C, i11 = ((size_t)y1 * W + x1) * C;
    float t00[C], t10[C], t01[C], t11[C];
    if (C == 4) {  // 16-byte texels: one vector load each
        const float4 a = __ldg(reinterpret_cast<const float4*>(p + i00)), b = __ldg(reinterpret_cast<const float4*>(p + i10));
        const float4 c = __ldg(reinterpret_cast<const float4*>(p + i01)), d = __ldg(reinterpret_cast<const float4*>(p + i11));
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
        const float cv[4] = {c.x, c.y, c.z, c.w}, dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
        for (int k = 0; k < C; k++) {
            t00[k] = av[k];
            t10[k] = bv[k];
            t01[k] = cv[k];
            t11[k] = dv[k];
        }
    } else if (C == 2) {
        const float2 a = __ldg(reinterpret_cast<const float2*>(p + i00)), b = __ldg(reinterpret_cast<const float2*>(p + i10));
        const float2 c = __ldg(reinterpret_cast<const float2*>(p + i01)), d = __ldg(reinterpret_cast<const float2*>(p + i11));
        const float av[2] = {a.x, a.y}, bv[2] = {b.x, b.y}, cv[2] = {c.x, c.y}, dv[2] = {d.x, d.y};
#pragma unroll
        for (int k = 0; k < C; k++) {
            t00[k] = av[k];
            t10[k] = bv[k];
            t01[k] = cv[k];
            t11[k] = dv[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < C; k++) {
            t00[k] = __ldg(p + i00 + k);
            t10[k] = __ldg(p + i10 + k);
            t01[k] = __ldg(p + i01 + k);
            t11[k] = __ldg(p + i11 + k);
        }
    }
#pragma unroll
    for (int k = 0; k < C; k++) {
        const float top = t00[k] * bx + t10[k] * ax;
        const float bot = t01[k] * bx + t11[k] * ax;
        out[k] = top * by + bot * ay;
    }
}
__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }
__device__ __forceinline__ float len3(const float* a, const float* b) {
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float d = dx * dx + dy * dy;
    d = d + dz * dz;
    return sqrtf(d);
}
__device__ __forceinline__ float len4(const float* a, const float* b) {
    const float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2], d3 = a[3] - b[3];
    float d = d0 * d0 + d1 * d1;
    d = d + d2 * d2;
    d = d + d3 * d3;
    return sqrtf(d);
}
__device__ __forceinline__ float dot3(const float* a, const float* b) {
    float d = a[0] * b[0] + a[1] * b[1];
    return d + a[2] * b[2];
}

// 32x4-pixel blocks: the spiral taps of neighbouring pixels overlap in L1
__global__ void __launch_bounds__(128) k_taa(const TaaIn I, float* __restrict__ out) {
    const int W = I.W, H = I.H;
    const int px = blockIdx.x * 32 + (threadIdx.x & 31), py = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (px >= W || py >= H) return;
    const int i = py * W + px;
    const float FAR = 4096.0f;
    const float GR = 2.118033988749895f;
    const float iResx = 1.0f / (float)W, iResy = 1.0f / (float)H;
    const float uvx = ((float)px + 0.5f) / (float)W, uvy = ((float)py + 0.5f) / (float)H;
    float motion[2], cl[4], cc[3], cm[4], cn[3], cd[1], ll[4];
    tex<2>(I.motion, W, H, uvx, uvy, motion);
    const float oux = uvx + motion[0], ouy = uvy + motion[1];
    tex<4>(I.light, W, H, uvx, uvy, cl);
    tex<3>(I.color, W, H, uvx, uvy, cc);
    tex<4>(I.material, W, H, uvx, uvy, cm);
    tex<3>(I.normal, W, H, uvx, uvy, cn);
    tex<1>(I.depth, W, H, uvx, uvy, cd);
    const float depth = cd[0];
    float* o = out + 4 * (size_t)i;
    if (depth == 1.0f) {
        o[0] = cl[0];
        o[1] = cl[1];
        o[2] = cl[2];
        o[3] = cl[3];
        return;
    }
    tex<4>(I.last, W, H, oux, ouy, ll);
    float lastVariance = ll[3];
    if (clampg(oux, 0.0f, 1.0f) != oux || clampg(ouy, 0.0f, 1.0f) != ouy) {
        // disocclusion: the current frame's 19x19 neighbourhood only
        float count = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (int x = -9; x <= 9; ++x)
            for (int y = -9; y <= 9; ++y) {
                const float ox = (float)x * iResx, oy = (float)y * iResy;
                const float u = clampg(uvx + ox, 0.001f, 0.999f), v = clampg(uvy + oy, 0.001f, 0.999f);
                float nmo[2], nco[3], nno[3], nma[4], nde[1], nli[4];
                tex<2>(I.motion, W, H, u, v, nmo);
                tex<3>(I.color, W, H, u, v, nco);
                tex<3>(I.normal, W, H, u, v, nno);
                tex<4>(I.material, W, H, u, v, nma);
                tex<1>(I.depth, W, H, u, v, nde);
                float factor = gmax(dot3(cn, nno), 0.0f);
                factor *= glsl_step(0.8f, 1.0f - len4(cm, nma));
                factor *= 1.0f - clampg(fabsf(depth - nde[0]) * FAR, 0.0f, 1.0f);
                factor *= 1.0f - clampg(len3(cc, nco), 0.0f, 1.0f);
                if (len2(motion[0] - nmo[0], motion[1] - nmo[1]) > 0.1f) factor = 0.0f;
                tex<4>(I.light, W, H, u, v, nli);
                s0 += factor * nli[0];
                s1 += factor * nli[1];
                s2 += factor * nli[2];
                count += factor;
            }
        o[0] = s0 / count;
        o[1] = s1 / count;
        o[2] = s2 / count;
        o[3] = 1.0f;
        return;
    }
    // 12-tap golden-angle spiral, neighbourhood clip, variance-driven blend
    float nmin[3] = {10000.0f, 10000.0f, 10000.0f}, nmax[3] = {0.0f, 0.0f, 0.0f};
    float ncol[3] = {0.0f, 0.0f, 0.0f};
    float diffSum = 1.0f, count = 0.0f;
    const float size = 12.0f;
    float radius = 1.0f;
    const float dscale = gmin(gmax(0.1f, 0.5f), 1.0f / depth);
    const float n0 = __ldg(I.noise + 4 * (size_t)i);
    for (float angle = n0 * 3.1415f * GR; radius <= size; angle += 2.39f) {
        radius += 1.0f;
        float sn, cs;
        sincos_own(angle, &sn, &cs);
        const float rv = radius * (lastVariance + 1.0f);
        const float ox = cs * iResx * rv * dscale, oy = sn * iResy * rv * dscale;
        const float u = clampg(uvx + ox, 0.001f, 0.999f), v = clampg(uvy + oy, 0.001f, 0.999f);
        float nmo[2], nco[3], nno[3], nma[4], nde[1], nli[4];
        tex<2>(I.motion, W, H, u, v, nmo);
        tex<3>(I.color, W, H, u, v, nco);
        tex<3>(I.normal, W, H, u, v, nno);
        tex<4>(I.material, W, H, u, v, nma);
        tex<1>(I.depth, W, H, u, v, nde);
        float factor = 1.212f - radius / size;
        factor *= glsl_step(0.8f, 1.0f - len4(cm, nma));
        factor *= gmax(dot3(cn, nno), 0.0f);
        factor *= 1.0f - clampg(fabsf(depth - nde[0]) * FAR, 0.0f, 1.0f);
        factor *= 1.0f - clampg(len3(cc, nco) * 10000.0f, 0.0f, 1.0f);
        if (len2(motion[0] - nmo[0], motion[1] - nmo[1]) > 0.1f) factor = 0.0f;
        tex<4>(I.light, W, H, u, v, nli);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            nmin[k] = gmin(nmin[k], nli[k]);
            nmax[k] = gmax(nmax[k], nli[k]);
            ncol[k] += factor * nli[k];
        }
        count += factor;
        diffSum += len3(nli, cl) * factor;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        cl[k] += ncol[k];
        cl[k] /= count + 1.0f;
    }
    diffSum /= radius;
#pragma unroll
    for (int k = 0; k < 3; k++) ll[k] = gmin(gmax(ll[k], nmin[k]), nmax[k]);
    const float a0 = fabsf(cl[0] - ll[0]), a1 = fabsf(cl[1] - ll[1]), a2 = fabsf(cl[2] - ll[2]);
    float lum = a0 * 0.2125f + a1 * 0.7154f;
    lum = lum + a2 * 0.0721f;
    const float variance = clampg(lum * 5.5f, 0.0f, 1.0f);
    lastVariance += variance;
    lastVariance -= diffSum * 0.08f;
    lastVariance += len2(motion[0], motion[1]) * 20.0f;
    const float t = clampg(1.0f - lastVariance, 0.3f, 0.9f);
    const float omt = 1.0f - t;
    o[0] = cl[0] * omt + ll[0] * t;
    o[1] = cl[1] * omt + ll[1] * t;
    o[2] = cl[2] * omt + ll[2] * t;
    o[3] = clampg(lastVariance * 0.7f, 0.0f, 1.0f);
}

}  // namespace

vxl_status launch_light_taa(vxl_ctx* ctx, const vxl_taa_frame* f, float* out, cudaStream_t s) {
    TaaIn I{f->light, f->last_light, f->color, f->normal, f->material, f->depth, f->motion, f->noise, f->width,
            f->height};
    const dim3 grid((unsigned)((f->width + 31) / 32), (unsigned)((f->height + 3) / 4));
    k_taa<<<grid, 128, 0, s>>>(I, out);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
