// taa.cu — temporal accumulation of the lighting buffer (the pass after the
// occlusion path): Sources/Shaders/LightTAA.frag:37-141, one thread per
// pixel, operation for operation. texture() is this library's sampler for the
// pass (bilinear, clamp to edge, texel centres at (i + 0.5) / size; the
// engine's light images use its default linear filter) and sin/cos are the
// library's own (sincos_own), as in the oracle.
//
// Every spiral tap samples six images at the same coordinates. A streaming
// pre-pass (k_taa_pack) gathers the 16 floats a tap uses of each texel --
// material, normal, depth, colour, motion and the light's rgb -- into four
// float4 planes, so a bilinear tap is 16 vector loads instead of 40 loads
// over six planar images; the interpolated values are the same floats
// combined in the same order. Planes rather than 64-byte records: the 16-byte
// loads of a warp's scattered taps then spread over eight L1 bank groups
// (texel mod 8) instead of two.
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

// texture() of a 4-channel image with the pass's sampler (16-byte texels: one
// vector load each)
__device__ __forceinline__ void tex4(const float* __restrict__ p, int W, int H, float u, float v, float* out) {
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
    const float bx = 1.0f - ax, by = 1.0f - ay;
    const float4* q = reinterpret_cast<const float4*>(p);
    const float4 a = __ldg(q + ((size_t)y0 * W + x0)), b = __ldg(q + ((size_t)y0 * W + x1));
    const float4 c = __ldg(q + ((size_t)y1 * W + x0)), d = __ldg(q + ((size_t)y1 * W + x1));
    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
    const float cv[4] = {c.x, c.y, c.z, c.w}, dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float top = av[k] * bx + bv[k] * ax;
        const float bot = cv[k] * bx + dv[k] * ax;
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

// Texel planes (n texels each): q0 = material, q1 = (normal, depth),
// q2 = (colour, motion.x), q3 = (light rgb, motion.y).
constexpr int kTaaPlanes = 4;

__global__ void __launch_bounds__(256) k_taa_pack(const TaaIn I, float4* __restrict__ rec) {
    const int n = I.W * I.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 m = __ldg(reinterpret_cast<const float4*>(I.material) + i);
        const float4 l = __ldg(reinterpret_cast<const float4*>(I.light) + i);
        const float2 mo = __ldg(reinterpret_cast<const float2*>(I.motion) + i);
        const float* nr = I.normal + 3 * (size_t)i;
        const float* co = I.color + 3 * (size_t)i;
        rec[i] = m;
        rec[(size_t)n + i] = make_float4(__ldg(nr), __ldg(nr + 1), __ldg(nr + 2), __ldg(I.depth + i));
        rec[2 * (size_t)n + i] = make_float4(__ldg(co), __ldg(co + 1), __ldg(co + 2), mo.x);
        rec[3 * (size_t)n + i] = make_float4(l.x, l.y, l.z, mo.y);
    }
}

// One bilinear tap of every image a spiral / neighbourhood sample reads.
struct Tap {
    float mo[2], co[3], no[3], ma[4], de, li[3];
};

__device__ __forceinline__ void lerp4(const float4& a, const float4& b, const float4& c, const float4& d, float ax,
                                      float bx, float ay, float by, float* o) {
    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
    const float cv[4] = {c.x, c.y, c.z, c.w}, dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float top = av[k] * bx + bv[k] * ax;
        const float bot = cv[k] * bx + dv[k] * ax;
        o[k] = top * by + bot * ay;
    }
}

// The same coordinates, clamping and weights as tex4, over the planes.
__device__ __forceinline__ void tap(const float4* __restrict__ rec, int W, int H, float u, float v, Tap* t) {
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
    const float bx = 1.0f - ax, by = 1.0f - ay;
    const size_t n = (size_t)W * H;
    const float4* r00 = rec + ((size_t)y0 * W + x0);
    const float4* r10 = rec + ((size_t)y0 * W + x1);
    const float4* r01 = rec + ((size_t)y1 * W + x0);
    const float4* r11 = rec + ((size_t)y1 * W + x1);
    float o[4];
    lerp4(__ldg(r00), __ldg(r10), __ldg(r01), __ldg(r11), ax, bx, ay, by, t->ma);
    lerp4(__ldg(r00 + n), __ldg(r10 + n), __ldg(r01 + n), __ldg(r11 + n), ax, bx, ay, by, o);
    t->no[0] = o[0];
    t->no[1] = o[1];
    t->no[2] = o[2];
    t->de = o[3];
    lerp4(__ldg(r00 + 2 * n), __ldg(r10 + 2 * n), __ldg(r01 + 2 * n), __ldg(r11 + 2 * n), ax, bx, ay, by, o);
    t->co[0] = o[0];
    t->co[1] = o[1];
    t->co[2] = o[2];
    t->mo[0] = o[3];
    lerp4(__ldg(r00 + 3 * n), __ldg(r10 + 3 * n), __ldg(r01 + 3 * n), __ldg(r11 + 3 * n), ax, bx, ay, by, o);
    t->li[0] = o[0];
    t->li[1] = o[1];
    t->li[2] = o[2];
    t->mo[1] = o[3];
}

// Centre values a disocclusion tap compares against.
struct Centre {
    float uvx, uvy, no[3], ma[4], de, co[3], mo[2];
};

// One tap (x, y) of the 19x19 disocclusion neighbourhood (LightTAA.frag:61-80):
// (factor * light.rgb, factor), the terms its sums add in order.
__device__ __forceinline__ float4 disocc_tap(const float4* __restrict__ rec, int W, int H, float iResx, float iResy,
                                             const Centre& c, int x, int y) {
    const float FAR = 4096.0f;
    const float ox = (float)x * iResx, oy = (float)y * iResy;
    const float u = clampg(c.uvx + ox, 0.001f, 0.999f), v = clampg(c.uvy + oy, 0.001f, 0.999f);
    Tap t;
    tap(rec, W, H, u, v, &t);
    float factor = gmax(dot3(c.no, t.no), 0.0f);
    factor *= glsl_step(0.8f, 1.0f - len4(c.ma, t.ma));
    factor *= 1.0f - clampg(fabsf(c.de - t.de) * FAR, 0.0f, 1.0f);
    factor *= 1.0f - clampg(len3(c.co, t.co), 0.0f, 1.0f);
    if (len2(c.mo[0] - t.mo[0], c.mo[1] - t.mo[1]) > 0.1f) factor = 0.0f;
    return make_float4(factor * t.li[0], factor * t.li[1], factor * t.li[2], factor);
}

constexpr int kDisTaps = 19 * 19;
constexpr int kDisCoopMax = 16;  // warps with more disoccluded pixels run them one per lane

// 32x4-pixel blocks: the spiral taps of neighbouring pixels overlap in L1.
// A pixel whose reprojection leaves the screen samples 361 taps instead of 12;
// when a warp holds few such pixels, all 32 lanes compute each one's taps
// (x-major order, as the shader's loops) into shared memory and lanes 0-3
// add the four sums up in that order, so the result is the same float.
__global__ void __launch_bounds__(128) k_taa(const TaaIn I, const float4* __restrict__ rec, float* __restrict__ out) {
    __shared__ float4 s_dis[4][kDisTaps];
    const int W = I.W, H = I.H;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int px = blockIdx.x * 32 + lane, py = blockIdx.y * 4 + wib;
    const bool valid = px < W && py < H;
    const int i = valid ? py * W + px : 0;
    const float GR = 2.118033988749895f;
    const float iResx = 1.0f / (float)W, iResy = 1.0f / (float)H;
    float* o = out + 4 * (size_t)i;
    Centre c;
    c.uvx = ((float)px + 0.5f) / (float)W;
    c.uvy = ((float)py + 0.5f) / (float)H;
    float cl[4], ll[4];
    int mode = 0;  // 0 done, 1 disoccluded, 2 spiral
    if (valid) {
        Tap t;
        tap(rec, W, H, c.uvx, c.uvy, &t);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            c.no[k] = t.no[k];
            c.co[k] = t.co[k];
        }
#pragma unroll
        for (int k = 0; k < 4; k++) c.ma[k] = t.ma[k];
        c.de = t.de;
        c.mo[0] = t.mo[0];
        c.mo[1] = t.mo[1];
        tex4(I.light, W, H, c.uvx, c.uvy, cl);
        if (c.de == 1.0f) {
            o[0] = cl[0];
            o[1] = cl[1];
            o[2] = cl[2];
            o[3] = cl[3];
        } else {
            const float oux = c.uvx + c.mo[0], ouy = c.uvy + c.mo[1];
            tex4(I.last, W, H, oux, ouy, ll);
            mode = (clampg(oux, 0.0f, 1.0f) != oux || clampg(ouy, 0.0f, 1.0f) != ouy) ? 1 : 2;
        }
    }
    // disocclusion: the current frame's 19x19 neighbourhood only
    unsigned dis = __ballot_sync(0xffffffffu, mode == 1);
    if (dis != 0u && __popc(dis) <= kDisCoopMax) {
        float4* sd = s_dis[wib];
        while (dis) {
            const int p = __ffs(dis) - 1;
            dis &= dis - 1u;
            Centre q;
            q.uvx = __shfl_sync(0xffffffffu, c.uvx, p);
            q.uvy = __shfl_sync(0xffffffffu, c.uvy, p);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                q.no[k] = __shfl_sync(0xffffffffu, c.no[k], p);
                q.co[k] = __shfl_sync(0xffffffffu, c.co[k], p);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) q.ma[k] = __shfl_sync(0xffffffffu, c.ma[k], p);
            q.de = __shfl_sync(0xffffffffu, c.de, p);
            q.mo[0] = __shfl_sync(0xffffffffu, c.mo[0], p);
            q.mo[1] = __shfl_sync(0xffffffffu, c.mo[1], p);
            for (int t = lane; t < kDisTaps; t += 32) sd[t] = disocc_tap(rec, W, H, iResx, iResy, q, t / 19 - 9, t % 19 - 9);
            __syncwarp();
            float acc = 0.0f;
            if (lane < 4) {
                const float* f = reinterpret_cast<const float*>(sd) + lane;
                for (int t = 0; t < kDisTaps; t++) acc += f[4 * t];
            }
            const float s0 = __shfl_sync(0xffffffffu, acc, 0), s1 = __shfl_sync(0xffffffffu, acc, 1);
            const float s2 = __shfl_sync(0xffffffffu, acc, 2), count = __shfl_sync(0xffffffffu, acc, 3);
            if (lane == p) {
                o[0] = s0 / count;
                o[1] = s1 / count;
                o[2] = s2 / count;
                o[3] = 1.0f;
            }
            __syncwarp();
        }
        if (mode == 1) mode = 0;
    }
    if (mode == 1) {
        float count = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (int x = -9; x <= 9; ++x)
            for (int y = -9; y <= 9; ++y) {
                const float4 r = disocc_tap(rec, W, H, iResx, iResy, c, x, y);
                s0 += r.x;
                s1 += r.y;
                s2 += r.z;
                count += r.w;
            }
        o[0] = s0 / count;
        o[1] = s1 / count;
        o[2] = s2 / count;
        o[3] = 1.0f;
        return;
    }
    if (mode != 2) return;
    const float* motion = c.mo;
    const float* cc = c.co;
    const float* cm = c.ma;
    const float* cn = c.no;
    const float depth = c.de;
    const float uvx = c.uvx, uvy = c.uvy;
    const float FAR = 4096.0f;
    float lastVariance = ll[3];
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
        Tap t;
        tap(rec, W, H, u, v, &t);
        const float* nli = t.li;
        float factor = 1.212f - radius / size;
        factor *= glsl_step(0.8f, 1.0f - len4(cm, t.ma));
        factor *= gmax(dot3(cn, t.no), 0.0f);
        factor *= 1.0f - clampg(fabsf(depth - t.de) * FAR, 0.0f, 1.0f);
        factor *= 1.0f - clampg(len3(cc, t.co) * 10000.0f, 0.0f, 1.0f);
        if (len2(motion[0] - t.mo[0], motion[1] - t.mo[1]) > 0.1f) factor = 0.0f;
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
    const size_t n = (size_t)f->width * f->height;
    VXL_TRY(ctx_grow(&ctx->d_taa, &ctx->taa_bytes, n * kTaaPlanes * sizeof(float4)));
    float4* rec = (float4*)ctx->d_taa;
    const unsigned pack_blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)ctx->sm_count * 8);
    k_taa_pack<<<pack_blocks, 256, 0, s>>>(I, rec);
    ctx->launches++;
    const dim3 grid((unsigned)((f->width + 31) / 32), (unsigned)((f->height + 3) / 4));
    k_taa<<<grid, 128, 0, s>>>(I, rec, out);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
