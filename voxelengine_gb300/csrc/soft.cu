// soft.cu — differentiable soft-opacity / albedo variant of the occlusion
// pass: forward kernel and a hand-written adjoint that walks each ray again
// instead of storing per-ray segments between the two calls.
//
// Model (no reference counterpart; the reference grid is binary): every ray
// visits the cells that the reference DDA (Sources/Shaders/lib/Light.frag:29-81)
// visits on an empty grid up to t = len — same fp32 stepping, same tie
// handling, same inclusive upper bound dims+1, same 256-step cap — and stops
// early once its transmittance is below 2^-40. Cells outside the data are
// empty. With a = clamp(opacity, 0, 1 - 2^-12):
//   T = prod (1 - a_i),   C = sum_i T_<i a_i albedo_i
//   light[c] = k_sun T_sh + k_amb / K sum_k (T_k + C_k[c]),  image = albedo_s * light
//
// Layout: one CTA per 32 consecutive pixels, one warp per ray of those
// pixels (warp k = ray k, lane = pixel), so a warp's lanes trace the same ray
// index of neighbouring pixels (one light direction for the shadow warp).
// The forward pass combines the R per-ray results of a pixel in a fixed
// order in shared memory (deterministic). The adjoint records the visited
// cells and their prefix transmittance in a per-thread list (at most 256
// cells, the DDA's step cap), then runs the list backwards carrying suffix
// products, so no division and no cancellation is involved; gradients are
// scattered with 16-byte vector atomics.
#include "vxl_device.cuh"
#include "vxl_internal.h"

namespace vxl {
namespace {

constexpr float kSoftAmax = 1.0f - 1.0f / 4096.0f;
constexpr float kSoftTmin = 9.094947017729282e-13f;  // 2^-40
constexpr int kSoftMaxCells = 256;                   // DDA step cap: n < 256

struct SoftConsts {
    const float4* vox;
    int nx, ny, nz;
    const float* pos;
    const float* nrm;
    int npix;
    f3 light;
    float bias, len, ks, ka;
    int n_shadow, R;
    uint32_t seed_h;
};

// Cell sequence of raycastShadowVolume (Light.frag:29-81) on an empty grid of
// fine dims nx, ny, nz. Directions whose components all satisfy |d| >= 1e-30
// use the register form of dda_run (exact for them); the others follow the
// shader's select/step arithmetic literally, as dda_literal does.
struct CellWalk {
    int cx, cy, cz;
    float tx, ty, tz, tdx, tdy, tdz;
    float ssx, ssy, ssz;
    float maxt;
    int ux, uy, uz;
    int n;
    bool fast, done;

    __device__ __forceinline__ void init(f3 o, f3 d, float mt, int nx, int ny, int nz) {
        ux = nx + 1;
        uy = ny + 1;
        uz = nz + 1;
        maxt = mt;
        n = 0;
        done = !ray_domain_ok(o, d);
        fast = dir_fast_ok(d);
        ssx = glsl_sign(d.x);
        ssy = glsl_sign(d.y);
        ssz = glsl_sign(d.z);
        cx = (int)floorf(o.x);
        cy = (int)floorf(o.y);
        cz = (int)floorf(o.z);
        if (fast) {
            tdx = 1.0f / fabsf(d.x);
            tdy = 1.0f / fabsf(d.y);
            tdz = 1.0f / fabsf(d.z);
            tx = (((float)cx + (ssx > 0.0f ? 1.0f : 0.0f)) - o.x) / d.x;
            ty = (((float)cy + (ssy > 0.0f ? 1.0f : 0.0f)) - o.y) / d.y;
            tz = (((float)cz + (ssz > 0.0f ? 1.0f : 0.0f)) - o.z) / d.z;
        } else {
            tdx = 1.0f / (d.x * ssx);
            tdy = 1.0f / (d.y * ssy);
            tdz = 1.0f / (d.z * ssz);
            tx = ((float)cx + (ssx * 0.5f + 0.5f) - o.x) / d.x;
            ty = ((float)cy + (ssy * 0.5f + 0.5f) - o.y) / d.y;
            tz = ((float)cz + (ssz * 0.5f + 0.5f) - o.z) / d.z;
        }
    }
    // The current cell if the walk goes on (bounds test of Light.frag:53-55).
    __device__ __forceinline__ bool cell() {
        if (done) return false;
        if (cx < 0 || cy < 0 || cz < 0 || cx > ux || cy > uy || cz > uz) {
            done = true;
            return false;
        }
        return true;
    }
    // The no-hit branch of the loop body and the loop condition (:62-75).
    __device__ __forceinline__ void advance() {
        float best;
        if (fast) {
            const float m = fminf(fminf(tx, ty), tz);
            const bool bx = tx == m, by = ty == m, bz = tz == m;
            best = m + 0.0f;
            if ((bx && (by || bz)) || (by && bz)) {
                best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
                best = best + (bz ? tz : 0.0f);
            }
            if (bx) { cx += (int)ssx; tx = tx + tdx; }
            if (by) { cy += (int)ssy; ty = ty + tdy; }
            if (bz) { cz += (int)ssz; tz = tz + tdz; }
        } else {
            const float selx = glsl_step(tx, tz) * glsl_step(tx, ty);
            const float sely = glsl_step(ty, tx) * glsl_step(ty, tz);
            const float selz = glsl_step(tz, ty) * glsl_step(tz, tx);
            best = tx * selx + ty * sely;
            best = best + tz * selz;
            cx += (int)(selx * ssx);
            cy += (int)(sely * ssy);
            cz += (int)(selz * ssz);
            tx += tdx * selx;
            ty += tdy * sely;
            tz += tdz * selz;
        }
        if (!(++n < 256 && best < maxt)) done = true;
    }
};

__device__ __forceinline__ float soft_clamp(float a) { return fminf(fmaxf(a, 0.0f), kSoftAmax); }

// Pixel setup shared by both passes. Returns the surface voxel index, or -1
// when the pixel traces nothing (zero normal, or surface voxel off the grid).
__device__ __forceinline__ int pixel_setup(const SoftConsts& c, int pix, int k, f3* O, f3* D) {
    const f3 P = mk(c.pos[3 * pix], c.pos[3 * pix + 1], c.pos[3 * pix + 2]);
    const f3 N = mk(c.nrm[3 * pix], c.nrm[3 * pix + 1], c.nrm[3 * pix + 2]);
    if (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f) return -1;
    const int sx = (int)floorf(P.x - N.x * 0.5f), sy = (int)floorf(P.y - N.y * 0.5f),
              sz = (int)floorf(P.z - N.z * 0.5f);
    if (sx < 0 || sy < 0 || sz < 0 || sx >= c.nx || sy >= c.ny || sz >= c.nz) return -1;
    *O = add(P, mul(N, c.bias));
    if (k < c.n_shadow) {
        *D = c.light;
    } else {
        const uint32_t j = (uint32_t)(k - c.n_shadow);
        f3 T, B;
        tangent_frame(N, &T, &B);
        const float u1 = rand01(c.seed_h, (uint32_t)pix, 64u + 2u * j);
        const float u2 = rand01(c.seed_h, (uint32_t)pix, 65u + 2u * j);
        *D = frame_dir(T, B, N, cosine_sample(u1, u2));
    }
    return sx + sy * c.nx + sz * c.nx * c.ny;
}

__global__ void __launch_bounds__(1024) k_soft_fwd(const SoftConsts c, float* __restrict__ image,
                                                   float* __restrict__ light) {
    extern __shared__ float4 s_ray[];  // [R][32]: T, C rgb
    const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
    const int pix = blockIdx.x * 32 + lane;
    float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f;
    int s = -1;
    if (pix < c.npix) {
        f3 O, D;
        s = pixel_setup(c, pix, k, &O, &D);
        if (s >= 0) {
            CellWalk w;
            w.init(O, D, c.len, c.nx, c.ny, c.nz);
            while (w.cell()) {
                if (w.cx < c.nx && w.cy < c.ny && w.cz < c.nz) {
                    const float4 v = __ldg(c.vox + (w.cx + w.cy * c.nx + w.cz * c.nx * c.ny));
                    const float a = soft_clamp(v.x);
                    const float ta = T * a;
                    C0 = C0 + ta * v.y;
                    C1 = C1 + ta * v.z;
                    C2 = C2 + ta * v.w;
                    T = T * (1.0f - a);
                    if (T < kSoftTmin) break;
                }
                w.advance();
            }
        }
    }
    s_ray[k * 32 + lane] = make_float4(T, C0, C1, C2);
    __syncthreads();
    if (k != 0 || pix >= c.npix) return;
    float L0 = 0.0f, L1 = 0.0f, L2 = 0.0f, I0 = 0.0f, I1 = 0.0f, I2 = 0.0f;
    if (s >= 0) {
        float Tsh = 1.0f, Ts = 0.0f, S0 = 0.0f, S1 = 0.0f, S2 = 0.0f;
        if (c.n_shadow) Tsh = s_ray[lane].x;
        for (int r = c.n_shadow; r < c.R; r++) {
            const float4 q = s_ray[r * 32 + lane];
            Ts = Ts + q.x;
            S0 = S0 + q.y;
            S1 = S1 + q.z;
            S2 = S2 + q.w;
        }
        const float sun = c.ks * Tsh;
        L0 = sun + c.ka * (Ts + S0);
        L1 = sun + c.ka * (Ts + S1);
        L2 = sun + c.ka * (Ts + S2);
        const float4 rs = __ldg(c.vox + s);
        I0 = rs.y * L0;
        I1 = rs.z * L1;
        I2 = rs.w * L2;
    }
    image[3 * pix] = I0;
    image[3 * pix + 1] = I1;
    image[3 * pix + 2] = I2;
    if (light) {
        light[3 * pix] = L0;
        light[3 * pix + 1] = L1;
        light[3 * pix + 2] = L2;
    }
}

__global__ void __launch_bounds__(1024) k_soft_bwd(const SoftConsts c, const float* __restrict__ gimg,
                                                   const float* __restrict__ light, float4* __restrict__ grad) {
    const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
    const int pix = blockIdx.x * 32 + lane;
    if (pix >= c.npix) return;
    f3 O, D;
    const int s = pixel_setup(c, pix, k, &O, &D);
    if (s < 0) return;
    const float g0 = gimg[3 * pix], g1 = gimg[3 * pix + 1], g2 = gimg[3 * pix + 2];
    const float4 rs = __ldg(c.vox + s);
    if (k == 0) {  // d image / d albedo_s = light
        const float4 ga = make_float4(0.0f, g0 * light[3 * pix], g1 * light[3 * pix + 1], g2 * light[3 * pix + 2]);
        atomicAdd(grad + s, ga);
    }
    const bool shadow = k < c.n_shadow;
    const float kk = shadow ? c.ks : c.ka;
    const float w0 = g0 * rs.y * kk, w1 = g1 * rs.z * kk, w2 = g2 * rs.w * kk;
    const float wsum = (w0 + w1) + w2;

    int2 cell[kSoftMaxCells];  // (voxel index, prefix transmittance bits): one 8-byte local store per cell
    int m = 0;
    {
        CellWalk w;
        w.init(O, D, c.len, c.nx, c.ny, c.nz);
        float T = 1.0f;
        while (w.cell()) {
            if (w.cx < c.nx && w.cy < c.ny && w.cz < c.nz) {
                const int idx = w.cx + w.cy * c.nx + w.cz * c.nx * c.ny;
                const float a = soft_clamp(__ldg(&c.vox[idx].x));
                cell[m] = make_int2(idx, __float_as_int(T));
                m++;
                T = T * (1.0f - a);
                if (T < kSoftTmin) break;
            }
            w.advance();
        }
    }
    // suffix pass: suf = prod_{l>j} (1 - a_l); S = colour seen from just past j
    float suf = 1.0f, S0 = 0.0f, S1 = 0.0f, S2 = 0.0f;
    for (int j = m - 1; j >= 0; j--) {
        const int2 ce = cell[j];
        const int idx = ce.x;
        const float pre = __int_as_float(ce.y);
        const float4 v = __ldg(c.vox + idx);
        const float a = soft_clamp(v.x);
        const float dcl = (v.x >= 0.0f && v.x <= kSoftAmax) ? 1.0f : 0.0f;
        const float ps = pre * suf;
        if (shadow) {
            atomicAdd(&grad[idx].x, -wsum * ps * dcl);
        } else {
            float ga = -wsum * ps;
            ga = ga + w0 * (pre * v.y - pre * S0);
            ga = ga + w1 * (pre * v.z - pre * S1);
            ga = ga + w2 * (pre * v.w - pre * S2);
            const float pa = pre * a;
            atomicAdd(grad + idx, make_float4(ga * dcl, w0 * pa, w1 * pa, w2 * pa));
            const float ia = 1.0f - a;
            S0 = a * v.y + ia * S0;
            S1 = a * v.z + ia * S1;
            S2 = a * v.w + ia * S2;
        }
        suf = suf * (1.0f - a);
    }
}

SoftConsts soft_consts(const float* soft, int nx, int ny, int nz, const vxl_gbuffer* gb, const vxl_soft_params* p) {
    SoftConsts c;
    c.vox = reinterpret_cast<const float4*>(soft);
    c.nx = nx;
    c.ny = ny;
    c.nz = nz;
    c.pos = gb->pos;
    c.nrm = gb->nrm;
    c.npix = (int)gb->npix;
    c.light = mk(p->light_dir[0], p->light_dir[1], p->light_dir[2]);
    c.bias = p->bias;
    c.len = p->len;
    c.n_shadow = p->n_shadow;
    c.R = p->n_shadow + p->n_ao;
    c.ks = p->n_shadow > 0 ? p->k_sun : 0.0f;
    c.ka = p->n_ao > 0 ? p->k_amb / (float)p->n_ao : 0.0f;
    c.seed_h = pcg(p->seed);
    return c;
}

}  // namespace

vxl_status launch_soft_fwd(vxl_ctx* ctx, const float* soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                           const vxl_soft_params* p, float* image, float* light, cudaStream_t st) {
    if (gb->npix == 0) return VXL_OK;
    const SoftConsts c = soft_consts(soft, nx, ny, nz, gb, p);
    const unsigned blocks = (unsigned)((gb->npix + 31) / 32);
    k_soft_fwd<<<blocks, 32 * c.R, (size_t)c.R * 32 * sizeof(float4), st>>>(c, image, light);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_soft_bwd(vxl_ctx* ctx, const float* soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                           const vxl_soft_params* p, const float* grad_image, const float* light, float* grad_soft,
                           cudaStream_t st) {
    if (gb->npix == 0) return VXL_OK;
    const SoftConsts c = soft_consts(soft, nx, ny, nz, gb, p);
    const unsigned blocks = (unsigned)((gb->npix + 31) / 32);
    k_soft_bwd<<<blocks, 32 * c.R, 0, st>>>(c, grad_image, light, reinterpret_cast<float4*>(grad_soft));
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
