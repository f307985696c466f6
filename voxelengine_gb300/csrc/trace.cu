// trace.cu — occlusion tracing kernels: raw ray batches (DDA / Sparse /
// SuperSparse), the DDA-mode occlusion pass over a G-buffer, and the
// reference light passes (ambient, reflection, point/spot).
#include "vxl_device.cuh"

namespace vxl {

// ------------------------------------------------------------ ray batches
template <int MODE>
__global__ void __launch_bounds__(128) k_trace_rays(GridView g, const float* __restrict__ rays, int64_t n,
                                                    vxl_ray_record* __restrict__ rec) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* q = rays + 7 * i;
        f3 o = mk(q[0], q[1], q[2]), d = mk(q[3], q[4], q[5]);
        float maxt = q[6];
        Hit h;
        if (MODE == VXL_MODE_DDA)
            h = dda(g, o, d, maxt);
        else
            h = march(g, o, d, maxt, MODE == VXL_MODE_SPARSE ? 0.5f : 2.5f);
        store_record(rec + i, h);
    }
}

// ------------------------------------------------------ DDA-mode occlusion
struct TraceConsts {
    f3 light;
    f3 cam;
    float bias, shadow_len, ao_len, spec_len, default_rough;
    int n_shadow, n_ao, n_spec;
    uint32_t seed_h;
};

// One thread per pixel; rays of a pixel in the order shadow, AO 0..n-1,
// spec 0..n-1. Same ray generation as the oracle's occlusion_pixel.
template <bool RECORDS>
__global__ void __launch_bounds__(128) k_occlusion(GridView g, const float* __restrict__ pos,
                                                   const float* __restrict__ nrm, const float* __restrict__ rough,
                                                   int64_t npix, TraceConsts c, float* __restrict__ o_shadow,
                                                   float* __restrict__ o_ao, float* __restrict__ o_vis,
                                                   float* __restrict__ o_spec, float* __restrict__ o_spec_t,
                                                   vxl_ray_record* __restrict__ rec) {
    const int R = c.n_shadow + c.n_ao + c.n_spec;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
         i += (int64_t)gridDim.x * blockDim.x) {
        f3 P = ld3(pos + 3 * i), N = ld3(nrm + 3 * i);
        float sh = 1.0f, ao = 1.0f, vis = 1.0f, sp = 1.0f, st = c.spec_len;
        if (!(N.x == 0.0f && N.y == 0.0f && N.z == 0.0f)) {
            f3 O = add(P, mul(N, c.bias));
            int slot = 0;
            if (c.n_shadow > 0) {
                Hit h = dda(g, O, c.light, c.shadow_len);
                sh = (h.flags & VXL_RF_HIT) ? 0.0f : 1.0f;
                if (RECORDS) store_record(rec + i * R + slot, h);
                slot++;
            }
            f3 T, B;
            tangent_frame(N, &T, &B);
            float acc = 0.0f, v = 0.0f;
            for (int k = 0; k < c.n_ao; k++) {
                float u1 = rand01(c.seed_h, (uint32_t)i, 64u + 2u * k);
                float u2 = rand01(c.seed_h, (uint32_t)i, 65u + 2u * k);
                f3 d = frame_dir(T, B, N, cosine_sample(u1, u2));
                Hit h = dda(g, O, d, c.ao_len);
                bool hit = h.flags & VXL_RF_HIT;
                float tt = hit ? (h.t < c.ao_len ? h.t : c.ao_len) : c.ao_len;
                float q = tt / c.ao_len;
                acc += q * q;
                v += hit ? 0.0f : 1.0f;
                if (RECORDS) store_record(rec + i * R + slot, h);
                slot++;
            }
            if (c.n_ao > 0) {
                ao = acc / (float)c.n_ao;
                vis = v / (float)c.n_ao;
            }
            if (c.n_spec > 0) {
                float ro = rough ? rough[i] : c.default_rough;
                float a = ro * ro;
                float a2 = a * a;
                f3 V = normalize(sub(c.cam, P));
                float spa = 0.0f, sta = 0.0f;
                for (int j = 0; j < c.n_spec; j++) {
                    float u1 = rand01(c.seed_h, (uint32_t)i, 2u * j);
                    float u2 = rand01(c.seed_h, (uint32_t)i, 2u * j + 1u);
                    float ct = sqrtf((1.0f - u1) / (1.0f + (a2 - 1.0f) * u1));
                    float st2 = 1.0f - ct * ct;
                    float sn = sqrtf(st2 > 0.0f ? st2 : 0.0f);
                    float s, cs;
                    sincos_own(6.2831855f * u2, &s, &cs);
                    f3 H = frame_dir(T, B, N, mk(sn * cs, sn * s, ct));
                    float vh = dot(V, H);
                    f3 d = normalize(sub(mul(H, 2.0f * vh), V));
                    Hit h = dda(g, O, d, c.spec_len);
                    bool hit = h.flags & VXL_RF_HIT;
                    spa += hit ? 0.0f : 1.0f;
                    sta += hit ? h.t : c.spec_len;
                    if (RECORDS) store_record(rec + i * R + slot, h);
                    slot++;
                }
                sp = spa / (float)c.n_spec;
                st = sta / (float)c.n_spec;
            }
        } else if (RECORDS) {
            Hit z{0, 0, 0, 0.0f, 0, 0};
            for (int k = 0; k < R; k++) store_record(rec + i * R + k, z);
        }
        if (o_shadow) o_shadow[i] = sh;
        if (o_ao) o_ao[i] = ao;
        if (o_vis) o_vis[i] = vis;
        if (o_spec) o_spec[i] = sp;
        if (o_spec_t) o_spec_t[i] = st;
    }
}

// -------------------------------------------------- reference light passes
// LightAmbient.frag:148-173
__global__ void k_light_ambient(GridView g, const float* __restrict__ wcp_in, const float* __restrict__ nrm,
                                const float* __restrict__ depth, const float4* __restrict__ noise, int64_t npix,
                                f3 sun, float* __restrict__ shadow, float* __restrict__ irr,
                                vxl_ray_record* __restrict__ rec) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 nz = noise[i];
        f3 normal = ld3(nrm + 3 * i);
        f3 wcp = ld3(wcp_in + 3 * i);
        f3 randomVec = mul(cosine_sample(nz.x, nz.y), 0.1f);
        randomVec.z *= glsl_sign(nz.z - 0.5f);
        f3 wd = normalize(mix(sun, randomVec, 0.5f));
        wcp = add(wcp, mul(wd, nz.w * 1.0f));
        wcp = add(wcp, mul(randomVec, 2.5f));
        float bias = smoothstep(0.0f, 0.2f, depth[i]) * 50.0f + 1.5f;
        f3 o = add(wcp, mul(normal, bias));
        Hit h0 = march(g, o, wd, 128.0f, 0.5f);
        shadow[i] = (h0.t != 128.0f) ? 0.0f : 1.0f;
        f3 T, B;
        tangent_frame(normal, &T, &B);
        f3 dir = frame_dir(T, B, normal, cosine_sample(nz.x, nz.y));
        Hit h1 = march(g, o, dir, 128.0f, 2.5f);
        float dd = h1.t / 128.0f;
        irr[i] = dd * dd * 0.05f;
        if (rec) {
            store_record(rec + 2 * i, h0);
            store_record(rec + 2 * i + 1, h1);
        }
    }
}

// LightReflection.frag:92-113
__global__ void k_light_reflection(GridView g, const float* __restrict__ wcp_in, const float* __restrict__ nrm,
                                   const float* __restrict__ view_r, const float* __restrict__ rough,
                                   const float4* __restrict__ noise, int64_t npix, float* __restrict__ t_out,
                                   vxl_ray_record* __restrict__ rec) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 nz = noise[i];
        f3 normal = ld3(nrm + 3 * i);
        f3 wd = normalize(ld3(view_r + 3 * i));
        f3 wcp = ld3(wcp_in + 3 * i);
        f3 randomVec = cosine_sample(nz.x, nz.y);
        randomVec.z *= glsl_sign(nz.z - 0.5f);
        wd = mix(wd, randomVec, rough[i] * 0.1f);
        wcp = add(wcp, mul(normal, nz.w));
        wd = mul(wd, 1.0f + nz.w * 0.5f);
        Hit h = march(g, add(wcp, normal), wd, 256.0f, 0.5f);
        t_out[i] = h.t;
        if (rec) store_record(rec + i, h);
    }
}

// LightPoint.frag:234-267 (spot = 0), LightSpot.frag:83-117 (spot = 1)
__global__ void k_light_point(GridView g, const float* __restrict__ wpos, const float* __restrict__ nrm,
                              const float4* __restrict__ noise, int64_t npix, f3 L, float range, int spot,
                              float* __restrict__ shadow, vxl_ray_record* __restrict__ rec) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 nz = noise[i];
        f3 worldPos = ld3(wpos + 3 * i);
        f3 normal = ld3(nrm + 3 * i);
        f3 lightDir = sub(L, worldPos);
        float lightDistance = sqrtf(dot(lightDir, lightDir));
        if (lightDistance > range) {  // discard: output untouched
            if (rec) {
                Hit z{0, 0, 0, -1.0f, 0, 0};
                store_record(rec + i, z);
            }
            continue;
        }
        f3 wd;
        float hitDist;
        if (spot) {
            wd = mul(normalize(lightDir), 10.0f);
            hitDist = lightDistance * 10.0f;
        } else {
            wd = lightDir;
            hitDist = lightDistance * 10.5f;
        }
        f3 wcp = mul(worldPos, 10.0f);
        f3 randomVec = mul(cosine_sample(nz.x, nz.y), 0.1f);
        randomVec.z *= glsl_sign(nz.z - 0.5f);
        wd = normalize(mix(wd, randomVec, 0.5f));
        wcp = add(wcp, mul(wd, nz.w * 1.0f));
        wcp = add(wcp, mul(randomVec, 2.5f));
        Hit h = march(g, add(wcp, mul(normal, 0.5f)), wd, hitDist, spot ? 2.5f : 0.5f);
        shadow[i] = (h.t < hitDist) ? 0.0f : 1.0f;
        if (rec) store_record(rec + i, h);
    }
}

// Fused point / spot shadows for up to 64 lights (vxl_light_points): a light
// grid narrows each pixel's candidate lights, pass 1 runs the exact range
// tests and lists the pairs in range, pass 2 traces each listed pair's ray --
// the one k_light_point traces for that light alone -- and sets its bit in the
// pixel's 64-bit mask.
struct LightDev {
    f3 pos;
    float range;
    int spot;
};
struct LightTable {
    LightDev l[64];
    int n;
};

// The shadow ray of one (pixel, light) pair in range, as vxl_light_point traces
// it (LightPoint.frag:105-129, LightSpot.frag:93-117): true when unshadowed.
__device__ __forceinline__ bool light_pair_lit(const GridView& g, f3 worldPos, f3 normal, float4 nz, const LightDev& Lt,
                                               f3 lightDir, float lightDistance) {
    f3 wd;
    float hitDist;
    if (Lt.spot) {
        wd = mul(normalize(lightDir), 10.0f);
        hitDist = lightDistance * 10.0f;
    } else {
        wd = lightDir;
        hitDist = lightDistance * 10.5f;
    }
    f3 wcp = mul(worldPos, 10.0f);
    f3 randomVec = mul(cosine_sample(nz.x, nz.y), 0.1f);
    randomVec.z *= glsl_sign(nz.z - 0.5f);
    wd = normalize(mix(wd, randomVec, 0.5f));
    wcp = add(wcp, mul(wd, nz.w * 1.0f));
    wcp = add(wcp, mul(randomVec, 2.5f));
    const Hit h = march(g, add(wcp, mul(normal, 0.5f)), wd, hitDist, Lt.spot ? 2.5f : 0.5f);
    return !(h.t < hitDist);
}

// Light grid of the fused lights: kLightCells^3 cells over the box that holds
// every light's sphere; each cell keeps the mask of lights whose sphere, grown
// by a margin, touches the cell grown by a margin, so a pixel needs the exact
// range test for its cell's lights only (a pixel outside the box is in range
// of none). The margins cover the fp32 rounding of the cell index and of the
// box distance.
constexpr int kLightCells = 32;
struct LightGrid {
    f3 lo;         // box corner
    float cell;    // cell edge
    float inv;     // 1 / cell
    float slack;   // absolute margin: a few ulps of the largest light coordinate
    int on;        // 0: every pixel tests every light
};

__global__ void k_light_grid(const __grid_constant__ LightTable T, LightGrid LG, unsigned long long* __restrict__ masks) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kLightCells * kLightCells * kLightCells) return;
    const int cx = c % kLightCells, cy = (c / kLightCells) % kLightCells, cz = c / (kLightCells * kLightCells);
    const float m = LG.cell * 0.01f + LG.slack;
    const f3 a = mk(LG.lo.x + (float)cx * LG.cell - m, LG.lo.y + (float)cy * LG.cell - m,
                    LG.lo.z + (float)cz * LG.cell - m);
    const f3 b = mk(a.x + LG.cell + 2.0f * m, a.y + LG.cell + 2.0f * m, a.z + LG.cell + 2.0f * m);
    unsigned long long mask = 0ull;
    for (int l = 0; l < T.n; l++) {
        const LightDev& Lt = T.l[l];
        const float dx = fmaxf(fmaxf(a.x - Lt.pos.x, Lt.pos.x - b.x), 0.0f);
        const float dy = fmaxf(fmaxf(a.y - Lt.pos.y, Lt.pos.y - b.y), 0.0f);
        const float dz = fmaxf(fmaxf(a.z - Lt.pos.z, Lt.pos.z - b.z), 0.0f);
        const float r = fabsf(Lt.range) * 1.0001f + 1e-4f;
        if (!(dx * dx + dy * dy + dz * dz > r * r)) mask |= 1ull << l;
    }
    masks[c] = mask;
}

// Pass 1 of the fused lights: one thread per pixel. The pixel's candidate
// lights come from the light grid (all lights for a NaN position or without a
// grid); the exact per-pixel range test of each candidate sets the in-range
// mask. Pairs in range are appended to a list (one atomic per warp) for pass 2,
// which traces them with full warps; pairs past the list's capacity are traced
// here.
__global__ void __launch_bounds__(256) k_light_points(GridView g, const float* __restrict__ wpos,
                                                      const float* __restrict__ nrm, const float4* __restrict__ noise,
                                                      int64_t npix, const __grid_constant__ LightTable T, LightGrid LG,
                                                      const unsigned long long* __restrict__ masks,
                                                      unsigned long long* __restrict__ lit,
                                                      unsigned long long* __restrict__ in_range,
                                                      unsigned long long* __restrict__ pairs,
                                                      unsigned long long* __restrict__ npairs, uint64_t cap) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned long long all = T.n >= 64 ? ~0ull : ((1ull << T.n) - 1ull);
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < npix; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const bool valid = i < npix;
        const f3 worldPos = valid ? ld3(wpos + 3 * i) : mk(0.0f, 0.0f, 0.0f);
        unsigned long long cand = 0ull;
        if (valid) {
            cand = all;
            const bool nan_pos = worldPos.x != worldPos.x || worldPos.y != worldPos.y || worldPos.z != worldPos.z;
            if (LG.on && !nan_pos) {
                const float fx = floorf((worldPos.x - LG.lo.x) * LG.inv), fy = floorf((worldPos.y - LG.lo.y) * LG.inv),
                            fz = floorf((worldPos.z - LG.lo.z) * LG.inv);
                const float top = (float)kLightCells;
                if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < top && fy < top && fz < top)
                    cand = masks[((int)fz * kLightCells + (int)fy) * kLightCells + (int)fx];
                else
                    cand = 0ull;  // outside every light's sphere
            }
        }
        unsigned long long inr = 0ull;
        for (unsigned long long c = cand; c; c &= c - 1ull) {
            const int l = __ffsll((long long)c) - 1;
            const LightDev& Lt = T.l[l];
            const f3 lightDir = sub(Lt.pos, worldPos);
            const float lightDistance = sqrtf(dot(lightDir, lightDir));
            if (!(lightDistance > Lt.range)) inr |= 1ull << l;  // else the light's pass discards this pixel
        }
        // one list slot per pair in range: warp prefix sum, one atomic per warp
        const int cnt = __popcll(inr);
        int pre = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(full, pre, o);
            if (lane >= o) pre += y;
        }
        const int total = __shfl_sync(full, pre, 31);
        unsigned long long at0 = 0ull;
        if (lane == 0 && total > 0) at0 = atomicAdd(npairs, (unsigned long long)total);
        at0 = __shfl_sync(full, at0, 0) + (unsigned long long)(pre - cnt);
        unsigned long long litm = 0ull;
        for (unsigned long long c = inr; c; c &= c - 1ull, at0++) {
            const int l = __ffsll((long long)c) - 1;
            if (at0 < cap) {
                pairs[at0] = ((unsigned long long)i << 6) | (unsigned long long)l;
            } else {
                const LightDev& Lt = T.l[l];
                const f3 lightDir = sub(Lt.pos, worldPos);
                const float lightDistance = sqrtf(dot(lightDir, lightDir));
                if (light_pair_lit(g, worldPos, ld3(nrm + 3 * i), noise[i], Lt, lightDir, lightDistance))
                    litm |= 1ull << l;
            }
        }
        if (valid) {
            lit[i] = litm;
            if (in_range) in_range[i] = inr;
        }
    }
}

// Pass 2: the listed (pixel, light) pairs, one per thread.
__global__ void __launch_bounds__(256) k_light_pairs(GridView g, const float* __restrict__ wpos,
                                                     const float* __restrict__ nrm, const float4* __restrict__ noise,
                                                     const __grid_constant__ LightTable T,
                                                     const unsigned long long* __restrict__ pairs,
                                                     const unsigned long long* __restrict__ npairs, uint64_t cap,
                                                     unsigned long long* __restrict__ lit) {
    const unsigned long long n = *npairs < cap ? *npairs : cap;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long pr = pairs[e];
        const int64_t i = (int64_t)(pr >> 6);
        const int l = (int)(pr & 63ull);
        const LightDev& Lt = T.l[l];
        const f3 worldPos = ld3(wpos + 3 * i);
        const f3 lightDir = sub(Lt.pos, worldPos);
        const float lightDistance = sqrtf(dot(lightDir, lightDir));
        if (light_pair_lit(g, worldPos, ld3(nrm + 3 * i), noise[i], Lt, lightDir, lightDistance))
            atomicOr(lit + i, 1ull << l);
    }
}

// ---------------------------------------------------------------- launchers
static unsigned grid_blocks(vxl_ctx* ctx, int64_t n, int threads, int per_sm) {
    int64_t need = (n + threads - 1) / threads;
    int64_t cap = (int64_t)ctx->sm_count * per_sm;
    if (need > cap) need = cap;
    if (need < 1) need = 1;
    return (unsigned)need;
}

vxl_status launch_trace_rays(vxl_ctx* ctx, const vxl_grid* g, const float* rays, int64_t n, int mode,
                             vxl_ray_record* rec, cudaStream_t s) {
    if (n <= 0) return VXL_OK;
    GridView v = view_of(g);
    unsigned b = grid_blocks(ctx, n, 128, 16);
    if (mode == VXL_MODE_DDA)
        k_trace_rays<VXL_MODE_DDA><<<b, 128, 0, s>>>(v, rays, n, rec);
    else if (mode == VXL_MODE_SPARSE)
        k_trace_rays<VXL_MODE_SPARSE><<<b, 128, 0, s>>>(v, rays, n, rec);
    else
        k_trace_rays<VXL_MODE_SUPERSPARSE><<<b, 128, 0, s>>>(v, rays, n, rec);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_trace_occlusion(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p,
                                  const vxl_outputs* out, cudaStream_t s) {
    if (gb->npix <= 0) return VXL_OK;
    if (occl_pool_supported(g, p)) {
        unsigned long long* counter = nullptr;
        VXL_TRY(ctx_take_counter(ctx, s, &counter));
        return launch_trace_occlusion_pool(ctx, g, gb, p, out, counter, ctx->tune, s);
    }
    GridView v = view_of(g);
    TraceConsts c;
    c.light = mk(p->light_dir[0], p->light_dir[1], p->light_dir[2]);
    c.cam = mk(p->cam_pos[0], p->cam_pos[1], p->cam_pos[2]);
    c.bias = p->bias;
    c.shadow_len = p->shadow_len;
    c.ao_len = p->ao_len;
    c.spec_len = p->spec_len;
    c.default_rough = p->default_rough;
    c.n_shadow = p->n_shadow;
    c.n_ao = p->n_ao;
    c.n_spec = p->n_spec;
    c.seed_h = pcg(p->seed);
    unsigned b = grid_blocks(ctx, gb->npix, 128, 16);
    if (out->records)
        k_occlusion<true><<<b, 128, 0, s>>>(v, gb->pos, gb->nrm, gb->rough, gb->npix, c, out->shadow, out->ao,
                                            out->ao_vis, out->spec, out->spec_t, out->records);
    else
        k_occlusion<false><<<b, 128, 0, s>>>(v, gb->pos, gb->nrm, gb->rough, gb->npix, c, out->shadow, out->ao,
                                             out->ao_vis, out->spec, out->spec_t, nullptr);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

// SUN_DIR = normalize(vec3(0.3,0.4,0.5)) (LightAmbient.frag:15), glm's form
static f3 sun_dir() {
    float x = 0.3f, y = 0.4f, z = 0.5f;
    float d = x * x + y * y;
    d = d + z * z;
    float r = 1.0f / sqrtf(d);
    return mk(x * r, y * r, z * r);
}

vxl_status launch_light_ambient(vxl_ctx* ctx, const vxl_grid* g, const float* wcp, const float* nrm,
                                const float* depth, const float* noise, int64_t npix, float* shadow, float* irr,
                                vxl_ray_record* rec, cudaStream_t s) {
    if (npix <= 0) return VXL_OK;
    GridView v = view_of(g);
    k_light_ambient<<<grid_blocks(ctx, npix, 128, 16), 128, 0, s>>>(v, wcp, nrm, depth, (const float4*)noise, npix,
                                                                    sun_dir(), shadow, irr, rec);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_light_reflection(vxl_ctx* ctx, const vxl_grid* g, const float* wcp, const float* nrm,
                                   const float* view_r, const float* rough, const float* noise, int64_t npix,
                                   float* t, vxl_ray_record* rec, cudaStream_t s) {
    if (npix <= 0) return VXL_OK;
    GridView v = view_of(g);
    k_light_reflection<<<grid_blocks(ctx, npix, 128, 16), 128, 0, s>>>(v, wcp, nrm, view_r, rough,
                                                                       (const float4*)noise, npix, t, rec);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_light_point(vxl_ctx* ctx, const vxl_grid* g, const float* wpos, const float* nrm,
                              const float* noise, int64_t npix, const float lp[3], float range, int spot,
                              float* shadow, vxl_ray_record* rec, cudaStream_t s) {
    if (npix <= 0) return VXL_OK;
    GridView v = view_of(g);
    k_light_point<<<grid_blocks(ctx, npix, 128, 16), 128, 0, s>>>(v, wpos, nrm, (const float4*)noise, npix,
                                                                  mk(lp[0], lp[1], lp[2]), range, spot, shadow, rec);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_light_points(vxl_ctx* ctx, const vxl_grid* g, const float* wpos, const float* nrm,
                               const float* noise, int64_t npix, const vxl_light* lights, int nlights,
                               unsigned long long* lit, unsigned long long* in_range, cudaStream_t s) {
    if (npix <= 0) return VXL_OK;
    LightTable T;
    T.n = nlights > 0 ? nlights : 0;
    for (int l = 0; l < T.n; l++) {
        T.l[l].pos = mk(lights[l].pos[0], lights[l].pos[1], lights[l].pos[2]);
        T.l[l].range = lights[l].range;
        T.l[l].spot = lights[l].spot ? 1 : 0;
    }
    // light grid over the box of every light's sphere (off when a light's
    // position or range is not finite)
    constexpr int kCells = kLightCells * kLightCells * kLightCells;
    LightGrid LG{mk(0.0f, 0.0f, 0.0f), 1.0f, 1.0f, 0.0f, T.n > 0 ? 1 : 0};
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, maxabs = 0.0f;
    for (int l = 0; l < T.n; l++) {
        const float r = std::fabs(lights[l].range);
        for (int a = 0; a < 3; a++) {
            if (!std::isfinite(lights[l].pos[a]) || !std::isfinite(r)) LG.on = 0;
            lo[a] = std::min(lo[a], lights[l].pos[a] - r);
            hi[a] = std::max(hi[a], lights[l].pos[a] + r);
            maxabs = std::max(maxabs, std::fabs(lights[l].pos[a]) + r);
        }
    }
    if (LG.on) {
        LG.slack = 1e-4f + maxabs * 4e-7f;
        float ext = 0.0f;
        for (int a = 0; a < 3; a++) ext = std::max(ext, hi[a] - lo[a]);
        ext = std::max(ext + 2.0f * LG.slack, 1e-3f) * 1.002f;
        LG.cell = ext / (float)kLightCells;
        LG.inv = 1.0f / LG.cell;
        LG.lo = mk(lo[0] - LG.slack - 0.001f * ext, lo[1] - LG.slack - 0.001f * ext, lo[2] - LG.slack - 0.001f * ext);
        if (!std::isfinite(LG.cell) || !std::isfinite(LG.inv) || !std::isfinite(maxabs)) LG.on = 0;
    }
    // pair list: two pairs per pixel (frames with more trace the rest in pass 1)
    const uint64_t cap = (uint64_t)std::max<int64_t>(2 * npix, 1 << 16);
    VXL_TRY(ctx_grow(&ctx->d_lpairs, &ctx->lpairs_bytes, (size_t)(cap + 1 + kCells) * sizeof(unsigned long long)));
    unsigned long long* npairs = (unsigned long long*)ctx->d_lpairs;
    unsigned long long* masks = npairs + 1;
    unsigned long long* pairs = masks + kCells;
    VXL_TRY_CUDA(cudaMemsetAsync(npairs, 0, sizeof(unsigned long long), s));
    GridView v = view_of(g);
    if (LG.on) {
        k_light_grid<<<(kCells + 255) / 256, 256, 0, s>>>(T, LG, masks);
        ctx->launches++;
    }
    const int64_t bx = std::min<int64_t>((npix + 255) / 256, (int64_t)ctx->sm_count * 8);
    k_light_points<<<(unsigned)bx, 256, 0, s>>>(v, wpos, nrm, (const float4*)noise, npix, T, LG, masks, lit, in_range,
                                                pairs, npairs, cap);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    if (T.n > 0) {
        k_light_pairs<<<(unsigned)ctx->sm_count * 8, 256, 0, s>>>(v, wpos, nrm, (const float4*)noise, T, pairs, npairs,
                                                                  cap, lit);
        ctx->launches++;
        VXL_TRY_CUDA(cudaGetLastError());
    }
    return VXL_OK;
}

}  // namespace vxl
