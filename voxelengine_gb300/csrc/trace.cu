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

// Fused point / spot shadows: threads over (pixel, light) with the light as
// blockIdx.y, so a warp traces one light's rays from 32 neighbouring pixels.
// The ray of each pair is the one k_light_point traces for that light alone;
// the results are OR-ed into per-pixel 64-bit masks.
struct LightDev {
    f3 pos;
    float range;
    int spot;
};
__global__ void k_light_points(GridView g, const float* __restrict__ wpos, const float* __restrict__ nrm,
                               const float4* __restrict__ noise, int64_t npix, const LightDev* __restrict__ lights,
                               unsigned long long* __restrict__ lit, unsigned long long* __restrict__ in_range) {
    const int l = blockIdx.y;
    const LightDev Lt = lights[l];
    const unsigned long long bit = 1ull << l;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix;
         i += (int64_t)gridDim.x * blockDim.x) {
        const f3 worldPos = ld3(wpos + 3 * i);
        const f3 lightDir = sub(Lt.pos, worldPos);
        const float lightDistance = sqrtf(dot(lightDir, lightDir));
        if (lightDistance > Lt.range) continue;  // the light's pass discards this pixel
        const float4 nz = noise[i];
        const f3 normal = ld3(nrm + 3 * i);
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
        if (in_range) atomicOr(in_range + i, bit);
        if (!(h.t < hitDist)) atomicOr(lit + i, bit);
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
    if (occl_pool_supported(g, p))
        return launch_trace_occlusion_pool(ctx, g, gb, p, out, ctx_next_counter(ctx), ctx->tune, s);
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
    VXL_TRY_CUDA(cudaMemsetAsync(lit, 0, sizeof(unsigned long long) * (size_t)npix, s));
    if (in_range) VXL_TRY_CUDA(cudaMemsetAsync(in_range, 0, sizeof(unsigned long long) * (size_t)npix, s));
    if (npix <= 0 || nlights <= 0) return VXL_OK;
    LightDev h[64];
    for (int l = 0; l < nlights; l++) {
        h[l].pos = mk(lights[l].pos[0], lights[l].pos[1], lights[l].pos[2]);
        h[l].range = lights[l].range;
        h[l].spot = lights[l].spot ? 1 : 0;
    }
    void* p;
    VXL_TRY(ctx_scratch(ctx, sizeof(LightDev) * 64, &p));
    VXL_TRY_CUDA(cudaMemcpyAsync(p, h, sizeof(LightDev) * (size_t)nlights, cudaMemcpyHostToDevice, s));
    GridView v = view_of(g);
    int64_t bx = (npix + 127) / 128;
    const int64_t cap = (int64_t)ctx->sm_count * 16 * 4 / nlights + 1;
    if (bx > cap) bx = cap;
    dim3 grid((unsigned)bx, (unsigned)nlights);
    k_light_points<<<grid, 128, 0, s>>>(v, wpos, nrm, (const float4*)noise, npix, (const LightDev*)p, lit, in_range);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
