// occlusion.cu — DDA-mode occlusion pass (vxl_trace_occlusion) and its
// batched form (vxl_batch_*): persistent, warp-pooled.
//
// Each warp repeatedly takes `grab` tiles of TP pixels from a global counter
// (one counter for a whole batch of scenes: work stealing across scenes):
//  A. Generation: the warp's lanes build every ray of the tile (shadow, AO,
//     spec; same generator and arithmetic as the per-pixel reference kernel)
//     and store each ray's DDA start state (cell, t_max, t_delta, signs) as a
//     32-byte slot in shared memory, compacted so live rays are contiguous.
//     All lanes run the same generator code.
//  B. Traversal: each lane takes the next slot whenever its ray ends, so the
//     warp stays full while the pool lasts (rays end after very different
//     numbers of steps). A lane runs up to KSTEP DDA iterations between refills.
//  C. Reduction: one lane per pixel folds the ray results in the fixed order
//     shadow, AO 0..n-1, spec 0..n-1, so outputs are bit-identical to the
//     sequential per-pixel evaluation.
// A tile is either a run of TP consecutive pixels or, when the image width is
// known, a tile_w x (TP / tile_w) block of the image.
#include "occl_common.cuh"

namespace vxl {

// Phases A-C for one tile of one scene.
// HIT_T: the single-scene form: write a ray's t for hits only (the fold reads
// no other), step under one counter, and run a warp's KSTEP steps unrolled
// without the bounds test and the counter where none of its lanes can reach
// the bounds or the 256-step cap in them; the batched kernel keeps writing
// every t, two counters and both tests at every step, which its register
// allocation prefers
template <int TP, int KSTEP, bool LEAP, bool RECORDS, bool HIT_T = false, bool CACHE = true, bool CLEAR = false>
__device__ __forceinline__ void process_tile(const SceneDesc& S, const GridView& g, int64_t tile, PSlot* slots,
                                             float* res_t, uint32_t* res_hit, int lane) {
    constexpr int LPP = 32 / TP;  // lanes per pixel during generation
    const TraceConstsP& c = S.c;
    const int R = c.R;
    const unsigned ux = g.ux, uy = g.uy, uz = g.uz;

    // ---------------------------------------------------------- A
    const int p = lane % TP;
    int64_t gpix;
    const bool inimg = tile_pixel<TP>(S, tile, p, &gpix);
    f3 P = mk(0.0f, 0.0f, 0.0f), N = mk(0.0f, 0.0f, 0.0f);
    float ro = c.default_rough;
    if (inimg) {
        P = ld3(S.pos + 3 * gpix);
        N = ld3(S.nrm + 3 * gpix);
        if (S.rough) ro = S.rough[gpix];
    }
    const bool sky = !inimg || (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f);
    const uint32_t hpix = pcg(c.seed_h + ((uint32_t)gpix + S.pix_base));  // rand01's per-pixel hash
    const f3 O = add(P, mul(N, c.bias));
    f3 T, B;
    tangent_frame(N, &T, &B);
    for (int k = lane; k < R; k += 32) res_hit[k] = 0u;
    int live = 0;
    const int rounds = (R + LPP - 1) / LPP;
    for (int j = 0; j < rounds; j++) {
        // generation (= dispatch) order: spec rays first, then shadow, then
        // AO, so the longest rays start early and the pool drains on short ones
        const int kk = j * LPP + lane / TP;
        const int k = !c.spec_first ? kk : (kk < c.n_spec ? c.n_shadow + c.n_ao + kk : kk - c.n_spec);
        bool is_live = false;
        PSlot sl;
        if (kk < R && !sky) {
            const f3 d = gen_dir(c, k, hpix, P, N, T, B, ro);
            const float maxt = kind_maxt(c, k);
            int meta = (p << 4) | (k << 9);
            Hit h0{0, 0, 0, 0.0f, 0, VXL_RF_EXIT_BOUNDS};
            bool born_done = false;
            if (!ray_domain_ok(O, d)) {
                born_done = true;
            } else if (!dir_fast_ok(d)) {
                is_live = true;
                sl.c01 = 0;
                sl.c2m = (meta | kMetaLit) << 16;
                sl.a0 = O.x; sl.a1 = O.y; sl.a2 = O.z;
                sl.b0 = d.x; sl.b1 = d.y; sl.b2 = d.z;
            } else {
                DState s;
                dda_init(s, O, d, maxt);
                if ((unsigned)s.cx > ux || (unsigned)s.cy > uy || (unsigned)s.cz > uz) {
                    born_done = true;  // origin cell out of bounds: the first test exits (Light.frag:53)
                    h0 = Hit{s.cx, s.cy, s.cz, 0.0f, 0, VXL_RF_EXIT_BOUNDS};
                } else {
                    is_live = true;
                    meta |= (s.sx < 0 ? 1 : 0) | (s.sy < 0 ? 2 : 0) | (s.sz < 0 ? 4 : 0);
                    if (LEAP && !RECORDS && leap_allowed(d, maxt)) meta |= kMetaLeap;
                    sl.c01 = (s.cx & 0xffff) | (s.cy << 16);
                    sl.c2m = (s.cz & 0xffff) | (meta << 16);
                    sl.a0 = s.tx; sl.a1 = s.ty; sl.a2 = s.tz;
                    sl.b0 = s.tdx; sl.b1 = s.tdy; sl.b2 = s.tdz;
                }
            }
            if (born_done) {
                res_t[k * TP + p] = h0.t;
                if (RECORDS) store_record(S.rec + gpix * R + k, h0);
            }
        } else if (kk < R && RECORDS && inimg) {
            Hit z{0, 0, 0, 0.0f, 0, 0};
            store_record(S.rec + gpix * R + k, z);
        }
        const unsigned lv = __ballot_sync(0xffffffffu, is_live);
        if (is_live) slots[live + __popc(lv & lanes_below())] = sl;
        live += __popc(lv);
    }
    __syncwarp();

    // ---------------------------------------------------------- B
    int base = 0;
    bool busy = false;  // the lane holds a ray
    bool retired = false;
    int next_clear = 0;  // CLEAR: step count at which the lane next tries to prove its path empty
    DState s;
    int meta = 0;
    for (;;) {
        const bool need = !busy && !retired;
        const unsigned nm = __ballot_sync(0xffffffffu, need);
        if (nm) {
            if (need) {
                const int at = base + __popc(nm & lanes_below());
                if (at < live) {
                    const PSlot sl = slots[at];
                    meta = (unsigned)sl.c2m >> 16;
                    const int k = (meta >> 9) & 31;
                    const float maxt = kind_maxt(c, k);
                    if (meta & kMetaLit) {
                        const Hit h = dda_literal(g, mk(sl.a0, sl.a1, sl.a2), mk(sl.b0, sl.b1, sl.b2), maxt);
                        const int pp = (meta >> 4) & 31;
                        if (!HIT_T || (h.flags & VXL_RF_HIT)) res_t[k * TP + pp] = h.t;
                        if (h.flags & VXL_RF_HIT) atomicOr(&res_hit[k], 1u << pp);
                        if (RECORDS) {
                            int64_t gp;
                            tile_pixel<TP>(S, tile, pp, &gp);
                            store_record(S.rec + gp * R + k, h);
                        }
                    } else {
                        busy = true;
                        s.cx = lo16(sl.c01);
                        s.cy = hi16(sl.c01);
                        s.cz = lo16(sl.c2m);
                        s.tx = sl.a0; s.ty = sl.a1; s.tz = sl.a2;
                        s.tdx = sl.b0; s.tdy = sl.b1; s.tdz = sl.b2;
                        s.sx = (meta & 1) ? -1 : 1;
                        s.sy = (meta & 2) ? -1 : 1;
                        s.sz = (meta & 4) ? -1 : 1;
                        s.maxt = maxt;
                        s.tot = 0.0f;
                        s.n = 0;
                        s.leap = (meta & kMetaLeap) != 0;
                        s.wcur = 0xffffffffu;
                        s.word = 0;
                        next_clear = KSTEP;
                    }
                } else {
                    retired = true;
                }
            }
            base += __popc(nm);
        }
        if (!__any_sync(0xffffffffu, busy) && base >= live) break;
        if (CLEAR && busy && s.n >= next_clear) {
            // a ray whose remaining path is provably empty is a miss: it ends here
            next_clear = s.n + 4 * KSTEP;
            // (the cell may be one step out of bounds, which the DDA's next test ends)
            if ((unsigned)s.cx <= g.ux && (unsigned)s.cy <= g.uy && (unsigned)s.cz <= g.uz &&
                !map_bit(S.cm.c1, s.cx >> 3, s.cy >> 3, s.cz >> 3, S.cm.tx, S.cm.ty) && path_clear(S.cm, s))
                busy = false;
        }
        if (busy) {
            Hit h;
            const int f = dda_run<LEAP, CACHE, HIT_T, HIT_T>(g, s, h, KSTEP);
            if (f) {
                const int k = (meta >> 9) & 31, pp = (meta >> 4) & 31;
                if (!HIT_T || (f & VXL_RF_HIT)) res_t[k * TP + pp] = h.t;
                if (f & VXL_RF_HIT) atomicOr(&res_hit[k], 1u << pp);
                if (RECORDS) {
                    int64_t gp;
                    tile_pixel<TP>(S, tile, pp, &gp);
                    store_record(S.rec + gp * R + k, h);
                }
                busy = false;
            }
        }
    }
    __syncwarp();

    // ---------------------------------------------------------- C
    if (lane < TP && inimg) {
        float sh = 1.0f, ao = 1.0f, vis = 1.0f, sp = 1.0f, st = c.spec_len;
        if (!sky) {
            int k = 0;
            if (c.n_shadow > 0) {
                sh = ((res_hit[0] >> p) & 1u) ? 0.0f : 1.0f;
                k = 1;
            }
            float acc = 0.0f, v = 0.0f;
            for (int j = 0; j < c.n_ao; j++, k++) {
                const bool hit = (res_hit[k] >> p) & 1u;
                const float t = res_t[k * TP + p];
                float tt = hit ? (t < c.ao_len ? t : c.ao_len) : c.ao_len;
                float q = tt / c.ao_len;
                acc += q * q;
                v += hit ? 0.0f : 1.0f;
            }
            if (c.n_ao > 0) {
                ao = acc / (float)c.n_ao;
                vis = v / (float)c.n_ao;
            }
            if (c.n_spec > 0) {
                float spa = 0.0f, sta = 0.0f;
                for (int j = 0; j < c.n_spec; j++, k++) {
                    const bool hit = (res_hit[k] >> p) & 1u;
                    spa += hit ? 0.0f : 1.0f;
                    sta += hit ? res_t[k * TP + p] : c.spec_len;
                }
                sp = spa / (float)c.n_spec;
                st = sta / (float)c.n_spec;
            }
        }
        if (S.o_shadow) S.o_shadow[gpix] = sh;
        if (S.o_ao) S.o_ao[gpix] = ao;
        if (S.o_vis) S.o_vis[gpix] = vis;
        if (S.o_spec) S.o_spec[gpix] = sp;
        if (S.o_spec_t) S.o_spec_t[gpix] = st;
    }
    __syncwarp();
}

#ifndef VXL_POOL_MIN_BLOCKS
#define VXL_POOL_MIN_BLOCKS 8  // 8 blocks of 4 warps: 64 registers per thread
#endif

// one scene; its descriptor lives in kernel parameter space
template <int TP, int KSTEP, bool LEAP, bool RECORDS, bool CACHE = true, bool CLEAR = false>
__global__ void __launch_bounds__(128, VXL_POOL_MIN_BLOCKS) k_occl_pool(const SceneDesc S, unsigned long long* __restrict__ counter,
                                                                        int grab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * pool_bytes(TP, S.c.R);
    PSlot* slots = reinterpret_cast<PSlot*>(wbase);
    float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * S.c.R * sizeof(PSlot));
    uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * S.c.R * (sizeof(PSlot) + sizeof(float)));
    const GridView g = S.g;
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= S.ntiles) break;
        for (int k = 0; k < grab && t0 + k < S.ntiles; k++)
            process_tile<TP, KSTEP, LEAP, RECORDS, !RECORDS, CACHE, CLEAR>(S, g, t0 + k, slots, res_t, res_hit, lane);
    }
}

// many scenes, one counter over all their tiles (work stealing across scenes);
// tiles are numbered scene after scene, table[i].tile_begin ascending
template <int TP, int KSTEP, bool LEAP, bool CACHE = true>
__global__ void __launch_bounds__(128, VXL_POOL_MIN_BLOCKS) k_occl_batch(const SceneDesc* __restrict__ table,
                                                                         int nscenes, int64_t total_tiles,
                                                                         int max_r, unsigned long long* __restrict__ counter,
                                                                         int grab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * pool_bytes(TP, max_r);
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= total_tiles) break;
        for (int k = 0; k < grab && t0 + k < total_tiles; k++) {
            const int64_t t = t0 + k;
            int lo = 0, hi = nscenes - 1;  // last scene with tile_begin <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (table[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
            }
            const SceneDesc& S = table[lo];
            const int R = S.c.R;
            PSlot* slots = reinterpret_cast<PSlot*>(wbase);
            float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * R * sizeof(PSlot));
            uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * R * (sizeof(PSlot) + sizeof(float)));
            const GridView g = S.g;
            process_tile<TP, KSTEP, LEAP, false, false, CACHE>(S, g, t - S.tile_begin, slots, res_t, res_hit, lane);
        }
    }
}

// ---------------------------------------------------------------- host side
TraceConstsP consts_of(const vxl_trace_params* p, const vxl_tuning& tune) {
    TraceConstsP c;
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
    c.R = p->n_shadow + p->n_ao + p->n_spec;
    c.seed_h = pcg(p->seed);
    c.spec_first = tune.order == 1;
    return c;
}

// scene descriptor and its tile count for the given tile size / shape
SceneDesc scene_of(const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p, const vxl_outputs* o,
                          const vxl_tuning& tune) {
    SceneDesc S;
    S.g = view_of(g);
    S.cm = ClearMaps{g->clear1, g->clear2, g->tx, g->ty, g->tz, g->sx2, g->sy2};
    S.pos = gb->pos;
    S.nrm = gb->nrm;
    S.rough = gb->rough;
    S.o_shadow = o->shadow;
    S.o_ao = o->ao;
    S.o_vis = o->ao_vis;
    S.o_spec = o->spec;
    S.o_spec_t = o->spec_t;
    S.rec = o->records;
    S.npix = gb->npix;
    S.tile_begin = 0;
    S.pix_base = 0;
    const int TP = tune.tile_px;
    S.tile_w = TP;
    S.width = S.height = 0;
    if (tune.tile_w > 0 && tune.tile_w < TP && gb->width > 0 && gb->height > 0 &&
        (int64_t)gb->width * gb->height == gb->npix) {
        S.tile_w = tune.tile_w;
        S.width = gb->width;
        S.height = gb->height;
        const int th = TP / tune.tile_w;
        S.ntiles = (int64_t)((gb->width + tune.tile_w - 1) / tune.tile_w) * ((gb->height + th - 1) / th);
    } else {
        S.ntiles = (gb->npix + TP - 1) / TP;
    }
    S.c = consts_of(p, tune);
    return S;
}

template <typename K>
static vxl_status blocks_for_kernel(vxl_ctx* ctx, K kern, size_t smem, int* blocks_per_sm) {
    VXL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VXL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kern, 128, smem));
    if (*blocks_per_sm < 1)
        return fail(VXL_ERR_NOT_SUPPORTED, "occlusion pool: %zu bytes of shared memory per block", smem);
    return VXL_OK;
}

template <int TP, int KSTEP, bool LEAP, bool REC, bool CACHE = true, bool CLEAR = false>
static vxl_status launch_pool_t(vxl_ctx* ctx, const SceneDesc& S, unsigned long long* counter, int grab,
                                cudaStream_t s) {
    const size_t smem = pool_bytes(TP, S.c.R) * 4;
    auto kern = k_occl_pool<TP, KSTEP, LEAP, REC, CACHE, CLEAR>;
    int per_sm = 0;
    VXL_TRY(blocks_for_kernel(ctx, kern, smem, &per_sm));
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (S.ntiles + grab - 1) / grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(S, counter, grab);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

template <int TP, bool LEAP, bool CACHE, bool CLEAR = false>
static vxl_status launch_pool_k(vxl_ctx* ctx, const SceneDesc& S, unsigned long long* counter, const vxl_tuning& t,
                                cudaStream_t s) {
    switch (t.kstep) {
        case 1: return launch_pool_t<TP, 1, LEAP, false, CACHE, CLEAR>(ctx, S, counter, t.grab, s);
        case 2: return launch_pool_t<TP, 2, LEAP, false, CACHE, CLEAR>(ctx, S, counter, t.grab, s);
        case 4: return launch_pool_t<TP, 4, LEAP, false, CACHE, CLEAR>(ctx, S, counter, t.grab, s);
        default: return launch_pool_t<TP, 8, LEAP, false, CACHE, CLEAR>(ctx, S, counter, t.grab, s);
    }
}

// Grids up to this many bytes of brick words stay in L2 while a frame is
// traced: the traversal then reads the brick word at every step rather than
// caching it per ray (measured on GB300: +1.8% on a 16 MiB grid, -14% on a
// 1 GiB one)
constexpr size_t kStepLoadMaxBytes = (size_t)64 << 20;

bool occl_pool_supported(const vxl_grid* g, const vxl_trace_params* p) {
    int R = p->n_shadow + p->n_ao + p->n_spec;
    // 16-bit packed cells hold [-1, n+2]
    return R >= 1 && R <= kPoolMaxR && g->nx <= 32760 && g->ny <= 32760 && g->nz <= 32760;
}

// the exact-step kernels here run 16- or 32-pixel tiles (8-pixel tiles are
// chosen below for many rays per pixel); an 8-pixel tuning runs as 16
static vxl_tuning pool_tuning(const vxl_tuning& t) {
    vxl_tuning r = t;
    if (r.kstep == 16) r.kstep = 8;  // 16-iteration batches exist in the trace-layout kernel only
    if (r.tile_px == 8) {
        r.tile_px = 16;
        if (r.tile_w == 8) r.tile_w = 16;
    }
    return r;
}

vxl_status launch_trace_occlusion_pool(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb,
                                       const vxl_trace_params* p, const vxl_outputs* out,
                                       unsigned long long* d_counter, const vxl_tuning& tune_in, cudaStream_t s,
                                       uint32_t pix_base) {
    if (occl_lean_supported(g, out, tune_in))
        return launch_trace_occlusion_lean(ctx, g, gb, p, out, d_counter, tune_in, s, pix_base);
    const vxl_tuning tune = pool_tuning(tune_in);
    // Many rays per pixel: the 16-pixel pool's shared memory would hold the SM
    // below the 8 blocks its registers allow, so such frames run 8-pixel tiles
    // (runs of pixels) in the exact-step kernel.
    const int R = p->n_shadow + p->n_ao + p->n_spec;
    if (!out->records && tune.leap != 1 && tune.tile_px == 16 && tune.kstep == 8 &&
        (pool_bytes(16, R) * 4 + 1024) * VXL_POOL_MIN_BLOCKS > (size_t)ctx->smem_per_sm) {
        vxl_tuning t8 = tune;
        t8.tile_px = 8;
        t8.tile_w = 8;
        SceneDesc S8 = scene_of(g, gb, p, out, t8);
        S8.pix_base = pix_base;
        VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
        const bool cache8 = g->nwords * sizeof(uint64_t) > kStepLoadMaxBytes;
        if (cache8 && g->clear1 && tune.leap == 3) {
            // grids beyond L2: rays prove their remaining path empty on the two-level map
            VXL_TRY(launch_build_clear_maps(g, s));
            return launch_pool_t<8, 8, false, false, true, true>(ctx, S8, d_counter, t8.grab, s);
        }
        if (cache8) return launch_pool_t<8, 8, false, false, true>(ctx, S8, d_counter, t8.grab, s);
        return launch_pool_t<8, 8, false, false, false>(ctx, S8, d_counter, t8.grab, s);
    }
    SceneDesc S = scene_of(g, gb, p, out, tune);
    S.pix_base = pix_base;
    VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
    // per-ray records need the exact iteration count: no leaps there
    if (out->records) {
        if (tune.tile_px == 16) return launch_pool_t<16, 4, false, true>(ctx, S, d_counter, tune.grab, s);
        return launch_pool_t<32, 4, false, true>(ctx, S, d_counter, tune.grab, s);
    }
    if (tune.leap == 1) {
        if (tune.tile_px == 16) return launch_pool_k<16, true, true>(ctx, S, d_counter, tune, s);
        return launch_pool_k<32, true, true>(ctx, S, d_counter, tune, s);
    }
    const bool cache = g->nwords * sizeof(uint64_t) > kStepLoadMaxBytes;
    if (cache && g->clear1 && tune.leap == 3 && tune.tile_px == 16) {
        VXL_TRY(launch_build_clear_maps(g, s));
        return launch_pool_k<16, false, true, true>(ctx, S, d_counter, tune, s);
    }
    if (tune.tile_px == 16) {
        if (cache) return launch_pool_k<16, false, true>(ctx, S, d_counter, tune, s);
        return launch_pool_k<16, false, false>(ctx, S, d_counter, tune, s);
    }
    if (cache) return launch_pool_k<32, false, true>(ctx, S, d_counter, tune, s);
    return launch_pool_k<32, false, false>(ctx, S, d_counter, tune, s);
}

// ------------------------------------------------------------------ batch
struct BatchPlan {
    SceneDesc* d_table;
    int n;
    int max_r;
    int64_t total_tiles;
    vxl_tuning tune;
    unsigned long long* counter;
    bool cache;  // some grid of the batch is larger than kStepLoadMaxBytes
};

template <int TP, int KSTEP, bool CACHE>
static vxl_status launch_batch_t(vxl_ctx* ctx, const BatchPlan& b, cudaStream_t s) {
    const size_t smem = pool_bytes(TP, b.max_r) * 4;
    auto kern = k_occl_batch<TP, KSTEP, false, CACHE>;
    int per_sm = 0;
    VXL_TRY(blocks_for_kernel(ctx, kern, smem, &per_sm));
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (b.total_tiles + b.tune.grab - 1) / b.tune.grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(b.d_table, b.n, b.total_tiles, b.max_r, b.counter, b.tune.grab);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

template <int TP, bool CACHE>
static vxl_status launch_batch_k(vxl_ctx* ctx, const BatchPlan& b, cudaStream_t s) {
    switch (b.tune.kstep) {
        case 1: return launch_batch_t<TP, 1, CACHE>(ctx, b, s);
        case 2: return launch_batch_t<TP, 2, CACHE>(ctx, b, s);
        case 4: return launch_batch_t<TP, 4, CACHE>(ctx, b, s);
        default: return launch_batch_t<TP, 8, CACHE>(ctx, b, s);
    }
}

size_t batch_desc_bytes() { return sizeof(SceneDesc); }

vxl_status batch_build_table(const vxl_batch_item* items, int n, const vxl_tuning& tune_in, void* h_table, int* max_r,
                             int64_t* total_tiles, int64_t* total_rays, size_t* max_grid_bytes) {
    const vxl_tuning tune = pool_tuning(tune_in);
    SceneDesc* t = (SceneDesc*)h_table;
    int64_t tiles = 0, rays = 0;
    int mr = 1;
    size_t gb = 0;
    for (int i = 0; i < n; i++) {
        gb = std::max(gb, items[i].grid->nwords * sizeof(uint64_t));
        t[i] = scene_of(items[i].grid, &items[i].gbuf, &items[i].params, &items[i].out, tune);
        t[i].tile_begin = tiles;
        tiles += t[i].ntiles;
        rays += items[i].gbuf.npix * t[i].c.R;
        if (t[i].c.R > mr) mr = t[i].c.R;
    }
    *max_r = mr;
    *total_tiles = tiles;
    *total_rays = rays;
    *max_grid_bytes = gb;
    return VXL_OK;
}

vxl_status launch_batch(vxl_ctx* ctx, void* d_table, int n, int max_r, int64_t total_tiles, const vxl_tuning& tune_in,
                        unsigned long long* d_counter, size_t max_grid_bytes, cudaStream_t s) {
    const vxl_tuning tune = pool_tuning(tune_in);
    BatchPlan b{(SceneDesc*)d_table, n, max_r, total_tiles, tune, d_counter, max_grid_bytes > kStepLoadMaxBytes};
    VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
    if (tune.tile_px == 16) return b.cache ? launch_batch_k<16, true>(ctx, b, s) : launch_batch_k<16, false>(ctx, b, s);
    return b.cache ? launch_batch_k<32, true>(ctx, b, s) : launch_batch_k<32, false>(ctx, b, s);
}

}  // namespace vxl
