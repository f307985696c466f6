// occl_lean.cu — the DDA-mode occlusion pass (vxl_trace_occlusion without
// per-ray records) on the grid's trace layout.
//
// Same ray generator, dispatch order, warp pools and per-pixel fold as the
// kernels of occlusion.cu, so the outputs are bit-identical; what changes is
// the inner loop of raycastShadowVolume (Sources/Shaders/lib/Light.frag:50-75):
//  - The cell is held as a bit address A = ax + ay + az in the trace layout,
//    one term per axis (vxl_device.cuh, AxisCode). A step along an axis is an
//    add and a mask on that axis's term; the fetch is one 32-bit load and a
//    funnel shift.
//  - No bounds test: the trace layout's border cells (one cell outside the
//    DDA's inclusive bounds) read as set. A set cell is a hit unless it lies
//    outside [0, n+1] on some axis, which is the reference's bounds exit at
//    that same iteration (Light.frag:53).
//  - The `totalt < maxt` test of the loop (Light.frag:75) is taken out of the
//    loop body. Without exact ties, totalt of an iteration is the smallest
//    t_max component, which never decreases from one iteration to the next,
//    so the first iteration whose totalt reaches maxt is found later: at a set
//    cell (the previous iteration's totalt) and at the end of a batch of
//    KSTEP iterations. An iteration with an exact tie (totalt = the sum of the
//    tied components, which can exceed later ones) is tested at once. Steps a
//    lane takes past its ray's end only touch cells inside the border.
//  - The 256-iteration cap (Light.frag:75) is tested per batch: a batch that
//    might reach it runs the iterations with the cap and maxt tests in place.
#include <algorithm>
#include <cstring>

#include "occl_common.cuh"

namespace vxl {

struct LeanGrid {
    const uint32_t* __restrict__ w;  // trace layout, as 32-bit halves of the brick words
    uint32_t field[3];                // bits of A owned by each axis
    uint32_t keep[3];                 // mask after a step (clears the axis's gap)
    uint32_t inc[3];                  // +1 step increment; a -1 step adds -unit
    uint32_t unit[3];
    uint32_t lo[3], span[3];          // axis term of shifted coordinate 4 and the span up to n+5
    uint32_t one, two27;              // 1 and 2^27 as data: multiply-adds by them stay multiply-adds
    int hs[3];                        // shift of each axis's brick index
};

struct __align__(16) LeanScene {
    SceneDesc S;
    LeanGrid L;
};

LeanGrid lean_grid_of(const vxl_grid* g) {
    LeanGrid L;
    L.w = reinterpret_cast<const uint32_t*>(g->tl_words);
    const int n[3] = {g->nx, g->ny, g->nz};
    for (int a = 0; a < 3; a++) {
        const AxisCode c = axis_code(a, g->tl_lbx, g->tl_lby);
        L.field[a] = c.field;
        L.keep[a] = c.keep;
        L.inc[a] = c.inc;
        L.unit[a] = c.unit;
        L.hs[a] = c.hi_shift;
        // interior cells 0 .. n+1 are shifted cells 4 .. n+5
        L.lo[a] = axis_term(c, 4);
        L.span[a] = axis_term(c, n[a] + 5) - L.lo[a];
    }
    L.one = 1u;
    L.two27 = 1u << 27;
    return L;
}

// One iteration of Light.frag:50-75 on the trace layout. Returns 0 while the
// ray goes on, 1 for a hit (t in *ht), 2 when the ray ends without one.
// `tot` is the previous iteration's totalt (-inf before the first).
__device__ __forceinline__ int lean_step(const LeanGrid& L, uint32_t& ax, uint32_t& ay, uint32_t& az, float& tx,
                                         float& ty, float& tz, float tdx, float tdy, float tdz, uint32_t kx,
                                         uint32_t ky, uint32_t kz, float maxt, float& tot, float* ht) {
    const uint32_t a = ax + ay + az;  // the terms' bit fields do not overlap
    const uint32_t w = __ldg(L.w + (a >> 5));
    const float m = fminf(fminf(tx, ty), tz);
    // select = step(t.xyz, t.zxy) * step(t.xyz, t.yzx): the components equal to the minimum
    const bool bx = tx == m, by = ty == m, bz = tz == m;
    const bool tie = (bx && (by || bz)) || (by && bz);
    if (__funnelshift_r(w, w, a) & 1u) {
        if (!(tot < maxt)) return 2;  // the loop had ended before this iteration
        // a border cell: the bounds test of this iteration fails (Light.frag:53)
        if (ax - L.lo[0] > L.span[0] || ay - L.lo[1] > L.span[1] || az - L.lo[2] > L.span[2]) return 2;
        // dot(t_max, select); +0.0f turns a -0 minimum into the +0 the dot product gives
        float best = m + 0.0f;
        if (tie) {
            best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
            best = best + (bz ? tz : 0.0f);
        }
        *ht = best;
        return 1;
    }
    float best = m;
    if (tie) {
        best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
        best = best + (bz ? tz : 0.0f);
        if (!(best < maxt)) return 2;
    }
    if (bx) {
        ax = (ax + kx) & L.keep[0];
        tx = tx + tdx;
    }
    if (by) {
        ay = (ay + ky) & L.keep[1];
        ty = ty + tdy;
    }
    if (bz) {
        az = (az + kz) & L.keep[2];
        tz = tz + tdz;
    }
    tot = best;
    return 0;
}

// A set cell met by the hot form (lean_batch), with the state of its
// iteration: a hit (returns true, t in *t) unless the loop had already ended
// at the previous iteration (totalt >= maxt) or the cell lies on the border,
// i.e. the bounds test of this iteration fails (Light.frag:53).
__device__ __forceinline__ bool lean_set_cell(const LeanGrid& L, uint32_t ax, uint32_t ay, uint32_t az, float tx,
                                              float ty, float tz, float tot, float maxt, float* t) {
    if (!(tot < maxt)) return false;
    if (ax - L.lo[0] > L.span[0] || ay - L.lo[1] > L.span[1] || az - L.lo[2] > L.span[2]) return false;
    const float m = fminf(fminf(tx, ty), tz);
    const bool bx = tx == m, by = ty == m, bz = tz == m;
    // dot(t_max, select); +0.0f turns a -0 minimum into the +0 the dot product gives
    float best = m + 0.0f;
    if ((bx && (by || bz)) || (by && bz)) {
        best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
        best = best + (bz ? tz : 0.0f);
    }
    *t = best;
    return true;
}

// The hot form: KSTEP iterations of Light.frag:50-75 as one block of
// hand-written PTX, for batches that cannot reach the 256-iteration cap.
// The traversal is bound by the SM's ALU pipe (compares, min/max, logic,
// shifts, predicate and move operations issue there at half the FMA pipe's
// rate), so the integer adds and the address shift are multiply-adds by a
// register holding 1 and a high multiply by 2^27, which run on the FMA pipe,
// and the per-axis updates run under predicates. Each iteration:
//   a = ax + ay + az; the cell's bit set -> leave with stop = 1, the state of
//   this iteration kept (lean_set_cell classifies it);
//   m = min(t); select = "t_i == m" (step(t.xyz, t.zxy) * step(t.xyz, t.yzx));
//   the selected axes advance; totalt = m, or on an exact tie (two or more
//   selected) the sum of the tied components, all equal to m, which is
//   tested against maxt at once in an out-of-line block (stop = 2 when
//   reached). After the last iteration stop = 0.
#define VXL_LEAN_IT(i)                     \
    "mad.lo.u32 a, %0, %16, %1;\n\t"       \
    "mad.lo.u32 a, %2, %16, a;\n\t"        \
    "mul.hi.u32 s, a, %17;\n\t"            \
    "mad.wide.u32 ad, s, 4, %18;\n\t"      \
    "ld.global.nc.u32 w, [ad];\n\t"        \
    "min.f32 m, %3, %4;\n\t"               \
    "min.f32 m, m, %5;\n\t"                \
    "setp.eq.f32 px, %3, m;\n\t"           \
    "setp.eq.f32 py, %4, m;\n\t"           \
    "setp.eq.f32 pz, %5, m;\n\t"           \
    "shf.r.wrap.b32 s, w, w, a;\n\t"       \
    "and.b32 s, s, 1;\n\t"                 \
    "setp.ne.u32 pb, s, 0;\n\t"            \
    "@pb bra VXL_SET;\n\t"                 \
    "@px mad.lo.u32 %0, %11, %16, %0;\n\t" \
    "@py mad.lo.u32 %1, %12, %16, %1;\n\t" \
    "@pz mad.lo.u32 %2, %13, %16, %2;\n\t" \
    "@px and.b32 %0, %0, 0xFFFFFFC3;\n\t"  \
    "@py and.b32 %1, %1, %14;\n\t"         \
    "@pz and.b32 %2, %2, %15;\n\t"         \
    "@px add.rn.f32 %3, %3, %8;\n\t"       \
    "@py add.rn.f32 %4, %4, %9;\n\t"       \
    "@pz add.rn.f32 %5, %5, %10;\n\t"      \
    "and.pred q, px, py;\n\t"              \
    "and.pred r, px, pz;\n\t"              \
    "or.pred q, q, r;\n\t"                 \
    "and.pred r, py, pz;\n\t"              \
    "or.pred q, q, r;\n\t"                 \
    "mov.f32 %6, m;\n\t"                   \
    "@q bra VXL_TIE" #i ";\n"              \
    "VXL_BACK" #i ":\n\t"
#define VXL_LEAN_TIE(i)                    \
    "VXL_TIE" #i ":\n\t"                   \
    "and.pred r, px, py;\n\t"              \
    "and.pred r, r, pz;\n\t"               \
    "add.rn.f32 b, m, m;\n\t"              \
    "@r add.rn.f32 b, b, m;\n\t"           \
    "@!r add.rn.f32 b, b, 0f00000000;\n\t" \
    "setp.lt.f32 pn, b, %19;\n\t"          \
    "@!pn bra VXL_END;\n\t"                \
    "mov.f32 %6, b;\n\t"                   \
    "bra VXL_BACK" #i ";\n"
#define VXL_LEAN_BLOCK(ITERS, TIES)                                                                      \
    asm volatile("{\n\t"                                                                                 \
                 ".reg .pred px, py, pz, pb, q, r, pn;\n\t"                                              \
                 ".reg .b32 a, s, w;\n\t"                                                                \
                 ".reg .b64 ad;\n\t"                                                                     \
                 ".reg .f32 m, b;\n\t" ITERS                                                             \
                 "mov.u32 %7, 0;\n\t"                                                                    \
                 "bra VXL_DONE;\n"                                                                       \
                 "VXL_SET:\n\t"                                                                          \
                 "mov.u32 %7, 1;\n\t"                                                                    \
                 "bra VXL_DONE;\n"                                                                       \
                 "VXL_END:\n\t"                                                                          \
                 "mov.u32 %7, 2;\n\t"                                                                    \
                 "bra VXL_DONE;\n" TIES "VXL_DONE:\n\t"                                                  \
                 "}"                                                                                     \
                 : "+r"(ax), "+r"(ay), "+r"(az), "+f"(tx), "+f"(ty), "+f"(tz), "+f"(tot), "=r"(stop)     \
                 : "f"(tdx), "f"(tdy), "f"(tdz), "r"(kx), "r"(ky), "r"(kz), "r"(keep_y), "r"(keep_z),      \
                   "r"(one), "r"(two27), "l"(w), "f"(maxt))
#define VXL_LEAN_IT4(o) VXL_LEAN_IT(o##0) VXL_LEAN_IT(o##1) VXL_LEAN_IT(o##2) VXL_LEAN_IT(o##3)
#define VXL_LEAN_TIE4(o) VXL_LEAN_TIE(o##0) VXL_LEAN_TIE(o##1) VXL_LEAN_TIE(o##2) VXL_LEAN_TIE(o##3)

template <int KSTEP>
__device__ __forceinline__ int lean_batch(const uint32_t* __restrict__ w, uint32_t& ax, uint32_t& ay, uint32_t& az,
                                          float& tx, float& ty, float& tz, float tdx, float tdy, float tdz,
                                          uint32_t kx, uint32_t ky, uint32_t kz, uint32_t keep_y, uint32_t keep_z,
                                          uint32_t one, uint32_t two27, float maxt, float& tot) {
    static_assert(KSTEP == 4 || KSTEP == 8 || KSTEP == 16, "batch of 4, 8 or 16 iterations");
    int stop;
    if (KSTEP == 4) VXL_LEAN_BLOCK(VXL_LEAN_IT4(1), VXL_LEAN_TIE4(1));
    if (KSTEP == 8) VXL_LEAN_BLOCK(VXL_LEAN_IT4(1) VXL_LEAN_IT4(2), VXL_LEAN_TIE4(1) VXL_LEAN_TIE4(2));
    if (KSTEP == 16)
        VXL_LEAN_BLOCK(VXL_LEAN_IT4(1) VXL_LEAN_IT4(2) VXL_LEAN_IT4(3) VXL_LEAN_IT4(4),
                       VXL_LEAN_TIE4(1) VXL_LEAN_TIE4(2) VXL_LEAN_TIE4(3) VXL_LEAN_TIE4(4));
    return stop;
}

#ifndef VXL_LEAN_MIN_BLOCKS
#define VXL_LEAN_MIN_BLOCKS 8
#endif

// One tile of TP pixels of one scene: generation into the warp's pool,
// traversal, fold (the phases of the pooled kernels in occlusion.cu). `one`
// and `two27` (1 and 2^27) come from a kernel parameter at a fixed offset, so
// the compiler can use them as constant operands rather than registers.
template <int TP, int KSTEP>
__device__ __forceinline__ void lean_tile(const SceneDesc& S, const LeanGrid& L, int64_t tile, PSlot* slots,
                                          float* res_t, uint32_t* res_hit, int lane, uint32_t one, uint32_t two27) {
    const TraceConstsP& c = S.c;
    const int R = c.R;
    const unsigned ux = S.g.ux, uy = S.g.uy, uz = S.g.uz;
    const uint32_t keep_y = L.keep[1], keep_z = L.keep[2];
    constexpr int LPP = 32 / TP;  // lanes per pixel during generation
    // ------------------------------------------------ A: generation
    const int p = lane % TP;
    int64_t gpix;
    const bool inimg = tile_pixel<TP>(S, tile, p, &gpix);
    f3 Pp = mk(0.0f, 0.0f, 0.0f), N = mk(0.0f, 0.0f, 0.0f);
    float ro = c.default_rough;
    if (inimg) {
        Pp = ld3(S.pos + 3 * gpix);
        N = ld3(S.nrm + 3 * gpix);
        if (S.rough) ro = S.rough[gpix];
    }
    const bool sky = !inimg || (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f);
    const uint32_t hpix = pcg(c.seed_h + ((uint32_t)gpix + S.pix_base));  // rand01's per-pixel hash
    const f3 O = add(Pp, mul(N, c.bias));
    f3 T, B;
    tangent_frame(N, &T, &B);
    for (int k = lane; k < R; k += 32) res_hit[k] = 0u;
    int live = 0, nlit = 0;
    const int rounds = (R + LPP - 1) / LPP;
    for (int j = 0; j < rounds; j++) {
        const int kk = j * LPP + lane / TP;
        const int k = !c.spec_first ? kk : (kk < c.n_spec ? c.n_shadow + c.n_ao + kk : kk - c.n_spec);
        bool is_live = false, is_lit = false;
        PSlot sl;
        if (kk < R && !sky) {
            const f3 d = gen_dir(c, k, hpix, Pp, N, T, B, ro);
            const float maxt = kind_maxt(c, k);
            const int meta = (p << 4) | (k << 9);
            if (!ray_domain_ok(O, d)) {
                // no traversal: a miss
            } else if (!dir_fast_ok(d)) {
                is_lit = true;
                sl.c01 = 0;
                sl.c2m = (meta | kMetaLit) << 16;
                sl.a0 = O.x; sl.a1 = O.y; sl.a2 = O.z;
                sl.b0 = d.x; sl.b1 = d.y; sl.b2 = d.z;
            } else {
                DState s;
                dda_init(s, O, d, maxt);
                // an origin cell outside the bounds ends the ray at the first test (Light.frag:53)
                if ((unsigned)s.cx <= ux && (unsigned)s.cy <= uy && (unsigned)s.cz <= uz) {
                    is_live = true;
                    const int sg = (s.sx < 0 ? 1 : 0) | (s.sy < 0 ? 2 : 0) | (s.sz < 0 ? 4 : 0);
                    const uint32_t xs = (uint32_t)(s.cx + 4), ys = (uint32_t)(s.cy + 4), zs = (uint32_t)(s.cz + 4);
                    sl.c01 = (int)((xs & 3u) | ((xs >> 2) << L.hs[0]) | ((ys & 3u) << 2) | ((ys >> 2) << L.hs[1]) |
                                   ((zs & 3u) << 4) | ((zs >> 2) << L.hs[2]));
                    sl.c2m = (meta | sg) << 16;
                    sl.a0 = s.tx; sl.a1 = s.ty; sl.a2 = s.tz;
                    sl.b0 = s.tdx; sl.b1 = s.tdy; sl.b2 = s.tdz;
                }
            }
        }
        const unsigned lv = __ballot_sync(0xffffffffu, is_live);
        if (is_live) slots[live + __popc(lv & lanes_below())] = sl;
        live += __popc(lv);
        // rays with a direction component below 1e-30 take the literal form of the DDA after the
        // traversal loop (no call inside it): their slots fill the pool from its top down
        const unsigned lm = __ballot_sync(0xffffffffu, is_lit);
        if (lm) {
            if (is_lit) slots[TP * R - 1 - (nlit + __popc(lm & lanes_below()))] = sl;
            nlit += __popc(lm);
        }
    }
    __syncwarp();

    // ------------------------------------------------- B: traversal
    int base = 0;
    bool busy = false, retired = false;
    uint32_t ax = 0, ay = 0, az = 0, kx = 0, ky = 0, kz = 0;
    float tx = 0.0f, ty = 0.0f, tz = 0.0f, tdx = 0.0f, tdy = 0.0f, tdz = 0.0f, maxt = 0.0f, tot = 0.0f;
    int n = 0, meta = 0;
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
                    maxt = kind_maxt(c, k);
                    {
                        busy = true;
                        const uint32_t A = (uint32_t)sl.c01;
                        ax = A & L.field[0];
                        ay = A & L.field[1];
                        az = A & L.field[2];
                        kx = (meta & 1) ? 0u - L.unit[0] : L.inc[0];
                        ky = (meta & 2) ? 0u - L.unit[1] : L.inc[1];
                        kz = (meta & 4) ? 0u - L.unit[2] : L.inc[2];
                        tx = sl.a0; ty = sl.a1; tz = sl.a2;
                        tdx = sl.b0; tdy = sl.b1; tdz = sl.b2;
                        tot = -INFINITY;
                        n = 0;
                    }
                } else {
                    retired = true;
                }
            }
            base += __popc(nm);
        }
        if (!__any_sync(0xffffffffu, busy) && base >= live) break;
        if (busy) {
            int res = 0;
            float ht = 0.0f;
            if (__all_sync(__activemask(), n + KSTEP <= 256)) {
                const int st = lean_batch<KSTEP>(L.w, ax, ay, az, tx, ty, tz, tdx, tdy, tdz, kx, ky, kz,
                                                 keep_y, keep_z, one, two27, maxt, tot);
                if (st == 1)
                    res = lean_set_cell(L, ax, ay, az, tx, ty, tz, tot, maxt, &ht) ? 1 : 2;
                else if (st == 2)
                    res = 2;
                else {
                    n += KSTEP;
                    if (!(tot < maxt)) res = 2;
                }
            } else {
                // the batch may reach the 256-iteration cap: test it, and maxt, at every iteration
                for (int it = 0; it < KSTEP; it++) {
                    if (n >= 256) {
                        res = 2;
                        break;
                    }
                    res = lean_step(L, ax, ay, az, tx, ty, tz, tdx, tdy, tdz, kx, ky, kz, maxt, tot, &ht);
                    if (res) break;
                    n++;
                    if (!(tot < maxt) || n >= 256) {
                        res = 2;
                        break;
                    }
                }
            }
            if (res) {
                if (res == 1) {
                    const int k = (meta >> 9) & 31, pp = (meta >> 4) & 31;
                    res_t[k * TP + pp] = ht;
                    atomicOr(&res_hit[k], 1u << pp);
                }
                busy = false;
            }
        }
    }
    for (int i = lane; i < nlit; i += 32) {
        const PSlot sl = slots[TP * R - 1 - i];
        const int m = (unsigned)sl.c2m >> 16, k = (m >> 9) & 31;
        const Hit h = dda_literal(S.g, mk(sl.a0, sl.a1, sl.a2), mk(sl.b0, sl.b1, sl.b2), kind_maxt(c, k));
        if (h.flags & VXL_RF_HIT) {
            const int pp = (m >> 4) & 31;
            res_t[k * TP + pp] = h.t;
            atomicOr(&res_hit[k], 1u << pp);
        }
    }
    __syncwarp();

    // ------------------------------------------------------ C: fold
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

// one scene; its descriptor lives in kernel parameter space
template <int TP, int KSTEP>
__global__ void __launch_bounds__(128, VXL_LEAN_MIN_BLOCKS) k_occl_lean(const __grid_constant__ LeanScene P,
                                                                        unsigned long long* __restrict__ counter,
                                                                        int grab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int R = P.S.c.R;
    unsigned char* wbase = smem + warp * pool_bytes(TP, R);
    PSlot* slots = reinterpret_cast<PSlot*>(wbase);
    float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * R * sizeof(PSlot));
    uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * R * (sizeof(PSlot) + sizeof(float)));
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= P.S.ntiles) break;
        for (int gi = 0; gi < grab && t0 + gi < P.S.ntiles; gi++)
            lean_tile<TP, KSTEP>(P.S, P.L, t0 + gi, slots, res_t, res_hit, lane, P.L.one, P.L.two27);
    }
}

// many scenes, one counter over all their tiles (work stealing across
// scenes); tiles are numbered scene after scene, table[i].S.tile_begin ascending
template <int TP, int KSTEP>
__global__ void __launch_bounds__(128, VXL_LEAN_MIN_BLOCKS) k_occl_lean_batch(const LeanScene* __restrict__ table,
                                                                              int nscenes, int64_t total_tiles,
                                                                              int max_r,
                                                                              unsigned long long* __restrict__ counter,
                                                                              int grab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * pool_bytes(TP, max_r);
    // each warp keeps the descriptor of the scene it works on in shared memory
    // (after the four pools): it changes only when a warp's tiles move on to
    // another scene, and the tile loop reads it many times
    LeanScene* desc = reinterpret_cast<LeanScene*>(smem + 4 * pool_bytes(TP, max_r)) + warp;
    int cur = -1;
    int64_t cur_begin = 0, cur_end = 0;
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= total_tiles) break;
        for (int gi = 0; gi < grab && t0 + gi < total_tiles; gi++) {
            const int64_t t = t0 + gi;
            if (t < cur_begin || t >= cur_end) {
                int lo = 0, hi = nscenes - 1;  // last scene with tile_begin <= t
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (table[mid].S.tile_begin <= t) lo = mid; else hi = mid - 1;
                }
                if (lo != cur) {
                    __syncwarp();
                    const uint32_t* src = reinterpret_cast<const uint32_t*>(table + lo);
                    uint32_t* dst = reinterpret_cast<uint32_t*>(desc);
                    for (int k = lane; k < (int)(sizeof(LeanScene) / 4); k += 32) dst[k] = src[k];
                    __syncwarp();
                    cur = lo;
                }
                cur_begin = desc->S.tile_begin;
                cur_end = cur_begin + desc->S.ntiles;
            }
            const int R = desc->S.c.R;
            PSlot* slots = reinterpret_cast<PSlot*>(wbase);
            float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * R * sizeof(PSlot));
            uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * R * (sizeof(PSlot) + sizeof(float)));
            lean_tile<TP, KSTEP>(desc->S, desc->L, t - cur_begin, slots, res_t, res_hit, lane, desc->L.one,
                                 desc->L.two27);
        }
    }
}

// A batch of up to kLeanBatchMax scenes passed by value as the kernel's
// parameters (32 KB of parameter space on this GPU): every warp then reads its
// scene's constants from the constant bank, as the single-scene kernel does.
constexpr int kLeanBatchMax = 64;
struct LeanBatchParams {
    LeanScene s[kLeanBatchMax];
};
static_assert(sizeof(LeanBatchParams) + 64 <= 32764, "the batch table fits the kernel parameter space");

// The batched kernel: on moving to another scene a warp copies that scene's
// descriptor from the parameter table into its slot of shared memory, and
// the tile code reads the descriptor there (4.5% faster on the 64-scene mix
// than reading the table at run-time offsets, which held the scene's
// constants in registers). 7 blocks per SM (72 registers): at 8 the loop
// spilled and ran 19% slower. The scene-independent constants 1 and 2^27 are
// separate parameters at fixed offsets (2% faster than reading them from the
// table).
#ifndef VXL_LEAN_BATCH_MIN_BLOCKS
#define VXL_LEAN_BATCH_MIN_BLOCKS 7
#endif

template <int TP, int KSTEP>
__global__ void __launch_bounds__(128, VXL_LEAN_BATCH_MIN_BLOCKS) k_occl_lean_batch_p(
    const __grid_constant__ LeanBatchParams T, int nscenes, int64_t total_tiles, int max_r,
    unsigned long long* __restrict__ counter, int grab, uint32_t one, uint32_t two27) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * pool_bytes(TP, max_r);
    LeanScene* desc = reinterpret_cast<LeanScene*>(smem + 4 * pool_bytes(TP, max_r)) + warp;
    int cur = -1;
    int64_t cur_begin = 0, cur_end = 0;
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= total_tiles) break;
        for (int gi = 0; gi < grab && t0 + gi < total_tiles; gi++) {
            const int64_t t = t0 + gi;
            if (t < cur_begin || t >= cur_end) {
                int lo = 0, hi = nscenes - 1;  // last scene with tile_begin <= t
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (T.s[mid].S.tile_begin <= t) lo = mid; else hi = mid - 1;
                }
                if (lo != cur) {
                    __syncwarp();
                    const uint32_t* src = reinterpret_cast<const uint32_t*>(&T.s[lo]);
                    uint32_t* dst = reinterpret_cast<uint32_t*>(desc);
                    for (int k = lane; k < (int)(sizeof(LeanScene) / 4); k += 32) dst[k] = src[k];
                    __syncwarp();
                    cur = lo;
                }
                cur_begin = T.s[lo].S.tile_begin;
                cur_end = cur_begin + T.s[lo].S.ntiles;
            }
            const int R = desc->S.c.R;
            PSlot* slots = reinterpret_cast<PSlot*>(wbase);
            float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * R * sizeof(PSlot));
            uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * R * (sizeof(PSlot) + sizeof(float)));
            lean_tile<TP, KSTEP>(desc->S, desc->L, t - cur_begin, slots, res_t, res_hit, lane, one, two27);
        }
    }
}

template <int TP, int KSTEP>
static vxl_status launch_lean_t(vxl_ctx* ctx, const LeanScene& P, unsigned long long* counter, int grab,
                                cudaStream_t s) {
    const size_t smem = pool_bytes(TP, P.S.c.R) * 4;
    auto kern = k_occl_lean<TP, KSTEP>;
    VXL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VXL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem));
    if (per_sm < 1) return fail(VXL_ERR_NOT_SUPPORTED, "occlusion pool: %zu bytes of shared memory per block", smem);
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (P.S.ntiles + grab - 1) / grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(P, counter, grab);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

template <int TP>
static vxl_status launch_lean_k(vxl_ctx* ctx, const LeanScene& P, unsigned long long* counter, const vxl_tuning& t,
                                cudaStream_t s) {
    switch (t.kstep) {
        case 1:
        case 2:
        case 4: return launch_lean_t<TP, 4>(ctx, P, counter, t.grab, s);
        case 16: return launch_lean_t<TP, 16>(ctx, P, counter, t.grab, s);
        default: return launch_lean_t<TP, 8>(ctx, P, counter, t.grab, s);
    }
}

// ------------------------------------------------------ wide trace layout
// Grids whose bit addresses need 33 to 37 bits (cubic grids from about 1020^3
// cells, where a row passes 256 bricks; 2048^3 needs 35): the x and y terms
// stay 32-bit, the z term is 64-bit (its brick
// index lies above bit 31), and a cell's 32-bit word index is the 64-bit
// address >> 5. Such a grid does not stay in L1 the way a 512^3 one does, so
// each ray keeps the word it last read and loads only when its word index
// changes (a 4x4x2 half-brick: about every second step).
struct LeanGridW {
    const uint32_t* __restrict__ w;
    uint32_t field[2], keep[2], inc[2], unit[2], lo[2], span[2];
    uint64_t fieldz, keepz, incz, unitz, loz, spanz;
    uint32_t one;
    int hs[3];
};

struct __align__(16) LeanSceneW {
    SceneDesc S;
    LeanGridW L;
};

static LeanGridW lean_grid_w_of(const vxl_grid* g) {
    LeanGridW L;
    L.w = reinterpret_cast<const uint32_t*>(g->tl_words);
    const int n[3] = {g->nx, g->ny, g->nz};
    for (int a = 0; a < 2; a++) {
        const AxisCode c = axis_code(a, g->tl_lbx, g->tl_lby);
        L.field[a] = c.field;
        L.keep[a] = c.keep;
        L.inc[a] = c.inc;
        L.unit[a] = c.unit;
        L.hs[a] = c.hi_shift;
        L.lo[a] = axis_term(c, 4);
        L.span[a] = axis_term(c, n[a] + 5) - L.lo[a];
    }
    // z: bits 4-5 and the brick index from bit 6 + lbx + lby up (64-bit)
    const int hz = 6 + g->tl_lbx + g->tl_lby;
    L.hs[2] = hz;
    const uint64_t gap = ((1ull << hz) - 1ull) & ~((4ull << 4) - 1ull);
    L.fieldz = (3ull << 4) | ~((1ull << hz) - 1ull);
    L.keepz = ~gap;
    L.unitz = 1ull << 4;
    L.incz = gap + L.unitz;
    auto zterm = [&](int v) { return ((uint64_t)(v & 3) << 4) | ((uint64_t)(v >> 2) << hz); };
    L.loz = zterm(4);
    L.spanz = zterm(n[2] + 5) - L.loz;
    L.one = 1u;
    return L;
}

// one iteration of Light.frag:50-75 on the wide layout with the word cache
// (wc: index of the cached word wd); as lean_step
__device__ __forceinline__ int lean_step_w(const LeanGridW& L, uint32_t& ax, uint32_t& ay, uint64_t& az, float& tx,
                                           float& ty, float& tz, float tdx, float tdy, float tdz, uint32_t kx,
                                           uint32_t ky, uint64_t kz, float maxt, float& tot, float* ht, uint32_t& wc,
                                           uint32_t& wd) {
    const uint64_t A = (uint64_t)(ax + ay) + az;
    const uint32_t wi = (uint32_t)(A >> 5);
    if (wi != wc) {
        wc = wi;
        wd = __ldg(L.w + wi);
    }
    const float m = fminf(fminf(tx, ty), tz);
    const bool bx = tx == m, by = ty == m, bz = tz == m;
    const bool tie = (bx && (by || bz)) || (by && bz);
    if (__funnelshift_r(wd, wd, (uint32_t)A) & 1u) {
        if (!(tot < maxt)) return 2;
        if (ax - L.lo[0] > L.span[0] || ay - L.lo[1] > L.span[1] || az - L.loz > L.spanz) return 2;
        float best = m + 0.0f;
        if (tie) {
            best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
            best = best + (bz ? tz : 0.0f);
        }
        *ht = best;
        return 1;
    }
    float best = m;
    if (tie) {
        best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
        best = best + (bz ? tz : 0.0f);
        if (!(best < maxt)) return 2;
    }
    if (bx) {
        ax = (ax + kx) & L.keep[0];
        tx = tx + tdx;
    }
    if (by) {
        ay = (ay + ky) & L.keep[1];
        ty = ty + tdy;
    }
    if (bz) {
        az = (az + kz) & L.keepz;
        tz = tz + tdz;
    }
    tot = best;
    return 0;
}

__device__ __forceinline__ bool lean_set_cell_w(const LeanGridW& L, uint32_t ax, uint32_t ay, uint64_t az, float tx,
                                                float ty, float tz, float tot, float maxt, float* t) {
    if (!(tot < maxt)) return false;
    if (ax - L.lo[0] > L.span[0] || ay - L.lo[1] > L.span[1] || az - L.loz > L.spanz) return false;
    const float m = fminf(fminf(tx, ty), tz);
    const bool bx = tx == m, by = ty == m, bz = tz == m;
    float best = m + 0.0f;
    if ((bx && (by || bz)) || (by && bz)) {
        best = (bx ? tx : 0.0f) + (by ? ty : 0.0f);
        best = best + (bz ? tz : 0.0f);
    }
    *t = best;
    return true;
}

// The hot form on the wide layout: the iteration of VXL_LEAN_IT with the
// adds as multiply-adds by 1 (the z term's as a signed 32-bit step times 1
// plus the 64-bit term), the z mask on the term's low half (its gap lies
// below bit 32), the word index as a funnel shift of the address's two
// halves, and the load only when that index differs from the cached one.
#define VXL_LEANW_IT(i)                       \
    "mov.b64 {zl, zh}, %2;\n\t"               \
    "mad.lo.u32 a, %0, %21, %1;\n\t"          \
    "mad.lo.u32 a, zl, %21, a;\n\t"           \
    "shf.r.clamp.b32 s, a, zh, 5;\n\t"        \
    "setp.ne.u32 pw, s, %8;\n\t"              \
    "@pw mad.wide.u32 ad, s, 4, %18;\n\t"     \
    "@pw ld.global.nc.u32 %9, [ad];\n\t"      \
    "@pw mov.u32 %8, s;\n\t"                  \
    "min.f32 m, %3, %4;\n\t"                  \
    "min.f32 m, m, %5;\n\t"                   \
    "setp.eq.f32 px, %3, m;\n\t"              \
    "setp.eq.f32 py, %4, m;\n\t"              \
    "setp.eq.f32 pz, %5, m;\n\t"              \
    "shf.r.wrap.b32 s, %9, %9, a;\n\t"        \
    "and.b32 s, s, 1;\n\t"                    \
    "setp.ne.u32 pb, s, 0;\n\t"               \
    "@pb bra VXL_WSET;\n\t"                   \
    "@px mad.lo.u32 %0, %13, %21, %0;\n\t"    \
    "@py mad.lo.u32 %1, %14, %21, %1;\n\t"    \
    "@pz mad.wide.s32 %2, %15, %21, %2;\n\t"  \
    "@px and.b32 %0, %0, 0xFFFFFFC3;\n\t"     \
    "@py and.b32 %1, %1, %16;\n\t"            \
    "mov.b64 {zl, zh}, %2;\n\t"               \
    "@pz and.b32 zl, zl, %17;\n\t"            \
    "mov.b64 %2, {zl, zh};\n\t"               \
    "@px add.rn.f32 %3, %3, %10;\n\t"         \
    "@py add.rn.f32 %4, %4, %11;\n\t"         \
    "@pz add.rn.f32 %5, %5, %12;\n\t"         \
    "and.pred q, px, py;\n\t"                 \
    "and.pred r, px, pz;\n\t"                 \
    "or.pred q, q, r;\n\t"                    \
    "and.pred r, py, pz;\n\t"                 \
    "or.pred q, q, r;\n\t"                    \
    "mov.f32 %6, m;\n\t"                      \
    "@q bra VXL_WTIE" #i ";\n"                \
    "VXL_WBACK" #i ":\n\t"
#define VXL_LEANW_TIE(i)                      \
    "VXL_WTIE" #i ":\n\t"                     \
    "and.pred r, px, py;\n\t"                 \
    "and.pred r, r, pz;\n\t"                  \
    "add.rn.f32 b, m, m;\n\t"                 \
    "@r add.rn.f32 b, b, m;\n\t"              \
    "@!r add.rn.f32 b, b, 0f00000000;\n\t"    \
    "setp.lt.f32 pn, b, %19;\n\t"             \
    "@!pn bra VXL_WEND;\n\t"                  \
    "mov.f32 %6, b;\n\t"                      \
    "bra VXL_WBACK" #i ";\n"
#define VXL_LEANW_IT4(o) VXL_LEANW_IT(o##0) VXL_LEANW_IT(o##1) VXL_LEANW_IT(o##2) VXL_LEANW_IT(o##3)
#define VXL_LEANW_TIE4(o) VXL_LEANW_TIE(o##0) VXL_LEANW_TIE(o##1) VXL_LEANW_TIE(o##2) VXL_LEANW_TIE(o##3)

// 16 iterations per batch: the stress frame's rays are long (57 reference
// steps on average), so half the batch ends cost less than the lane slots
// idle after a ray ends (1.1% faster than 8 on C5)
#ifndef VXL_LEANW_KSTEP
#define VXL_LEANW_KSTEP 16
#endif
#if VXL_LEANW_KSTEP == 16
#define VXL_LEANW_ITERS VXL_LEANW_IT4(1) VXL_LEANW_IT4(2) VXL_LEANW_IT4(3) VXL_LEANW_IT4(4)
#define VXL_LEANW_TIES VXL_LEANW_TIE4(1) VXL_LEANW_TIE4(2) VXL_LEANW_TIE4(3) VXL_LEANW_TIE4(4)
#else
#define VXL_LEANW_ITERS VXL_LEANW_IT4(1) VXL_LEANW_IT4(2)
#define VXL_LEANW_TIES VXL_LEANW_TIE4(1) VXL_LEANW_TIE4(2)
#endif

// VXL_LEANW_KSTEP iterations; returns 0 (batch done), 1 (set cell: state of its
// iteration kept) or 2 (ended by a tie's totalt)
__device__ __forceinline__ int lean_batch_w(const uint32_t* __restrict__ w, uint32_t& ax, uint32_t& ay, uint64_t& az,
                                            float& tx, float& ty, float& tz, float tdx, float tdy, float tdz,
                                            uint32_t kx, uint32_t ky, int32_t kz, uint32_t keep_y, uint32_t keep_z,
                                            uint32_t one, float maxt, float& tot, uint32_t& wc, uint32_t& wd) {
    int stop;
    uint32_t unused = 0;
    asm volatile("{\n\t"
                 ".reg .pred px, py, pz, pb, q, r, pn, pw;\n\t"
                 ".reg .b32 a, s, zl, zh;\n\t"
                 ".reg .b64 ad;\n\t"
                 ".reg .f32 m, b;\n\t" VXL_LEANW_ITERS
                 "mov.u32 %7, 0;\n\t"
                 "bra VXL_WDONE;\n"
                 "VXL_WSET:\n\t"
                 "mov.u32 %7, 1;\n\t"
                 "bra VXL_WDONE;\n"
                 "VXL_WEND:\n\t"
                 "mov.u32 %7, 2;\n\t"
                 "bra VXL_WDONE;\n" VXL_LEANW_TIES "VXL_WDONE:\n\t"
                 "}"
                 : "+r"(ax), "+r"(ay), "+l"(az), "+f"(tx), "+f"(ty), "+f"(tz), "+f"(tot), "=r"(stop), "+r"(wc),
                   "+r"(wd)
                 : "f"(tdx), "f"(tdy), "f"(tdz), "r"(kx), "r"(ky), "r"(kz), "r"(keep_y), "r"(keep_z), "l"(w),
                   "f"(maxt), "r"(unused), "r"(one));
    return stop;
}

// 9 blocks per SM (56 registers): 2.4% faster on the 2048^3 stress frame than
// 8 at 64, whose 8-pixel pools (18 rays per pixel) leave room for a ninth
#ifndef VXL_LEANW_MIN_BLOCKS
#define VXL_LEANW_MIN_BLOCKS 9
#endif

// lean_tile on the wide layout (KSTEP 8)
template <int TP>
__device__ __forceinline__ void lean_tile_w(const SceneDesc& S, const LeanGridW& L, int64_t tile, PSlot* slots,
                                            float* res_t, uint32_t* res_hit, int lane, uint32_t one) {
    constexpr int KSTEP = VXL_LEANW_KSTEP;
    const TraceConstsP& c = S.c;
    const int R = c.R;
    const unsigned ux = S.g.ux, uy = S.g.uy, uz = S.g.uz;
    const uint32_t keep_y = L.keep[1];
    const uint32_t keep_z = (uint32_t)L.keepz;  // the z gap lies below bit 32: the high half of the mask is all ones
    constexpr int LPP = 32 / TP;
    // ------------------------------------------------ A: generation
    const int p = lane % TP;
    int64_t gpix;
    const bool inimg = tile_pixel<TP>(S, tile, p, &gpix);
    f3 Pp = mk(0.0f, 0.0f, 0.0f), N = mk(0.0f, 0.0f, 0.0f);
    float ro = c.default_rough;
    if (inimg) {
        Pp = ld3(S.pos + 3 * gpix);
        N = ld3(S.nrm + 3 * gpix);
        if (S.rough) ro = S.rough[gpix];
    }
    const bool sky = !inimg || (N.x == 0.0f && N.y == 0.0f && N.z == 0.0f);
    const uint32_t hpix = pcg(c.seed_h + ((uint32_t)gpix + S.pix_base));
    const f3 O = add(Pp, mul(N, c.bias));
    f3 T, B;
    tangent_frame(N, &T, &B);
    for (int k = lane; k < R; k += 32) res_hit[k] = 0u;
    int live = 0, nlit = 0;
    const int rounds = (R + LPP - 1) / LPP;
    for (int j = 0; j < rounds; j++) {
        const int kk = j * LPP + lane / TP;
        const int k = !c.spec_first ? kk : (kk < c.n_spec ? c.n_shadow + c.n_ao + kk : kk - c.n_spec);
        bool is_live = false, is_lit = false;
        PSlot sl;
        if (kk < R && !sky) {
            const f3 d = gen_dir(c, k, hpix, Pp, N, T, B, ro);
            const float maxt = kind_maxt(c, k);
            const int meta = (p << 4) | (k << 9);
            if (!ray_domain_ok(O, d)) {
            } else if (!dir_fast_ok(d)) {
                is_lit = true;
                sl.c01 = 0;
                sl.c2m = (meta | kMetaLit) << 16;
                sl.a0 = O.x; sl.a1 = O.y; sl.a2 = O.z;
                sl.b0 = d.x; sl.b1 = d.y; sl.b2 = d.z;
            } else {
                DState s;
                dda_init(s, O, d, maxt);
                if ((unsigned)s.cx <= ux && (unsigned)s.cy <= uy && (unsigned)s.cz <= uz) {
                    is_live = true;
                    const int sg = (s.sx < 0 ? 1 : 0) | (s.sy < 0 ? 2 : 0) | (s.sz < 0 ? 4 : 0);
                    const uint32_t xs = (uint32_t)(s.cx + 4), ys = (uint32_t)(s.cy + 4), zs = (uint32_t)(s.cz + 4);
                    const uint64_t A = (uint64_t)((xs & 3u) | ((xs >> 2) << L.hs[0]) | ((ys & 3u) << 2) |
                                                  ((ys >> 2) << L.hs[1]) | ((zs & 3u) << 4)) |
                                       ((uint64_t)(zs >> 2) << L.hs[2]);
                    sl.c01 = (int)(uint32_t)A;
                    sl.c2m = ((meta | sg) << 16) | (int)(A >> 32);
                    sl.a0 = s.tx; sl.a1 = s.ty; sl.a2 = s.tz;
                    sl.b0 = s.tdx; sl.b1 = s.tdy; sl.b2 = s.tdz;
                }
            }
        }
        const unsigned lv = __ballot_sync(0xffffffffu, is_live);
        if (is_live) slots[live + __popc(lv & lanes_below())] = sl;
        live += __popc(lv);
        // rays with a direction component below 1e-30 take the literal form of the DDA after the
        // traversal loop (no call inside it): their slots fill the pool from its top down
        const unsigned lm = __ballot_sync(0xffffffffu, is_lit);
        if (lm) {
            if (is_lit) slots[TP * R - 1 - (nlit + __popc(lm & lanes_below()))] = sl;
            nlit += __popc(lm);
        }
    }
    __syncwarp();

    // ------------------------------------------------- B: traversal
    int base = 0;
    bool busy = false, retired = false;
    uint32_t ax = 0, ay = 0, kx = 0, ky = 0, wc = 0xffffffffu, wd = 0;
    uint64_t az = 0, kz = 0;
    float tx = 0.0f, ty = 0.0f, tz = 0.0f, tdx = 0.0f, tdy = 0.0f, tdz = 0.0f, maxt = 0.0f, tot = 0.0f;
    int n = 0, meta = 0;
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
                    maxt = kind_maxt(c, k);
                    {
                        busy = true;
                        const uint64_t A = (uint64_t)(uint32_t)sl.c01 | ((uint64_t)(sl.c2m & 0xffff) << 32);
                        ax = (uint32_t)A & L.field[0];
                        ay = (uint32_t)A & L.field[1];
                        az = A & L.fieldz;
                        kx = (meta & 1) ? 0u - L.unit[0] : L.inc[0];
                        ky = (meta & 2) ? 0u - L.unit[1] : L.inc[1];
                        kz = (meta & 4) ? 0ull - L.unitz : L.incz;
                        tx = sl.a0; ty = sl.a1; tz = sl.a2;
                        tdx = sl.b0; tdy = sl.b1; tdz = sl.b2;
                        tot = -INFINITY;
                        n = 0;
                        wc = 0xffffffffu;
                    }
                } else {
                    retired = true;
                }
            }
            base += __popc(nm);
        }
        if (!__any_sync(0xffffffffu, busy) && base >= live) break;
        if (busy) {
            int res = 0;
            float ht = 0.0f;
            if (__all_sync(__activemask(), n + KSTEP <= 256)) {
                const int st = lean_batch_w(L.w, ax, ay, az, tx, ty, tz, tdx, tdy, tdz, kx, ky, (int32_t)kz, keep_y,
                                            keep_z, one, maxt, tot, wc, wd);
                if (st == 1)
                    res = lean_set_cell_w(L, ax, ay, az, tx, ty, tz, tot, maxt, &ht) ? 1 : 2;
                else if (st == 2)
                    res = 2;
                else {
                    n += KSTEP;
                    if (!(tot < maxt)) res = 2;
                }
            } else {
                for (int it = 0; it < KSTEP; it++) {
                    if (n >= 256) {
                        res = 2;
                        break;
                    }
                    res = lean_step_w(L, ax, ay, az, tx, ty, tz, tdx, tdy, tdz, kx, ky, kz, maxt, tot, &ht, wc, wd);
                    if (res) break;
                    n++;
                    if (!(tot < maxt) || n >= 256) {
                        res = 2;
                        break;
                    }
                }
            }
            if (res) {
                if (res == 1) {
                    const int k = (meta >> 9) & 31, pp = (meta >> 4) & 31;
                    res_t[k * TP + pp] = ht;
                    atomicOr(&res_hit[k], 1u << pp);
                }
                busy = false;
            }
        }
    }
    for (int i = lane; i < nlit; i += 32) {
        const PSlot sl = slots[TP * R - 1 - i];
        const int m = (unsigned)sl.c2m >> 16, k = (m >> 9) & 31;
        const Hit h = dda_literal(S.g, mk(sl.a0, sl.a1, sl.a2), mk(sl.b0, sl.b1, sl.b2), kind_maxt(c, k));
        if (h.flags & VXL_RF_HIT) {
            const int pp = (m >> 4) & 31;
            res_t[k * TP + pp] = h.t;
            atomicOr(&res_hit[k], 1u << pp);
        }
    }
    __syncwarp();

    // ------------------------------------------------------ C: fold
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

template <int TP>
__global__ void __launch_bounds__(128, VXL_LEANW_MIN_BLOCKS) k_occl_lean_w(const __grid_constant__ LeanSceneW P,
                                                                           unsigned long long* __restrict__ counter,
                                                                           int grab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int R = P.S.c.R;
    unsigned char* wbase = smem + warp * pool_bytes(TP, R);
    PSlot* slots = reinterpret_cast<PSlot*>(wbase);
    float* res_t = reinterpret_cast<float*>(wbase + (size_t)TP * R * sizeof(PSlot));
    uint32_t* res_hit = reinterpret_cast<uint32_t*>(wbase + (size_t)TP * R * (sizeof(PSlot) + sizeof(float)));
    for (;;) {
        int64_t t0 = 0;
        if (lane == 0) t0 = (int64_t)atomicAdd(counter, (unsigned long long)grab);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= P.S.ntiles) break;
        for (int gi = 0; gi < grab && t0 + gi < P.S.ntiles; gi++)
            lean_tile_w<TP>(P.S, P.L, t0 + gi, slots, res_t, res_hit, lane, P.L.one);
    }
}

template <int TP>
static vxl_status launch_lean_w(vxl_ctx* ctx, const LeanSceneW& P, unsigned long long* counter, int grab,
                                cudaStream_t s) {
    const size_t smem = pool_bytes(TP, P.S.c.R) * 4;
    auto kern = k_occl_lean_w<TP>;
    VXL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VXL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem));
    if (per_sm < 1) return fail(VXL_ERR_NOT_SUPPORTED, "occlusion pool: %zu bytes of shared memory per block", smem);
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (P.S.ntiles + grab - 1) / grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(P, counter, grab);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

bool occl_lean_supported(const vxl_grid* g, const vxl_outputs* out, const vxl_tuning& tune) {
    // leap 3 (the two-level map of empty space) runs on the exact-step kernel
    return g->tl_words != nullptr && !out->records && tune.leap != 1 && !(g->tl_wide && tune.leap == 3);
}

vxl_status launch_trace_occlusion_lean(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb,
                                       const vxl_trace_params* p, const vxl_outputs* out,
                                       unsigned long long* d_counter, const vxl_tuning& tune, cudaStream_t s,
                                       uint32_t pix_base) {
    const int R = p->n_shadow + p->n_ao + p->n_spec;
    vxl_tuning t = tune;
    // many rays per pixel: 8-pixel tiles keep the pool's shared memory within 8 blocks per SM
    if (t.tile_px == 16 && (pool_bytes(16, R) * 4 + 1024) * VXL_LEAN_MIN_BLOCKS > (size_t)ctx->smem_per_sm) {
        t.tile_px = 8;
        t.tile_w = 8;
    }
    if (g->tl_wide) {
        LeanSceneW PW;
        PW.S = scene_of(g, gb, p, out, t);
        PW.S.pix_base = pix_base;
        PW.L = lean_grid_w_of(g);
        VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
        if (t.tile_px == 8) return launch_lean_w<8>(ctx, PW, d_counter, t.grab, s);
        if (t.tile_px == 32) return launch_lean_w<32>(ctx, PW, d_counter, t.grab, s);
        return launch_lean_w<16>(ctx, PW, d_counter, t.grab, s);
    }
    LeanScene P;
    P.S = scene_of(g, gb, p, out, t);
    P.S.pix_base = pix_base;
    P.L = lean_grid_of(g);
    VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
    if (t.tile_px == 8) return launch_lean_k<8>(ctx, P, d_counter, t, s);
    if (t.tile_px == 32) return launch_lean_k<32>(ctx, P, d_counter, t, s);
    return launch_lean_k<16>(ctx, P, d_counter, t, s);
}

// ------------------------------------------------------------------ batch
bool lean_batch_supported(const vxl_batch_item* items, int n, const vxl_tuning& tune) {
    if (tune.leap == 1) return false;
    for (int i = 0; i < n; i++)
        if (!items[i].grid->tl_words || items[i].grid->tl_wide) return false;
    return true;
}

size_t lean_batch_desc_bytes() { return sizeof(LeanScene); }

// the launch shape of a batch: 8-pixel tiles when the 16-pixel pools of its
// largest ray count would hold the SM below 8 blocks
vxl_tuning lean_batch_tuning(const vxl_ctx* ctx, const vxl_batch_item* items, int n, const vxl_tuning& tune) {
    int mr = 1;
    for (int i = 0; i < n; i++)
        mr = std::max(mr, items[i].params.n_shadow + items[i].params.n_ao + items[i].params.n_spec);
    vxl_tuning t = tune;
    if (t.tile_px == 16 && (pool_bytes(16, mr) * 4 + 1024) * VXL_LEAN_MIN_BLOCKS > (size_t)ctx->smem_per_sm) {
        t.tile_px = 8;
        t.tile_w = 8;
    }
    return t;
}

vxl_status lean_batch_build_table(const vxl_batch_item* items, int n, const vxl_tuning& tune, void* h_table,
                                  int* max_r, int64_t* total_tiles, int64_t* total_rays) {
    LeanScene* t = (LeanScene*)h_table;
    int64_t tiles = 0, rays = 0;
    int mr = 1;
    for (int i = 0; i < n; i++) {
        t[i].S = scene_of(items[i].grid, &items[i].gbuf, &items[i].params, &items[i].out, tune);
        t[i].S.tile_begin = tiles;
        t[i].L = lean_grid_of(items[i].grid);
        tiles += t[i].S.ntiles;
        rays += items[i].gbuf.npix * t[i].S.c.R;
        mr = std::max(mr, t[i].S.c.R);
    }
    *max_r = mr;
    *total_tiles = tiles;
    *total_rays = rays;
    return VXL_OK;
}

template <int TP, int KSTEP>
static vxl_status launch_lean_batch_t(vxl_ctx* ctx, const LeanScene* d_table, int n, int max_r, int64_t total_tiles,
                                      unsigned long long* counter, int grab, cudaStream_t s) {
    static_assert(sizeof(LeanScene) % 16 == 0, "descriptor copies keep 16-byte alignment");
    const size_t smem = pool_bytes(TP, max_r) * 4 + 4 * sizeof(LeanScene);
    auto kern = k_occl_lean_batch<TP, KSTEP>;
    VXL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VXL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem));
    if (per_sm < 1) return fail(VXL_ERR_NOT_SUPPORTED, "batch pool: %zu bytes of shared memory per block", smem);
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (total_tiles + grab - 1) / grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(d_table, n, total_tiles, max_r, counter, grab);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

template <int TP, int KSTEP>
static vxl_status launch_lean_batch_pt(vxl_ctx* ctx, const LeanBatchParams& T, int n, int max_r, int64_t total_tiles,
                                       unsigned long long* counter, int grab, cudaStream_t s) {
    const size_t smem = pool_bytes(TP, max_r) * 4 + 4 * sizeof(LeanScene);
    auto kern = k_occl_lean_batch_p<TP, KSTEP>;
    VXL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VXL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem));
    if (per_sm < 1) return fail(VXL_ERR_NOT_SUPPORTED, "batch pool: %zu bytes of shared memory per block", smem);
    int64_t blocks = (int64_t)ctx->sm_count * per_sm;
    const int64_t warps_needed = (total_tiles + grab - 1) / grab;
    if (blocks * 4 > warps_needed) blocks = (warps_needed + 3) / 4;
    kern<<<(unsigned)blocks, 128, smem, s>>>(T, n, total_tiles, max_r, counter, grab, 1u, 1u << 27);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

template <int TP>
static vxl_status launch_lean_batch_k(vxl_ctx* ctx, const LeanScene* d_table, const LeanScene* h_table, int n,
                                      int max_r, int64_t total_tiles, unsigned long long* counter, const vxl_tuning& t,
                                      cudaStream_t s) {
    if (h_table && n <= kLeanBatchMax) {
        // the table by value (unused entries stay zero and are never read)
        static thread_local LeanBatchParams T;
        std::memset(&T, 0, sizeof(T));
        std::memcpy(T.s, h_table, (size_t)n * sizeof(LeanScene));
        if (t.kstep <= 4) return launch_lean_batch_pt<TP, 4>(ctx, T, n, max_r, total_tiles, counter, t.grab, s);
        return launch_lean_batch_pt<TP, 8>(ctx, T, n, max_r, total_tiles, counter, t.grab, s);
    }
    if (t.kstep <= 4) return launch_lean_batch_t<TP, 4>(ctx, d_table, n, max_r, total_tiles, counter, t.grab, s);
    return launch_lean_batch_t<TP, 8>(ctx, d_table, n, max_r, total_tiles, counter, t.grab, s);
}

vxl_status launch_lean_batch(vxl_ctx* ctx, void* d_table, const void* h_table, int n, int max_r, int64_t total_tiles,
                             const vxl_tuning& t, unsigned long long* d_counter, cudaStream_t s) {
    VXL_TRY_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s));
    const LeanScene* tab = (const LeanScene*)d_table;
    const LeanScene* htab = (const LeanScene*)h_table;
    if (t.tile_px == 8) return launch_lean_batch_k<8>(ctx, tab, htab, n, max_r, total_tiles, d_counter, t, s);
    if (t.tile_px == 32) return launch_lean_batch_k<32>(ctx, tab, htab, n, max_r, total_tiles, d_counter, t, s);
    return launch_lean_batch_k<16>(ctx, tab, htab, n, max_r, total_tiles, d_counter, t, s);
}

}  // namespace vxl
