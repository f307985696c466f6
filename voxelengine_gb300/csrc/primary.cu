// primary.cu — primary visibility (the G-buffer producer of the reference's
// GeometryVoxel pass) and the VoxAsset mip builder.
//
// The reference rasterizes one cube per VoxCmd instance (GeometryVoxel.vert,
// GeometryVoxelPipeline.h:50-70) and, per fragment, traces the model's
// three-mip volume with intersectVolume (GeometryVoxel.frag:63-125) after
// clipToAABB (:50-61); the depth test keeps the nearest hit. Here the cube
// rasterization becomes screen binning: each instance's volume box is
// projected to a conservative pixel rectangle and listed in every 16x16
// screen tile it overlaps; one CTA per tile then runs, per pixel, the exact
// test "the pixel ray enters the volume box" and the traversal for every
// listed instance, keeping the nearest hit by view depth (ties to the lower
// instance index, so the list order does not matter).
//
// Spaces: the camera and instance matrices are in world units; a volume's
// local space is its voxel grid (world = R (local * 0.1) + t, the reference's
// `hitPos*0.1` and `*10.0`); output positions are in fine-voxel units
// (world * 10), the ShadowVox grid's units, so the G-buffer feeds
// vxl_trace_occlusion directly.
#include <algorithm>
#include <cstring>
#include <vector>

#include "vxl_device.cuh"
#include "vxl_internal.h"

namespace vxl {

namespace {

constexpr int kPrimTile = 16;  // screen tile edge (pixels); one CTA per tile

__host__ __device__ __forceinline__ int mip_dim(int d) { return d > 1 ? d / 2 : 1; }

// VoxAsset::Upload (VoxAsset.cpp:3-63), one level: child voxel = the first
// non-zero of its children probed in the order vi = 0..8
__global__ void k_mip_down(const uint8_t* __restrict__ parent, int psx, int psy, uint8_t* __restrict__ child, int csx,
                           int csy, int csz) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = (uint32_t)csx * csy * csz;
    if (i >= n) return;
    const int x = (int)(i % (uint32_t)csx), y = (int)((i / (uint32_t)csx) % (uint32_t)csy),
              z = (int)(i / ((uint32_t)csx * csy));
    uint8_t vox = 0;
    for (int vi = 0; vi < 9; vi++) {
        const uint8_t up = parent[(size_t)(2 * x + ((vi >> 0) & 1)) + (size_t)(2 * y + ((vi >> 1) & 1)) * psx +
                                  (size_t)(2 * z + ((vi >> 2) & 1)) * psx * psy];
        if (up) {
            vox = up;
            break;
        }
    }
    child[i] = vox;
}

__device__ __forceinline__ float glsl_mod(float x, float y) { return x - y * floorf(x / y); }

// glm's scalar max / min
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }

struct VolDev {
    const uint8_t* m[3];
    int sx, sy, sz;        // mip 0
    int dx[3], dy[3], dz[3];  // per mip
};

// one instance, prepared on the device
struct PrimInst {
    float ri[9];   // R^-1, row-major
    float ti[3];   // -R^-1 t
    float M[12];   // columns 0-2 (R) and 3 (t) of the world matrix
    float lc[3];   // camera in the volume's local space
    int vol;
    int tx0, ty0, tx1, ty1;  // screen tiles covered (inclusive); tx0 > tx1: none
    float near;              // least view depth of the box's corners (a lower bound of any hit's depth)
};

struct PrimCam {
    f3 cam, fwd, right, upv;
    float tanh_, aspect;
    int W, H, frame;
    int tiles_x, tiles_y;
};

__device__ __forceinline__ f3 rmul3(const float* r, f3 v) {
    float x = r[0] * v.x + r[1] * v.y;
    float y = r[3] * v.x + r[4] * v.y;
    float z = r[6] * v.x + r[7] * v.y;
    return mk(x + r[2] * v.z, y + r[5] * v.z, z + r[8] * v.z);
}
__device__ __forceinline__ f3 cmul3(const float* M, f3 v) {  // M[0..8] = columns 0-2
    float x = M[0] * v.x + M[3] * v.y;
    float y = M[1] * v.x + M[4] * v.y;
    float z = M[2] * v.x + M[5] * v.y;
    return mk(x + M[6] * v.z, y + M[7] * v.z, z + M[8] * v.z);
}

// affine inverse with the same operation order as the oracle's affine_inverse
__device__ __forceinline__ void affine_inverse(const float* m, float* ri, float* ti) {
    const float a00 = m[0], a10 = m[1], a20 = m[2];
    const float a01 = m[4], a11 = m[5], a21 = m[6];
    const float a02 = m[8], a12 = m[9], a22 = m[10];
    const float c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
    const float c10 = a02 * a21 - a01 * a22, c11 = a00 * a22 - a02 * a20, c12 = a01 * a20 - a00 * a21;
    const float c20 = a01 * a12 - a02 * a11, c21 = a02 * a10 - a00 * a12, c22 = a00 * a11 - a01 * a10;
    float det = a00 * c00 + a01 * c01;
    det = det + a02 * c02;
    const float id = 1.0f / det;
    ri[0] = c00 * id; ri[1] = c10 * id; ri[2] = c20 * id;
    ri[3] = c01 * id; ri[4] = c11 * id; ri[5] = c21 * id;
    ri[6] = c02 * id; ri[7] = c12 * id; ri[8] = c22 * id;
    for (int r = 0; r < 3; r++) {
        float v = ri[r * 3 + 0] * m[12] + ri[r * 3 + 1] * m[13];
        v = v + ri[r * 3 + 2] * m[14];
        ti[r] = -v;
    }
}

// Per instance: inverse, local camera, and the screen tiles its volume box
// can cover (the 8 corners projected with a margin; the full screen when a
// corner is not in front of the camera). Writes the tile count of each.
// The tiles of the 32 rectangles a warp's lanes hold, spread over its lanes:
// rectangle j of lane j is visited by all lanes (tile q of its row-major order
// by lane q mod 32), so one instance covering much of the screen does not
// leave its tiles to one thread. Called by whole warps (empty rectangles for
// lanes past the end); f(j, tile) runs once per tile of rectangle j.
template <class F>
__device__ __forceinline__ void warp_rects(int tx0, int ty0, int tx1, int ty1, int tiles_x, F f) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int j = 0; j < 32; j++) {
        const int a0 = __shfl_sync(full, tx0, j), b0 = __shfl_sync(full, ty0, j);
        const int a1 = __shfl_sync(full, tx1, j), b1 = __shfl_sync(full, ty1, j);
        const int w = a1 - a0 + 1, h = b1 - b0 + 1;
        if (w <= 0 || h <= 0) continue;
        const int cnt = w * h;
        for (int q = lane; q < cnt; q += 32) f(j, (b0 + q / w) * tiles_x + a0 + q % w);
    }
}

__device__ __forceinline__ void prim_prep_one(const vxl_voxcmd* __restrict__ cmds, int k,
                                              const VolDev* __restrict__ vols, const PrimCam& C,
                                              PrimInst* __restrict__ out, int* rtx0, int* rty0, int* rtx1,
                                              int* rty1);

// Per instance: inverse, local camera, screen-tile rectangle and its tile
// count (pair_count, scanned for the list fill); per tile: instances listed.
__global__ void k_prim_prep(const vxl_voxcmd* __restrict__ cmds, int n, const VolDev* __restrict__ vols, PrimCam C,
                            PrimInst* __restrict__ out, int* __restrict__ tile_count, int* __restrict__ pair_count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int tx0 = 0, ty0 = 0, tx1 = -1, ty1 = -1;
    if (k < n) {
        prim_prep_one(cmds, k, vols, C, out, &tx0, &ty0, &tx1, &ty1);
        pair_count[k] = (tx1 >= tx0 && ty1 >= ty0) ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0;
    }
    warp_rects(tx0, ty0, tx1, ty1, C.tiles_x, [&](int, int t) { atomicAdd(&tile_count[t], 1); });
}

__device__ __forceinline__ void prim_prep_one(const vxl_voxcmd* __restrict__ cmds, int k,
                                              const VolDev* __restrict__ vols, const PrimCam& C,
                                              PrimInst* __restrict__ out, int* rtx0, int* rty0, int* rtx1,
                                              int* rty1) {
    const float* m = cmds[k].world;
    PrimInst P;
    affine_inverse(m, P.ri, P.ti);
    for (int c = 0; c < 3; c++) {
        P.M[c] = m[c];
        P.M[3 + c] = m[4 + c];
        P.M[6 + c] = m[8 + c];
        P.M[9 + c] = m[12 + c];
    }
    const f3 lc0 = rmul3(P.ri, C.cam);
    const f3 lc = mul(add(lc0, mk(P.ti[0], P.ti[1], P.ti[2])), 10.0f);
    P.lc[0] = lc.x;
    P.lc[1] = lc.y;
    P.lc[2] = lc.z;
    P.vol = cmds[k].volume;
    const VolDev V = vols[P.vol];
    // screen rectangle of the box [0, dims] * 0.1 in world space
    float x0 = 1e30f, y0 = 1e30f, x1 = -1e30f, y1 = -1e30f;
    float zmin = 1e30f;
    bool behind = false;
    for (int c = 0; c < 8; c++) {
        const f3 l = mk((c & 1) ? V.sx * 0.1f : 0.0f, (c & 2) ? V.sy * 0.1f : 0.0f, (c & 4) ? V.sz * 0.1f : 0.0f);
        const f3 w = add(cmul3(P.M, l), mk(P.M[9], P.M[10], P.M[11]));
        const f3 r = sub(w, C.cam);
        const float zc = dot(r, C.fwd);
        zmin = fminf(zmin, zc);
        if (!(zc > 1e-3f)) behind = true;
        if (behind) continue;
        const float sx = dot(r, C.right) / (zc * C.tanh_ * C.aspect);
        const float sy = dot(r, C.upv) / (zc * C.tanh_);
        const float px = (sx + 1.0f) * 0.5f * (float)C.W;
        const float py = (1.0f - sy) * 0.5f * (float)C.H;
        x0 = fminf(x0, px);
        x1 = fmaxf(x1, px);
        y0 = fminf(y0, py);
        y1 = fmaxf(y1, py);
    }
    int tx0, ty0, tx1, ty1;
    if (behind) {
        tx0 = 0;
        ty0 = 0;
        tx1 = C.tiles_x - 1;
        ty1 = C.tiles_y - 1;
    } else {
        // 2-pixel margin: the exact box test runs per pixel, this only has to be conservative
        const float fx0 = floorf((x0 - 2.0f) / kPrimTile), fx1 = floorf((x1 + 2.0f) / kPrimTile);
        const float fy0 = floorf((y0 - 2.0f) / kPrimTile), fy1 = floorf((y1 + 2.0f) / kPrimTile);
        tx0 = (int)fminf(fmaxf(fx0, 0.0f), (float)C.tiles_x);
        ty0 = (int)fminf(fmaxf(fy0, 0.0f), (float)C.tiles_y);
        tx1 = (int)fminf(fmaxf(fx1, -1.0f), (float)(C.tiles_x - 1));
        ty1 = (int)fminf(fmaxf(fy1, -1.0f), (float)(C.tiles_y - 1));
    }
    P.tx0 = tx0;
    P.ty0 = ty0;
    P.tx1 = tx1;
    P.ty1 = ty1;
    P.near = zmin;
    out[k] = P;
    *rtx0 = tx0;
    *rty0 = ty0;
    *rtx1 = tx1;
    *rty1 = ty1;
}

// exclusive scan by one CTA of 1024 threads, any length, 8 consecutive
// elements per thread (8192 per pass: one pass for a 1080p frame's tiles):
// offsets[t] = sum of counts before t; offsets[ntiles] = total
constexpr int kScanItems = 8;
__device__ __forceinline__ void cta_scan(const int* __restrict__ counts, int ntiles, int* __restrict__ offsets) {
    __shared__ int warp_sums[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < ntiles; base += 1024 * kScanItems) {
        const int i0 = base + threadIdx.x * kScanItems;
        int v[kScanItems];
        int x = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            v[j] = i0 + j < ntiles ? counts[i0 + j] : 0;
            x += v[j];
        }
        const int own = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        int run = (warp > 0 ? warp_sums[warp - 1] : 0) + carry + x - own;
#pragma unroll
        for (int j = 0; j < kScanItems; j++) {
            if (i0 + j < ntiles) offsets[i0 + j] = run;
            run += v[j];
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = run;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[ntiles] = carry;
}

// CTA 0 scans the per-tile counts, CTA 1 the per-instance tile counts
__global__ void k_prim_scan(const int* __restrict__ tile_count, int ntiles, int* __restrict__ tile_off,
                            const int* __restrict__ pair_count, int n, int* __restrict__ pair_off) {
    if (blockIdx.x == 0)
        cta_scan(tile_count, ntiles, tile_off);
    else
        cta_scan(pair_count, n, pair_off);
}

// entries beyond the list capacity are dropped; k_primary then scans every
// instance for every tile (exact, slower) and the host grows the lists
__global__ void k_prim_fill(const PrimInst* __restrict__ insts, int n, int tiles_x, const int* __restrict__ offsets,
                            int* __restrict__ cursor, int* __restrict__ lists, int64_t cap,
                            const int* __restrict__ pair_off) {
    // every (instance, tile) pair of the frame, spread evenly over the grid:
    // pair e belongs to the instance k with pair_off[k] <= e < pair_off[k + 1]
    const int total = pair_off[n];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(pair_off + mid) <= e)
                lo = mid;
            else
                hi = mid - 1;
        }
        const PrimInst& P = insts[lo];
        const int w = P.tx1 - P.tx0 + 1, q = e - __ldg(pair_off + lo);
        const int t = (P.ty0 + q / w) * tiles_x + P.tx0 + q % w;
        const int64_t at = (int64_t)offsets[t] + atomicAdd(&cursor[t], 1);
        if (at < cap) lists[at] = lo;
    }
}

// clipToAABB, GeometryVoxel.frag:50-61
// (inv = 1 / d per component, computed once by the caller)
__device__ __forceinline__ f3 clip_to_aabb(f3 o, f3 d, f3 inv, f3 size) {
    const f3 c = mk(gmin(gmax(o.x, 0.0f), size.x), gmin(gmax(o.y, 0.0f), size.y), gmin(gmax(o.z, 0.0f), size.z));
    if (c.x == o.x && c.y == o.y && c.z == o.z) return o;
    const f3 sgn = mk(glsl_step(d.x, 0.0f), glsl_step(d.y, 0.0f), glsl_step(d.z, 0.0f));
    const f3 t = mk((sgn.x * size.x - o.x) * inv.x, (sgn.y * size.y - o.y) * inv.y, (sgn.z * size.z - o.z) * inv.z);
    const float tmin = gmax(gmax(t.x, t.y), t.z);
    return add(o, mul(d, tmin - 0.001f));
}

// One mip level of a volume: texels and dimensions, loaded from the volume
// table when the walk enters the level (only the level in use is held in
// registers)
struct VolLevel {
    const uint8_t* m;
    int sx, sy, sz;
};
__device__ __forceinline__ VolLevel vol_level(const VolDev* __restrict__ vp, int mip) {
    return VolLevel{vp->m[mip], vp->dx[mip], vp->dy[mip], vp->dz[mip]};
}

// texelFetch(VOLUME_TEXTURE, p, mip).r with robust out-of-range = 0
__device__ __forceinline__ uint32_t vol_texel(const VolLevel& L, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= L.sx || y >= L.sy || z >= L.sz) return 0u;
    return __ldg(L.m + ((size_t)x + (size_t)y * L.sx + (size_t)z * L.sx * L.sy));
}

// 1 / (d * sign(d)) from inv = 1 / d: for d != 0, d * sign(d) = |d| exactly and
// IEEE division is symmetric in sign, so the quotient is |inv|; for d = +-0,
// sign(d) = +0 and the quotient is an infinity with the sign of d * +0
// (a NaN d gives the canonical NaN either way)
__device__ __forceinline__ float abs_recip(float d, float sgn, float inv) {
    const float a = d * sgn;
    return a == 0.0f ? __int_as_float(0x7f800000 | (__float_as_int(a) & 0x80000000)) : fabsf(inv);
}

// intersectVolume, GeometryVoxel.frag:63-125 (LOD 1, MIP_COUNT 2,
// TRANSPARENCY 1), operation for operation (inv = 1 / direction)
__device__ __forceinline__ bool intersect_volume(const VolDev* __restrict__ vp, f3 origin, f3 direction, f3 inv, f3 lcam, float uvx,
                                                 float uvy, float resx, float resy, int frame, f3* hit, f3* normal,
                                                 uint32_t* material) {
    const f3 ss = mk(glsl_sign(direction.x), glsl_sign(direction.y), glsl_sign(direction.z));
    const f3 td = mk(abs_recip(direction.x, ss.x, inv.x), abs_recip(direction.y, ss.y, inv.y),
                     abs_recip(direction.z, ss.z, inv.z));
    // int(select * sign) with select in {0, 1} and sign in {-1, 0, 1}: the
    // integer sign where the axis is selected
    const int isx = (int)ss.x, isy = (int)ss.y, isz = (int)ss.z;
    int mip = 2;
    int i = 0;
    do {
        const float mipSize = (float)(1 << mip);
        // x / mipSize for mipSize = 1, 2, 4: the exact reciprocal times x rounds the
        // same real value, so the multiply gives the division's float
        const float invMip = mip == 2 ? 0.25f : (mip == 1 ? 0.5f : 1.0f);
        origin = mk(origin.x * invMip, origin.y * invMip, origin.z * invMip);
        int cx = (int)floorf(origin.x), cy = (int)floorf(origin.y), cz = (int)floorf(origin.z);
        const f3 nb = mk((float)cx + (ss.x * 0.5f + 0.5f), (float)cy + (ss.y * 0.5f + 0.5f),
                         (float)cz + (ss.z * 0.5f + 0.5f));
        f3 tm = mk((nb.x - origin.x) / direction.x, (nb.y - origin.y) / direction.y, (nb.z - origin.z) / direction.z);
        const int ux = (int)((float)vp->sx * invMip) + 1, uy = (int)((float)vp->sy * invMip) + 1,
                  uz = (int)((float)vp->sz * invMip) + 1;
        const VolLevel L = vol_level(vp, mip);
        int n = 0;
        do {
            const float selx = glsl_step(tm.x, tm.z) * glsl_step(tm.x, tm.y);
            const float sely = glsl_step(tm.y, tm.x) * glsl_step(tm.y, tm.z);
            const float selz = glsl_step(tm.z, tm.y) * glsl_step(tm.z, tm.x);
            cx += selx != 0.0f ? isx : 0;
            cy += sely != 0.0f ? isy : 0;
            cz += selz != 0.0f ? isz : 0;
            if (cx < -1 || cy < -1 || cz < -1 || cx > ux || cy > uy || cz > uz) return false;
            const uint32_t voxel = vol_texel(L, cx, cy, cz);
            if (voxel != 0u) {
                float best_t = tm.x * selx + tm.y * sely;
                best_t = best_t + tm.z * selz;
                bool accept = mip == 0;
                if (!accept) {
                    const f3 p = mul(add(origin, mul(direction, best_t)), mipSize);
                    const f3 dd = sub(p, lcam);
                    accept = (float)mip < 0.001f * sqrtf(dot(dd, dd));
                }
                if (accept) {
                    const float kx = roundf(uvx * resx * 0.5f), ky = roundf(uvy * resy * 0.5f);
                    const bool glass = voxel < 16u && glsl_mod(ky + kx, 2.0f) == (float)(frame % 2);
                    if (!glass) {
                        *normal = mk(-ss.x * selx, -ss.y * sely, -ss.z * selz);
                        *hit = mul(add(origin, mul(direction, best_t)), mipSize);
                        *material = voxel;
                        return true;
                    }
                } else {
                    mip--;
                    const f3 st = mul(direction, best_t);
                    origin = add(origin, mk(st.x * invMip, st.y * invMip, st.z * invMip));
                    break;
                }
            }
            tm = mk(tm.x + td.x * selx, tm.y + td.y * sely, tm.z + td.z * selz);
        } while (++n < 512);
        origin = mul(origin, mipSize);
    } while (++i < 4);
    return false;
}

// One CTA per 16x16 screen tile, one thread per pixel. The tile's instance
// list is taken in chunks of 256, each sorted in shared memory by the
// instances' nearest corner depth; a pixel stops scanning a chunk once that
// depth, less a safety margin for rounding, is beyond its current hit (no
// instance further in the chunk can be nearer).
__global__ void __launch_bounds__(256, 4) k_primary(const PrimInst* __restrict__ insts, const VolDev* __restrict__ vols,
                                                    PrimCam C, const int* __restrict__ offsets,
                                                    const int* __restrict__ lists, int64_t cap, int ninst,
                                                    float* __restrict__ pos, float* __restrict__ nrm,
                                                    float* __restrict__ depth, int32_t* __restrict__ material,
                                                    int32_t* __restrict__ instance) {
    __shared__ float s_near[256];
    __shared__ int s_id[256];
    const int tile = blockIdx.x;
    const int tx = tile % C.tiles_x, ty = tile / C.tiles_x;
    const int px = tx * kPrimTile + (threadIdx.x % kPrimTile), py = ty * kPrimTile + (threadIdx.x / kPrimTile);
    const bool live = px < C.W && py < C.H;
    const int i = live ? py * C.W + px : 0;
    const float uvx = ((float)px + 0.5f) * 2.0f / (float)C.W - 1.0f;
    const float uvy = ((float)py + 0.5f) * 2.0f / (float)C.H - 1.0f;
    const float u = uvx * C.tanh_ * C.aspect;
    const float v = (1.0f - ((float)py + 0.5f) * 2.0f / (float)C.H) * C.tanh_;
    const f3 d = normalize(add(add(C.fwd, mul(C.right, u)), mul(C.upv, v)));
    float best = 0.0f;
    int bi = -1;
    f3 bp = mk(0.0f, 0.0f, 0.0f), bn = mk(0.0f, 0.0f, 0.0f);
    uint32_t bm = 0;
    // lists that overflowed their capacity: every instance, in index order
    const bool all = (int64_t)offsets[C.tiles_x * C.tiles_y] > cap;
    const int e0 = all ? 0 : offsets[tile], e1 = all ? ninst : offsets[tile + 1];
    for (int c0 = e0; c0 < e1; c0 += 256) {
        const int cn = min(256, e1 - c0);
        __syncthreads();
        if ((int)threadIdx.x < cn) {
            const int k = all ? c0 + (int)threadIdx.x : lists[c0 + threadIdx.x];
            s_id[threadIdx.x] = k;
            s_near[threadIdx.x] = insts[k].near;
        } else {
            s_id[threadIdx.x] = 0x7fffffff;
            s_near[threadIdx.x] = INFINITY;
        }
        __syncthreads();
        // bitonic sort of the first n2 (near, id) pairs, ascending: n2 = the power of
        // two at or above the chunk's length (the padding entries sort last)
        int n2 = 2;
        while (n2 < cn) n2 <<= 1;
        for (int size = 2; size <= n2; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                const int a = threadIdx.x, b = a ^ stride;
                if (b > a && b < n2) {
                    const bool up = (a & size) == 0;
                    const float na = s_near[a], nb = s_near[b];
                    const int ia = s_id[a], ib = s_id[b];
                    const bool gt = na > nb || (na == nb && ia > ib);
                    if (gt == up) {
                        s_near[a] = nb;
                        s_near[b] = na;
                        s_id[a] = ib;
                        s_id[b] = ia;
                    }
                }
                __syncthreads();
            }
        if (live) {
            for (int e = 0; e < cn; e++) {
                const float nz = s_near[e];
                if (bi >= 0 && nz - (1e-3f * fabsf(nz) + 1e-3f) > best) break;
                const int k = s_id[e];
                const PrimInst& P = insts[k];
                const VolDev* vp = vols + P.vol;
                const f3 lc = mk(P.lc[0], P.lc[1], P.lc[2]);
                const f3 ld = normalize(rmul3(P.ri, d));
                // the pixel ray enters the volume box
                const float dims[3] = {(float)vp->sx, (float)vp->sy, (float)vp->sz};
                const f3 inv = mk(1.0f / ld.x, 1.0f / ld.y, 1.0f / ld.z);
                const float lo[3] = {lc.x, lc.y, lc.z}, iv[3] = {inv.x, inv.y, inv.z};
                float t0 = -INFINITY, t1 = INFINITY;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const float ta = (0.0f - lo[a]) * iv[a], tb = (dims[a] - lo[a]) * iv[a];
                    t0 = fmaxf(t0, fminf(ta, tb));
                    t1 = fminf(t1, fmaxf(ta, tb));
                }
                if (!(t0 <= t1 && t1 >= 0.0f)) continue;
                const f3 o = clip_to_aabb(lc, ld, inv, mk(dims[0], dims[1], dims[2]));
                f3 h, nn;
                uint32_t mat;
                if (!intersect_volume(vp, o, ld, inv, lc, uvx, uvy, (float)C.W, (float)C.H, C.frame, &h, &nn, &mat))
                    continue;
                const f3 wl = cmul3(P.M, mul(h, 0.1f));
                const f3 wp = mk(wl.x + P.M[9], wl.y + P.M[10], wl.z + P.M[11]);
                const float dep = dot(sub(wp, C.cam), C.fwd);
                if (bi < 0 || dep < best || (dep == best && k < bi)) {
                    best = dep;
                    bi = k;
                    bp = wp;
                    bn = nn;
                    bm = mat;
                }
            }
        }
    }
    if (!live) return;
    float* po = pos + 3 * (size_t)i;
    float* no = nrm + 3 * (size_t)i;
    if (bi >= 0) {
        const f3 nw = normalize(cmul3(insts[bi].M, bn));
        po[0] = bp.x * 10.0f;
        po[1] = bp.y * 10.0f;
        po[2] = bp.z * 10.0f;
        no[0] = nw.x;
        no[1] = nw.y;
        no[2] = nw.z;
        if (depth) depth[i] = best;
    } else {
        po[0] = po[1] = po[2] = 0.0f;
        no[0] = no[1] = no[2] = 0.0f;
        if (depth) depth[i] = 0.0f;
    }
    if (material) material[i] = (int32_t)bm;
    if (instance) instance[i] = bi;
}

inline unsigned blocks_of(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// host-side camera basis, same arithmetic as the oracle (no FMA contraction)
void h_normalize3(const float* v, float* o) {
    float d = v[0] * v[0] + v[1] * v[1];
    d = d + v[2] * v[2];
    const float r = 1.0f / sqrtf(d);
    o[0] = v[0] * r;
    o[1] = v[1] * r;
    o[2] = v[2] * r;
}
void h_cross3(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

}  // namespace

vxl_status launch_volume_mips(vxl_ctx* ctx, const uint8_t* mip0, int sx, int sy, int sz, uint8_t* mip1, uint8_t* mip2,
                              cudaStream_t s) {
    const int x1 = mip_dim(sx), y1 = mip_dim(sy), z1 = mip_dim(sz);
    const int x2 = mip_dim(x1), y2 = mip_dim(y1), z2 = mip_dim(z1);
    k_mip_down<<<blocks_of((size_t)x1 * y1 * z1, 256), 256, 0, s>>>(mip0, sx, sy, mip1, x1, y1, z1);
    k_mip_down<<<blocks_of((size_t)x2 * y2 * z2, 256), 256, 0, s>>>(mip1, x1, y1, mip2, x2, y2, z2);
    ctx->launches += 2;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_trace_primary(vxl_ctx* ctx, const vxl_volume* volumes, int nvol, const vxl_voxcmd* cmds, int ncmd,
                                const vxl_camera* cam, const vxl_primary_out* out, cudaStream_t s) {
    PrimCam C;
    float t[3] = {cam->target[0] - cam->pos[0], cam->target[1] - cam->pos[1], cam->target[2] - cam->pos[2]};
    float fwd[3], right[3], upv[3], up[3] = {0.0f, 1.0f, 0.0f}, tmp[3];
    h_normalize3(t, fwd);
    h_cross3(fwd, up, tmp);
    h_normalize3(tmp, right);
    h_cross3(right, fwd, upv);
    C.cam = mk(cam->pos[0], cam->pos[1], cam->pos[2]);
    C.fwd = mk(fwd[0], fwd[1], fwd[2]);
    C.right = mk(right[0], right[1], right[2]);
    C.upv = mk(upv[0], upv[1], upv[2]);
    C.tanh_ = cam->tan_half_fov;
    C.aspect = (float)cam->width / (float)cam->height;
    C.W = cam->width;
    C.H = cam->height;
    C.frame = cam->frame;
    C.tiles_x = (C.W + kPrimTile - 1) / kPrimTile;
    C.tiles_y = (C.H + kPrimTile - 1) / kPrimTile;
    const int ntiles = C.tiles_x * C.tiles_y;
    const int n = ncmd;
    // device scratch: volumes, commands, prepared instances, tile counts / offsets / cursors
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_vol = al(sizeof(VolDev) * (size_t)(nvol > 0 ? nvol : 1));
    const size_t b_cmd = al(sizeof(vxl_voxcmd) * (size_t)(n > 0 ? n : 1));
    const size_t b_ins = al(sizeof(PrimInst) * (size_t)(n > 0 ? n : 1));
    const size_t b_cnt = al(sizeof(int) * (size_t)(ntiles + 1));
    const size_t b_pc = al(sizeof(int) * (size_t)(n + 1));
    const size_t head = b_vol + b_cmd + b_ins + 3 * b_cnt + 2 * b_pc;
    void* p;
    VXL_TRY(ctx_scratch(ctx, head, &p));
    char* base = (char*)p;
    VolDev* d_vol = (VolDev*)base;
    vxl_voxcmd* d_cmd = (vxl_voxcmd*)(base + b_vol);
    PrimInst* d_ins = (PrimInst*)(base + b_vol + b_cmd);
    int* d_count = (int*)(base + b_vol + b_cmd + b_ins);
    int* d_off = (int*)(base + b_vol + b_cmd + b_ins + b_cnt);
    int* d_cur = (int*)(base + b_vol + b_cmd + b_ins + 2 * b_cnt);
    int* d_pcount = (int*)(base + b_vol + b_cmd + b_ins + 3 * b_cnt);
    int* d_poff = (int*)(base + b_vol + b_cmd + b_ins + 3 * b_cnt + b_pc);
    std::vector<VolDev> hv((size_t)(nvol > 0 ? nvol : 1));
    for (int v = 0; v < nvol; v++) {
        hv[v].m[0] = volumes[v].mip[0];
        hv[v].m[1] = volumes[v].mip[1];
        hv[v].m[2] = volumes[v].mip[2];
        hv[v].sx = volumes[v].sx;
        hv[v].sy = volumes[v].sy;
        hv[v].sz = volumes[v].sz;
        hv[v].dx[0] = volumes[v].sx;
        hv[v].dy[0] = volumes[v].sy;
        hv[v].dz[0] = volumes[v].sz;
        for (int q = 1; q < 3; q++) {
            hv[v].dx[q] = mip_dim(hv[v].dx[q - 1]);
            hv[v].dy[q] = mip_dim(hv[v].dy[q - 1]);
            hv[v].dz[q] = mip_dim(hv[v].dz[q - 1]);
        }
    }
    // the previous frame's staging copy and list-size read-back have finished
    // (normally long ago) before the pinned buffers are reused
    if (ctx->pev) VXL_TRY_CUDA(cudaEventSynchronize(ctx->pev));
    const size_t b_vol_h = sizeof(VolDev) * (size_t)nvol, b_cmd_h = sizeof(vxl_voxcmd) * (size_t)n;
    if (ctx->h_pin_bytes < b_vol_h + b_cmd_h) {
        if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
        ctx->h_pin = nullptr;
        ctx->h_pin_bytes = 0;
        const size_t want = (b_vol_h + b_cmd_h) * 3 / 2 + 4096;
        VXL_TRY_CUDA(cudaHostAlloc(&ctx->h_pin, want, cudaHostAllocDefault));
        ctx->h_pin_bytes = want;
    }
    if (!ctx->h_ptotal) {
        VXL_TRY_CUDA(cudaHostAlloc((void**)&ctx->h_ptotal, sizeof(int), cudaHostAllocDefault));
        *ctx->h_ptotal = 0;
    }
    if (!ctx->pev) VXL_TRY_CUDA(cudaEventCreateWithFlags(&ctx->pev, cudaEventDisableTiming));
    // list capacity from the previous frame's total (and a floor for the first)
    const int64_t want_cap = std::max<int64_t>((int64_t)*ctx->h_ptotal, (int64_t)n * 16 + ntiles);
    if ((int64_t)ctx->plist_cap < want_cap) {
        if (ctx->d_plist) VXL_TRY_CUDA(cudaFree(ctx->d_plist));
        ctx->d_plist = nullptr;
        ctx->plist_cap = 0;
        const size_t cap = (size_t)want_cap * 3 / 2;
        VXL_TRY_CUDA(cudaMalloc((void**)&ctx->d_plist, cap * sizeof(int)));
        ctx->plist_cap = cap;
    }
    std::memcpy(ctx->h_pin, hv.data(), b_vol_h);
    if (n > 0) std::memcpy((char*)ctx->h_pin + b_vol_h, cmds, b_cmd_h);
    VXL_TRY_CUDA(cudaMemcpyAsync(d_vol, ctx->h_pin, b_vol_h, cudaMemcpyHostToDevice, s));
    if (n > 0) VXL_TRY_CUDA(cudaMemcpyAsync(d_cmd, (char*)ctx->h_pin + b_vol_h, b_cmd_h, cudaMemcpyHostToDevice, s));
    VXL_TRY_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int) * (size_t)(ntiles + 1), s));
    VXL_TRY_CUDA(cudaMemsetAsync(d_cur, 0, sizeof(int) * (size_t)(ntiles + 1), s));
    if (n > 0) {
        k_prim_prep<<<blocks_of((size_t)n, 32), 32, 0, s>>>(d_cmd, n, d_vol, C, d_ins, d_count, d_pcount);
        ctx->launches++;
    }
    k_prim_scan<<<n > 0 ? 2 : 1, 1024, 0, s>>>(d_count, ntiles, d_off, d_pcount, n, d_poff);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    // the list length goes back to the host without a wait; it sizes the next frame's lists
    VXL_TRY_CUDA(cudaMemcpyAsync(ctx->h_ptotal, d_off + ntiles, sizeof(int), cudaMemcpyDeviceToHost, s));
    VXL_TRY_CUDA(cudaEventRecord(ctx->pev, s));
    const int64_t cap = (int64_t)ctx->plist_cap;
    if (n > 0) {
        k_prim_fill<<<(unsigned)ctx->sm_count * 4, 256, 0, s>>>(d_ins, n, C.tiles_x, d_off, d_cur, ctx->d_plist, cap,
                                                               d_poff);
        ctx->launches++;
    }
    k_primary<<<ntiles, kPrimTile * kPrimTile, 0, s>>>(d_ins, d_vol, C, d_off, ctx->d_plist, cap, n, out->pos,
                                                       out->nrm, out->depth, out->material, out->instance);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
