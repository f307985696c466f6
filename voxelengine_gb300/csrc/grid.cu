// grid.cu — grid layout conversions, tile map, and the seeded scene /
// G-buffer generators used by tests and benchmarks.
#include "vxl_device.cuh"

namespace vxl {

// fine coordinates of bit b of word w (inverse of word_index / bit_index)
__device__ __forceinline__ void word_origin(const GridView& g, uint32_t w, int* x0, int* y0, int* z0) {
    uint32_t bz = w / g.bxy, rem = w - bz * g.bxy;
    uint32_t by = rem / (uint32_t)g.bx, bx = rem - by * (uint32_t)g.bx;
    *x0 = (int)(bx * 4u);
    *y0 = (int)(by * 4u);
    *z0 = (int)(bz * 4u);
}

// ---------------------------------------------------------------- R8 in/out
// ShadowVox R8 layout: byte (bx,by,bz) at bx + by*sx + bz*sx*sy holds fine
// voxels 2b + {0,1}^3, bit (x&1)|(y&1)<<1|(z&1)<<2 (ShadowVoxSystem.cpp:82-94).
__global__ void k_import_r8(GridView g, uint64_t* words, const uint8_t* __restrict__ bytes, uint32_t nwords) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    int x0, y0, z0;
    word_origin(g, w, &x0, &y0, &z0);
    const int sx = g.nx >> 1, sy = g.ny >> 1, sz = g.nz >> 1;
    uint64_t out = 0;
    for (int dz = 0; dz < 2; dz++)
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                int bx = (x0 >> 1) + dx, by = (y0 >> 1) + dy, bz = (z0 >> 1) + dz;
                if (bx >= sx || by >= sy || bz >= sz) continue;
                uint32_t v = bytes[(size_t)bx + (size_t)by * sx + (size_t)bz * sx * sy];
                for (int b = 0; b < 8; b++)
                    if (v & (1u << b)) {
                        int lx = 2 * dx + (b & 1), ly = 2 * dy + ((b >> 1) & 1), lz = 2 * dz + ((b >> 2) & 1);
                        out |= 1ull << (lx | (ly << 2) | (lz << 4));
                    }
            }
    words[w] = out;
}

__global__ void k_export_r8(GridView g, uint8_t* __restrict__ bytes, uint32_t nbytes) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbytes) return;
    const uint32_t sx = g.nx >> 1, sy = g.ny >> 1;
    uint32_t bz = i / (sx * sy), rem = i - bz * sx * sy;
    uint32_t by = rem / sx, bx = rem - by * sx;
    int x = 2 * bx, y = 2 * by, z = 2 * bz;
    uint64_t w = g.words[word_index(g, x, y, z)];
    uint32_t sh = bit_index(x, y, z);
    uint32_t v = 0;
    for (int b = 0; b < 8; b++) {
        uint32_t bit = sh + (b & 1) + ((b >> 1) & 1) * 4 + ((b >> 2) & 1) * 16;
        v |= (uint32_t)((w >> bit) & 1ull) << b;
    }
    bytes[i] = (uint8_t)v;
}

// dense palette volume [nz][ny][nx] -> bits (index >= opaque_min)
// pal4 (optional): the grid's 4-bit palette plane, four uint64 per brick
// (word z of a brick holds layer z, nibble x + 4y): the index's low 4 bits for
// set voxels, 0 for empty ones.
__global__ void k_import_palette(GridView g, uint64_t* words, uint64_t* pal4, const uint8_t* __restrict__ pal,
                                 int opaque_min, uint32_t nwords) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    int x0, y0, z0;
    word_origin(g, w, &x0, &y0, &z0);
    uint64_t out = 0;
    for (int lz = 0; lz < 4; lz++) {
        uint64_t layer = 0;
        for (int ly = 0; ly < 4; ly++)
            for (int lx = 0; lx < 4; lx++) {
                int x = x0 + lx, y = y0 + ly, z = z0 + lz;
                if (x >= g.nx || y >= g.ny || z >= g.nz) continue;
                const uint8_t v = pal[(size_t)x + (size_t)y * g.nx + (size_t)z * g.nx * g.ny];
                if (v >= opaque_min) {
                    out |= 1ull << (lx | (ly << 2) | (lz << 4));
                    layer |= (uint64_t)(v & 15u) << (4 * (lx | (ly << 2)));
                }
            }
        if (pal4) pal4[4 * (size_t)w + lz] = layer;
    }
    words[w] = out;
}

// the palette plane as a dense uint8 volume [nz][ny][nx] (one thread per voxel)
__global__ void k_export_palette(GridView g, const uint64_t* __restrict__ pal4, uint8_t* out, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t nxy = (uint64_t)g.nx * g.ny;
    const int z = (int)(i / nxy), r = (int)(i - (uint64_t)z * nxy);
    const int y = r / g.nx, x = r - y * g.nx;
    const uint64_t layer = pal4[4 * (size_t)word_index(g, x, y, z) + (z & 3)];
    out[i] = (uint8_t)((layer >> (4 * ((x & 3) | ((y & 3) << 2)))) & 15u);
}

// seeded palette indices for the set voxels (synthetic scenes): 1 + hash % 15
__global__ void k_scene_palette(GridView g, uint64_t* pal4, uint32_t seed, uint32_t nwords) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    const uint64_t occ = g.words[w];
    for (int lz = 0; lz < 4; lz++) {
        uint64_t layer = 0;
        for (int b = 0; b < 16; b++) {
            if ((occ >> (b + 16 * lz)) & 1ull) {
                const uint32_t h = pcg(seed + pcg(w * 64u + (uint32_t)(b + 16 * lz)));
                layer |= (uint64_t)(1u + h % 15u) << (4 * b);
            }
        }
        pal4[4 * (size_t)w + lz] = layer;
    }
}

// one bit per 8^3 tile: any of its 2x2x2 bricks non-zero
__global__ void k_tile_mask(GridView g, uint32_t* mask, int by_, int bz_, uint32_t ntiles, uint32_t nmask) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmask * 32u) return;
    bool any = false;
    if (t < ntiles) {
        uint32_t tz = t / g.txy, rem = t - tz * g.txy;
        uint32_t ty = rem / (uint32_t)g.tx, tx = rem - ty * (uint32_t)g.tx;
        for (int k = 0; k < 8 && !any; k++) {
            int bx = 2 * tx + (k & 1), by = 2 * ty + ((k >> 1) & 1), bz = 2 * tz + ((k >> 2) & 1);
            if (bx < g.bx && by < by_ && bz < bz_) any = g.words[(uint32_t)bx + (uint32_t)by * g.bx + bz * g.bxy] != 0ull;
        }
    }
    unsigned m = __ballot_sync(0xffffffffu, any);
    if ((threadIdx.x & 31) == 0) mask[t >> 5] = m;
}

// Trace layout word i: the grid's brick at (bricks shifted by one on every
// axis) plus the border cells it holds.
__global__ void k_trace_layout(GridView g, TraceLayout t, uint32_t nwords) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwords) return;
    const int qx = (int)(i & ((1u << t.lbx) - 1u));
    const int qy = (int)((i >> t.lbx) & ((1u << t.lby) - 1u));
    const int qz = (int)(i >> (t.lbx + t.lby));
    uint64_t w = 0;
    const int cx = qx - 1, cy = qy - 1, cz = qz - 1;  // the grid's brick
    const int gby = (int)(g.bxy / (uint32_t)g.bx), gbz = ((g.nz + 3) >> 2) + 1;
    if (cx >= 0 && cy >= 0 && cz >= 0 && cx < g.bx && cy < gby && cz < gbz)
        w = g.words[(uint32_t)cx + (uint32_t)cy * (uint32_t)g.bx + (uint32_t)cz * g.bxy];
    // border: shifted coordinates 3 (cell -1) and n+6 (cell n+2)
    const int ex = t.nx + 6, ey = t.ny + 6, ez = t.nz + 6;
    const bool touches = qx == 0 || qx == (ex >> 2) || qy == 0 || qy == (ey >> 2) || qz == 0 || qz == (ez >> 2);
    if (touches) {
        for (int b = 0; b < 64; b++) {
            const int x = 4 * qx + (b & 3), y = 4 * qy + ((b >> 2) & 3), z = 4 * qz + (b >> 4);
            const bool inbox = x >= 3 && x <= ex && y >= 3 && y <= ey && z >= 3 && z <= ez;
            const bool face = x == 3 || x == ex || y == 3 || y == ey || z == 3 || z == ez;
            if (inbox && face) w |= 1ull << b;
        }
    }
    t.words[i] = w;
}

// level 1 of the map of empty space: tile t's bit is the OR of the tile
// map's bits of t and its 26 neighbours
__global__ void k_clear1(const uint32_t* __restrict__ tmask, uint32_t* __restrict__ out, int tx, int ty, int tz,
                         uint32_t ntiles, uint32_t nmask) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmask * 32u) return;
    bool any = false;
    if (t < ntiles) {
        const uint32_t txy = (uint32_t)tx * (uint32_t)ty;
        const int z = (int)(t / txy), r = (int)(t - (uint32_t)z * txy);
        const int y = r / tx, x = r - y * tx;
        for (int dz = -1; dz <= 1 && !any; dz++)
            for (int dy = -1; dy <= 1 && !any; dy++)
                for (int dx = -1; dx <= 1 && !any; dx++) {
                    const int xx = x + dx, yy = y + dy, zz = z + dz;
                    if (xx < 0 || yy < 0 || zz < 0 || xx >= tx || yy >= ty || zz >= tz) continue;
                    const uint32_t i = (uint32_t)xx + (uint32_t)yy * (uint32_t)tx + (uint32_t)zz * txy;
                    any = (tmask[i >> 5] >> (i & 31)) & 1u;
                }
    }
    const unsigned m = __ballot_sync(0xffffffffu, any);
    if ((threadIdx.x & 31) == 0) out[t >> 5] = m;
}

// level 2: one bit per 8^3 tiles, the OR of their level-1 bits
__global__ void k_clear2(const uint32_t* __restrict__ c1, uint32_t* __restrict__ out, int tx, int ty, int tz, int sx,
                         int sy, uint32_t nsuper, uint32_t nwords) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nwords * 32u) return;
    bool any = false;
    if (q < nsuper) {
        const uint32_t sxy = (uint32_t)sx * (uint32_t)sy;
        const int Z = (int)(q / sxy), r = (int)(q - (uint32_t)Z * sxy);
        const int Y = r / sx, X = r - Y * sx;
        const uint32_t txy = (uint32_t)tx * (uint32_t)ty;
        for (int z = 8 * Z; z < min(8 * Z + 8, tz) && !any; z++)
            for (int y = 8 * Y; y < min(8 * Y + 8, ty) && !any; y++)
                for (int x = 8 * X; x < min(8 * X + 8, tx) && !any; x++) {
                    const uint32_t i = (uint32_t)x + (uint32_t)y * (uint32_t)tx + (uint32_t)z * txy;
                    any = (c1[i >> 5] >> (i & 31)) & 1u;
                }
    }
    const unsigned m = __ballot_sync(0xffffffffu, any);
    if ((threadIdx.x & 31) == 0) out[q >> 5] = m;
}

__global__ void k_count(const uint64_t* __restrict__ words, size_t n, unsigned long long* out) {
    unsigned long long c = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        c += __popcll(words[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ------------------------------------------------------------- scene noise
// value noise with a PCG lattice, smoothstep-weighted trilinear; same
// arithmetic as the oracle's value_noise3 / noise_octaves
__device__ __forceinline__ float lattice(int ix, int iy, int iz, uint32_t seed) {
    return u01(pcg((uint32_t)ix + pcg((uint32_t)iy + pcg((uint32_t)iz + seed))));
}
__device__ float value_noise3(float x, float y, float z, uint32_t seed) {
    float fx0 = floorf(x), fy0 = floorf(y), fz0 = floorf(z);
    int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    float fx = x - fx0, fy = y - fy0, fz = z - fz0;
    float wx = fx * fx * (3.0f - 2.0f * fx);
    float wy = fy * fy * (3.0f - 2.0f * fy);
    float wz = fz * fz * (3.0f - 2.0f * fz);
    float c000 = lattice(ix, iy, iz, seed), c100 = lattice(ix + 1, iy, iz, seed);
    float c010 = lattice(ix, iy + 1, iz, seed), c110 = lattice(ix + 1, iy + 1, iz, seed);
    float c001 = lattice(ix, iy, iz + 1, seed), c101 = lattice(ix + 1, iy, iz + 1, seed);
    float c011 = lattice(ix, iy + 1, iz + 1, seed), c111 = lattice(ix + 1, iy + 1, iz + 1, seed);
    float x00 = c000 + (c100 - c000) * wx;
    float x10 = c010 + (c110 - c010) * wx;
    float x01 = c001 + (c101 - c001) * wx;
    float x11 = c011 + (c111 - c011) * wx;
    float y0 = x00 + (x10 - x00) * wy;
    float y1 = x01 + (x11 - x01) * wy;
    return y0 + (y1 - y0) * wz;
}
// octave convention of Sources/Util/Noise.cpp:108-122
__device__ float noise_octaves(float x, float y, float z, uint32_t seed, float freq, int octaves) {
    float total = 0.0f, frequency = freq, amplitude = 1.0f, maxValue = 0.0f;
    for (int i = 0; i < octaves; i++) {
        total += value_noise3(x * frequency, y * frequency, z * frequency, seed + (uint32_t)i * 0x9E3779B9u) *
                 amplitude;
        maxValue += amplitude;
        amplitude *= 0.5f;
        frequency *= 2.0f;
    }
    return total / maxValue;
}

// one thread per word; ORs into the grid
__global__ void k_scene_noise(GridView g, uint64_t* words, uint32_t seed, float thresh, float freq, int ground_y,
                              uint32_t nwords) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    int x0, y0, z0;
    word_origin(g, w, &x0, &y0, &z0);
    if (x0 >= g.nx || y0 >= g.ny || z0 >= g.nz) return;
    uint64_t out = 0;
    for (int lz = 0; lz < 4; lz++)
        for (int ly = 0; ly < 4; ly++)
            for (int lx = 0; lx < 4; lx++) {
                int x = x0 + lx, y = y0 + ly, z = z0 + lz;
                if (x >= g.nx || y >= g.ny || z >= g.nz) continue;
                bool on = y < ground_y;
                if (!on) on = noise_octaves((float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f, seed, freq, 3) > thresh;
                if (on) out |= 1ull << (lx | (ly << 2) | (lz << 4));
            }
    if (out) words[w] |= out;
}

// heightfield terrain: column height base + amp * fbm(x + 0.5, 0.5, z + 0.5)
__global__ void k_heightmap(float* h, int nx, int nz, uint32_t seed, float base, float amp, float freq, int octaves) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)nx * (uint32_t)nz) return;
    const int x = (int)(i % (uint32_t)nx), z = (int)(i / (uint32_t)nx);
    const float v = noise_octaves((float)x + 0.5f, 0.5f, (float)z + 0.5f, seed, freq, octaves);
    h[i] = base + amp * v;
}
// one thread per word; voxel (x, y, z) is solid when (float)y < h(x, z)
__global__ void k_scene_terrain(GridView g, uint64_t* words, const float* __restrict__ h, uint32_t nwords) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    int x0, y0, z0;
    word_origin(g, w, &x0, &y0, &z0);
    if (x0 >= g.nx || y0 >= g.ny || z0 >= g.nz) return;
    uint64_t out = 0;
    for (int lz = 0; lz < 4; lz++)
        for (int lx = 0; lx < 4; lx++) {
            const int x = x0 + lx, z = z0 + lz;
            if (x >= g.nx || z >= g.nz) continue;
            const float hh = h[(size_t)z * g.nx + x];
            for (int ly = 0; ly < 4; ly++) {
                const int y = y0 + ly;
                if (y < g.ny && (float)y < hh) out |= 1ull << (lx | (ly << 2) | (lz << 4));
            }
        }
    if (out) words[w] |= out;
}

// soft grid: one thread per voxel, float4 (opacity, albedo rgb)
__global__ void k_scene_soft(float4* soft, int nx, int ny, int nz, uint32_t seed, float thresh, float sharp,
                             float freq, int ground_y, uint32_t aseed_h, uint32_t nvox) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvox) return;
    const int x = (int)(i % (uint32_t)nx), y = (int)((i / (uint32_t)nx) % (uint32_t)ny),
              z = (int)(i / ((uint32_t)nx * (uint32_t)ny));
    (void)nz;
    float a = 1.0f;
    if (y >= ground_y) {
        const float v = noise_octaves((float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f, seed, freq, 3);
        a = 1.0f / (1.0f + expf(-sharp * (v - thresh)));
    }
    const uint32_t h = pcg(aseed_h + i);
    soft[i] = make_float4(a, u01(pcg(h)), u01(pcg(h + 1u)), u01(pcg(h + 2u)));
}

// box i: per axis size smin + pcg(base+2a) % (smax-smin+1) (clamped to the
// grid), position pcg(base+2a+1) % (n-size+1); base = pcg(pcg(seed^0x5bd1e995)+i)
__device__ __forceinline__ void box_params(uint32_t seed, int i, const int* n, int smin, int smax, int* b) {
    uint32_t base = pcg(pcg(seed ^ 0x5bd1e995u) + (uint32_t)i);
    for (int a = 0; a < 3; a++) {
        uint32_t r1 = pcg(base + 2u * a), r2 = pcg(base + 2u * a + 1u);
        int s = smin + (int)(r1 % (uint32_t)(smax - smin + 1));
        if (s > n[a]) s = n[a];
        b[a] = (int)(r2 % (uint32_t)(n[a] - s + 1));
        b[3 + a] = s;
    }
}
// one block per box, threads over the 4^3 bricks it overlaps
__global__ void k_scene_boxes(GridView g, uint64_t* words, uint32_t seed, int smin, int smax) {
    int n[3] = {g.nx, g.ny, g.nz};
    int b[6];
    box_params(seed, blockIdx.x, n, smin, smax, b);
    int wx0 = b[0] >> 2, wy0 = b[1] >> 2, wz0 = b[2] >> 2;
    int wx1 = (b[0] + b[3] - 1) >> 2, wy1 = (b[1] + b[4] - 1) >> 2, wz1 = (b[2] + b[5] - 1) >> 2;
    int cx = wx1 - wx0 + 1, cy = wy1 - wy0 + 1, cz = wz1 - wz0 + 1;
    for (int k = threadIdx.x; k < cx * cy * cz; k += blockDim.x) {
        int bz = wz0 + k / (cx * cy), rem = k % (cx * cy);
        int by = wy0 + rem / cx, bx = wx0 + rem % cx;
        uint64_t m = 0;
        for (int lz = 0; lz < 4; lz++)
            for (int ly = 0; ly < 4; ly++)
                for (int lx = 0; lx < 4; lx++) {
                    int x = 4 * bx + lx, y = 4 * by + ly, z = 4 * bz + lz;
                    if (x >= b[0] && x < b[0] + b[3] && y >= b[1] && y < b[1] + b[4] && z >= b[2] && z < b[2] + b[5])
                        m |= 1ull << (lx | (ly << 2) | (lz << 4));
                }
        if (m) atomicOr((unsigned long long*)(words + word_index(g, 4 * bx, 4 * by, 4 * bz)), (unsigned long long)m);
    }
}

// -------------------------------------------------------------- G-buffer
// Pinhole camera at cam looking at target (up +y); rays clipped to the grid
// box and walked with an entry-face DDA (same arithmetic as the oracle's
// vo_gbuffer). Sky pixels: pos = nrm = 0.
__global__ void k_gbuffer(GridView g, f3 cam, f3 fwd, f3 right, f3 upv, float tanh_, float aspect, int W, int H,
                          uint32_t seed_h, float* pos, float* nrm, float* rough) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    int px = i % W, py = i / W;
    const int Nd[3] = {g.nx, g.ny, g.nz};
    float u = (((float)px + 0.5f) * 2.0f / (float)W - 1.0f) * tanh_ * aspect;
    float v = (1.0f - ((float)py + 0.5f) * 2.0f / (float)H) * tanh_;
    f3 d = normalize(add(add(fwd, mul(right, u)), mul(upv, v)));
    float dv[3] = {d.x, d.y, d.z}, cv[3] = {cam.x, cam.y, cam.z};
    for (int a = 0; a < 3; a++)
        if (dv[a] == 0.0f) dv[a] = 1e-20f;
    float inv[3], tn[3], tf[3];
    for (int a = 0; a < 3; a++) {
        inv[a] = 1.0f / dv[a];
        float t0 = (0.0f - cv[a]) * inv[a], t1 = ((float)Nd[a] - cv[a]) * inv[a];
        tn[a] = t0 < t1 ? t0 : t1;
        tf[a] = t0 < t1 ? t1 : t0;
    }
    int ax = 0;
    float tenter = tn[0];
    if (tn[1] > tenter) { tenter = tn[1]; ax = 1; }
    if (tn[2] > tenter) { tenter = tn[2]; ax = 2; }
    float texit = tf[0] < tf[1] ? tf[0] : tf[1];
    texit = texit < tf[2] ? texit : tf[2];
    float* po = pos + 3 * (size_t)i;
    float* no = nrm + 3 * (size_t)i;
    float P[3] = {0.0f, 0.0f, 0.0f}, Nn[3] = {0.0f, 0.0f, 0.0f};
    rough[i] = 0.05f + 0.95f * rand01(seed_h, (uint32_t)i, 7777u);
    if (!(tenter > texit || texit <= 0.0f)) {
        float tent = tenter > 0.0f ? tenter : 0.0f;
        int c[3], st[3];
        float tmax[3], tdel[3];
        for (int a = 0; a < 3; a++) {
            st[a] = dv[a] > 0.0f ? 1 : -1;
            if (a == ax && tenter > 0.0f) {
                c[a] = dv[a] > 0.0f ? 0 : Nd[a] - 1;
            } else {
                float pa = cv[a] + dv[a] * tent;
                int ci = (int)floorf(pa);
                c[a] = ci < 0 ? 0 : (ci > Nd[a] - 1 ? Nd[a] - 1 : ci);
            }
            tmax[a] = ((float)(c[a] + (st[a] > 0 ? 1 : 0)) - cv[a]) * inv[a];
            tdel[a] = fabsf(inv[a]);
        }
        int last = tenter > 0.0f ? ax : -1;
        for (int it = 0; it < Nd[0] + Nd[1] + Nd[2] + 3; it++) {
            if (fine_at(g, c[0], c[1], c[2])) {
                if (last >= 0) {
                    for (int a = 0; a < 3; a++) P[a] = cv[a] + dv[a] * tent;
                    Nn[last] = (float)(-st[last]);
                }
                break;
            }
            int a = (tmax[0] <= tmax[1] && tmax[0] <= tmax[2]) ? 0 : (tmax[1] <= tmax[2] ? 1 : 2);
            tent = tmax[a];
            c[a] += st[a];
            tmax[a] += tdel[a];
            last = a;
            if (c[a] < 0 || c[a] >= Nd[a]) break;
        }
    }
    po[0] = P[0];
    po[1] = P[1];
    po[2] = P[2];
    no[0] = Nn[0];
    no[1] = Nn[1];
    no[2] = Nn[2];
}

// ---------------------------------------------------------------- launchers
static inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

vxl_status launch_grid_import_r8(vxl_grid* g, const uint8_t* bytes, cudaStream_t s) {
    GridView v = view_of(g);
    k_import_r8<<<blocks_for(g->nwords, 256), 256, 0, s>>>(v, g->words, bytes, (uint32_t)g->nwords);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return launch_build_tile_mask(g, s);
}

vxl_status launch_grid_export_r8(const vxl_grid* g, uint8_t* bytes, cudaStream_t s) {
    GridView v = view_of(g);
    uint32_t nb = (uint32_t)((size_t)(g->nx / 2) * (g->ny / 2) * (g->nz / 2));
    k_export_r8<<<blocks_for(nb, 256), 256, 0, s>>>(v, bytes, nb);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_grid_import_palette(vxl_grid* g, const uint8_t* pal, int opaque_min, cudaStream_t s) {
    GridView v = view_of(g);
    k_import_palette<<<blocks_for(g->nwords, 128), 128, 0, s>>>(v, g->words, g->pal4, pal, opaque_min,
                                                                 (uint32_t)g->nwords);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return launch_build_tile_mask(g, s);
}

vxl_status launch_grid_export_palette(const vxl_grid* g, uint8_t* out, cudaStream_t s) {
    const uint64_t n = (uint64_t)g->nx * g->ny * g->nz;
    k_export_palette<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(view_of(g), g->pal4, out, n);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_scene_palette(vxl_grid* g, uint32_t seed, cudaStream_t s) {
    k_scene_palette<<<blocks_for(g->nwords, 128), 128, 0, s>>>(view_of(g), g->pal4, seed, (uint32_t)g->nwords);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

void trace_layout_dims(vxl_grid* g) {
    auto lg = [](int v) {
        int l = 0;
        while ((1 << l) < v) l++;
        return l;
    };
    // bricks covering shifted cells [3, n+6] (cells -1 .. n+2)
    const int cx = ((g->nx + 6) >> 2) + 1, cy = ((g->ny + 6) >> 2) + 1, cz = ((g->nz + 6) >> 2) + 1;
    g->tl_lbx = lg(cx);
    g->tl_lby = lg(cy);
    g->tl_bz = cz;
    const int sh = 6 + g->tl_lbx + g->tl_lby;
    // every bit address fits in 32 bits (the x and y terms always must), or in
    // 37 bits with the z term's brick index above bit 31 (wide: 32-bit word
    // indices, kept below 2^32 - 1)
    const unsigned long long bits = (unsigned long long)cz << sh;
    g->tl_wide = 0;
    if (sh >= 32 || bits >= (1ull << 37)) {
        g->tl_nwords = 0;
        return;
    }
    g->tl_wide = bits > (1ull << 32) ? 1 : 0;
    g->tl_nwords = (size_t)cz << (g->tl_lbx + g->tl_lby);
}

cudaError_t launch_trace_layout_view(const GridView& v, const TraceLayout& t, cudaStream_t s) {
    const size_t n = (size_t)t.bz << (t.lbx + t.lby);
    k_trace_layout<<<blocks_for(n, 256), 256, 0, s>>>(v, t, (uint32_t)n);
    return cudaGetLastError();
}

vxl_status launch_build_tile_mask(vxl_grid* g, cudaStream_t s) {
    uint32_t ntiles = (uint32_t)((size_t)g->tx * g->ty * g->tz);
    k_tile_mask<<<blocks_for(g->nmask * 32, 256), 256, 0, s>>>(view_of(g), g->tmask, g->by, g->bz, ntiles,
                                                             (uint32_t)g->nmask);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    if (g->tl_words) {
        TraceLayout t{g->tl_words, g->tl_lbx, g->tl_lby, g->tl_bz, g->nx, g->ny, g->nz};
        VXL_TRY_CUDA(launch_trace_layout_view(view_of(g), t, s));
        g->ctx->launches++;
    }
    return VXL_OK;
}

vxl_status launch_build_clear_maps(const vxl_grid* g, cudaStream_t s) {
    if (!g->clear1 || !g->clear2) return fail(VXL_ERR_NOT_SUPPORTED, "clear maps: grid has none");
    const uint32_t ntiles = (uint32_t)((size_t)g->tx * g->ty * g->tz);
    k_clear1<<<blocks_for(g->nmask * 32, 256), 256, 0, s>>>(g->tmask, g->clear1, g->tx, g->ty, g->tz, ntiles,
                                                          (uint32_t)g->nmask);
    const uint32_t nsuper = (uint32_t)((size_t)g->sx2 * g->sy2 * g->sz2);
    k_clear2<<<blocks_for(g->nclear2 * 32, 128), 128, 0, s>>>(g->clear1, g->clear2, g->tx, g->ty, g->tz, g->sx2,
                                                             g->sy2, nsuper, (uint32_t)g->nclear2);
    g->ctx->launches += 2;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

cudaError_t launch_tile_mask_view(const GridView& v, uint32_t* mask, int by, int bz, int tx, int ty, int tz,
                                  cudaStream_t s) {
    uint32_t ntiles = (uint32_t)((size_t)tx * ty * tz);
    uint32_t nmask = (ntiles + 31) / 32;
    k_tile_mask<<<blocks_for((size_t)nmask * 32, 256), 256, 0, s>>>(v, mask, by, bz, ntiles, nmask);
    return cudaGetLastError();
}

vxl_status launch_grid_count(const vxl_grid* g, unsigned long long* d_out, cudaStream_t s) {
    k_count<<<g->ctx->sm_count * 4, 256, 0, s>>>(g->words, g->nwords, d_out);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_scene_noise(vxl_grid* g, uint32_t seed, float thresh, float freq, int ground_y, cudaStream_t s) {
    GridView v = view_of(g);
    k_scene_noise<<<blocks_for(g->nwords, 128), 128, 0, s>>>(v, g->words, seed, thresh, freq, ground_y,
                                                             (uint32_t)g->nwords);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return launch_build_tile_mask(g, s);
}

vxl_status launch_scene_soft(vxl_ctx* ctx, float* soft, int nx, int ny, int nz, uint32_t seed, float thresh,
                             float sharpness, float freq, int ground_y, uint32_t albedo_seed, cudaStream_t s) {
    const size_t n = (size_t)nx * ny * nz;
    if (n == 0) return VXL_OK;
    k_scene_soft<<<blocks_for(n, 256), 256, 0, s>>>(reinterpret_cast<float4*>(soft), nx, ny, nz, seed, thresh,
                                                   sharpness, freq, ground_y, pcg(albedo_seed), (uint32_t)n);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

vxl_status launch_scene_terrain(vxl_grid* g, uint32_t seed, float base, float amp, float freq, int octaves,
                                float* d_height, cudaStream_t s) {
    const size_t ncol = (size_t)g->nx * g->nz;
    float* h = d_height;
    if (!h) {
        void* p;
        VXL_TRY(ctx_scratch(g->ctx, ncol * sizeof(float), &p));
        h = (float*)p;
    }
    k_heightmap<<<blocks_for(ncol, 256), 256, 0, s>>>(h, g->nx, g->nz, seed, base, amp, freq, octaves);
    GridView v = view_of(g);
    k_scene_terrain<<<blocks_for(g->nwords, 128), 128, 0, s>>>(v, g->words, h, (uint32_t)g->nwords);
    g->ctx->launches += 2;
    VXL_TRY_CUDA(cudaGetLastError());
    return launch_build_tile_mask(g, s);
}

vxl_status launch_scene_boxes(vxl_grid* g, uint32_t seed, int nboxes, int smin, int smax, cudaStream_t s) {
    if (nboxes <= 0) return VXL_OK;
    GridView v = view_of(g);
    k_scene_boxes<<<nboxes, 128, 0, s>>>(v, g->words, seed, smin, smax);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return launch_build_tile_mask(g, s);
}

// host-side camera basis, same arithmetic as the oracle (compiled without FMA contraction)
static void h_normalize(const float* v, float* o) {
    float d = v[0] * v[0] + v[1] * v[1];
    d = d + v[2] * v[2];
    float r = 1.0f / sqrtf(d);
    o[0] = v[0] * r;
    o[1] = v[1] * r;
    o[2] = v[2] * r;
}
static void h_cross(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

vxl_status launch_scene_gbuffer(const vxl_grid* g, const float cam[3], const float target[3], float tan_half_fov,
                                int W, int H, uint32_t seed, float* pos, float* nrm, float* rough, cudaStream_t s) {
    float t[3] = {target[0] - cam[0], target[1] - cam[1], target[2] - cam[2]};
    float fwd[3], right[3], upv[3], up[3] = {0.0f, 1.0f, 0.0f}, tmp[3];
    h_normalize(t, fwd);
    h_cross(fwd, up, tmp);
    h_normalize(tmp, right);
    h_cross(right, fwd, upv);
    float aspect = (float)W / (float)H;
    GridView v = view_of(g);
    k_gbuffer<<<blocks_for((size_t)W * H, 128), 128, 0, s>>>(
        v, mk(cam[0], cam[1], cam[2]), mk(fwd[0], fwd[1], fwd[2]), mk(right[0], right[1], right[2]),
        mk(upv[0], upv[1], upv[2]), tan_half_fov, aspect, W, H, pcg(seed), pos, nrm, rough);
    g->ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

// Surface positions from a linear-depth G-buffer as LightAmbient places a
// pixel (LightAmbient.vert:32-36, LightAmbient.frag:136-150); the oracle's
// vo_rebuild_from_depth is the same arithmetic in the same order.
struct ViewMats {
    float iv[16], ip[16];
};

__device__ __forceinline__ void mat4_vec(const float* m, float x, float y, float z, float w, float* o) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
        float a = m[r] * x;
        a = a + m[4 + r] * y;
        a = a + m[8 + r] * z;
        a = a + m[12 + r] * w;
        o[r] = a;
    }
}

__global__ void k_rebuild_from_depth(const float* __restrict__ depth, const float* __restrict__ nrm, int W, int H,
                                     const ViewMats M, float* __restrict__ wcp, float* __restrict__ nrm_out) {
    const int64_t n = (int64_t)W * H;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(k % W), j = (int)(k / W);
        const float d = depth[k];
        float* p = wcp + 3 * k;
        float* o = nrm_out + 3 * k;
        if (!(d < 0.999f)) {
            p[0] = p[1] = p[2] = 0.0f;
            o[0] = o[1] = o[2] = 0.0f;
            continue;
        }
        const float nx = ((float)i + 0.5f) * 2.0f / (float)W - 1.0f;
        const float ny = 1.0f - ((float)j + 0.5f) * 2.0f / (float)H;
        float v[4], q[4];
        mat4_vec(M.ip, nx, ny, 1.0f, 1.0f, v);
        const float s = d * (1.0f + 1.0f / 4096.0f);
        const float px = (v[0] / v[3]) * s, py = (v[1] / v[3]) * s, pz = (v[2] / v[3]) * s;
        mat4_vec(M.iv, px, py, pz, 1.0f, q);
        p[0] = q[0] * 10.0f;
        p[1] = q[1] * 10.0f;
        p[2] = q[2] * 10.0f;
        o[0] = nrm[3 * k];
        o[1] = nrm[3 * k + 1];
        o[2] = nrm[3 * k + 2];
    }
}

vxl_status launch_rebuild_from_depth(vxl_ctx* ctx, const float* depth, const float* nrm, int W, int H,
                                     const vxl_view* view, float* wcp, float* nrm_out, cudaStream_t s) {
    ViewMats M;
    for (int k = 0; k < 16; k++) {
        M.iv[k] = view->inverse_view[k];
        M.ip[k] = view->inverse_projection[k];
    }
    const int64_t n = (int64_t)W * H;
    const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 16);
    k_rebuild_from_depth<<<blocks, 256, 0, s>>>(depth, nrm, W, H, M, wcp, nrm_out);
    ctx->launches++;
    VXL_TRY_CUDA(cudaGetLastError());
    return VXL_OK;
}

}  // namespace vxl
