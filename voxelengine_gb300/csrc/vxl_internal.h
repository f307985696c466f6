// vxl_internal.h — library-internal declarations shared by the host API
// (vxl_api.cpp) and the kernel translation units (*.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/vxl.h"

struct vxl_ctx {
    int device;
    int sm_count;
    int smem_per_sm;  // shared memory per SM, bytes
    uint64_t launches;
    // growable device scratch (voxelizer tables, host-API staging, counters)
    void* d_scratch;
    size_t d_scratch_bytes;
    void* d_stage;
    size_t d_stage_bytes;
    // work-queue counters of the persistent kernels. Uncaptured launches take
    // the next slot of a ring of kCounterRing, so launches in flight on
    // different streams never share a counter. A launch recorded into a CUDA
    // graph keeps its counter for the graph's life: it takes one of
    // kCaptureCounters further slots, each handed out once per context.
    unsigned long long* d_counters;
    uint32_t counter_next;
    uint32_t capture_next;
    vxl_tuning tune;  // occlusion kernel launch shape (vxl_ctx_set_tuning)
    // copy / compute pipeline of the host-buffer entry point (created on first use)
    cudaStream_t pipe[2];
    cudaEvent_t pipe_start;
    bool pipe_ready;
    // primary visibility: screen-tile instance lists (grown from the previous
    // frame's size, read back asynchronously), pinned staging for the
    // command table, and the event after that frame's staging copy / read-back
    int* d_plist;
    size_t plist_cap;
    int* h_ptotal;
    void* h_pin;
    size_t h_pin_bytes;
    cudaEvent_t pev;
    // temporal accumulation: the per-texel records the spiral taps read
    void* d_taa;
    size_t taa_bytes;
    // positions and sky-masked normals rebuilt from a depth G-buffer
    void* d_fd;
    size_t fd_bytes;
    // fused lights: count and list of (pixel, light) pairs in range
    void* d_lpairs;
    size_t lpairs_bytes;
};
constexpr uint32_t kCounterRing = 4096;
constexpr uint32_t kCaptureCounters = 4096;

struct vxl_grid {
    vxl_ctx* ctx;
    int device;      // ctx->device, kept so that the grid can be destroyed after its context
    int nx, ny, nz;
    int bx, by, bz;  // 4^3 bricks per axis, one padding brick included
    int tx, ty, tz;  // 8^3 tiles per axis (tile map)
    uint64_t* words;
    size_t nwords;
    uint32_t* tmask;
    size_t nmask;  // uint32 words of the tile map
    // Trace layout: the same 4^3 bricks with cells shifted by +4 on every
    // axis, bricks per x row and per y column padded to powers of two
    // (2^tl_lbx, 2^tl_lby, tl_bz z slabs), and a solid border one cell outside
    // the DDA's inclusive bounds (cells -1 and n+2). Rebuilt from `words` with
    // the tile map; NULL when the bit addresses would not fit in 37 bits.
    uint64_t* tl_words;
    size_t tl_nwords;
    int tl_lbx, tl_lby, tl_bz;
    // 1: the bit addresses need more than 32 bits (up to 37: about 2048^3 cells);
    // the z term then has its brick index above bit 31 and is traced by
    // k_occl_lean_w
    int tl_wide;
    // Two-level map of empty space, for grids without a trace layout: level 1
    // is the tile map dilated by one tile (a tile's bit is set when it or one
    // of its 26 neighbours has a voxel), level 2 has one bit per 64^3 cells
    // (8^3 tiles), set when any level-1 bit in it is. Rebuilt from the tile map
    // by each occlusion call that reads them.
    uint32_t* clear1;
    uint32_t* clear2;
    int sx2, sy2, sz2;  // 64^3 super-tiles per axis
    size_t nclear2;     // uint32 words of level 2
    // 4-bit palette plane (vxl_grid_palette_alloc), 4 * nwords uint64, or
    // NULL: word 4b + z of brick b holds its layer z, nibble x + 4y. The
    // traversal does not read it.
    uint64_t* pal4;
};

namespace vxl {

// error plumbing (vxl_api.cpp)
vxl_status fail(vxl_status s, const char* fmt, ...);
vxl_status cuda_fail(cudaError_t e, const char* what);
#define VXL_TRY_CUDA(expr)                                      \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return ::vxl::cuda_fail(e_, #expr); \
    } while (0)
#define VXL_TRY(expr)                       \
    do {                                    \
        vxl_status s_ = (expr);             \
        if (s_ != VXL_OK) return s_;        \
    } while (0)

// device scratch owned by the context (grows, never shrinks)
vxl_status ctx_scratch(vxl_ctx* ctx, size_t bytes, void** out);
// grows a context-owned device buffer to at least `need` bytes (contents not kept)
vxl_status ctx_grow(void** p, size_t* have, size_t need);
vxl_status ctx_stage(vxl_ctx* ctx, size_t bytes, void** out);

struct DevInstance {
    float m[16];
    int32_t model;
    int32_t op;
};
struct DevModel {
    const uint8_t* data;
    int32_t sx, sy, sz;
    int32_t pad;
};

// launchers (kernels in grid.cu / trace.cu / voxelize.cu); each returns the
// launch error and counts launches in ctx
vxl_status launch_grid_import_r8(vxl_grid* g, const uint8_t* bytes, cudaStream_t s);
vxl_status launch_grid_export_r8(const vxl_grid* g, uint8_t* bytes, cudaStream_t s);
vxl_status launch_grid_import_palette(vxl_grid* g, const uint8_t* pal, int opaque_min, cudaStream_t s);
vxl_status launch_grid_export_palette(const vxl_grid* g, uint8_t* out, cudaStream_t s);
vxl_status launch_scene_palette(vxl_grid* g, uint32_t seed, cudaStream_t s);
// the tile map and the trace layout, from the words
vxl_status launch_build_tile_mask(vxl_grid* g, cudaStream_t s);
// the two-level map of empty space, from the tile map
vxl_status launch_build_clear_maps(const vxl_grid* g, cudaStream_t s);
// sets tl_lbx, tl_lby, tl_bz and tl_nwords (0: no trace layout) from the dims
void trace_layout_dims(vxl_grid* g);
vxl_status launch_grid_count(const vxl_grid* g, unsigned long long* d_out, cudaStream_t s);
vxl_status launch_scene_noise(vxl_grid* g, uint32_t seed, float thresh, float freq, int ground_y, cudaStream_t s);
vxl_status launch_scene_boxes(vxl_grid* g, uint32_t seed, int nboxes, int smin, int smax, cudaStream_t s);
vxl_status launch_scene_terrain(vxl_grid* g, uint32_t seed, float base, float amp, float freq, int octaves,
                                float* d_height, cudaStream_t s);
vxl_status launch_light_taa(vxl_ctx* ctx, const vxl_taa_frame* f, float* out, cudaStream_t s);
vxl_status launch_rebuild_from_depth(vxl_ctx* ctx, const float* depth, const float* nrm, int W, int H,
                                     const vxl_view* view, float* wcp, float* nrm_out, cudaStream_t s);
vxl_status launch_light_points(vxl_ctx* ctx, const vxl_grid* g, const float* wpos, const float* nrm,
                               const float* noise, int64_t npix, const vxl_light* lights, int nlights,
                               unsigned long long* lit, unsigned long long* in_range, cudaStream_t s);
vxl_status launch_volume_mips(vxl_ctx* ctx, const uint8_t* mip0, int sx, int sy, int sz, uint8_t* mip1, uint8_t* mip2,
                              cudaStream_t s);
vxl_status launch_trace_primary(vxl_ctx* ctx, const vxl_volume* volumes, int nvol, const vxl_voxcmd* cmds, int ncmd,
                                const vxl_camera* cam, const vxl_primary_out* out, cudaStream_t s);
vxl_status launch_scene_soft(vxl_ctx* ctx, float* soft, int nx, int ny, int nz, uint32_t seed, float thresh,
                             float sharpness, float freq, int ground_y, uint32_t albedo_seed, cudaStream_t s);
vxl_status launch_soft_fwd(vxl_ctx* ctx, const float* soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                           const vxl_soft_params* p, float* image, float* light, cudaStream_t st);
vxl_status launch_soft_bwd(vxl_ctx* ctx, const float* soft, int nx, int ny, int nz, const vxl_gbuffer* gb,
                           const vxl_soft_params* p, const float* grad_image, const float* light, float* grad_soft,
                           cudaStream_t st);
vxl_status launch_scene_gbuffer(const vxl_grid* g, const float cam[3], const float target[3], float tan_half_fov,
                                int W, int H, uint32_t seed, float* pos, float* nrm, float* rough, cudaStream_t s);

vxl_status launch_trace_rays(vxl_ctx* ctx, const vxl_grid* g, const float* rays, int64_t n, int mode,
                             vxl_ray_record* rec, cudaStream_t s);
vxl_status launch_trace_occlusion(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb, const vxl_trace_params* p,
                                  const vxl_outputs* out, cudaStream_t s);
bool occl_pool_supported(const vxl_grid* g, const vxl_trace_params* p);
vxl_status launch_trace_occlusion_pool(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb,
                                       const vxl_trace_params* p, const vxl_outputs* out,
                                       unsigned long long* d_counter, const vxl_tuning& tune, cudaStream_t s,
                                       uint32_t pix_base = 0);
// the same pass on the grid's trace layout (occl_lean.cu): used when the grid has
// one, no per-ray records are asked for and the exact-leap tuning is off
bool occl_lean_supported(const vxl_grid* g, const vxl_outputs* out, const vxl_tuning& tune);
vxl_status launch_trace_occlusion_lean(vxl_ctx* ctx, const vxl_grid* g, const vxl_gbuffer* gb,
                                       const vxl_trace_params* p, const vxl_outputs* out,
                                       unsigned long long* d_counter, const vxl_tuning& tune, cudaStream_t s,
                                       uint32_t pix_base);
// batched occlusion on the trace layouts: every grid of the batch has one and
// the exact-leap tuning is off (occl_lean.cu)
bool lean_batch_supported(const vxl_batch_item* items, int n, const vxl_tuning& tune);
size_t lean_batch_desc_bytes();
vxl_tuning lean_batch_tuning(const vxl_ctx* ctx, const vxl_batch_item* items, int n, const vxl_tuning& tune);
vxl_status lean_batch_build_table(const vxl_batch_item* items, int n, const vxl_tuning& tune, void* h_table,
                                  int* max_r, int64_t* total_tiles, int64_t* total_rays);
// h_table: the host copy of the table; batches of up to 64 scenes pass it by
// value as kernel parameters, larger ones read d_table
vxl_status launch_lean_batch(vxl_ctx* ctx, void* d_table, const void* h_table, int n, int max_r, int64_t total_tiles,
                             const vxl_tuning& t, unsigned long long* d_counter, cudaStream_t s);
// the work-queue counter for one persistent launch on stream s (see d_counters)
vxl_status ctx_take_counter(vxl_ctx* ctx, cudaStream_t s, unsigned long long** out);
// batched occlusion: scene table built on the host, uploaded once, one launch
size_t batch_desc_bytes();
vxl_status batch_build_table(const vxl_batch_item* items, int n, const vxl_tuning& tune, void* h_table, int* max_r,
                             int64_t* total_tiles, int64_t* total_rays, size_t* max_grid_bytes);
vxl_status launch_batch(vxl_ctx* ctx, void* d_table, int n, int max_r, int64_t total_tiles, const vxl_tuning& tune,
                        unsigned long long* d_counter, size_t max_grid_bytes, cudaStream_t s);
vxl_status launch_light_ambient(vxl_ctx* ctx, const vxl_grid* g, const float* wcp, const float* nrm,
                                const float* depth, const float* noise, int64_t npix, float* shadow, float* irr,
                                vxl_ray_record* rec, cudaStream_t s);
vxl_status launch_light_reflection(vxl_ctx* ctx, const vxl_grid* g, const float* wcp, const float* nrm,
                                   const float* view_r, const float* rough, const float* noise, int64_t npix,
                                   float* t, vxl_ray_record* rec, cudaStream_t s);
vxl_status launch_light_point(vxl_ctx* ctx, const vxl_grid* g, const float* wpos, const float* nrm,
                              const float* noise, int64_t npix, const float lp[3], float range, int spot,
                              float* shadow, vxl_ray_record* rec, cudaStream_t s);

// one pass of instances that all carry the same op (they commute)
vxl_status launch_voxelize_run(vxl_grid* g, const DevInstance* d_inst, const DevModel* d_models,
                               const int2* d_chunks, int nchunks, int value, int32_t* d_aabb, cudaStream_t s);

constexpr int kVoxChunk = 1024;  // source voxels per voxelizer block

}  // namespace vxl
