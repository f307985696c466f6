/*
 * vxl.h — C ABI of libvxl, a GB300 (sm_103a) implementation of VoxelEngine's
 * voxel-lighting path: the ShadowVox voxelizer and the voxel ray traversal
 * behind raytraced shadows, ambient occlusion and specular occlusion.
 *
 * Conventions
 *  - Every entry point returns vxl_status; nothing is thrown across the ABI.
 *    vxl_last_error_string() gives a thread-local message for the last failure.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    All device work is stream-ordered and asynchronous unless stated.
 *  - Pointers documented as "device" are caller-owned device memory on the
 *    context's GPU; "host" pointers are read before the call returns.
 *  - Coordinates are in fine-voxel units: one unit is one ShadowVox bit,
 *    0.1 world units (Sources/World/Systems/ShadowVoxSystem.cpp:147, x10).
 *  - A grid of fine dimensions (nx,ny,nz) corresponds to the reference's R8
 *    ShadowVox image of (nx/2, ny/2, nz/2) bytes, 2x2x2 voxels per byte.
 *  - Stream capture (CUDA graphs). Some calls only enqueue kernels and
 *    memsets on `stream`: they neither synchronize, nor allocate, nor read
 *    results back to the host. These may be captured:
 *      - vxl_trace_rays, vxl_trace_occlusion, vxl_light_ambient,
 *        vxl_light_reflection, vxl_light_point;
 *      - vxl_trace_soft_fwd, vxl_trace_soft_bwd, vxl_volume_build_mips;
 *      - vxl_grid_clear, vxl_grid_build_bricks, vxl_grid_import_r8,
 *        vxl_grid_export_r8, vxl_grid_import_palette, vxl_grid_export_palette;
 *      - vxl_scene_noise, vxl_scene_boxes, vxl_scene_palette, vxl_scene_soft,
 *        vxl_scene_gbuffer;
 *      - vxl_batch_run of a batch created with use_graph = 0 (with
 *        use_graph = 1 the batch replays its own graph).
 *    A second group grows a context workspace the first time it sees a
 *    larger frame. These may be captured only after an uncaptured call of
 *    the same or a larger size on that context: vxl_trace_occlusion_from_depth,
 *    vxl_light_points, vxl_light_taa, vxl_scene_terrain.
 *    The rest must not be captured:
 *      - vxl_trace_primary reads its tile-list total back to the host;
 *      - the voxelizer calls upload host tables and wait for them;
 *      - vxl_trace_occlusion_host and vxl_grid_count are synchronous;
 *      - the create and destroy calls, and vxl_grid_palette_alloc, allocate or
 *        free.
 *    A captured call fixes its scalar arguments and pointers in the graph,
 *    and replays of one graph must not overlap.
 */
#ifndef VXL_H
#define VXL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VXL_ABI_VERSION 2

typedef enum vxl_status {
    VXL_OK = 0,
    VXL_ERR_INVALID_ARG = 1,
    VXL_ERR_OOM = 2,
    VXL_ERR_CUDA = 3,
    VXL_ERR_TIMEOUT = 4,
    VXL_ERR_OUT_OF_RANGE = 5,
    VXL_ERR_IO = 6,
    VXL_ERR_NOT_SUPPORTED = 7
} vxl_status;

typedef struct vxl_ctx vxl_ctx;
typedef struct vxl_grid vxl_grid;

/* ---------------------------------------------------------------- basics */
int vxl_abi_version(void);
const char* vxl_last_error_string(void);
const char* vxl_status_string(vxl_status s);

/* Context on one CUDA device. Owns library scratch buffers; one context per
 * host thread, or guard it with a mutex. Replaces the engine's Graphics
 * singleton for this path (Sources/Graphics/Graphics.h:23-32).
 * The calls that use a context workspace (primary visibility, the fused
 * lights, temporal accumulation, the depth-buffer and host-buffer occlusion
 * entries, the voxelizer's tables) reuse it from call to call: on one context,
 * such calls on different streams must not overlap (order them, or use one
 * context per stream). vxl_trace_occlusion and vxl_trace_rays may overlap
 * freely: each uncaptured occlusion call takes its own work-queue counter
 * from a ring of 4096 per context, so at most 4096 such calls may be in flight
 * at once. An occlusion call made while its stream is capturing a CUDA graph
 * keeps its counter for the life of that graph: it gets one of 4096 further
 * counters that no other call of the context ever uses, so graph replays
 * never share a counter with a direct call or another capture. A context
 * accepts at most 4096 captured occlusion calls; the next one fails with
 * VXL_ERR_NOT_SUPPORTED. Replays of one graph must not overlap. */
vxl_status vxl_ctx_create(int device, vxl_ctx** out);
vxl_status vxl_ctx_destroy(vxl_ctx* ctx);
/* number of kernels this library launched through ctx (diagnostics) */
vxl_status vxl_ctx_launch_count(const vxl_ctx* ctx, uint64_t* out);

/* Launch-shape knobs of the occlusion kernel (results do not depend on them).
 * Zero fields keep the current value. Picked per device by the autotuner
 * (voxelengine_gb300/autotune.py). */
typedef struct vxl_tuning {
    int32_t tile_px;   /* pixels per warp tile: 8, 16 or 32 (the exact-step and batched kernels run 8 as 16) */
    int32_t kstep;     /* DDA iterations between pool refills: 1, 2, 4, 8 or 16 (16: the single-scene
                          trace-layout kernel; the others run 8 for it) */
    int32_t leap;      /* empty-space skipping: 1 = cross empty bricks in one step where exact; 2 = none;
                          3 = on grids without a trace layout (its bit addresses would not fit in 32 bits: about
                          1000^3 cells and up), end a ray once its remaining path is proved empty on the two-level
                          map (dilated 8^3 tiles, 64^3 regions) */
    int32_t order;     /* 1: dispatch spec, shadow, AO; 2: shadow, AO, spec */
    int32_t tile_w;    /* tile shape: pixels per tile row (tile_px = runs of pixels; 4 or 8 = image blocks,
                          used when the G-buffer's width * height == npix) */
    int32_t grab;      /* tiles a warp takes per work-queue access: 1, 2 or 4 */
} vxl_tuning;
vxl_status vxl_ctx_set_tuning(vxl_ctx* ctx, const vxl_tuning* t);
vxl_status vxl_ctx_get_tuning(const vxl_ctx* ctx, vxl_tuning* out);

/* ------------------------------------------------------------------ grid
 * Replaces ShadowVoxSystem's R8Uint volume (ShadowVoxSystem.cpp:55-79,
 * ShadowVoxSystem.h:29 GetVolumeImage). Storage: 1 bit per fine voxel in
 * 4x4x4 bricks, one uint64 each (bit (x&3) + 4*(y&3) + 16*(z&3)), bricks in
 * x-fastest order, plus one zero brick of padding on the + side of every
 * axis; and a tile map with 1 bit per 8^3 tile (2x2x2 bricks), x-fastest.
 * nx, ny, nz must be even and in [2, 32768].
 *
 * Derived from the words, for the occlusion traversal: the trace layout. The
 * same 4^3 bricks, with every cell shifted by +4 on each axis (cell x is at
 * x + 4), 2^trace_lbx bricks per x row and 2^trace_lby per y column (powers
 * of two, padding included) and trace_bz z slabs, brick (i, j, k) at word
 * i + (j << trace_lbx) + (k << (trace_lbx + trace_lby)). A cell holds the
 * grid's voxel inside [0, n), 0 in the DDA's two extra cells n and n+1
 * (Light.frag:53 tests up to 2S+1 inclusive) and 1 on the border just
 * outside those bounds (a coordinate equal to -1 or n+2). The traversal then
 * needs no bounds test: the first cell outside the bounds reads as set, and
 * is reported as the bounds exit. Present when every bit address fits in 37
 * bits (trace_words != NULL; cubic grids up to about 4000^3 cells),
 * trace_wide = 1 when they need more than 32 (cubic grids from about 1020^3;
 * such a layout takes about 4x the grid's words, 4.3 GB at 2048^3; where it
 * cannot be allocated the grid has none and is traced on its own words);
 * rebuilt with the tile map. */
typedef struct vxl_grid_desc {
    int32_t nx, ny, nz;        /* fine dimensions */
    int32_t bx, by, bz;        /* 4^3 bricks per axis, padding included */
    int32_t tx, ty, tz;        /* 8^3 tiles per axis */
    uint64_t* words;           /* device: bx*by*bz uint64 */
    size_t words_bytes;
    uint32_t* tile_mask;       /* device: 1 bit per tile, "tile has any voxel set" */
    size_t tile_mask_bytes;
    uint64_t* trace_words;     /* device: the trace layout, or NULL */
    size_t trace_words_bytes;
    int32_t trace_lbx, trace_lby, trace_bz;
    int32_t trace_wide;        /* 1: bit addresses above 32 bits (see above) */
} vxl_grid_desc;

vxl_status vxl_grid_create(vxl_ctx* ctx, int nx, int ny, int nz, vxl_grid** out);
/* frees the grid's device memory; allowed after its context was destroyed
 * (no other call may use a grid whose context is gone) */
vxl_status vxl_grid_destroy(vxl_grid* grid);
vxl_status vxl_grid_describe(const vxl_grid* grid, vxl_grid_desc* out);
/* zero every voxel */
vxl_status vxl_grid_clear(vxl_grid* grid, void* stream);
/* rebuild the tile occupancy map and the trace layout after the words
 * changed (the trace entry points read them); every call of this library
 * that writes a grid (vxl_voxelize, vxl_voxelize_noalloc, the imports, the
 * scene generators, vxl_grid_clear) rebuilds them itself */
vxl_status vxl_grid_build_bricks(vxl_grid* grid, void* stream);
/* Reference layout in/out: device bytes [nz/2][ny/2][nx/2], byte x+y*sx+z*sx*sy,
 * bit (x&1)|(y&1)<<1|(z&1)<<2 (ShadowVoxSystem.cpp:82-94, Light.frag:14-20). */
vxl_status vxl_grid_import_r8(vxl_grid* grid, const uint8_t* d_bytes, void* stream);
vxl_status vxl_grid_export_r8(const vxl_grid* grid, uint8_t* d_bytes, void* stream);
/* Dense palette-index volume, device uint8 [nz][ny][nx]: voxel set where
 * index >= opaque_min (16 in the reference: ShadowVoxSystem.cpp:145). A grid
 * with a palette plane also keeps the index's low 4 bits of every set voxel
 * (0 for empty ones). */
vxl_status vxl_grid_import_palette(vxl_grid* grid, const uint8_t* d_palette, int opaque_min, void* stream);
/* 4-bit palette plane beside the occupancy bits (4 bits per fine voxel, 32
 * bytes per 4^3 brick: 64 MiB for 512^3), allocated zeroed on the first call.
 * No counterpart in the reference, whose ShadowVox image holds occupancy
 * only: the plane carries a grid's palette indices with it, and the occlusion
 * traversal never reads it. Written by vxl_grid_import_palette and
 * vxl_scene_palette, zeroed by vxl_grid_clear; the voxelizer changes
 * occupancy only. */
vxl_status vxl_grid_palette_alloc(vxl_grid* grid);
/* the plane as a dense device uint8 volume [nz][ny][nx] of indices 0..15;
 * VXL_ERR_NOT_SUPPORTED when the grid has no plane */
vxl_status vxl_grid_export_palette(const vxl_grid* grid, uint8_t* d_palette, void* stream);
/* number of set voxels (synchronous) */
vxl_status vxl_grid_count(const vxl_grid* grid, uint64_t* out, void* stream);

/* ------------------------------------------------------------- traversal */
typedef enum vxl_mode {
    VXL_MODE_DDA = 0,          /* raycastShadowVolume, Light.frag:29-81 (exact DDA) */
    VXL_MODE_SPARSE = 1,       /* raycastShadowVolumeSparse, Light.frag:131-173 */
    VXL_MODE_SUPERSPARSE = 2   /* raycastShadowVolumeSuperSparse, Light.frag:175-217 */
} vxl_mode;

/* per-ray result record (24 bytes) */
typedef struct vxl_ray_record {
    int32_t vx, vy, vz;  /* hit cell, or last cell tested on a miss */
    float t;             /* DDA: best_t of the hit cell (Light.frag:57,62); marchers: returned distance */
    int32_t steps;       /* occupancy fetches made */
    int32_t flags;       /* VXL_RF_* */
} vxl_ray_record;

enum {
    VXL_RF_HIT = 1,
    VXL_RF_SELX = 2, VXL_RF_SELY = 4, VXL_RF_SELZ = 8, /* DDA axis select at the hit: normal = -sign(dir)*sel */
    VXL_RF_EXIT_BOUNDS = 16,
    VXL_RF_EXIT_STEPS = 32,
    VXL_RF_EXIT_MAXT = 64,
    VXL_RF_COARSE = 128
};

/* Trace n independent rays. Device rays float[n][7] = origin xyz, dir xyz,
 * maxt (DDA) or dist (marchers). Device records[n]. Direct replacement for
 * calls to raycastShadowVolume / ...Sparse / ...SuperSparse (Light.frag:29,131,175). */
vxl_status vxl_trace_rays(vxl_ctx* ctx, const vxl_grid* grid, const float* d_rays, int64_t n, vxl_mode mode,
                          vxl_ray_record* d_records, void* stream);

/* G-buffer: device pointers, fine-voxel units. A pixel whose normal is
 * (0,0,0) is sky: nothing is traced and its outputs are 1 (spec_t = spec_len). */
typedef struct vxl_gbuffer {
    const float* pos;    /* [npix][3] surface position */
    const float* nrm;    /* [npix][3] unit surface normal */
    const float* rough;  /* [npix] roughness, or NULL (then params.default_rough) */
    int64_t npix;
    int32_t width, height; /* informational; npix is authoritative */
} vxl_gbuffer;

/* DDA-mode ray generation (this library's definition; the reference's passes
 * fire one jittered Sparse/SuperSparse ray each, see vxl_light_*):
 *  origin  O = pos + nrm*bias
 *  shadow  dir = light_dir, maxt = shadow_len                      -> shadow = hit ? 0 : 1
 *  AO k    cosine-weighted (cosineSampleHemisphere, LightAmbient.frag:81-87) in the
 *          tangent frame of LightAmbient.frag:112-113, u = PCG(seed, pixel, 64+2k / 65+2k),
 *          maxt = ao_len -> ao = mean_k (min(t_k, ao_len)/ao_len)^2, ao_vis = mean_k miss
 *  spec j  GGX half-vector (alpha = rough^2) about the normal, u = PCG(seed, pixel, 2j / 2j+1),
 *          reflection of V = normalize(cam_pos - pos), maxt = spec_len
 *          -> spec = mean_j miss, spec_t = mean_j (hit ? t : spec_len)
 * Same layout as the oracle's params struct. */
typedef struct vxl_trace_params {
    float light_dir[3];   /* unit vector toward the light */
    float cam_pos[3];     /* camera position (spec rays) */
    float bias;           /* origin offset along the normal */
    float shadow_len;     /* 100 in the reference's DDA call (LightAmbient.frag:163) */
    float ao_len;
    float spec_len;       /* 256 in the reference's DDA call (LightReflection.frag:104) */
    float default_rough;
    int32_t n_shadow;     /* 0 or 1 */
    int32_t n_ao;         /* 0..64 */
    int32_t n_spec;       /* 0..8 */
    uint32_t seed;
    int32_t mode;         /* VXL_MODE_DDA */
} vxl_trace_params;

/* Outputs: device float[npix] each, any may be NULL. records, if not NULL,
 * is device vxl_ray_record[npix * (n_shadow + n_ao + n_spec)] in the order
 * shadow, AO 0..n_ao-1, spec 0..n_spec-1 per pixel. */
typedef struct vxl_outputs {
    float* shadow;
    float* ao;
    float* ao_vis;
    float* spec;
    float* spec_t;
    vxl_ray_record* records;
} vxl_outputs;

/* The drop-in for the traversal consumers of LightAmbientPipeline::Use /
 * LightReflectionPipeline::Use (LightAmbientPipeline.h:35, LightReflectionPipeline.h:34):
 * G-buffer and grid in, occlusion buffers out. */
vxl_status vxl_trace_occlusion(vxl_ctx* ctx, const vxl_grid* grid, const vxl_gbuffer* gbuf,
                               const vxl_trace_params* params, const vxl_outputs* out, void* stream);

/* The two ViewBuffer matrices a light pass reads to place a pixel (ViewData,
 * Sources/Graphics/Renderer/View.h:16-31; Common.frag:45-71), column-major as
 * glm stores them. */
typedef struct vxl_view {
    float inverse_view[16];        /* InverseViewMatrix */
    float inverse_projection[16];  /* InverseProjectionMatrix */
} vxl_view;

/* vxl_trace_occlusion with the surface positions rebuilt from the G-buffer's
 * linear depth the way LightAmbient places a pixel (LightAmbient.vert:32-36,
 * LightAmbient.frag:136-150), replacing the pass's own G-buffer reads. For
 * texel (i, j) of a width x height image (row j, row 0 first in memory):
 *   ndc    = ((i + 0.5)*2/width - 1, 1 - (j + 0.5)*2/height)   (the pass's flipped UV)
 *   farvec = (inverse_projection * (ndc, 1, 1)).xyz / w
 *   pos    = farvec * (depth * (1 + 1/4096))                    (FAR = 4096)
 *   wcp    = (inverse_view * (pos, 1)).xyz * 10                 (fine-voxel units)
 * each product adding the column terms in column order, fp32, no FMA.
 * Texels with !(depth < 0.999) are sky: outputs as for a zero normal.
 * d_depth: float[height][width], (w - NEAR)/(FAR - NEAR) as GeometryVoxel.frag:169
 * writes it; d_nrm: float[height*width][3] world normals; d_rough optional.
 * Outputs per texel. Uses a context workspace of 24 bytes per texel. */
vxl_status vxl_trace_occlusion_from_depth(vxl_ctx* ctx, const vxl_grid* grid, const float* d_depth,
                                          const float* d_nrm, const float* d_rough, int32_t width, int32_t height,
                                          const vxl_view* view, const vxl_trace_params* params,
                                          const vxl_outputs* out, void* stream);

/* Same, with the G-buffer held in host memory (pinned or pageable).
 * When every given buffer is pinned host memory mapped into the device's
 * address space (cudaHostAlloc / cudaMallocHost / registered memory), the
 * kernel reads the G-buffer and writes the outputs there directly over the
 * CPU-GPU link. Otherwise the library copies through its context staging
 * buffers in a pipeline of pixel chunks, traces, and copies the outputs back.
 * Both give the same results. Synchronous on `stream`. Host outputs may be
 * NULL. */
vxl_status vxl_trace_occlusion_host(vxl_ctx* ctx, const vxl_grid* grid, const float* h_pos, const float* h_nrm,
                                    const float* h_rough, int64_t npix, const vxl_trace_params* params,
                                    float* h_shadow, float* h_ao, float* h_ao_vis, float* h_spec, float* h_spec_t,
                                    void* stream);

/* ------------------------------------------------------------ batched form
 * Many scenes (grids of any size, G-buffers of any size) traced by ONE
 * persistent launch: all scenes' pixel tiles share one work queue, so large
 * and small scenes keep every SM busy (no reference counterpart: the engine
 * traces one view per frame). The plan uploads the scene table once and
 * captures the launch (queue reset + kernel) in a CUDA graph; each run
 * replays the graph. The items' buffers must stay valid while the batch
 * exists. Runs of the same batch must not overlap (they share one queue). */
typedef struct vxl_batch vxl_batch;
typedef struct vxl_batch_item {
    const vxl_grid* grid;
    vxl_gbuffer gbuf;
    vxl_trace_params params;
    vxl_outputs out;        /* records must be NULL in a batch */
} vxl_batch_item;

/* use_graph: 1 = capture the launch in a CUDA graph (run replays it), 0 = launch directly */
vxl_status vxl_batch_create(vxl_ctx* ctx, const vxl_batch_item* items, int n, int use_graph, vxl_batch** out);
vxl_status vxl_batch_run(vxl_batch* batch, void* stream);
vxl_status vxl_batch_destroy(vxl_batch* batch);
/* total pixel tiles and traced-ray upper bound (pixels x rays per pixel) of a batch */
vxl_status vxl_batch_info(const vxl_batch* batch, int64_t* tiles, int64_t* rays);

/* ------------------------------------------------ reference light passes
 * Bit-exact replacements for the live shader passes (Sparse/SuperSparse
 * marchers with the reference's jitter). `noise` is the per-pixel blue-noise
 * texel the shader reads with getNoise() (device float[npix][4]).
 * records (optional) get one record per traced ray. */

/* LightAmbient.frag:148-173. wcp = world position in fine units, i.e.
 * (InverseView*pos).xyz*10 (:150); depth = linear depth (:136).
 * Out: shadow (:167-169) and the ambient irradiance scalar d*d*0.05 (:121-125). */
vxl_status vxl_light_ambient(vxl_ctx* ctx, const vxl_grid* grid, const float* d_wcp, const float* d_nrm,
                             const float* d_depth, const float* d_noise, int64_t npix, float* d_shadow,
                             float* d_irradiance, vxl_ray_record* d_records, void* stream);
/* LightReflection.frag:92-113. view_r = (InverseView*vec4(R,0)).xyz before
 * normalisation (:92). Out: t of raycastShadowVolumeSparse (256 = miss, :121). */
vxl_status vxl_light_reflection(vxl_ctx* ctx, const vxl_grid* grid, const float* d_wcp, const float* d_nrm,
                                const float* d_view_r, const float* d_rough, const float* d_noise, int64_t npix,
                                float* d_t, vxl_ray_record* d_records, void* stream);
/* LightPoint.frag:234-267 (spot = 0) / LightSpot.frag:83-117 (spot = 1).
 * wpos in world units. Pixels beyond `range` are discarded (output untouched). */
vxl_status vxl_light_point(vxl_ctx* ctx, const vxl_grid* grid, const float* d_wpos, const float* d_nrm,
                           const float* d_noise, int64_t npix, const float light_pos[3], float range, int spot,
                           float* d_shadow, vxl_ray_record* d_records, void* stream);

/* Fused point / spot shadows for up to 64 lights (the per-light passes of
 * LightPointPipeline / LightSpotPipeline, LightPoint.frag:94-129,
 * LightSpot.frag:83-117, in one launch). For pixel i and light l: in range
 * when |light.pos - wpos| <= range (the pass's discard test); then the same
 * jittered shadow ray vxl_light_point traces for that light. Out (device
 * uint64 per pixel): bit l of d_lit = in range and unshadowed; bit l of
 * d_in_range (optional) = in range. Host light table. Uses a context
 * workspace of 16 bytes per pixel plus 256 KB (the light grid and the list
 * of pairs in range). */
typedef struct vxl_light {
    float pos[3];      /* world units */
    float range;
    int32_t spot;      /* 0: point light (Sparse marcher), 1: spot light (SuperSparse marcher) */
    int32_t pad[3];
} vxl_light;
vxl_status vxl_light_points(vxl_ctx* ctx, const vxl_grid* grid, const float* d_wpos, const float* d_nrm,
                            const float* d_noise, int64_t npix, const vxl_light* lights, int nlights,
                            uint64_t* d_lit, uint64_t* d_in_range, void* stream);

/* Temporal accumulation of the lighting buffer (LightTAA.frag:37-141): the
 * pass after the occlusion terms. Device fp32 images, [height][width][c]
 * row-major, sampled with this library's sampler for the pass (bilinear,
 * clamp to edge, texel centres at (i + 0.5) / size) at UV = ((px + .5) / W,
 * (py + .5) / H); sin/cos are the library's own. Out: float[npix][4]
 * (accumulated rgb, variance), the next frame's last_light. The 4-channel
 * images must be 16-byte aligned and motion 8-byte aligned. Uses a context
 * workspace of 64 bytes per pixel (the texels the taps read, regrouped). */
typedef struct vxl_taa_frame {
    const float* light;       /* [4] this frame's lighting */
    const float* last_light;  /* [4] the previous output (rgb, variance in a) */
    const float* color;       /* [3] albedo */
    const float* normal;      /* [3] world normal */
    const float* material;    /* [4] */
    const float* depth;       /* [1] depth in [0, 1]; 1 = sky (copied through) */
    const float* motion;      /* [2] UV offset to the previous frame */
    const float* noise;       /* [4] blue-noise texel of getNoise() (x is used) */
    int32_t width, height;
} vxl_taa_frame;
vxl_status vxl_light_taa(vxl_ctx* ctx, const vxl_taa_frame* frame, float* d_out, void* stream);

/* ------------------------------------------------------------ voxelizer */
typedef struct vxl_model {
    const uint8_t* data;   /* device palette indices [sz][sy][sx] (VoxAsset::PixelAt, VoxAsset.h:52-56) */
    int32_t sx, sy, sz;
} vxl_model;

typedef enum vxl_op { VXL_OP_CLEAR = 0, VXL_OP_SET = 1 } vxl_op;

/* One placement: matrix = World * translate(-Pivot), column-major 4x4
 * (ShadowVoxSystem.cpp:134-140). Every model voxel with index >= 16 maps to
 * fine voxel ivec3((o + x*dx + y*dy + z*dz)*10), o = matrix[3], d* = matrix[0..2]*0.1,
 * and is set or cleared there (ShadowVoxSystem.cpp:142-155, SetVolumeAt :82-94). */
typedef struct vxl_instance {
    float matrix[16];
    int32_t model;
    int32_t op;            /* vxl_op */
} vxl_instance;

/* Apply instances (host array) in array order: the result equals applying
 * them one after another, as the reference's single-threaded loop does.
 * aabb (optional, device int32[n][6]): per instance min xyz, max xyz of every
 * mapped fine voxel, in or out of the grid, min/max-ed into the values the
 * caller initialised it with (the reference starts them at (S-1,S-1,S-1) and
 * (0,0,0), ShadowVoxSystem.cpp:128-132). Rebuilds the tile map. */
vxl_status vxl_voxelize(vxl_ctx* ctx, vxl_grid* grid, const vxl_model* models, int nmodels,
                        const vxl_instance* instances, int n, int32_t* d_aabb, void* stream);

/* One moved entity (ShadowVoxSystem::OnUpdate): previous and current world
 * matrices (column-major), pivot, model index. */
typedef struct vxl_entity {
    float prev_world[16];
    float world[16];
    float pivot[3];
    int32_t model;
} vxl_entity;

/* ShadowVoxSystem::OnUpdate (ShadowVoxSystem.cpp:116-191): entities in order,
 * each clears its previous pose then sets its current one. regions (optional,
 * host int32[n][6]) receives the dirty byte region x,y,z,w,h,d per entity
 * (:180-190), or -1s when the reference would push none. Synchronous. */
vxl_status vxl_shadowvox_update(vxl_ctx* ctx, vxl_grid* grid, const vxl_model* models, int nmodels,
                                const vxl_entity* entities, int n, int32_t* h_regions, void* stream);
/* ShadowVoxSystem::OnVoxDestroyed (ShadowVoxSystem.cpp:7-53): clears the
 * model at `world` (no -Pivot, as the reference). region as above. */
vxl_status vxl_vox_destroyed(vxl_ctx* ctx, vxl_grid* grid, const vxl_model* model, const float world[16],
                             int32_t* h_region, void* stream);

/* vxl_voxelize for callers that cannot allocate device memory: an engine or
 * render loop that commits its device memory up front, code that runs on a
 * pool-managed budget, or updates issued between frames where a cudaMalloc
 * would stall the GPU. This entry point has no counterpart in the reference
 * (whose voxelizer runs on the CPU); it exists for such callers only.
 *  - It allocates nothing: no context, no grid handle, no cudaMalloc/cudaFree
 *    and no heap allocation. The caller passes the grid descriptor (device
 *    words and tile map in the vxl_grid_desc layout, e.g. from
 *    vxl_grid_describe), the models and instances (host arrays, as for
 *    vxl_voxelize) and the optional device aabb output.
 *  - Its scratch is a fixed table in the library's static device memory
 *    (about 1.2 MiB, held on every GPU that loads libvxl until the process
 *    exits): at most VXL_NOALLOC_MAX_INSTANCES instances and
 *    VXL_NOALLOC_MAX_MODELS models per call; larger calls are rejected with
 *    VXL_ERR_OUT_OF_RANGE.
 *  - The first call on a device looks up the table's device address (once per
 *    device, with that device current); make that first call before any stream
 *    capture. The address is kept for the life of the process and belongs to
 *    the device's primary context (the one the CUDA runtime uses): calls must
 *    run in that context, and not after cudaDeviceReset on that device.
 *  - All calls share the one table: calls that overlap on the GPU (other
 *    streams, other host threads) race and must be serialised by the caller.
 *  - Same result as vxl_voxelize; returns when the update is complete. */
#define VXL_NOALLOC_MAX_INSTANCES 16384
#define VXL_NOALLOC_MAX_MODELS 4096
vxl_status vxl_voxelize_noalloc(const vxl_grid_desc* grid, const vxl_model* models, int nmodels,
                                const vxl_instance* instances, int n, int32_t* d_aabb, void* stream);

/* ------------------------------------------- differentiable soft variant
 * No counterpart in the reference (its grid is binary). A soft grid is a
 * device float4 per fine voxel (opacity, albedo r, g, b), x fastest, dims
 * nx, ny, nz even. Each G-buffer pixel with a non-zero normal traces
 * n_shadow (0 or 1) rays along light_dir and n_ao cosine-weighted AO rays
 * (the directions vxl_trace_occlusion's DDA mode uses for AO samples), all
 * from pos + bias * nrm. A ray walks exactly the cells the reference DDA
 * (Light.frag:29-81) visits up to t = len on an empty grid, cells outside the
 * data being empty, and stops early once its transmittance is below 2^-40.
 * With a = clamp(opacity, 0, 1 - 2^-12):
 *   shadow ray  T_sh = prod (1 - a_i)
 *   AO ray k    T_k = prod (1 - a_i),  C_k = sum_i (prod_{l<i} (1 - a_l)) a_i albedo_i
 *   light[c]  = k_sun T_sh + k_amb / n_ao * sum_k (T_k + C_k[c])
 *   image[c]  = albedo_s[c] * light[c]
 * where s = floor(pos - 0.5 nrm) is the surface voxel (no contribution when it
 * lies outside the grid). */
typedef struct vxl_soft_params {
    float light_dir[3];
    float bias;
    float len;     /* maxt of every ray */
    float k_sun;
    float k_amb;
    int32_t n_shadow; /* 0 or 1 */
    int32_t n_ao;     /* n_shadow + n_ao in [1, 32] */
    uint32_t seed;
} vxl_soft_params;

/* Forward: image and light are device float[npix][3]; light (optional, may be
 * NULL) is what vxl_trace_soft_bwd needs for the albedo gradient of the
 * surface voxel. Deterministic. */
vxl_status vxl_trace_soft_fwd(vxl_ctx* ctx, const float* d_soft, int nx, int ny, int nz, const vxl_gbuffer* gbuf,
                              const vxl_soft_params* p, float* d_image, float* d_light, void* stream);
/* Adjoint: ACCUMULATES dL/d(opacity, albedo) into d_grad_soft (float4 per
 * voxel, same layout as d_soft) given d_grad_image = dL/dimage and the light
 * from the forward call on the same inputs. The rays are walked again (no
 * per-ray state is kept between the calls); float atomics make the low bits
 * of the sum order-dependent. The opacity clamp's derivative is 1 on the
 * closed interval [0, 1 - 2^-12]. */
vxl_status vxl_trace_soft_bwd(vxl_ctx* ctx, const float* d_soft, int nx, int ny, int nz, const vxl_gbuffer* gbuf,
                              const vxl_soft_params* p, const float* d_grad_image, const float* d_light,
                              float* d_grad_soft, void* stream);

/* ------------------------------------------------- primary visibility
 * Replaces GeometryVoxelPipeline::Use (GeometryVoxelPipeline.h:50-70) with
 * GeometryVoxel.{vert,frag}: per pixel, the nearest voxel hit over all
 * instances, as a G-buffer for vxl_trace_occlusion. */
/* A VoxAsset image with its mips (VoxAsset.h:26-31, VoxAsset.cpp:3-63):
 * device R8 palette indices, mip m of size max(1, s >> m) per axis
 * (p > 1 ? p / 2 : 1), x fastest. VoxAsset rounds sizes up to multiples of 4;
 * here each size must be >= 4. */
typedef struct vxl_volume {
    const uint8_t* mip[3];
    int32_t sx, sy, sz;
    int32_t pad;
} vxl_volume;
/* Build mips 1 and 2 from mip 0 (VoxAsset::Upload's first-non-zero-child rule). */
vxl_status vxl_volume_build_mips(vxl_ctx* ctx, const uint8_t* d_mip0, int sx, int sy, int sz, uint8_t* d_mip1,
                                 uint8_t* d_mip2, void* stream);
/* GeometryVoxelPipeline::Cmd (GeometryVoxelPipeline.h:30-36): world matrix
 * (column-major; WorldMatrix * translate(-Pivot), WorldRenderer.cpp:213-218)
 * mapping volume voxel v to world units as world = R (v * 0.1) + t (its
 * projective row is ignored), the volume (index into the volume table) and
 * the palette index (passed through, not used here). */
typedef struct vxl_voxcmd {
    float world[16];
    int32_t volume;
    int32_t palette;
} vxl_voxcmd;
/* Pinhole camera in world units: pixel (px, py) looks along
 * normalize(fwd + right * u + up * v), u = ((px + .5) * 2 / W - 1) * tan_half_fov * W / H,
 * v = (1 - (py + .5) * 2 / H) * tan_half_fov, fwd = normalize(target - pos),
 * right = normalize(cross(fwd, (0,1,0))), up = cross(right, fwd) (as
 * vxl_scene_gbuffer). frame = GetFrame() (dithers glass voxels, palette < 16). */
typedef struct vxl_camera {
    float pos[3];
    float target[3];
    float tan_half_fov;
    int32_t width, height;
    int32_t frame;
} vxl_camera;
/* Outputs, device, [W*H] row-major; NULL to skip (pos and nrm are required).
 * Sky pixels: pos = nrm = 0, depth = 0, material = 0, instance = -1. */
typedef struct vxl_primary_out {
    float* pos;          /* [npix][3] hit position in fine-voxel units (world * 10) */
    float* nrm;          /* [npix][3] world normal */
    float* depth;        /* [npix] view depth along fwd, world units */
    int32_t* material;   /* [npix] palette index of the hit voxel */
    int32_t* instance;   /* [npix] index of the hit command */
} vxl_primary_out;
/* Per pixel: for every command whose volume box [0, dims] the pixel ray
 * (moved into the volume's space: local = R^-1 (p - t) * 10) enters,
 * clipToAABB + intersectVolume (GeometryVoxel.frag:50-125, LOD and
 * transparency on, UV = ((px + .5) * 2 / W - 1, (py + .5) * 2 / H - 1)); the
 * nearest hit by view depth wins, ties to the lower command index. Host
 * arrays, copied before the call returns; the frame is queued on `stream`
 * without waiting for it. Screen-bin lists are sized from the previous
 * frame's; a frame that outgrows them scans every command (same result). */
vxl_status vxl_trace_primary(vxl_ctx* ctx, const vxl_volume* volumes, int nvolumes, const vxl_voxcmd* cmds, int ncmds,
                             const vxl_camera* camera, const vxl_primary_out* out, void* stream);

/* ---------------------------------------------------------- scene assets
 * Host-side readers for the reference's shipped scenes (no device work). */
/* Asset GUID of a mod-relative path such as "default/FarmHouse/0.v":
 * Assets::Hash (Assets.h:207-210), std::hash<std::string> as the shipped
 * files were written with it (MSVC: FNV-1a 64). */
uint64_t vxl_asset_guid(const char* mod_path);
/* .p palette (PalleteAsset::Serialize, PalleteAsset.h:63-69): 256 VoxMaterial
 * of 7 bytes (r, g, b, a, roughness, metallic, emit) into h_materials[1792]. */
vxl_status vxl_read_palette(const char* path, uint8_t* h_materials);
/* TransformSystem::RealculateMatrix (TransformSystem.cpp:124-135):
 * out = parent * T(pos) Rz(rot.z) Ry(rot.y) Rx(rot.x) S(scale), column-major,
 * radians; parent NULL = identity. glm's operation order, C library cos/sin. */
vxl_status vxl_transform_matrix(const float pos[3], const float rot[3], const float scale[3], const float* parent,
                                float out[16]);
/* A spawned .pf prefab (PrefabAsset::Spawn, PrefabAsset.cpp:30-120) without a
 * world: mods_dir holds the mod folders ("Assets/Mods"), mod_path names the
 * prefab ("default/FarmHouse.pf"). GUIDs resolve to files under mods_dir by
 * vxl_asset_guid of their mod-relative paths; nested prefab instances spawn
 * under the instance entity's parent and take its components. Each entity
 * with a VoxRenderer whose Vox GUID is not null gives one renderer, in
 * creation order; volumes and palettes are listed once each, in order of
 * first use. A non-null GUID that resolves to no file is an error. */
typedef struct vxl_prefab vxl_prefab;
typedef struct vxl_prefab_renderer {
    float world[16];   /* the entity's WorldMatrix; voxelize / draw with world * translate(-pivot) */
    float pivot[3];
    int32_t volume;    /* index into the prefab's volumes */
    int32_t palette;   /* index into the prefab's palettes */
    int32_t entity;    /* creation order of the entity */
} vxl_prefab_renderer;
vxl_status vxl_prefab_load(const char* mods_dir, const char* mod_path, vxl_prefab** out);
vxl_status vxl_prefab_info(const vxl_prefab* prefab, int32_t* n_renderers, int32_t* n_volumes, int32_t* n_palettes);
vxl_status vxl_prefab_renderer_at(const vxl_prefab* prefab, int i, vxl_prefab_renderer* out);
/* volume i: sizes, host data (owned by the prefab, [sz][sy][sx]) and GUID */
vxl_status vxl_prefab_volume_at(const vxl_prefab* prefab, int i, int32_t* sx, int32_t* sy, int32_t* sz,
                                const uint8_t** h_data, uint64_t* guid);
vxl_status vxl_prefab_palette_at(const vxl_prefab* prefab, int i, const uint8_t** h_materials, uint64_t* guid);
vxl_status vxl_prefab_destroy(vxl_prefab* prefab);

/* MagicaVoxel .vox import as the engine's importer does it
 * (Sources/Editor/Importer/VoxImporter.cpp): one model per shape instance of
 * the scene graph, in the importer's depth-first order, each with the name,
 * size (a multiple of 4 per axis) and voxel bytes the importer writes to
 * <name>.v, and the world position of its entity; and the 256-material
 * palette (7 bytes each: r, g, b, a, roughness, metallic, emit) it writes to
 * the .p file. Host memory, owned by the scene. */
typedef struct vxl_vox_scene vxl_vox_scene;
vxl_status vxl_vox_load(const char* path, vxl_vox_scene** out);
vxl_status vxl_vox_info(const vxl_vox_scene* scene, int32_t* n_models);
/* name: NUL-terminated, truncated to name_cap bytes; size: x, y, z of the
 * .v file (data is x fastest, valid until vxl_vox_destroy); position: world
 * units */
vxl_status vxl_vox_model_at(const vxl_vox_scene* scene, int32_t i, char* name, int32_t name_cap, int32_t size[3],
                            const uint8_t** h_data, float position[3]);
vxl_status vxl_vox_palette(const vxl_vox_scene* scene, uint8_t* h_materials /* 256 * 7 bytes */);
vxl_status vxl_vox_destroy(vxl_vox_scene* scene);

/* .v asset reader (VoxAsset::Serialize, VoxAsset.h:42-50): u32 sx,sy,sz then
 * sx*sy*sz bytes. Query with data == NULL to get the sizes, then read into a
 * host buffer of sx*sy*sz bytes. */
vxl_status vxl_read_v(const char* path, int32_t* sx, int32_t* sy, int32_t* sz, uint8_t* h_data, size_t capacity);

/* ---------------------------------------------------- synthetic scenes
 * Seeded generators for benchmarks and tests (not part of the reference). */
/* OR into the grid: voxels where the 3-octave value noise at the voxel
 * centre exceeds thresh, plus the slab y < ground_y */
vxl_status vxl_scene_noise(vxl_ctx* ctx, vxl_grid* grid, uint32_t seed, float thresh, float freq, int ground_y,
                           void* stream);
/* Soft grid (float4 per voxel, layout of vxl_trace_soft_fwd): opacity =
 * sigmoid(sharpness * (noise - thresh)) with the noise of vxl_scene_noise
 * (so opacity > 0.5 exactly where vxl_scene_noise sets a voxel, up to
 * rounding at the threshold), opacity 1 in the slab y < ground_y; albedo
 * r, g, b uniform in [0, 1) from a hash of (albedo_seed, voxel, channel). */
vxl_status vxl_scene_soft(vxl_ctx* ctx, float* d_soft, int nx, int ny, int nz, uint32_t seed, float thresh,
                          float sharpness, float freq, int ground_y, uint32_t albedo_seed, void* stream);
/* OR into the grid: heightfield terrain, voxel (x, y, z) set where
 * (float)y < h(x, z) = base + amplitude * fbm(x + 0.5, 0.5, z + 0.5), fbm the
 * octave noise of vxl_scene_noise with `octaves` octaves at frequency freq
 * (values in [0, 1]). d_height (optional, device float[nz][nx]) receives h. */
vxl_status vxl_scene_terrain(vxl_ctx* ctx, vxl_grid* grid, uint32_t seed, float base, float amplitude, float freq,
                             int octaves, float* d_height, void* stream);
/* OR into the grid: nboxes seeded axis-aligned boxes with edges in [smin, smax] */
vxl_status vxl_scene_boxes(vxl_ctx* ctx, vxl_grid* grid, uint32_t seed, int nboxes, int smin, int smax, void* stream);
/* seeded palette plane for the grid's set voxels: index 1 + pcg(seed + pcg(64*brick + bit)) % 15, 0 for empty
 * voxels (the grid needs a plane: vxl_grid_palette_alloc) */
vxl_status vxl_scene_palette(vxl_ctx* ctx, vxl_grid* grid, uint32_t seed, void* stream);
/* primary-visibility G-buffer from a pinhole camera (entry-face DDA):
 * device pos/nrm float[W*H][3], rough float[W*H] */
vxl_status vxl_scene_gbuffer(vxl_ctx* ctx, const vxl_grid* grid, const float cam[3], const float target[3],
                             float tan_half_fov, int W, int H, uint32_t seed, float* d_pos, float* d_nrm,
                             float* d_rough, void* stream);

/* ------------------------------------------------------------ diagnostics
 * No counterpart in the reference. The L2 read bandwidth of this GPU: a
 * kernel streams a device buffer of `bytes` (at least 1 MiB, a multiple of
 * 16; it allocates it and frees it again), small enough to stay in L2,
 * `reps` timed times after three untimed ones; the best time gives GB/s.
 * Synchronous. The occlusion benchmark reports its roofline against it for
 * grids that stay in L2. */
vxl_status vxl_diag_l2_read_gbs(vxl_ctx* ctx, size_t bytes, int reps, double* best_gbs, double* best_ms);

#ifdef __cplusplus
}
#endif
#endif /* VXL_H */
