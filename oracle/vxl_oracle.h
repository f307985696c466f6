/*
 * vxl_oracle.h — CPU restatement of VoxelEngine's voxel-lighting path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA
 * path in voxelengine_gb300/: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it. The product never
 * links or calls it.
 *
 * Parity pin: the traversal functions (getVolumeAt, raycastShadowVolume,
 * raycastShadowVolumeSparse/SuperSparse, cosineSampleHemisphere) and the
 * ShadowVox voxelizer are checked bit-for-bit against the reference's own
 * sources compiled on the host by oracle/ref/Makefile (tests/test_oracle_ref.py),
 * and against the golden vectors generated from that build (tests/golden/).
 *
 * Grid layout used here is the reference's ShadowVox layout: an R8 3-D image
 * of sx*sy*sz bytes, byte (x,y,z) at x + y*sx + z*sx*sy, each byte holding a
 * 2x2x2 block of fine voxels, bit = (x&1) | (y&1)<<1 | (z&1)<<2
 * (Sources/World/Systems/ShadowVoxSystem.cpp:82-94, Sources/Shaders/lib/Light.frag:14-27).
 * All arithmetic is IEEE fp32 without contraction (-ffp-contract=off).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-ray result, same layout as vxl_ray_record in include/vxl.h. */
typedef struct vo_rec {
    int32_t vx, vy, vz; /* hit cell (fine voxel), or last cell tested on a miss */
    float t;            /* DDA: best_t at the hit (Light.frag:57); marchers: returned distance */
    int32_t steps;      /* number of occupancy fetches */
    int32_t flags;      /* VO_F_* */
} vo_rec;

enum {
    VO_F_HIT = 1,
    VO_F_SELX = 2, VO_F_SELY = 4, VO_F_SELZ = 8, /* DDA axis select at the hit */
    VO_F_EXIT_BOUNDS = 16,
    VO_F_EXIT_STEPS = 32,
    VO_F_EXIT_MAXT = 64,
    VO_F_COARSE = 128,    /* marcher hit in its 2^3 coarse phase */
};

enum { VO_MODE_DDA = 0, VO_MODE_SPARSE = 1, VO_MODE_SUPERSPARSE = 2 };

/* Same layout as vxl_trace_params in include/vxl.h. */
typedef struct vo_params {
    float light_dir[3];
    float cam_pos[3];
    float bias;
    float shadow_len;
    float ao_len;
    float spec_len;
    float default_rough;
    int32_t n_shadow;
    int32_t n_ao;
    int32_t n_spec;
    uint32_t seed;
    int32_t mode;
} vo_params;

int vo_version(void);

/* math helpers shared with the CUDA path's algorithm */
void vo_sincos(float x, float* s, float* c);
uint32_t vo_pcg(uint32_t v);
float vo_rand01(uint32_t seed, uint32_t pixel, uint32_t sample);

/* a1: getVolumeAt (Light.frag:14-27) */
int vo_get_volume_at(const uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int mip);
/* a2: raycastShadowVolume (Light.frag:29-81), single pass (equivalent) and literal 4-pass form */
int vo_dda(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float maxt, vo_rec* r);
int vo_dda_literal(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float maxt,
                   float* hit, float* normal, int* fetches);
/* a3/a4: raycastShadowVolumeSparse / SuperSparse (Light.frag:131-217) */
float vo_sparse(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float dist, vo_rec* r);
float vo_supersparse(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float dist, vo_rec* r);
/* cosineSampleHemisphere (LightAmbient.frag:81-87) with this library's sin/cos */
void vo_cosine_sample(float u1, float u2, float* out3);

/* batch of rays: rays[i*7 .. i*7+6] = ox,oy,oz,dx,dy,dz,maxt */
void vo_trace_rays(const uint8_t* g, int sx, int sy, int sz, const float* rays, int n, int mode,
                   vo_rec* recs, int threads);

/* DDA-mode occlusion over a G-buffer (the drop-in's "trace_occlusion") */
void vo_occlusion(const uint8_t* g, int sx, int sy, int sz, const float* pos, const float* nrm,
                  const float* rough, int npix, const vo_params* p, float* shadow, float* ao,
                  float* ao_vis, float* spec, float* spec_t, vo_rec* recs, int p0, int p1, int threads);

/* reference light passes (REF modes) */
void vo_light_ambient(const uint8_t* g, int sx, int sy, int sz, const float* wcp, const float* nrm,
                      const float* depth, const float* noise, int npix, float* shadow, float* irradiance,
                      vo_rec* recs, int threads);
void vo_light_reflection(const uint8_t* g, int sx, int sy, int sz, const float* wcp, const float* nrm,
                         const float* view_r, const float* rough, const float* noise, int npix,
                         float* t_out, vo_rec* recs, int threads);
void vo_light_point(const uint8_t* g, int sx, int sy, int sz, const float* wpos, const float* nrm,
                    const float* noise, int npix, const float* light_pos, float range, int spot,
                    float* shadow, vo_rec* recs, int threads);

/* synthetic scenes (seeded), written as fine occupancy into the R8 layout */
void vo_scene_noise(uint8_t* g, int sx, int sy, int sz, uint32_t seed, float thresh, float freq,
                    int ground_y, int threads);
float vo_value_noise3(float x, float y, float z, uint32_t seed);
float vo_noise_octaves(float x, float y, float z, uint32_t seed, float freq, int octaves);
void vo_scene_terrain(uint8_t* g, int sx, int sy, int sz, uint32_t seed, float base, float amp, float freq,
                      int octaves, float* height, int threads);
void vo_scene_boxes(uint8_t* g, int sx, int sy, int sz, uint32_t seed, int nboxes, int smin, int smax);
void vo_box_params(uint32_t seed, int i, int nx, int ny, int nz, int smin, int smax, int* out6);

/* primary visibility G-buffer (pinhole camera looking at target) */
void vo_gbuffer(const uint8_t* g, int sx, int sy, int sz, const float* cam, const float* target,
                float tan_half_fov, int W, int H, uint32_t seed, float* pos, float* nrm, float* rough,
                int threads);

/* voxelizer (ShadowVoxSystem.cpp:82-94, :116-191, :7-53) */
void vo_set_volume_at(uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int value);
void vo_voxelize_model(uint8_t* g, int sx, int sy, int sz, const uint8_t* model, int msx, int msy,
                       int msz, const float* M, int value, int* aabb);
void vo_translate(const float* m, const float* v, float* out);
void vo_shadowvox_update(uint8_t* g, int sx, int sy, int sz, int n, const uint8_t* const* models,
                         const int* mdims, const float* prev, const float* cur, const float* pivot,
                         int* regions);
void vo_vox_destroyed(uint8_t* g, int sx, int sy, int sz, const uint8_t* model, int msx, int msy,
                      int msz, const float* world, int* region);

uint64_t vo_fnv1a64(const char* s);

/* Soft-opacity / albedo variant (no reference counterpart), FP64. Same layout
 * as vxl_soft_params in include/vxl.h. */
typedef struct vo_soft_params {
    float light_dir[3];
    float bias;
    float len;
    float k_sun;
    float k_amb;
    int32_t n_shadow;
    int32_t n_ao;
    uint32_t seed;
} vo_soft_params;

/* vox: float4 per voxel (opacity, albedo rgb), x fastest, nx,ny,nz even.
 * image: double[npix*3]. grad_image (optional, float[npix*3]) = dL/dI; then
 * grad_vox (double[nvox*4]) receives dL/d(opacity, albedo). perturb_voxel >= 0
 * adds perturb_delta (in double) to that voxel's opacity (finite differences). */
void vo_soft_render(const float* vox, int nx, int ny, int nz, const float* pos, const float* nrm, int npix,
                    const vo_soft_params* p, const float* grad_image, int64_t perturb_voxel, double perturb_delta,
                    double* image, double* grad_vox, int threads);

/* Primary visibility (GeometryVoxel.frag / VoxAsset.cpp) */
/* VoxAsset::Upload mips (VoxAsset.cpp:3-63): mip1/mip2 of an R8 volume */
void vo_volume_mips(const uint8_t* mip0, int sx, int sy, int sz, uint8_t* mip1, uint8_t* mip2);
/* [clipToAABB then] intersectVolume (GeometryVoxel.frag:50-61, :63-125) */
int vo_clip_intersect(const uint8_t* mip0, const uint8_t* mip1, const uint8_t* mip2, int sx, int sy, int sz,
                      const float* origin, const float* dir, const float* lcam, float uvx, float uvy, float resx,
                      float resy, int frame, int clip, float* hit, float* normal, uint32_t* material, int* fetches);
void vo_affine_inverse(const float* m, float* ri, float* ti);
/* per-pixel primary visibility over instances; camera in world units, pos out in fine units (x10) */
void vo_primary(const uint8_t* const* mip0s, const uint8_t* const* mip1s, const uint8_t* const* mip2s,
                const int* vdims, const float* worlds, const int* vol_of, int ninst, const float* cam,
                const float* target, float tan_half_fov, int W, int H, int frame, float* pos, float* nrm,
                float* depth, int32_t* material, int32_t* instance, int threads);

/* Surface position from the G-buffer's linear depth, as LightAmbient places a
 * pixel (LightAmbient.vert:32-36 FarVec with the pass's flipped UV;
 * LightAmbient.frag:138-150): wcp[npix][3] in fine units, nrm_out = nrm, or 0
 * for sky texels (!(depth < 0.999)). Matrices column-major. */
void vo_rebuild_from_depth(const float* depth, const float* nrm, int W, int H, const float* inv_view,
                           const float* inv_proj, float* wcp, float* nrm_out);

/* RayVoxCast (Sources/World/Systems/PhysicsSystem.cpp:98-145), the engine's
 * picking DDA against one model of msx*msy*msz bytes (x fastest). inv_obb is
 * glm::inverse(obb), column-major; the ray is in world units. Returns 1 on a
 * hit with *t_out = entry time * 0.1; cell_out = the last cell reached (the
 * hit cell, or the first one outside the model); iters_out = iterations run. */
int vo_ray_vox_cast(const uint8_t* model, int msx, int msy, int msz, const float* inv_obb, const float* ray_pos,
                    const float* ray_dir, float* t_out, int* cell_out, int* iters_out);

#ifdef __cplusplus
}
#endif
