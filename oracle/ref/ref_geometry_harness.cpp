// ref_geometry_harness.cpp — compiles the reference's primary-visibility
// shader code (clipToAABB, intersectVolume from Sources/Shaders/GeometryVoxel.frag)
// and VoxAsset::Upload's mip loop (Sources/Asset/VoxAsset.cpp) as C++
// (TEST INFRASTRUCTURE ONLY; see build_ref.py). The .inc files are generated
// into oracle/_ref/ at build time.
//
// VOLUME_TEXTURE is an R8 volume with three mips; texelFetch returns 0
// outside a mip (robust image access) and counts every fetch. The varyings
// and view-buffer getters the functions read (In.localCameraPos, GetRes(),
// GetFrame()) are globals set per call.
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>

#include <cmath>
#include <cstdint>

using namespace glm;
typedef unsigned int uint;

struct VolumeTexture {
    const uint8_t* m[3];
    int sx[3], sy[3], sz[3];
};
static VolumeTexture g_volume;
static long long g_vfetches;

static inline uvec4 texelFetch(const VolumeTexture& t, ivec3 p, int mip) {
    g_vfetches++;
    if (mip < 0 || mip > 2 || p.x < 0 || p.y < 0 || p.z < 0 || p.x >= t.sx[mip] || p.y >= t.sy[mip] ||
        p.z >= t.sz[mip])
        return uvec4(0u);
    return uvec4((uint)t.m[mip][(size_t)p.x + (size_t)p.y * t.sx[mip] + (size_t)p.z * t.sx[mip] * t.sy[mip]], 0u,
                 0u, 0u);
}
#define VOLUME_TEXTURE g_volume

static ivec3 volumeDimension;
static struct {
    vec3 localDirection;
    vec3 localCameraPos;
    mat4 MVPMatrix;
} In;
static vec2 g_res;
static int g_frame;
static inline vec2 GetRes() { return g_res; }
static inline int GetFrame() { return g_frame; }

// GLSL's implicit int -> float promotions the shader relies on
static inline vec3 operator/(ivec3 a, float b) { return vec3(a) / b; }
static inline float mod(float x, int y) { return glm::mod(x, float(y)); }

#define LOD 1
#define MIP_COUNT 2
#define TRANSPARENCY 1
#include "geometry_clip.inc"
#include "geometry_intersect.inc"

static inline int mip_dim(int d) { return d > 1 ? d / 2 : 1; }

extern "C" int ref_clip_intersect(const uint8_t* mip0, const uint8_t* mip1, const uint8_t* mip2, int sx, int sy,
                                  int sz, const float* origin, const float* dir, const float* lcam, float uvx,
                                  float uvy, float resx, float resy, int frame, int clip, float* hit, float* normal,
                                  uint32_t* material, int* fetches) {
    g_volume.m[0] = mip0;
    g_volume.m[1] = mip1;
    g_volume.m[2] = mip2;
    g_volume.sx[0] = sx;
    g_volume.sy[0] = sy;
    g_volume.sz[0] = sz;
    for (int k = 1; k < 3; k++) {
        g_volume.sx[k] = mip_dim(g_volume.sx[k - 1]);
        g_volume.sy[k] = mip_dim(g_volume.sy[k - 1]);
        g_volume.sz[k] = mip_dim(g_volume.sz[k - 1]);
    }
    volumeDimension = ivec3(sx, sy, sz);
    In.localCameraPos = vec3(lcam[0], lcam[1], lcam[2]);
    g_res = vec2(resx, resy);
    g_frame = frame;
    g_vfetches = 0;
    vec3 o(origin[0], origin[1], origin[2]), d(dir[0], dir[1], dir[2]);
    if (clip) o = clipToAABB(o, d, vec3(sx, sy, sz));
    vec3 h(0.0f), n(0.0f);
    uint mat = 0u;
    const bool r = intersectVolume(o, d, h, n, mat, vec2(uvx, uvy));
    hit[0] = h.x; hit[1] = h.y; hit[2] = h.z;
    normal[0] = n.x; normal[1] = n.y; normal[2] = n.z;
    *material = r ? mat : 0u;
    *fetches = (int)g_vfetches;
    return r ? 1 : 0;
}

// one mip step of VoxAsset::Upload: parent level -> child level (the loop body
// is the reference's; the child sizes follow its `p > 1 ? p / 2 : 1`)
extern "C" void ref_mip_down(const uint8_t* parentData, int parentSizeX, int parentSizeY, int parentSizeZ,
                             uint8_t* data) {
    const int mipSizeX = parentSizeX > 1 ? parentSizeX / 2 : 1;
    const int mipSizeY = parentSizeY > 1 ? parentSizeY / 2 : 1;
    const int mipSizeZ = parentSizeZ > 1 ? parentSizeZ / 2 : 1;
    (void)parentSizeZ;
#include "voxasset_mip.inc"
}
