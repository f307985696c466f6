// ref_light_harness.cpp — compiles the reference's lighting shader code as C++
// (TEST INFRASTRUCTURE ONLY; see build_ref.py). The .inc files are generated
// into oracle/_ref/ from Sources/Shaders/*.frag at build time.
//
// SHADOW_VOX_TEXTURE is an R8 byte grid (the ShadowVox layout); texelFetch
// returns 0 outside it (robust image access) and counts every fetch.
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>

#include <cmath>
#include <cstdint>

using namespace glm;
typedef unsigned int uint;

struct ShadowVoxTexture {
    const uint8_t* g;
    int sx, sy, sz;
};
static ShadowVoxTexture g_shadow_vox;
static long long g_fetches;
static ivec3 g_last_texel;

static inline uvec4 texelFetch(const ShadowVoxTexture& t, ivec3 p, int) {
    g_fetches++;
    g_last_texel = p;
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= t.sx || p.y >= t.sy || p.z >= t.sz) return uvec4(0u);
    return uvec4((uint)t.g[(size_t)p.x + (size_t)p.y * t.sx + (size_t)p.z * t.sx * t.sy], 0u, 0u, 0u);
}
static inline ivec3 textureSize(const ShadowVoxTexture& t, int) { return ivec3(t.sx, t.sy, t.sz); }
#define SHADOW_VOX_TEXTURE g_shadow_vox

// GLSL's implicit int -> float promotions that Light.frag relies on
static inline vec3 operator/(ivec3 a, float b) { return vec3(a) / b; }
static inline vec3 operator/(vec3 a, int b) { return a / float(b); }

#define COMMON_H  // Common.frag holds only Vulkan bindings: skip it
#include "Light_frag.inc"

// sin/cos supplied at run time (the oracle's own), for the "own trig" variants
static void (*g_sincos)(float, float*, float*) = nullptr;

// Pass-level state the extracted shader blocks read through getNoise() and
// GetInverseViewMatrix().
static vec4 g_noise;
static mat4 g_inv_view(1.0f);

#define VXL_PASS_BODY                                                                \
    static inline vec4 getNoise() { return g_noise; }                                \
    static inline mat4 GetInverseViewMatrix() { return g_inv_view; }                 \
    struct Amb {                                                                     \
        static void run(vec3 pos, vec3 normal, float depth, vec3* wcp0, float* shadow, \
                        float* irr);                                                 \
    };

namespace trig_libm {
VXL_PASS_BODY
#include "ambient_sundir.inc"
#include "ambient_cosine.inc"
#include "ambient_irradiance.inc"
}  // namespace trig_libm

namespace trig_own {
VXL_PASS_BODY
static inline float cos(float x) {
    float s, c;
    g_sincos(x, &s, &c);
    return c;
}
static inline float sin(float x) {
    float s, c;
    g_sincos(x, &s, &c);
    return s;
}
#include "ambient_sundir.inc"
#include "ambient_cosine.inc"
#include "ambient_irradiance.inc"
}  // namespace trig_own

// LightAmbient.frag:141-173 around the extracted blocks
namespace trig_libm {
void Amb::run(vec3 pos, vec3 normal, float depth, vec3* wcp0, float* shadow, float* irr) {
    *wcp0 = (GetInverseViewMatrix() * vec4(pos, 1.0)).xyz() * 10.0;
#include "ambient_shadow_setup.inc"
    *shadow = (raycastShadowVolumeSparse(wcp + normal * bias, wd, 128.0) != 128.0) ? 0.0f : 1.0f;  // :167
    *irr = calculateAmbientIrradiance(wcp + normal * bias, normal).x;                               // :173
}
}  // namespace trig_libm
namespace trig_own {
void Amb::run(vec3 pos, vec3 normal, float depth, vec3* wcp0, float* shadow, float* irr) {
    *wcp0 = (GetInverseViewMatrix() * vec4(pos, 1.0)).xyz() * 10.0;
#include "ambient_shadow_setup.inc"
    *shadow = (raycastShadowVolumeSparse(wcp + normal * bias, wd, 128.0) != 128.0) ? 0.0f : 1.0f;  // :167
    *irr = calculateAmbientIrradiance(wcp + normal * bias, normal).x;                               // :173
}

// LightReflection.frag:79-113 (R is the view-space reflection vector)
static float reflection(vec3 pos, vec3 R, vec3 normal, float roughness, vec3* wcp0, vec3* wd0) {
    *wcp0 = (GetInverseViewMatrix() * vec4(pos, 1.0)).xyz() * 10.0;
    *wd0 = (GetInverseViewMatrix() * vec4(R, 0.0)).xyz();
#include "reflection_setup.inc"
    return raycastShadowVolumeSparse(wcp + normal, wd, 256.0);  // :113
}

// LightPoint.frag:234-267 / LightSpot.frag:83-117 (worldPos in world units)
static float point(vec3 worldPos, vec3 lightPosition, vec3 normal, float range, int* discarded) {
    vec3 lightDir = lightPosition - worldPos;
    float lightDistance = length(lightDir);
    *discarded = lightDistance > range;
    if (*discarded) return 1.0f;
#include "point_setup.inc"
    return raycastShadowVolumeSparse(wcp + normal * 0.5, wd, hitDist) < hitDist ? 0.0f : 1.0f;  // LightPoint.frag:125
}
static float spot(vec3 worldPos, vec3 lightPosition, vec3 normal, float range, int* discarded) {
    vec3 lightDir = lightPosition - worldPos;
    float lightDistance = length(lightDir);
    *discarded = lightDistance > range;
    if (*discarded) return 1.0f;
#include "spot_setup.inc"
    return raycastShadowVolumeSuperSparse(wcp + normal * 0.5, wd, hitDist) < hitDist ? 0.0f : 1.0f;  // LightSpot.frag:113
}
}  // namespace trig_own

static inline void set_grid(const uint8_t* g, int sx, int sy, int sz) {
    g_shadow_vox = ShadowVoxTexture{g, sx, sy, sz};
    g_fetches = 0;
    g_last_texel = ivec3(0);
}

extern "C" {

void ref_set_sincos(void (*fn)(float, float*, float*)) { g_sincos = fn; }

int ref_get_volume_at(const uint8_t* g, int sx, int sy, int sz, int x, int y, int z, int mip) {
    set_grid(g, sx, sy, sz);
    return getVolumeAt(ivec3(x, y, z), mip) ? 1 : 0;
}

int ref_raycast(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float maxt, float* hit,
                float* normal, long long* fetches, int* last_texel) {
    set_grid(g, sx, sy, sz);
    vec3 h(0.0f), n(0.0f);
    bool r = raycastShadowVolume(vec3(o[0], o[1], o[2]), vec3(d[0], d[1], d[2]), maxt, h, n);
    for (int a = 0; a < 3; a++) {
        hit[a] = h[a];
        normal[a] = n[a];
        last_texel[a] = g_last_texel[a];
    }
    *fetches = g_fetches;
    return r ? 1 : 0;
}

float ref_march(const uint8_t* g, int sx, int sy, int sz, const float* o, const float* d, float dist, int super_sparse,
                long long* fetches, int* last_texel) {
    set_grid(g, sx, sy, sz);
    vec3 O(o[0], o[1], o[2]), D(d[0], d[1], d[2]);
    float t = super_sparse ? raycastShadowVolumeSuperSparse(O, D, dist) : raycastShadowVolumeSparse(O, D, dist);
    for (int a = 0; a < 3; a++) last_texel[a] = g_last_texel[a];
    *fetches = g_fetches;
    return t;
}

void ref_cosine_sample(float u1, float u2, int own_trig, float* out3) {
    vec3 v = own_trig ? trig_own::cosineSampleHemisphere(vec2(u1, u2)) : trig_libm::cosineSampleHemisphere(vec2(u1, u2));
    out3[0] = v.x;
    out3[1] = v.y;
    out3[2] = v.z;
}

void ref_sun_dir(float* out3) {
    for (int a = 0; a < 3; a++) out3[a] = trig_own::SUN_DIR[a];
}

// One ambient-pass pixel: inputs are the view-space position `pos`, the
// inverse view matrix (column-major), the world normal, linear depth and the
// pixel's blue-noise texel. Outputs wcp0 = (InvView*pos)*10, shadow, irradiance.
void ref_ambient(const uint8_t* g, int sx, int sy, int sz, const float* pos, const float* inv_view, const float* nrm,
                 float depth, const float* noise, int own_trig, float* wcp0, float* shadow, float* irr) {
    set_grid(g, sx, sy, sz);
    g_noise = vec4(noise[0], noise[1], noise[2], noise[3]);
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) g_inv_view[c][r] = inv_view[4 * c + r];
    vec3 w;
    if (own_trig)
        trig_own::Amb::run(vec3(pos[0], pos[1], pos[2]), vec3(nrm[0], nrm[1], nrm[2]), depth, &w, shadow, irr);
    else
        trig_libm::Amb::run(vec3(pos[0], pos[1], pos[2]), vec3(nrm[0], nrm[1], nrm[2]), depth, &w, shadow, irr);
    for (int a = 0; a < 3; a++) wcp0[a] = w[a];
}

float ref_reflection(const uint8_t* g, int sx, int sy, int sz, const float* pos, const float* inv_view, const float* R,
                     const float* nrm, float roughness, const float* noise, float* wcp0, float* wd0) {
    set_grid(g, sx, sy, sz);
    g_noise = vec4(noise[0], noise[1], noise[2], noise[3]);
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) g_inv_view[c][r] = inv_view[4 * c + r];
    vec3 w, wd;
    float t = trig_own::reflection(vec3(pos[0], pos[1], pos[2]), vec3(R[0], R[1], R[2]), vec3(nrm[0], nrm[1], nrm[2]),
                                   roughness, &w, &wd);
    for (int a = 0; a < 3; a++) {
        wcp0[a] = w[a];
        wd0[a] = wd[a];
    }
    return t;
}

float ref_point(const uint8_t* g, int sx, int sy, int sz, const float* wpos, const float* light_pos, const float* nrm,
                float range, const float* noise, int spot, int* discarded) {
    set_grid(g, sx, sy, sz);
    g_noise = vec4(noise[0], noise[1], noise[2], noise[3]);
    vec3 W(wpos[0], wpos[1], wpos[2]), L(light_pos[0], light_pos[1], light_pos[2]), N(nrm[0], nrm[1], nrm[2]);
    return spot ? trig_own::spot(W, L, N, range, discarded) : trig_own::point(W, L, N, range, discarded);
}

}  // extern "C"
