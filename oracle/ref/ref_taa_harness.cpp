// ref_taa_harness.cpp — compiles the reference's temporal accumulation shader
// (main and luminance of Sources/Shaders/LightTAA.frag) as C++ against the
// vendored glm (TEST INFRASTRUCTURE ONLY; see build_ref.py). The .inc file is
// generated into oracle/_ref/ at build time.
//
// texture() is the sampler the library defines for this pass: bilinear,
// clamp to edge, texel centres at (i + 0.5) / size (the engine samples these
// images with its default linear filter). cos/sin are the oracle's own,
// supplied at run time as in ref_light_harness.cpp. getNoise() returns the
// pixel's blue-noise texel, set per call.
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>

#include <cmath>
#include <cstdint>

using namespace glm;

#define GOLDEN_RATIO 2.118033988749895
static const float FAR = 4096.0f;

struct Tex {
    const float* p;
    int c, W, H;
};
static Tex g_light, g_last, g_color, g_normal, g_material, g_depth, g_motion;
#define LIGHT_TEXTURE g_light
#define LAST_LIGHT_TEXTURE g_last
#define COLOR_TEXTURE g_color
#define NORMAL_TEXTURE g_normal
#define MATERIAL_TEXTURE g_material
#define DEPTH_TEXTURE g_depth
#define MOTION_TEXTURE g_motion

static inline vec4 texture(const Tex& t, vec2 uv) {
    const int W = t.W, H = t.H;
    const float x = uv.x * (float)W - 0.5f, y = uv.y * (float)H - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy, x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > W - 1 ? W - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > W - 1 ? W - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > H - 1 ? H - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > H - 1 ? H - 1 : y1);
    const float bx = 1.0f - ax, by = 1.0f - ay;
    float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < t.c; k++) {
        const float t00 = t.p[((size_t)y0 * W + x0) * t.c + k], t10 = t.p[((size_t)y0 * W + x1) * t.c + k];
        const float t01 = t.p[((size_t)y1 * W + x0) * t.c + k], t11 = t.p[((size_t)y1 * W + x1) * t.c + k];
        const float top = t00 * bx + t10 * ax;
        const float bot = t01 * bx + t11 * ax;
        out[k] = top * by + bot * ay;
    }
    return vec4(out[0], out[1], out[2], out[3]);
}
static inline ivec2 textureSize(const Tex& t, int) { return ivec2(t.W, t.H); }

// GLSL's implicit int -> float promotions the shader relies on
static inline vec2 operator/(float a, ivec2 b) { return vec2(a) / vec2(b); }
static inline float clamp(float x, int lo, int hi) { return glm::clamp(x, float(lo), float(hi)); }
static inline float max(float x, int y) { return glm::max(x, float(y)); }

static void (*g_sincos)(float, float*, float*) = nullptr;
static vec4 g_noise;
static vec4 out_Color;
static struct {
    vec2 UV;
} In;

namespace taa {
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
static inline vec4 getNoise() { return g_noise; }
#include "taa_main.inc"
}  // namespace taa

extern "C" void ref_taa_set_sincos(void* f) { g_sincos = (void (*)(float, float*, float*))f; }

extern "C" void ref_taa(const float* light, const float* last, const float* color, const float* normal,
                        const float* material, const float* depth, const float* motion, const float* noise, int W,
                        int H, float* out) {
    g_light = {light, 4, W, H};
    g_last = {last, 4, W, H};
    g_color = {color, 3, W, H};
    g_normal = {normal, 3, W, H};
    g_material = {material, 4, W, H};
    g_depth = {depth, 1, W, H};
    g_motion = {motion, 2, W, H};
    for (int i = 0; i < W * H; i++) {
        const int px = i % W, py = i / W;
        In.UV = vec2(((float)px + 0.5f) / (float)W, ((float)py + 0.5f) / (float)H);
        g_noise = vec4(noise[4 * i], noise[4 * i + 1], noise[4 * i + 2], noise[4 * i + 3]);
        taa::taa_main();
        out[4 * i] = out_Color.x;
        out[4 * i + 1] = out_Color.y;
        out[4 * i + 2] = out_Color.z;
        out[4 * i + 3] = out_Color.w;
    }
}
