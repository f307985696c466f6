// ref_transform_harness.cpp — compiles TransformSystem::RealculateMatrix
// (Sources/World/Systems/TransformSystem.cpp:124-135) as a free function
// against the reference's vendored glm (TEST INFRASTRUCTURE ONLY; see
// build_ref.py). The .inc file is generated into oracle/_ref/ at build time.
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>

#include <cstring>

namespace entt {
enum class entity : unsigned {};
}
struct Transform {
    glm::vec3 Position, Rotation, Scale;
    glm::mat4 Matrix, WorldMatrix;
};

#include "transform_realculate.inc"

extern "C" void ref_transform(const float* pos, const float* rot, const float* scale, const float* parent,
                              float* out) {
    Transform t;
    t.Position = glm::vec3(pos[0], pos[1], pos[2]);
    t.Rotation = glm::vec3(rot[0], rot[1], rot[2]);
    t.Scale = glm::vec3(scale[0], scale[1], scale[2]);
    glm::mat4 p(1.0f);
    if (parent) std::memcpy(&p[0][0], parent, 64);
    RealculateMatrix(entt::entity{}, t, p);
    std::memcpy(out, &t.WorldMatrix[0][0], 64);
}

// RayVoxCast (Sources/World/Systems/PhysicsSystem.cpp:98-145), cut out
// unmodified into physics_rayvox.inc. Stand-ins for the engine's asset types:
// a model of bytes, x fastest, addressed as VoxAsset::PixelAt addresses it.
typedef unsigned char uint8;
struct VoxAsset {
    uint8* data;
    size_t SizeX, SizeY;
    uint8* PixelAt(int x, int y, int z) { return data + ((size_t)x + (size_t)y * SizeX + (size_t)z * SizeX * SizeY); }
};
template <class T>
struct AssetRefT {
    T* p;
    T* operator->() { return p; }
};

#include "physics_rayvox.inc"

extern "C" int ref_ray_vox_cast(const float* obb, unsigned char* model, int sx, int sy, int sz, const float* pos,
                                const float* dir, float* t) {
    glm::mat4 m;
    std::memcpy(&m[0][0], obb, 64);
    VoxAsset a{model, (size_t)sx, (size_t)sy};
    AssetRefT<VoxAsset> ref{&a};
    float tt = -1.0f;
    const bool hit = RayVoxCast(m, glm::vec3((float)sx, (float)sy, (float)sz), ref, glm::vec3(pos[0], pos[1], pos[2]),
                                glm::vec3(dir[0], dir[1], dir[2]), tt);
    *t = tt;
    return hit ? 1 : 0;
}

// glm::inverse of a column-major 4x4, the matrix RayVoxCast works with
extern "C" void ref_glm_inverse(const float* in, float* out) {
    glm::mat4 m;
    std::memcpy(&m[0][0], in, 64);
    const glm::mat4 r = glm::inverse(m);
    std::memcpy(out, &r[0][0], 64);
}
