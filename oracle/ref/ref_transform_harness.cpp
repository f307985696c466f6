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
