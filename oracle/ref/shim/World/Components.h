// Stand-in for the engine's World/Components.h with just the Transform and
// VoxRenderer fields ShadowVoxSystem.cpp reads, a VoxAsset holding a dense
// palette-index block (PixelAt indexes x + y*SizeX + z*SizeX*SizeY as
// Sources/Asset/VoxAsset.h:52-56 does), and the entity store behind the entt
// stand-in. Reference-build recipe only (test infrastructure).
#pragma once
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <vector>

#include "Graphics/Graphics.h"
#include "World/Systems/TransformSystem.h"
#include <entt/entt.hpp>

struct VoxImage {
    Extent ext;
    Extent getExtent() { return ext; }
};
class VoxAsset {
public:
    uint32 SizeX = 0, SizeY = 0, SizeZ = 0;
    std::vector<uint8> Data;
    VoxImage img;
    VoxImage& GetImage() { return img; }
    inline uint8* PixelAt(int32 X, int32 Y, int32 Z) {
        return Data.data() + ((size_t)X + ((size_t)Y * (size_t)SizeX) + ((size_t)Z * (size_t)SizeX * (size_t)SizeY));
    }
};
template <class T>
struct AssetRefT {
    T* ptr = nullptr;
    bool IsValid() const { return ptr != nullptr; }
    T* operator->() { return ptr; }
};
template <class T>
struct AssetSlot : AssetRefT<T> {};

struct VoxRenderer {
    AssetSlot<VoxAsset> Vox;
    int VoxSlot{-1};
    glm::vec3 Pivot{0.0f, 0.0f, 0.0f};
};
struct Transform {
    glm::mat4 PreviousWorldMatrix{1.0f};
    glm::mat4 WorldMatrix{1.0f};
    glm::mat4 Matrix{1.0f};
};

struct ShimEntity {
    Transform t;
    VoxRenderer vr;
    bool changed = false;
    bool alive = true;
};
inline std::vector<ShimEntity>& shim_entities() {
    static std::vector<ShimEntity> v;
    return v;
}
template <class F>
void shim_each(entt::registry&, F& f, entt::basic_view<Transform, VoxRenderer, Changed>*) {
    auto& E = shim_entities();
    for (size_t i = 0; i < E.size(); i++)
        if (E[i].alive && E[i].changed) f((entt::entity)i, E[i].t, E[i].vr);
}
inline Transform& shim_get(entt::registry&, entt::entity e, Transform*) { return shim_entities()[(size_t)e].t; }
inline VoxRenderer& shim_get(entt::registry&, entt::entity e, VoxRenderer*) {
    return shim_entities()[(size_t)e].vr;
}
