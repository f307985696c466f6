// ref_voxelizer_harness.cpp — drives the reference's own ShadowVoxSystem
// (Sources/World/Systems/ShadowVoxSystem.cpp, compiled unmodified against the
// stand-in headers in oracle/ref/shim/). TEST INFRASTRUCTURE ONLY.
#include "ShadowVoxSystem.h"
#include "World/Components.h"

#include <cstring>

static ShadowVoxSystem* g_sys = nullptr;
static entt::registry g_reg;
static std::vector<VoxAsset*> g_models;

extern "C" {

// Creates the system (fixed 524x188x524-byte ShadowVox, ShadowVoxSystem.cpp:55-79).
void ref_vox_reset(void) {
    for (auto* m : g_models) delete m;
    g_models.clear();
    shim_entities().clear();
    delete g_sys;
    g_reg = entt::registry();
    shim_log() = ShimTransferLog();
    g_sys = new ShadowVoxSystem();
    g_sys->R = &g_reg;
    g_sys->W = nullptr;
    g_sys->OnCreate();
}

void ref_vox_dims(int* out3) {
    out3[0] = 524;
    out3[1] = 188;
    out3[2] = 524;
}

uint8_t* ref_vox_buffer(void) { return shim_log().last_buffer ? shim_log().last_buffer->data() : nullptr; }

int ref_vox_add_model(const uint8_t* data, int sx, int sy, int sz) {
    VoxAsset* m = new VoxAsset();
    m->SizeX = sx;
    m->SizeY = sy;
    m->SizeZ = sz;
    m->Data.assign(data, data + (size_t)sx * sy * sz);
    m->img.ext = Extent{(uint32_t)sx, (uint32_t)sy, (uint32_t)sz};
    g_models.push_back(m);
    return (int)g_models.size() - 1;
}

// prev/cur are column-major 4x4 world matrices; returns the entity id
int ref_vox_add_entity(int model, const float* prev, const float* cur, const float* pivot) {
    ShimEntity e;
    std::memcpy(&e.t.PreviousWorldMatrix[0][0], prev, 16 * sizeof(float));
    std::memcpy(&e.t.WorldMatrix[0][0], cur, 16 * sizeof(float));
    e.vr.Vox.ptr = g_models[model];
    e.vr.Pivot = glm::vec3(pivot[0], pivot[1], pivot[2]);
    e.changed = true;
    shim_entities().push_back(e);
    return (int)shim_entities().size() - 1;
}

void ref_vox_set_changed(int e, int changed) { shim_entities()[e].changed = changed != 0; }

// Runs ShadowVoxSystem::OnUpdate; returns the number of regions it uploaded
// and copies up to `max` of them (x,y,z,w,h,d) into out.
int ref_vox_update(int* out, int max) {
    shim_log().regions.clear();
    g_sys->OnUpdate(0.0f);
    int n = (int)shim_log().regions.size();
    for (int i = 0; i < n && i < max; i++) {
        const ImageRegion& r = shim_log().regions[i];
        int v[6] = {r.x, r.y, r.z, (int)r.width, (int)r.height, (int)r.depth};
        std::memcpy(out + 6 * i, v, sizeof(v));
    }
    return n;
}

// Fires the registry's on_destroy<VoxRenderer> hook (ShadowVoxSystem::OnVoxDestroyed)
void ref_vox_destroy(int e) {
    g_reg.on_destroy_cb(g_reg, (entt::entity)e);
    shim_entities()[e].alive = false;
}

// Regions pushed by OnVoxDestroyed wait for the next OnUpdate upload; this
// flushes them by running OnUpdate with no changed entity.
int ref_vox_flush(int* out, int max) {
    for (auto& e : shim_entities()) e.changed = false;
    return ref_vox_update(out, max);
}

}  // extern "C"
