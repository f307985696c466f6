// assets.cpp — host-side readers for the reference's shipped scenes: asset
// GUIDs, .p palettes, .pf prefabs (with nested prefab instances) and the
// transform composition that turns a prefab's Transform components into the
// world matrices the voxelizer and primary visibility consume.
//
//  - GUID: Assets::Hash (Sources/Asset/Assets.h:207-210) is std::hash of the
//    mod-relative path ("default/FarmHouse/0.v"); the shipped .pf files were
//    written with MSVC's std::hash, which is FNV-1a 64 (offset basis
//    14695981039346656037, prime 1099511628211).
//  - Palette: PalleteAsset::Serialize (Sources/Asset/PalleteAsset.h:63-69),
//    256 VoxMaterial of 7 bytes (r, g, b, a, roughness, metallic, emit).
//  - Prefab: PrefabAsset::Spawn (Sources/Asset/PrefabAsset.cpp:30-120): a
//    JSON array of entities {Id, Parent, Instance, Transform{Position,
//    Rotation, Scale as "x y z"}, VoxRenderer{Pallete, Vox (hex GUIDs),
//    Pivot}}; an entity with Instance spawns that prefab under the entity's
//    parent and the entity's own components then apply to the spawned root.
//  - Transform: TransformSystem::RealculateMatrix (TransformSystem.cpp:124-135),
//    Local = T(Position) Rz Ry Rx S(Scale), World = ParentWorld * Local, with
//    glm's operation order for translate / rotate / scale / mat4 * mat4 so
//    the matrices match the engine's bit for bit (cos / sin from the C library,
//    as glm calls them).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "vxl_internal.h"

namespace vxl {
namespace {

// ------------------------------------------------------------------ JSON
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

struct JParser {
    const char* p;
    const char* end;
    std::string err;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end - p) >= n && std::memcmp(p, s, n) == 0) {
            p += n;
            return true;
        }
        return false;
    }
    bool string(std::string& out) {
        if (p >= end || *p != '"') return fail("expected a string");
        p++;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c == '\\') {
                if (p >= end) return fail("bad escape");
                char e = *p++;
                switch (e) {
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case '/': out += '/'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'n': out += '\n'; break;
                    case 'r': out += '\r'; break;
                    case 't': out += '\t'; break;
                    case 'u': {
                        if (end - p < 4) return fail("bad \\u escape");
                        unsigned v = (unsigned)std::strtoul(std::string(p, 4).c_str(), nullptr, 16);
                        p += 4;
                        if (v < 0x80) {
                            out += (char)v;
                        } else if (v < 0x800) {
                            out += (char)(0xC0 | (v >> 6));
                            out += (char)(0x80 | (v & 0x3F));
                        } else {
                            out += (char)(0xE0 | (v >> 12));
                            out += (char)(0x80 | ((v >> 6) & 0x3F));
                            out += (char)(0x80 | (v & 0x3F));
                        }
                        break;
                    }
                    default: return fail("bad escape");
                }
            } else {
                out += c;
            }
        }
        if (p >= end) return fail("unterminated string");
        p++;
        return true;
    }
    bool fail(const char* m) {
        if (err.empty()) err = m;
        return false;
    }
    bool value(JVal& v, int depth) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        if (*p == '{') {
            p++;
            v.kind = JVal::Obj;
            ws();
            if (p < end && *p == '}') {
                p++;
                return true;
            }
            for (;;) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p >= end || *p != ':') return fail("expected ':'");
                p++;
                JVal x;
                if (!value(x, depth + 1)) return false;
                v.obj.emplace_back(std::move(k), std::move(x));
                ws();
                if (p < end && *p == ',') {
                    p++;
                    continue;
                }
                if (p < end && *p == '}') {
                    p++;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (*p == '[') {
            p++;
            v.kind = JVal::Arr;
            ws();
            if (p < end && *p == ']') {
                p++;
                return true;
            }
            for (;;) {
                JVal x;
                if (!value(x, depth + 1)) return false;
                v.arr.push_back(std::move(x));
                ws();
                if (p < end && *p == ',') {
                    p++;
                    continue;
                }
                if (p < end && *p == ']') {
                    p++;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (*p == '"') {
            v.kind = JVal::Str;
            return string(v.str);
        }
        if (lit("true")) {
            v.kind = JVal::Bool;
            v.b = true;
            return true;
        }
        if (lit("false")) {
            v.kind = JVal::Bool;
            return true;
        }
        if (lit("null")) return true;
        char* q = nullptr;
        const std::string tok(p, (size_t)std::min<ptrdiff_t>(end - p, 64));
        const double d = std::strtod(tok.c_str(), &q);
        if (q == tok.c_str()) return fail("bad value");
        p += q - tok.c_str();
        v.kind = JVal::Num;
        v.num = d;
        return true;
    }
};

bool read_file(const std::string& path, std::string* out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out->resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? std::fread(&(*out)[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == out->size();
}

// ------------------------------------------------------------ transforms
// column-major 4x4; glm's operation order throughout
void mat_identity(float* m) {
    for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}
void mat_translate(const float* m, const float* v, float* out) {
    float r[16];
    std::memcpy(r, m, sizeof(r));
    for (int k = 0; k < 4; k++) {
        float a = m[0 + k] * v[0] + m[4 + k] * v[1];
        a = a + m[8 + k] * v[2];
        r[12 + k] = a + m[12 + k];
    }
    std::memcpy(out, r, sizeof(r));
}
// rotation by `angle` about a unit axis (Rodrigues' matrix), applied as m * R
void mat_rotate(const float* m, float angle, const float* axis_in, float* out) {
    const float c = std::cos(angle), s = std::sin(angle);
    float dd = axis_in[0] * axis_in[0] + axis_in[1] * axis_in[1];
    dd = dd + axis_in[2] * axis_in[2];
    const float inv = 1.0f / std::sqrt(dd);
    const float ax[3] = {axis_in[0] * inv, axis_in[1] * inv, axis_in[2] * inv};
    const float omc = 1.0f - c;
    const float t[3] = {omc * ax[0], omc * ax[1], omc * ax[2]};
    float R[3][3];
    R[0][0] = c + t[0] * ax[0];
    R[0][1] = t[0] * ax[1] + s * ax[2];
    R[0][2] = t[0] * ax[2] - s * ax[1];
    R[1][0] = t[1] * ax[0] - s * ax[2];
    R[1][1] = c + t[1] * ax[1];
    R[1][2] = t[1] * ax[2] + s * ax[0];
    R[2][0] = t[2] * ax[0] + s * ax[1];
    R[2][1] = t[2] * ax[1] - s * ax[0];
    R[2][2] = c + t[2] * ax[2];
    float r[16];
    for (int col = 0; col < 3; col++)
        for (int k = 0; k < 4; k++) {
            float a = m[0 + k] * R[col][0] + m[4 + k] * R[col][1];
            r[col * 4 + k] = a + m[8 + k] * R[col][2];
        }
    for (int k = 0; k < 4; k++) r[12 + k] = m[12 + k];
    std::memcpy(out, r, sizeof(r));
}
void mat_scale(const float* m, const float* v, float* out) {
    float r[16];
    for (int col = 0; col < 3; col++)
        for (int k = 0; k < 4; k++) r[col * 4 + k] = m[col * 4 + k] * v[col];
    for (int k = 0; k < 4; k++) r[12 + k] = m[12 + k];
    std::memcpy(out, r, sizeof(r));
}
void mat_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int col = 0; col < 4; col++)
        for (int k = 0; k < 4; k++) {
            float v = a[0 + k] * b[col * 4 + 0] + a[4 + k] * b[col * 4 + 1];
            v = v + a[8 + k] * b[col * 4 + 2];
            r[col * 4 + k] = v + a[12 + k] * b[col * 4 + 3];
        }
    std::memcpy(out, r, sizeof(r));
}
void transform_matrix(const float* pos, const float* rot, const float* scale, const float* parent, float* out) {
    static const float ZA[3] = {0.0f, 0.0f, 1.0f}, YA[3] = {0.0f, 1.0f, 0.0f}, XA[3] = {1.0f, 0.0f, 0.0f};
    float m[16];
    mat_identity(m);
    mat_translate(m, pos, m);
    mat_rotate(m, rot[2], ZA, m);
    mat_rotate(m, rot[1], YA, m);
    mat_rotate(m, rot[0], XA, m);
    mat_scale(m, scale, m);
    if (parent) {
        mat_mul(parent, m, out);
    } else {
        float id[16];
        mat_identity(id);
        mat_mul(id, m, out);
    }
}

}  // namespace
}  // namespace vxl

// ----------------------------------------------------------------- prefab
struct vxl_prefab {
    struct Entity {
        int parent = -1;
        float pos[3] = {0, 0, 0}, rot[3] = {0, 0, 0}, scale[3] = {1, 1, 1};
        bool has_vox = false;
        uint64_t vox = 0, pal = 0;
        float pivot[3] = {0, 0, 0};
        float world[16];
    };
    std::string mods_dir;
    std::unordered_map<uint64_t, std::string> index;  // GUID -> file path
    std::vector<Entity> ents;
    struct Vol {
        uint64_t guid;
        int32_t sx, sy, sz;
        std::vector<uint8_t> data;
    };
    struct Pal {
        uint64_t guid;
        std::vector<uint8_t> mats;
    };
    std::vector<Vol> vols;
    std::vector<Pal> pals;
    std::map<uint64_t, int> vol_of, pal_of;
    struct Ren {
        int entity, vol, pal;
    };
    std::vector<Ren> rens;
};

namespace vxl {
namespace {

bool parse_vec3(const std::string& s, float* v) {
    // PrefabAsset.cpp:8-18: three numbers separated by single spaces
    const char* c = s.c_str();
    for (int i = 0; i < 3; i++) {
        char* q = nullptr;
        v[i] = std::strtof(c, &q);
        if (q == c) return false;
        c = q;
    }
    return true;
}
bool parse_guid(const std::string& s, uint64_t* g) {
    if (s.empty()) return false;
    char* q = nullptr;
    *g = std::strtoull(s.c_str(), &q, 16);
    return q && *q == '\0';
}

vxl_status spawn(vxl_prefab* P, uint64_t prefab_guid, const std::string& path, int parent_entity, int depth,
                 int* root_out) {
    if (depth > 16) return fail(VXL_ERR_INVALID_ARG, "prefab_load: prefab instances nested too deep (%s)", path.c_str());
    std::string text;
    if (!read_file(path, &text)) return fail(VXL_ERR_IO, "prefab_load: cannot read %s", path.c_str());
    JParser jp{text.data(), text.data() + text.size(), {}};
    JVal doc;
    if (!jp.value(doc, 0) || doc.kind != JVal::Arr)
        return fail(VXL_ERR_IO, "prefab_load: %s: %s", path.c_str(), jp.err.empty() ? "not a JSON array" : jp.err.c_str());
    (void)prefab_guid;
    std::unordered_map<int, int> id_map;
    int root = -1;
    for (const JVal& ent : doc.arr) {
        if (ent.kind != JVal::Obj) return fail(VXL_ERR_IO, "prefab_load: %s: entity is not an object", path.c_str());
        int parent = -1;
        const JVal* jp_ = ent.get("Parent");
        if (jp_ && jp_->kind == JVal::Num) {
            auto it = id_map.find((int)jp_->num);
            parent = it == id_map.end() ? -1 : it->second;
        }
        const bool is_root = parent < 0;
        int e;
        const JVal* inst = ent.get("Instance");
        if (inst && inst->kind == JVal::Str) {
            uint64_t g;
            auto it = parse_guid(inst->str, &g) ? P->index.find(g) : P->index.end();
            if (it == P->index.end())
                return fail(VXL_ERR_IO, "prefab_load: %s: unresolved prefab instance %s", path.c_str(),
                            inst->str.c_str());
            VXL_TRY(spawn(P, g, it->second, parent, depth + 1, &e));
        } else {
            e = (int)P->ents.size();
            P->ents.emplace_back();
        }
        const JVal* jid = ent.get("Id");
        if (jid && jid->kind == JVal::Num) id_map[(int)jid->num] = e;
        if (is_root) {
            root = e;
            P->ents[e].parent = parent_entity;
        } else {
            P->ents[e].parent = parent;
        }
        const JVal* tr = ent.get("Transform");
        if (tr && tr->kind == JVal::Obj) {
            vxl_prefab::Entity& E = P->ents[e];
            const JVal* a = tr->get("Position");
            const JVal* b = tr->get("Rotation");
            const JVal* c = tr->get("Scale");
            if (!a || !b || !c || a->kind != JVal::Str || b->kind != JVal::Str || c->kind != JVal::Str ||
                !parse_vec3(a->str, E.pos) || !parse_vec3(b->str, E.rot) || !parse_vec3(c->str, E.scale))
                return fail(VXL_ERR_IO, "prefab_load: %s: bad Transform", path.c_str());
        }
        const JVal* vr = ent.get("VoxRenderer");
        if (vr && vr->kind == JVal::Obj) {
            vxl_prefab::Entity& E = P->ents[e];
            const JVal* pa = vr->get("Pallete");
            const JVal* vo = vr->get("Vox");
            if (!pa || !vo || pa->kind != JVal::Str || vo->kind != JVal::Str || !parse_guid(pa->str, &E.pal) ||
                !parse_guid(vo->str, &E.vox))
                return fail(VXL_ERR_IO, "prefab_load: %s: bad VoxRenderer", path.c_str());
            const JVal* pv = vr->get("Pivot");
            E.pivot[0] = E.pivot[1] = E.pivot[2] = 0.0f;
            if (pv && pv->kind == JVal::Str && !parse_vec3(pv->str, E.pivot))
                return fail(VXL_ERR_IO, "prefab_load: %s: bad Pivot", path.c_str());
            E.has_vox = true;
        }
    }
    if (root < 0) return fail(VXL_ERR_IO, "prefab_load: %s: no root entity", path.c_str());
    *root_out = root;
    return VXL_OK;
}

}  // namespace
}  // namespace vxl

using namespace vxl;

extern "C" {

uint64_t vxl_asset_guid(const char* path) {
    uint64_t h = 14695981039346656037ull;
    for (const unsigned char* c = (const unsigned char*)(path ? path : ""); *c; c++) {
        h ^= (uint64_t)*c;
        h *= 1099511628211ull;
    }
    return h;
}

vxl_status vxl_read_palette(const char* path, uint8_t* h_materials) {
    if (!path || !h_materials) return fail(VXL_ERR_INVALID_ARG, "read_palette: NULL argument");
    std::string t;
    if (!read_file(path, &t)) return fail(VXL_ERR_IO, "read_palette: cannot read %s", path);
    if (t.size() != 256 * 7) return fail(VXL_ERR_IO, "read_palette: %s: %zu bytes, expected 1792", path, t.size());
    std::memcpy(h_materials, t.data(), t.size());
    return VXL_OK;
}

vxl_status vxl_transform_matrix(const float pos[3], const float rot[3], const float scale[3], const float* parent,
                                float out[16]) {
    if (!pos || !rot || !scale || !out) return fail(VXL_ERR_INVALID_ARG, "transform_matrix: NULL argument");
    transform_matrix(pos, rot, scale, parent, out);
    return VXL_OK;
}

vxl_status vxl_prefab_load(const char* mods_dir, const char* mod_path, vxl_prefab** out) {
    if (!mods_dir || !mod_path || !out) return fail(VXL_ERR_INVALID_ARG, "prefab_load: NULL argument");
    *out = nullptr;
    std::unique_ptr<vxl_prefab> P(new vxl_prefab());
    P->mods_dir = mods_dir;
    namespace fs = std::filesystem;
    std::error_code ec;
    const fs::path root(mods_dir);
    if (!fs::is_directory(root, ec)) return fail(VXL_ERR_IO, "prefab_load: %s is not a directory", mods_dir);
    for (fs::recursive_directory_iterator it(root, ec), e; !ec && it != e; it.increment(ec)) {
        if (!it->is_regular_file(ec)) continue;
        const std::string rel = fs::relative(it->path(), root, ec).generic_string();
        if (ec) continue;
        P->index[vxl_asset_guid(rel.c_str())] = it->path().string();
    }
    const std::string rel(mod_path);
    auto it = P->index.find(vxl_asset_guid(rel.c_str()));
    if (it == P->index.end()) return fail(VXL_ERR_IO, "prefab_load: %s not found under %s", mod_path, mods_dir);
    int r = -1;
    VXL_TRY(spawn(P.get(), vxl_asset_guid(rel.c_str()), it->second, -1, 0, &r));
    // world matrices, parents first (an entity's parent is created before it
    // or is an instance root spawned before its own children)
    std::vector<int> done(P->ents.size(), 0);
    for (size_t pass = 0; pass <= P->ents.size(); pass++) {
        bool all = true;
        for (size_t i = 0; i < P->ents.size(); i++) {
            if (done[i]) continue;
            auto& E = P->ents[i];
            if (E.parent >= 0 && !done[(size_t)E.parent]) {
                all = false;
                continue;
            }
            transform_matrix(E.pos, E.rot, E.scale, E.parent >= 0 ? P->ents[(size_t)E.parent].world : nullptr,
                             E.world);
            done[i] = 1;
        }
        if (all) break;
    }
    for (size_t i = 0; i < P->ents.size(); i++)
        if (!done[i]) return fail(VXL_ERR_IO, "prefab_load: %s: cyclic parents", mod_path);
    // volumes and palettes, in order of first use
    for (size_t i = 0; i < P->ents.size(); i++) {
        const auto& E = P->ents[i];
        // a VoxRenderer whose Vox is the null GUID draws nothing (the systems
        // skip renderers whose asset is not valid, ShadowVoxSystem.cpp:121)
        if (!E.has_vox || E.vox == 0) continue;
        int vi, pi;
        auto fv = P->vol_of.find(E.vox);
        if (fv == P->vol_of.end()) {
            auto f = P->index.find(E.vox);
            if (f == P->index.end())
                return fail(VXL_ERR_IO, "prefab_load: unresolved Vox GUID %016llX", (unsigned long long)E.vox);
            vxl_prefab::Vol V;
            V.guid = E.vox;
            int32_t sx, sy, sz;
            VXL_TRY(vxl_read_v(f->second.c_str(), &sx, &sy, &sz, nullptr, 0));
            V.sx = sx;
            V.sy = sy;
            V.sz = sz;
            V.data.resize((size_t)sx * sy * sz);
            VXL_TRY(vxl_read_v(f->second.c_str(), &sx, &sy, &sz, V.data.data(), V.data.size()));
            vi = (int)P->vols.size();
            P->vols.push_back(std::move(V));
            P->vol_of[E.vox] = vi;
        } else {
            vi = fv->second;
        }
        auto fp = P->pal_of.find(E.pal);
        if (fp == P->pal_of.end()) {
            auto f = P->index.find(E.pal);
            if (f == P->index.end())
                return fail(VXL_ERR_IO, "prefab_load: unresolved Pallete GUID %016llX", (unsigned long long)E.pal);
            vxl_prefab::Pal Q;
            Q.guid = E.pal;
            Q.mats.resize(256 * 7);
            VXL_TRY(vxl_read_palette(f->second.c_str(), Q.mats.data()));
            pi = (int)P->pals.size();
            P->pals.push_back(std::move(Q));
            P->pal_of[E.pal] = pi;
        } else {
            pi = fp->second;
        }
        P->rens.push_back({(int)i, vi, pi});
    }
    *out = P.release();
    return VXL_OK;
}

vxl_status vxl_prefab_info(const vxl_prefab* P, int32_t* n_renderers, int32_t* n_volumes, int32_t* n_palettes) {
    if (!P) return fail(VXL_ERR_INVALID_ARG, "prefab_info: NULL prefab");
    if (n_renderers) *n_renderers = (int32_t)P->rens.size();
    if (n_volumes) *n_volumes = (int32_t)P->vols.size();
    if (n_palettes) *n_palettes = (int32_t)P->pals.size();
    return VXL_OK;
}

vxl_status vxl_prefab_renderer_at(const vxl_prefab* P, int i, vxl_prefab_renderer* out) {
    if (!P || !out) return fail(VXL_ERR_INVALID_ARG, "prefab_renderer_at: NULL argument");
    if (i < 0 || i >= (int)P->rens.size()) return fail(VXL_ERR_OUT_OF_RANGE, "prefab_renderer_at: index %d", i);
    const auto& R = P->rens[(size_t)i];
    const auto& E = P->ents[(size_t)R.entity];
    std::memcpy(out->world, E.world, sizeof(out->world));
    std::memcpy(out->pivot, E.pivot, sizeof(out->pivot));
    out->volume = R.vol;
    out->palette = R.pal;
    out->entity = R.entity;
    return VXL_OK;
}

vxl_status vxl_prefab_volume_at(const vxl_prefab* P, int i, int32_t* sx, int32_t* sy, int32_t* sz,
                                const uint8_t** h_data, uint64_t* guid) {
    if (!P) return fail(VXL_ERR_INVALID_ARG, "prefab_volume_at: NULL prefab");
    if (i < 0 || i >= (int)P->vols.size()) return fail(VXL_ERR_OUT_OF_RANGE, "prefab_volume_at: index %d", i);
    const auto& V = P->vols[(size_t)i];
    if (sx) *sx = V.sx;
    if (sy) *sy = V.sy;
    if (sz) *sz = V.sz;
    if (h_data) *h_data = V.data.data();
    if (guid) *guid = V.guid;
    return VXL_OK;
}

vxl_status vxl_prefab_palette_at(const vxl_prefab* P, int i, const uint8_t** h_materials, uint64_t* guid) {
    if (!P) return fail(VXL_ERR_INVALID_ARG, "prefab_palette_at: NULL prefab");
    if (i < 0 || i >= (int)P->pals.size()) return fail(VXL_ERR_OUT_OF_RANGE, "prefab_palette_at: index %d", i);
    if (h_materials) *h_materials = P->pals[(size_t)i].mats.data();
    if (guid) *guid = P->pals[(size_t)i].guid;
    return VXL_OK;
}

vxl_status vxl_prefab_destroy(vxl_prefab* P) {
    delete P;
    return VXL_OK;
}

}  // extern "C"
