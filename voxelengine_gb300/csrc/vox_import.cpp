// vox_import.cpp — MagicaVoxel .vox import as the engine's importer does it
// (Sources/Editor/Importer/VoxImporter.cpp): the models it writes as .v files,
// one per shape instance of the scene graph, and the palette it writes as .p.
//
//  - Chunk loop (VoxImporter.cpp:280-393): after "VOX " and the version, each
//    chunk header (4 bytes, content size, children size) is dispatched on its
//    first letter(s) and its content read field by field -- sizes are never
//    used to skip. An unknown letter ends the import, and so does the first
//    chunk the loop misreads (rCAM is read as a dictionary); in the shipped
//    files that happens after every shape, node, palette and material chunk.
//    Reads past the end leave the destination as it was (an ifstream).
//  - Nodes are indexed in file order (nTRN, nGRP, nSHP as they come); shapes
//    are the SIZE + XYZI pairs in file order.
//  - Entities (VoxImporter.cpp:396-480): from node 0 (a transform) down;
//    a transform's position is (x, z, -y) * 0.1 of its "_t"; a group's
//    children are transforms; a shape under a transform becomes a model of
//    size (x, z, y) of its rotated size (rotation "_r", a byte of axis indices
//    and signs), each voxel (x, y, z, colour) placed at (x', z', Y - 1 - y')
//    of its rotated coordinates, the model's position less its centre * 0.1;
//    its name is the transform's "_name" or a running counter.
//  - VoxAsset sizes round up to a multiple of 4 (VoxAsset.h:26-33), bytes x
//    fastest (VoxAsset.h:52-56).
//  - Palette (VoxImporter.cpp:500-512): material i takes the RGBA chunk's
//    colour i - 1 (MagicaVoxel's index offset) and the MATL chunk of id i
//    (roughness, metallic, emit scaled by 255 and truncated); alpha and
//    anything no chunk set are left unset by the importer (zero here).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "vxl_internal.h"

namespace vxl {
namespace {

// byte stream with the engine's read semantics: a short read copies what is
// left and leaves the rest of the destination untouched
struct VoxReader {
    const std::vector<uint8_t>& b;
    size_t off = 0;
    explicit VoxReader(const std::vector<uint8_t>& bytes) : b(bytes) {}
    void read(void* dst, size_t n) {
        const size_t k = off < b.size() ? std::min(n, b.size() - off) : 0;
        if (k) std::memcpy(dst, b.data() + off, k);
        off += k;
    }
    int32_t i32(int32_t init = 0) {
        int32_t v = init;
        read(&v, 4);
        return v;
    }
    bool str(std::string* s) {
        const int32_t n = i32();
        if (n < 0 || (size_t)n > b.size()) return false;  // the engine would fail to allocate
        s->assign((size_t)n, '\0');
        read(&(*s)[0], (size_t)n);
        return true;
    }
    bool dict(std::map<std::string, std::string>* m) {
        const int32_t n = i32();
        if (n < 0 || (size_t)n > b.size()) return false;
        for (int32_t i = 0; i < n; i++) {
            std::string k, v;
            if (!str(&k) || !str(&v)) return false;
            (*m)[k] = v;
        }
        return true;
    }
};

// std::from_chars for an int: optional '-', digits; 0 digits leaves v as it was
bool parse_int(const char* p, const char* e, int* v) {
    bool neg = false;
    if (p < e && *p == '-') {
        neg = true;
        p++;
    }
    if (p >= e || *p < '0' || *p > '9') return false;
    long long x = 0;
    while (p < e && *p >= '0' && *p <= '9') x = x * 10 + (*p++ - '0');
    *v = (int)(neg ? -x : x);
    return true;
}

// std::from_chars for a float in the plain decimal forms MATL values use
bool parse_float(const std::string& s, float* v) {
    char* end = nullptr;
    const float x = std::strtof(s.c_str(), &end);
    if (end == s.c_str()) return false;
    *v = x;
    return true;
}

// the rotation byte of nTRN "_r" (VoxImporter.cpp:20-81)
struct VoxRot {
    int rx = 0, ry = 1, rz = 2, sx = 0, sy = 0, sz = 0;
    explicit VoxRot(uint8_t r = 4) {
        rx = r & 3;
        ry = (r >> 2) & 3;
        rz = 3 - (rx | ry);
        sx = (r >> 4) & 1;
        sy = (r >> 5) & 1;
        sz = (r >> 6) & 1;
    }
    static int at(int i, const int v[3]) { return v[i < 0 ? 0 : (i > 2 ? 2 : i)]; }
    void size(const int s[3], int o[3]) const {
        o[0] = at(rx, s);
        o[1] = at(ry, s);
        o[2] = at(rz, s);
    }
    void apply(const int v[3], const int s[3], int o[3]) const {
        const int x = at(rx, v), y = at(ry, v), z = at(rz, v);
        o[0] = sx ? at(rx, s) - x - 1 : x;
        o[1] = sy ? at(ry, s) - y - 1 : y;
        o[2] = sz ? at(rz, s) - z - 1 : z;
    }
};

struct VoxNode {
    int kind = 0;  // 1 transform, 2 group, 3 shape
    // transform
    int x = 0, y = 0, z = 0, child = -1;
    VoxRot rot;
    std::string name;
    // group
    std::vector<int> children;
    // shape
    int shape = -1;
};

struct VoxShapeData {
    int size[3];
    std::vector<uint32_t> voxels;
};

int round4(int v) { return ((v - 1) & ~3) + 4; }

}  // namespace
}  // namespace vxl

struct vxl_vox_scene {
    struct Model {
        std::string name;
        int32_t size[3];
        std::vector<uint8_t> data;
        float position[3];  // world position (the entity's and its groups' translations)
    };
    std::vector<Model> models;
    uint8_t palette[256 * 7];
};

namespace vxl {
namespace {

struct VoxImport {
    std::vector<VoxNode> nodes;
    std::vector<VoxShapeData> shapes;
    uint8_t rgba[257][4] = {};
    uint8_t surf[257][3] = {};  // emit, roughness, metallic
    int sizeX = 0, sizeY = 0, sizeZ = 0;
    int counter = 0;
    std::string err;

    bool parse(const std::vector<uint8_t>& bytes) {
        VoxReader s(bytes);
        char magic[4] = {0, 0, 0, 0};
        s.read(magic, 4);
        if (std::memcmp(magic, "VOX ", 4) != 0) {
            err = "not a .vox file";
            return false;
        }
        s.i32();  // version
        for (;;) {
            char h[4] = {' ', ' ', ' ', ' '};
            s.read(h, 4);
            s.i32();  // content size
            s.i32();  // children size
            switch (h[0]) {
                case 'M':
                    if (h[2] == 'T' && !matl(s)) return true;  // MATL; MAIN has no content
                    break;
                case 'P':
                    s.i32();  // PACK
                    break;
                case 'S':
                    sizeX = s.i32(sizeX);
                    sizeY = s.i32(sizeY);
                    sizeZ = s.i32(sizeZ);
                    break;
                case 'X': {
                    const int32_t n = s.i32();
                    if (n < 0 || (size_t)n > bytes.size()) return true;
                    VoxShapeData d;
                    d.voxels.assign((size_t)n, 0u);
                    s.read(d.voxels.data(), (size_t)n * 4);
                    d.size[0] = sizeX;
                    d.size[1] = sizeY;
                    d.size[2] = sizeZ;
                    shapes.push_back(std::move(d));
                    break;
                }
                case 'R':
                    s.read(&rgba[1][0], 256 * 4);
                    break;
                case 'L': {
                    s.i32();
                    std::map<std::string, std::string> m;
                    if (!s.dict(&m)) return true;
                    s.i32();
                    break;
                }
                case 'I': {
                    uint8_t remap[256];
                    s.read(remap, 256);  // read, not applied (as the importer)
                    break;
                }
                case 'r': {
                    std::map<std::string, std::string> m;
                    if (!s.dict(&m)) return true;
                    break;
                }
                case 'n':
                    if (!node(s, h[1])) return true;
                    break;
                default:
                    return true;
            }
        }
    }

    bool matl(VoxReader& s) {
        const int32_t id = s.i32();
        std::map<std::string, std::string> p;
        if (!s.dict(&p)) return false;
        float rough = 0.0f, emit = 0.0f, metal = 0.0f;
        const std::string type = p["_type"];
        if (type == "_metal" || type == "_blend") {
            if (p.count("_rough")) parse_float(p["_rough"], &rough);
            if (p.count("_metal")) parse_float(p["_metal"], &metal);
        } else if (type == "_emit") {
            if (p.count("_emit")) parse_float(p["_emit"], &emit);
        } else if (type == "_diffuse") {
            rough = 0.9f;
        }
        if (id >= 0 && id < 257) {
            surf[id][0] = (uint8_t)(int)(emit * 255.0f);
            surf[id][1] = (uint8_t)(int)(rough * 255.0f);
            surf[id][2] = (uint8_t)(int)(metal * 255.0f);
        }
        return true;
    }

    bool node(VoxReader& s, char type) {
        s.i32();  // node id: nodes are indexed in file order
        std::map<std::string, std::string> attr;
        if (!s.dict(&attr)) return false;
        VoxNode n;
        n.name = attr.count("_name") ? attr["_name"] : std::string();
        if (type == 'T') {
            n.kind = 1;
            n.child = s.i32();
            s.i32();  // reserved
            s.i32();  // layer
            s.i32();  // frames
            std::map<std::string, std::string> f;
            if (!s.dict(&f)) return false;
            const std::string t = f["_t"];
            if (!t.empty()) {
                // three integers separated by single spaces (the importer's find / from_chars walk)
                const char* p = t.data();
                const char* e = p + t.size();
                const char* a = std::find(p + 1 < e ? p + 1 : e, e, ' ');
                parse_int(p, a, &n.x);
                const char* b = a < e ? std::find(a + 2 < e ? a + 2 : e, e, ' ') : e;
                parse_int(a < e ? a + 1 : e, b, &n.y);
                parse_int(b < e ? b + 1 : e, e, &n.z);
            }
            int r = 4;
            const std::string rs = f["_r"];
            if (!rs.empty()) parse_int(rs.data(), rs.data() + rs.size(), &r);
            n.rot = VoxRot((uint8_t)r);
        } else if (type == 'G') {
            n.kind = 2;
            const int32_t k = s.i32();
            if (k < 0 || (size_t)k > s.b.size()) return false;
            n.children.resize((size_t)k);
            for (int32_t i = 0; i < k; i++) n.children[(size_t)i] = s.i32();
        } else if (type == 'S') {
            n.kind = 3;
            s.i32();  // models: always 1
            n.shape = s.i32();
            std::map<std::string, std::string> m;
            if (!s.dict(&m)) return false;
        } else {
            return true;  // another 'n' chunk: its header and attributes are read, nothing kept
        }
        nodes.push_back(std::move(n));
        return true;
    }

    // CreateEntity (VoxImporter.cpp:396-480) for transform node `ti` whose
    // parent group sits at `base` (world position)
    bool entity(int ti, const float base[3], vxl_vox_scene* out, int depth) {
        if (depth > 256 || ti < 0 || ti >= (int)nodes.size() || nodes[(size_t)ti].kind != 1) {
            err = "malformed scene graph";
            return false;
        }
        const VoxNode& T = nodes[(size_t)ti];
        float pos[3] = {(float)T.x * 0.1f, (float)T.z * 0.1f, (float)(-T.y) * 0.1f};
        if (T.child < 0 || T.child >= (int)nodes.size()) {
            err = "malformed scene graph";
            return false;
        }
        const VoxNode& C = nodes[(size_t)T.child];
        if (C.kind == 2) {
            const float w[3] = {base[0] + pos[0], base[1] + pos[1], base[2] + pos[2]};
            for (int c : C.children)
                if (!entity(c, w, out, depth + 1)) return false;
            return true;
        }
        if (C.kind != 3) return true;  // the importer creates an empty entity
        if (C.shape < 0 || C.shape >= (int)shapes.size()) {
            err = "shape index out of range";
            return false;
        }
        const VoxShapeData& D = shapes[(size_t)C.shape];
        int ts[3];
        T.rot.size(D.size, ts);
        vxl_vox_scene::Model M;
        M.size[0] = round4(ts[0]);
        M.size[1] = round4(ts[2]);
        M.size[2] = round4(ts[1]);
        M.data.assign((size_t)M.size[0] * M.size[1] * M.size[2], 0);
        const int center[3] = {T.rot.sx ? ts[0] - ts[0] / 2 : ts[0] / 2, T.rot.sz ? ts[2] - ts[2] / 2 : ts[2] / 2,
                               !T.rot.sy ? ts[1] - ts[1] / 2 : ts[1] / 2};
        for (int a = 0; a < 3; a++) pos[a] = pos[a] - (float)center[a] * 0.1f;
        for (uint32_t v : D.voxels) {
            const int c[3] = {(int)(v & 0xff), (int)((v >> 8) & 0xff), (int)((v >> 16) & 0xff)};
            int o[3];
            T.rot.apply(c, D.size, o);
            const int64_t X = o[0], Y = o[2], Z = ts[1] - 1 - o[1];
            if (X < 0 || Y < 0 || Z < 0 || X >= M.size[0] || Y >= M.size[1] || Z >= M.size[2]) {
                err = "voxel outside its model";
                return false;
            }
            M.data[(size_t)(X + Y * M.size[0] + Z * (int64_t)M.size[0] * M.size[1])] = (uint8_t)(v >> 24);
        }
        M.name = T.name.empty() ? std::to_string(counter++) : T.name;
        for (int a = 0; a < 3; a++) M.position[a] = base[a] + pos[a];
        out->models.push_back(std::move(M));
        return true;
    }
};

}  // namespace
}  // namespace vxl

using namespace vxl;

extern "C" {

vxl_status vxl_vox_load(const char* path, vxl_vox_scene** out) {
    if (!path || !out) return fail(VXL_ERR_INVALID_ARG, "vox_load: NULL argument");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(VXL_ERR_IO, "vox_load: cannot read %s", path);
    std::vector<uint8_t> bytes;
    uint8_t buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + k);
    std::fclose(f);
    VoxImport I;
    if (!I.parse(bytes)) return fail(VXL_ERR_INVALID_ARG, "vox_load: %s: %s", path, I.err.c_str());
    if (I.nodes.empty()) return fail(VXL_ERR_INVALID_ARG, "vox_load: %s: no scene graph", path);
    std::unique_ptr<vxl_vox_scene> S(new vxl_vox_scene());
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    if (!I.entity(0, zero, S.get(), 0)) return fail(VXL_ERR_INVALID_ARG, "vox_load: %s: %s", path, I.err.c_str());
    for (int i = 0; i < 256; i++) {
        uint8_t* m = S->palette + 7 * i;
        m[0] = I.rgba[i][0];
        m[1] = I.rgba[i][1];
        m[2] = I.rgba[i][2];
        m[3] = 0;
        m[4] = I.surf[i][1];
        m[5] = I.surf[i][2];
        m[6] = I.surf[i][0];
    }
    *out = S.release();
    return VXL_OK;
}

vxl_status vxl_vox_info(const vxl_vox_scene* s, int32_t* n_models) {
    if (!s || !n_models) return fail(VXL_ERR_INVALID_ARG, "vox_info: NULL argument");
    *n_models = (int32_t)s->models.size();
    return VXL_OK;
}

vxl_status vxl_vox_model_at(const vxl_vox_scene* s, int32_t i, char* name, int32_t name_cap, int32_t size[3],
                            const uint8_t** h_data, float position[3]) {
    if (!s) return fail(VXL_ERR_INVALID_ARG, "vox_model_at: NULL scene");
    if (i < 0 || i >= (int32_t)s->models.size()) return fail(VXL_ERR_OUT_OF_RANGE, "vox_model_at: index %d", i);
    const auto& M = s->models[(size_t)i];
    if (name && name_cap > 0) {
        std::snprintf(name, (size_t)name_cap, "%s", M.name.c_str());
    }
    if (size) std::memcpy(size, M.size, sizeof(M.size));
    if (h_data) *h_data = M.data.data();
    if (position) std::memcpy(position, M.position, sizeof(M.position));
    return VXL_OK;
}

vxl_status vxl_vox_palette(const vxl_vox_scene* s, uint8_t* h_materials) {
    if (!s || !h_materials) return fail(VXL_ERR_INVALID_ARG, "vox_palette: NULL argument");
    std::memcpy(h_materials, s->palette, sizeof(s->palette));
    return VXL_OK;
}

vxl_status vxl_vox_destroy(vxl_vox_scene* s) {
    delete s;
    return VXL_OK;
}

}  // extern "C"
