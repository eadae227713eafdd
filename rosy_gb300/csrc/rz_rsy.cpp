// Reader for Rosy's .rsy asset files, so that real assets feed the C ABI.
//
// The format is the one rosy_asset::asset::write produces
// (src/Asset/Asset.cpp:28-407, read back by 409-848): little-endian raw records
// of the x64 layouts in src/Asset/Asset.h, with every count a 64-bit size_t:
//   header (80 bytes: magic "RSYF", version 1, endianness 1, coordinate system
//     float[16], root scene u32)
//   6 counts: materials, samplers, scenes, nodes, images, meshes
//   materials (68 bytes each), samplers (4 x u16 each)
//   per scene: node count, u32 node indices
//   per node: 7 counts (1, 1, 1, 1, 1, children, name chars), world translate
//     float[3], world scale, world yaw, transform float[16], mesh id u32,
//     u32 child indices, name chars
//   per image: 2 counts (1, name chars), image type u32, name chars
//   per mesh: 3 counts (positions, indices, surfaces), 64-byte positions,
//     u32 indices, 36-byte surfaces
// Fields are decoded one by one from bytes (no struct punning), and every
// count is checked against the bytes left in the file before anything is
// allocated, so a truncated or corrupt file fails with RZ_READ_FAILED.
//
// rz_rsy_get_scene flattens the root scene the way the level does when it
// receives a new asset (src/Engine/Level.cpp:922-1160 with the node transform
// of src/Engine/Node.cpp:96-103): breadth first from the root scene's nodes;
// a node's world transform is T(world_translate) * R(-y axis, world_yaw) *
// S(world_scale) * coordinate_system * parent_object_space * transform, where
// parent_object_space accumulates the ancestors' transforms; every node with a
// mesh yields one graphics object and one surface per mesh surface; nodes
// named "mobs" and their descendants are dynamic and are placed after all the
// static objects (their surfaces carry graphic_objects_offset = number of
// static objects). The matrices are formed in double precision and rounded to
// float once.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/rosy_gb300.h"

namespace {

constexpr uint32_t kMagic = 0x52535946u;  // "RSYF"
constexpr uint32_t kVersion = 1;
constexpr size_t kHeaderBytes = 80;
constexpr size_t kMaterialBytes = 68;
constexpr size_t kSamplerBytes = 8;
constexpr size_t kPositionBytes = 64;
constexpr size_t kSurfaceBytes = 36;

struct Node {
    float world_translate[3] = {0, 0, 0};
    float world_scale = 1.0f;
    float world_yaw = 0.0f;
    float transform[16] = {};
    uint32_t mesh_id = RZ_INVALID_INDEX;
    std::vector<uint32_t> children;
    std::string name;
};

struct Surface {
    uint32_t start_index = 0, count = 0, material = RZ_INVALID_INDEX;
    float min_bounds[3] = {0, 0, 0}, max_bounds[3] = {0, 0, 0};
};

struct Mesh {
    std::vector<rz_vertex> positions;
    std::vector<uint32_t> indices;
    std::vector<Surface> surfaces;
};

struct Image {
    uint32_t type = 0;
    std::string name;
};

class Reader {
public:
    explicit Reader(std::vector<unsigned char> b) : buf_(std::move(b)) {}
    bool ok() const { return ok_; }
    size_t left() const { return buf_.size() - pos_; }
    bool need(size_t n) {
        if (!ok_ || n > left()) ok_ = false;
        return ok_;
    }
    uint32_t u32() {
        if (!need(4)) return 0;
        const unsigned char* p = &buf_[pos_];
        pos_ += 4;
        return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    }
    uint16_t u16() {
        if (!need(2)) return 0;
        const unsigned char* p = &buf_[pos_];
        pos_ += 2;
        return (uint16_t)(p[0] | (p[1] << 8));
    }
    uint8_t u8() {
        if (!need(1)) return 0;
        return buf_[pos_++];
    }
    uint64_t u64() {
        const uint64_t lo = u32();
        const uint64_t hi = u32();
        return lo | (hi << 32);
    }
    float f32() {
        const uint32_t v = u32();
        float f;
        std::memcpy(&f, &v, 4);
        return f;
    }
    void skip(size_t n) {
        if (need(n)) pos_ += n;
    }
    // A count of records of `bytes` each that must still fit in the file.
    size_t count(size_t bytes) {
        const uint64_t n = u64();
        if (!ok_ || (bytes > 0 && n > left() / bytes) || n > 0xFFFFFFFFull) {
            ok_ = false;
            return 0;
        }
        return (size_t)n;
    }

private:
    std::vector<unsigned char> buf_;
    size_t pos_ = 0;
    bool ok_ = true;
};

// 4x4 column-major double matrices (element (row r, column c) at [c * 4 + r]).
struct M4 {
    double m[16];
};
M4 identity() {
    M4 a{};
    for (int i = 0; i < 4; ++i) a.m[i * 5] = 1.0;
    return a;
}
M4 mul(const M4& a, const M4& b) {
    M4 c{};
    for (int col = 0; col < 4; ++col)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a.m[k * 4 + r] * b.m[col * 4 + k];
            c.m[col * 4 + r] = s;
        }
    return c;
}
M4 from_floats(const float* f) {
    M4 a{};
    for (int i = 0; i < 16; ++i) a.m[i] = f[i];
    return a;
}
bool invert(const M4& a, M4& out) {  // Gauss-Jordan with partial pivoting
    double w[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            w[r][c] = a.m[c * 4 + r];
            w[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
        if (w[p][c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(w[p][k], w[c][k]);
        const double inv = 1.0 / w[c][c];
        for (int k = 0; k < 8; ++k) w[c][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = w[r][c];
            for (int k = 0; k < 8; ++k) w[r][k] -= f * w[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out.m[c * 4 + r] = w[r][c + 4];
    return true;
}

// T(t) * R(axis -y, yaw) * S(s) (src/Engine/Node.cpp:96-101).
M4 world_trs(const float t[3], float yaw, float s) {
    M4 T = identity();
    T.m[12] = t[0];
    T.m[13] = t[1];
    T.m[14] = t[2];
    // rotation by yaw about (0, -1, 0) = rotation by -yaw about +y
    const double c = std::cos((double)yaw), sn = std::sin(-(double)yaw);
    M4 R = identity();
    R.m[0] = c;
    R.m[8] = sn;
    R.m[2] = -sn;
    R.m[10] = c;
    M4 S = identity();
    S.m[0] = S.m[5] = S.m[10] = s;
    return mul(mul(T, R), S);
}

}  // namespace

struct rz_rsy {
    float coordinate_system[16] = {};
    uint32_t root_scene = 0;
    std::vector<rz_material> materials;
    std::vector<rz_sampler> samplers;
    std::vector<std::vector<uint32_t>> scenes;
    std::vector<Node> nodes;
    std::vector<Image> images;
    std::vector<Mesh> meshes;
    // flattened root scene
    std::vector<rz_object> objects;
    std::vector<rz_surface> surfaces;
    uint32_t static_objects = 0;
    bool scene_ok = false;
};

namespace {

int parse(Reader& r, rz_rsy& a) {
    if (!r.need(kHeaderBytes)) return RZ_READ_FAILED;
    if (r.u32() != kMagic) return RZ_READ_FAILED;
    if (r.u32() != kVersion) return RZ_READ_FAILED;
    if (r.u32() != 1u) return RZ_READ_FAILED;  // little-endian marker
    for (float& f : a.coordinate_system) f = r.f32();
    a.root_scene = r.u32();
    const size_t n_materials = r.count(kMaterialBytes);
    const size_t n_samplers = r.count(kSamplerBytes);
    const size_t n_scenes = r.count(8);
    const size_t n_nodes = r.count(56 + 88);
    const size_t n_images = r.count(16 + 4);
    const size_t n_meshes = r.count(24);
    if (!r.ok()) return RZ_READ_FAILED;
    a.materials.resize(n_materials);
    for (rz_material& m : a.materials) {
        m.double_sided = r.u8();
        r.skip(3);
        for (float& f : m.base_color_factor) f = r.f32();
        m.metallic_factor = r.f32();
        m.roughness_factor = r.f32();
        m.alpha_mode = r.u8();
        r.skip(3);
        m.alpha_cutoff = r.f32();
        m.color_image_index = r.u32();
        m.color_sampler_index = r.u32();
        m.normal_image_index = r.u32();
        m.normal_sampler_index = r.u32();
        m.metallic_image_index = r.u32();
        m.metallic_sampler_index = r.u32();
        m.mixmap_image_index = r.u32();
        m.mixmap_sampler_index = r.u32();
    }
    a.samplers.resize(n_samplers);
    for (rz_sampler& s : a.samplers) {
        s.min_filter = r.u16();
        s.mag_filter = r.u16();
        s.wrap_s = r.u16();
        s.wrap_t = r.u16();
    }
    a.scenes.resize(n_scenes);
    for (auto& s : a.scenes) {
        const size_t n = r.count(4);
        s.resize(n);
        for (uint32_t& v : s) v = r.u32();
    }
    a.nodes.resize(n_nodes);
    for (Node& n : a.nodes) {
        const uint64_t ones[5] = {r.u64(), r.u64(), r.u64(), r.u64(), r.u64()};
        for (uint64_t o : ones)
            if (o != 1) return RZ_READ_FAILED;  // one translate, scale, yaw, transform and mesh id per node
        const size_t n_children = r.count(4);
        const size_t n_chars = r.count(1);
        for (float& f : n.world_translate) f = r.f32();
        n.world_scale = r.f32();
        n.world_yaw = r.f32();
        for (float& f : n.transform) f = r.f32();
        n.mesh_id = r.u32();
        n.children.resize(n_children);
        for (uint32_t& c : n.children) c = r.u32();
        n.name.resize(n_chars);
        for (char& ch : n.name) ch = (char)r.u8();
        if (!r.ok()) return RZ_READ_FAILED;
    }
    a.images.resize(n_images);
    for (Image& im : a.images) {
        if (r.u64() != 1) return RZ_READ_FAILED;
        const size_t n_chars = r.count(1);
        im.type = r.u32();
        im.name.resize(n_chars);
        for (char& ch : im.name) ch = (char)r.u8();
    }
    a.meshes.resize(n_meshes);
    for (Mesh& m : a.meshes) {
        const size_t n_pos = r.count(kPositionBytes);
        const size_t n_idx = r.count(4);
        const size_t n_surf = r.count(kSurfaceBytes);
        if (!r.ok()) return RZ_READ_FAILED;
        m.positions.resize(n_pos);
        for (rz_vertex& v : m.positions) {
            for (float& f : v.position) f = r.f32();
            for (float& f : v.normal) f = r.f32();
            for (float& f : v.tangent) f = r.f32();
            for (float& f : v.color) f = r.f32();
            for (float& f : v.uv) f = r.f32();
        }
        m.indices.resize(n_idx);
        for (uint32_t& v : m.indices) v = r.u32();
        m.surfaces.resize(n_surf);
        for (Surface& s : m.surfaces) {
            s.start_index = r.u32();
            s.count = r.u32();
            s.material = r.u32();
            for (float& f : s.min_bounds) f = r.f32();
            for (float& f : s.max_bounds) f = r.f32();
        }
        if (!r.ok()) return RZ_READ_FAILED;
    }
    return r.ok() ? RZ_OK : RZ_READ_FAILED;
}

rz_object object_of(const M4& world) {
    rz_object o{};
    for (int i = 0; i < 16; ++i) o.transform[i] = (float)world.m[i];
    M4 inv;
    if (!invert(world, inv)) inv = identity();
    for (int i = 0; i < 16; ++i) o.to_object_space_transform[i] = (float)inv.m[i];
    // transpose(inverse(mat3(world))) = the upper 3x3 of inverse(world), transposed, when the
    // last row of world is (0, 0, 0, 1): computed from the 3x3 directly for generality.
    double m3[9], i3[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) m3[c * 3 + r] = world.m[c * 4 + r];
    const double det = m3[0] * (m3[4] * m3[8] - m3[7] * m3[5]) - m3[3] * (m3[1] * m3[8] - m3[7] * m3[2]) +
                       m3[6] * (m3[1] * m3[5] - m3[4] * m3[2]);
    if (det != 0.0) {
        // inverse via the adjugate (column-major)
        i3[0] = (m3[4] * m3[8] - m3[7] * m3[5]) / det;
        i3[3] = -(m3[3] * m3[8] - m3[6] * m3[5]) / det;
        i3[6] = (m3[3] * m3[7] - m3[6] * m3[4]) / det;
        i3[1] = -(m3[1] * m3[8] - m3[7] * m3[2]) / det;
        i3[4] = (m3[0] * m3[8] - m3[6] * m3[2]) / det;
        i3[7] = -(m3[0] * m3[7] - m3[6] * m3[1]) / det;
        i3[2] = (m3[1] * m3[5] - m3[4] * m3[2]) / det;
        i3[5] = -(m3[0] * m3[5] - m3[3] * m3[2]) / det;
        i3[8] = (m3[0] * m3[4] - m3[3] * m3[1]) / det;
    } else {
        for (int i = 0; i < 9; ++i) i3[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) o.normal_transform[c * 3 + r] = (float)i3[r * 3 + c];  // transpose
    return o;
}

int flatten(rz_rsy& a) {
    if (a.root_scene >= a.scenes.size()) return RZ_INVALID_ARGUMENT;
    const auto& roots = a.scenes[a.root_scene];
    if (roots.empty()) return RZ_INVALID_ARGUMENT;
    struct Item {
        uint32_t node;
        M4 parent_object_space;
        bool mob;
    };
    std::deque<Item> queue;
    for (uint32_t n : roots) {
        if (n >= a.nodes.size()) return RZ_INVALID_ARGUMENT;
        queue.push_back({n, identity(), false});
    }
    const M4 coord = from_floats(a.coordinate_system);
    std::vector<rz_object> statics, mobs;
    std::vector<rz_surface> static_surfs, mob_surfs;
    size_t visited = 0;
    while (!queue.empty()) {
        const Item it = queue.front();
        queue.pop_front();
        if (++visited > 16u * a.nodes.size() + 16u) return RZ_INVALID_ARGUMENT;  // a cycle in the node graph
        const Node& n = a.nodes[it.node];
        const M4 object_space = mul(it.parent_object_space, from_floats(n.transform));
        const M4 world = mul(mul(world_trs(n.world_translate, n.world_yaw, n.world_scale), coord), object_space);
        if (n.mesh_id < a.meshes.size()) {
            const Mesh& m = a.meshes[n.mesh_id];
            auto& objs = it.mob ? mobs : statics;
            auto& surfs = it.mob ? mob_surfs : static_surfs;
            const uint32_t index = (uint32_t)objs.size();
            objs.push_back(object_of(world));
            for (const Surface& s : m.surfaces) {
                rz_surface sg{};
                sg.mesh_index = n.mesh_id;
                sg.graphic_objects_offset = 0;
                sg.graphics_object_index = index;
                sg.material_index = s.material;
                sg.index_count = s.count;
                sg.start_index = s.start_index;
                sg.blended = (s.material < a.materials.size() && a.materials[s.material].alpha_mode != 0) ? 1u : 0u;
                surfs.push_back(sg);
            }
        }
        for (uint32_t c : n.children) {
            if (c >= a.nodes.size()) return RZ_INVALID_ARGUMENT;
            queue.push_back({c, object_space, it.mob || a.nodes[c].name == "mobs"});
        }
    }
    a.static_objects = (uint32_t)statics.size();
    for (rz_surface& s : mob_surfs) s.graphic_objects_offset = a.static_objects;
    a.objects = statics;
    a.objects.insert(a.objects.end(), mobs.begin(), mobs.end());
    a.surfaces = static_surfs;
    a.surfaces.insert(a.surfaces.end(), mob_surfs.begin(), mob_surfs.end());
    a.scene_ok = true;
    return RZ_OK;
}

}  // namespace

extern "C" {

int rz_rsy_read(const char* path, rz_rsy** out) {
    if (!path || !out) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return RZ_OPEN_FAILED;
    std::vector<unsigned char> bytes;
    unsigned char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) bytes.insert(bytes.end(), chunk, chunk + n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return RZ_READ_FAILED;
    rz_rsy* a = new rz_rsy();
    Reader r(std::move(bytes));
    int rc = parse(r, *a);
    if (rc == RZ_OK) flatten(*a);  // a bad scene graph leaves the arrays readable; rz_rsy_get_scene reports it
    if (rc != RZ_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return RZ_OK;
}

void rz_rsy_free(rz_rsy* a) { delete a; }

int rz_rsy_get_info(const rz_rsy* a, rz_rsy_info* out) {
    if (!a || !out) return RZ_INVALID_ARGUMENT;
    rz_rsy_info i{};
    i.mesh_count = (uint32_t)a->meshes.size();
    i.material_count = (uint32_t)a->materials.size();
    i.sampler_count = (uint32_t)a->samplers.size();
    i.image_count = (uint32_t)a->images.size();
    i.node_count = (uint32_t)a->nodes.size();
    i.scene_count = (uint32_t)a->scenes.size();
    i.root_scene = a->root_scene;
    i.object_count = (uint32_t)a->objects.size();
    i.surface_count = (uint32_t)a->surfaces.size();
    i.static_object_count = a->static_objects;
    std::memcpy(i.coordinate_system, a->coordinate_system, sizeof(i.coordinate_system));
    *out = i;
    return RZ_OK;
}

int rz_rsy_get_meshes(const rz_rsy* a, rz_mesh* out, uint32_t capacity) {
    if (!a || (!out && capacity)) return RZ_INVALID_ARGUMENT;
    if (capacity < a->meshes.size()) return RZ_OVERFLOW;
    for (size_t i = 0; i < a->meshes.size(); ++i) {
        const Mesh& m = a->meshes[i];
        out[i].positions = m.positions.data();
        out[i].position_count = (uint32_t)m.positions.size();
        out[i].index_count = (uint32_t)m.indices.size();
        out[i].indices = m.indices.data();
    }
    return RZ_OK;
}

int rz_rsy_get_materials(const rz_rsy* a, rz_material* out, uint32_t capacity) {
    if (!a || (!out && capacity)) return RZ_INVALID_ARGUMENT;
    if (capacity < a->materials.size()) return RZ_OVERFLOW;
    std::copy(a->materials.begin(), a->materials.end(), out);
    return RZ_OK;
}

int rz_rsy_get_samplers(const rz_rsy* a, rz_sampler* out, uint32_t capacity) {
    if (!a || (!out && capacity)) return RZ_INVALID_ARGUMENT;
    if (capacity < a->samplers.size()) return RZ_OVERFLOW;
    std::copy(a->samplers.begin(), a->samplers.end(), out);
    return RZ_OK;
}

int rz_rsy_get_image(const rz_rsy* a, uint32_t index, uint32_t* image_type, char* name, uint32_t name_capacity,
                     uint32_t* name_length) {
    if (!a || index >= a->images.size()) return RZ_INVALID_ARGUMENT;
    const Image& im = a->images[index];
    if (image_type) *image_type = im.type;
    if (name_length) *name_length = (uint32_t)im.name.size();
    if (name && name_capacity) {
        const size_t n = std::min<size_t>(name_capacity - 1, im.name.size());
        std::memcpy(name, im.name.data(), n);
        name[n] = '\0';
    }
    return RZ_OK;
}

int rz_rsy_get_scene(const rz_rsy* a, rz_object* objects, uint32_t object_capacity, rz_surface* surfaces,
                     uint32_t surface_capacity) {
    if (!a) return RZ_INVALID_ARGUMENT;
    if (!a->scene_ok) return RZ_INVALID_ARGUMENT;
    if (object_capacity < a->objects.size() || surface_capacity < a->surfaces.size()) return RZ_OVERFLOW;
    if ((!objects && !a->objects.empty()) || (!surfaces && !a->surfaces.empty())) return RZ_INVALID_ARGUMENT;
    std::copy(a->objects.begin(), a->objects.end(), objects);
    std::copy(a->surfaces.begin(), a->surfaces.end(), surfaces);
    return RZ_OK;
}

}  // extern "C"
