// ORACLE — test infrastructure only. Drives the reference's own .rsy code
// (rosy_asset::asset::write and ::read, src/Asset/Asset.cpp:28-848, compiled
// from the reference's sources by the Makefile beside this file): builds an
// asset from a seed, writes it with asset::write, reads the file back with
// asset::read, and prints what the reference's reader decoded as JSON, so that
// the renderer's reader (rz_rsy_read) can be pinned to files and values the
// reference itself produced.
//
//   rsy_writer <out.rsy> <seed> <meshes> > out.json
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

#include "Asset/Asset.h"

namespace {

uint64_t g_state = 1;
uint32_t next_u32() {
    g_state = g_state * 6364136223846793005ull + 1442695040888963407ull;
    return (uint32_t)(g_state >> 33);
}
float next_f(float lo, float hi) { return lo + (hi - lo) * (float)(next_u32() & 0xFFFFFF) / 16777216.0f; }

void print_floats(const float* v, size_t n) {
    std::printf("[");
    for (size_t i = 0; i < n; ++i) std::printf("%s%.9g", i ? "," : "", (double)v[i]);
    std::printf("]");
}

void print_u32s(const uint32_t* v, size_t n) {
    std::printf("[");
    for (size_t i = 0; i < n; ++i) std::printf("%s%" PRIu32, i ? "," : "", v[i]);
    std::printf("]");
}

void print_chars(const std::vector<char>& c) {
    std::printf("\"");
    for (char ch : c) std::printf("%c", ch);
    std::printf("\"");
}

rosy_asset::asset make_asset(const std::string& path, uint32_t meshes) {
    rosy_asset::asset a;
    a.asset_path = path;
    for (int i = 0; i < 16; ++i) a.asset_coordinate_system[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    a.asset_coordinate_system[10] = -1.0f;  // a z flip, as an FBX import gives
    const uint32_t n_images = 5;
    for (uint32_t i = 0; i < n_images; ++i) {
        rosy_asset::image im;
        im.image_type = i % 4;
        const std::string name = "texture_" + std::to_string(i) + ".dds";
        im.name.assign(name.begin(), name.end());
        a.images.push_back(im);
    }
    for (uint32_t i = 0; i < 3; ++i) {
        rosy_asset::sampler s;
        s.min_filter = (uint16_t)(i * 2);
        s.mag_filter = (uint16_t)(5 - i);
        s.wrap_s = (uint16_t)(i % 3);
        s.wrap_t = (uint16_t)((i + 1) % 3);
        a.samplers.push_back(s);
    }
    for (uint32_t i = 0; i < 4; ++i) {
        rosy_asset::material m;
        m.double_sided = (uint8_t)(i & 1);
        for (int k = 0; k < 4; ++k) m.base_color_factor[k] = next_f(0.1f, 1.0f);
        m.metallic_factor = next_f(0.0f, 1.0f);
        m.roughness_factor = next_f(0.0f, 1.0f);
        m.alpha_mode = (uint8_t)(i == 3 ? 2 : (i == 2 ? 1 : 0));
        m.alpha_cutoff = i == 2 ? 0.5f : 0.0f;
        m.color_image_index = i % n_images;
        m.color_sampler_index = i % 3;
        m.normal_image_index = i == 1 ? UINT32_MAX : (i + 1) % n_images;
        m.normal_sampler_index = i == 1 ? UINT32_MAX : 0;
        m.metallic_image_index = (i + 2) % n_images;
        m.metallic_sampler_index = 1;
        m.mixmap_image_index = i == 0 ? 3 : UINT32_MAX;
        m.mixmap_sampler_index = i == 0 ? 2 : UINT32_MAX;
        a.materials.push_back(m);
    }
    for (uint32_t mi = 0; mi < meshes; ++mi) {
        rosy_asset::mesh me;
        const uint32_t nv = 24 + 12 * mi;
        for (uint32_t v = 0; v < nv; ++v) {
            rosy_asset::position p;
            for (int k = 0; k < 3; ++k) p.vertex[k] = next_f(-1.0f, 1.0f);
            for (int k = 0; k < 3; ++k) p.normal[k] = next_f(-1.0f, 1.0f);
            for (int k = 0; k < 3; ++k) p.tangents[k] = next_f(-1.0f, 1.0f);
            p.tangents[3] = (v & 1) ? 1.0f : -1.0f;
            for (int k = 0; k < 4; ++k) p.color[k] = next_f(0.0f, 1.0f);
            for (int k = 0; k < 2; ++k) p.texture_coordinates[k] = next_f(-0.5f, 1.5f);
            me.positions.push_back(p);
        }
        const uint32_t nt = nv;  // triangles
        for (uint32_t t = 0; t < 3 * nt; ++t) me.indices.push_back(next_u32() % nv);
        const uint32_t split = 3 * (nt / 2);
        rosy_asset::surface s0, s1;
        s0.start_index = 0;
        s0.count = split;
        s0.material = mi % 4;
        s1.start_index = split;
        s1.count = 3 * nt - split;
        s1.material = (mi + 3) % 4;
        for (int k = 0; k < 3; ++k) {
            s0.min_bounds[k] = s1.min_bounds[k] = -1.0f;
            s0.max_bounds[k] = s1.max_bounds[k] = 1.0f;
        }
        me.surfaces.push_back(s0);
        me.surfaces.push_back(s1);
        a.meshes.push_back(me);
    }
    // nodes: two scenes; the root scene holds a static hierarchy and a "mobs" subtree
    auto add_node = [&](const char* name, uint32_t mesh, std::vector<uint32_t> children) {
        rosy_asset::node n;
        for (int k = 0; k < 3; ++k) n.world_translate[k] = next_f(-2.0f, 2.0f);
        n.world_scale = next_f(0.5f, 1.5f);
        n.world_yaw = next_f(-3.0f, 3.0f);
        for (int k = 0; k < 16; ++k) n.transform[k] = (k % 5 == 0) ? next_f(0.8f, 1.2f) : 0.0f;
        n.transform[12] = next_f(-1.0f, 1.0f);
        n.transform[13] = next_f(-1.0f, 1.0f);
        n.transform[14] = next_f(-1.0f, 1.0f);
        n.mesh_id = mesh;
        n.child_nodes = children;
        const std::string s(name);
        n.name.assign(s.begin(), s.end());
        a.nodes.push_back(n);
    };
    add_node("unused_scene_node", 0, {});                 // 0: only in scene 0
    add_node("level", UINT32_MAX, {2, 3, 5});            // 1
    add_node("rock", 0, {});                             // 2
    add_node("tree", meshes > 1 ? 1 : 0, {4});           // 3
    add_node("branch", 0, {});                           // 4
    add_node("mobs", UINT32_MAX, {6, 7});                // 5
    add_node("mob_a", meshes > 1 ? 1 : 0, {});           // 6
    add_node("mob_b", 0, {});                            // 7
    rosy_asset::scene s0, s1;
    s0.nodes = {0};
    s1.nodes = {1};
    a.scenes.push_back(s0);
    a.scenes.push_back(s1);
    a.root_scene = 1;
    return a;
}

void print_asset(const rosy_asset::asset& a) {
    std::printf("{\"root_scene\":%u,\"coordinate_system\":", a.root_scene);
    print_floats(a.asset_coordinate_system.data(), 16);
    std::printf(",\"images\":[");
    for (size_t i = 0; i < a.images.size(); ++i) {
        std::printf("%s{\"type\":%u,\"name\":", i ? "," : "", a.images[i].image_type);
        print_chars(a.images[i].name);
        std::printf("}");
    }
    std::printf("],\"samplers\":[");
    for (size_t i = 0; i < a.samplers.size(); ++i) {
        const auto& s = a.samplers[i];
        std::printf("%s[%u,%u,%u,%u]", i ? "," : "", s.min_filter, s.mag_filter, s.wrap_s, s.wrap_t);
    }
    std::printf("],\"materials\":[");
    for (size_t i = 0; i < a.materials.size(); ++i) {
        const auto& m = a.materials[i];
        std::printf("%s{\"double_sided\":%u,\"base_color_factor\":", i ? "," : "", m.double_sided);
        print_floats(m.base_color_factor.data(), 4);
        std::printf(",\"metallic_factor\":%.9g,\"roughness_factor\":%.9g,\"alpha_mode\":%u,\"alpha_cutoff\":%.9g,",
                    (double)m.metallic_factor, (double)m.roughness_factor, m.alpha_mode, (double)m.alpha_cutoff);
        const uint32_t idx[8] = {m.color_image_index, m.color_sampler_index, m.normal_image_index,
                                 m.normal_sampler_index, m.metallic_image_index, m.metallic_sampler_index,
                                 m.mixmap_image_index, m.mixmap_sampler_index};
        std::printf("\"indices\":");
        print_u32s(idx, 8);
        std::printf("}");
    }
    std::printf("],\"scenes\":[");
    for (size_t i = 0; i < a.scenes.size(); ++i) {
        std::printf("%s", i ? "," : "");
        print_u32s(a.scenes[i].nodes.data(), a.scenes[i].nodes.size());
    }
    std::printf("],\"nodes\":[");
    for (size_t i = 0; i < a.nodes.size(); ++i) {
        const auto& n = a.nodes[i];
        std::printf("%s{\"world_translate\":", i ? "," : "");
        print_floats(n.world_translate.data(), 3);
        std::printf(",\"world_scale\":%.9g,\"world_yaw\":%.9g,\"transform\":", (double)n.world_scale,
                    (double)n.world_yaw);
        print_floats(n.transform.data(), 16);
        std::printf(",\"mesh_id\":%u,\"children\":", n.mesh_id);
        print_u32s(n.child_nodes.data(), n.child_nodes.size());
        std::printf(",\"name\":");
        print_chars(n.name);
        std::printf("}");
    }
    std::printf("],\"meshes\":[");
    for (size_t i = 0; i < a.meshes.size(); ++i) {
        const auto& me = a.meshes[i];
        std::printf("%s{\"positions\":", i ? "," : "");
        print_floats(reinterpret_cast<const float*>(me.positions.data()), me.positions.size() * 16);
        std::printf(",\"indices\":");
        print_u32s(me.indices.data(), me.indices.size());
        std::printf(",\"surfaces\":[");
        for (size_t k = 0; k < me.surfaces.size(); ++k) {
            const auto& s = me.surfaces[k];
            std::printf("%s{\"start_index\":%u,\"count\":%u,\"material\":%u}", k ? "," : "", s.start_index, s.count,
                        s.material);
        }
        std::printf("]}");
    }
    std::printf("]}\n");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s out.rsy seed meshes\n", argv[0]);
        return 2;
    }
    g_state = std::strtoull(argv[2], nullptr, 10) * 2654435761ull + 12345ull;
    auto log = std::make_shared<rosy_logger::log>();
    log->level = rosy_logger::log_level::disabled;
    rosy_asset::asset a = make_asset(argv[1], (uint32_t)std::strtoul(argv[3], nullptr, 10));
    if (a.write(log) != rosy::result::ok) {
        std::fprintf(stderr, "asset::write failed\n");
        return 1;
    }
    rosy_asset::asset b;
    b.asset_path = argv[1];
    if (b.read(log) != rosy::result::ok) {
        std::fprintf(stderr, "asset::read failed\n");
        return 1;
    }
    print_asset(b);
    return 0;
}
