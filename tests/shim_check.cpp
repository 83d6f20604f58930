// tests/shim_check.cpp — drives the CudaRasterizer shim (rhizome_v24.15_gb300/shim/) the
// way the reference application calls it, for tests/test_shim.py. Reads a triangle soup
// and a mesh from binary files, writes the outputs and what the shim reported.
//   shim_check <tris.bin> <T> <h> <mnx mny mnz> <mxx mxy mxz> <verts.bin> <V> <idx.bin> <I> <out_prefix>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "engine/sdf/cuda_rasterizer.hpp"

namespace rhizome {
void RhizomeLog(const char* category, const char* message) { std::fprintf(stderr, "[%s] %s\n", category, message); }
}  // namespace rhizome

template <class T>
static std::vector<T> load(const char* path, size_t n) {
    std::vector<T> v(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) std::exit(2);
    std::fclose(f);
    return v;
}

static void save(const std::string& path, const void* p, size_t bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(p, 1, bytes, f) != bytes) std::exit(3);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc != 15) return 1;
    using namespace rhizome;
    const size_t T = std::strtoull(argv[2], nullptr, 10);
    const float h = std::strtof(argv[3], nullptr);
    const glm::ivec3 mn(std::atoi(argv[4]), std::atoi(argv[5]), std::atoi(argv[6]));
    const glm::ivec3 mx(std::atoi(argv[7]), std::atoi(argv[8]), std::atoi(argv[9]));
    std::vector<CudaTriangle> tris = load<CudaTriangle>(argv[1], T);
    const std::string out = argv[14];
    FILE* rep = std::fopen((out + "report.txt").c_str(), "w");
    // 1. compute_mesh_sdf on the triangle soup
    std::vector<float> d;
    float ms = 0.0f;
    bool ok = CudaRasterizer::compute_mesh_sdf(tris, h, mn, mx, d, ms);
    std::fprintf(rep, "compute %d %zu\n", ok ? 1 : 0, d.size());
    save(out + "compute.bin", d.data(), d.size() * 4);
    // 2. no triangles: false after the resize to the lattice, the new entries 1e6
    std::vector<float> e(3, -5.0f);
    std::vector<CudaTriangle> none;
    ok = CudaRasterizer::compute_mesh_sdf(none, h, mn, mx, e, ms);
    size_t n1e6 = 0;
    for (size_t i = 3; i < e.size(); ++i) n1e6 += e[i] == 1e6f;
    std::fprintf(rep, "empty %d %zu %zu %d\n", ok ? 1 : 0, e.size(), n1e6, e[0] == -5.0f ? 1 : 0);
    // 3. an empty lattice: false, vector untouched, time 0
    std::vector<float> g(7, 2.0f);
    ms = 9.0f;
    ok = CudaRasterizer::compute_mesh_sdf(tris, h, mx, mn, g, ms);
    std::fprintf(rep, "inverted %d %zu %g\n", ok ? 1 : 0, g.size(), ms);
    // 4. build_from_mesh on the indexed mesh
    TriangleMesh mesh;
    mesh.vertices = load<float>(argv[10], 3 * std::strtoull(argv[11], nullptr, 10));
    mesh.indices = load<uint32_t>(argv[12], std::strtoull(argv[13], nullptr, 10));
    auto vol = CudaRasterizer::build_from_mesh(mesh, h, ms);
    if (vol) {
        std::fprintf(rep, "build 1 %d %d %d %d %d %d %llu\n", vol->min_coord.x, vol->min_coord.y, vol->min_coord.z,
                     vol->max_coord.x, vol->max_coord.y, vol->max_coord.z, (unsigned long long)vol->version);
        save(out + "build.bin", vol->data.data(), vol->data.size() * 4);
    } else {
        std::fprintf(rep, "build 0\n");
    }
    TriangleMesh empty;
    std::fprintf(rep, "build_empty %d\n", CudaRasterizer::build_from_mesh(empty, h, ms) ? 1 : 0);
    std::fclose(rep);
    return 0;
}
