// cuda_rasterizer_gbsdf.cpp — the reference application's two mesh-to-SDF statics of
// CudaRasterizer (native/src/engine/sdf/cuda_rasterizer.hpp:21-35) implemented on the
// engine's C ABI (include/gbsdf.h). A maintainer compiles this file into the reference's
// core library and removes the two bodies from cuda_rasterizer.cu (:1163-1265 and
// :1340-1435); signatures, grid layout and error behaviour stay the same:
//
//   compute_mesh_sdf: an empty lattice returns false with out_time_ms = 0 and the vector
//     untouched; otherwise the vector is resized to the lattice's voxel count, new entries
//     1e6, before the attempt (cuda_rasterizer.cu:1180), so a caller that reads its size
//     after a false sees the reference's; no triangles return false after that resize
//     (:1183, :1263). The reference dispatch (legacy exact kernel below 32M voxels, fast
//     path at or above, legacy again when the fast path declines) is the library's
//     GBSDF_PATH_AUTO. A failure leaves the entries untouched and is logged.
//   build_from_mesh: nullptr for an empty mesh or a failed build; the lattice is the
//     reference's (bounding box padded by 10 voxels, floor / ceil, :1354-1372); the
//     triangles are built on the device in index order (degenerate and out-of-range faces
//     dropped); every successful build gets a fresh version number (:1430-1432).
#include <chrono>
#include <cstdint>
#include <memory>
#include <vector>

#include "core/unified_logger.hpp"
#include "engine/sdf/cuda_rasterizer.hpp"
#include "gbsdf.h"

namespace rhizome {

static_assert(sizeof(CudaTriangle) == sizeof(gbsdf_tri), "CudaTriangle and gbsdf_tri share the 48-byte record");

bool CudaRasterizer::compute_mesh_sdf(const std::vector<CudaTriangle>& triangles, float voxel_size,
                                      glm::ivec3 min_coord, glm::ivec3 max_coord, std::vector<float>& out_distances,
                                      float& out_time_ms) {
    const auto t0 = std::chrono::high_resolution_clock::now();
    const int dim_x = max_coord.x - min_coord.x + 1;
    const int dim_y = max_coord.y - min_coord.y + 1;
    const int dim_z = max_coord.z - min_coord.z + 1;
    if (dim_x <= 0 || dim_y <= 0 || dim_z <= 0) {
        out_time_ms = 0.0f;
        return false;
    }
    const size_t total = (size_t)dim_x * dim_y * dim_z;
    out_distances.resize(total, 1e6f);
    if (triangles.empty()) {
        RhizomeLog("CUDA", "compute_mesh_sdf: no triangles");
        return false;
    }
    const int32_t mn[3] = {min_coord.x, min_coord.y, min_coord.z};
    const int32_t mx[3] = {max_coord.x, max_coord.y, max_coord.z};
    gbsdf_options opt;
    gbsdf_default_options(&opt);  // reference mode, the reference's 32M-voxel dispatch
    gbsdf_stats st;
    char err[256];
    const int rc = gbsdf_compute_mesh_sdf(reinterpret_cast<const gbsdf_tri*>(triangles.data()),
                                          (int64_t)triangles.size(), voxel_size, mn, mx, out_distances.data(),
                                          /*out_on_device=*/0, &opt, &st, err, sizeof(err));
    out_time_ms = std::chrono::duration<float, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
    if (rc != GBSDF_OK) {
        RhizomeLog("CUDA", err);
        return false;
    }
    return true;
}

std::shared_ptr<CudaVolumeGrid> CudaRasterizer::build_from_mesh(const TriangleMesh& mesh, float voxel_size,
                                                                float& out_time_ms) {
    if (mesh.vertex_count() == 0 || mesh.triangle_count() == 0) return nullptr;
    const auto t0 = std::chrono::high_resolution_clock::now();
    auto volume = std::make_shared<CudaVolumeGrid>();
    volume->voxel_size = voxel_size;
    int32_t mn[3], mx[3];
    char err[256];
    if (gbsdf_mesh_lattice(mesh.vertices.data(), (int64_t)mesh.vertex_count(), voxel_size, mn, mx, err,
                           sizeof(err)) != GBSDF_OK) {
        RhizomeLog("CUDA", err);
        return nullptr;
    }
    volume->min_coord = glm::ivec3(mn[0], mn[1], mn[2]);
    volume->max_coord = glm::ivec3(mx[0], mx[1], mx[2]);
    volume->dims = volume->max_coord - volume->min_coord + glm::ivec3(1);
    volume->data.resize((size_t)volume->dims.x * volume->dims.y * volume->dims.z, 1e6f);
    gbsdf_stats st;
    const int rc = gbsdf_build_from_mesh(mesh.vertices.data(), (int64_t)mesh.vertex_count(), mesh.indices.data(),
                                         (int64_t)mesh.indices.size(), voxel_size, mn, mx, volume->data.data(),
                                         /*out_on_device=*/0, nullptr, &st, err, sizeof(err));
    out_time_ms = std::chrono::duration<float, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
    if (rc != GBSDF_OK) {
        RhizomeLog("CUDA", err);
        return nullptr;
    }
    static uint64_t s_next_vol_version = 2;
    volume->version = ++s_next_vol_version;
    return volume;
}

}  // namespace rhizome
