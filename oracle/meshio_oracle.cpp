// meshio_oracle.cpp — TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's mesh
// decoders (native/src/engine/io/cuda_mesh_io.cu); the tests compare the engine's GPU
// decoders (rhizome_v24.15_gb300/csrc/k_io.cu) with it. Never linked into the product.
//
// * binary STL: CudaRasterizer::parse_binary_stl_gpu (cuda_mesh_io.cu:592-722) with the
//   record decode of gpu_decode_binary_stl_kernel (:524-590): 80-byte header, uint32
//   triangle count, 50-byte records (normal, 3 vertices, attribute); normals normalised
//   (geometric fallback, then +z); vertices welded on round(coordinate * 10000) keys in
//   first-occurrence order (:675-708); triangles whose welded corners repeat are dropped.
// * ASCII OBJ: CudaRasterizer::parse_obj_text_gpu (cuda_mesh_io.cu:962-1090) with
//   gpu_find_obj_lines_kernel (:859-888), gpu_parse_obj_vertices_kernel (:890-907),
//   gpu_parse_obj_faces_kernel (:909-960) and device_fast_atof / _atoi (:810-857): lines
//   starting "v " / "f " in file order (at most text_length / 10 + 1024 of each), three
//   numbers per vertex, up to four 1-based (or negative, relative) indices per face, quads
//   split (0,1,2) (0,2,3).
// * ASCII STL: CudaRasterizer::parse_ascii_stl_gpu (cuda_mesh_io.cu:1201-1325) with
//   gpu_find_ascii_stl_vertices_kernel (:1094-1118), the OBJ number parser and
//   gpu_weld_raw_vertices_kernel (:1146-1186): "vertex" tokens (at the text start or after
//   a space, tab, CR or LF, followed by a space or tab, ending before the last 7 bytes) in
//   file order, at most the reference's offset capacity, the count cut to whole facets;
//   three numbers after each token; corners welded on the reference's 64-bit hash of
//   round(coordinate * 10000) (dev_quantize_vec3_key, :1146-1156), every corner kept. The
//   reference numbers vertices in the order its threads win the table slots and keeps the
//   winner's coordinates; this restatement numbers them in order of first occurrence and
//   keeps the first corner's coordinates (the engine does the same).
// * iso-surface: CudaRasterizer::extract_iso_surface (cuda_marching_cubes.cu:829-951): border
//   seal to iso + h (:312-332), inside when value - iso <= 0 (:334-360), one vertex per
//   crossing grid edge at the clamped linear interpolation (:415-489), triangles from a
//   256 x 16 edge table passed in (the engine's generated table: the reference's own
//   table is hand-written and its atomic counters order the output by thread timing);
//   vertices numbered in voxel order (x, y, z edges of a voxel in turn), triangles in cube
//   order.
// Every expression is restated as written in the reference source, each operation rounded
// once (compile with -ffp-contract=off; oracle.py does), the same convention as the engine
// (-fmad=false). A build of the reference that fuses multiply-adds can differ from this by
// an ulp in parsed coordinates and normals.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

struct QKey {
    int32_t x, y, z;
    bool operator==(const QKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct QHash {
    size_t operator()(const QKey& k) const {
        return (size_t)((uint64_t)(uint32_t)k.x * 0x9E3779B97F4A7C15ull ^ (uint64_t)(uint32_t)k.y * 0xC2B2AE3D27D4EB4Full ^
                        (uint64_t)(uint32_t)k.z * 0x165667B19E3779F9ull);
    }
};

float rd_f32(const uint8_t* p) {
    float v;
    std::memcpy(&v, p, 4);
    return v;
}

int32_t quant(float v) { return (int32_t)std::round(v * 10000.0f); }

// device_fast_atof (cuda_mesh_io.cu:810-843)
float fast_atof(const char*& p) {
    while (*p == ' ' || *p == '\t') ++p;
    float sign = 1.0f;
    if (*p == '-') {
        sign = -1.0f;
        ++p;
    } else if (*p == '+') {
        ++p;
    }
    float val = 0.0f;
    while (*p >= '0' && *p <= '9') {
        val = val * 10.0f + (float)(*p - '0');
        ++p;
    }
    if (*p == '.') {
        ++p;
        float factor = 0.1f;
        while (*p >= '0' && *p <= '9') {
            val += (float)(*p - '0') * factor;
            factor *= 0.1f;
            ++p;
        }
    }
    if (*p == 'e' || *p == 'E') {
        ++p;
        float es = 1.0f;
        if (*p == '-') {
            es = -1.0f;
            ++p;
        } else if (*p == '+') {
            ++p;
        }
        int ev = 0;
        while (*p >= '0' && *p <= '9') {
            ev = ev * 10 + (*p - '0');
            ++p;
        }
        val *= std::pow(10.0f, es * (float)ev);
    }
    return sign * val;
}

// device_fast_atoi (cuda_mesh_io.cu:845-857)
int fast_atoi(const char*& p) {
    while (*p == ' ' || *p == '\t') ++p;
    int sign = 1;
    if (*p == '-') {
        sign = -1;
        ++p;
    } else if (*p == '+') {
        ++p;
    }
    int val = 0;
    while (*p >= '0' && *p <= '9') {
        val = val * 10 + (*p - '0');
        ++p;
    }
    return sign * val;
}

}  // namespace

extern "C" {

// Returns 0 on success, 1 on a malformed buffer (shorter than its header says).
int orc_parse_binary_stl(const uint8_t* bytes, size_t n, float* verts, uint32_t* idx, float* normals, int64_t* nv,
                         int64_t* ni) {
    *nv = 0;
    *ni = 0;
    if (n < 84) return 1;
    uint32_t T = 0;
    std::memcpy(&T, bytes + 80, 4);
    if (T == 0) return 0;
    if (n < 84 + (size_t)T * 50) return 1;
    std::unordered_map<QKey, uint32_t, QHash> map;
    map.reserve((size_t)T * 3);
    int64_t V = 0, I = 0;
    for (uint32_t t = 0; t < T; ++t) {
        const uint8_t* rec = bytes + 84 + (size_t)t * 50;
        float nx = rd_f32(rec), ny = rd_f32(rec + 4), nz = rd_f32(rec + 8);
        float v[3][3];
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) v[k][c] = rd_f32(rec + 12 + 12 * k + 4 * c);
        const float len = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (len > 1e-7f) {
            nx /= len;
            ny /= len;
            nz /= len;
        } else {
            const float e1x = v[1][0] - v[0][0], e1y = v[1][1] - v[0][1], e1z = v[1][2] - v[0][2];
            const float e2x = v[2][0] - v[0][0], e2y = v[2][1] - v[0][1], e2z = v[2][2] - v[0][2];
            nx = e1y * e2z - e1z * e2y;
            ny = e1z * e2x - e1x * e2z;
            nz = e1x * e2y - e1y * e2x;
            const float gl = std::sqrt(nx * nx + ny * ny + nz * nz);
            if (gl > 1e-7f) {
                nx /= gl;
                ny /= gl;
                nz /= gl;
            } else {
                nx = 0.0f;
                ny = 0.0f;
                nz = 1.0f;
            }
        }
        if (normals) {
            normals[3 * t] = nx;
            normals[3 * t + 1] = ny;
            normals[3 * t + 2] = nz;
        }
        uint32_t id[3];
        for (int k = 0; k < 3; ++k) {
            const QKey q{quant(v[k][0]), quant(v[k][1]), quant(v[k][2])};
            auto it = map.find(q);
            if (it != map.end()) {
                id[k] = it->second;
            } else {
                id[k] = (uint32_t)V;
                map.emplace(q, id[k]);
                for (int c = 0; c < 3; ++c) verts[3 * V + c] = v[k][c];
                ++V;
            }
        }
        if (id[0] != id[1] && id[1] != id[2] && id[2] != id[0]) {
            idx[I++] = id[0];
            idx[I++] = id[1];
            idx[I++] = id[2];
        }
    }
    *nv = V;
    *ni = I;
    return 0;
}

// Returns 0 on success, 1 when the text holds no vertex or face line or no triangle.
// verts / idx must hold (n / 10 + 1024) * 3 floats / (n / 10 + 1024) * 6 indices.
int orc_parse_obj(const char* text_in, size_t n, float* verts, uint32_t* idx, int64_t* nv, int64_t* ni) {
    *nv = 0;
    *ni = 0;
    if (n == 0 || !text_in) return 1;
    std::vector<char> text(text_in, text_in + n);
    text.push_back('\0');
    const size_t max_lines = n / 10 + 1024;
    std::vector<size_t> vo, fo;
    for (size_t i = 0; i + 1 < n; ++i) {
        const bool start = (i == 0) || text[i - 1] == '\n';
        if (!start) continue;
        if (text[i] == 'v' && text[i + 1] == ' ') {
            if (vo.size() < max_lines) vo.push_back(i + 2);
        } else if (text[i] == 'f' && text[i + 1] == ' ') {
            if (fo.size() < max_lines) fo.push_back(i + 2);
        }
    }
    if (vo.empty() || fo.empty()) return 1;
    const int64_t V = (int64_t)vo.size();
    for (int64_t k = 0; k < V; ++k) {
        const char* p = text.data() + vo[k];
        verts[3 * k] = fast_atof(p);
        verts[3 * k + 1] = fast_atof(p);
        verts[3 * k + 2] = fast_atof(p);
    }
    int64_t I = 0;
    for (size_t k = 0; k < fo.size(); ++k) {
        const char* p = text.data() + fo[k];
        int f[4];
        int c = 0;
        while (*p != '\n' && *p != '\r' && *p != '\0' && c < 4) {
            while (*p == ' ' || *p == '\t') ++p;
            if (*p == '\n' || *p == '\r' || *p == '\0') break;
            int vi = fast_atoi(p);
            while (*p != ' ' && *p != '\t' && *p != '\n' && *p != '\r' && *p != '\0') ++p;
            if (vi < 0) vi = (int)V + vi + 1;
            if (vi > 0) f[c++] = vi - 1;
        }
        if (c == 3) {
            idx[I++] = (uint32_t)f[0];
            idx[I++] = (uint32_t)f[1];
            idx[I++] = (uint32_t)f[2];
        } else if (c == 4) {
            idx[I++] = (uint32_t)f[0];
            idx[I++] = (uint32_t)f[1];
            idx[I++] = (uint32_t)f[2];
            idx[I++] = (uint32_t)f[0];
            idx[I++] = (uint32_t)f[2];
            idx[I++] = (uint32_t)f[3];
        }
    }
    if (I == 0) return 1;
    *nv = V;
    *ni = I;
    return 0;
}

// Counts (out pointers NULL) or extracts the iso-surface; returns 0.
int orc_extract_iso_surface(const float* g, const int32_t* dims, float h, const float* origin, float iso,
                            const int8_t* table, float* verts, uint32_t* idx, int64_t* nv, int64_t* ni) {
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    *nv = 0;
    *ni = 0;
    if (dx < 2 || dy < 2 || dz < 2) return 0;
    const float seal = iso + h;
    auto val = [&](int x, int y, int z) {
        float v = g[((size_t)z * dy + y) * dx + x];
        if ((x == 0 || x == dx - 1 || y == 0 || y == dy - 1 || z == 0 || z == dz - 1) && v < seal) v = seal;
        return v - iso;
    };
    const size_t N = (size_t)dx * dy * dz;
    std::vector<uint32_t> vbase(N);
    std::vector<uint8_t> mask(N);
    int64_t V = 0;
    for (int z = 0; z < dz; ++z)
        for (int y = 0; y < dy; ++y)
            for (int x = 0; x < dx; ++x) {
                const size_t i = ((size_t)z * dy + y) * dx + x;
                const float v0 = val(x, y, z);
                const bool s0 = v0 <= 0.0f;
                const float px = origin[0] + (float)x * h, py = origin[1] + (float)y * h, pz = origin[2] + (float)z * h;
                vbase[i] = (uint32_t)V;
                uint8_t m = 0;
                for (int a = 0; a < 3; ++a) {
                    const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
                    if (x1 >= dx || y1 >= dy || z1 >= dz) continue;
                    const float v1 = val(x1, y1, z1);
                    if (s0 == (v1 <= 0.0f)) continue;
                    m |= (uint8_t)(1 << a);
                    if (verts) {
                        const float den = v0 - v1;
                        const float t = (std::fabs(den) > 1e-7f) ? std::fmin(std::fmax(v0 / den, 0.001f), 0.999f) : 0.5f;
                        verts[3 * V] = (a == 0) ? px + t * h : px;
                        verts[3 * V + 1] = (a == 1) ? py + t * h : py;
                        verts[3 * V + 2] = (a == 2) ? pz + t * h : pz;
                    }
                    ++V;
                }
                mask[i] = m;
            }
    static const int own[12][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {1, 0, 1},
                                   {0, 1, 1}, {0, 0, 1}, {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
    static const int axis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
    static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    int64_t I = 0;
    for (int z = 0; z + 1 < dz; ++z)
        for (int y = 0; y + 1 < dy; ++y)
            for (int x = 0; x + 1 < dx; ++x) {
                int cs = 0;
                for (int c = 0; c < 8; ++c)
                    if (val(x + corner[c][0], y + corner[c][1], z + corner[c][2]) <= 0.0f) cs |= 1 << c;
                for (int k = 0; k < 15 && table[16 * cs + k] >= 0; ++k) {
                    const int e = table[16 * cs + k];
                    const size_t w = ((size_t)(z + own[e][2]) * dy + (y + own[e][1])) * dx + (x + own[e][0]);
                    const int a = axis[e];
                    const uint32_t rank = (a == 0) ? 0u : (a == 1) ? (mask[w] & 1u) : (uint32_t)((mask[w] & 1u) + ((mask[w] >> 1) & 1u));
                    if (idx) idx[I] = vbase[w] + rank;
                    ++I;
                }
            }
    *nv = V;
    *ni = I;
    return 0;
}

// Returns 0 on success, 1 when the text is shorter than 15 bytes or holds no whole facet.
// verts must hold 3 * cap floats and idx cap indices, cap = ascii_stl_capacity(n).
int64_t orc_ascii_stl_capacity(size_t n) {
    const size_t max_verts = n / 12 + 1024;
    size_t cap = 1024;
    while (cap < max_verts && cap < ((size_t)1 << 26)) cap <<= 1;
    return (int64_t)cap;
}

int orc_parse_ascii_stl(const char* text_in, size_t n, float* verts, uint32_t* idx, int64_t* nv, int64_t* ni) {
    *nv = 0;
    *ni = 0;
    if (!text_in || n < 15) return 1;
    std::vector<char> text(text_in, text_in + n);
    text.push_back('\0');
    const size_t cap = (size_t)orc_ascii_stl_capacity(n);
    std::vector<size_t> vo;
    for (size_t i = 0; i + 7 < n; ++i) {
        const bool start = (i == 0) || text[i - 1] == ' ' || text[i - 1] == '\t' || text[i - 1] == '\n' ||
                           text[i - 1] == '\r';
        if (!start) continue;
        if (std::memcmp(text.data() + i, "vertex", 6) == 0 && (text[i + 6] == ' ' || text[i + 6] == '\t')) {
            if (vo.size() < cap) vo.push_back(i + 6);
        }
    }
    const size_t m = vo.size() - vo.size() % 3;
    if (m == 0) return 1;
    std::unordered_map<uint64_t, uint32_t> ids;
    int64_t V = 0;
    for (size_t k = 0; k < m; ++k) {
        const char* p = text.data() + vo[k];
        const float x = fast_atof(p);
        const float y = fast_atof(p);
        const float z = fast_atof(p);
        // dev_quantize_vec3_key (cuda_mesh_io.cu:1146-1156)
        const uint64_t ux = (uint64_t)(uint32_t)quant(x), uy = (uint64_t)(uint32_t)quant(y),
                       uz = (uint64_t)(uint32_t)quant(z);
        uint64_t key = (ux * 73856093ull) ^ (uy * 19349663ull) ^ (uz * 83492791ull) ^ ((ux & 0xFFFFFull) << 42) ^
                       ((uy & 0xFFFFFull) << 21) ^ (uz & 0x1FFFFFull);
        if (key == 0) key = 1;
        auto it = ids.find(key);
        if (it == ids.end()) {
            it = ids.emplace(key, (uint32_t)V).first;
            verts[3 * V] = x;
            verts[3 * V + 1] = y;
            verts[3 * V + 2] = z;
            ++V;
        }
        idx[k] = it->second;
    }
    *nv = V;
    *ni = (int64_t)m;
    return 0;
}

}  // extern "C"

// ---- orientation pre-pass ------------------------------------------------------------
// CudaRasterizer::orient_mesh_gpu (native/src/engine/mesh/cuda_mesh_topology.cu:707-842,
// kernels :303-455): an edge shared by exactly two triangles links them, "same direction"
// when both traverse it the same way (inconsistent winding); each connected component is
// oriented like its smallest triangle (flip parity along any path), a component whose
// links contradict themselves is non-orientable; flips are applied when any link was
// inconsistent; the mesh is inverted when its signed volume sum(v0 . (v1 x v2)) / 6 is
// below -1e-5. Restated with a breadth-first search per component and an FP64 volume.
#include <algorithm>
#include <map>
#include <queue>

extern "C" int orc_orient_mesh(const float* verts, int64_t nv, uint32_t* idx, int64_t ni, int32_t* orientable,
                               int32_t* inconsistent, int32_t* inverted, double* volume) {
    (void)nv;
    const int64_t T = ni / 3;
    *orientable = 1;
    *inconsistent = 0;
    *inverted = 0;
    *volume = 0.0;
    if (T <= 0) return 0;
    struct Use {
        int64_t tri;
        bool fwd;
    };
    std::map<std::pair<uint32_t, uint32_t>, std::vector<Use>> edges;
    for (int64_t t = 0; t < T; ++t)
        for (int e = 0; e < 3; ++e) {
            const uint32_t u = idx[3 * t + e], v = idx[3 * t + (e + 1) % 3];
            if (u == v) continue;
            edges[{std::min(u, v), std::max(u, v)}].push_back({t, u < v});
        }
    std::vector<std::vector<std::pair<int64_t, int>>> adj(T);
    for (auto& kv : edges) {
        if (kv.second.size() != 2) continue;
        const Use a = kv.second[0], b = kv.second[1];
        if (a.tri == b.tri) continue;
        const int same = (a.fwd == b.fwd) ? 1 : 0;
        if (same) *inconsistent = 1;
        adj[a.tri].push_back({b.tri, same});
        adj[b.tri].push_back({a.tri, same});
    }
    std::vector<int> flip(T, -1);
    for (int64_t r = 0; r < T; ++r) {
        if (flip[r] >= 0) continue;
        flip[r] = 0;
        std::queue<int64_t> q;
        q.push(r);
        while (!q.empty()) {
            const int64_t t = q.front();
            q.pop();
            for (auto [nb, same] : adj[t]) {
                const int req = flip[t] ^ same;
                if (flip[nb] < 0) {
                    flip[nb] = req;
                    q.push(nb);
                } else if (flip[nb] != req) {
                    *orientable = 0;
                }
            }
        }
    }
    if (*inconsistent)
        for (int64_t t = 0; t < T; ++t)
            if (flip[t]) std::swap(idx[3 * t + 1], idx[3 * t + 2]);
    double v6 = 0.0;
    for (int64_t t = 0; t < T; ++t) {
        const float* a = verts + 3 * (size_t)idx[3 * t];
        const float* b = verts + 3 * (size_t)idx[3 * t + 1];
        const float* c = verts + 3 * (size_t)idx[3 * t + 2];
        const double cx = (double)b[1] * c[2] - (double)b[2] * c[1];
        const double cy = (double)b[2] * c[0] - (double)b[0] * c[2];
        const double cz = (double)b[0] * c[1] - (double)b[1] * c[0];
        v6 += (double)a[0] * cx + (double)a[1] * cy + (double)a[2] * cz;
    }
    double vol = v6 / 6.0;
    if (vol < -1e-5) {
        for (int64_t t = 0; t < T; ++t) std::swap(idx[3 * t + 1], idx[3 * t + 2]);
        vol = -vol;
        *inverted = 1;
    }
    *volume = vol;
    return 0;
}
