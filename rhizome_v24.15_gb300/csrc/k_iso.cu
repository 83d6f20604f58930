// k_iso.cu — iso-surface extraction (marching cubes) straight from a device-resident grid.
//
// Reference: CudaRasterizer::extract_iso_surface (cuda_marching_cubes.cu:829-951) with
// gpu_mc_seal_border_kernel (:312-332), dev_mc_cube_index (:334-360), the count pass
// (:362-413), gpu_mc_emit_vertices_kernel (:415-489) and gpu_mc_emit_triangles_kernel
// (:491-555). The reference takes the grid as a host vector and uploads it (2.6 GB for
// the 860 x 860 x 880 grid); here the grid may be the engine's device output, read in
// place. Its rules are kept:
//   * boundary voxels read below iso + h read as iso + h (the seal; the caller's grid is
//     not written);
//   * a corner is inside when value - iso <= 0; one vertex per grid edge whose ends
//     differ, at p0 + t h along the edge, t = (v0 / (v0 - v1)) clamped to [0.001, 0.999]
//     (0.5 when |v0 - v1| <= 1e-7), each operation rounded once (-fmad=false);
//   * triangles connect the vertices on a cube's edges, outward (towards values above iso).
// What differs:
//   * order: the reference numbers vertices and triangles with atomic counters (the order
//     changes from run to run); here vertices follow the voxel order (x, y, z edges of a
//     voxel in turn) and triangles the cube order, by scans;
//   * the triangle table: the reference's is a hand-written table; this one is generated
//     (mc_table_init) from one rule: on each cube face the crossing edges pair up so that
//     inside corners are cut off separately -- on a face with two inside corners on a
//     diagonal they stay apart -- and the resulting loops are triangulated without chords
//     across a cube face. Both cubes that share a face see its four corners alike, so they
//     pair its edges alike and the surface is closed and consistently oriented for any grid
//     (the reference's table can pair an ambiguous face differently in the two cubes). On
//     ambiguous cubes the vertices may be connected differently from the reference's table.
//
// Passes:
//   1. count: crossing mask (3 bits) per voxel, triangles per cube; per-row totals;
//   2. exclusive scans of the row totals;
//   3. vertices: row offsets plus within-row prefixes give each voxel's first vertex number
//      (stored, 4 B per voxel); the vertices are written;
//   4. triangles: the same for each cube's first triangle; a cube's edge vertex is its
//      owner voxel's first vertex plus the edge's rank in the owner's mask.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gbsdf.h"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

// Cube corners (x, y, z bits as in the reference's corner order), edges (corner pairs)
// and faces (corners in cyclic order).
constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

__device__ int8_t c_tri[256][16];  // read with divergent per-lane cases: global memory, L1-cached
__device__ int8_t c_ntri[256];

int8_t g_tri[256][16];
std::once_flag g_tri_once;

int edge_of(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
    return -1;
}

// The triangle table from the face rule above. Per case: on each face, pair the crossing
// edges (cutting inside corners off separately) into segments directed so that the inside
// corners lie on their left seen from outside the cube; follow the segments into closed
// loops (every crossing edge lies on two faces) and walk each loop backwards, which turns
// its triangles outward (from the inside corners to the outside ones). The two cubes that
// share a face direct its segments oppositely, so the surface is closed and consistently
// oriented. A loop of more than 3 edges is split by the first triangulation (in a fixed
// enumeration) none of whose diagonals joins two edges of one cube face: such a chord would
// also be drawn by the neighbouring cube and leave an edge with four triangles. Every loop
// of the 256 cases has one; at most 5 triangles per case.
bool on_face(int e, const int* f) {
    bool a = false, b = false;
    for (int k = 0; k < 4; ++k) {
        a |= f[k] == kEdge[e][0];
        b |= f[k] == kEdge[e][1];
    }
    return a && b;
}

bool share_face(int e0, int e1) {
    for (const auto& f : kFace)
        if (on_face(e0, f) && on_face(e1, f)) return true;
    return false;
}

// all triangulations of the polygon p[0..n-1]: triangle (p0, pk, p(n-1)) plus the two sides
void triangulations(const std::vector<int>& p, std::vector<std::vector<std::array<int, 3>>>& out) {
    const int n = (int)p.size();
    out.clear();
    if (n < 3) {
        out.push_back({});
        return;
    }
    for (int k = 1; k + 1 < n; ++k) {
        std::vector<std::vector<std::array<int, 3>>> L, R;
        triangulations(std::vector<int>(p.begin(), p.begin() + k + 1), L);
        triangulations(std::vector<int>(p.begin() + k, p.end()), R);
        for (const auto& l : L)
            for (const auto& r : R) {
                std::vector<std::array<int, 3>> t = l;
                t.insert(t.end(), r.begin(), r.end());
                t.push_back({p[0], p[k], p[n - 1]});
                out.push_back(t);
            }
    }
}

void mc_table_init() {
    std::memset(g_tri, -1, sizeof(g_tri));
    static const int kNormal[6][3] = {{0, 0, -1}, {0, 0, 1}, {0, -1, 0}, {0, 1, 0}, {-1, 0, 0}, {1, 0, 0}};
    auto mid = [](int e, int c) { return 0.5 * (kCorner[kEdge[e][0]][c] + kCorner[kEdge[e][1]][c]); };
    for (int cs = 0; cs < 256; ++cs) {
        int in[8];
        for (int i = 0; i < 8; ++i) in[i] = (cs >> i) & 1;
        int nxt[12];
        for (int e = 0; e < 12; ++e) nxt[e] = -1;
        auto segment = [&](int a, int b, const double* c, const int* fn) {
            double pq[3], pc[3];
            for (int k = 0; k < 3; ++k) {
                pq[k] = mid(b, k) - mid(a, k);
                pc[k] = c[k] - mid(a, k);
            }
            const double t = fn[0] * (pq[1] * pc[2] - pq[2] * pc[1]) + fn[1] * (pq[2] * pc[0] - pq[0] * pc[2]) +
                             fn[2] * (pq[0] * pc[1] - pq[1] * pc[0]);
            if (t < 0) std::swap(a, b);
            nxt[a] = b;
        };
        for (int fi = 0; fi < 6; ++fi) {
            const int* f = kFace[fi];
            int cross[4], nc = 0;
            for (int k = 0; k < 4; ++k)
                if (in[f[k]] != in[f[(k + 1) % 4]]) cross[nc++] = k;
            if (nc == 2) {
                double c[3] = {0, 0, 0};
                int ni = 0;
                for (int k = 0; k < 4; ++k)
                    if (in[f[k]]) {
                        for (int j = 0; j < 3; ++j) c[j] += kCorner[f[k]][j];
                        ++ni;
                    }
                for (int j = 0; j < 3; ++j) c[j] /= ni;
                segment(edge_of(f[cross[0]], f[(cross[0] + 1) % 4]), edge_of(f[cross[1]], f[(cross[1] + 1) % 4]), c,
                        kNormal[fi]);
            } else if (nc == 4) {  // two inside corners on a diagonal: cut each off
                for (int k = 0; k < 4; ++k)
                    if (in[f[k]]) {
                        const double c[3] = {(double)kCorner[f[k]][0], (double)kCorner[f[k]][1],
                                             (double)kCorner[f[k]][2]};
                        segment(edge_of(f[(k + 3) % 4], f[k]), edge_of(f[k], f[(k + 1) % 4]), c, kNormal[fi]);
                    }
            }
        }
        bool seen[12] = {false};
        int nt = 0;
        for (int s = 0; s < 12; ++s) {
            if (nxt[s] < 0 || seen[s]) continue;
            std::vector<int> loop;
            for (int cur = s; !seen[cur]; cur = nxt[cur]) {
                loop.push_back(cur);
                seen[cur] = true;
            }
            std::reverse(loop.begin() + 1, loop.end());  // walk backwards: outward triangles
            const int n = (int)loop.size();
            std::vector<std::vector<std::array<int, 3>>> all;
            triangulations(loop, all);
            for (const auto& tri : all) {
                bool chord = false;
                for (const auto& t : tri)
                    for (int k = 0; k < 3; ++k) {
                        const int a = t[k], b = t[(k + 1) % 3];
                        int ia = 0, ib = 0;
                        for (int i = 0; i < n; ++i) {
                            if (loop[i] == a) ia = i;
                            if (loop[i] == b) ib = i;
                        }
                        const int d = ia > ib ? ia - ib : ib - ia;
                        if (d != 1 && d != n - 1 && share_face(a, b)) chord = true;
                    }
                if (chord) continue;
                for (const auto& t : tri) {
                    if (nt == 5) break;
                    for (int k = 0; k < 3; ++k) g_tri[cs][3 * nt + k] = (int8_t)t[k];
                    ++nt;
                }
                break;
            }
        }
    }
}

// Work layout: rows are the x lines (y, z), numbered y + z dy; the count pass totals each
// row, scans over the rows give every row its first vertex and first triangle, and the emit
// passes number within a row in x order -- so vertices and triangles come in linear voxel
// order. A CTA takes kGR = 4 consecutive rows of one z plane and walks them in chunks of 128
// x; a thread takes the 4 voxels at its x, loading their cubes' 20 corner values
// ((y .. y+4) x (z, z+1) x (x, x+1)) at once. The within-row prefixes of the 4 rows come
// from one CTA scan of a 64-bit word holding four 16-bit counts (a chunk holds at most
// 128 x 5 triangles per row).
constexpr int kIsoThreads = 128;
constexpr int kGR = 4;

struct IsoGeom {
    int dx, dy, dz, gpz;  // gpz: row groups per z plane
    float iso, seal;
};

// value relative to iso, with the reference's border seal
__device__ __forceinline__ float iso_val(const float* __restrict__ g, int x, int y, int z, const IsoGeom& G) {
    float v = __ldg(&g[((size_t)z * G.dy + y) * G.dx + x]);
    if ((x == 0 || x == G.dx - 1 || y == 0 || y == G.dy - 1 || z == 0 || z == G.dz - 1) && v < G.seal) v = G.seal;
    return v - G.iso;
}

struct Quad {
    int x, y0, z, nr;   // voxels (x, y0 + r, z), r < nr
    float v[kGR + 1][2][2];  // value at (x + i, y0 + r, z + k): v[r][k][i]
};

__device__ __forceinline__ void group_of(const IsoGeom& G, int& y0, int& z, int& nr) {
    z = blockIdx.x / G.gpz;
    y0 = (blockIdx.x - z * G.gpz) * kGR;
    nr = min(kGR, G.dy - y0);
}

__device__ __forceinline__ void load_quad(const float* __restrict__ g, const IsoGeom& G, Quad& q) {
    const int xs = min(q.x, G.dx - 1), x1 = min(q.x + 1, G.dx - 1), z1 = min(q.z + 1, G.dz - 1);
#pragma unroll
    for (int r = 0; r <= kGR; ++r) {
        const int y = min(q.y0 + r, G.dy - 1);
        q.v[r][0][0] = iso_val(g, xs, y, q.z, G);
        q.v[r][0][1] = iso_val(g, x1, y, q.z, G);
        q.v[r][1][0] = iso_val(g, xs, y, z1, G);
        q.v[r][1][1] = iso_val(g, x1, y, z1, G);
    }
}

__device__ __forceinline__ bool quad_in(const IsoGeom& G, const Quad& q, int r) { return q.x < G.dx && r < q.nr; }

__device__ __forceinline__ unsigned quad_mask(const IsoGeom& G, const Quad& q, int r) {
    if (!quad_in(G, q, r)) return 0u;
    const bool s0 = q.v[r][0][0] <= 0.0f;
    unsigned m = 0;
    if (q.x + 1 < G.dx && s0 != (q.v[r][0][1] <= 0.0f)) m |= 1;
    if (q.y0 + r + 1 < G.dy && s0 != (q.v[r + 1][0][0] <= 0.0f)) m |= 2;
    if (q.z + 1 < G.dz && s0 != (q.v[r][1][0] <= 0.0f)) m |= 4;
    return m;
}

// cube case of the cube at voxel r (reference corner order), -1 when there is no cube
__device__ __forceinline__ int quad_case(const IsoGeom& G, const Quad& q, int r) {
    if (!quad_in(G, q, r) || q.x + 1 >= G.dx || q.y0 + r + 1 >= G.dy || q.z + 1 >= G.dz) return -1;
    const float c[8] = {q.v[r][0][0], q.v[r][0][1], q.v[r + 1][0][1], q.v[r + 1][0][0],
                        q.v[r][1][0], q.v[r][1][1], q.v[r + 1][1][1], q.v[r + 1][1][0]};
    int cs = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (c[i] <= 0.0f) cs |= 1 << i;
    return cs;
}

__device__ __forceinline__ int tri_count(int cs) { return cs < 0 ? 0 : __ldg(&c_ntri[cs]); }

// exclusive prefix over the CTA in thread order of a word of four 16-bit counts; the
// CTA total in *tot
__device__ __forceinline__ unsigned long long cta_exclusive4(unsigned long long val, unsigned long long* tot) {
    __shared__ unsigned long long warp_sum[kIsoThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long inc = val;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sum[w] = inc;
    __syncthreads();
    unsigned long long before = 0, all = 0;
#pragma unroll
    for (int i = 0; i < kIsoThreads / 32; ++i) {
        if (i < w) before += warp_sum[i];
        all += warp_sum[i];
    }
    __syncthreads();  // warp_sum is reused by the next chunk
    *tot = all;
    return before + inc - val;
}

__device__ __forceinline__ unsigned field(unsigned long long w, int r) { return (unsigned)(w >> (16 * r)) & 0xffffu; }

// 1. masks and per-row totals
__global__ void __launch_bounds__(kIsoThreads) iso_count_kernel(const float* __restrict__ g, IsoGeom G,
                                                                uint8_t* __restrict__ mask,
                                                                unsigned* __restrict__ row_v,
                                                                unsigned* __restrict__ row_t) {
    Quad q;
    group_of(G, q.y0, q.z, q.nr);
    unsigned tv[kGR] = {0, 0, 0, 0}, tt[kGR] = {0, 0, 0, 0};
    for (int x0 = 0; x0 < G.dx; x0 += kIsoThreads) {
        q.x = x0 + threadIdx.x;
        load_quad(g, G, q);
#pragma unroll
        for (int r = 0; r < kGR; ++r) {
            const unsigned m = quad_mask(G, q, r);
            if (quad_in(G, q, r)) mask[((size_t)q.z * G.dy + q.y0 + r) * G.dx + q.x] = (uint8_t)m;
            tv[r] += __popc(m);
            tt[r] += tri_count(quad_case(G, q, r));
        }
    }
    __shared__ unsigned red[2 * kGR][kIsoThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < kGR; ++r) {
        unsigned a = tv[r], b = tt[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (lane == 0) {
            red[r][w] = a;
            red[kGR + r][w] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < q.nr) {
        unsigned a = 0, b = 0;
        for (int i = 0; i < kIsoThreads / 32; ++i) {
            a += red[threadIdx.x][i];
            b += red[kGR + threadIdx.x][i];
        }
        const size_t row = (size_t)q.z * G.dy + q.y0 + threadIdx.x;
        row_v[row] = a;
        row_t[row] = b;
    }
}

// 3. vertex numbers and positions
__global__ void __launch_bounds__(kIsoThreads) iso_vertex_kernel(const float* __restrict__ g, IsoGeom G, float h,
                                                                 float ox, float oy, float oz,
                                                                 const unsigned long long* __restrict__ row_vpos,
                                                                 uint32_t* __restrict__ vbase,
                                                                 float* __restrict__ out_v) {
    Quad q;
    group_of(G, q.y0, q.z, q.nr);
    unsigned long long carry[kGR];
#pragma unroll
    for (int r = 0; r < kGR; ++r)
        carry[r] = (r < q.nr) ? row_vpos[(size_t)q.z * G.dy + q.y0 + r] : 0ull;
    const float pz = oz + (float)q.z * h;
    for (int x0 = 0; x0 < G.dx; x0 += kIsoThreads) {
        q.x = x0 + threadIdx.x;
        load_quad(g, G, q);
        unsigned m[kGR];
        unsigned long long word = 0;
#pragma unroll
        for (int r = 0; r < kGR; ++r) {
            m[r] = quad_mask(G, q, r);
            word |= (unsigned long long)__popc(m[r]) << (16 * r);
        }
        unsigned long long tot;
        const unsigned long long pre = cta_exclusive4(word, &tot);
        const float px = ox + (float)q.x * h;
#pragma unroll
        for (int r = 0; r < kGR; ++r) {
            if (quad_in(G, q, r)) {
                const unsigned long long base = carry[r] + field(pre, r);
                vbase[((size_t)q.z * G.dy + q.y0 + r) * G.dx + q.x] = (uint32_t)base;
                const float v0 = q.v[r][0][0];
                const float py = oy + (float)(q.y0 + r) * h;
                unsigned long long n = base;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if (!((m[r] >> a) & 1)) continue;
                    const float v1 = (a == 0) ? q.v[r][0][1] : (a == 1) ? q.v[r + 1][0][0] : q.v[r][1][0];
                    const float den = v0 - v1;
                    const float t = (fabsf(den) > 1e-7f) ? fminf(fmaxf(v0 / den, 0.001f), 0.999f) : 0.5f;
                    float* o = out_v + 3ull * n;
                    o[0] = (a == 0) ? px + t * h : px;
                    o[1] = (a == 1) ? py + t * h : py;
                    o[2] = (a == 2) ? pz + t * h : pz;
                    ++n;
                }
            }
            carry[r] += field(tot, r);
        }
    }
}

// 4. triangles: edge e of the cube at (x, y, z) belongs to voxel (x, y, z) + c_owner[e]
// along axis c_axis[e]
__constant__ int c_owner[12][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {1, 0, 1},
                                   {0, 1, 1}, {0, 0, 1}, {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
__constant__ int c_axis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};

__global__ void __launch_bounds__(kIsoThreads) iso_triangle_kernel(const float* __restrict__ g, IsoGeom G,
                                                                   const uint8_t* __restrict__ mask,
                                                                   const uint32_t* __restrict__ vbase,
                                                                   const unsigned long long* __restrict__ row_tpos,
                                                                   uint32_t* __restrict__ out_i) {
    Quad q;
    group_of(G, q.y0, q.z, q.nr);
    unsigned long long carry[kGR];
#pragma unroll
    for (int r = 0; r < kGR; ++r)
        carry[r] = (r < q.nr) ? row_tpos[(size_t)q.z * G.dy + q.y0 + r] : 0ull;
    const long long sy = G.dx, sz = (long long)G.dx * G.dy;
    for (int x0 = 0; x0 < G.dx; x0 += kIsoThreads) {
        q.x = x0 + threadIdx.x;
        load_quad(g, G, q);
        int cs[kGR];
        unsigned long long word = 0;
#pragma unroll
        for (int r = 0; r < kGR; ++r) {
            cs[r] = quad_case(G, q, r);
            word |= (unsigned long long)tri_count(cs[r]) << (16 * r);
        }
        unsigned long long tot;
        const unsigned long long pre = cta_exclusive4(word, &tot);
#pragma unroll
        for (int r = 0; r < kGR; ++r) {
            const int nt = (int)field(word, r);
            if (nt) {
                uint32_t* o = out_i + 3ull * (carry[r] + field(pre, r));
                const long long v = ((long long)q.z * G.dy + q.y0 + r) * G.dx + q.x;
                for (int j = 0; j < 3 * nt; ++j) {
                    const int e = __ldg(&c_tri[cs[r]][j]);
                    const long long w = v + c_owner[e][0] + c_owner[e][1] * sy + c_owner[e][2] * sz;
                    const unsigned mw = mask[w];
                    const int a = c_axis[e];
                    const unsigned rank = (a == 0) ? 0u : (a == 1) ? (mw & 1u) : (unsigned)__popc(mw & 3u);
                    o[j] = vbase[w] + rank;
                }
            }
            carry[r] += field(tot, r);
        }
    }
}

// ---- other consumers of the SDF: interior volume, default seed -----------------------
// CudaRasterizer::compute_sdf_interior_volume_gpu (cuda_viewport_gl.cu:702-741, kernel
// :84-112) and find_default_seed_gpu (cuda_viewport_packers.cu:304-384, kernel :235-276,
// min reduce cuda_rasterizer.cu:1632-1665): both read the grid in place here. Counts and
// minima are integer atomics, so the results do not depend on the launch.
__device__ __forceinline__ unsigned ordered_u32(float f) {  // order-preserving float key
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void sdf_inside_min_kernel(const float* __restrict__ g, long long n,
                                      unsigned long long* __restrict__ inside, unsigned* __restrict__ min_key) {
    unsigned long long c = 0;
    float mn = 1e30f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = __ldg(&g[i]);
        c += (v <= 0.0f);
        if (v < mn) mn = v;
    }
    unsigned k = ordered_u32(mn);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_down_sync(0xffffffffu, c, o);
        k = min(k, __shfl_down_sync(0xffffffffu, k, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (c) atomicAdd(inside, c);
        atomicMin(min_key, k);
    }
}

__global__ void sdf_seed_kernel(const float* __restrict__ g, int dx, int dy, int dz, int mx, int my, int mz, float h,
                                float minpz, float cx, float cy, float margin, unsigned long long* __restrict__ best) {
    const long long n = (long long)dx * dy * dz;
    unsigned long long b = ~0ull;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = __ldg(&g[i]);
        if (d > margin) continue;
        const int x = (int)(i % dx), y = (int)((i / dx) % dy), z = (int)(i / ((long long)dx * dy));
        const float px = (float)(mx + x) * h, py = (float)(my + y) * h, pz = (float)(mz + z) * h;
        const float ex = px - cx, ey = py - cy;
        const float xy = sqrtf(ex * ex + ey * ey);
        const float zh = fmaxf(0.0f, pz - minpz);
        const float score = zh * 10.0f + xy * 0.5f;
        const unsigned long long key = ((unsigned long long)ordered_u32(score) << 32) | (unsigned long long)(i & 0xffffffffLL);
        b = key < b ? key : b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
        b = t < b ? t : b;
    }
    if ((threadIdx.x & 31) == 0 && b != ~0ull) atomicMin(best, b);
}

struct IsoErr {
    char* buf;
    size_t len;
    int set(int status, const char* fmt, ...) {
        if (buf && len > 0) {
            va_list ap;
            va_start(ap, fmt);
            vsnprintf(buf, len, fmt, ap);
            va_end(ap);
        }
        return status;
    }
};

// Per-device scratch kept across calls (grow-only, one allocation, carved 256-byte
// aligned): the query call and the emit call that follows it, and repeated extractions of
// one lattice, allocate nothing. Calls on one device hold its lock for their duration.
struct IsoCache {
    std::mutex mu;
    void* base = nullptr;  // scratch
    size_t bytes = 0;
    void* out = nullptr;   // library-owned mesh (gbsdf_extract_iso_surface_device)
    size_t out_bytes = 0;
};
IsoCache g_iso[64];

struct IsoScratch {
    IsoCache& c;
    size_t need = 0;
    bool sizing = true;
    char* cur = nullptr;
    template <class T>
    T* get(size_t count, cudaError_t& err) {
        const size_t b = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        if (sizing) {
            need += b;
            return nullptr;
        }
        if (err != cudaSuccess) return nullptr;
        T* p = reinterpret_cast<T*>(cur);
        cur += b;
        return p;
    }
    cudaError_t commit() {  // after the sizing pass: grow the cache, start carving
        if (need > c.bytes) {
            if (c.base) cudaFree(c.base);
            c.base = nullptr;
            c.bytes = 0;
            const cudaError_t ce = cudaMalloc(&c.base, need);
            if (ce != cudaSuccess) return ce;
            c.bytes = need;
        }
        sizing = false;
        cur = static_cast<char*>(c.base);
        return cudaSuccess;
    }
};

bool table_to_device() {
    std::call_once(g_tri_once, mc_table_init);
    int8_t n[256];
    for (int cs = 0; cs < 256; ++cs) {
        n[cs] = 0;
        while (n[cs] < 5 && g_tri[cs][3 * n[cs]] >= 0) ++n[cs];
    }
    return cudaMemcpyToSymbol(c_tri, g_tri, sizeof(g_tri)) == cudaSuccess &&
           cudaMemcpyToSymbol(c_ntri, n, sizeof(n)) == cudaSuccess;
}

}  // namespace

void release_iso_workspace(int device) {
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lock(g_iso[device].mu);
    if (g_iso[device].base) cudaFree(g_iso[device].base);
    if (g_iso[device].out) cudaFree(g_iso[device].out);
    g_iso[device].base = g_iso[device].out = nullptr;
    g_iso[device].bytes = g_iso[device].out_bytes = 0;
}

}  // namespace gbsdf

using namespace gbsdf;

// outputs: 0 caller's host arrays, 1 caller's device arrays, 2 library-owned device arrays
// (their addresses returned through *lib_v / *lib_i)
static int extract_iso(const float* grid, int32_t grid_on_device, const int32_t dims[3], float voxel_size,
                       const float origin[3], float iso_value, float* out_vertices, int64_t vertex_capacity,
                       uint32_t* out_indices, int64_t index_capacity, int outputs, float** lib_v, uint32_t** lib_i,
                       int64_t* n_vertices, int64_t* n_indices, int32_t device, char* err, size_t errlen) {
    IsoErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!n_vertices || !n_indices || !dims || !origin) return e.set(GBSDF_EINVAL, "null argument");
    *n_vertices = 0;
    *n_indices = 0;
    const int dx = dims[0], dy = dims[1], dz = dims[2];
    if (dx < 2 || dy < 2 || dz < 2) return GBSDF_OK;  // no cube: an empty mesh (cuda_marching_cubes.cu:842-845)
    if (!grid) return e.set(GBSDF_EINVAL, "null grid");
    if (!(voxel_size > 0.0f) || !std::isfinite(voxel_size)) return e.set(GBSDF_EINVAL, "voxel size must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device available");
    }
    if (device < 0 || device >= ndev || device >= 64)
        return e.set(GBSDF_ENODEV, "device %d out of range", device);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ECUDA, "cudaSetDevice failed");
    }
    if (!table_to_device()) {
        cudaGetLastError();
        return e.set(GBSDF_ECUDA, "triangle table upload failed");
    }
    const long long N = (long long)dx * dy * dz;
    const int gpz = (dy + kGR - 1) / kGR;  // row groups per z plane
    const long long groups = (long long)gpz * dz;
    const long long tiles = (long long)dy * dz;  // rows: the units of the scans
    if (groups > 0x7fffffffLL) return e.set(GBSDF_EINVAL, "lattice too large (%lld row groups)", groups);
    const IsoGeom G{dx, dy, dz, gpz, iso_value, iso_value + voxel_size};
    cudaError_t ce = cudaSuccess;
    std::lock_guard<std::mutex> lock(g_iso[device].mu);
    IsoScratch s{g_iso[device]};
    // two passes over the same carving: sizing, then placing
    const float* g = grid;
    float* d_up = nullptr;
    uint8_t* d_mask = nullptr;
    unsigned *d_tv = nullptr, *d_tt = nullptr;
    unsigned long long *d_pv = nullptr, *d_pt = nullptr, *d_scan = nullptr;
    uint32_t* d_vbase = nullptr;
    for (int pass = 0; pass < 2; ++pass) {
        if (!grid_on_device) d_up = s.get<float>((size_t)N, ce);
        d_mask = s.get<uint8_t>((size_t)N, ce);
        d_tv = s.get<unsigned>((size_t)tiles, ce);
        d_tt = s.get<unsigned>((size_t)tiles, ce);
        d_pv = s.get<unsigned long long>((size_t)tiles + 1, ce);
        d_pt = s.get<unsigned long long>((size_t)tiles + 1, ce);
        d_scan = s.get<unsigned long long>((size_t)scan_tmp_elems(tiles), ce);
        d_vbase = s.get<uint32_t>((size_t)N, ce);
        if (pass == 0) ce = s.commit();
    }
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    cudaStream_t st = 0;
    if (!grid_on_device) {  // the reference's path: the host grid is uploaded
        ce = cudaMemcpyAsync(d_up, grid, (size_t)N * 4, cudaMemcpyHostToDevice, st);
        if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "grid upload: %s", cudaGetErrorString(ce));
        g = d_up;
    }
    GBSDF_COUNT_LAUNCH();
    iso_count_kernel<<<(unsigned)groups, kIsoThreads, 0, st>>>(g, G, d_mask, d_tv, d_tt);
    launch_exclusive_scan(d_tv, d_pv, tiles, d_scan, 0, st);
    launch_exclusive_scan(d_tt, d_pt, tiles, d_scan, 0, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "iso-surface count launch: %s", cudaGetErrorString(ce));
    unsigned long long pv = 0, pt = 0;
    unsigned lv = 0, lt = 0;
    cudaMemcpyAsync(&pv, d_pv + (tiles - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&pt, d_pt + (tiles - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&lv, d_tv + (tiles - 1), 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&lt, d_tt + (tiles - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "iso-surface count: %s", cudaGetErrorString(ce));
    const long long V = (long long)(pv + lv), T = (long long)(pt + lt);
    *n_vertices = V;
    *n_indices = 3 * T;
    if (V > 0xffffffffLL) return e.set(GBSDF_EINVAL, "%lld vertices exceed 32-bit indices", V);
    if (V == 0 || T == 0) {
        *n_vertices = 0;
        *n_indices = 0;
        return GBSDF_OK;
    }
    if (outputs == 2) {  // library-owned: grow the cache's mesh region
        IsoCache& c = g_iso[device];
        const size_t vb = ((size_t)V * 12 + 255) & ~size_t(255), need = vb + (size_t)T * 12;
        if (need > c.out_bytes) {
            if (c.out) cudaFree(c.out);
            c.out = nullptr;
            c.out_bytes = 0;
            ce = cudaMalloc(&c.out, need);
            if (ce != cudaSuccess) {
                cudaGetLastError();
                return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
            }
            c.out_bytes = need;
        }
        out_vertices = static_cast<float*>(c.out);
        out_indices = reinterpret_cast<uint32_t*>(static_cast<char*>(c.out) + vb);
        vertex_capacity = V;
        index_capacity = 3 * T;
        *lib_v = out_vertices;
        *lib_i = out_indices;
    }
    const bool outputs_on_device = outputs != 0;
    if (vertex_capacity < V || index_capacity < 3 * T || !out_vertices || !out_indices)
        return e.set(GBSDF_EINVAL, "outputs must hold %lld vertices and %lld indices", V, 3 * T);
    float* d_v = out_vertices;
    uint32_t* d_i = out_indices;
    void* stage = nullptr;  // host outputs: device staging of the mesh, per call
    if (!outputs_on_device) {
        ce = cudaMalloc(&stage, (size_t)V * 12 + (size_t)T * 12 + 256);
        if (ce != cudaSuccess) {
            cudaGetLastError();
            return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
        }
        d_v = static_cast<float*>(stage);
        d_i = reinterpret_cast<uint32_t*>(static_cast<char*>(stage) + (((size_t)V * 12 + 255) & ~size_t(255)));
    }
    struct FreeStage {
        void* p;
        ~FreeStage() {
            if (p) cudaFree(p);
        }
    } free_stage{stage};
    GBSDF_COUNT_LAUNCH();
    iso_vertex_kernel<<<(unsigned)groups, kIsoThreads, 0, st>>>(g, G, voxel_size, origin[0], origin[1], origin[2],
                                                               d_pv, d_vbase, d_v);
    GBSDF_COUNT_LAUNCH();
    iso_triangle_kernel<<<(unsigned)groups, kIsoThreads, 0, st>>>(g, G, d_mask, d_vbase, d_pt, d_i);
    ce = cudaGetLastError();
    if (ce == cudaSuccess && !outputs_on_device) {
        ce = cudaMemcpyAsync(out_vertices, d_v, (size_t)V * 12, cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(out_indices, d_i, (size_t)T * 12, cudaMemcpyDeviceToHost, st);
    }
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "iso-surface emit: %s", cudaGetErrorString(ce));
    return GBSDF_OK;
}


extern "C" {

int gbsdf_iso_surface_table(int8_t* out_table) {
    if (!out_table) return GBSDF_EINVAL;
    std::call_once(g_tri_once, mc_table_init);
    std::memcpy(out_table, g_tri, sizeof(g_tri));
    return GBSDF_OK;
}

int gbsdf_extract_iso_surface(const float* grid, int32_t grid_on_device, const int32_t dims[3], float voxel_size,
                              const float origin[3], float iso_value, float* out_vertices, int64_t vertex_capacity,
                              uint32_t* out_indices, int64_t index_capacity, int32_t outputs_on_device,
                              int64_t* n_vertices, int64_t* n_indices, int32_t device, char* err, size_t errlen) {
    return extract_iso(grid, grid_on_device, dims, voxel_size, origin, iso_value, out_vertices, vertex_capacity,
                       out_indices, index_capacity, outputs_on_device ? 1 : 0, nullptr, nullptr, n_vertices, n_indices,
                       device, err, errlen);
}

int gbsdf_extract_iso_surface_device(const float* grid, int32_t grid_on_device, const int32_t dims[3],
                                     float voxel_size, const float origin[3], float iso_value, float** vertices_dev,
                                     uint32_t** indices_dev, int64_t* n_vertices, int64_t* n_indices, int32_t device,
                                     char* err, size_t errlen) {
    if (!vertices_dev || !indices_dev) {
        if (err && errlen) std::snprintf(err, errlen, "null output pointers");
        return GBSDF_EINVAL;
    }
    *vertices_dev = nullptr;
    *indices_dev = nullptr;
    return extract_iso(grid, grid_on_device, dims, voxel_size, origin, iso_value, nullptr, 0, nullptr, 0, 2,
                       vertices_dev, indices_dev, n_vertices, n_indices, device, err, errlen);
}

// shared set-up of the two reductions: device, grid on the device, a small result block
struct SdfReduce {
    float* dgrid = nullptr;
    unsigned long long* res = nullptr;  // [0] inside count, [1] min key (low 32), [2] best seed key
    ~SdfReduce() {
        if (dgrid) cudaFree(dgrid);
        if (res) cudaFree(res);
    }
};

static int sdf_reduce_setup(const float* grid, int32_t on_dev, long long n, int32_t device, IsoErr& e,
                            SdfReduce& r, const float** g) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) return e.set(GBSDF_ENODEV, "device %d out of range", device);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ECUDA, "cudaSetDevice failed");
    }
    cudaError_t ce = cudaMalloc(&r.res, 3 * sizeof(unsigned long long));
    if (ce == cudaSuccess && !on_dev) {  // the reference's path: the host grid is uploaded
        ce = cudaMalloc(&r.dgrid, (size_t)n * 4);
        if (ce == cudaSuccess) ce = cudaMemcpy(r.dgrid, grid, (size_t)n * 4, cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(ce == cudaErrorMemoryAllocation ? GBSDF_ENOMEM : GBSDF_ECUDA, "device set-up: %s",
                     cudaGetErrorString(ce));
    }
    *g = on_dev ? grid : r.dgrid;
    const unsigned long long init[3] = {0ull, 0xffffffffull, ~0ull};
    ce = cudaMemcpy(r.res, init, sizeof(init), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "device set-up: %s", cudaGetErrorString(ce));
    GBSDF_COUNT_LAUNCH();
    sdf_inside_min_kernel<<<152 * 8, 256>>>(*g, n, &r.res[0], reinterpret_cast<unsigned*>(&r.res[1]));
    return GBSDF_OK;
}

static float ordered_to_float(unsigned k) {
    const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int gbsdf_interior_volume(const float* grid, int32_t grid_on_device, int64_t n_voxels, float voxel_size,
                          float* out_volume_mm3, int64_t* out_inside_voxels, int32_t device, char* err,
                          size_t errlen) {
    IsoErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!out_volume_mm3) return e.set(GBSDF_EINVAL, "null output");
    *out_volume_mm3 = 0.0f;
    if (out_inside_voxels) *out_inside_voxels = 0;
    if (!grid || n_voxels <= 0) return e.set(GBSDF_EINVAL, "empty grid");  // the reference returns false
    SdfReduce r;
    const float* g = nullptr;
    int rc = sdf_reduce_setup(grid, grid_on_device, n_voxels, device, e, r, &g);
    if (rc != GBSDF_OK) return rc;
    unsigned long long cnt = 0;
    const cudaError_t ce = cudaMemcpy(&cnt, &r.res[0], 8, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "interior volume: %s", cudaGetErrorString(ce));
    const float vox = voxel_size * voxel_size * voxel_size;
    *out_volume_mm3 = (float)cnt * vox;
    if (out_inside_voxels) *out_inside_voxels = (int64_t)cnt;
    return GBSDF_OK;
}

int gbsdf_find_default_seed(const float* grid, int32_t grid_on_device, const int32_t dims[3],
                            const int32_t min_coord[3], float voxel_size, const float min_p[3], const float max_p[3],
                            float desired_margin, float out_seed[3], int32_t device, char* err, size_t errlen) {
    IsoErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!dims || !min_coord || !min_p || !max_p || !out_seed) return e.set(GBSDF_EINVAL, "null argument");
    const float cx = (min_p[0] + max_p[0]) * 0.5f, cy = (min_p[1] + max_p[1]) * 0.5f;
    out_seed[0] = cx;
    out_seed[1] = cy;
    out_seed[2] = min_p[2] + 2.0f * voxel_size;
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    if (!grid || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return e.set(GBSDF_EINVAL, "empty grid");
    SdfReduce r;
    const float* g = nullptr;
    int rc = sdf_reduce_setup(grid, grid_on_device, n, device, e, r, &g);
    if (rc != GBSDF_OK) return rc;
    unsigned long long mk = 0;
    cudaError_t ce = cudaMemcpy(&mk, &r.res[1], 8, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "default seed: %s", cudaGetErrorString(ce));
    const float mn = std::min(1e30f, ordered_to_float((unsigned)mk));
    const float margin = (mn < 0.0f) ? std::max(desired_margin, mn * 0.65f) : (mn + voxel_size);
    GBSDF_COUNT_LAUNCH();
    sdf_seed_kernel<<<152 * 8, 256>>>(g, dims[0], dims[1], dims[2], min_coord[0], min_coord[1], min_coord[2],
                                      voxel_size, min_p[2], cx, cy, margin, &r.res[2]);
    unsigned long long best = ~0ull;
    ce = cudaMemcpy(&best, &r.res[2], 8, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "default seed: %s", cudaGetErrorString(ce));
    if (best != ~0ull) {
        const long long i = (long long)(best & 0xffffffffull);
        if (i < n) {
            const int x = (int)(i % dims[0]), y = (int)((i / dims[0]) % dims[1]),
                      z = (int)(i / ((long long)dims[0] * dims[1]));
            out_seed[0] = (float)(min_coord[0] + x) * voxel_size;
            out_seed[1] = (float)(min_coord[1] + y) * voxel_size;
            out_seed[2] = (float)(min_coord[2] + z) * voxel_size;
        }
    }
    return GBSDF_OK;
}

}  // extern "C"
