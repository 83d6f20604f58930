// k_io.cu — GPU decoders of the mesh wire formats that feed the SDF path.
//
// Reference: CudaRasterizer::parse_binary_stl_gpu (cuda_mesh_io.cu:592-722, record decode
// gpu_decode_binary_stl_kernel :524-590) and CudaRasterizer::parse_obj_text_gpu
// (cuda_mesh_io.cu:962-1090, kernels :859-960, number parsers :810-857).
//
// Binary STL: the reference decodes on the GPU but welds on the host (one hash-map pass
// over every corner, cuda_mesh_io.cu:675-708). Here the weld is on the GPU and keeps the
// reference's result exactly -- vertices identified by their round(coordinate * 10000)
// key, numbered in order of first occurrence, triangles with a repeated welded corner
// dropped in order:
//   1. decode: one thread per record (unaligned 50-byte records read bytewise), the
//      normal normalised with the reference's fallbacks, the corners' keys;
//   2. insert: a lock-free open-addressing table of corner indices; a slot's content is a
//      corner index whose key never changes once claimed, and equal keys keep the
//      smallest corner index (atomicMin), so the table ends the same whatever the order;
//   3. first flags (corner == its key's smallest corner), an exclusive scan numbers the
//      first corners in file order, every corner takes its first corner's number;
//   4. a scan over the kept triangles compacts the index list in order.
// ASCII STL (CudaRasterizer::parse_ascii_stl_gpu, cuda_mesh_io.cu:1201-1325): the reference
// collects "vertex" token offsets with atomics and bitonic-sorts them, then welds on the
// GPU with slots claimed in thread order, so its vertex numbering varies from run to run.
// Here a scan over per-byte token flags gives the file order, the corners go through the
// same order-independent weld as binary STL, keyed on the reference's 64-bit hash of the
// quantised coordinates, and vertices are numbered in order of first occurrence.
// OBJ: the reference finds "v " / "f " line starts with atomics and sorts the offsets on
// the host; here a scan over per-byte flags gives the file order directly. Faces are
// counted (0, 1 or 2 triangles), scanned and written in file order (the reference's
// atomic append order varies from run to run). Arithmetic follows the reference source
// expression by expression, each operation rounded once (-fmad=false).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gbsdf.h"
#include "gbsdf_internal.h"

namespace gbsdf {
namespace {

constexpr uint32_t kEmpty = 0xffffffffu;

__device__ __forceinline__ float ld_f32(const uint8_t* p) {
    const uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    return __uint_as_float(u);
}

__device__ __forceinline__ int32_t quant(float v) { return (int32_t)roundf(v * 10000.0f); }

__device__ __forceinline__ uint32_t key_hash(int3 k) {
    uint64_t h = (uint64_t)(uint32_t)k.x * 0x9E3779B97F4A7C15ull ^ (uint64_t)(uint32_t)k.y * 0xC2B2AE3D27D4EB4Full ^
                 (uint64_t)(uint32_t)k.z * 0x165667B19E3779F9ull;
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (uint32_t)h;
}

__device__ __forceinline__ bool key_eq(int3 a, int3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

__device__ __forceinline__ uint32_t key_hash(unsigned long long k) {
    uint64_t h = k * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (uint32_t)h;
}

__device__ __forceinline__ bool key_eq(unsigned long long a, unsigned long long b) { return a == b; }

// 1. decode (gpu_decode_binary_stl_kernel, cuda_mesh_io.cu:524-590)
__global__ void stl_decode_kernel(const uint8_t* __restrict__ payload, long long T, float* __restrict__ raw,
                                  float* __restrict__ normals, int3* __restrict__ keys) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint8_t* rec = payload + t * 50;
    float nx = ld_f32(rec), ny = ld_f32(rec + 4), nz = ld_f32(rec + 8);
    float v[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[k][c] = ld_f32(rec + 12 + 12 * k + 4 * c);
    const float len = sqrtf(nx * nx + ny * ny + nz * nz);
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
        const float gl = sqrtf(nx * nx + ny * ny + nz * nz);
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
    normals[3 * t] = nx;
    normals[3 * t + 1] = ny;
    normals[3 * t + 2] = nz;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const long long c = 3 * t + k;
        raw[3 * c] = v[k][0];
        raw[3 * c + 1] = v[k][1];
        raw[3 * c + 2] = v[k][2];
        keys[c] = make_int3(quant(v[k][0]), quant(v[k][1]), quant(v[k][2]));
    }
}

// 2. insert every corner; equal keys keep their smallest corner index
template <class K>
__global__ void weld_insert_kernel(const K* __restrict__ keys, long long n, uint32_t* __restrict__ table,
                                   uint32_t mask) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const K k = keys[i];
    uint32_t h = key_hash(k) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        uint32_t cur = table[h];
        if (cur == kEmpty) {
            const uint32_t prev = atomicCAS(&table[h], kEmpty, (uint32_t)i);
            if (prev == kEmpty) return;
            cur = prev;
        }
        if (key_eq(keys[cur], k)) {
            atomicMin(&table[h], (uint32_t)i);
            return;
        }
        h = (h + 1) & mask;
    }
}

// 3a. first-occurrence flags and each corner's first corner
template <class K>
__global__ void weld_first_kernel(const K* __restrict__ keys, long long n, const uint32_t* __restrict__ table,
                                  uint32_t mask, unsigned* __restrict__ first, uint32_t* __restrict__ rep) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const K k = keys[i];
    uint32_t h = key_hash(k) & mask;
    uint32_t r = (uint32_t)i;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint32_t cur = table[h];
        if (cur != kEmpty && key_eq(keys[cur], k)) {
            r = cur;
            break;
        }
        h = (h + 1) & mask;
    }
    rep[i] = r;
    first[i] = (r == (uint32_t)i) ? 1u : 0u;
}

// 3b. number the vertices, write them in first-occurrence order
__global__ void weld_assign_kernel(const float* __restrict__ raw, long long n, const uint32_t* __restrict__ rep,
                                   const unsigned long long* __restrict__ first_pos, uint32_t* __restrict__ vid,
                                   float* __restrict__ out_v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = rep[i];
    const uint32_t id = (uint32_t)first_pos[r];
    vid[i] = id;
    if (r == (uint32_t)i) {
        out_v[3ull * id] = raw[3 * i];
        out_v[3ull * id + 1] = raw[3 * i + 1];
        out_v[3ull * id + 2] = raw[3 * i + 2];
    }
}

// 4. triangles with three distinct welded corners, compacted in order
__global__ void tri_keep_kernel(const uint32_t* __restrict__ vid, long long T, unsigned* __restrict__ keep) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint32_t a = vid[3 * t], b = vid[3 * t + 1], c = vid[3 * t + 2];
    keep[t] = (a != b && b != c && c != a) ? 1u : 0u;
}

__global__ void tri_write_kernel(const uint32_t* __restrict__ vid, long long T, const unsigned* __restrict__ keep,
                                 const unsigned long long* __restrict__ pos, uint32_t* __restrict__ out_idx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T || !keep[t]) return;
    const unsigned long long o = 3ull * pos[t];
    out_idx[o] = vid[3 * t];
    out_idx[o + 1] = vid[3 * t + 1];
    out_idx[o + 2] = vid[3 * t + 2];
}

// ---- OBJ ----------------------------------------------------------------------------
// line-start flags (gpu_find_obj_lines_kernel, cuda_mesh_io.cu:859-888)
__global__ void obj_flags_kernel(const char* __restrict__ text, long long n, unsigned* __restrict__ fv,
                                 unsigned* __restrict__ ff) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned v = 0, f = 0;
    if ((i == 0 || text[i - 1] == '\n') && i + 1 < n && text[i + 1] == ' ') {
        v = text[i] == 'v';
        f = text[i] == 'f';
    }
    fv[i] = v;
    ff[i] = f;
}

__global__ void obj_offsets_kernel(long long n, const unsigned* __restrict__ fv, const unsigned* __restrict__ ff,
                                   const unsigned long long* __restrict__ pv, const unsigned long long* __restrict__ pf,
                                   long long cap, long long* __restrict__ vo, long long* __restrict__ fo) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (fv[i] && (long long)pv[i] < cap) vo[pv[i]] = i + 2;
    if (ff[i] && (long long)pf[i] < cap) fo[pf[i]] = i + 2;
}

// device_fast_atof / device_fast_atoi (cuda_mesh_io.cu:810-857)
__device__ float obj_atof(const char*& p) {
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
        val *= powf(10.0f, es * (float)ev);
    }
    return sign * val;
}

__device__ int obj_atoi(const char*& p) {
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

__global__ void obj_vertices_kernel(const char* __restrict__ text, const long long* __restrict__ vo, long long nv,
                                    float* __restrict__ out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nv) return;
    const char* p = text + vo[k];
    const float x = obj_atof(p);
    const float y = obj_atof(p);
    const float z = obj_atof(p);
    out[3 * k] = x;
    out[3 * k + 1] = y;
    out[3 * k + 2] = z;
}

// one face line (gpu_parse_obj_faces_kernel, cuda_mesh_io.cu:909-960): up to 4 indices
__device__ int obj_face(const char* p, int nverts, int f[4]) {
    int c = 0;
    while (*p != '\n' && *p != '\r' && *p != '\0' && c < 4) {
        while (*p == ' ' || *p == '\t') ++p;
        if (*p == '\n' || *p == '\r' || *p == '\0') break;
        int vi = obj_atoi(p);
        while (*p != ' ' && *p != '\t' && *p != '\n' && *p != '\r' && *p != '\0') ++p;
        if (vi < 0) vi = nverts + vi + 1;
        if (vi > 0) f[c++] = vi - 1;
    }
    return c;
}

__global__ void obj_face_count_kernel(const char* __restrict__ text, const long long* __restrict__ fo, long long nf,
                                      int nverts, unsigned* __restrict__ ntri) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    int f[4];
    const int c = obj_face(text + fo[k], nverts, f);
    ntri[k] = (c == 3) ? 1u : (c == 4) ? 2u : 0u;
}

__global__ void obj_face_write_kernel(const char* __restrict__ text, const long long* __restrict__ fo, long long nf,
                                      int nverts, const unsigned long long* __restrict__ pos,
                                      uint32_t* __restrict__ out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    int f[4];
    const int c = obj_face(text + fo[k], nverts, f);
    uint32_t* o = out + 3ull * pos[k];
    if (c == 3 || c == 4) {
        o[0] = (uint32_t)f[0];
        o[1] = (uint32_t)f[1];
        o[2] = (uint32_t)f[2];
    }
    if (c == 4) {
        o[3] = (uint32_t)f[0];
        o[4] = (uint32_t)f[2];
        o[5] = (uint32_t)f[3];
    }
}

// ---- host helpers --------------------------------------------------------------------
struct IErr {
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

// Device allocations of one call, freed on every exit.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* get(size_t count, cudaError_t& err) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

// ---- ASCII STL ----------------------------------------------------------------------
// "vertex" token flags (gpu_find_ascii_stl_vertices_kernel, cuda_mesh_io.cu:1094-1118): at
// the text start or after a space, tab, CR or LF, followed by a space or tab, and starting
// before the last 7 bytes.
__global__ void stla_flags_kernel(const char* __restrict__ text, long long n, unsigned* __restrict__ fl) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned f = 0;
    if (i + 7 < n) {
        const char b = (i == 0) ? ' ' : text[i - 1];
        const bool start = b == ' ' || b == '\t' || b == '\n' || b == '\r';
        f = start && text[i] == 'v' && text[i + 1] == 'e' && text[i + 2] == 'r' && text[i + 3] == 't' &&
            text[i + 4] == 'e' && text[i + 5] == 'x' && (text[i + 6] == ' ' || text[i + 6] == '\t');
    }
    fl[i] = f;
}

__global__ void stla_offsets_kernel(long long n, const unsigned* __restrict__ fl,
                                    const unsigned long long* __restrict__ pos, long long cap,
                                    long long* __restrict__ vo) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (fl[i] && (long long)pos[i] < cap) vo[pos[i]] = i + 6;
}

// the reference's weld key (dev_quantize_vec3_key, cuda_mesh_io.cu:1146-1156): a 64-bit
// mix of the round(coordinate * 10000) integers; corners with equal keys are one vertex
__global__ void stla_keys_kernel(const float* __restrict__ raw, long long n, unsigned long long* __restrict__ keys) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long ux = (uint32_t)quant(raw[3 * i]), uy = (uint32_t)quant(raw[3 * i + 1]),
                             uz = (uint32_t)quant(raw[3 * i + 2]);
    unsigned long long h = (ux * 73856093ull) ^ (uy * 19349663ull) ^ (uz * 83492791ull) ^ ((ux & 0xFFFFFull) << 42) ^
                           ((uy & 0xFFFFFull) << 21) ^ (uz & 0x1FFFFFull);
    keys[i] = h ? h : 1ull;
}

unsigned blocks_for(long long n, int threads = 256) { return (unsigned)((n + threads - 1) / threads); }

int set_device(int32_t device, IErr& e) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return e.set(GBSDF_ENODEV, "no CUDA device available");
    }
    if (device < 0 || device >= n) return e.set(GBSDF_ENODEV, "device %d out of range", device);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ECUDA, "cudaSetDevice failed");
    }
    return GBSDF_OK;
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" {

int gbsdf_parse_binary_stl(const uint8_t* bytes, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                           uint32_t* out_indices, int64_t index_capacity, float* out_normals, int64_t* n_vertices,
                           int64_t* n_indices, int32_t device, char* err, size_t errlen) {
    IErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!n_vertices || !n_indices) return e.set(GBSDF_EINVAL, "null count pointers");
    *n_vertices = 0;
    *n_indices = 0;
    if (!bytes || n_bytes < 84) return e.set(GBSDF_EINVAL, "binary STL shorter than its 84-byte header");
    uint32_t T32 = 0;
    std::memcpy(&T32, bytes + 80, 4);
    const long long T = T32;
    if (T == 0) return GBSDF_OK;  // an empty mesh (cuda_mesh_io.cu:611-615)
    if (n_bytes < 84 + (size_t)T * 50)
        return e.set(GBSDF_EINVAL, "binary STL holds %zu bytes, its header announces %lld records", n_bytes, T);
    if (3 * T > 0x7fffffffLL) return e.set(GBSDF_EINVAL, "too many triangles");
    if (vertex_capacity < 3 * T || index_capacity < 3 * T || !out_vertices || !out_indices)
        return e.set(GBSDF_EINVAL, "outputs must hold 3 x %lld vertices and indices", T);
    int rc = set_device(device, e);
    if (rc != GBSDF_OK) return rc;
    const long long n = 3 * T;
    uint32_t cap = 1024;
    while ((long long)cap < 2 * n) cap <<= 1;
    cudaError_t ce = cudaSuccess;
    Scratch s;
    uint8_t* d_payload = s.get<uint8_t>((size_t)T * 50, ce);
    float* d_raw = s.get<float>((size_t)n * 3, ce);
    float* d_norm = s.get<float>((size_t)T * 3, ce);
    int3* d_keys = s.get<int3>((size_t)n, ce);
    uint32_t* d_table = s.get<uint32_t>(cap, ce);
    unsigned* d_first = s.get<unsigned>((size_t)n, ce);
    uint32_t* d_rep = s.get<uint32_t>((size_t)n, ce);
    unsigned long long* d_fpos = s.get<unsigned long long>((size_t)n + 1, ce);
    uint32_t* d_vid = s.get<uint32_t>((size_t)n, ce);
    float* d_outv = s.get<float>((size_t)n * 3, ce);
    unsigned* d_keep = s.get<unsigned>((size_t)T, ce);
    unsigned long long* d_tpos = s.get<unsigned long long>((size_t)T + 1, ce);
    uint32_t* d_outi = s.get<uint32_t>((size_t)n, ce);
    unsigned long long* d_scan = s.get<unsigned long long>((size_t)std::max(scan_tmp_elems(n), scan_tmp_elems(T)), ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    cudaStream_t st = 0;
    cudaMemcpyAsync(d_payload, bytes + 84, (size_t)T * 50, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_table, 0xff, (size_t)cap * 4, st);
    GBSDF_COUNT_LAUNCH();
    stl_decode_kernel<<<blocks_for(T), 256, 0, st>>>(d_payload, T, d_raw, d_norm, d_keys);
    GBSDF_COUNT_LAUNCH();
    weld_insert_kernel<int3><<<blocks_for(n), 256, 0, st>>>(d_keys, n, d_table, cap - 1);
    GBSDF_COUNT_LAUNCH();
    weld_first_kernel<int3><<<blocks_for(n), 256, 0, st>>>(d_keys, n, d_table, cap - 1, d_first, d_rep);
    launch_exclusive_scan(d_first, d_fpos, n, d_scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    weld_assign_kernel<<<blocks_for(n), 256, 0, st>>>(d_raw, n, d_rep, d_fpos, d_vid, d_outv);
    GBSDF_COUNT_LAUNCH();
    tri_keep_kernel<<<blocks_for(T), 256, 0, st>>>(d_vid, T, d_keep);
    launch_exclusive_scan(d_keep, d_tpos, T, d_scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    tri_write_kernel<<<blocks_for(T), 256, 0, st>>>(d_vid, T, d_keep, d_tpos, d_outi);
    // totals: last exclusive prefix plus the last flag
    unsigned long long fl = 0, tl = 0;
    unsigned flast = 0, klast = 0;
    cudaMemcpyAsync(&fl, d_fpos + (n - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&flast, d_first + (n - 1), 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&tl, d_tpos + (T - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&klast, d_keep + (T - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "STL decode: %s", cudaGetErrorString(ce));
    const long long V = (long long)fl + flast, nt = (long long)tl + klast;
    ce = cudaMemcpy(out_vertices, d_outv, (size_t)V * 12, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && nt > 0) ce = cudaMemcpy(out_indices, d_outi, (size_t)nt * 12, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && out_normals) ce = cudaMemcpy(out_normals, d_norm, (size_t)T * 12, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "STL download: %s", cudaGetErrorString(ce));
    *n_vertices = V;
    *n_indices = 3 * nt;
    return GBSDF_OK;
}

int gbsdf_parse_obj(const char* text, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                    uint32_t* out_indices, int64_t index_capacity, int64_t* n_vertices, int64_t* n_indices,
                    int32_t device, char* err, size_t errlen) {
    IErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!n_vertices || !n_indices) return e.set(GBSDF_EINVAL, "null count pointers");
    *n_vertices = 0;
    *n_indices = 0;
    if (!text || n_bytes == 0) return e.set(GBSDF_EINVAL, "empty OBJ text");
    int rc = set_device(device, e);
    if (rc != GBSDF_OK) return rc;
    const long long n = (long long)n_bytes;
    const long long cap = n / 10 + 1024;  // the reference's line cap (cuda_mesh_io.cu:980)
    cudaError_t ce = cudaSuccess;
    Scratch s;
    char* d_text = s.get<char>((size_t)n + 1, ce);
    unsigned* d_fv = s.get<unsigned>((size_t)n, ce);
    unsigned* d_ff = s.get<unsigned>((size_t)n, ce);
    unsigned long long* d_pv = s.get<unsigned long long>((size_t)n + 1, ce);
    unsigned long long* d_pf = s.get<unsigned long long>((size_t)n + 1, ce);
    long long* d_vo = s.get<long long>((size_t)cap, ce);
    long long* d_fo = s.get<long long>((size_t)cap, ce);
    unsigned long long* d_scan = s.get<unsigned long long>((size_t)scan_tmp_elems(n), ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    cudaStream_t st = 0;
    cudaMemcpyAsync(d_text, text, (size_t)n, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_text + n, 0, 1, st);
    GBSDF_COUNT_LAUNCH();
    obj_flags_kernel<<<blocks_for(n), 256, 0, st>>>(d_text, n, d_fv, d_ff);
    launch_exclusive_scan(d_fv, d_pv, n, d_scan, 0, st);
    launch_exclusive_scan(d_ff, d_pf, n, d_scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    obj_offsets_kernel<<<blocks_for(n), 256, 0, st>>>(n, d_fv, d_ff, d_pv, d_pf, cap, d_vo, d_fo);
    unsigned long long pv = 0, pf = 0;
    unsigned lv = 0, lf = 0;
    cudaMemcpyAsync(&pv, d_pv + (n - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&pf, d_pf + (n - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&lv, d_fv + (n - 1), 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&lf, d_ff + (n - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "OBJ scan: %s", cudaGetErrorString(ce));
    const long long V = std::min<long long>((long long)pv + lv, cap);
    const long long F = std::min<long long>((long long)pf + lf, cap);
    if (V == 0 || F == 0) return e.set(GBSDF_EINVAL, "OBJ text holds no vertex or no face line");
    if (V > 0x7fffffffLL) return e.set(GBSDF_EINVAL, "too many vertices");
    if (vertex_capacity < V || !out_vertices)
        return e.set(GBSDF_EINVAL, "vertex output holds %lld of %lld vertices", (long long)vertex_capacity, V);
    float* d_v = s.get<float>((size_t)V * 3, ce);
    unsigned* d_nt = s.get<unsigned>((size_t)F, ce);
    unsigned long long* d_tp = s.get<unsigned long long>((size_t)F + 1, ce);
    unsigned long long* d_scan2 = s.get<unsigned long long>((size_t)scan_tmp_elems(F), ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    GBSDF_COUNT_LAUNCH();
    obj_vertices_kernel<<<blocks_for(V), 256, 0, st>>>(d_text, d_vo, V, d_v);
    GBSDF_COUNT_LAUNCH();
    obj_face_count_kernel<<<blocks_for(F), 256, 0, st>>>(d_text, d_fo, F, (int)V, d_nt);
    launch_exclusive_scan(d_nt, d_tp, F, d_scan2, 0, st);
    unsigned long long tl = 0;
    unsigned tlast = 0;
    cudaMemcpyAsync(&tl, d_tp + (F - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&tlast, d_nt + (F - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "OBJ faces: %s", cudaGetErrorString(ce));
    const long long NT = (long long)tl + tlast;
    if (NT == 0) return e.set(GBSDF_EINVAL, "OBJ text holds no triangle or quad face");
    if (index_capacity < 3 * NT || !out_indices)
        return e.set(GBSDF_EINVAL, "index output holds %lld of %lld indices", (long long)index_capacity, 3 * NT);
    uint32_t* d_i = s.get<uint32_t>((size_t)NT * 3, ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    GBSDF_COUNT_LAUNCH();
    obj_face_write_kernel<<<blocks_for(F), 256, 0, st>>>(d_text, d_fo, F, (int)V, d_tp, d_i);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpy(out_vertices, d_v, (size_t)V * 12, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(out_indices, d_i, (size_t)NT * 12, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "OBJ download: %s", cudaGetErrorString(ce));
    *n_vertices = V;
    *n_indices = 3 * NT;
    return GBSDF_OK;
}

int gbsdf_ascii_stl_capacity(size_t n_bytes, int64_t* vertex_capacity) {
    if (!vertex_capacity) return GBSDF_EINVAL;
    const size_t max_verts = n_bytes / 12 + 1024;
    size_t cap = 1024;
    while (cap < max_verts && cap < ((size_t)1 << 26)) cap <<= 1;
    *vertex_capacity = (int64_t)cap;
    return GBSDF_OK;
}

int gbsdf_parse_ascii_stl(const char* text, size_t n_bytes, float* out_vertices, int64_t vertex_capacity,
                          uint32_t* out_indices, int64_t index_capacity, int64_t* n_vertices, int64_t* n_indices,
                          int32_t device, char* err, size_t errlen) {
    IErr e{err, errlen};
    if (err && errlen) err[0] = 0;
    if (!n_vertices || !n_indices) return e.set(GBSDF_EINVAL, "null count pointers");
    *n_vertices = 0;
    *n_indices = 0;
    if (!text || n_bytes < 15) return e.set(GBSDF_EINVAL, "ASCII STL text shorter than 15 bytes");
    int64_t cap = 0;
    gbsdf_ascii_stl_capacity(n_bytes, &cap);
    int rc = set_device(device, e);
    if (rc != GBSDF_OK) return rc;
    const long long n = (long long)n_bytes;
    cudaError_t ce = cudaSuccess;
    Scratch s;
    char* d_text = s.get<char>((size_t)n + 1, ce);
    unsigned* d_fl = s.get<unsigned>((size_t)n, ce);
    unsigned long long* d_pos = s.get<unsigned long long>((size_t)n + 1, ce);
    long long* d_vo = s.get<long long>((size_t)cap, ce);
    unsigned long long* d_scan = s.get<unsigned long long>((size_t)scan_tmp_elems(n), ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    cudaStream_t st = 0;
    cudaMemcpyAsync(d_text, text, (size_t)n, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_text + n, 0, 1, st);
    GBSDF_COUNT_LAUNCH();
    stla_flags_kernel<<<blocks_for(n), 256, 0, st>>>(d_text, n, d_fl);
    launch_exclusive_scan(d_fl, d_pos, n, d_scan, 0, st);
    GBSDF_COUNT_LAUNCH();
    stla_offsets_kernel<<<blocks_for(n), 256, 0, st>>>(n, d_fl, d_pos, cap, d_vo);
    unsigned long long pl = 0;
    unsigned fl = 0;
    cudaMemcpyAsync(&pl, d_pos + (n - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&fl, d_fl + (n - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "ASCII STL scan: %s", cudaGetErrorString(ce));
    const long long tokens = std::min<long long>((long long)pl + fl, cap);
    const long long m = tokens - tokens % 3;  // whole facets
    if (m == 0) return e.set(GBSDF_EINVAL, "ASCII STL text holds no whole facet");
    if (vertex_capacity < m || index_capacity < m || !out_vertices || !out_indices)
        return e.set(GBSDF_EINVAL, "outputs must hold %lld vertices and indices", m);
    uint32_t tcap = 1024;
    while ((long long)tcap < 2 * m) tcap <<= 1;
    float* d_raw = s.get<float>((size_t)m * 3, ce);
    unsigned long long* d_keys = s.get<unsigned long long>((size_t)m, ce);
    uint32_t* d_table = s.get<uint32_t>(tcap, ce);
    unsigned* d_first = s.get<unsigned>((size_t)m, ce);
    uint32_t* d_rep = s.get<uint32_t>((size_t)m, ce);
    unsigned long long* d_fpos = s.get<unsigned long long>((size_t)m + 1, ce);
    uint32_t* d_vid = s.get<uint32_t>((size_t)m, ce);
    float* d_outv = s.get<float>((size_t)m * 3, ce);
    unsigned long long* d_scan2 = s.get<unsigned long long>((size_t)scan_tmp_elems(m), ce);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return e.set(GBSDF_ENOMEM, "device allocation failed: %s", cudaGetErrorString(ce));
    }
    cudaMemsetAsync(d_table, 0xff, (size_t)tcap * 4, st);
    GBSDF_COUNT_LAUNCH();
    obj_vertices_kernel<<<blocks_for(m), 256, 0, st>>>(d_text, d_vo, m, d_raw);
    GBSDF_COUNT_LAUNCH();
    stla_keys_kernel<<<blocks_for(m), 256, 0, st>>>(d_raw, m, d_keys);
    GBSDF_COUNT_LAUNCH();
    weld_insert_kernel<unsigned long long><<<blocks_for(m), 256, 0, st>>>(d_keys, m, d_table, tcap - 1);
    GBSDF_COUNT_LAUNCH();
    weld_first_kernel<unsigned long long><<<blocks_for(m), 256, 0, st>>>(d_keys, m, d_table, tcap - 1, d_first,
                                                                         d_rep);
    launch_exclusive_scan(d_first, d_fpos, m, d_scan2, 0, st);
    GBSDF_COUNT_LAUNCH();
    weld_assign_kernel<<<blocks_for(m), 256, 0, st>>>(d_raw, m, d_rep, d_fpos, d_vid, d_outv);
    unsigned long long vl = 0;
    unsigned vlast = 0;
    cudaMemcpyAsync(&vl, d_fpos + (m - 1), 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&vlast, d_first + (m - 1), 4, cudaMemcpyDeviceToHost, st);
    ce = cudaGetLastError();  // launch errors are not reported by the synchronisation
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "ASCII STL weld: %s", cudaGetErrorString(ce));
    const long long V = (long long)vl + vlast;
    ce = cudaMemcpy(out_vertices, d_outv, (size_t)V * 12, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(out_indices, d_vid, (size_t)m * 4, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return e.set(GBSDF_ECUDA, "ASCII STL download: %s", cudaGetErrorString(ce));
    *n_vertices = V;
    *n_indices = m;
    return GBSDF_OK;
}

}  // extern "C"
