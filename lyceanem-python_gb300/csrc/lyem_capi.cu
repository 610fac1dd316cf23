// lyem_capi.cu -- extern "C" entry points declared in include/lyem.h.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <vector>

#include "lyem.h"
#include "lyem_device.cuh"
#include "lyem_grid.cuh"
#include "lyem_internal.cuh"

using namespace lyem;

namespace {

thread_local int g_last_cuda_error = 0;

int cuda_fail(cudaError_t e) {
    record_cuda_error(e);
    return e == cudaErrorMemoryAllocation ? LYEM_ERR_NOMEM : LYEM_ERR_CUDA;
}

#define LYEM_CK(call)                                  \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(e_);   \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

__global__ void pack_triangles_kernel(const float* __restrict__ verts, long long n_verts, const int* __restrict__ idx,
                                      long long n_tris, float4* __restrict__ out, unsigned int* err) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n_tris;
         t += (long long)gridDim.x * blockDim.x) {
        int a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
        if (a < 0 || b < 0 || c < 0 || a >= n_verts || b >= n_verts || c >= n_verts) {
            if (err) atomicOr(err, 2u);
            out[3 * t] = out[3 * t + 1] = out[3 * t + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        float ax = verts[3LL * a], ay = verts[3LL * a + 1], az = verts[3LL * a + 2];
        float bx = verts[3LL * b], by = verts[3LL * b + 1], bz = verts[3LL * b + 2];
        float cx = verts[3LL * c], cy = verts[3LL * c + 1], cz = verts[3LL * c + 2];
        out[3 * t] = make_float4(ax, ay, az, 0.f);
        out[3 * t + 1] = make_float4(__fsub_rn(bx, ax), __fsub_rn(by, ay), __fsub_rn(bz, az), 0.f);
        out[3 * t + 2] = make_float4(__fsub_rn(cx, ax), __fsub_rn(cy, ay), __fsub_rn(cz, az), 0.f);
    }
}

__global__ void mask_to_bytes_kernel(const unsigned* __restrict__ bits, long long n_src, long long n_snk,
                                     long long words, unsigned char* __restrict__ out) {
    const long long total = n_src * n_snk;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        long long n = i / n_snk, m = i - n * n_snk;
        out[i] = (bits[n * words + (m >> 5)] >> (m & 31)) & 1u;
    }
}

unsigned blocks_for(long long n, int threads) { return capped_blocks(n, threads, 32); }

BinSpec grid_spec(const float* origin3, float cell, const int32_t* dims3) {
    BinSpec b;
    for (int k = 0; k < 3; ++k) {
        b.org[k] = origin3[k];
        b.dims[k] = dims3[k];
        b.comp[k] = k;
    }
    b.cell = cell;
    b.inv_cell = 1.0f / cell;
    b.pad = 1e-3f * cell;
    return b;
}

bool valid_grid(const float* origin3, float cell, const int32_t* dims3) {
    if (!origin3 || !dims3 || !(cell > 0.f) || !isfinite(cell)) return false;
    long long nc = 1;
    for (int k = 0; k < 3; ++k) {
        if (dims3[k] < 1 || !isfinite(origin3[k])) return false;
        nc *= dims3[k];
    }
    return nc < (1LL << 30);
}

size_t stage_ws_bytes(long long n_src, long long n_snk, int chunk) {
    long long chunks = (n_src + chunk - 1) / chunk;
    return (size_t)chunks * (size_t)n_snk * 6 * sizeof(float) + 256;
}

// Owning device buffer for the host-buffer mirrors (stream-ordered).
struct DevBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t alloc(size_t bytes, cudaStream_t stream) {
        s = stream;
        return cudaMallocAsync(&p, bytes > 0 ? bytes : 16, stream);
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
    ~DevBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

}  // namespace

void lyem::record_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }

// Sources per thread block when the caller passes 0.  Brute force: as many
// as keep about four waves of blocks in flight (the triangle tiles are
// re-staged per block).  Grid: 16, or 64 for 16,384 sources and more, fewer
// when that would leave under four waves.  On the 28 GHz one-bounce scene the
// scatter->sink stage (50,000 sources) measured 539.7 / 536.8 / 537.7 ms at
// 16 / 32 / 64, and 64 writes a quarter of the per-chunk partial sums of 16;
// the 1,024-source stages were faster at 16.
int lyem::auto_src_chunk(long long n_src, long long n_snk, bool grid) {
    const long long tiles = (n_snk + stage_block_threads() - 1) / stage_block_threads();
    const long long waves = (long long)device_sm_count() * 8 * 4;
    long long c;
    if (grid) {
        c = n_src >= 16384 ? 64 : 16;
        while (c > 1 && ((n_src + c - 1) / c) * tiles < waves) c /= 2;
    } else {
        c = (n_src * tiles) / waves;
    }
    const long long cap = grid ? grid_max_src_chunk() : brute_max_src_chunk();
    return (int)std::max(1LL, std::min(c, cap));
}


extern "C" {

LYEM_API int lyem_version(void) { return 100; }

LYEM_API const char* lyem_status_string(int status) {
    switch (status) {
        case LYEM_OK: return "ok";
        case LYEM_ERR_INVALID: return "invalid argument";
        case LYEM_ERR_CUDA: return "CUDA runtime error";
        case LYEM_ERR_NOMEM: return "device allocation failed";
        case LYEM_ERR_TIMEOUT: return "bounded device wait expired";
        case LYEM_ERR_OVERFLOW: return "size exceeds 32-bit index range";
        case LYEM_ERR_WORKSPACE: return "workspace too small";
        default: return "unknown status";
    }
}

LYEM_API int lyem_last_cuda_error(void) { return g_last_cuda_error; }

LYEM_API uint64_t lyem_kernel_launches(void) { return (uint64_t)launches_so_far(); }

LYEM_API int lyem_fp32_fma_probe(int64_t iterations, double* fma_per_second, void* stream) {
    if (iterations < 16 || !fma_per_second) return LYEM_ERR_INVALID;
    LYEM_CK(fma_probe(iterations, fma_per_second, as_stream(stream)));
    return LYEM_OK;
}

LYEM_API int lyem_device_errors(void* stream, uint32_t* flags_out) {
    unsigned int flags = 0;
    LYEM_CK(read_clear_device_errors(&flags, as_stream(stream)));
    if (flags_out) *flags_out = flags;
    return (flags & 1u) ? LYEM_ERR_TIMEOUT : LYEM_OK;
}

LYEM_API int lyem_pack_triangles(const float* d_verts, int64_t n_verts, const int32_t* d_idx, int64_t n_tris,
                                 float* d_tris, void* stream) {
    if (n_verts < 0 || n_tris < 0) return LYEM_ERR_INVALID;
    if (n_tris == 0) return LYEM_OK;
    if (!d_verts || !d_idx || !d_tris || !aligned16(d_tris)) return LYEM_ERR_INVALID;
    pack_triangles_kernel<<<blocks_for(n_tris, 256), 256, 0, as_stream(stream)>>>(
        d_verts, n_verts, d_idx, n_tris, reinterpret_cast<float4*>(d_tris), device_error_word()); note_launches(1);
    LYEM_CK(cudaGetLastError());
    return LYEM_OK;
}

LYEM_API int lyem_tris_bounds(const float* d_tris, int64_t n_tris, float* d_bounds6, void* stream) {
    if (n_tris < 0 || !d_bounds6 || (n_tris > 0 && (!d_tris || !aligned16(d_tris)))) return LYEM_ERR_INVALID;
    LYEM_CK(launch_tris_bounds(reinterpret_cast<const float4*>(d_tris), n_tris, d_bounds6, as_stream(stream)));
    return LYEM_OK;
}

LYEM_API int lyem_grid_plan(const float* bounds6, int64_t n_tris, float cell, float* origin3_out, float* cell_out,
                            int32_t* dims3_out) {
    if (!bounds6 || !origin3_out || !cell_out || !dims3_out || n_tris < 0) return LYEM_ERR_INVALID;
    double lo[3], ext[3], emax = 0.0;
    for (int k = 0; k < 3; ++k) {
        lo[k] = bounds6[k];
        double hi = bounds6[3 + k];
        if (!isfinite(lo[k]) || !isfinite(hi) || hi < lo[k]) {  // empty mesh: unit box at the origin
            lo[k] = 0.0;
            hi = 1.0;
        }
        ext[k] = hi - lo[k];
        emax = std::max(emax, ext[k]);
    }
    if (emax <= 0.0) emax = 1.0;
    double c = cell;
    if (!(c > 0.0)) {
        const double target = std::max<double>(1.0, (double)n_tris);
        auto count = [&](double h) {
            double n = 1.0;
            for (int k = 0; k < 3; ++k) n *= std::max(1.0, std::ceil(ext[k] / h));
            return n;
        };
        double a = emax / 1024.0, b = emax;  // count(a) large, count(b) small
        for (int it = 0; it < 60; ++it) {
            double mid = std::sqrt(a * b);
            if (count(mid) > target) a = mid;
            else b = mid;
        }
        c = b;
    }
    const double pad = 1e-3 * c;
    long long nc = 1;
    for (int k = 0; k < 3; ++k) {
        double org = lo[k] - 2.0 * pad;
        double d = std::ceil((lo[k] + ext[k] + 2.0 * pad - org) / c);
        if (d < 1.0) d = 1.0;
        if (d > 65536.0) return LYEM_ERR_OVERFLOW;
        origin3_out[k] = (float)org;
        dims3_out[k] = (int32_t)d;
        nc *= (long long)d;
    }
    if (nc >= (1LL << 30)) return LYEM_ERR_OVERFLOW;
    *cell_out = (float)c;
    return LYEM_OK;
}

LYEM_API size_t lyem_grid_count_workspace(int64_t n_tris) { return grid_count_workspace_bytes(n_tris < 0 ? 0 : n_tris); }

LYEM_API int lyem_grid_count(const float* d_tris, int64_t n_tris, const float* origin3, float cell,
                             const int32_t* dims3, int32_t* d_tri_offsets, int64_t* d_total_refs, void* d_ws,
                             size_t ws_bytes, void* stream) {
    if (n_tris < 0 || !d_tri_offsets || !d_total_refs || !valid_grid(origin3, cell, dims3)) return LYEM_ERR_INVALID;
    if (n_tris > 0 && (!d_tris || !aligned16(d_tris))) return LYEM_ERR_INVALID;
    if (n_tris >= (1LL << 31) - 1) return LYEM_ERR_OVERFLOW;
    if (!d_ws || ws_bytes < grid_count_workspace_bytes(n_tris)) return LYEM_ERR_WORKSPACE;
    BinSpec b = grid_spec(origin3, cell, dims3);
    LYEM_CK(grid_count(b, reinterpret_cast<const float4*>(d_tris), n_tris, d_tri_offsets,
                       reinterpret_cast<unsigned long long*>(d_total_refs), d_ws, as_stream(stream)));
    return LYEM_OK;
}

LYEM_API size_t lyem_grid_fill_workspace(int64_t n_refs, int64_t n_cells) {
    return grid_fill_workspace_bytes(n_refs < 0 ? 0 : n_refs, n_cells);
}

LYEM_API int lyem_grid_fill(const float* d_tris, int64_t n_tris, const float* origin3, float cell,
                            const int32_t* dims3, const int32_t* d_tri_offsets, int64_t n_refs, int32_t* d_cell_start,
                            float* d_cell_tris, float* d_cell_box, void* d_ws, size_t ws_bytes, void* stream) {
    if (n_tris < 0 || n_refs < 0 || !d_tri_offsets || !d_cell_start || !valid_grid(origin3, cell, dims3))
        return LYEM_ERR_INVALID;
    if (!d_cell_box || !aligned16(d_cell_box)) return LYEM_ERR_INVALID;
    if (n_refs > 0 && (!d_cell_tris || !aligned16(d_cell_tris) || !d_tris || !aligned16(d_tris))) return LYEM_ERR_INVALID;
    if (n_refs >= (1LL << 31) - 64) return LYEM_ERR_OVERFLOW;
    const long long ncells = (long long)dims3[0] * dims3[1] * dims3[2];
    if (!d_ws || ws_bytes < grid_fill_workspace_bytes(n_refs, ncells)) return LYEM_ERR_WORKSPACE;
    BinSpec b = grid_spec(origin3, cell, dims3);
    LYEM_CK(grid_fill(b, reinterpret_cast<const float4*>(d_tris), n_tris, d_tri_offsets, n_refs, d_cell_start,
                      reinterpret_cast<float4*>(d_cell_tris), reinterpret_cast<float4*>(d_cell_box), d_ws,
                      as_stream(stream)));
    return LYEM_OK;
}

LYEM_API size_t lyem_spatial_order_workspace(int64_t n_points) {
    return spatial_order_workspace_bytes(n_points < 0 ? 0 : n_points);
}

LYEM_API int lyem_spatial_order(const float* d_points, int64_t n_points, int32_t* d_order, void* d_ws,
                                size_t ws_bytes, void* stream) {
    if (n_points < 0) return LYEM_ERR_INVALID;
    if (n_points == 0) return LYEM_OK;
    if (!d_points || !d_order) return LYEM_ERR_INVALID;
    if (n_points >= (1LL << 31) - 64) return LYEM_ERR_OVERFLOW;
    if (!d_ws || ws_bytes < spatial_order_workspace_bytes(n_points)) return LYEM_ERR_WORKSPACE;
    LYEM_CK(spatial_order(d_points, n_points, d_order, d_ws, as_stream(stream)));
    return LYEM_OK;
}

LYEM_API int lyem_direction_order(const float* d_points, int64_t n_points, const float* centre3, int32_t* d_order,
                                  void* d_ws, size_t ws_bytes, void* stream) {
    if (n_points < 0) return LYEM_ERR_INVALID;
    if (n_points == 0) return LYEM_OK;
    if (!d_points || !d_order || !centre3) return LYEM_ERR_INVALID;
    for (int k = 0; k < 3; ++k)
        if (!isfinite(centre3[k])) return LYEM_ERR_INVALID;
    if (n_points >= (1LL << 31) - 64) return LYEM_ERR_OVERFLOW;
    if (!d_ws || ws_bytes < spatial_order_workspace_bytes(n_points)) return LYEM_ERR_WORKSPACE;
    LYEM_CK(direction_order(d_points, n_points, centre3, d_order, d_ws, as_stream(stream)));
    return LYEM_OK;
}

LYEM_API size_t lyem_pair_stage_workspace(int64_t n_src, int64_t n_snk, int64_t n_tris, int32_t use_grid,
                                          int32_t src_chunk) {
    (void)n_tris;
    if (n_src <= 0 || n_snk <= 0) return 256;
    int chunk = src_chunk > 0 ? src_chunk : auto_src_chunk(n_src, n_snk, use_grid != 0);
    chunk = std::min(chunk, use_grid ? grid_max_src_chunk() : brute_max_src_chunk());
    return stage_ws_bytes(n_src, n_snk, chunk);
}

LYEM_API int lyem_pair_stage(const float* d_src_pos, const float* d_src_E, const float* d_src_W, int64_t n_src,
                             const float* d_snk_pos, const float* d_snk_nrm, int64_t n_snk, const float* d_tris,
                             int64_t n_tris, const int32_t* d_cell_start, const float* d_cell_tris,
                             const float* d_cell_box, const float* grid_origin3, float grid_cell,
                             const int32_t* grid_dims3, double alpha, double beta, int32_t self_to_self, int32_t cull,
                             float eps, float* d_sink_out,
                             int32_t accumulate, float* d_pair_out, uint32_t* d_mask_bits, uint64_t* d_counters,
                             int32_t* d_src_visible, int32_t* d_snk_visible, const int32_t* d_src_order,
                             const int32_t* d_snk_order, int32_t src_chunk, int32_t traversal, void* d_ws,
                             size_t ws_bytes, void* stream) {
    if (n_src < 0 || n_snk < 0 || n_tris < 0) return LYEM_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const bool use_grid = d_cell_start != nullptr;
    if (n_src == 0 || n_snk == 0) {
        if (d_sink_out && !accumulate && n_snk > 0) LYEM_CK(cudaMemsetAsync(d_sink_out, 0, 24 * (size_t)n_snk, s));
        return LYEM_OK;
    }
    if (!d_src_pos || !d_src_E || !d_snk_pos || !d_snk_nrm) return LYEM_ERR_INVALID;
    if (!(eps >= 0.f) || !isfinite(eps)) return LYEM_ERR_INVALID;  // the culling test relies on A >= eps >= 0
    // the stage kernels index sources and sinks in 32 bits
    if (n_src >= (1LL << 31) - 256 || n_snk >= (1LL << 31) - 256) return LYEM_ERR_OVERFLOW;
    if (use_grid) {
        if (!d_cell_tris || !aligned16(d_cell_tris) || !d_cell_box || !aligned16(d_cell_box) ||
            !valid_grid(grid_origin3, grid_cell, grid_dims3))
            return LYEM_ERR_INVALID;
    } else if (n_tris > 0 && (!d_tris || !aligned16(d_tris))) {
        return LYEM_ERR_INVALID;
    }
    if (((uintptr_t)d_src_E & 7u) || ((uintptr_t)d_src_W & 7u) || ((uintptr_t)d_pair_out & 7u) ||
        ((uintptr_t)d_sink_out & 7u))
        return LYEM_ERR_INVALID;
    int chunk = src_chunk > 0 ? src_chunk : auto_src_chunk(n_src, n_snk, use_grid);
    chunk = std::min(chunk, use_grid ? grid_max_src_chunk() : brute_max_src_chunk());
    if (use_grid && traversal == 38) chunk = transposed_src_chunk();  // one lane per source of a chunk
    if ((n_snk + stage_block_threads() - 1) / stage_block_threads() > 0x7fffffffLL) return LYEM_ERR_OVERFLOW;
    const size_t need = stage_ws_bytes(n_src, n_snk, chunk);
    if (!d_ws || ws_bytes < need) return LYEM_ERR_WORKSPACE;

    StageParams p;
    memset(&p, 0, sizeof(p));
    p.src_pos = d_src_pos;
    p.src_E = d_src_E;
    p.src_W = d_src_W;
    p.n_src = n_src;
    p.snk_pos = d_snk_pos;
    p.snk_nrm = d_snk_nrm;
    p.n_snk = n_snk;
    p.tris = reinterpret_cast<const float4*>(d_tris);
    p.n_tris = use_grid ? 0 : n_tris;
    if (use_grid) {
        p.cell_start = d_cell_start;
        p.cell_tris = reinterpret_cast<const float4*>(d_cell_tris);
        p.cell_box = reinterpret_cast<const float4*>(d_cell_box);
        for (int k = 0; k < 3; ++k) {
            p.g0[k] = grid_origin3[k];
            p.g1[k] = grid_origin3[k] + grid_dims3[k] * grid_cell;
            p.dims[k] = grid_dims3[k];
        }
        p.cell = grid_cell;
        p.inv_cell = 1.0f / grid_cell;
    }
    p.alpha = (float)alpha;
    p.beta_f = (float)beta;
    p.beta_d = beta;
    p.eps = eps;
    p.skip_diag = self_to_self ? 0 : 1;
    p.src_chunk = chunk;
    p.partial = static_cast<float*>(d_ws);
    p.pair_out = d_pair_out;
    p.mask_bits = d_mask_bits;
    p.mask_words = (n_snk + 31) / 32;
    p.counters = reinterpret_cast<unsigned long long*>(d_counters);
    p.src_visible = d_src_visible;
    p.snk_visible = d_snk_visible;
    p.src_order = d_src_order;
    p.snk_order = d_snk_order;
    const bool two_phase = (traversal >= 101 && traversal <= 164) || (traversal >= 201 && traversal <= 264);
    if ((traversal < 0 || traversal > 38 || traversal == 37) && !two_phase) return LYEM_ERR_INVALID;
    static const int kCapped[3] = {-10, -12, -16};  // traversal 34, 35, 36
    if (two_phase) {
        p.refill_lanes = traversal < 200 ? -116 : -112;
        p.near_dist = (float)(traversal % 100) * (use_grid ? grid_cell : 1.f);
    } else {
        p.refill_lanes = traversal == 0 ? -16 : traversal == 1 ? 0 : traversal <= 33 ? traversal - 1
                         : traversal == 38 ? -38 : kCapped[traversal - 34];
    }
    if (d_mask_bits && d_snk_order)  // permuted sinks set their mask bits one by one
        LYEM_CK(cudaMemsetAsync(d_mask_bits, 0, sizeof(uint32_t) * (size_t)n_src * (size_t)p.mask_words, s));
    LYEM_CK(launch_pair_stage(p, cull, s));
    if (d_sink_out) {
        const long long chunks = (n_src + chunk - 1) / chunk;
        LYEM_CK(launch_reduce_partials(p.partial, chunks, n_snk, d_sink_out, accumulate, s));
    }
    return LYEM_OK;
}

LYEM_API int lyem_mask_to_bytes(const uint32_t* d_mask_bits, int64_t n_src, int64_t n_snk, uint8_t* d_out,
                                void* stream) {
    if (n_src < 0 || n_snk < 0) return LYEM_ERR_INVALID;
    if (n_src * n_snk == 0) return LYEM_OK;
    if (!d_mask_bits || !d_out) return LYEM_ERR_INVALID;
    mask_to_bytes_kernel<<<blocks_for(n_src * n_snk, 256), 256, 0, as_stream(stream)>>>(
        d_mask_bits, n_src, n_snk, (n_snk + 31) / 32, d_out); note_launches(1);
    LYEM_CK(cudaGetLastError());
    return LYEM_OK;
}

}  // extern "C"

// ------------------------------------------------- host-buffer mirrors

namespace {

cudaStream_t em_stream() { return cudaStreamPerThread; }

template <typename T>
cudaError_t upload(DevBuf& b, const T* host, size_t count, cudaStream_t s) {
    cudaError_t e = b.alloc(count * sizeof(T), s);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpyAsync(b.p, host, count * sizeof(T), cudaMemcpyHostToDevice, s);
}

// y-z bins of the reference's tile structure: axis 0 = z, axis 1 = y, axis 2 = x (one layer).
BinSpec yz_spec(int ncells_y_axis, int ncells_z_axis, float ymin, float width, float zmin) {
    BinSpec b;
    b.org[0] = zmin;
    b.org[1] = ymin;
    b.org[2] = 0.f;
    b.cell = width;
    b.inv_cell = 1.0f / width;
    b.dims[0] = ncells_z_axis;
    b.dims[1] = ncells_y_axis;
    b.dims[2] = 1;
    b.comp[0] = 2;
    b.comp[1] = 1;
    b.comp[2] = 0;
    b.pad = 1e-3f * width;
    return b;
}

int em_bin_common(const float* tri_vertex, int64_t n_vertex, const int32_t* tri_index, int64_t n_tris,
                  int32_t ncells_x, int32_t ncells_y, float ymin, float cell_width, float z_min,
                  int32_t* counts_out, const int32_t* expect_counts, int64_t sum_expect, int32_t* index_out) {
    if (n_vertex < 0 || n_tris < 0 || ncells_x < 1 || ncells_y < 1 || !(cell_width > 0.f)) return LYEM_ERR_INVALID;
    if ((n_vertex > 0 && !tri_vertex) || (n_tris > 0 && !tri_index)) return LYEM_ERR_INVALID;
    if ((long long)ncells_x * ncells_y >= (1LL << 30)) return LYEM_ERR_OVERFLOW;
    cudaStream_t s = em_stream();
    const long long ncells = (long long)ncells_x * ncells_y;
    DevBuf dv, di, dt, doff, dtot, dws, dstart;
    LYEM_CK(upload(dv, tri_vertex, 3 * (size_t)n_vertex, s));
    LYEM_CK(upload(di, tri_index, 3 * (size_t)n_tris, s));
    LYEM_CK(dt.alloc(48 * (size_t)n_tris, s));
    if (n_tris > 0) {
        pack_triangles_kernel<<<blocks_for(n_tris, 256), 256, 0, s>>>(dv.as<float>(), n_vertex, di.as<int>(), n_tris,
                                                                     dt.as<float4>(), device_error_word()); note_launches(1);
        LYEM_CK(cudaGetLastError());
    }
    BinSpec b = yz_spec(ncells_x, ncells_y, ymin, cell_width, z_min);
    LYEM_CK(doff.alloc(sizeof(int) * (size_t)(n_tris + 1), s));
    LYEM_CK(dtot.alloc(sizeof(unsigned long long), s));
    LYEM_CK(dws.alloc(grid_count_workspace_bytes(n_tris), s));
    LYEM_CK(grid_count(b, dt.as<float4>(), n_tris, doff.as<int>(), dtot.as<unsigned long long>(), dws.p, s));
    unsigned long long total = 0;
    LYEM_CK(cudaMemcpyAsync(&total, dtot.p, sizeof(total), cudaMemcpyDeviceToHost, s));
    LYEM_CK(cudaStreamSynchronize(s));
    if (total >= (1ULL << 31) - 64) return LYEM_ERR_OVERFLOW;
    const long long R = (long long)total;
    LYEM_CK(dstart.alloc(sizeof(int) * (size_t)(ncells + 1), s));
    DevBuf dws2, dout;
    LYEM_CK(dws2.alloc(grid_fill_workspace_bytes(R, ncells), s));
    LYEM_CK(dout.alloc(3 * sizeof(int) * (size_t)R, s));
    LYEM_CK(bin_fill_index(b, dt.as<float4>(), n_tris, doff.as<int>(), R, di.as<int>(), dstart.as<int>(),
                           dout.as<int>(), dws2.p, s));
    std::vector<int> start((size_t)ncells + 1);
    LYEM_CK(cudaMemcpyAsync(start.data(), dstart.p, sizeof(int) * (ncells + 1), cudaMemcpyDeviceToHost, s));
    LYEM_CK(cudaStreamSynchronize(s));
    if (counts_out) {
        for (long long c = 0; c < ncells; ++c) counts_out[c] = start[c + 1] - start[c];
    }
    if (index_out) {
        // The caller sizes `out` from the counts it was given; they must be this binning's counts.
        if (sum_expect != R) return LYEM_ERR_INVALID;
        for (long long c = 0; c < ncells; ++c)
            if (expect_counts[c] != start[c + 1] - start[c]) return LYEM_ERR_INVALID;
        if (R > 0) LYEM_CK(cudaMemcpyAsync(index_out, dout.p, 3 * sizeof(int) * R, cudaMemcpyDeviceToHost, s));
        LYEM_CK(cudaStreamSynchronize(s));
    }
    return LYEM_OK;
}

// Shared body of the two calculate_scattering_* mirrors.
int em_scatter(const float* source, int64_t n_source, const float* end, int64_t n_end, const float* tri_vertex,
               int64_t n_vertex, const int32_t* tri_idx, int64_t n_tris, bool use_grid, const float* ex_real,
               const float* ex_imag, const float* ey_real, const float* ey_imag, const float* ez_real,
               const float* ez_imag, const float* normal, float alpha, float beta, int32_t not_self_to_self,
               float* out) {
    if (n_source < 0 || n_end < 0 || n_vertex < 0 || n_tris < 0) return LYEM_ERR_INVALID;
    if (n_source * n_end == 0) return LYEM_OK;
    if (!source || !end || !ex_real || !ex_imag || !ey_real || !ey_imag || !ez_real || !ez_imag || !normal || !out)
        return LYEM_ERR_INVALID;
    if (n_tris > 0 && (!tri_vertex || !tri_idx)) return LYEM_ERR_INVALID;
    cudaStream_t s = em_stream();
    std::vector<float> E(6 * (size_t)n_source);
    for (int64_t n = 0; n < n_source; ++n) {
        E[6 * n] = ex_real[n]; E[6 * n + 1] = ex_imag[n];
        E[6 * n + 2] = ey_real[n]; E[6 * n + 3] = ey_imag[n];
        E[6 * n + 4] = ez_real[n]; E[6 * n + 5] = ez_imag[n];
    }
    DevBuf dsrc, dend, dnrm, dE, dv, di, dt, dpair;
    LYEM_CK(upload(dsrc, source, 3 * (size_t)n_source, s));
    LYEM_CK(upload(dend, end, 3 * (size_t)n_end, s));
    // the reference's normal array holds the source normals then the sink normals; only the sink ones are used
    LYEM_CK(upload(dnrm, normal + 3 * n_source, 3 * (size_t)n_end, s));
    LYEM_CK(upload(dE, E.data(), E.size(), s));
    LYEM_CK(upload(dv, tri_vertex, 3 * (size_t)n_vertex, s));
    LYEM_CK(upload(di, tri_idx, 3 * (size_t)n_tris, s));
    LYEM_CK(dt.alloc(48 * (size_t)n_tris, s));
    if (n_tris > 0) {
        pack_triangles_kernel<<<blocks_for(n_tris, 256), 256, 0, s>>>(dv.as<float>(), n_vertex, di.as<int>(), n_tris,
                                                                     dt.as<float4>(), device_error_word()); note_launches(1);
        LYEM_CK(cudaGetLastError());
    }
    const size_t pair_bytes = 24 * (size_t)n_source * (size_t)n_end;
    LYEM_CK(dpair.alloc(pair_bytes, s));

    DevBuf dstart, dcell, dbox, dws;
    float org[3] = {0, 0, 0}, cell = 1.f;
    int32_t dims[3] = {1, 1, 1};
    if (use_grid && n_tris > 0) {
        DevBuf db, doff, dtot, dcw;
        LYEM_CK(db.alloc(6 * sizeof(float), s));
        LYEM_CK(launch_tris_bounds(dt.as<float4>(), n_tris, db.as<float>(), s));
        float bounds[6];
        LYEM_CK(cudaMemcpyAsync(bounds, db.p, sizeof(bounds), cudaMemcpyDeviceToHost, s));
        LYEM_CK(cudaStreamSynchronize(s));
        int st = lyem_grid_plan(bounds, n_tris, 0.f, org, &cell, dims);
        if (st != LYEM_OK) return st;
        BinSpec b = grid_spec(org, cell, dims);
        LYEM_CK(doff.alloc(sizeof(int) * (size_t)(n_tris + 1), s));
        LYEM_CK(dtot.alloc(sizeof(unsigned long long), s));
        LYEM_CK(dcw.alloc(grid_count_workspace_bytes(n_tris), s));
        LYEM_CK(grid_count(b, dt.as<float4>(), n_tris, doff.as<int>(), dtot.as<unsigned long long>(), dcw.p, s));
        unsigned long long total = 0;
        LYEM_CK(cudaMemcpyAsync(&total, dtot.p, sizeof(total), cudaMemcpyDeviceToHost, s));
        LYEM_CK(cudaStreamSynchronize(s));
        if (total >= (1ULL << 31) - 64) return LYEM_ERR_OVERFLOW;
        const long long ncells = (long long)dims[0] * dims[1] * dims[2];
        LYEM_CK(dstart.alloc(sizeof(int) * (size_t)(ncells + 1), s));
        LYEM_CK(dcell.alloc(48 * (size_t)total, s));
        LYEM_CK(dbox.alloc(64 * (size_t)ncells, s));
        DevBuf dfw;
        LYEM_CK(dfw.alloc(grid_fill_workspace_bytes((long long)total, ncells), s));
        LYEM_CK(grid_fill(b, dt.as<float4>(), n_tris, doff.as<int>(), (long long)total, dstart.as<int>(),
                          dcell.as<float4>(), dbox.as<float4>(), dfw.p, s));
    }
    const bool grid_on = use_grid && n_tris > 0;
    const size_t ws = lyem_pair_stage_workspace(n_source, n_end, n_tris, grid_on, 0);
    LYEM_CK(dws.alloc(ws, s));
    int st = lyem_pair_stage(dsrc.as<float>(), dE.as<float>(), nullptr, n_source, dend.as<float>(), dnrm.as<float>(),
                             n_end, dt.as<float>(), n_tris, grid_on ? dstart.as<int32_t>() : nullptr,
                             grid_on ? dcell.as<float>() : nullptr, grid_on ? dbox.as<float>() : nullptr, org, cell,
                             dims, (double)alpha, (double)beta,
                             not_self_to_self, 1, kEpsilon, nullptr, 0, dpair.as<float>(), nullptr, nullptr, nullptr,
                             nullptr, nullptr, nullptr, 0, 0, dws.p, ws, s);
    if (st != LYEM_OK) return st;
    LYEM_CK(cudaMemcpyAsync(out, dpair.p, pair_bytes, cudaMemcpyDeviceToHost, s));
    LYEM_CK(cudaStreamSynchronize(s));
    uint32_t flags = 0;
    return lyem_device_errors(s, &flags);
}

}  // namespace

extern "C" {

LYEM_API int lyem_em_bin_counts(const float* tri_vertex, int64_t n_vertex, const int32_t* tri_index, int64_t n_tris,
                                int32_t ncells_x, int32_t ncells_y, float ymin, float cell_width, float z_min,
                                int32_t* counts_out) {
    if (!counts_out) return LYEM_ERR_INVALID;
    return em_bin_common(tri_vertex, n_vertex, tri_index, n_tris, ncells_x, ncells_y, ymin, cell_width, z_min,
                         counts_out, nullptr, 0, nullptr);
}

LYEM_API int lyem_em_bin_triangles(const float* tri_vertex, int64_t n_vertex, const int32_t* tri_index,
                                   int64_t n_tris, int32_t ncells_x, int32_t ncells_y, float ymin, float cell_width,
                                   float z_min, const int32_t* bin_counts, int64_t sum_bin_counts, int32_t* out) {
    if (!bin_counts || sum_bin_counts < 0 || (sum_bin_counts > 0 && !out)) return LYEM_ERR_INVALID;
    return em_bin_common(tri_vertex, n_vertex, tri_index, n_tris, ncells_x, ncells_y, ymin, cell_width, z_min,
                         nullptr, bin_counts, sum_bin_counts, out);
}

LYEM_API int lyem_em_calculate_scattering_brute_force(
    const float* source, int64_t n_source, const float* end, int64_t n_end, const int32_t* triangles, int64_t n_tris,
    const float* triangle_vertex, int64_t n_vertex, float wave_length, const float* ex_real, const float* ex_imag,
    const float* ey_real, const float* ey_imag, const float* ez_real, const float* ez_imag, const float* normal,
    float alpha, float beta, int32_t not_self_to_self, float* out) {
    (void)wave_length;  // unused by the reference's em_wave as well (lyceanem/src/em.cuh:64)
    return em_scatter(source, n_source, end, n_end, triangle_vertex, n_vertex, triangles, n_tris, false, ex_real,
                      ex_imag, ey_real, ey_imag, ez_real, ez_imag, normal, alpha, beta, not_self_to_self, out);
}

LYEM_API int lyem_em_calculate_scattering_tiles(
    const float* source, int64_t n_source, const float* end, int64_t n_end, const float* triangle_vertex,
    int64_t n_vertex, float wave_length, const float* ex_real, const float* ex_imag, const float* ey_real,
    const float* ey_imag, const float* ez_real, const float* ez_imag, const float* normal, float xmin, float xmax,
    float ymin, float ymax, float zmin, float zmax, float tile_size, const int32_t* bin_count,
    const int32_t* bin_triangles, int32_t n_cellsx, int32_t n_cellsy, int32_t binned_tri_num, float alpha,
    float beta, int32_t not_self_to_self, float* out) {
    (void)wave_length; (void)xmin; (void)xmax; (void)ymin; (void)ymax; (void)zmin; (void)zmax; (void)tile_size;
    if (n_cellsx < 0 || n_cellsy < 0 || binned_tri_num < 0) return LYEM_ERR_INVALID;
    if (binned_tri_num > 0 && !bin_triangles) return LYEM_ERR_INVALID;
    if (bin_count) {
        long long sum = 0;
        for (long long c = 0; c < (long long)n_cellsx * n_cellsy; ++c) {
            if (bin_count[c] < 0) return LYEM_ERR_INVALID;
            sum += bin_count[c];
        }
        if (sum != binned_tri_num) return LYEM_ERR_INVALID;
    }
    // The triangle set is the distinct vertex triples among the binned slots;
    // slots the reference's binning left unfilled hold (-1, -1, -1) and are skipped.
    std::vector<std::array<int32_t, 3>> tri;
    tri.reserve((size_t)binned_tri_num);
    for (int32_t i = 0; i < binned_tri_num; ++i) {
        std::array<int32_t, 3> t = {bin_triangles[3 * i], bin_triangles[3 * i + 1], bin_triangles[3 * i + 2]};
        if (t[0] < 0 || t[1] < 0 || t[2] < 0) continue;
        if (t[0] >= n_vertex || t[1] >= n_vertex || t[2] >= n_vertex) return LYEM_ERR_INVALID;
        tri.push_back(t);
    }
    std::sort(tri.begin(), tri.end());
    tri.erase(std::unique(tri.begin(), tri.end()), tri.end());
    return em_scatter(source, n_source, end, n_end, triangle_vertex, n_vertex,
                      tri.empty() ? nullptr : tri.front().data(), (int64_t)tri.size(), true, ex_real, ex_imag,
                      ey_real, ey_imag, ez_real, ez_imag, normal, alpha, beta, not_self_to_self, out);
}

}  // extern "C"
