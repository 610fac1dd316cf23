// lyem_noalloc.cu -- the pair stage for callers that may not allocate device memory.
//
// Some host applications own every byte of device memory through their own
// allocator (a plugin host that budgets memory for all its plugins, or a
// real-time loop that forbids allocation calls once it is running); such a
// caller cannot call cudaMalloc and cannot size and pass the scratch buffer
// that lyem_pair_stage needs.  lyem_pair_stage_noalloc takes the same inputs
// and outputs but keeps its scratch (the per-chunk partial sums of the sink
// field) in a file-scope __device__ array of kNoallocScratchBytes, which every
// GPU that loads this library holds until the process exits.
//
// The array is shared by every call and keeps the last call's contents.  The
// stage writes every partial-sum element it later reads, so nothing in it has
// to start at zero.  Calls whose work overlaps on the GPU (e.g. on two streams)
// race on the array.
#include <cuda_runtime.h>

#include "lyem.h"
#include "lyem_internal.cuh"

namespace {

constexpr size_t kNoallocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of g_noalloc_scratch in the current device's context.  In host
// code the array's name stands for a host-side shadow, not a device address,
// so the address is looked up with that device current.  It is looked up on
// every call rather than cached: a cached address would go stale once the
// caller resets the device (cudaDeviceReset) and the module is loaded again.
int scratch_address(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        lyem::record_cuda_error(e);
        return LYEM_ERR_CUDA;
    }
    *out = p;
    return LYEM_OK;
}

// Source chunk for the fixed scratch: the caller's chunk, else the automatic
// one when its partial sums fit, else the smallest larger chunk whose partial
// sums fit; 0 when even the largest chunk's do not.
int32_t noalloc_chunk(int64_t n_src, int64_t n_snk, bool use_grid, int32_t src_chunk) {
    const int32_t cap = use_grid ? lyem::grid_max_src_chunk() : lyem::brute_max_src_chunk();
    if (src_chunk > 0) return src_chunk < cap ? src_chunk : cap;
    const int32_t automatic = lyem::auto_src_chunk(n_src, n_snk, use_grid);
    // lyem_pair_stage's workspace: ceil(n_src / chunk) * n_snk * 24 bytes + 256
    const long long max_chunks = (long long)((kNoallocScratchBytes - 256) / (24ull * (unsigned long long)n_snk));
    if (max_chunks < 1) return 0;
    const long long need = (n_src + max_chunks - 1) / max_chunks;
    const long long chunk = need > automatic ? need : automatic;
    return chunk <= cap ? (int32_t)chunk : 0;
}

}  // namespace

extern "C" {

LYEM_API size_t lyem_pair_stage_noalloc_scratch_bytes(void) { return kNoallocScratchBytes; }

LYEM_API int lyem_pair_stage_noalloc(const float* d_src_pos, const float* d_src_E, const float* d_src_W,
                                     int64_t n_src, const float* d_snk_pos, const float* d_snk_nrm, int64_t n_snk,
                                     const float* d_tris, int64_t n_tris, const int32_t* d_cell_start,
                                     const float* d_cell_tris, const float* d_cell_box, const float* grid_origin3,
                                     float grid_cell,
                                     const int32_t* grid_dims3, double alpha, double beta, int32_t self_to_self,
                                     int32_t cull, float eps, float* d_sink_out, int32_t accumulate,
                                     float* d_pair_out, uint32_t* d_mask_bits, uint64_t* d_counters,
                                     int32_t* d_src_visible, int32_t* d_snk_visible, const int32_t* d_src_order,
                                     const int32_t* d_snk_order, int32_t src_chunk, int32_t traversal,
                                     void* stream) {
    if (n_src < 0 || n_snk < 0) return LYEM_ERR_INVALID;
    const bool use_grid = d_cell_start != nullptr;
    int32_t chunk = src_chunk;
    if (n_src > 0 && n_snk > 0) {
        chunk = noalloc_chunk(n_src, n_snk, use_grid, src_chunk);
        if (chunk <= 0 || lyem_pair_stage_workspace(n_src, n_snk, n_tris, use_grid, chunk) > kNoallocScratchBytes)
            return LYEM_ERR_WORKSPACE;
    }
    void* scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != LYEM_OK) return st;
    return lyem_pair_stage(d_src_pos, d_src_E, d_src_W, n_src, d_snk_pos, d_snk_nrm, n_snk, d_tris, n_tris,
                           d_cell_start, d_cell_tris, d_cell_box, grid_origin3, grid_cell, grid_dims3, alpha, beta,
                           self_to_self,
                           cull, eps, d_sink_out, accumulate, d_pair_out, d_mask_bits, d_counters, d_src_visible,
                           d_snk_visible, d_src_order, d_snk_order, chunk, traversal, scratch, kNoallocScratchBytes,
                           stream);
}

}  // extern "C"
