// lyem_internal.cuh -- parameter blocks and host helpers shared by the .cu files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyem.h"

namespace lyem {

// Bounded device waits give up after this many SM cycles (about one second at
// GB300 clocks) and raise LYEM_ERR_TIMEOUT instead of hanging.
constexpr long long kWaitCycles = 2000000000LL;

// Device-wide sticky error word (bit 0: a bounded wait expired, bit 1: an index
// check failed), defined in lyem_stage.cu.  Kernels of other translation units
// receive its device address from device_error_word().
unsigned int* device_error_word();
cudaError_t read_clear_device_errors(unsigned int* flags, cudaStream_t stream);

// One "pair stage": every (source n, sink m) segment is tested for visibility
// against the scene; visible pairs contribute their field to sink m.
//   out[m, c] (+)= sum_n W[n, c] * S[n, m, c]      (W == nullptr means 1)
// Optional outputs: the full per-pair network S (the reference's layout,
// source-major, 6 floats per pair) and a bit mask of visible pairs.
struct StageParams {
    const float* src_pos;  // [n_src, 3]
    const float* src_E;    // [n_src, 6] complex excitation (re, im) x (x, y, z)
    const float* src_W;    // [n_src, 6] per-component output weights or nullptr
    long long n_src;
    const float* snk_pos;  // [n_snk, 3]
    const float* snk_nrm;  // [n_snk, 3]
    long long n_snk;
    // brute force
    const float4* tris;  // [n_tris, 3] float4 (v0, e1, e2)
    long long n_tris;
    // uniform grid (used when cell_start != nullptr)
    const int* cell_start;     // [ncells + 1]
    const float4* cell_tris;   // [n_refs, 3] float4, triangles in cell order
    const float4* cell_box;    // [ncells, 2] float4: box of the cell's triangles and ref range
    float g0[3], g1[3];        // grid box
    float cell, inv_cell;
    int dims[3];
    // physics
    float alpha, beta_f;
    double beta_d;
    float eps;
    int skip_diag;
    // processing order (nullptr = natural): the thread block handles the
    // sources src_order[chunk] and the sinks snk_order[tile], so spatially
    // sorted orders give coherent warps; results are indexed by the original ids
    const int* src_order;
    const int* snk_order;
    // launch shape: blockIdx.y + chunk_base is the source chunk
    int src_chunk;
    long long chunk_base;
    int refill_lanes;  // grid stage schedule: 0 = lockstep, k > 0 = batched refill once k lanes are idle,
                       // -10 / -12 / -16 = lockstep with registers capped for that many blocks per SM,
                       // -116 / -112 = two phases split at near_dist, capped for 16 / 12 blocks per SM
    float near_dist;   // two-phase schedule: ray parameter (m) where phase 1 hands open rays to phase 2
    // outputs
    float* partial;              // [n_chunks, n_snk, 6]
    float* pair_out;             // [n_src, n_snk, 6] or nullptr
    unsigned int* mask_bits;     // [n_src, mask_words] or nullptr
    long long mask_words;
    unsigned long long* counters;  // [0] visible pairs, [1] ray/triangle tests (may be nullptr)
    int* src_visible;              // [n_src] visible sinks per source (may be nullptr)
    int* snk_visible;              // [n_snk] visible sources per sink (may be nullptr)
};

// Streaming multiprocessors of the current device, queried once per device and
// cached (the count of a device never changes); 1 if the query fails.
int device_sm_count();
// Blocks of `threads` threads covering n items of a grid-stride loop, at least
// one and at most per_sm blocks per SM of the current device.
unsigned capped_blocks(long long n, int threads, int per_sm);

// Records the CUDA error that lyem_last_cuda_error() reports (lyem_capi.cu).
void record_cuda_error(cudaError_t e);

// Host-side count of kernel launches made by this library (lyem_kernel_launches()).
void note_launches(unsigned long long n);
unsigned long long launches_so_far();

// FP32 FMA lane-operations per second of this device (calibration probe).
cudaError_t fma_probe(long long iters, double* fma_per_s, cudaStream_t stream);

// Host-side launchers (lyem_stage.cu).
cudaError_t launch_pair_stage(const StageParams& p, int cull, cudaStream_t stream);
cudaError_t launch_reduce_partials(const float* partial, long long n_chunks, long long n_snk, float* out,
                                   int accumulate, cudaStream_t stream);
int stage_block_threads();
// Sources per thread block of a pair stage when the caller passes 0 (lyem_capi.cu).
int auto_src_chunk(long long n_src, long long n_snk, bool grid);
int brute_max_src_chunk();
int grid_max_src_chunk();
int transposed_src_chunk();  // sources per block of the transposed grid schedule (traversal 38)

// Beam sweep on the tensor cores (lyem_sweep_tc.cu).  Operand buffers start
// with a header of kSweepHeaderBytes holding the power-of-two scales (floats
// [0, 3) of the network, float 0 of the weights) ahead of the K-major planes.
constexpr size_t kSweepHeaderBytes = 256;
extern int sweep_tc_k_tile;  // sources per pipeline stage: 32 (64-byte rows, default) or 64 (128-byte rows)
extern int sweep_tc_multicast;  // 1: clusters of two CTAs sharing the weight tile by multicast; 0 (default): single CTAs
int launch_sweep_tc(const void* network, const void* weights, int64_t n_src, int64_t n_snk, int64_t ld,
                    int64_t n_beams, bool bf16, float* out, int64_t ldc, cudaStream_t stream);

// Grid build (lyem_grid.cu).
cudaError_t launch_tris_bounds(const float4* tris, long long n_tris, float* bounds6, cudaStream_t stream);

}  // namespace lyem
