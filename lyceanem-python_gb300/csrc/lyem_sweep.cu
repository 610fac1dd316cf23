// lyem_sweep.cu -- beam sweeps over a formed propagation network.
//
// Once the per-pair network G[n, m, c] of a scene is formed (pair stage,
// complex64 [N, M, 3]), the sink fields of K excitation vectors W[k, n] are
//     E[m, k, c] = sum_n G[n, m, c] W[k, n]
// three complex GEMMs (M x N) x (N x K), i.e. 8 M N K real flops per component.
// This replaces the reference's per-excitation re-run of the whole model
// (lyceanem/models/frequency_domain.py:858-921) and its host GEMMs
// (lyceanem/models/frequency_domain.py:258-260).
//
// Modes:
//   0  plain complex64 FP32 (cublasCgemm), the comparison path;
//   3  BF16 split on the tensor cores: each real operand x = hi + lo with
//      hi = bf16(x), lo = bf16(x - hi); the complex product from three real
//      products (Gauss: Gr Wr, Gi Wi, (Gr + Gi)(Wr + Wi)), each as
//      hi*hi + lo*hi + hi*lo with FP32 accumulation (lyem_sweep_tc.cu);
//   4  the same with FP16 halves, after a power-of-two scaling of the network
//      (per component) and of the weights that puts their largest magnitude at
//      2^14, so that no half overflows and few are subnormal.
// Modes 3 and 4 read K-major operand planes written here (sources contiguous):
// a 256-byte header (the scales) followed by 18 network planes [ld][kpad] or 6
// weight planes [n_beams][kpad], kpad = n_src rounded up to a multiple of 8.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "lyem.h"
#include "lyem_internal.cuh"

namespace lyem {

template <typename T>
__device__ __forceinline__ T to_lp(float x);
template <>
__device__ __forceinline__ __nv_bfloat16 to_lp<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <>
__device__ __forceinline__ __half to_lp<__half>(float x) { return __float2half_rn(x); }
template <typename T>
__device__ __forceinline__ float from_lp(T x);
template <>
__device__ __forceinline__ float from_lp<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }
template <>
__device__ __forceinline__ float from_lp<__half>(__half x) { return __half2float(x); }

// Largest |Gr|, |Gi|, |Gr + Gi| per component of the network [N][M][3]
// (max_bits[c], float bits: non-negative floats order as their bit patterns).
__global__ void network_maxabs_kernel(const float2* __restrict__ pairs, long long n_pairs,
                                      unsigned int* __restrict__ max_bits) {
    float mx[3] = {0.f, 0.f, 0.f};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_pairs;
         i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 g = pairs[3 * i + c];
            mx[c] = fmaxf(mx[c], fmaxf(fmaxf(fabsf(g.x), fabsf(g.y)), fabsf(__fadd_rn(g.x, g.y))));
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float v = mx[c];
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31) == 0 && v > 0.f) atomicMax(max_bits + c, __float_as_uint(v));
    }
}

// Largest |Wr|, |Wi|, |Wr + Wi| of the weights [K][N] (max_bits[0]).
__global__ void weights_maxabs_kernel(const float2* __restrict__ W, long long n, unsigned int* __restrict__ max_bits) {
    float mx = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 w = W[i];
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(w.x), fabsf(w.y)), fabsf(__fadd_rn(w.x, w.y))));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(max_bits, __float_as_uint(mx));
}

// Header floats [0, n): the scales 2^(14 - e) with max < 2^e (FP16), or 1 (BF16).
__global__ void sweep_scales_kernel(float* __restrict__ hdr, int n, int unit) {
    const int i = threadIdx.x;
    if (i >= n) return;
    const float mx = __uint_as_float(reinterpret_cast<const unsigned int*>(hdr)[4 + i]);
    float s = 1.f;
    if (!unit && mx > 0.f && isfinite(mx)) {
        int e = 0;
        frexpf(mx, &e);  // mx = f 2^e, 0.5 <= f < 1
        s = ldexpf(1.f, 14 - e);
    }
    hdr[i] = s;
}

// hi and lo halves of x (already scaled) as 16-bit bit patterns.
template <typename T>
__device__ __forceinline__ void split16(float x, unsigned short& hi, unsigned short& lo) {
    const T h = to_lp<T>(x);
    const T l = to_lp<T>(__fsub_rn(x, from_lp<T>(h)));
    hi = *reinterpret_cast<const unsigned short*>(&h);
    lo = *reinterpret_cast<const unsigned short*>(&l);
}

// Network [N][M][3] complex64 -> 18 K-major planes [ld][kpad] (plane (3 c + q) 2 + h for component c,
// part q in (r, i, s = r + i), half h), scaled by hdr[c].  A block transposes a tile of 32 sinks x 32
// sources through shared memory: loads run along the sinks, stores along the sources.
template <typename T>
__global__ void __launch_bounds__(256) split_network_kmajor_kernel(const float2* __restrict__ pairs, long long N,
                                                                   long long M, long long ld, long long kpad,
                                                                   const float* __restrict__ hdr,
                                                                   unsigned short* __restrict__ planes) {
    __shared__ float2 tile[3][32][33];
    const long long m0 = (long long)blockIdx.x * 32, n0 = (long long)blockIdx.y * 32;
    const int tid = threadIdx.x;
#pragma unroll
    for (int r = 0; r < 12; ++r) {  // 32 sources x 96 (sink, component) floats2, contiguous per source
        const int i = tid + 256 * r;
        const int n = i / 96, j = i - n * 96, m = j / 3, c = j - m * 3;
        float2 g = make_float2(0.f, 0.f);
        if (n0 + n < N && m0 + m < M) g = pairs[((n0 + n) * M + m0) * 3 + j];
        tile[c][n][m] = g;
    }
    __syncthreads();
    const float sc[3] = {hdr[0], hdr[1], hdr[2]};
    const long long plane = ld * kpad;
#pragma unroll
    for (int r = 0; r < 6; ++r) {  // 3 components x 32 sinks x 16 source pairs
        const int i = tid + 256 * r;
        const int np = i & 15, m = (i >> 4) & 31, c = i >> 9;
        const long long row = m0 + m, col = n0 + 2 * np;
        if (row >= ld || col >= kpad) continue;
        const float2 g0 = tile[c][2 * np][m], g1 = tile[c][2 * np + 1][m];
        const float p0[3] = {g0.x * sc[c], g0.y * sc[c], __fadd_rn(g0.x, g0.y) * sc[c]};
        const float p1[3] = {g1.x * sc[c], g1.y * sc[c], __fadd_rn(g1.x, g1.y) * sc[c]};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            unsigned short h0, l0, h1, l1;
            split16<T>(p0[q], h0, l0);
            split16<T>(p1[q], h1, l1);
            unsigned short* hp = planes + (long long)((c * 3 + q) * 2) * plane + row * kpad + col;
            *reinterpret_cast<unsigned int*>(hp) = (unsigned int)h0 | ((unsigned int)h1 << 16);
            *reinterpret_cast<unsigned int*>(hp + plane) = (unsigned int)l0 | ((unsigned int)l1 << 16);
        }
    }
}

// Weights W [K][N] complex64 -> 6 K-major planes [K][kpad] (plane 2 q + h), scaled by hdr[0].
template <typename T>
__global__ void split_weights_kmajor_kernel(const float2* __restrict__ W, long long N, long long K, long long kpad,
                                            const float* __restrict__ hdr, unsigned short* __restrict__ planes) {
    const float s = hdr[0];
    const long long plane = K * kpad;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < K * kpad;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / kpad, n = i - k * kpad;
        const float2 w = n < N ? W[k * N + n] : make_float2(0.f, 0.f);
        const float part[3] = {w.x * s, w.y * s, __fadd_rn(w.x, w.y) * s};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            unsigned short h, l;
            split16<T>(part[q], h, l);
            planes[(2 * q) * plane + i] = h;
            planes[(2 * q + 1) * plane + i] = l;
        }
    }
}

// Network -> complex64 column-major (ld x N) per component.
__global__ void complex_network_kernel(const float2* __restrict__ pairs, long long N, long long M, long long ld,
                                       float2* __restrict__ out) {
    const long long total = N * ld;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long n = i / ld, m = i - n * ld;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[(long long)c * N * ld + i] = m < M ? pairs[(n * M + m) * 3 + c] : make_float2(0.f, 0.f);
    }
}

namespace {
std::mutex g_cublas_mutex;
cublasHandle_t g_cublas[64] = {};

cublasHandle_t cublas_for_current_device(cudaStream_t stream, int* err) {
    int dev = 0;
    *err = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        *err = 1;
        return nullptr;
    }
    if (!g_cublas[dev]) {
        if (cublasCreate(&g_cublas[dev]) != CUBLAS_STATUS_SUCCESS) {
            *err = 1;
            return nullptr;
        }
    }
    if (cublasSetStream(g_cublas[dev], stream) != CUBLAS_STATUS_SUCCESS) *err = 1;
    return g_cublas[dev];
}

unsigned sweep_blocks(long long n) { return capped_blocks(n, 256, 32); }
}  // namespace

}  // namespace lyem

using namespace lyem;

extern "C" {

namespace {
bool split_mode(int32_t mode) { return mode == 3 || mode == 4; }
bool valid_mode(int32_t mode) { return mode == 0 || split_mode(mode); }
long long kpad_of(long long n_src) { return (n_src + 7) / 8 * 8; }
}  // namespace

LYEM_API size_t lyem_sweep_network_bytes(int64_t n_src, int64_t ld, int32_t mode) {
    if (n_src <= 0 || ld <= 0 || !valid_mode(mode)) return 0;
    if (mode == 0) return (size_t)3 * n_src * ld * 8;
    return kSweepHeaderBytes + (size_t)18 * ld * kpad_of(n_src) * 2;
}

LYEM_API size_t lyem_sweep_weights_bytes(int64_t n_src, int64_t n_beams, int32_t mode) {
    if (n_src <= 0 || n_beams <= 0 || !split_mode(mode)) return 0;
    return kSweepHeaderBytes + (size_t)6 * n_beams * kpad_of(n_src) * 2;
}

LYEM_API size_t lyem_sweep_workspace_bytes(int64_t ld, int64_t n_beams, int32_t mode) {
    (void)ld;
    (void)n_beams;
    (void)mode;
    return 0;  // the tensor-core kernel combines the three products in TMEM
}

LYEM_API int lyem_sweep_set_k_tile(int32_t k_tile) {
    if (k_tile != 32 && k_tile != 64) return LYEM_ERR_INVALID;
    sweep_tc_k_tile = k_tile;
    return LYEM_OK;
}

LYEM_API int lyem_sweep_set_multicast(int32_t on) {
    if (on != 0 && on != 1) return LYEM_ERR_INVALID;
    sweep_tc_multicast = on;
    return LYEM_OK;
}

LYEM_API int lyem_sweep_prepare_network(const float* d_pairs, int64_t n_src, int64_t n_snk, int32_t mode, int64_t ld,
                                        void* d_network, void* stream) {
    if (n_src < 0 || n_snk < 0 || !valid_mode(mode) || ld < n_snk || (ld & 7)) return LYEM_ERR_INVALID;
    if (n_src == 0 || n_snk == 0) return LYEM_OK;
    if (!d_pairs || !d_network || (reinterpret_cast<uintptr_t>(d_network) & 255)) return LYEM_ERR_INVALID;
    if (split_mode(mode) && (n_src > 0x7fffffffLL || ld > 0x7fffffffLL)) return LYEM_ERR_OVERFLOW;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const float2* P = reinterpret_cast<const float2*>(d_pairs);
    if (mode == 0) {
        complex_network_kernel<<<sweep_blocks(n_src * ld), 256, 0, s>>>(P, n_src, n_snk, ld,
                                                                      reinterpret_cast<float2*>(d_network));
        note_launches(1);
        return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
    }
    float* hdr = static_cast<float*>(d_network);
    unsigned short* planes = reinterpret_cast<unsigned short*>(static_cast<unsigned char*>(d_network) + kSweepHeaderBytes);
    if (cudaMemsetAsync(hdr, 0, 32, s) != cudaSuccess) return LYEM_ERR_CUDA;
    if (mode == 4) {
        network_maxabs_kernel<<<sweep_blocks(n_src * n_snk), 256, 0, s>>>(P, n_src * n_snk,
                                                                         reinterpret_cast<unsigned int*>(hdr) + 4);
        note_launches(1);
    }
    sweep_scales_kernel<<<1, 32, 0, s>>>(hdr, 3, mode == 3);
    const long long kpad = kpad_of(n_src);
    const dim3 grid((unsigned)((ld + 31) / 32), (unsigned)((kpad + 31) / 32));
    if (grid.y > 65535u) return LYEM_ERR_OVERFLOW;
    if (mode == 3)
        split_network_kmajor_kernel<__nv_bfloat16><<<grid, 256, 0, s>>>(P, n_src, n_snk, ld, kpad, hdr, planes);
    else
        split_network_kmajor_kernel<__half><<<grid, 256, 0, s>>>(P, n_src, n_snk, ld, kpad, hdr, planes);
    note_launches(2);
    return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
}

LYEM_API int lyem_sweep_prepare_weights(const float* d_W, int64_t n_src, int64_t n_beams, int32_t mode, void* d_B,
                                        void* stream) {
    if (n_src < 0 || n_beams < 0 || !valid_mode(mode)) return LYEM_ERR_INVALID;
    if (mode == 0 || n_src == 0 || n_beams == 0) return LYEM_OK;
    if (!d_W || !d_B || (reinterpret_cast<uintptr_t>(d_B) & 255)) return LYEM_ERR_INVALID;
    if (n_src > 0x7fffffffLL || n_beams > 0x7fffffffLL) return LYEM_ERR_OVERFLOW;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const float2* W = reinterpret_cast<const float2*>(d_W);
    float* hdr = static_cast<float*>(d_B);
    unsigned short* planes = reinterpret_cast<unsigned short*>(static_cast<unsigned char*>(d_B) + kSweepHeaderBytes);
    if (cudaMemsetAsync(hdr, 0, 32, s) != cudaSuccess) return LYEM_ERR_CUDA;
    if (mode == 4) {
        weights_maxabs_kernel<<<sweep_blocks(n_src * n_beams), 256, 0, s>>>(W, n_src * n_beams,
                                                                           reinterpret_cast<unsigned int*>(hdr) + 4);
        note_launches(1);
    }
    sweep_scales_kernel<<<1, 32, 0, s>>>(hdr, 1, mode == 3);
    const long long kpad = kpad_of(n_src);
    const unsigned b = sweep_blocks(n_beams * kpad);
    if (mode == 3)
        split_weights_kmajor_kernel<__nv_bfloat16><<<b, 256, 0, s>>>(W, n_src, n_beams, kpad, hdr, planes);
    else
        split_weights_kmajor_kernel<__half><<<b, 256, 0, s>>>(W, n_src, n_beams, kpad, hdr, planes);
    note_launches(2);
    return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
}

LYEM_API int lyem_sweep_run_ws(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                               const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* d_ws,
                               size_t ws_bytes, void* stream);

LYEM_API int lyem_sweep_run(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                            const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* stream) {
    return lyem_sweep_run_ws(d_network, n_src, n_snk, ld, d_W, d_B, n_beams, mode, d_out, ldc, nullptr, 0, stream);
}

LYEM_API int lyem_sweep_run_ws(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                               const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* d_ws,
                               size_t ws_bytes, void* stream) {
    (void)d_ws;
    (void)ws_bytes;
    if (n_src <= 0 || n_snk <= 0 || n_beams <= 0 || !valid_mode(mode) || ld < n_snk || ldc < ld)
        return LYEM_ERR_INVALID;
    if (!d_network || !d_out || (mode == 0 && !d_W) || (mode != 0 && !d_B)) return LYEM_ERR_INVALID;
    if (n_src > 0x7fffffffLL || ld > 0x7fffffffLL || n_beams > 0x7fffffffLL) return LYEM_ERR_OVERFLOW;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (split_mode(mode)) {
        if ((reinterpret_cast<uintptr_t>(d_network) & 255) || (reinterpret_cast<uintptr_t>(d_B) & 255) ||
            (reinterpret_cast<uintptr_t>(d_out) & 7))
            return LYEM_ERR_INVALID;
        return launch_sweep_tc(d_network, d_B, n_src, n_snk, ld, n_beams, mode == 3, d_out, ldc, s);
    }
    std::lock_guard<std::mutex> lock(g_cublas_mutex);
    int err = 0;
    cublasHandle_t h = cublas_for_current_device(s, &err);
    if (err) return LYEM_ERR_CUDA;
    const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
    for (int c = 0; c < 3; ++c) {
        const cuComplex* A = reinterpret_cast<const cuComplex*>(d_network) + (size_t)c * n_src * ld;
        // the operand rows past n_snk are zero padding: run the aligned row count
        const cublasStatus_t st =
            cublasCgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)ld, (int)n_beams, (int)n_src, &one, A, (int)ld,
                        reinterpret_cast<const cuComplex*>(d_W), (int)n_src, &zero,
                        reinterpret_cast<cuComplex*>(d_out) + (size_t)c * n_beams * ldc, (int)ldc);
        note_launches(1);
        if (st != CUBLAS_STATUS_SUCCESS) return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

}  // extern "C"
