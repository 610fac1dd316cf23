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
//   0  plain complex64 FP32: cublasCgemm on the complex matrices;
//   1  BF16 split: x = hi + lo with hi = bf16(x), lo = bf16(x - hi); the
//      product is hi*hi + hi*lo + lo*hi on the tensor cores with FP32
//      accumulation (lo*lo, ~2^-16 relative, is dropped);
//   2  FP16 split, same scheme with binary16 (11 + 11 significant bits).
//   3, 4  BF16 / FP16 split with the complex product in three real products
//      (Gauss): with G = Gr + j Gi and W = Wr + j Wi,
//        T1 = Gr Wr,  T2 = Gi Wi,  T3 = (Gr + Gi)(Wr + Wi),
//        Re E = T1 - T2,  Im E = T3 - T1 - T2,
//      each T a real (M x N)(N x K) GEMM of split operands (6 M N K flops per
//      component against 8 M N K), the sums Gr + Gi and Wr + Wi formed in FP32
//      before the split.  The three split products of one T run as two GEMMs:
//      [hi | lo] (M x 2N) times [hi ; hi] (2N x K), then hi times lo.
// For the split modes 1, 2 the complex product is one real GEMM in interleaved form:
//   A' = [G | jG] as a (2M x 2N) real column-major matrix (column n holds the
//   interleaved (re, im) of G[:, n]; column N + n holds j G[:, n] = (-im, re)),
//   B' = [Re W^T ; Im W^T] (2N x K),
// so C' = A' B' is (2M x K) real and, read as complex64 (M x K) column-major,
// is exactly E[:, :, c] in the layout cublasCgemm writes.
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

// Network [N][M][3] complex64 -> per component A' hi/lo planes, each
// (2 ld x 2N) column-major; rows past 2M are zero padding.
template <typename T>
__global__ void split_network_kernel(const float2* __restrict__ pairs, long long N, long long M, long long ld,
                                     float scale, T* __restrict__ out) {
    const long long plane = 2 * ld * 2 * N;  // elements of one (hi or lo) plane
    const long long total = N * ld;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long n = i / ld, m = i - n * ld;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float2 g = m < M ? pairs[(n * M + m) * 3 + c] : make_float2(0.f, 0.f);
            g.x *= scale;
            g.y *= scale;
            const T hr = to_lp<T>(g.x), hi_ = to_lp<T>(g.y);
            const T lr = to_lp<T>(g.x - from_lp<T>(hr)), li = to_lp<T>(g.y - from_lp<T>(hi_));
            T* hp = out + (long long)(2 * c) * plane;
            T* lp = hp + plane;
            const long long col = 2 * ld * n, colj = 2 * ld * (N + n);
            hp[col + 2 * m] = hr;
            hp[col + 2 * m + 1] = hi_;
            lp[col + 2 * m] = lr;
            lp[col + 2 * m + 1] = li;
            // j G = (-im, re)
            hp[colj + 2 * m] = to_lp<T>(-from_lp<T>(hi_));
            hp[colj + 2 * m + 1] = hr;
            lp[colj + 2 * m] = to_lp<T>(-from_lp<T>(li));
            lp[colj + 2 * m + 1] = lr;
        }
    }
}

// Network [N][M][3] -> per component six planes (ld x N, column-major, rows
// past M zero): Gr hi, Gr lo, Gi hi, Gi lo, Gs hi, Gs lo (Gs = Gr + Gi), so that
// each part's hi and lo planes form one (ld x 2N) matrix.
template <typename T>
__global__ void split_network_gauss_kernel(const float2* __restrict__ pairs, long long N, long long M, long long ld,
                                           T* __restrict__ out) {
    const long long plane = ld * N;
    const long long total = N * ld;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long n = i / ld, m = i - n * ld;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 g = m < M ? pairs[(n * M + m) * 3 + c] : make_float2(0.f, 0.f);
            const float part[3] = {g.x, g.y, __fadd_rn(g.x, g.y)};
            T* base = out + (long long)(6 * c) * plane;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const T h = to_lp<T>(part[q]);
                base[(2 * q) * plane + i] = h;
                base[(2 * q + 1) * plane + i] = to_lp<T>(part[q] - from_lp<T>(h));
            }
        }
    }
}

// Weights W [K][N] -> per part (r, i, s = r + i) a (2N x K) column-major
// [hi ; hi] matrix followed by a (N x K) lo matrix.
template <typename T>
__global__ void split_weights_gauss_kernel(const float2* __restrict__ W, long long N, long long K, T* __restrict__ out) {
    const long long part_elems = 3 * N * K;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N * K;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / N, n = i - k * N;
        const float2 w = W[i];
        const float part[3] = {w.x, w.y, __fadd_rn(w.x, w.y)};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            T* dup = out + q * part_elems;
            T* lo = dup + 2 * N * K;
            const T h = to_lp<T>(part[q]);
            dup[k * 2 * N + n] = h;
            dup[k * 2 * N + N + n] = h;
            lo[k * N + n] = to_lp<T>(part[q] - from_lp<T>(h));
        }
    }
}

// out (complex64, column-major ld x K with leading dimension ldc) from the three
// real products T1, T2, T3 (ld x K each, consecutive in t).
__global__ void gauss_combine_kernel(const float* __restrict__ t, long long ld, long long K, long long ldc,
                                     float2* __restrict__ out) {
    const long long n = ld * K;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float t1 = t[i], t2 = t[n + i], t3 = t[2 * n + i];
        const long long k = i / ld, m = i - k * ld;
        out[k * ldc + m] = make_float2(__fsub_rn(t1, t2), __fsub_rn(__fsub_rn(t3, t1), t2));
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

// Weights W [K][N] complex64 -> B' hi/lo planes (2N x K) column-major.
template <typename T>
__global__ void split_weights_kernel(const float2* __restrict__ W, long long N, long long K, T* __restrict__ out) {
    const long long plane = 2 * N * K;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N * K;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / N, n = i - k * N;
        const float2 w = W[i];
        const T hr = to_lp<T>(w.x), hi_ = to_lp<T>(w.y);
        out[k * 2 * N + n] = hr;
        out[k * 2 * N + N + n] = hi_;
        out[plane + k * 2 * N + n] = to_lp<T>(w.x - from_lp<T>(hr));
        out[plane + k * 2 * N + N + n] = to_lp<T>(w.y - from_lp<T>(hi_));
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

LYEM_API size_t lyem_sweep_network_bytes(int64_t n_src, int64_t ld, int32_t mode) {
    if (n_src <= 0 || ld <= 0) return 0;
    if (mode == 0) return (size_t)3 * n_src * ld * 8;
    if (mode >= 3) return (size_t)3 * 6 * ld * n_src * 2;
    return (size_t)3 * 2 * (2 * ld) * (2 * n_src) * 2;
}

LYEM_API size_t lyem_sweep_weights_bytes(int64_t n_src, int64_t n_beams, int32_t mode) {
    if (n_src <= 0 || n_beams <= 0 || mode == 0) return 0;
    if (mode >= 3) return (size_t)3 * 3 * n_src * n_beams * 2;
    return (size_t)2 * (2 * n_src) * n_beams * 2;
}

LYEM_API size_t lyem_sweep_workspace_bytes(int64_t ld, int64_t n_beams, int32_t mode) {
    if (ld <= 0 || n_beams <= 0 || mode < 3) return 0;
    return (size_t)3 * ld * n_beams * 4;
}

LYEM_API int lyem_sweep_prepare_network(const float* d_pairs, int64_t n_src, int64_t n_snk, int32_t mode, int64_t ld,
                                        void* d_network, void* stream) {
    if (n_src < 0 || n_snk < 0 || mode < 0 || mode > 4 || ld < n_snk || (ld & 7)) return LYEM_ERR_INVALID;
    if (n_src == 0 || n_snk == 0) return LYEM_OK;
    if (!d_pairs || !d_network) return LYEM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const float2* P = reinterpret_cast<const float2*>(d_pairs);
    const unsigned b = sweep_blocks(n_src * ld);
    if (mode == 0)
        complex_network_kernel<<<b, 256, 0, s>>>(P, n_src, n_snk, ld, reinterpret_cast<float2*>(d_network));
    else if (mode == 1)
        split_network_kernel<__nv_bfloat16><<<b, 256, 0, s>>>(P, n_src, n_snk, ld, 1.f,
                                                             reinterpret_cast<__nv_bfloat16*>(d_network));
    else if (mode == 3)
        split_network_gauss_kernel<__nv_bfloat16><<<b, 256, 0, s>>>(P, n_src, n_snk, ld,
                                                                   reinterpret_cast<__nv_bfloat16*>(d_network));
    else if (mode == 4)
        split_network_gauss_kernel<__half><<<b, 256, 0, s>>>(P, n_src, n_snk, ld, reinterpret_cast<__half*>(d_network));
    else
        split_network_kernel<__half><<<b, 256, 0, s>>>(P, n_src, n_snk, ld, 1.f, reinterpret_cast<__half*>(d_network));
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
}

LYEM_API int lyem_sweep_prepare_weights(const float* d_W, int64_t n_src, int64_t n_beams, int32_t mode, void* d_B,
                                        void* stream) {
    if (n_src < 0 || n_beams < 0 || mode < 0 || mode > 4) return LYEM_ERR_INVALID;
    if (mode == 0 || n_src == 0 || n_beams == 0) return LYEM_OK;
    if (!d_W || !d_B) return LYEM_ERR_INVALID;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const float2* W = reinterpret_cast<const float2*>(d_W);
    const unsigned b = sweep_blocks(n_src * n_beams);
    if (mode == 1)
        split_weights_kernel<__nv_bfloat16><<<b, 256, 0, s>>>(W, n_src, n_beams, reinterpret_cast<__nv_bfloat16*>(d_B));
    else if (mode == 2)
        split_weights_kernel<__half><<<b, 256, 0, s>>>(W, n_src, n_beams, reinterpret_cast<__half*>(d_B));
    else if (mode == 3)
        split_weights_gauss_kernel<__nv_bfloat16><<<b, 256, 0, s>>>(W, n_src, n_beams,
                                                                   reinterpret_cast<__nv_bfloat16*>(d_B));
    else
        split_weights_gauss_kernel<__half><<<b, 256, 0, s>>>(W, n_src, n_beams, reinterpret_cast<__half*>(d_B));
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
}

LYEM_API int lyem_sweep_run_ws(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                               const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* d_ws,
                               size_t ws_bytes, void* stream);

LYEM_API int lyem_sweep_run(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                            const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* stream) {
    if (mode > 2) return LYEM_ERR_INVALID;  // the three-product modes need lyem_sweep_run_ws
    return lyem_sweep_run_ws(d_network, n_src, n_snk, ld, d_W, d_B, n_beams, mode, d_out, ldc, nullptr, 0, stream);
}

LYEM_API int lyem_sweep_run_ws(const void* d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float* d_W,
                               const void* d_B, int64_t n_beams, int32_t mode, float* d_out, int64_t ldc, void* d_ws,
                               size_t ws_bytes, void* stream) {
    if (n_src <= 0 || n_snk <= 0 || n_beams <= 0 || mode < 0 || mode > 4 || ld < n_snk || ldc < ld)
        return LYEM_ERR_INVALID;
    if (mode >= 3 && (!d_ws || ws_bytes < lyem_sweep_workspace_bytes(ld, n_beams, mode))) return LYEM_ERR_WORKSPACE;
    if (!d_network || !d_out || (mode == 0 && !d_W) || (mode != 0 && !d_B)) return LYEM_ERR_INVALID;
    if (n_src > 0x7fffffffLL / 2 || 2 * ld > 0x7fffffffLL || n_beams > 0x7fffffffLL) return LYEM_ERR_OVERFLOW;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(g_cublas_mutex);
    int err = 0;
    cublasHandle_t h = cublas_for_current_device(s, &err);
    if (err) return LYEM_ERR_CUDA;
    for (int c = 0; c < 3; ++c) {
        cublasStatus_t st = CUBLAS_STATUS_SUCCESS;
        if (mode >= 3) {
            const cudaDataType_t dt = mode == 3 ? CUDA_R_16BF : CUDA_R_16F;
            const size_t plane = (size_t)ld * n_src;
            const size_t part_b = (size_t)3 * n_src * n_beams;
            float* T = static_cast<float*>(d_ws);
            const float one = 1.f, zero = 0.f;
            const int m = (int)ld, n = (int)n_beams, k = (int)n_src;
            for (int q = 0; q < 3 && st == CUBLAS_STATUS_SUCCESS; ++q) {
                const unsigned short* Ahi = reinterpret_cast<const unsigned short*>(d_network) + (6 * c + 2 * q) * plane;
                const unsigned short* Bdup = reinterpret_cast<const unsigned short*>(d_B) + q * part_b;
                const unsigned short* Blo = Bdup + (size_t)2 * n_src * n_beams;
                float* C = T + (size_t)q * ld * n_beams;
                // [hi | lo] x [hi ; hi] = hi*hi + lo*hi, then += hi*lo
                st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, 2 * k, &one, Ahi, dt, m, Bdup, dt, 2 * k, &zero,
                                  C, CUDA_R_32F, m, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
                if (st == CUBLAS_STATUS_SUCCESS)
                    st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, Ahi, dt, m, Blo, dt, k, &one, C,
                                      CUDA_R_32F, m, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
                note_launches(2);
            }
            if (st == CUBLAS_STATUS_SUCCESS) {
                gauss_combine_kernel<<<sweep_blocks(ld * n_beams), 256, 0, s>>>(
                    T, ld, n_beams, ldc, reinterpret_cast<float2*>(d_out) + (size_t)c * n_beams * ldc);
                note_launches(1);
                if (cudaGetLastError() != cudaSuccess) return LYEM_ERR_CUDA;
            }
        } else if (mode == 0) {
            const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
            const cuComplex* A = reinterpret_cast<const cuComplex*>(d_network) + (size_t)c * n_src * ld;
            // the operand rows past n_snk are zero padding: run the aligned row count
            st = cublasCgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)ld, (int)n_beams, (int)n_src, &one, A, (int)ld,
                             reinterpret_cast<const cuComplex*>(d_W), (int)n_src, &zero,
                             reinterpret_cast<cuComplex*>(d_out) + (size_t)c * n_beams * ldc, (int)ldc);
            note_launches(1);
        } else {
            const cudaDataType_t dt = mode == 1 ? CUDA_R_16BF : CUDA_R_16F;
            const size_t plane = (size_t)(2 * ld) * (2 * n_src);
            const unsigned short* A = reinterpret_cast<const unsigned short*>(d_network) + (size_t)(2 * c) * plane;
            const unsigned short* Alo = A + plane;
            const unsigned short* B = reinterpret_cast<const unsigned short*>(d_B);
            const unsigned short* Blo = B + (size_t)(2 * n_src) * n_beams;
            float* C = d_out + (size_t)c * n_beams * 2 * ldc;
            const float one = 1.f, zero = 0.f;
            const int m = (int)(2 * ld), n = (int)n_beams, k = (int)(2 * n_src);  // padded rows are zero
            const int lda = (int)(2 * ld), ldb = (int)(2 * n_src), ldo = (int)(2 * ldc);
            st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A, dt, lda, B, dt, ldb, &zero, C,
                              CUDA_R_32F, ldo, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
            if (st == CUBLAS_STATUS_SUCCESS)
                st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A, dt, lda, Blo, dt, ldb, &one, C,
                                  CUDA_R_32F, ldo, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
            if (st == CUBLAS_STATUS_SUCCESS)
                st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, Alo, dt, lda, B, dt, ldb, &one, C,
                                  CUDA_R_32F, ldo, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
            note_launches(3);
        }
        if (st != CUBLAS_STATUS_SUCCESS) return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

}  // extern "C"
