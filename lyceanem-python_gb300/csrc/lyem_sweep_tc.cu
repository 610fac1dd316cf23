// lyem_sweep_tc.cu -- the beam-sweep contraction on the tensor cores (tcgen05).
//
// E[m, k, c] = sum_n G[n, m, c] W[k, n] for the three components c, with the
// complex product formed from three real products (Gauss):
//     T1 = Gr Wr,  T2 = Gi Wi,  T3 = Gs Ws   (Gs = Gr + Gi, Ws = Wr + Wi)
//     Re E = T1 - T2,  Im E = T3 - T1 - T2,
// and every real operand split as x = hi + lo in BF16 or FP16, each real
// product accumulated in FP32 as hi*hi + lo*hi + hi*lo (lo*lo, about 2^-16
// relative for BF16, is dropped).  This replaces the reference's per-excitation
// re-run of the model (lyceanem/models/frequency_domain.py:858-921) and its
// host GEMMs (lyceanem/models/frequency_domain.py:258-260).
//
// Operands (written by lyem_sweep_prepare_network / _weights) are K-major
// (sources contiguous): 18 network planes [rows = sinks][sources] (component c,
// part q in (r, i, s), hi / lo at plane (3 c + q) 2 + h) and 6 weight planes
// [beams][sources] (part q, hi / lo at plane 2 q + h).  FP16 operands carry a
// power-of-two scale per network component and one for the weights (chosen
// from the largest magnitude so that no hi or lo overflows and few are
// subnormal); the epilogue divides it out exactly.
//
// Kernel: persistent, one CTA of 192 threads per SM; a tile is 128 sinks x 256
// beams of one component.  Warp 0 issues TMA loads of [A hi | A lo | B hi | B lo]
// k-blocks into a ring of shared-memory stages; warp 1 owns the 512 TMEM
// columns and issues the MMAs (M 128, N 256, K 16 per instruction) from one
// thread; warps 2-5 (one TMEM lane quadrant each) run the epilogue.  A tile
// runs three passes over the sources: q = r into accumulator 0 (T1), q = i into
// accumulator 1 (T2); then the epilogue rewrites accumulator 0 as T1 - T2 (Re)
// and accumulator 1 as -(T1 + T2), and pass q = s accumulates T3 onto it (Im).
// Re is written out while pass s runs; Im while the next tile's first pass
// runs, so the tensor pipe waits only for the in-TMEM rewrite.  Every wait is
// bounded: on expiry the kernel sets bit 0 of the device error word, drains
// its copies and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "lyem.h"
#include "lyem_device.cuh"
#include "lyem_internal.cuh"
#include "lyem_tc.cuh"

namespace lyem {
namespace {

constexpr int kBM = 128;         // sinks per tile: TMEM lanes
constexpr int kBN = 256;         // beams per tile: columns of one accumulator
constexpr int kTcThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2-5 epilogue
constexpr int kTmemCols = 512;   // two accumulators of kBN FP32 columns

template <int BK>
struct TcCfg {
    static constexpr int kRowBytes = BK * 2;                      // one swizzled operand row
    static constexpr int kStages = BK == 64 ? 2 : 4;
    static constexpr int kABytes = kBM * BK * 2;                  // one network tile (hi or lo)
    static constexpr int kBBytes = kBN * BK * 2;                  // one weight tile (hi or lo)
    static constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes;
    static constexpr int kKSteps = BK / 16;                       // MMAs per operand pair and stage
    static constexpr int kBarriers = 2 * kStages + 6;
    static constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024 + 8 * kBarriers + 16;
};

struct TcParams {
    int n_src, n_snk, n_beams;
    int n_mt, n_kt, n_kb;
    long long ldc;
    float* out;              // complex64 [3][n_beams][ldc] as floats
    const float* scale_a;    // [3] per-component network scales
    const float* scale_w;    // [1] weight scale
    unsigned int* err;       // device error word
};

// MC: CTAs run in clusters of two that take the row tiles 2 i and 2 i + 1 of one
// beam tile; each loads half of the shared weight tile and multicasts it to both,
// so each SM requests 2/3 of the operand bytes of a stage, and a stage is
// refilled only after both CTAs' MMAs have read it (its empty barrier counts an
// arrival from each).
template <int BK, bool BF16, bool MC>
__global__ void __launch_bounds__(kTcThreads, 1)
    sweep_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const TcParams p) {
    using C = TcCfg<BK>;
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // swizzled tiles need 1024-byte alignment
    unsigned char* sm = smem_raw + (base - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + (size_t)C::kStages * C::kStageBytes);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + C::kBarriers);
    volatile int* s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
    constexpr int FULL = 0, EMPTY = C::kStages, MID_FULL = 2 * C::kStages, MID_DONE = MID_FULL + 1,
                  ACC_FULL = MID_FULL + 2, ACC0_EMPTY = MID_FULL + 3, ACC1_EMPTY = MID_FULL + 4,
                  DRAIN = MID_FULL + 5;
    auto bar = [&](int i) { return smem_addr(bars + i); };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::kStages; ++s) {
            mbar_init(bar(FULL + s), 1);
            mbar_init(bar(EMPTY + s), MC ? 2 : 1);
        }
        mbar_init(bar(MID_FULL), 1);
        mbar_init(bar(MID_DONE), 4);
        mbar_init(bar(ACC_FULL), 1);
        mbar_init(bar(ACC0_EMPTY), 4);
        mbar_init(bar(ACC1_EMPTY), 4);
        mbar_init(bar(DRAIN), 1);
        *s_abort = 0;
        fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(smem_addr(s_tmem), kTmemCols);
    tc::fence_before();
    if (MC)
        tc::cluster_sync();  // the peer's multicast copies and commits may target these barriers from now on
    else
        __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *s_tmem;
    // tile t -> (component, row tile, beam tile); with MC a cluster takes tile t and the CTA of rank r its row
    // tile 2 mt + r (past the last row tile for an odd count: zero rows, nothing stored)
    const int rank = MC ? (int)tc::cluster_ctarank() : 0;
    const int first = MC ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int step = MC ? (int)(gridDim.x >> 1) : (int)gridDim.x;
    const int n_rt = MC ? (p.n_mt + 1) / 2 : p.n_mt;
    const int tiles = 3 * n_rt * p.n_kt;
    auto decode = [&](int t, int& c, int& mt, int& kt) {
        c = t / (n_rt * p.n_kt);
        const int rem = t - c * (n_rt * p.n_kt);
        mt = rem / p.n_kt;
        kt = rem - mt * p.n_kt;
        if (MC) mt = 2 * mt + rank;
    };

    // Bounded wait; gives up early once another role has given up.
    auto wait = [&](uint32_t b, uint32_t parity) -> bool {
        const long long t0 = clock64();
        while (!tc::mbar_try(b, parity)) {
            if (*s_abort) return false;
            if (clock64() - t0 > kWaitCycles) {
                *s_abort = 1;
                atomicOr(p.err, 1u);
                return false;
            }
        }
        return true;
    };
    // Bounded wait that ignores the abort flag (draining copies and MMAs in flight).
    auto drain = [&](uint32_t b, uint32_t parity) {
        const long long t0 = clock64();
        while (!tc::mbar_try(b, parity)) {
            if (clock64() - t0 > kWaitCycles) {
                atomicOr(p.err, 1u);
                return;
            }
        }
    };

    if (warp == 0) {
        if (lane == 0) {  // TMA producer
            int s = 0;
            uint32_t ph = 0, last_par[C::kStages];
            bool issued[C::kStages];
            for (int i = 0; i < C::kStages; ++i) issued[i] = false;
            bool ok = true;
            for (int t = first; ok && t < tiles; t += step) {
                int c, mt, kt;
                decode(t, c, mt, kt);
                for (int q = 0; ok && q < 3; ++q) {
                    for (int kb = 0; kb < p.n_kb; ++kb) {
                        if (!wait(bar(EMPTY + s), ph ^ 1u)) {
                            ok = false;
                            break;
                        }
                        const uint32_t st = base + (uint32_t)s * C::kStageBytes;
                        const uint32_t fb = bar(FULL + s);
                        tc::mbar_expect_tx(fb, C::kStageBytes);
                        const int x = kb * BK, pa = (c * 3 + q) * 2;
                        tc::tma_load_3d(st, &tmA, x, mt * kBM, pa, fb);
                        tc::tma_load_3d(st + C::kABytes, &tmA, x, mt * kBM, pa + 1, fb);
                        if (MC) {  // this CTA's half of the weight rows, into both CTAs
                            const uint32_t half = (uint32_t)rank * (C::kBBytes / 2);
                            const int y = kt * kBN + rank * (kBN / 2);
                            tc::tma_load_3d_mc(st + 2 * C::kABytes + half, &tmB, x, y, 2 * q, fb, 0x3);
                            tc::tma_load_3d_mc(st + 2 * C::kABytes + C::kBBytes + half, &tmB, x, y, 2 * q + 1, fb,
                                               0x3);
                        } else {
                            tc::tma_load_3d(st + 2 * C::kABytes, &tmB, x, kt * kBN, 2 * q, fb);
                            tc::tma_load_3d(st + 2 * C::kABytes + C::kBBytes, &tmB, x, kt * kBN, 2 * q + 1, fb);
                        }
                        issued[s] = true;
                        last_par[s] = ph;
                        if (++s == C::kStages) {
                            s = 0;
                            ph ^= 1u;
                        }
                    }
                }
            }
            for (int i = 0; i < C::kStages; ++i)
                if (issued[i]) drain(bar(FULL + i), last_par[i]);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            constexpr uint32_t idesc = tc::idesc_f16(BF16, kBM, kBN);
            int s = 0, it = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int t = first; ok && t < tiles; t += step, ++it) {
                for (int q = 0; ok && q < 3; ++q) {
                    const uint32_t acc = tmem + (q == 0 ? 0u : (uint32_t)kBN);
                    bool w = true;
                    if (q == 0 && it > 0) w = wait(bar(ACC0_EMPTY), (uint32_t)(it - 1) & 1u);
                    if (q == 1 && it > 0) w = wait(bar(ACC1_EMPTY), (uint32_t)(it - 1) & 1u);
                    if (q == 2) w = wait(bar(MID_DONE), (uint32_t)it & 1u);
                    if (!w) {
                        ok = false;
                        break;
                    }
                    tc::fence_after();
                    for (int kb = 0; kb < p.n_kb; ++kb) {
                        if (!wait(bar(FULL + s), ph)) {
                            ok = false;
                            break;
                        }
                        tc::fence_after();
                        const uint32_t st = base + (uint32_t)s * C::kStageBytes;
#pragma unroll
                        for (int kk = 0; kk < C::kKSteps; ++kk) {
                            const uint32_t off = (uint32_t)kk * 32u;  // 16 elements of 2 bytes
                            const uint64_t ah = tc::smem_desc(st + off, C::kRowBytes);
                            const uint64_t al = tc::smem_desc(st + C::kABytes + off, C::kRowBytes);
                            const uint64_t bh = tc::smem_desc(st + 2 * C::kABytes + off, C::kRowBytes);
                            const uint64_t bl = tc::smem_desc(st + 2 * C::kABytes + C::kBBytes + off, C::kRowBytes);
                            const uint32_t first = (q < 2 && kb == 0 && kk == 0) ? 0u : 1u;
                            // hi*hi and hi*lo share A hi: it is read from shared memory once
                            tc::mma_f16_fill_a(acc, ah, bh, idesc, first);
                            tc::mma_f16_lastuse_a(acc, ah, bl, idesc, 1u);
                            tc::mma_f16(acc, al, bh, idesc, 1u);
                        }
                        // the stage is free once these MMAs (and, with MC, the peer's) complete
                        if (MC)
                            tc::commit_mc(bar(EMPTY + s), 0x3);
                        else
                            tc::commit(bar(EMPTY + s));
                        if (++s == C::kStages) {
                            s = 0;
                            ph ^= 1u;
                        }
                    }
                    if (ok && q == 1) tc::commit(bar(MID_FULL));
                    if (ok && q == 2) tc::commit(bar(ACC_FULL));
                }
            }
            tc::commit(bar(DRAIN));
            drain(bar(DRAIN), 0);
        }
    } else {  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31, one sink row per thread
        const int quad = warp & 3;
        const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
        const unsigned full = 0xffffffffu;
        auto wait_warp = [&](uint32_t b, uint32_t parity) -> bool {
            bool r = false;
            if (lane == 0) r = wait(b, parity);
            return __shfl_sync(full, r ? 1 : 0, 0) != 0;
        };
        auto signal = [&](uint32_t b) {
            tc::fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(b);
        };
        int it = 0;
        for (int t = first; t < tiles; t += step, ++it) {
            int c, mt, kt;
            decode(t, c, mt, kt);
            const long long m = (long long)mt * kBM + quad * 32 + lane;
            const float inv = 1.0f / (p.scale_a[c] * p.scale_w[0]);  // powers of two: exact
            float* out = p.out + (size_t)c * p.n_beams * p.ldc * 2;
            auto write_part = [&](uint32_t col0, int part) {
#pragma unroll 1
                for (int j = 0; j < kBN / 32; ++j) {
                    float v[32];
                    __syncwarp();  // tcgen05.ld is a .sync.aligned warp instruction
                    tc::tmem_ld32(tmem + lane_off + col0 + (uint32_t)j * 32u, v);
                    if (m < p.n_snk) {
#pragma unroll
                        for (int i = 0; i < 32; ++i) {
                            const long long k = (long long)kt * kBN + j * 32 + i;
                            if (k < p.n_beams) out[(k * p.ldc + m) * 2 + part] = v[i] * inv;
                        }
                    }
                }
            };
            // accumulators hold T1, T2: rewrite them as Re = T1 - T2 and -(T1 + T2)
            if (!wait_warp(bar(MID_FULL), (uint32_t)it & 1u)) break;
            tc::fence_after();
#pragma unroll 1
            for (int j = 0; j < kBN / 32; ++j) {
                float a[32], b[32];
                const uint32_t ta = tmem + lane_off + (uint32_t)j * 32u, tb = ta + (uint32_t)kBN;
                __syncwarp();
                tc::tmem_ld32x2(ta, tb, a, b);
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float t1 = a[i], t2 = b[i];
                    a[i] = __fsub_rn(t1, t2);
                    b[i] = -__fadd_rn(t1, t2);
                }
                tc::tmem_st32(ta, a);
                tc::tmem_st32(tb, b);
            }
            __syncwarp();
            tc::tmem_wait_st();
            signal(bar(MID_DONE));  // pass s may now accumulate T3 onto -(T1 + T2)
            write_part(0u, 0);
            signal(bar(ACC0_EMPTY));
            if (!wait_warp(bar(ACC_FULL), (uint32_t)it & 1u)) break;
            tc::fence_after();
            write_part((uint32_t)kBN, 1);
            signal(bar(ACC1_EMPTY));
        }
    }
    tc::fence_before();
    if (MC)
        tc::cluster_sync();  // neither CTA leaves while the other may still copy into or arrive on it
    else
        __syncthreads();
    if (warp == 1) {
        __syncwarp();  // dealloc is a .sync.aligned warp instruction
        tc::fence_after();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's tensor-map encoder, fetched through the runtime (no link to libcuda).
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(f);
    });
    return fn;
}

// 3-D K-major operand map: [planes][rows][k] 16-bit elements, row stride kpad elements.
bool make_map(CUtensorMap* m, const void* base, bool bf16, int k, int rows, int planes, long long kpad,
              long long rows_stride, int box_k, int box_rows) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)rows_stride * kpad * 2};
    const cuuint32_t box[3] = {(cuuint32_t)box_k, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapSwizzle swz = box_k * 2 == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    return enc(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3,
               const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BK, bool BF16, bool MC>
cudaError_t launch_tc(const CUtensorMap& a, const CUtensorMap& b, const TcParams& p, cudaStream_t stream,
                      bool* launched) {
    using C = TcCfg<BK>;
    auto kern = sweep_tc_kernel<BK, BF16, MC>;
    *launched = false;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::kSmem);
    if (e != cudaSuccess) return e;
    const int sms = device_sm_count();
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = C::kSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    if (MC) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const int tiles = 3 * ((p.n_mt + 1) / 2) * p.n_kt;
        cfg.gridDim = dim3(2 * sms);  // the occupancy query needs a grid shape
        int clusters = 0;
        e = cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg);
        if (e != cudaSuccess || clusters < 1) {
            (void)cudaGetLastError();
            return cudaSuccess;  // no co-resident pair: the caller uses the single-CTA kernel
        }
        cfg.gridDim = dim3(2 * (unsigned)(tiles < clusters ? tiles : clusters));
    } else {
        const int tiles = 3 * p.n_mt * p.n_kt;
        cfg.gridDim = dim3((unsigned)(tiles < sms ? tiles : sms));
    }
    e = cudaLaunchKernelEx(&cfg, kern, a, b, p);
    if (e != cudaSuccess) return e;
    *launched = true;
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace

int sweep_tc_k_tile = 32;
int sweep_tc_multicast = 0;

int launch_sweep_tc(const void* network, const void* weights, int64_t n_src, int64_t n_snk, int64_t ld,
                    int64_t n_beams, bool bf16, float* out, int64_t ldc, cudaStream_t stream) {
    const int bk = sweep_tc_k_tile;
    const long long kpad = (n_src + 7) / 8 * 8;
    const unsigned char* na = static_cast<const unsigned char*>(network);
    const unsigned char* wb = static_cast<const unsigned char*>(weights);
    CUtensorMap ma, mb, mb_half;
    if (!make_map(&ma, na + kSweepHeaderBytes, bf16, (int)n_src, (int)n_snk, 18, kpad, ld, bk, kBM) ||
        !make_map(&mb, wb + kSweepHeaderBytes, bf16, (int)n_src, (int)n_beams, 6, kpad, n_beams, bk, kBN) ||
        !make_map(&mb_half, wb + kSweepHeaderBytes, bf16, (int)n_src, (int)n_beams, 6, kpad, n_beams, bk, kBN / 2))
        return LYEM_ERR_CUDA;
    TcParams p;
    p.n_src = (int)n_src;
    p.n_snk = (int)n_snk;
    p.n_beams = (int)n_beams;
    p.n_mt = (int)((n_snk + kBM - 1) / kBM);
    p.n_kt = (int)((n_beams + kBN - 1) / kBN);
    p.n_kb = (int)((n_src + bk - 1) / bk);
    p.ldc = ldc;
    p.out = out;
    p.scale_a = reinterpret_cast<const float*>(na);
    p.scale_w = reinterpret_cast<const float*>(wb);
    p.err = device_error_word();
    if (!p.err) return LYEM_ERR_CUDA;
    cudaError_t e = cudaSuccess;
    bool done = false;
    if (sweep_tc_multicast) {  // clusters of two sharing the weight tile; the single-CTA kernel if none fit
        if (bk == 64)
            e = bf16 ? launch_tc<64, true, true>(ma, mb_half, p, stream, &done)
                     : launch_tc<64, false, true>(ma, mb_half, p, stream, &done);
        else
            e = bf16 ? launch_tc<32, true, true>(ma, mb_half, p, stream, &done)
                     : launch_tc<32, false, true>(ma, mb_half, p, stream, &done);
    }
    if (e == cudaSuccess && !done) {
        if (bk == 64)
            e = bf16 ? launch_tc<64, true, false>(ma, mb, p, stream, &done)
                     : launch_tc<64, false, false>(ma, mb, p, stream, &done);
        else
            e = bf16 ? launch_tc<32, true, false>(ma, mb, p, stream, &done)
                     : launch_tc<32, false, false>(ma, mb, p, stream, &done);
    }
    if (e != cudaSuccess) {
        record_cuda_error(e);
        return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

}  // namespace lyem
