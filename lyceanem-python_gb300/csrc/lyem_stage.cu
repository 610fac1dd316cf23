// lyem_stage.cu -- visibility + fused field kernels ("pair stages").
//
// Thread block = 128 sinks (one per thread) x a chunk of sources.  Each thread
// resolves the visibility of its sink from every source of the chunk, then
// evaluates the field of the visible pairs and sums them over the chunk in
// registers.  Chunk partial sums go to a [n_chunks, n_snk, 6] buffer and a
// second kernel reduces them in FP64 in a fixed order, so results are
// reproducible run to run.  Optionally the kernels also write the per-pair
// network (the reference's output layout) and a visibility bit mask.
//
// Brute force (replaces raycast_brute_force, lyceanem/src/raycasting_brute_force.cuh:68-88):
// triangle tiles of 64 are staged in shared memory by TMA bulk copies
// (double-buffered, mbarrier-completed, bounded waits); for each source of
// the chunk the block derives the ray-independent part of the test once per
// triangle (tvec, qvec, e2.qvec) and every thread tests its ray against the
// tile.  A ray stops at its first hit; a tile step is skipped when no thread
// of the block still has an unresolved ray (block vote), and the block stops
// loading tiles once every ray is resolved.
//
// Grid (replaces raycast_tiles + DDA, lyceanem/src/raycasting_accelerated.cuh:106-268, 458-482):
// each thread walks its segment through a uniform 3-D grid (Amanatides-Woo,
// boundary crossings recomputed from the cell index so no error accumulates)
// and tests the triangles stored contiguously per cell (float4 loads), stopping
// at the first hit.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "lyem_device.cuh"
#include "lyem_internal.cuh"
#include "lyem_walk.cuh"

namespace lyem {

__device__ unsigned int g_device_error = 0;

static std::atomic<unsigned long long> g_launches{0};
void note_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void fma_probe_kernel(long long iters, float seed, float* sink) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float b = 0.999999f, c = 1e-7f;
#pragma unroll 16
    for (long long i = 0; i < iters; ++i) {
        a0 = __fmaf_rn(a0, b, c); a1 = __fmaf_rn(a1, b, c); a2 = __fmaf_rn(a2, b, c); a3 = __fmaf_rn(a3, b, c);
        a4 = __fmaf_rn(a4, b, c); a5 = __fmaf_rn(a5, b, c); a6 = __fmaf_rn(a6, b, c); a7 = __fmaf_rn(a7, b, c);
    }
    float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.f) sink[0] = s;  // keeps the chains alive
}

cudaError_t fma_probe(long long iters, double* fma_per_s, cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    float* sink = nullptr;
    e = cudaMallocAsync(&sink, 16, stream);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256;
    fma_probe_kernel<<<blocks, threads, 0, stream>>>(iters / 4, 1.f, sink); note_launches(1);
    cudaEventRecord(a, stream);
    fma_probe_kernel<<<blocks, threads, 0, stream>>>(iters, 1.f, sink); note_launches(1);
    cudaEventRecord(b, stream);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFreeAsync(sink, stream);
    if (e != cudaSuccess) return e;
    *fma_per_s = (double)blocks * threads * 8.0 * (double)iters / (ms * 1e-3);
    return cudaGetLastError();
}

int device_sm_count() {
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < kMaxDev) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return 1;
    if (dev >= 0 && dev < kMaxDev) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

unsigned capped_blocks(long long n, int threads, int per_sm) {
    long long b = (n + threads - 1) / threads;
    const long long cap = (long long)device_sm_count() * per_sm;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

unsigned int* device_error_word() {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) return nullptr;
    return static_cast<unsigned int*>(p);
}

cudaError_t read_clear_device_errors(unsigned int* flags, cudaStream_t stream) {
    unsigned int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(flags, g_device_error, sizeof(unsigned int), 0,
                                              cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyToSymbolAsync(g_device_error, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

constexpr int kThreads = 128;
// Brute-force triangle tile: 64 triangles (3 KB raw + 4 KB derived per buffer)
// leave room for more resident blocks than 128 did (8-array direct scene
// 0.336 -> 0.277 ms; 32 measured 0.297 ms).
constexpr int kTile = 64;
constexpr int kBruteMaxChunk = 32;  // one bit per source in a 32-bit mask
constexpr int kGridMaxChunk = 64;   // one bit per source in a 64-bit mask

int stage_block_threads() { return kThreads; }
int brute_max_src_chunk() { return kBruteMaxChunk; }
int grid_max_src_chunk() { return kGridMaxChunk; }
int transposed_src_chunk() { return 32; }

struct BruteSmem {
    float4 raw[2][kTile * 3];
    TriPre pre[2][kTile];
    unsigned long long mbar[2];
};

__device__ __forceinline__ void load_E(const float* base, long long n, float* E) {
    const float2* p = reinterpret_cast<const float2*>(base + 6 * n);
    float2 a = p[0], b = p[1], c = p[2];
    E[0] = a.x; E[1] = a.y; E[2] = b.x; E[3] = b.y; E[4] = c.x; E[5] = c.y;
}

// Field epilogue for one (n, m) pair shared by both kernels.
template <bool WEIGHTED, bool PAIR_OUT>
__device__ __forceinline__ void pair_epilogue(const StageParams& p, long long n, long long m, bool m_ok, bool vis,
                                              float ox, float oy, float oz, float ex, float ey, float ez, float nx,
                                              float ny, float nz, float* acc) {
    if (vis) {
        Ray r = make_ray(ox, oy, oz, ex, ey, ez);
        double rl = path_length_fp64(ox, oy, oz, ex, ey, ez, r.len);
        float E[6], out[6];
        load_E(p.src_E, n, E);
        pair_field(r, rl, E, nx, ny, nz, p.alpha, p.beta_f, p.beta_d, out);
        if (PAIR_OUT) {
            float2* po = reinterpret_cast<float2*>(p.pair_out + 6 * (n * p.n_snk + m));
            po[0] = make_float2(out[0], out[1]);
            po[1] = make_float2(out[2], out[3]);
            po[2] = make_float2(out[4], out[5]);
        }
        if (WEIGHTED) {
            float W[6];
            load_E(p.src_W, n, W);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                acc[2 * k] += W[2 * k] * out[2 * k] - W[2 * k + 1] * out[2 * k + 1];
                acc[2 * k + 1] += W[2 * k] * out[2 * k + 1] + W[2 * k + 1] * out[2 * k];
            }
        } else {
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[k] += out[k];
        }
    } else if (PAIR_OUT && m_ok) {
        float2* po = reinterpret_cast<float2*>(p.pair_out + 6 * (n * p.n_snk + m));
        po[0] = po[1] = po[2] = make_float2(0.f, 0.f);
    }
}

// Mask bits of the warp's 32 sinks for source n, and the per-source visible count.
// ms is the lane's sink slot (m = ms in natural order); lanes past the last
// sink have vis == false.
template <bool MASK_OUT>
__device__ __forceinline__ void record_visibility(const StageParams& p, long long n, long long m, long long ms,
                                                  bool vis) {
    if (!MASK_OUT && !p.src_visible) return;
    unsigned b = __ballot_sync(0xffffffffu, vis);
    if (MASK_OUT && p.snk_order) {
        // permuted sinks: the warp's lanes are not 32 consecutive sinks (mask zeroed by the host)
        if (vis) atomicOr(p.mask_bits + n * p.mask_words + (m >> 5), 1u << (m & 31));
    }
    if ((threadIdx.x & 31) == 0) {
        // natural order: the warp's slots ms .. ms + 31 are the sinks of word ms / 32
        const long long w = ms >> 5;
        if (MASK_OUT && !p.snk_order && w < p.mask_words) p.mask_bits[n * p.mask_words + w] = b;
        if (p.src_visible && b) atomicAdd(p.src_visible + n, __popc(b));
    }
}

__device__ __forceinline__ void flush_block(const StageParams& p, long long m, bool m_ok, const float* acc,
                                            unsigned long long vis_count, unsigned long long tests) {
    if (m_ok) {
        float2* dst = reinterpret_cast<float2*>(p.partial + 6 * ((p.chunk_base + (long long)blockIdx.y) * p.n_snk + m));
        dst[0] = make_float2(acc[0], acc[1]);
        dst[1] = make_float2(acc[2], acc[3]);
        dst[2] = make_float2(acc[4], acc[5]);
        if (p.snk_visible && vis_count) atomicAdd(p.snk_visible + m, (int)vis_count);
    }
    if (p.counters) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            vis_count += __shfl_down_sync(0xffffffffu, vis_count, o);
            tests += __shfl_down_sync(0xffffffffu, tests, o);
        }
        if ((threadIdx.x & 31) == 0) {
            if (vis_count) atomicAdd(p.counters + 0, vis_count);
            if (tests) atomicAdd(p.counters + 1, tests);
        }
    }
}

// Registers capped so that 9 blocks fit an SM (56 registers, almost no spill):
// the direct scene's 1,344 blocks then run in one wave on 152 SMs instead of
// 8 per SM plus a tail (stage 0.266 -> 0.219 ms; a cap for 12 blocks spills
// and measured 0.268 ms).
template <bool CULL, bool WEIGHTED, bool PAIR_OUT, bool MASK_OUT>
__global__ void __launch_bounds__(kThreads, 9) brute_stage_kernel(const StageParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    BruteSmem& sm = *reinterpret_cast<BruteSmem*>(smem_raw);

    const int tid = threadIdx.x;
    const long long ms = (long long)blockIdx.x * kThreads + tid;
    const bool m_ok = ms < p.n_snk;
    const long long m = m_ok ? (p.snk_order ? (long long)p.snk_order[ms] : ms) : 0;
    const long long n0 = (p.chunk_base + (long long)blockIdx.y) * p.src_chunk;
    const long long rem = p.n_src - n0;
    const int nsrc = (int)(rem < p.src_chunk ? rem : p.src_chunk);
    auto src_index = [&](int s) -> long long {
        return p.src_order ? (long long)p.src_order[n0 + s] : n0 + s;
    };

    float ex = 0.f, ey = 0.f, ez = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    if (m_ok) {
        ex = p.snk_pos[3 * m]; ey = p.snk_pos[3 * m + 1]; ez = p.snk_pos[3 * m + 2];
        nx = p.snk_nrm[3 * m]; ny = p.snk_nrm[3 * m + 1]; nz = p.snk_nrm[3 * m + 2];
    }
    uint32_t pending = 0, blocked = 0;
    for (int s = 0; s < nsrc; ++s)
        if (m_ok && !(p.skip_diag && src_index(s) == m)) pending |= 1u << s;

    const long long T = p.n_tris;
    const int ntiles = (int)((T + kTile - 1) / kTile);
    const uint32_t mb0 = smem_addr(&sm.mbar[0]), mb1 = smem_addr(&sm.mbar[1]);
    if (tid == 0) {
        mbar_init(mb0, 1);
        mbar_init(mb1, 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int k) {
        long long first = (long long)k * kTile;
        long long cnt = T - first < kTile ? T - first : kTile;
        tma_load_1d(smem_addr(&sm.raw[k & 1][0]), p.tris + 3 * first, (uint32_t)(cnt * 48), (k & 1) ? mb1 : mb0);
    };
    if (tid == 0) {
        if (ntiles > 0) issue(0);
        if (ntiles > 1) issue(1);
    }

    unsigned long long tests = 0;
    bool timed_out = false;
    // with one source per block (the automatic shape for few sources) the lane's
    // ray is formed once instead of once per tile
    Ray r1 = Ray{0.f, 0.f, 0.f, 0.f};
    if (nsrc == 1 && (pending & 1u)) {
        const float* so = p.src_pos + 3 * src_index(0);
        r1 = vis_ray<CULL>(so[0], so[1], so[2], ex, ey, ez);
    }
    int k = 0;
    for (; k < ntiles; ++k) {
        if (!__syncthreads_or(pending != 0)) break;
        bool ok = mbar_wait_bounded((k & 1) ? mb1 : mb0, (k >> 1) & 1, kWaitCycles);
        if (__syncthreads_or(!ok)) { timed_out = true; break; }
        const int cnt = (int)(T - (long long)k * kTile < kTile ? T - (long long)k * kTile : kTile);
        const float4* rt = sm.raw[k & 1];
        for (int s = 0; s < nsrc; ++s) {
            TriPre* pb = sm.pre[(k * nsrc + s) & 1];
            const float* so = p.src_pos + 3 * src_index(s);
            const float ox = so[0], oy = so[1], oz = so[2];
            if (tid < cnt) pb[tid] = make_tripre(ox, oy, oz, rt[3 * tid], rt[3 * tid + 1], rt[3 * tid + 2]);
            const bool mine = (pending >> s) & 1u;
            if (!__syncthreads_or(mine)) continue;
            if (mine) {
                const Ray r = nsrc == 1 ? r1 : vis_ray<CULL>(ox, oy, oz, ex, ey, ez);
                int j = 0;
                bool hitany = false;
                for (; j < cnt; ++j) {
                    if (hit_pre<CULL>(r, pb[j], p.eps)) { hitany = true; break; }
                }
                tests += hitany ? (unsigned long long)(j + 1) : (unsigned long long)cnt;
                if (hitany) {
                    pending &= ~(1u << s);
                    blocked |= 1u << s;
                }
            }
        }
        // Every thread has finished reading raw[k & 1] (the block vote of the
        // last source step above is a barrier): refill it with tile k + 2.
        if (tid == 0 && k + 2 < ntiles) {
            fence_proxy_async_smem();
            issue(k + 2);
        }
    }
    // Wait (bounded) for copies still in flight before the block may exit.
    {
        int hi = k + 2 < ntiles ? k + 2 : ntiles;
        for (int j = k; j < hi; ++j) {
            if (timed_out && j == k) continue;
            if (!mbar_wait_bounded((j & 1) ? mb1 : mb0, (j >> 1) & 1, kWaitCycles)) timed_out = true;
        }
    }
    if (timed_out) {
        if (tid == 0) atomicOr(&g_device_error, 1u);
        return;
    }

    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    unsigned long long vis_count = 0;
    for (int s = 0; s < nsrc; ++s) {
        const long long n = src_index(s);
        const bool vis = m_ok && !((blocked >> s) & 1u);
        record_visibility<MASK_OUT>(p, n, m, ms, vis);
        const float* so = p.src_pos + 3 * n;
        pair_epilogue<WEIGHTED, PAIR_OUT>(p, n, m, m_ok, vis, so[0], so[1], so[2], ex, ey, ez, nx, ny, nz, acc);
        vis_count += vis;
    }
    flush_block(p, m, m_ok, acc, vis_count, tests);
}

// Grid stage.  Each lane owns one sink and resolves the rays from the chunk's
// sources to it.  A ray walks the uniform grid (Amanatides-Woo; the boundary
// crossings are recomputed from the cell index, so no error accumulates) and
// tests the triangles stored contiguously per cell (float4 loads), stopping at
// its first hit.  Two schedules of the rays over the lanes:
//   lockstep  all lanes of a warp trace source s, then source s + 1, ...; ray
//             set-up runs in lockstep, a warp waits for its longest ray;
//   refill    each lane moves to its next source when its ray ends, but new
//             rays are started in batches (once `refill_lanes` lanes of the
//             warp are idle, or none is busy) so the set-up code is not
//             serialised lane by lane.
// Visibility of the chunk is kept as a 64-bit blocked mask; the field epilogue
// then runs over the sources in lockstep.
constexpr int kLockstep = 0;
constexpr int kRefill = 1;
// Lockstep with the registers capped so that 10, 12 or 16 blocks of 128
// threads fit an SM.  More resident warps hide more of the triangle-load
// latency: on the 28 GHz one-bounce scene the scatter->sink stage takes 1357 ms
// uncapped (60 registers, 8 blocks), 1184 / 1067 / 969 ms capped at 10 / 12 /
// 16 blocks, the last with some spilling; 16 is the default schedule.
constexpr int kLockstep10 = 2;
constexpr int kLockstep12 = 3;
constexpr int kLockstep16 = 4;
// Two phases (registers capped for 16 or 12 blocks per SM).  Phase 1 runs the
// lockstep schedule but walks each ray only up to parameter near_dist (most
// blocked rays end near their origin: the own-surface triangle, local
// clutter); the rays still open there are appended, source-major, to a queue
// of the warp in shared memory (ballot + prefix count).  Phase 2 takes them 32
// at a time, each lane one ray (the sink coordinates come from the owning lane
// by shuffle), and walks them from near_dist to their end, so the lanes of a
// warp hold live rays of one or two sources instead of idling behind the
// longest ray of each source.
constexpr int kTwoPhase16 = 5;
constexpr int kTwoPhase12 = 6;

// COUNT = false (only with the default schedule, when the caller asks for no
// counters) leaves the per-test counting out of the walk: one instruction and
// one register less in the innermost loop (scatter->sink stage of the 28 GHz
// scene 448 -> 440 ms).
template <bool CULL, bool WEIGHTED, bool PAIR_OUT, bool MASK_OUT, int MODE, bool COUNT = true>
__global__ void __launch_bounds__(kThreads, MODE == kLockstep10 ? 10 : (MODE == kLockstep12 || MODE == kTwoPhase12) ? 12 : (MODE == kLockstep16 || MODE == kTwoPhase16) ? 16 : 1) grid_stage_kernel(const StageParams p) {
    // 32-bit indices (fewer live registers in the walk): the entry point keeps
    // n_src and n_snk below 2^31 - 256
    const int tid = threadIdx.x;
    const int ms = (int)blockIdx.x * kThreads + tid;
    const bool m_ok = ms < p.n_snk;
    const int m = m_ok ? (p.snk_order ? p.snk_order[ms] : ms) : 0;
    const int n0 = (int)((p.chunk_base + (long long)blockIdx.y) * p.src_chunk);
    const int rem = (int)p.n_src - n0;
    const int nsrc = rem < p.src_chunk ? rem : p.src_chunk;
    auto src_index = [&](int s) -> int {
        return p.src_order ? p.src_order[n0 + s] : n0 + s;
    };
    float ex = 0.f, ey = 0.f, ez = 0.f;
    if (m_ok) {
        ex = p.snk_pos[3 * (long long)m]; ey = p.snk_pos[3 * (long long)m + 1]; ez = p.snk_pos[3 * (long long)m + 2];
    }
    unsigned long long blocked = 0;
    unsigned int tests = 0;  // diagnostic count of one lane (64 rays at most); wraps only past 2^32 tests
    Walk w;
    if (MODE == kTwoPhase16 || MODE == kTwoPhase12) {
        __shared__ int s_hint[kGridMaxChunk];
        __shared__ unsigned long long s_blk[kThreads / 32][32];
        extern __shared__ unsigned short s_queue[];  // per warp: src_chunk x 32 entries (source << 5 | lane)
        const int lane = tid & 31, warp = tid >> 5;
        unsigned short* queue = s_queue + (size_t)warp * p.src_chunk * 32;
        s_blk[warp][lane] = 0ull;
        for (int s = warp; s < nsrc; s += kThreads / 32) {
            const float* so = p.src_pos + 3 * (long long)src_index(s);
            const int h = warp_nearest_ref(p, so[0], so[1], so[2]);
            if (lane == 0) s_hint[s] = h;
        }
        __syncthreads();
        const float near = p.near_dist;
        const unsigned full = 0xffffffffu;
        int count = 0;  // the same in every lane of the warp
        for (int s = 0; s < nsrc; ++s) {
            const int n = src_index(s);
            bool far = false;
            if (m_ok && !(p.skip_diag && n == m)) {
                const float* so = p.src_pos + 3 * (long long)n;
                walk_ray<CULL>(w, so[0], so[1], so[2], ex, ey, ez);
                const int hint = s_hint[s];
                bool hit = false;
                if (hint >= 0) {
                    ++tests;
                    hit = walk_test_ref<CULL>(p, w, hint);
                }
                if (!hit && walk_setup(p, w)) {
                    while (true) {
                        while (w.q < w.q1) {
                            ++tests;
                            if (walk_test<CULL>(p, w)) { hit = true; break; }
                        }
                        if (hit) break;
                        const int st = walk_step_until(p, w, near, &g_device_error);
                        if (st != 1) {
                            far = st == 2;
                            break;
                        }
                    }
                }
                if (hit) blocked |= 1ull << s;
            }
            const unsigned fb = __ballot_sync(full, far);
            if (far) queue[count + __popc(fb & ((1u << lane) - 1u))] = (unsigned short)((s << 5) | lane);
            count += __popc(fb);
        }
        __syncwarp();
        for (int base = 0; base < count; base += 32) {
            const int i = base + lane;
            const bool has = i < count;
            const unsigned e = has ? queue[i] : 0u;
            const int owner = (int)(e & 31u), s = (int)(e >> 5);
            const float qx = __shfl_sync(full, ex, owner), qy = __shfl_sync(full, ey, owner),
                        qz = __shfl_sync(full, ez, owner);
            if (has) {
                const float* so = p.src_pos + 3 * (long long)src_index(s);
                walk_ray<CULL>(w, so[0], so[1], so[2], qx, qy, qz);
                bool hit = false;
                if (walk_setup_from(p, w, near)) {
                    while (!hit) {
                        while (w.q < w.q1) {
                            ++tests;
                            if (walk_test<CULL>(p, w)) { hit = true; break; }
                        }
                        if (hit || !walk_step(p, w, &g_device_error)) break;
                    }
                }
                if (hit) atomicOr(&s_blk[warp][owner], 1ull << s);
            }
        }
        __syncwarp();
        blocked |= s_blk[warp][lane];
    } else if (MODE != kRefill) {
        // per source of the chunk, the triangle nearest to it (one warp per source):
        // tried first by every ray from that source
        __shared__ int s_hint[kGridMaxChunk];
        for (int s = tid >> 5; s < nsrc; s += kThreads / 32) {
            const float* so = p.src_pos + 3 * (long long)src_index(s);
            const int h = warp_nearest_ref(p, so[0], so[1], so[2]);
            if ((tid & 31) == 0) s_hint[s] = h;
        }
        __syncthreads();
        for (int s = 0; s < nsrc; ++s) {
            const int n = src_index(s);
            if (!m_ok || (p.skip_diag && n == m)) continue;
            const float* so = p.src_pos + 3 * (long long)n;
            walk_ray<CULL>(w, so[0], so[1], so[2], ex, ey, ez);
            const int hint = s_hint[s];
            bool hit = false;
            if (hint >= 0) {  // a hit on any triangle blocks the segment, walked or not
                if (COUNT) ++tests;
                hit = walk_test_ref<CULL>(p, w, hint);
            }
            if (!hit && !walk_setup(p, w)) continue;
            while (!hit) {
                while (w.q < w.q1) {
                    if (COUNT) ++tests;
                    if (walk_test<CULL>(p, w)) { hit = true; break; }
                }
                if (hit || !walk_step(p, w, &g_device_error)) break;
            }
            if (hit) blocked |= 1ull << s;
        }
    } else {
        int s = -1;
        bool has = false;
        // next source of this lane that needs a walk (untested and off-grid rays are visible)
        auto refill = [&]() {
            while (++s < nsrc) {
                const int n = src_index(s);
                if (p.skip_diag && n == m) continue;
                const float* so = p.src_pos + 3 * (long long)n;
                if (walk_begin<CULL>(p, w, so[0], so[1], so[2], ex, ey, ez)) { has = true; return; }
            }
        };
        const unsigned full = 0xffffffffu;
        while (true) {
            const bool can = !has && m_ok && s + 1 < nsrc;
            const unsigned busy = __ballot_sync(full, has);
            const unsigned idle = __ballot_sync(full, can);
            if (busy == 0 && idle == 0) break;
            if (can && (busy == 0 || __popc(idle) >= p.refill_lanes)) refill();
            if (has) {
                while (w.q < w.q1) {
                    ++tests;
                    if (walk_test<CULL>(p, w)) {
                        blocked |= 1ull << s;
                        has = false;
                        break;
                    }
                }
                if (has && !walk_step(p, w, &g_device_error)) has = false;
            }
        }
    }

    float nx = 0.f, ny = 0.f, nz = 0.f;
    if (m_ok) {
        nx = p.snk_nrm[3 * (long long)m]; ny = p.snk_nrm[3 * (long long)m + 1]; nz = p.snk_nrm[3 * (long long)m + 2];
    }
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    unsigned long long vis_count = 0;
    for (int k = 0; k < nsrc; ++k) {
        const int n = src_index(k);
        const bool vis = m_ok && !((blocked >> k) & 1ull);
        record_visibility<MASK_OUT>(p, n, m, ms, vis);
        const float* so = p.src_pos + 3 * (long long)n;
        pair_epilogue<WEIGHTED, PAIR_OUT>(p, n, m, m_ok, vis, so[0], so[1], so[2], ex, ey, ez, nx, ny, nz, acc);
        vis_count += vis;
    }
    flush_block(p, m, m_ok, acc, vis_count, tests);
}

// Transposed grid stage (traversal 38).  The lanes of a warp are the 32
// sources of the block's chunk, and each warp traces its 32 sinks one after
// the other, so the 32 rays a warp walks together end at the same sink.  When
// the sources are the elements of an array (millimetres apart) those rays cross
// the same cells and test the same triangles, where a warp of the lockstep
// schedule holds 32 directions from one source (a CPU model of the walk on the
// 28 GHz scene: 78.5 instead of 124.8 test iterations per 32 array rays).  The
// field of each sink is summed over the warp's lanes in a fixed butterfly order
// and lane 0 writes the chunk's partial sum of that sink.
constexpr int kTChunk = 32;

template <bool CULL, bool WEIGHTED, bool PAIR_OUT, bool MASK_OUT, bool COUNT>
__global__ void __launch_bounds__(kThreads, 16) grid_transposed_kernel(const StageParams p) {
    const unsigned full = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long chunk = p.chunk_base + (long long)blockIdx.y;
    const int n0 = (int)(chunk * kTChunk);
    const int nsrc = (int)p.n_src - n0 < kTChunk ? (int)p.n_src - n0 : kTChunk;
    const bool n_ok = lane < nsrc;
    const int n = n_ok ? (p.src_order ? p.src_order[n0 + lane] : n0 + lane) : 0;
    // each source's own-surface triangle (one warp per source), tried before the walk
    __shared__ int s_hint[kTChunk];
    for (int s = warp; s < nsrc; s += kThreads / 32) {
        const int ns = p.src_order ? p.src_order[n0 + s] : n0 + s;
        const float* so = p.src_pos + 3 * (long long)ns;
        const int h = warp_nearest_ref(p, so[0], so[1], so[2]);
        if (lane == 0) s_hint[s] = h;
    }
    __syncthreads();
    float ox = 0.f, oy = 0.f, oz = 0.f;
    if (n_ok) {
        const float* so = p.src_pos + 3 * (long long)n;
        ox = so[0]; oy = so[1]; oz = so[2];
    }
    const int hint = n_ok ? s_hint[lane] : -1;
    const int ms0 = (int)blockIdx.x * kThreads + warp * 32;  // the warp's first sink slot
    unsigned vis_mask = 0;                                    // bit k: this lane's source sees slot ms0 + k
    unsigned int tests = 0;
    Walk w;
    for (int k = 0; k < 32; ++k) {
        const int ms = ms0 + k;
        if (ms >= p.n_snk) break;  // the same in every lane
        const int m = p.snk_order ? p.snk_order[ms] : ms;
        const float ex = p.snk_pos[3 * (long long)m], ey = p.snk_pos[3 * (long long)m + 1],
                    ez = p.snk_pos[3 * (long long)m + 2];
        bool vis = n_ok;  // untested pairs (the skipped diagonal, segments off the grid) are visible
        if (n_ok && !(p.skip_diag && n == m)) {
            walk_ray<CULL>(w, ox, oy, oz, ex, ey, ez);
            bool hit = false;
            if (hint >= 0) {
                if (COUNT) ++tests;
                hit = walk_test_ref<CULL>(p, w, hint);
            }
            if (!hit && walk_setup(p, w)) {
                while (!hit) {
                    while (w.q < w.q1) {
                        if (COUNT) ++tests;
                        if (walk_test<CULL>(p, w)) { hit = true; break; }
                    }
                    if (hit || !walk_step(p, w, &g_device_error)) break;
                }
            }
            vis = !hit;
        }
        if (vis) {
            vis_mask |= 1u << k;
            if (MASK_OUT && p.snk_order) atomicOr(p.mask_bits + (long long)n * p.mask_words + (m >> 5), 1u << (m & 31));
        }
        float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float nx = p.snk_nrm[3 * (long long)m], ny = p.snk_nrm[3 * (long long)m + 1],
                    nz = p.snk_nrm[3 * (long long)m + 2];
        pair_epilogue<WEIGHTED, PAIR_OUT>(p, n, m, n_ok, vis, ox, oy, oz, ex, ey, ez, nx, ny, nz, acc);
#pragma unroll
        for (int c = 0; c < 6; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(full, acc[c], o);
        const unsigned b = __ballot_sync(full, vis);
        if (lane == 0) {
            float2* dst = reinterpret_cast<float2*>(p.partial + 6 * (chunk * p.n_snk + m));
            dst[0] = make_float2(acc[0], acc[1]);
            dst[1] = make_float2(acc[2], acc[3]);
            dst[2] = make_float2(acc[4], acc[5]);
            if (p.snk_visible && b) atomicAdd(p.snk_visible + m, __popc(b));
        }
    }
    if (n_ok) {
        if (MASK_OUT && !p.snk_order && ms0 < p.n_snk) p.mask_bits[(long long)n * p.mask_words + (ms0 >> 5)] = vis_mask;
        if (p.src_visible && vis_mask) atomicAdd(p.src_visible + n, __popc(vis_mask));
    }
    if (p.counters) {
        unsigned long long v = __popc(vis_mask), t = tests;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v += __shfl_down_sync(full, v, o);
            t += __shfl_down_sync(full, t, o);
        }
        if (lane == 0) {
            if (v) atomicAdd(p.counters + 0, v);
            if (t) atomicAdd(p.counters + 1, t);
        }
    }
}

__global__ void reduce_partials_kernel(const float* __restrict__ partial, long long n_chunks, long long n_elem,
                                       float* __restrict__ out, int accumulate) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_elem;
         i += (long long)gridDim.x * blockDim.x) {
        double s = accumulate ? (double)out[i] : 0.0;
        for (long long c = 0; c < n_chunks; ++c) s += (double)partial[c * n_elem + i];
        out[i] = (float)s;
    }
}

template <bool CULL, bool WEIGHTED, bool PAIR_OUT, bool MASK_OUT>
static cudaError_t launch_t(const StageParams& p0, cudaStream_t stream) {
    const long long chunks = (p0.n_src + p0.src_chunk - 1) / p0.src_chunk;
    const unsigned tiles = (unsigned)((p0.n_snk + kThreads - 1) / kThreads);
    // gridDim.y is limited to 65535: launch the source chunks in slices
    for (long long base = 0; base < chunks; base += 65535) {
        StageParams p = p0;
        p.chunk_base = base;
        dim3 grid(tiles, (unsigned)(chunks - base < 65535 ? chunks - base : 65535));
        if (p.cell_start) {
            if (p.refill_lanes == -116 || p.refill_lanes == -112) {
                const size_t qbytes = (size_t)(kThreads / 32) * p.src_chunk * 32 * sizeof(unsigned short);
                if (p.refill_lanes == -116)
                    grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kTwoPhase16><<<grid, kThreads, qbytes, stream>>>(p);
                else
                    grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kTwoPhase12><<<grid, kThreads, qbytes, stream>>>(p);
            } else if (p.refill_lanes == -38) {
                if (p.counters)
                    grid_transposed_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, true><<<grid, kThreads, 0, stream>>>(p);
                else
                    grid_transposed_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, false><<<grid, kThreads, 0, stream>>>(p);
            } else if (p.refill_lanes == -16) {
                if (p.counters)
                    grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kLockstep16><<<grid, kThreads, 0, stream>>>(p);
                else
                    grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kLockstep16, false>
                        <<<grid, kThreads, 0, stream>>>(p);
            }
            else if (p.refill_lanes == -12)
                grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kLockstep12><<<grid, kThreads, 0, stream>>>(p);
            else if (p.refill_lanes == -10)
                grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kLockstep10><<<grid, kThreads, 0, stream>>>(p);
            else if (p.refill_lanes > 0)
                grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kRefill><<<grid, kThreads, 0, stream>>>(p);
            else
                grid_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT, kLockstep><<<grid, kThreads, 0, stream>>>(p);
            note_launches(1);
        } else {
            const size_t smem = sizeof(BruteSmem);
            auto kern = brute_stage_kernel<CULL, WEIGHTED, PAIR_OUT, MASK_OUT>;
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            kern<<<grid, kThreads, smem, stream>>>(p); note_launches(1);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <bool CULL, bool WEIGHTED, bool PAIR_OUT>
static cudaError_t launch_m(const StageParams& p, cudaStream_t s) {
    return p.mask_bits ? launch_t<CULL, WEIGHTED, PAIR_OUT, true>(p, s) : launch_t<CULL, WEIGHTED, PAIR_OUT, false>(p, s);
}
template <bool CULL, bool WEIGHTED>
static cudaError_t launch_p(const StageParams& p, cudaStream_t s) {
    return p.pair_out ? launch_m<CULL, WEIGHTED, true>(p, s) : launch_m<CULL, WEIGHTED, false>(p, s);
}
template <bool CULL>
static cudaError_t launch_w(const StageParams& p, cudaStream_t s) {
    return p.src_W ? launch_p<CULL, true>(p, s) : launch_p<CULL, false>(p, s);
}

cudaError_t launch_pair_stage(const StageParams& p, int cull, cudaStream_t stream) {
    if (p.n_src == 0 || p.n_snk == 0) return cudaSuccess;
    return cull ? launch_w<true>(p, stream) : launch_w<false>(p, stream);
}

cudaError_t launch_reduce_partials(const float* partial, long long n_chunks, long long n_snk, float* out,
                                   int accumulate, cudaStream_t stream) {
    const long long n_elem = 6 * n_snk;
    if (n_elem == 0) return cudaSuccess;
    const unsigned blocks = capped_blocks(n_elem, 256, 16);
    reduce_partials_kernel<<<blocks, 256, 0, stream>>>(partial, n_chunks, n_elem, out, accumulate); note_launches(1);
    return cudaGetLastError();
}

}  // namespace lyem
