// lyem_batch.cu -- many scenes x many frequencies, direct + one-bounce paths,
// in one persistent launch.
//
// Each scene is the composition of calculate_scattering_cuda
// (lyceanem/models/frequency_domain.py:195-264) summed over the sources
// (:847-849), evaluated at every frequency of a list:
//   e_p(f)  = sum_n S1_f(n, p)                           scatter excitation
//   E_f(m)  = sum_n S0_f(n, m) + sum_p e_p(f) (.) S2_f(p, m; e_p(f))
// with S_f the per-pair field of em_wave (lyceanem/src/em.cuh:18-120) at
// beta_f and the visibility of raycasting.cuh:19-95, which is the same for
// every frequency and is therefore resolved once.
//
// Work is a queue of items that the warps of a fixed set of resident blocks
// take in order, each warp on its own (no block-wide barrier: a warp whose
// rays end early moves on instead of waiting for the slowest warp of a tile):
//   V items  visibility of one source chunk (32 or 64 sources) against 32
//            sinks, for one of the three stages of a scene (sources ->
//            scatter points, sources -> sinks, scatter points -> sinks): grid
//            DDA, all lanes on the same source at a time; each lane stores
//            its sink's visibility of the chunk as bits of a sink-major mask
//            (one 32-bit word per 32 sources);
//   W items  e_p(f) for a run of (scatter point, frequency group) slots;
//   E items  E_f(m) for a run of (sink, frequency group) slots.
// The queue holds every V item, then every W item, then every E item.  A W
// item needs its scene's sources -> scatter visibility; an E item needs the
// two other visibility stages and all W items of its scene.  They wait on the
// scene's completion counters.  Every item waited on was taken from the queue
// earlier by a running warp that itself waits only on items taken before it,
// so each wait ends; the waits are bounded all the same and raise bit 0 of
// the error word on expiry.
//
// Frequencies: thread (sink, g) of a field item handles the frequencies
// g*FG .. g*FG+FG-1.  The phase beta_f * r of the first one is formed in
// float-float arithmetic (r from the exact coordinate differences, reduced mod
// 2 pi by a Cody-Waite step whose first product-subtraction is exact), and the
// next FG-1 frequencies follow by complex rotation with exp(-j dbeta r), dbeta
// being the uniform frequency step.  FP64 is not used on this path: its rate
// on this GPU is a small fraction of the FP32 rate.  FG = 1 evaluates every
// frequency from its own phase and accepts any frequency list.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "lyem.h"
#include "lyem_device.cuh"
#include "lyem_internal.cuh"
#include "lyem_walk.cuh"

namespace lyem {
namespace {

constexpr int kBT = 256;  // threads per block (8 independent warps)
constexpr int kWarpSinks = 32;               // sinks of a visibility item (one per lane)
constexpr long long kItemPairs = 1LL << 14;  // candidate pairs a field item should cover at least
constexpr int kKinds = 5;
enum Kind { kVisScat = 0, kVisDirect = 1, kVisBounce = 2, kFieldW = 3, kFieldE = 4 };

// The grid fields the walk helpers read (lyem_walk.cuh).
struct GridView {
    const int* cell_start;
    const float4* cell_tris;
    const float4* cell_box;
    float g0[3], g1[3];
    float cell, inv_cell;
    int dims[3];
    float eps;
};

struct DevScene {
    const float* src_pos;
    const float* src_E;
    const float* scat_pos;
    const float* scat_nrm;
    const int* scat_id;
    long long n_src, n_scat;
    GridView grid;
    unsigned int* mask[3];     // sink-major visibility bits of stages kVisScat, kVisDirect, kVisBounce
    long long mask_words[3];   // words per mask row
    float* w;                  // [n_scat][n_freq][6] scatter excitation
    int expect[kKinds];        // items of each kind
    int pad;
};

struct BatchParams {
    const DevScene* scenes;
    const int4* items;  // (kind, scene, a, b)
    int n_items;
    int n_scenes;
    unsigned int* head;  // queue position
    unsigned int* done;  // [n_scenes][kKinds] finished items
    const float* snk_pos;
    const float* snk_nrm;
    const int* snk_id;
    long long n_snk;
    const float2* beta_ff;  // [n_freq] beta as float-float (hi, lo)
    const float* beta_f;    // [n_freq] beta rounded to FP32
    float2 dbeta_ff;        // uniform frequency step of beta as float-float
    int n_freq;
    int n_groups;           // ceil(n_freq / FG); a field slot is (point, group), slot = point * n_groups + group
    int src_chunk;
    float alpha;
    int skip_diag;
    unsigned int* err;
    unsigned long long* counters;  // [n_scenes][4]: visible pairs of the three stages, ray-triangle tests
    float* field;                  // [n_scenes][n_freq][n_snk][6] output
};

// ---------------------------------------------------------------- queue

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded wait until *ctr >= target; false on expiry.
__device__ bool wait_count(const unsigned* ctr, unsigned target) {
    if (target == 0) return true;
    const long long t0 = clock64();
    while (true) {
        if (ld_acquire(ctr) >= target) return true;
        if (clock64() - t0 > kWaitCycles) return false;
        __nanosleep(200);
    }
}

__device__ bool wait_deps(const BatchParams& P, int kind, int scene) {
    const DevScene& S = P.scenes[scene];
    const unsigned* d = P.done + (long long)scene * kKinds;
    if (kind == kFieldW) return wait_count(d + kVisScat, (unsigned)S.expect[kVisScat]);
    bool ok = wait_count(d + kVisDirect, (unsigned)S.expect[kVisDirect]);
    ok = ok && wait_count(d + kVisBounce, (unsigned)S.expect[kVisBounce]);
    ok = ok && wait_count(d + kFieldW, (unsigned)S.expect[kFieldW]);
    return ok;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------- V items

// The scene's grid parameters are read from shared memory (sgrid, filled by
// the caller) rather than held in registers through the walk.
template <bool CULL>
__device__ void vis_item(const BatchParams& P, const DevScene& S, const GridView& G, int scene, int stage,
                         long long n0, long long m0) {
    const int lane = threadIdx.x & 31;
    const float* spos = stage == kVisBounce ? S.scat_pos : S.src_pos;
    const long long ns = stage == kVisBounce ? S.n_scat : S.n_src;
    const int* sid = stage == kVisBounce ? S.scat_id : nullptr;
    const float* kpos = stage == kVisScat ? S.scat_pos : P.snk_pos;
    const long long nk = stage == kVisScat ? S.n_scat : P.n_snk;
    const int* kid = stage == kVisScat ? S.scat_id : P.snk_id;
    const long long ms = m0 + lane;
    const bool ok = ms < nk;
    const long long rem = ns - n0;
    const int nsrc = (int)(rem < P.src_chunk ? rem : P.src_chunk);
    long long m_id = -1;
    float ex = 0.f, ey = 0.f, ez = 0.f;
    if (ok) {
        m_id = kid ? (long long)__ldg(kid + ms) : ms;
        ex = __ldg(kpos + 3 * ms);
        ey = __ldg(kpos + 3 * ms + 1);
        ez = __ldg(kpos + 3 * ms + 2);
    }
    unsigned long long vis = 0;
    unsigned int tests = 0;  // diagnostic count of one lane (64 rays at most); wraps only past 2^32 tests
    Walk w;
    for (int s = 0; s < nsrc; ++s) {
        if (!ok) continue;
        const long long n = n0 + s;
        const long long n_id = sid ? (long long)__ldg(sid + n) : n;
        if (P.skip_diag && n_id == m_id) {  // the pair is not tested: visible
            vis |= 1ull << s;
            continue;
        }
        const float* so = spos + 3 * n;
        if (!walk_begin<CULL>(G, w, __ldg(so), __ldg(so + 1), __ldg(so + 2), ex, ey, ez)) {
            vis |= 1ull << s;
            continue;
        }
        bool hit = false;
        while (true) {
            while (w.q < w.q1) {
                ++tests;
                if (walk_test<CULL>(G, w)) {
                    hit = true;
                    break;
                }
            }
            if (hit || !walk_step(G, w, P.err)) break;
        }
        if (!hit) vis |= 1ull << s;
    }
    if (ok) {
        unsigned int* row = S.mask[stage] + ms * S.mask_words[stage] + (n0 >> 5);
        row[0] = (unsigned int)vis;
        if (nsrc > 32) row[1] = (unsigned int)(vis >> 32);
    }
    if (P.counters) {
        const unsigned long long v = warp_sum((unsigned long long)__popcll(vis));
        const unsigned long long t = warp_sum((unsigned long long)tests);
        if (lane == 0) {
            atomicAdd(P.counters + 4LL * scene + stage, v);
            atomicAdd(P.counters + 4LL * scene + 3, t);
        }
    }
}

// ---------------------------------------------------------------- field items

// Adds one visible pair o -> (e, normal nrm) at frequencies f0 .. f0+cnt-1 to acc.
// Direct form (BOUNCE false): excitation E (6 floats) for every frequency.
// Bounce form: excitation and weight e_p(f) read from wrow[6 j .. 6 j + 5].
template <int FG, bool BOUNCE>
__device__ __forceinline__ void pair_freqs(const BatchParams& P, float ox, float oy, float oz, float ex, float ey,
                                           float ez, float nx, float ny, float nz, const float* E, const float* wrow,
                                           float2 b0, int f0, int cnt, float (&acc)[6 * FG]) {
    const Ray r = make_ray(ox, oy, oz, ex, ey, ez);
    const float inv_r = 1.0f / r.len;
    const float mag = expf(-P.alpha * r.len) * inv_r;
    const float a_re = -P.alpha - inv_r;
    const float nd = nx * r.dx + ny * r.dy + nz * r.dz;
    const float sc = -0.15915494309189535f * nd * mag;  // -(1/2pi) (n.d) exp(-alpha r)/r
    float rh, rl;
    ff_length(ox, oy, oz, ex, ey, ez, rh, rl);
    float sn, cs;
    sincosf(ff_phase(b0.x, b0.y, rh, rl), &sn, &cs);
    float cre = sc * cs, cim = -sc * sn;  // sc exp(-j beta_f0 r)
    float zre = 1.f, zim = 0.f;
    if (FG > 1) {
        float zs, zc;
        sincosf(ff_phase(P.dbeta_ff.x, P.dbeta_ff.y, rh, rl), &zs, &zc);
        zre = zc;
        zim = -zs;
    }
    float el[6];
    if (!BOUNCE) {  // E_L = E - (E.d) d, the same for every frequency
        const float ed_re = E[0] * r.dx + E[2] * r.dy + E[4] * r.dz;
        const float ed_im = E[1] * r.dx + E[3] * r.dy + E[5] * r.dz;
        el[0] = E[0] - ed_re * r.dx; el[1] = E[1] - ed_im * r.dx;
        el[2] = E[2] - ed_re * r.dy; el[3] = E[3] - ed_im * r.dy;
        el[4] = E[4] - ed_re * r.dz; el[5] = E[5] - ed_im * r.dz;
    }
#pragma unroll
    for (int j = 0; j < FG; ++j) {
        if (j < cnt) {
            const float b = __ldg(P.beta_f + f0 + j);
            // loss = (a_re - j beta) * c
            const float lre = a_re * cre + b * cim;
            const float lim = a_re * cim - b * cre;
            if (!BOUNCE) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    acc[6 * j + 2 * k] += el[2 * k] * lre - el[2 * k + 1] * lim;
                    acc[6 * j + 2 * k + 1] += el[2 * k] * lim + el[2 * k + 1] * lre;
                }
            } else {
                const float2 w0 = *reinterpret_cast<const float2*>(wrow + 6 * j);
                const float2 w1 = *reinterpret_cast<const float2*>(wrow + 6 * j + 2);
                const float2 w2 = *reinterpret_cast<const float2*>(wrow + 6 * j + 4);
                const float e[6] = {w0.x, w0.y, w1.x, w1.y, w2.x, w2.y};
                const float ed_re = e[0] * r.dx + e[2] * r.dy + e[4] * r.dz;
                const float ed_im = e[1] * r.dx + e[3] * r.dy + e[5] * r.dz;
                const float dd[3] = {r.dx, r.dy, r.dz};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float pr = e[2 * k] - ed_re * dd[k], pi = e[2 * k + 1] - ed_im * dd[k];
                    const float tr = pr * lre - pi * lim, ti = pr * lim + pi * lre;  // S2 component
                    acc[6 * j + 2 * k] += e[2 * k] * tr - e[2 * k + 1] * ti;      // weighted by e_p
                    acc[6 * j + 2 * k + 1] += e[2 * k] * ti + e[2 * k + 1] * tr;
                }
            }
            const float nre = cre * zre - cim * zim;
            cim = cre * zim + cim * zre;
            cre = nre;
        }
    }
}

// Sums the pairs of one stage into the thread's accumulator in shared memory
// (sacc[k * kBT + tid], k < 6 FG): per 32 sources in registers, then added.
template <int FG, bool BOUNCE>
__device__ __forceinline__ void field_stage(const BatchParams& P, const unsigned int* row, long long words,
                                            const float* spos, const float* src_E, const float* w, bool ok, float ex,
                                            float ey, float ez, float nx, float ny, float nz, float2 b0, int f0,
                                            int cnt, float* sacc) {
    const int tid = threadIdx.x;
    if (!ok) return;
    for (long long wi = 0; wi < words; ++wi) {
        unsigned int bits = row[wi];
        if (!bits) continue;
        float acc[6 * FG];
#pragma unroll
        for (int k = 0; k < 6 * FG; ++k) acc[k] = 0.f;
        while (bits) {
            const int j = __ffs(bits) - 1;
            bits &= bits - 1;
            const long long n = (wi << 5) + j;
            const float* so = spos + 3 * n;
            const float ox = __ldg(so), oy = __ldg(so + 1), oz = __ldg(so + 2);
            if (!BOUNCE) {
                float E[6];
                const float2* e2 = reinterpret_cast<const float2*>(src_E + 6 * n);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float2 v = __ldg(e2 + k);
                    E[2 * k] = v.x;
                    E[2 * k + 1] = v.y;
                }
                pair_freqs<FG, false>(P, ox, oy, oz, ex, ey, ez, nx, ny, nz, E, nullptr, b0, f0, cnt, acc);
            } else {
                const float* wrow = w + (n * P.n_freq + f0) * 6;
                pair_freqs<FG, true>(P, ox, oy, oz, ex, ey, ez, nx, ny, nz, nullptr, wrow, b0, f0, cnt, acc);
            }
        }
#pragma unroll
        for (int k = 0; k < 6 * FG; ++k) sacc[k * kBT + tid] += acc[k];
    }
}

// One warp's 32 consecutive slots (chunk of the scene's slot list).
template <int FG>
__device__ void field_item(const BatchParams& P, const DevScene& S, int scene, int kind, long long chunk,
                           float* sacc) {
    const int tid = threadIdx.x;
    const int G = P.n_groups;
    const bool at_sinks = kind == kFieldE;
    const long long nk = at_sinks ? P.n_snk : S.n_scat;
    const long long slot = chunk * 32 + (tid & 31);
    const long long ms = slot / G;
    const int g = (int)(slot - ms * G);
    const int f0 = g * FG;
    const int cnt = min(FG, P.n_freq - f0);
    const bool ok = ms < nk && cnt > 0;
#pragma unroll
    for (int k = 0; k < 6 * FG; ++k) sacc[k * kBT + tid] = 0.f;
    float ex = 0.f, ey = 0.f, ez = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    float2 b0 = make_float2(0.f, 0.f);
    if (ok) {
        const float* kp = (at_sinks ? P.snk_pos : S.scat_pos) + 3 * ms;
        const float* kn = (at_sinks ? P.snk_nrm : S.scat_nrm) + 3 * ms;
        ex = __ldg(kp); ey = __ldg(kp + 1); ez = __ldg(kp + 2);
        nx = __ldg(kn); ny = __ldg(kn + 1); nz = __ldg(kn + 2);
        b0 = __ldg(P.beta_ff + f0);
    }
    if (!at_sinks) {
        const long long words = S.mask_words[kVisScat];
        field_stage<FG, false>(P, S.mask[kVisScat] + ms * words, words, S.src_pos, S.src_E, nullptr, ok, ex, ey, ez,
                               nx, ny, nz, b0, f0, cnt, sacc);
        if (ok) {
            float* out = S.w + (ms * P.n_freq + f0) * 6;
            for (int k = 0; k < 6 * cnt; ++k) out[k] = sacc[k * kBT + tid];
        }
        return;
    }
    {
        const long long words = S.mask_words[kVisDirect];
        field_stage<FG, false>(P, S.mask[kVisDirect] + ms * words, words, S.src_pos, S.src_E, nullptr, ok, ex, ey,
                               ez, nx, ny, nz, b0, f0, cnt, sacc);
    }
    if (S.n_scat > 0) {
        const long long words = S.mask_words[kVisBounce];
        field_stage<FG, true>(P, S.mask[kVisBounce] + ms * words, words, S.scat_pos, nullptr, S.w, ok, ex, ey, ez,
                              nx, ny, nz, b0, f0, cnt, sacc);
    }
    if (ok) {
        const long long m = P.snk_id ? (long long)__ldg(P.snk_id + ms) : ms;
        for (int j = 0; j < cnt; ++j) {
            float* out = P.field + (((long long)scene * P.n_freq + f0 + j) * P.n_snk + m) * 6;
#pragma unroll
            for (int k = 0; k < 6; ++k) out[k] = sacc[(6 * j + k) * kBT + tid];
        }
    }
}

// ---------------------------------------------------------------- kernel

// MINB: blocks per SM the register allocation is capped for (1: uncapped).
// Each warp works on its own: lane 0 takes the next queue position while the
// warp works on the current item (the atomic's latency is hidden), so a warp
// holds one taken-but-unstarted item.  Progress still holds: the smallest
// unfinished queue position is always being worked on (its holder took it
// after every item it could be busy with), and it waits only on smaller
// positions, which are finished.
template <bool CULL, int FG, int MINB>
__global__ void __launch_bounds__(kBT, MINB) batch_kernel(const BatchParams P) {
    extern __shared__ float sacc[];
    __shared__ GridView s_grid[kBT / 32];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned nxt = 0;
    if (lane == 0) nxt = atomicAdd(P.head, 1u);
    while (true) {
        int kind = -1, scene = 0, a = 0, b = 0, run = 1;
        if (lane == 0) {
            const unsigned i = nxt;
            if (i < (unsigned)P.n_items) {
                const int4 it = P.items[i];
                kind = it.x;
                scene = it.y;
                a = it.z;
                b = it.w;
                nxt = atomicAdd(P.head, 1u);
                if (kind >= kFieldW && !wait_deps(P, kind, scene)) {
                    atomicOr(P.err, 1u);
                    run = 0;  // the item is skipped; its outputs are not valid
                }
                if (kind < kFieldW) s_grid[wid] = P.scenes[scene].grid;
            }
        }
        kind = __shfl_sync(full, kind, 0);
        scene = __shfl_sync(full, scene, 0);
        a = __shfl_sync(full, a, 0);
        b = __shfl_sync(full, b, 0);
        run = __shfl_sync(full, run, 0);
        __syncwarp();  // s_grid[wid] is visible to the warp
        if (kind < 0) break;
        if (run) {
            const DevScene& S = P.scenes[scene];
            if (kind < kFieldW)
                vis_item<CULL>(P, S, s_grid[wid], scene, kind, (long long)a, (long long)b);
            else
                for (int t = 0; t < b; ++t)  // b consecutive 32-slot chunks
                    field_item<FG>(P, S, scene, kind, (long long)a + t, sacc);
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) atomicAdd(P.done + (long long)scene * kKinds + kind, 1u);
    }
}

// ---------------------------------------------------------------- host plan

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Plan {
    std::vector<int4> items;
    std::vector<size_t> off_mask[3], off_w;
    std::vector<int> expect;  // [n_scenes][kKinds]
    size_t off_ctrl = 0, ctrl_bytes = 0, off_scenes = 0, off_items = 0, off_beta = 0, off_betaf = 0, total = 0;
};

bool config_ok(const lyem_batch_config* c) {
    if (!c) return false;
    if (!(c->freq_group == 1 || c->freq_group == 2 || c->freq_group == 4 || c->freq_group == 8)) return false;
    if (!(c->src_chunk == 32 || c->src_chunk == 64)) return false;
    if (c->blocks_per_sm < 0 || c->blocks_per_sm > 8) return false;
    if (!(c->eps >= 0.f) || !isfinite(c->eps) || !isfinite(c->alpha)) return false;
    return true;
}

// Items and workspace layout; a pure function of the sizes and the configuration.
int make_plan(const lyem_batch_scene* sc, int n_scenes, long long n_snk, int n_freq, const lyem_batch_config* cfg,
              Plan& pl) {
    if (!sc || n_scenes <= 0 || n_snk <= 0 || n_freq <= 0 || !config_ok(cfg)) return LYEM_ERR_INVALID;
    if (n_snk >= (1LL << 31) || n_freq > 4096) return LYEM_ERR_OVERFLOW;
    const int FG = cfg->freq_group;
    const long long groups = (n_freq + FG - 1) / FG;
    if ((n_snk * groups + 31) / 32 >= (1LL << 31)) return LYEM_ERR_OVERFLOW;  // 32-slot chunk index in an int
    const long long chunk = cfg->src_chunk;
    size_t off = 0;
    pl.off_ctrl = off;
    pl.ctrl_bytes = align256(sizeof(unsigned) * (1 + (size_t)n_scenes * kKinds));
    off += pl.ctrl_bytes;
    pl.off_scenes = off;
    off += align256(sizeof(DevScene) * (size_t)n_scenes);
    pl.off_beta = off;
    off += align256(sizeof(float2) * (size_t)n_freq);
    pl.off_betaf = off;
    off += align256(sizeof(float) * (size_t)n_freq);
    for (int k = 0; k < 3; ++k) pl.off_mask[k].assign(n_scenes, 0);
    pl.off_w.assign(n_scenes, 0);
    pl.expect.assign((size_t)n_scenes * kKinds, 0);
    // scenes in decreasing order of estimated work, so that the big ones start first
    std::vector<double> cost(n_scenes);
    std::vector<int> order(n_scenes);
    for (int s = 0; s < n_scenes; ++s) {
        const long long N = sc[s].n_src, P = sc[s].n_scat;
        if (N < 0 || P < 0 || N >= (1LL << 31) || P >= (1LL << 31)) return LYEM_ERR_INVALID;
        if (N > 0 && (!sc[s].src_pos || !sc[s].src_E)) return LYEM_ERR_INVALID;
        if (P > 0 && (!sc[s].scat_pos || !sc[s].scat_nrm)) return LYEM_ERR_INVALID;
        if (!sc[s].cell_start || !sc[s].cell_tris || (reinterpret_cast<uintptr_t>(sc[s].cell_tris) & 15u) ||
            !sc[s].cell_box || (reinterpret_cast<uintptr_t>(sc[s].cell_box) & 15u))
            return LYEM_ERR_INVALID;
        long long nc = 1;
        for (int k = 0; k < 3; ++k) {
            if (sc[s].grid_dims[k] < 1 || !isfinite(sc[s].grid_origin[k])) return LYEM_ERR_INVALID;
            nc *= sc[s].grid_dims[k];
        }
        if (!(sc[s].grid_cell > 0.f) || !isfinite(sc[s].grid_cell) || nc >= (1LL << 30)) return LYEM_ERR_INVALID;
        if ((P * groups + 31) / 32 >= (1LL << 31)) return LYEM_ERR_OVERFLOW;
        cost[s] = (double)N * (double)n_snk + (double)N * (double)P + (double)P * (double)n_snk;
        order[s] = s;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    for (int s = 0; s < n_scenes; ++s) {
        const long long N = sc[s].n_src, P = sc[s].n_scat;
        const long long wN = (N + 31) / 32, wP = (P + 31) / 32;
        pl.off_mask[kVisScat][s] = off;
        off += align256(sizeof(unsigned) * (size_t)(P * wN));
        pl.off_mask[kVisDirect][s] = off;
        off += align256(sizeof(unsigned) * (size_t)(n_snk * wN));
        pl.off_mask[kVisBounce][s] = off;
        off += align256(sizeof(unsigned) * (size_t)(n_snk * wP));
        pl.off_w[s] = off;
        off += align256(sizeof(float) * 6 * (size_t)P * (size_t)n_freq);
    }
    pl.items.clear();
    auto add_vis = [&](int s, int stage, long long ns, long long nk) {
        for (long long n0 = 0; n0 < ns; n0 += chunk)
            for (long long t = 0; t < nk; t += kWarpSinks) pl.items.push_back(make_int4(stage, s, (int)n0, (int)t));
        pl.expect[(size_t)s * kKinds + stage] =
            (int)(((ns + chunk - 1) / chunk) * ((nk + kWarpSinks - 1) / kWarpSinks));
    };
    for (int s : order) {
        const long long N = sc[s].n_src, P = sc[s].n_scat;
        add_vis(s, kVisScat, N, P);
        add_vis(s, kVisDirect, N, n_snk);
        add_vis(s, kVisBounce, P, n_snk);
    }
    // A field item is a run of 32-slot chunks (slot = point * groups + group),
    // long enough for about kItemPairs candidate (pair, group) evaluations, so
    // that scenes with few sources do not become very many tiny items.
    auto add_field = [&](int s, int kind, long long nk, long long pairs_per_sink) {
        const long long chunks = (nk * groups + 31) / 32;
        const long long per_chunk = std::max(1LL, pairs_per_sink * 32 / groups);
        const long long k = std::min(64LL, std::max(1LL, (kItemPairs + per_chunk - 1) / per_chunk));
        int count = 0;
        for (long long c = 0; c < chunks; c += k) {
            pl.items.push_back(make_int4(kind, s, (int)c, (int)std::min(k, chunks - c)));
            ++count;
        }
        pl.expect[(size_t)s * kKinds + kind] = count;
    };
    for (int s : order) add_field(s, kFieldW, sc[s].n_scat, sc[s].n_src);
    for (int s : order) add_field(s, kFieldE, n_snk, sc[s].n_src + sc[s].n_scat);
    if (pl.items.size() >= (size_t)0x7fffffff) return LYEM_ERR_OVERFLOW;
    pl.off_items = off;
    off += align256(sizeof(int4) * pl.items.size());
    pl.total = off;
    return LYEM_OK;
}

// beta as float-float, the uniform step, and whether the list is uniform
void beta_tables(const double* beta, int n, std::vector<float2>& ff, std::vector<float>& f32, float2& step,
                 bool& uniform) {
    ff.resize(n);
    f32.resize(n);
    for (int i = 0; i < n; ++i) {
        const float hi = (float)beta[i];
        ff[i] = make_float2(hi, (float)(beta[i] - (double)hi));
        f32[i] = hi;
    }
    const double d = n > 1 ? (beta[n - 1] - beta[0]) / (double)(n - 1) : 0.0;
    const float dh = (float)d;
    step = make_float2(dh, (float)(d - (double)dh));
    double bmax = 0.0, dev = 0.0;
    for (int i = 0; i < n; ++i) {
        bmax = std::max(bmax, fabs(beta[i]));
        dev = std::max(dev, fabs(beta[i] - (beta[0] + d * (double)i)));
    }
    uniform = dev <= 1e-12 * std::max(bmax, 1.0);
}

template <bool CULL, int FG, int MINB>
cudaError_t launch_batch_t(const BatchParams& P, int blocks_per_sm, cudaStream_t stream, int* blocks_out) {
    auto kern = batch_kernel<CULL, FG, MINB>;
    const size_t smem = sizeof(float) * 6 * FG * kBT;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int fit = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, kBT, smem);
    if (e != cudaSuccess) return e;
    const int per_sm = blocks_per_sm > 0 ? std::min(blocks_per_sm, std::max(fit, 1)) : std::max(fit, 1);
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorInvalidDevice;
    const int blocks = std::max(1, std::min(per_sm * sms, P.n_items));
    kern<<<blocks, kBT, smem, stream>>>(P);
    note_launches(1);
    if (blocks_out) *blocks_out = blocks;
    return cudaGetLastError();
}

template <bool CULL>
cudaError_t launch_batch_c(const BatchParams& P, int fg, int bps, cudaStream_t s, int* b) {
    // register-capped variants: 8 (32 registers) or 4 blocks per SM for up
    // to 4 frequencies per thread, also 6 (40 registers) for 2, 3 for 4 and 8;
    // other requests run the uncapped variant
    switch (fg) {
        case 1:
            if (bps == 8) return launch_batch_t<CULL, 1, 8>(P, bps, s, b);
            return bps == 4 ? launch_batch_t<CULL, 1, 4>(P, bps, s, b) : launch_batch_t<CULL, 1, 1>(P, bps, s, b);
        case 2:
            if (bps == 8) return launch_batch_t<CULL, 2, 8>(P, bps, s, b);
            if (bps == 6) return launch_batch_t<CULL, 2, 6>(P, bps, s, b);
            return bps == 4 ? launch_batch_t<CULL, 2, 4>(P, bps, s, b) : launch_batch_t<CULL, 2, 1>(P, bps, s, b);
        case 4:
            if (bps == 8) return launch_batch_t<CULL, 4, 8>(P, bps, s, b);
            if (bps == 4) return launch_batch_t<CULL, 4, 4>(P, bps, s, b);
            if (bps == 3) return launch_batch_t<CULL, 4, 3>(P, bps, s, b);
            return launch_batch_t<CULL, 4, 1>(P, bps, s, b);
        default: return bps == 3 ? launch_batch_t<CULL, 8, 3>(P, bps, s, b) : launch_batch_t<CULL, 8, 1>(P, bps, s, b);
    }
}

int fail(cudaError_t e) {
    record_cuda_error(e);
    return e == cudaErrorMemoryAllocation ? LYEM_ERR_NOMEM : LYEM_ERR_CUDA;
}

}  // namespace
}  // namespace lyem

using namespace lyem;

extern "C" {

LYEM_API size_t lyem_batch_workspace(const lyem_batch_scene* scenes, int32_t n_scenes, int64_t n_snk,
                                     int32_t n_freq, const lyem_batch_config* config) {
    Plan pl;
    if (make_plan(scenes, n_scenes, n_snk, n_freq, config, pl) != LYEM_OK) return 0;
    return pl.total;
}

LYEM_API int64_t lyem_batch_items(const lyem_batch_scene* scenes, int32_t n_scenes, int64_t n_snk, int32_t n_freq,
                                  const lyem_batch_config* config, int64_t* per_kind5) {
    Plan pl;
    const int st = make_plan(scenes, n_scenes, n_snk, n_freq, config, pl);
    if (st != LYEM_OK) return -(int64_t)st;
    if (per_kind5) {
        for (int k = 0; k < kKinds; ++k) per_kind5[k] = 0;
        for (const int4& it : pl.items) per_kind5[it.x] += 1;
    }
    return (int64_t)pl.items.size();
}

LYEM_API int lyem_batch_prepare(const lyem_batch_scene* scenes, int32_t n_scenes, int64_t n_snk,
                                const double* beta, int32_t n_freq, const lyem_batch_config* config, void* d_ws,
                                size_t ws_bytes, void* stream) {
    Plan pl;
    int st = make_plan(scenes, n_scenes, n_snk, n_freq, config, pl);
    if (st != LYEM_OK) return st;
    if (!beta) return LYEM_ERR_INVALID;
    for (int i = 0; i < n_freq; ++i)
        if (!isfinite(beta[i])) return LYEM_ERR_INVALID;
    std::vector<float2> ff;
    std::vector<float> f32;
    float2 step;
    bool uniform;
    beta_tables(beta, n_freq, ff, f32, step, uniform);
    if (config->freq_group > 1 && !uniform) return LYEM_ERR_INVALID;
    if (!d_ws || ws_bytes < pl.total || (reinterpret_cast<uintptr_t>(d_ws) & 255u)) return LYEM_ERR_WORKSPACE;
    char* base = static_cast<char*>(d_ws);
    std::vector<DevScene> ds(n_scenes);
    for (int s = 0; s < n_scenes; ++s) {
        const lyem_batch_scene& c = scenes[s];
        DevScene& d = ds[s];
        memset(&d, 0, sizeof(d));
        d.src_pos = c.src_pos;
        d.src_E = c.src_E;
        d.scat_pos = c.scat_pos;
        d.scat_nrm = c.scat_nrm;
        d.scat_id = c.scat_id;
        d.n_src = c.n_src;
        d.n_scat = c.n_scat;
        d.grid.cell_start = c.cell_start;
        d.grid.cell_tris = reinterpret_cast<const float4*>(c.cell_tris);
        d.grid.cell_box = reinterpret_cast<const float4*>(c.cell_box);
        for (int k = 0; k < 3; ++k) {
            d.grid.g0[k] = c.grid_origin[k];
            d.grid.g1[k] = c.grid_origin[k] + c.grid_dims[k] * c.grid_cell;
            d.grid.dims[k] = c.grid_dims[k];
        }
        d.grid.cell = c.grid_cell;
        d.grid.inv_cell = 1.0f / c.grid_cell;
        d.grid.eps = config->eps;
        const long long wN = (c.n_src + 31) / 32, wP = (c.n_scat + 31) / 32;
        for (int k = 0; k < 3; ++k) d.mask[k] = reinterpret_cast<unsigned int*>(base + pl.off_mask[k][s]);
        d.mask_words[kVisScat] = wN;
        d.mask_words[kVisDirect] = wN;
        d.mask_words[kVisBounce] = wP;
        d.w = reinterpret_cast<float*>(base + pl.off_w[s]);
        for (int k = 0; k < kKinds; ++k) d.expect[k] = pl.expect[(size_t)s * kKinds + k];
    }
    cudaStream_t strm = reinterpret_cast<cudaStream_t>(stream);
    auto put = [&](size_t off, const void* src, size_t bytes) -> cudaError_t {
        if (bytes == 0) return cudaSuccess;
        return cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, strm);
    };
    cudaError_t e;
    if ((e = put(pl.off_scenes, ds.data(), sizeof(DevScene) * ds.size())) != cudaSuccess) return fail(e);
    if ((e = put(pl.off_items, pl.items.data(), sizeof(int4) * pl.items.size())) != cudaSuccess) return fail(e);
    if ((e = put(pl.off_beta, ff.data(), sizeof(float2) * ff.size())) != cudaSuccess) return fail(e);
    if ((e = put(pl.off_betaf, f32.data(), sizeof(float) * f32.size())) != cudaSuccess) return fail(e);
    // the host tables are released on return: finish the copies first
    if ((e = cudaStreamSynchronize(strm)) != cudaSuccess) return fail(e);
    return LYEM_OK;
}

LYEM_API int lyem_batch_launch(const lyem_batch_scene* scenes, int32_t n_scenes, const float* d_snk_pos,
                               const float* d_snk_nrm, const int32_t* d_snk_id, int64_t n_snk, const double* beta,
                               int32_t n_freq, const lyem_batch_config* config, void* d_ws, size_t ws_bytes,
                               float* d_field_out, uint64_t* d_counters, int32_t* blocks_out, void* stream) {
    Plan pl;
    int st = make_plan(scenes, n_scenes, n_snk, n_freq, config, pl);
    if (st != LYEM_OK) return st;
    if (!beta || !d_snk_pos || !d_snk_nrm || !d_field_out || ((uintptr_t)d_field_out & 7u)) return LYEM_ERR_INVALID;
    if (!d_ws || ws_bytes < pl.total || (reinterpret_cast<uintptr_t>(d_ws) & 255u)) return LYEM_ERR_WORKSPACE;
    std::vector<float2> ff;
    std::vector<float> f32;
    float2 step;
    bool uniform;
    beta_tables(beta, n_freq, ff, f32, step, uniform);
    if (config->freq_group > 1 && !uniform) return LYEM_ERR_INVALID;
    char* base = static_cast<char*>(d_ws);
    cudaStream_t strm = reinterpret_cast<cudaStream_t>(stream);
    BatchParams P;
    memset(&P, 0, sizeof(P));
    P.scenes = reinterpret_cast<const DevScene*>(base + pl.off_scenes);
    P.items = reinterpret_cast<const int4*>(base + pl.off_items);
    P.n_items = (int)pl.items.size();
    P.n_scenes = n_scenes;
    P.head = reinterpret_cast<unsigned int*>(base + pl.off_ctrl);
    P.done = P.head + 1;
    P.snk_pos = d_snk_pos;
    P.snk_nrm = d_snk_nrm;
    P.snk_id = d_snk_id;
    P.n_snk = n_snk;
    P.beta_ff = reinterpret_cast<const float2*>(base + pl.off_beta);
    P.beta_f = reinterpret_cast<const float*>(base + pl.off_betaf);
    P.dbeta_ff = step;
    P.n_freq = n_freq;
    P.n_groups = (n_freq + config->freq_group - 1) / config->freq_group;
    P.src_chunk = config->src_chunk;
    P.alpha = (float)config->alpha;
    P.skip_diag = config->self_to_self ? 0 : 1;
    P.err = device_error_word();
    P.counters = reinterpret_cast<unsigned long long*>(d_counters);
    P.field = d_field_out;
    cudaError_t e = cudaMemsetAsync(base + pl.off_ctrl, 0, pl.ctrl_bytes, strm);
    if (e != cudaSuccess) return fail(e);
    if (d_counters) {
        e = cudaMemsetAsync(d_counters, 0, sizeof(uint64_t) * 4 * (size_t)n_scenes, strm);
        if (e != cudaSuccess) return fail(e);
    }
    int blocks = 0;
    e = config->cull ? launch_batch_c<true>(P, config->freq_group, config->blocks_per_sm, strm, &blocks)
                     : launch_batch_c<false>(P, config->freq_group, config->blocks_per_sm, strm, &blocks);
    if (e != cudaSuccess) return fail(e);
    if (blocks_out) *blocks_out = blocks;
    return LYEM_OK;
}

}  // extern "C"
