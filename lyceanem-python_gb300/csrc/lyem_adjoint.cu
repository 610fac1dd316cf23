// lyem_adjoint.cu -- reverse-mode derivatives of the direct + one-bounce sink field.
//
// Forward model (the composition of lyceanem/models/frequency_domain.py:195-264
// summed over sources, :847-849), with element n excited by a_n e_n (e_n a fixed
// complex polarisation, a_n a complex scalar) and visibility held fixed:
//   E[m] = sum_n a_n G0[n,m] + sum_p w_p (.) (B_pm w_p),  w_p = sum_n a_n G1[n,p],
//   G[s,t] = vis(s,t) L_st P(d_st) e_s,  B_pm w = vis(p,m) L_pm P(d_pm) w,
//   L_st = F(r) (n_t . d),  F(r) = -(1/2pi) (-alpha - 1/r - j beta) e^{-(alpha + j beta) r} / r
// (em_wave / ray_launch, lyceanem/src/em.cuh:18-120; P(d) = I - d d^T projects
// onto the plane normal to the ray).  Given the cotangent g = dL/dE* of a real
// loss (torch convention: grad = dL/dRe + j dL/dIm) the kernels return
//   grad a_n = sum_m G0[n,m]^H g_m + sum_p G1[n,p]^H Z_p
//   grad x_n = -Re( conj(a_n) [ sum_m J(n,m; e_n, g_m) + sum_p J(n,p; e_n, Z_p) ] )
//   grad y_m =  Re( sum_n conj(a_n) J(n,m; e_n, g_m) + sum_p J(p,m; w_p, conj(w_p) (.) g_m) )
// with Z_p = sum_m conj(L_pm) [ conj(P w_p) (.) g_m + P (conj(w_p) (.) g_m) ] and
// J_j(s,t; e, Y) = sum_c conj(d G_c / d r_j) Y_c for G = F(r) (n_t . d) P(d) e,
// r = t - s, evaluated analytically.  The phase beta*r is recomputed per pair
// in float-float (ff_length, ff_phase: r to about 1e-14 relative, the reduced
// phase to a few 1e-7 rad, as the forward's FP64 reduction rounded to FP32);
// FP64 would bound these kernels (86 % FP64-pipe activity on the
// differentiation scene).  Nothing of size N x M is stored (the N x M masks
// are bits).  Each kernel assigns one "owner" point per thread and a chunk of
// partners per block row; chunk partial sums are reduced in FP64.
#include <cuda_runtime.h>

#include "lyem.h"
#include "lyem_device.cuh"
#include "lyem_internal.cuh"

namespace lyem {
namespace {

constexpr int kAdjThreads = 128;
constexpr int kAdjChunk = 256;

struct cpx {
    float x, y;
};
__device__ __forceinline__ cpx cmul(cpx a, cpx b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cpx conjc(cpx a) { return {a.x, -a.y}; }
__device__ __forceinline__ cpx cadd(cpx a, cpx b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cpx cscale(cpx a, float s) { return {a.x * s, a.y * s}; }

struct PairGeo {
    float dx, dy, dz, r, s;  // unit direction, length, n_t . d
    cpx F, Fp;               // F(r) and dF/dr
};

// Geometry and radial factors of the ray s -> t (normal n at t).
__device__ __forceinline__ PairGeo pair_geo(float ox, float oy, float oz, float tx, float ty, float tz, float nx,
                                            float ny, float nz, float alpha, float beta_f, float beta_lo) {
    Ray ray = make_ray(ox, oy, oz, tx, ty, tz);
    float rh, rl;
    ff_length(ox, oy, oz, tx, ty, tz, rh, rl);
    const float ph = ff_phase(beta_f, beta_lo, rh, rl);
    float sn, cs;
    sincosf(ph, &sn, &cs);
    const float r = ray.len, ir = 1.0f / r;
    const float mag = expf(-alpha * r);
    const cpx ex = {mag * cs, -mag * sn};  // e^{-kappa r}
    const cpx kap = {alpha, beta_f};
    const float front = -0.15915494309189535f;
    // F = front * h, h = -(kappa/r + 1/r^2) e^{-kappa r}
    cpx h = cmul(cpx{-(kap.x * ir + ir * ir), -kap.y * ir}, ex);
    // dh/dr = (kappa^2/r + 2 kappa/r^2 + 2/r^3) e^{-kappa r}
    const cpx k2 = {kap.x * kap.x - kap.y * kap.y, 2.f * kap.x * kap.y};
    cpx hp = cmul(cpx{k2.x * ir + 2.f * kap.x * ir * ir + 2.f * ir * ir * ir, k2.y * ir + 2.f * kap.y * ir * ir}, ex);
    PairGeo g;
    g.dx = ray.dx; g.dy = ray.dy; g.dz = ray.dz; g.r = r;
    g.s = nx * ray.dx + ny * ray.dy + nz * ray.dz;
    g.F = cscale(h, front);
    g.Fp = cscale(hp, front);
    return g;
}

// q = e - (e.d) d for a complex 3-vector e.
__device__ __forceinline__ void project(const PairGeo& g, const cpx* e, cpx* q, cpx* ed) {
    *ed = {e[0].x * g.dx + e[1].x * g.dy + e[2].x * g.dz, e[0].y * g.dx + e[1].y * g.dy + e[2].y * g.dz};
    const float d[3] = {g.dx, g.dy, g.dz};
#pragma unroll
    for (int c = 0; c < 3; ++c) q[c] = {e[c].x - ed->x * d[c], e[c].y - ed->y * d[c]};
}

// J_j = sum_c conj(dG_c/dr_j) Y_c for G = F s P(d) e (see the file comment).
__device__ __forceinline__ void jac(const PairGeo& g, float nx, float ny, float nz, const cpx* e, const cpx* Y,
                                    cpx* J) {
    cpx q[3], ed;
    project(g, e, q, &ed);
    const float d[3] = {g.dx, g.dy, g.dz}, n[3] = {nx, ny, nz};
    cpx qY = {0.f, 0.f}, dY = {0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        qY = cadd(qY, cmul(conjc(q[c]), Y[c]));
        dY = cadd(dY, cscale(Y[c], d[c]));
    }
    const float ir = 1.0f / g.r;
    const cpx cF = conjc(g.F), cFp = conjc(g.Fp), ced = conjc(ed);
    const cpx a1 = cscale(cmul(cFp, qY), g.s);  // times d_j
    const cpx a2 = cscale(cmul(cF, qY), ir);    // times (n_j - s d_j)
    const cpx a3 = cscale(cF, -g.s * ir);       // times [conj(q_j) dY + conj(ed) (Y_j - d_j dY)]
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        cpx t = cadd(cmul(conjc(q[j]), dY), cmul(ced, cpx{Y[j].x - d[j] * dY.x, Y[j].y - d[j] * dY.y}));
        J[j] = cadd(cadd(cscale(a1, d[j]), cscale(a2, n[j] - g.s * d[j])), cmul(a3, t));
    }
}

__device__ __forceinline__ void load3(const float* base, long long i, cpx* v) {
    const float2* p = reinterpret_cast<const float2*>(base + 6 * i);
    float2 a = p[0], b = p[1], c = p[2];
    v[0] = {a.x, a.y};
    v[1] = {b.x, b.y};
    v[2] = {c.x, c.y};
}

__device__ __forceinline__ bool mask_bit(const unsigned* bits, long long words, long long row, long long col) {
    return (__ldg(bits + row * words + (col >> 5)) >> (col & 31)) & 1u;
}

struct AdjParams {
    const float* src_pos;  // [N,3]
    const float* src_pol;  // [N,6] e_n
    const float* src_a;    // [N,2] a_n
    long long N;
    const float* scat_pos;  // [P,3]
    const float* scat_nrm;  // [P,3]
    const float* scat_w;    // [P,6] w_p
    const float* scat_z;    // [P,6] Z_p (input of the source and sink kernels)
    long long P;
    const float* snk_pos;  // [M,3]
    const float* snk_nrm;  // [M,3]
    const float* grad_E;   // [M,6] cotangent g
    long long M;
    const unsigned* mask0;  // [N, ceil(M/32)]
    const unsigned* mask1;  // [N, ceil(P/32)]
    const unsigned* mask2;  // [P, ceil(M/32)]
    float alpha, beta_f, beta_lo;  // beta = beta_f + beta_lo (float-float)
    float* partial;
};

// Z_p: owner = scatter point p, partners = sinks.
__global__ void __launch_bounds__(kAdjThreads) adjoint_scatter_kernel(const AdjParams a) {
    const long long p = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
    const bool ok = p < a.P;
    const long long m0 = (long long)blockIdx.y * kAdjChunk;
    const long long m1 = m0 + kAdjChunk < a.M ? m0 + kAdjChunk : a.M;
    const long long wM = (a.M + 31) / 32;
    cpx Z[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (ok) {
        const float ox = a.scat_pos[3 * p], oy = a.scat_pos[3 * p + 1], oz = a.scat_pos[3 * p + 2];
        cpx w[3], cw[3];
        load3(a.scat_w, p, w);
        for (int c = 0; c < 3; ++c) cw[c] = conjc(w[c]);
        for (long long m = m0; m < m1; ++m) {
            if (!mask_bit(a.mask2, wM, p, m)) continue;
            const PairGeo g = pair_geo(ox, oy, oz, a.snk_pos[3 * m], a.snk_pos[3 * m + 1], a.snk_pos[3 * m + 2],
                                       a.snk_nrm[3 * m], a.snk_nrm[3 * m + 1], a.snk_nrm[3 * m + 2], a.alpha,
                                       a.beta_f, a.beta_lo);
            cpx gm[3], y[3], q[3], qy[3], ed, yd;
            load3(a.grad_E, m, gm);
            project(g, w, q, &ed);
            for (int c = 0; c < 3; ++c) y[c] = cmul(cw[c], gm[c]);
            project(g, y, qy, &yd);
            const cpx cL = cscale(conjc(g.F), g.s);
            for (int c = 0; c < 3; ++c) Z[c] = cadd(Z[c], cmul(cL, cadd(cmul(conjc(q[c]), gm[c]), qy[c])));
        }
        float2* o = reinterpret_cast<float2*>(a.partial + 6 * ((long long)blockIdx.y * a.P + p));
        for (int c = 0; c < 3; ++c) o[c] = make_float2(Z[c].x, Z[c].y);
    }
}

// grad a_n (complex) and the position sum J (3 complex): owner = source n,
// partners = sinks [0, M) then scatter points [M, M + P).
__global__ void __launch_bounds__(kAdjThreads) adjoint_source_kernel(const AdjParams a) {
    const long long n = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
    const bool ok = n < a.N;
    const long long j0 = (long long)blockIdx.y * kAdjChunk;
    const long long jn = a.M + a.P;
    const long long j1 = j0 + kAdjChunk < jn ? j0 + kAdjChunk : jn;
    const long long wM = (a.M + 31) / 32, wP = (a.P + 31) / 32;
    cpx ga = {0.f, 0.f}, J[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (ok) {
        const float ox = a.src_pos[3 * n], oy = a.src_pos[3 * n + 1], oz = a.src_pos[3 * n + 2];
        cpx e[3];
        load3(a.src_pol, n, e);
        for (long long j = j0; j < j1; ++j) {
            const bool is_snk = j < a.M;
            const long long t = is_snk ? j : j - a.M;
            if (is_snk ? !mask_bit(a.mask0, wM, n, t) : !mask_bit(a.mask1, wP, n, t)) continue;
            const float* tp = is_snk ? a.snk_pos : a.scat_pos;
            const float* tn = is_snk ? a.snk_nrm : a.scat_nrm;
            const float nx = tn[3 * t], ny = tn[3 * t + 1], nz = tn[3 * t + 2];
            const PairGeo g = pair_geo(ox, oy, oz, tp[3 * t], tp[3 * t + 1], tp[3 * t + 2], nx, ny, nz, a.alpha,
                                       a.beta_f, a.beta_lo);
            cpx Y[3], q[3], ed, jj[3];
            load3(is_snk ? a.grad_E : a.scat_z, t, Y);
            project(g, e, q, &ed);
            cpx qY = {0.f, 0.f};
            for (int c = 0; c < 3; ++c) qY = cadd(qY, cmul(conjc(q[c]), Y[c]));
            ga = cadd(ga, cmul(cscale(conjc(g.F), g.s), qY));
            jac(g, nx, ny, nz, e, Y, jj);
            for (int c = 0; c < 3; ++c) J[c] = cadd(J[c], jj[c]);
        }
        float* o = a.partial + 8 * ((long long)blockIdx.y * a.N + n);
        o[0] = ga.x; o[1] = ga.y;
        for (int c = 0; c < 3; ++c) { o[2 + 2 * c] = J[c].x; o[3 + 2 * c] = J[c].y; }
    }
}

// grad y_m: owner = sink m, partners = sources [0, N) then scatter points [N, N + P).
__global__ void __launch_bounds__(kAdjThreads) adjoint_sink_kernel(const AdjParams a) {
    const long long m = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
    const bool ok = m < a.M;
    const long long j0 = (long long)blockIdx.y * kAdjChunk;
    const long long jn = a.N + a.P;
    const long long j1 = j0 + kAdjChunk < jn ? j0 + kAdjChunk : jn;
    const long long wM = (a.M + 31) / 32;
    float gy[3] = {0.f, 0.f, 0.f};
    if (ok) {
        const float tx = a.snk_pos[3 * m], ty = a.snk_pos[3 * m + 1], tz = a.snk_pos[3 * m + 2];
        const float nx = a.snk_nrm[3 * m], ny = a.snk_nrm[3 * m + 1], nz = a.snk_nrm[3 * m + 2];
        cpx gm[3];
        load3(a.grad_E, m, gm);
        for (long long j = j0; j < j1; ++j) {
            const bool is_src = j < a.N;
            const long long s = is_src ? j : j - a.N;
            if (!mask_bit(is_src ? a.mask0 : a.mask2, wM, s, m)) continue;
            const float* sp = is_src ? a.src_pos : a.scat_pos;
            const PairGeo g = pair_geo(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2], tx, ty, tz, nx, ny, nz, a.alpha,
                                       a.beta_f, a.beta_lo);
            cpx e[3], Y[3], J[3];
            if (is_src) {
                load3(a.src_pol, s, e);
                for (int c = 0; c < 3; ++c) Y[c] = gm[c];
            } else {
                load3(a.scat_w, s, e);
                for (int c = 0; c < 3; ++c) Y[c] = cmul(conjc(e[c]), gm[c]);
            }
            jac(g, nx, ny, nz, e, Y, J);
            cpx f = {1.f, 0.f};
            if (is_src) f = conjc(cpx{a.src_a[2 * s], a.src_a[2 * s + 1]});
            for (int c = 0; c < 3; ++c) gy[c] += cmul(f, J[c]).x;
        }
        float* o = a.partial + 3 * ((long long)blockIdx.y * a.M + m);
        for (int c = 0; c < 3; ++c) o[c] = gy[c];
    }
}

__global__ void reduce_elems_kernel(const float* __restrict__ partial, long long chunks, long long n_elem,
                                    float* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_elem;
         i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (long long c = 0; c < chunks; ++c) s += (double)partial[c * n_elem + i];
        out[i] = (float)s;
    }
}

// grad a_n = partial sum; grad x_n = -Re(conj(a_n) J)
__global__ void finish_source_kernel(const float* __restrict__ acc, const float* __restrict__ src_a, long long N,
                                     float* __restrict__ grad_a, float* __restrict__ grad_x) {
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const float* v = acc + 8 * n;
        grad_a[2 * n] = v[0];
        grad_a[2 * n + 1] = v[1];
        const float ar = src_a[2 * n], ai = src_a[2 * n + 1];
        for (int c = 0; c < 3; ++c) grad_x[3 * n + c] = -(ar * v[2 + 2 * c] + ai * v[3 + 2 * c]);
    }
}

unsigned blocks_1d(long long n) { return capped_blocks(n, 256, 16); }

long long chunks_of(long long n) { return (n + kAdjChunk - 1) / kAdjChunk; }

}  // namespace
}  // namespace lyem

using namespace lyem;

extern "C" {

LYEM_API size_t lyem_adjoint_workspace(int64_t n_src, int64_t n_scat, int64_t n_snk) {
    if (n_src < 0 || n_scat < 0 || n_snk < 0) return 0;
    const size_t a = (size_t)chunks_of(n_snk) * n_scat * 6;
    const size_t b = (size_t)chunks_of(n_snk + n_scat) * n_src * 8 + (size_t)n_src * 8;
    const size_t c = (size_t)chunks_of(n_src + n_scat) * n_snk * 3;
    size_t m = a > b ? a : b;
    m = m > c ? m : c;
    return m * sizeof(float) + 256;
}

LYEM_API int lyem_adjoint(const float* d_src_pos, const float* d_src_pol, const float* d_src_a, int64_t n_src,
                          const float* d_scat_pos, const float* d_scat_nrm, const float* d_scat_w, int64_t n_scat,
                          const float* d_snk_pos, const float* d_snk_nrm, const float* d_grad_E, int64_t n_snk,
                          const uint32_t* d_mask0, const uint32_t* d_mask1, const uint32_t* d_mask2, double alpha,
                          double beta, float* d_grad_a, float* d_grad_x, float* d_grad_y, float* d_scat_z,
                          void* d_ws, size_t ws_bytes, void* stream) {
    if (n_src < 0 || n_scat < 0 || n_snk < 0) return LYEM_ERR_INVALID;
    if (n_src == 0 || n_snk == 0) return LYEM_OK;
    if (!d_src_pos || !d_src_pol || !d_src_a || !d_snk_pos || !d_snk_nrm || !d_grad_E || !d_mask0)
        return LYEM_ERR_INVALID;
    if (n_scat > 0 && (!d_scat_pos || !d_scat_nrm || !d_scat_w || !d_mask1 || !d_mask2 || !d_scat_z))
        return LYEM_ERR_INVALID;
    if ((d_grad_a == nullptr) != (d_grad_x == nullptr)) return LYEM_ERR_INVALID;
    if (!d_ws || ws_bytes < lyem_adjoint_workspace(n_src, n_scat, n_snk)) return LYEM_ERR_WORKSPACE;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    AdjParams a;
    a.src_pos = d_src_pos; a.src_pol = d_src_pol; a.src_a = d_src_a; a.N = n_src;
    a.scat_pos = d_scat_pos; a.scat_nrm = d_scat_nrm; a.scat_w = d_scat_w; a.scat_z = d_scat_z; a.P = n_scat;
    a.snk_pos = d_snk_pos; a.snk_nrm = d_snk_nrm; a.grad_E = d_grad_E; a.M = n_snk;
    a.mask0 = d_mask0; a.mask1 = d_mask1; a.mask2 = d_mask2;
    a.alpha = (float)alpha; a.beta_f = (float)beta; a.beta_lo = (float)(beta - (double)a.beta_f);
    a.partial = static_cast<float*>(d_ws);
    if (n_scat > 0) {
        dim3 g((unsigned)((n_scat + kAdjThreads - 1) / kAdjThreads), (unsigned)chunks_of(n_snk));
        adjoint_scatter_kernel<<<g, kAdjThreads, 0, s>>>(a); note_launches(1);
        reduce_elems_kernel<<<blocks_1d(6 * n_scat), 256, 0, s>>>(a.partial, chunks_of(n_snk), 6 * n_scat, d_scat_z); note_launches(1);
    }
    if (d_grad_a) {
        const long long ch = chunks_of(n_snk + n_scat);
        dim3 g((unsigned)((n_src + kAdjThreads - 1) / kAdjThreads), (unsigned)ch);
        adjoint_source_kernel<<<g, kAdjThreads, 0, s>>>(a); note_launches(1);
        float* acc = a.partial + (size_t)ch * n_src * 8;
        reduce_elems_kernel<<<blocks_1d(8 * n_src), 256, 0, s>>>(a.partial, ch, 8 * n_src, acc); note_launches(1);
        finish_source_kernel<<<blocks_1d(n_src), 256, 0, s>>>(acc, d_src_a, n_src, d_grad_a, d_grad_x); note_launches(1);
    }
    if (d_grad_y) {
        const long long ch = chunks_of(n_src + n_scat);
        dim3 g((unsigned)((n_snk + kAdjThreads - 1) / kAdjThreads), (unsigned)ch);
        adjoint_sink_kernel<<<g, kAdjThreads, 0, s>>>(a); note_launches(1);
        reduce_elems_kernel<<<blocks_1d(3 * n_snk), 256, 0, s>>>(a.partial, ch, 3 * n_snk, d_grad_y); note_launches(1);
    }
    return cudaGetLastError() == cudaSuccess ? LYEM_OK : LYEM_ERR_CUDA;
}

}  // extern "C"
