// lyem_device.cuh -- device arithmetic shared by every kernel of the library.
//
// Visibility arithmetic is fully specified: each operation is an IEEE binary32
// operation with round-to-nearest, written with the __f*_rn intrinsics so the
// compiler can neither contract nor reorder it.  The CPU oracle performs the
// same sequence with fmaf() under -ffp-contract=off, so masks agree bit for
// bit.  The operation order follows the reference formulas:
//   points_to_rays   lyceanem/src/raycasting.cuh:80-95
//   hit              lyceanem/src/raycasting.cuh:19-68 (cull) and
//                    lyceanem/raycasting/rayfunctions.py:37-104 (no cull)
//   cross/dot        contracted as fma(a, b, -(c*d)) and fma(z, z, fma(y, y, x*x))
// The reference computes F = 1.0/A in double and rounds to float; with a
// 53-bit intermediate for a 24-bit quotient that double rounding is innocuous,
// so F equals the correctly rounded FP32 reciprocal __frcp_rn(A).
//
// The field follows em_wave/ray_launch (lyceanem/src/em.cuh:18-120) in FP32
// except the phase beta*r, which is formed from FP64 differences of the input
// coordinates and reduced modulo 2*pi in FP64 before the FP32 sincos.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lyem {

constexpr float kEpsilon = 0.000001f;  // lyceanem/src/math_utility.cuh:9

struct Ray {
    float dx, dy, dz, len;
};

__device__ __forceinline__ Ray make_ray(float ox, float oy, float oz, float ex, float ey, float ez) {
    float rx = __fsub_rn(ex, ox), ry = __fsub_rn(ey, oy), rz = __fsub_rn(ez, oz);
    float w2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
    float w = __fsqrt_rn(w2);
    Ray r;
    r.dx = __fdiv_rn(rx, w);
    r.dy = __fdiv_rn(ry, w);
    r.dz = __fdiv_rn(rz, w);
    r.len = w;
    return r;
}

// The numba engine's ray set-up (charge_rays_environment1Dv2 -> calc_dv_norm,
// lyceanem/raycasting/rayfunctions.py:1790-1842, lyceanem/utility/math_functions.py:149-156):
// numpy float32 arithmetic on the host, nothing fused: the squared length is
// ((rx*rx + ry*ry) + rz*rz) with every step rounded, then sqrt and one division
// per component.
__device__ __forceinline__ Ray make_ray_numba(float ox, float oy, float oz, float ex, float ey, float ez) {
    float rx = __fsub_rn(ex, ox), ry = __fsub_rn(ey, oy), rz = __fsub_rn(ez, oz);
    float w2 = __fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz));
    float w = __fsqrt_rn(w2);
    Ray r;
    r.dx = __fdiv_rn(rx, w);
    r.dy = __fdiv_rn(ry, w);
    r.dz = __fdiv_rn(rz, w);
    r.len = w;
    return r;
}

// Ray of a visibility test: the CUDA engine's set-up in the culling mode, the
// numba engine's in the non-culling mode (the mode that reproduces that engine).
template <bool CULL>
__device__ __forceinline__ Ray vis_ray(float ox, float oy, float oz, float ex, float ey, float ez) {
    return CULL ? make_ray(ox, oy, oz, ex, ey, ez) : make_ray_numba(ox, oy, oz, ex, ey, ez);
}

// Per (source, triangle) quantities of the Moller-Trumbore test that do not
// depend on the ray direction: tvec = o - v0, qvec = tvec x e1, tq = e2 . qvec.
// Computing them once per source and reusing them gives the same bits as
// recomputing them per test.
struct TriPre {
    float4 a;  // e1.x e1.y e1.z e2.x
    float4 b;  // e2.y e2.z t.x t.y
    float4 c;  // t.z q.x q.y q.z
    float4 d;  // tq  -    -   -
};

__device__ __forceinline__ TriPre make_tripre(float ox, float oy, float oz, float4 v0, float4 e1, float4 e2) {
    float tx = __fsub_rn(ox, v0.x), ty = __fsub_rn(oy, v0.y), tz = __fsub_rn(oz, v0.z);
    float qx = __fmaf_rn(ty, e1.z, -__fmul_rn(tz, e1.y));
    float qy = __fmaf_rn(tz, e1.x, -__fmul_rn(tx, e1.z));
    float qz = __fmaf_rn(tx, e1.y, -__fmul_rn(ty, e1.x));
    float tq = __fmaf_rn(e2.z, qz, __fmaf_rn(e2.y, qy, __fmul_rn(e2.x, qx)));
    TriPre p;
    p.a = make_float4(e1.x, e1.y, e1.z, e2.x);
    p.b = make_float4(e2.y, e2.z, tx, ty);
    p.c = make_float4(tz, qx, qy, qz);
    p.d = make_float4(tq, 0.f, 0.f, 0.f);
    return p;
}

template <bool CULL>
__device__ __forceinline__ bool det_rejects(float A, float eps) {
    if (CULL) return !(A >= eps);  // |A| < eps or A < 0 (NaN also rejected; the reference returns 0 for it later)
    return fabsf(A) < eps;
}

// Guard band of the barycentric checks (used by hit_full's culling test, where
// A >= eps >= 0).  With F = rn(1/A) (relative error at most 2^-24) and x the
// unscaled numerator (u = t.p or v = d.q):
//   x < rn(A * -2^-20)          =>  rn(F*x) < -2^-21 < 0
//   x > rn(A + A 2^-19)          =>  F*x > (1 + 2^-20)(1 - 2^-24) > 1 + 2^-21, so rn(F*x) > 1
// so a test whose numerator lies there fails the reference's U (or V) check
// without the reciprocal being formed; for V > 1, U + V > 1 follows as U >= 0.
// With A = +-0 (eps = 0) F is infinite and every nonzero numerator fails there
// as well.  NaN numerators fail both comparisons and go on to cull_tail.

// The numba engine's decisions after the determinant (rayfunctions.py:55-100):
// there F = 1.0 / A, U = F u, V = F v and t = F w are FP64 (the float64 literal
// promotes the float32 determinant) and are compared in FP64.  With u, v and A
// float32 (A != 0), the U and V sign tests and U > 1 are exact FP32 comparisons:
//   F u < 0  <=>  u / A < 0: no FP64 product of float32-derived values
//             underflows, so the sign survives rounding (u = +-0 gives +-0);
//   F u > 1  <=>  s u > |A| (s = sign A): for float32 u != A of one sign,
//             |u / A - 1| >= 2^-25, far beyond the 2^-52 relative error of F u,
//             and u == A gives F u in {1, 1 - 2^-53}.
// U + V > 1 and the t range are evaluated in FP64 as there.  A NaN numerator
// fails every comparison, as in FP64; with a NaN determinant numba's t is NaN
// and the test is a miss, which an early miss here matches.
__device__ __forceinline__ bool ratio_negative(float x, float A) { return A < 0.f ? x > 0.f : x < 0.f; }
__device__ __forceinline__ bool ratio_above_one(float x, float A) { return (A < 0.f ? -x : x) > fabsf(A); }

__device__ __forceinline__ bool numba_tail(float A, float u, float v, float w, float len, float eps) {
    const double F = 1.0 / (double)A;
    const double U = F * (double)u, V = F * (double)v;
    if (U + V > 1.0) return false;
    const double t = F * (double)w;
    const double two_eps = 2.0 * (double)eps;
    return (t > two_eps) && (t < (double)len - two_eps);
}

// IEEE binary32 round-to-nearest operations usable on the host as well (the
// host build is for tests of the decision logic below; compile host code with
// -ffp-contract=off).
namespace rn {
__host__ __device__ __forceinline__ float mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float rcp(float a) {
#ifdef __CUDA_ARCH__
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}
}  // namespace rn

// The culling test's decisions after the determinant, as the reference makes
// them (lyceanem/src/raycasting.cuh:44-66): F = rn(1/A), U = rn(F u),
// V = rn(F v), t = rn(F w); hit iff 0 <= U <= 1, V >= 0, rn(U + V) <= 1,
// t > 2 eps and t < rn(len - 2 eps).
__host__ __device__ __forceinline__ bool cull_tail_exact(float A, float u, float v, float w, float len, float eps) {
    const float F = rn::rcp(A);
    const float U = rn::mul(F, u);
    if (U < 0.f || U > 1.f) return false;
    const float V = rn::mul(F, v);
    if (V < 0.f || rn::add(U, V) > 1.f) return false;
    const float t = rn::mul(F, w);
    const float two_eps = 2.f * eps;
    return (t > two_eps) && (t < rn::sub(len, two_eps));
}

// The same decisions without the reciprocal where they are certain.  For A in
// [2^-90, 2^90], F = rn(1/A) is within 2^-24 of 1/A, and each rounded product
// within 2^-24 of its exact value, so (all margins at least 2^-19 against a
// few units of 2^-24):
//   u, v >= 0 and rn(u + v) <= rn(A (1 - 2^-19))  =>  U, V in [0, 1], rn(U + V) <= 1;
//   rn(u + v) > ahi = rn(A + A 2^-19) (u, v past their guard bands)  =>  rn(U + V) > 1;
//   w <= 0  =>  t <= 0: a miss;
//   w > rn(A max(4 eps, 2^-30))  =>  t > 2 eps;
//   w < rn(rn(L (1 - 2^-18)) A)  =>  t < L,   w > rn(rn(L (1 + 2^-18)) A)  =>  t > L,
// with L = rn(len - 2 eps) in [2^-20, 2^30] (no product over- or underflows).
// Everything else (pairs within about 2^-19 of an edge of the test, or of the
// ends of the segment) takes the reference's own sequence, so the result is
// the reference's bit for bit.  ahi is the guard-band bound the caller used
// for u and v.
__host__ __device__ __forceinline__ bool cull_tail(float A, float u, float v, float w, float len, float eps,
                                                   float ahi) {
    if (A >= 0x1p-90f && A <= 0x1p90f) {
        // the usual misses first (the line meets the plane outside the triangle, or behind the origin);
        // neither claim depends on the segment's length
        const float uv = rn::add(u, v);
        if (uv > ahi || w <= 0.f) return false;
        const float L = rn::sub(len, 2.f * eps);
        if (L >= 0x1p-20f && L <= 0x1p30f) {
            if (w > rn::mul(rn::mul(L, 1.f + 0x1p-18f), A)) return false;
            const float alo = rn::mul(A, 1.f - 0x1p-19f);
            const float Llo = rn::mul(rn::mul(L, 1.f - 0x1p-18f), A);
            const float b4 = rn::mul(A, fmaxf(rn::mul(4.f, eps), 0x1p-30f));
            if (u >= 0.f && v >= 0.f && uv <= alo && w > b4 && w < Llo) return true;
        }
    }
    return cull_tail_exact(A, u, v, w, len, eps);
}

// hit() with the per-source quantities precomputed.
template <bool CULL>
__device__ __forceinline__ bool hit_pre(const Ray& r, const TriPre& p, float eps) {
    const float e1x = p.a.x, e1y = p.a.y, e1z = p.a.z;
    const float e2x = p.a.w, e2y = p.b.x, e2z = p.b.y;
    float px = __fmaf_rn(r.dy, e2z, -__fmul_rn(r.dz, e2y));
    float py = __fmaf_rn(r.dz, e2x, -__fmul_rn(r.dx, e2z));
    float pz = __fmaf_rn(r.dx, e2y, -__fmul_rn(r.dy, e2x));
    float A = __fmaf_rn(e1z, pz, __fmaf_rn(e1y, py, __fmul_rn(e1x, px)));
    if (det_rejects<CULL>(A, eps)) return false;
    if (!CULL) {
        const float u = __fmaf_rn(p.c.x, pz, __fmaf_rn(p.b.w, py, __fmul_rn(p.b.z, px)));
        if (ratio_negative(u, A) || ratio_above_one(u, A)) return false;
        const float v = __fmaf_rn(r.dz, p.c.w, __fmaf_rn(r.dy, p.c.z, __fmul_rn(r.dx, p.c.y)));
        if (ratio_negative(v, A)) return false;
        return numba_tail(A, u, v, p.d.x, r.len, eps);
    }
    // A >= eps >= 0: the guard band, then the reciprocal-free decisions
    const float aneg = __fmul_rn(A, -0x1p-20f), ahi = __fmaf_rn(A, 0x1p-19f, A);
    const float u = __fmaf_rn(p.c.x, pz, __fmaf_rn(p.b.w, py, __fmul_rn(p.b.z, px)));
    if (u < aneg || u > ahi) return false;
    const float v = __fmaf_rn(r.dz, p.c.w, __fmaf_rn(r.dy, p.c.z, __fmul_rn(r.dx, p.c.y)));
    if (v < aneg || v > ahi) return false;
    return cull_tail(A, u, v, p.d.x, r.len, eps, ahi);
}

// hit() from the packed triangle (v0, e1, e2) and the ray origin.
template <bool CULL>
__device__ __forceinline__ bool hit_full(const Ray& r, float ox, float oy, float oz, float4 v0, float4 e1,
                                         float4 e2, float eps) {
    float px = __fmaf_rn(r.dy, e2.z, -__fmul_rn(r.dz, e2.y));
    float py = __fmaf_rn(r.dz, e2.x, -__fmul_rn(r.dx, e2.z));
    float pz = __fmaf_rn(r.dx, e2.y, -__fmul_rn(r.dy, e2.x));
    float A = __fmaf_rn(e1.z, pz, __fmaf_rn(e1.y, py, __fmul_rn(e1.x, px)));
    if (det_rejects<CULL>(A, eps)) return false;
    float tx = __fsub_rn(ox, v0.x), ty = __fsub_rn(oy, v0.y), tz = __fsub_rn(oz, v0.z);
    const float u = __fmaf_rn(tz, pz, __fmaf_rn(ty, py, __fmul_rn(tx, px)));
    if (!CULL) {
        if (ratio_negative(u, A) || ratio_above_one(u, A)) return false;
        const float qx = __fmaf_rn(ty, e1.z, -__fmul_rn(tz, e1.y));
        const float qy = __fmaf_rn(tz, e1.x, -__fmul_rn(tx, e1.z));
        const float qz = __fmaf_rn(tx, e1.y, -__fmul_rn(ty, e1.x));
        const float v = __fmaf_rn(r.dz, qz, __fmaf_rn(r.dy, qy, __fmul_rn(r.dx, qx)));
        if (ratio_negative(v, A)) return false;
        return numba_tail(A, u, v, __fmaf_rn(e2.z, qz, __fmaf_rn(e2.y, qy, __fmul_rn(e2.x, qx))), r.len, eps);
    }
    // A >= eps >= 0 (the entry points reject a negative eps): the guard band
    // above (A = -0 or +0: every u other than zero is a miss there, as the
    // reference's infinite F makes it)
    const float aneg = __fmul_rn(A, -0x1p-20f), ahi = __fmaf_rn(A, 0x1p-19f, A);
    if (u < aneg || u > ahi) return false;
    float qx = __fmaf_rn(ty, e1.z, -__fmul_rn(tz, e1.y));
    float qy = __fmaf_rn(tz, e1.x, -__fmul_rn(tx, e1.z));
    float qz = __fmaf_rn(tx, e1.y, -__fmul_rn(ty, e1.x));
    const float v = __fmaf_rn(r.dz, qz, __fmaf_rn(r.dy, qy, __fmul_rn(r.dx, qx)));
    if (v < aneg || v > ahi) return false;
    const float w = __fmaf_rn(e2.z, qz, __fmaf_rn(e2.y, qy, __fmul_rn(e2.x, qx)));
    return cull_tail(A, u, v, w, r.len, eps, ahi);
}

// Path length in FP64 from the FP32 end points: the coordinate differences are
// exact in FP64, and one Newton step from the FP32 length w gives a relative
// error far below 1e-12.
__device__ __forceinline__ double path_length_fp64(float ox, float oy, float oz, float ex, float ey, float ez,
                                                   float w) {
    double dx = (double)ex - (double)ox;
    double dy = (double)ey - (double)oy;
    double dz = (double)ez - (double)oz;
    double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
    double wd = (double)w;
    double h = (double)(0.5f * __frcp_rn(w));
    return fma(fma(-wd, wd, r2), h, wd);
}

// beta * r reduced to [-pi, pi] in FP64 (Cody-Waite with a two-term 2*pi).
__device__ __forceinline__ float reduced_phase(double beta, double r) {
    const double kTwoPiHi = 6.283185307179586232;      // nearest double to 2*pi
    const double kTwoPiLo = 2.4492935982947064e-16;    // 2*pi - kTwoPiHi
    const double kInvTwoPi = 0.15915494309189534561;
    double ph = beta * r;
    double k = rint(ph * kInvTwoPi);
    double red = fma(-k, kTwoPiHi, ph);
    red = fma(-k, kTwoPiLo, red);
    return (float)red;
}

// Field of one visible pair: E_L * loss with
//   E_L  = E - (E.d) d  (= (E.u)u + (E.v)v of ray_launch, em.cuh:18-61)
//   G    = exp(-alpha r)/r * exp(-j beta r);  dG = (-alpha - 1/r - j beta) G
//   loss = -(1/(2 pi)) dG (n_sink . d)        (em.cuh:64-120)
// E and out are complex 3-vectors as 6 floats (re, im) x (x, y, z).
__device__ __forceinline__ void pair_field(const Ray& r, double rlen, const float* E, float nx, float ny, float nz,
                                           float alpha, float beta_f, double beta_d, float* out) {
    float ph = reduced_phase(beta_d, rlen);
    float s, c;
    sincosf(ph, &s, &c);
    float inv_r = 1.0f / r.len;
    float mag = expf(-alpha * r.len) * inv_r;
    float g_re = mag * c, g_im = -mag * s;
    float a_re = -alpha - inv_r, a_im = -beta_f;
    float dg_re = a_re * g_re - a_im * g_im;
    float dg_im = a_re * g_im + a_im * g_re;
    float nd = nx * r.dx + ny * r.dy + nz * r.dz;
    const float front = -0.15915494309189535f;  // -1/(2 pi)
    float l_re = front * nd * dg_re, l_im = front * nd * dg_im;
    float ed_re = E[0] * r.dx + E[2] * r.dy + E[4] * r.dz;
    float ed_im = E[1] * r.dx + E[3] * r.dy + E[5] * r.dz;
    float el_re[3] = {E[0] - ed_re * r.dx, E[2] - ed_re * r.dy, E[4] - ed_re * r.dz};
    float el_im[3] = {E[1] - ed_im * r.dx, E[3] - ed_im * r.dy, E[5] - ed_im * r.dz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        out[2 * k] = el_re[k] * l_re - el_im[k] * l_im;
        out[2 * k + 1] = el_re[k] * l_im + el_im[k] * l_re;
    }
}

// Float-float path length and phase, the FP32-pipe counterpart of
// path_length_fp64 + reduced_phase (FP64 runs at a small fraction of the FP32
// rate on this GPU), used where phases are recomputed per pair and frequency:
// the batched kernel (lyem_batch.cu) and the adjoint kernels (lyem_adjoint.cu).

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// |e - o| as rh + rl.  The coordinate differences are exact as (h, l) pairs,
// the squares exact as (p, q) pairs; the neglected l*l terms are below
// 2^-46 of r^2, and one Newton correction of the FP32 square root (whose
// residual fma(-rh, rh, s) is exact) carries the float-float precision.
__device__ __forceinline__ void ff_length(float ox, float oy, float oz, float ex, float ey, float ez, float& rh,
                                          float& rl) {
    float hx, lx, hy, ly, hz, lz;
    two_sum(ex, -ox, hx, lx);
    two_sum(ey, -oy, hy, ly);
    two_sum(ez, -oz, hz, lz);
    const float px = __fmul_rn(hx, hx), qx = __fmaf_rn(hx, hx, -px);
    const float py = __fmul_rn(hy, hy), qy = __fmaf_rn(hy, hy, -py);
    const float pz = __fmul_rn(hz, hz), qz = __fmaf_rn(hz, hz, -pz);
    float s1, e1, s2, e2;
    two_sum(px, py, s1, e1);
    two_sum(s1, pz, s2, e2);
    const float cross = __fmaf_rn(hx, lx, __fmaf_rn(hy, ly, __fmul_rn(hz, lz)));
    const float lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fadd_rn(qx, qy), __fmaf_rn(2.f, cross, qz)));
    rh = __fsqrt_rn(s2);
    rl = rh > 0.f ? __fmul_rn(__fadd_rn(__fmaf_rn(-rh, rh, s2), lo), __fmul_rn(0.5f, __frcp_rn(rh))) : 0.f;
}

// (bh + bl) * (rh + rl) reduced to about [-pi, pi].  2 pi = kC1 + kC2 + O(7e-15).
// x = p - k*kC1 is exact: |x| < 4 and both p and k*kC1 are multiples of
// 2^-22 there, so it fits 24 bits.  The error is a few 1e-7 rad for any k
// that the FP32 product admits.
__device__ __forceinline__ float ff_phase(float bh, float bl, float rh, float rl) {
    const float kC1 = 6.28318548202514648f;
    const float kC2 = -1.74845553146951715e-7f;
    const float kInv = 0.159154936671257019f;
    const float p = __fmul_rn(bh, rh);
    const float pe = __fmaf_rn(bh, rh, -p);
    const float lo = __fadd_rn(pe, __fmaf_rn(bh, rl, __fmul_rn(bl, rh)));
    const float k = rintf(__fmul_rn(p, kInv));
    float x = __fmaf_rn(-k, kC1, p);
    x = __fmaf_rn(-k, kC2, x);
    return __fadd_rn(x, lo);
}

// Bounded wait on an mbarrier phase.  Returns false if the deadline (in SM
// clock cycles) passes first; the caller then reports LYEM_ERR_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar_addr, uint32_t parity, long long max_cycles) {
    long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar_addr), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > max_cycles) return false;
    }
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t mbar_addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar_addr), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One-dimensional TMA bulk copy global -> shared, completing on an mbarrier.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void tma_load_1d(uint32_t dst_smem, const void* src_gmem, uint32_t bytes,
                                            uint32_t mbar_addr) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar_addr), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst_smem),
        "l"(src_gmem), "r"(bytes), "r"(mbar_addr)
        : "memory");
}

}  // namespace lyem
