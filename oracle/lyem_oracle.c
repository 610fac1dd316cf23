/*
 * lyem_oracle.c -- CPU restatement of LyceanEM's raycasting + frequency-domain
 * propagation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library in
 * lyceanem-python_gb300/csrc is compared with: the parity tests, the smoke
 * check and the CPU baseline leg of bench.py call it.  Nothing in the product path links, loads
 * or calls it.
 *
 * Two arithmetic modes:
 *   - visibility is FP32 and bit-faithful: every operation below is one IEEE
 *     binary32 operation with round-to-nearest, fused multiply-adds are
 *     explicit fmaf() calls, and the file must be compiled with
 *     -ffp-contract=off so that no other contraction happens.  The CUDA
 *     kernels perform exactly the same operations with __fmaf_rn/__fmul_rn/...
 *     so masks must agree bit for bit.
 *   - fields are FP64 restatements of the reference formulas, computed from
 *     the same FP32 inputs.
 *
 * Pinned against the reference itself: tests/test_reference_golden.py
 * compares this file's masks and fields with outputs of the reference's own
 * points_to_rays / hit / em_wave run on a GPU (oracle/ref_harness): masks
 * identical on every pair, fields within the reference's FP32 phase error.
 *
 * Reference formulas followed (paths within LyceanEM-Python):
 *   ray set-up            lyceanem/src/raycasting.cuh:80-95   (points_to_rays)
 *   ray/triangle test     lyceanem/src/raycasting.cuh:19-68   (hit, back-face cull)
 *                         lyceanem/raycasting/rayfunctions.py:37-104 (numba hit, no cull)
 *   EPSILON               lyceanem/src/math_utility.cuh:9
 *   pair skip rule        lyceanem/src/raycasting_brute_force.cuh:24-33
 *   polarisation launch   lyceanem/src/em.cuh:18-61            (ray_launch)
 *   propagation kernel    lyceanem/src/em.cuh:64-120           (em_wave)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { float x, y, z; } f3;

static inline f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }

/* cross(a, b) with each component a*b - c*d evaluated as fma(a, b, -(c*d)). */
static inline f3 cross3(f3 a, f3 b) {
    f3 r;
    r.x = fmaf(a.y, b.z, -(a.z * b.y));
    r.y = fmaf(a.z, b.x, -(a.x * b.z));
    r.z = fmaf(a.x, b.y, -(a.y * b.x));
    return r;
}

/* dot(a, b) evaluated left to right as fma(a.z, b.z, fma(a.y, b.y, a.x*b.x)). */
static inline float dot3(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }

/* ---------------------------------------------------------------------------
 * Triangle packing: 12 floats per triangle (v0, 0, e1, 0, e2, 0) with
 * e1 = v1 - v0 and e2 = v2 - v0 in FP32, the same subtraction the reference
 * performs per test (raycasting_brute_force.cuh:40-42).
 * ------------------------------------------------------------------------- */
void orc_pack_triangles(const float *verts, int64_t n_verts, const int32_t *idx, int64_t n_tris,
                        float *out) {
    (void)n_verts;
    for (int64_t t = 0; t < n_tris; ++t) {
        const float *a = verts + 3 * (int64_t)idx[3 * t + 0];
        const float *b = verts + 3 * (int64_t)idx[3 * t + 1];
        const float *c = verts + 3 * (int64_t)idx[3 * t + 2];
        float *o = out + 12 * t;
        o[0] = a[0]; o[1] = a[1]; o[2] = a[2]; o[3] = 0.0f;
        o[4] = b[0] - a[0]; o[5] = b[1] - a[1]; o[6] = b[2] - a[2]; o[7] = 0.0f;
        o[8] = c[0] - a[0]; o[9] = c[1] - a[1]; o[10] = c[2] - a[2]; o[11] = 0.0f;
    }
}

/* points_to_rays (raycasting.cuh:80-95): r = end - source, w = |r|, dir = r / w. */
static inline void orc_ray(const float *o, const float *e, f3 *d, float *len) {
    float rx = e[0] - o[0], ry = e[1] - o[1], rz = e[2] - o[2];
    float w2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
    float w = sqrtf(w2);
    d->x = rx / w;
    d->y = ry / w;
    d->z = rz / w;
    *len = w;
}

/* The numba engine's ray set-up: numpy float32 on the host with nothing fused
 * (calc_dv_norm, lyceanem/utility/math_functions.py:149-156, called by
 * charge_rays_environment1Dv2, lyceanem/raycasting/rayfunctions.py:1790-1842):
 * ((rx*rx + ry*ry) + rz*rz), sqrt, one division per component. */
static inline void orc_ray_numba(const float *o, const float *e, f3 *d, float *len) {
    float rx = e[0] - o[0], ry = e[1] - o[1], rz = e[2] - o[2];
    float w2 = (rx * rx + ry * ry) + rz * rz;
    float w = sqrtf(w2);
    d->x = rx / w;
    d->y = ry / w;
    d->z = rz / w;
    *len = w;
}

/* Visibility ray of a mode: the CUDA engine's with culling, the numba engine's without. */
static inline void orc_vis_ray(const float *o, const float *e, int cull, f3 *d, float *len) {
    if (cull)
        orc_ray(o, e, d, len);
    else
        orc_ray_numba(o, e, d, len);
}

/* Moller-Trumbore test (raycasting.cuh:19-68).  cull != 0 is the CUDA engine
 * (|A| < eps or A < 0 is a miss; F = 1/A is the correctly rounded FP32
 * reciprocal, which equals the reference's (float)(1.0/(double)A)).  cull == 0
 * is the numba engine (rayfunctions.py:37-104): only |A| < eps is a miss, and
 * F = 1.0 / A, U, V and t are FP64 there (the float64 literal promotes the
 * float32 determinant) and compared in FP64; the numerators stay FP32. */
int orc_hit(f3 d, float len, f3 o, f3 e1, f3 e2, f3 v0, int cull, float eps) {
    f3 p = cross3(d, e2);
    float A = dot3(e1, p);
    if (cull) {
        if (!(A >= eps)) return 0;
    } else {
        if (fabsf(A) < eps) return 0;
        f3 t = sub3(o, v0);
        double F = 1.0 / (double)A;
        double U = F * (double)dot3(t, p);
        if (U < 0.0 || U > 1.0) return 0;
        f3 q = cross3(t, e1);
        double V = F * (double)dot3(d, q);
        if (V < 0.0 || (U + V) > 1.0) return 0;
        double tt = F * (double)dot3(e2, q);
        double two_eps = 2.0 * (double)eps;
        return (tt > two_eps) && (tt < ((double)len - two_eps));
    }
    f3 t = sub3(o, v0);
    float F = 1.0f / A;
    float U = F * dot3(t, p);
    if (U < 0.0f || U > 1.0f) return 0;
    f3 q = cross3(t, e1);
    float V = F * dot3(d, q);
    if (V < 0.0f || (U + V) > 1.0f) return 0;
    float tt = F * dot3(e2, q);
    float two_eps = 2.0f * eps;
    return (tt > two_eps) && (tt < (len - two_eps));
}

static inline int orc_hit_packed(f3 d, float len, f3 o, const float *tri, int cull, float eps) {
    return orc_hit(d, len, o, mk3(tri[4], tri[5], tri[6]), mk3(tri[8], tri[9], tri[10]),
                   mk3(tri[0], tri[1], tri[2]), cull, eps);
}

static int orc_threads(int nthreads) {
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* Brute-force visibility over all triangles (raycasting_brute_force.cuh:19-67).
 * mask[n*M+m] = 1 when the segment source n -> sink m is unobstructed.  With
 * skip_diag != 0 the pair n == m is not tested (treated as visible), which is
 * the reference's behaviour when self_to_self is False. */
void orc_mask_brute(const float *src, int64_t N, const float *snk, int64_t M, const float *tris,
                    int64_t T, int skip_diag, int cull, float eps, uint8_t *mask, int nthreads) {
    int nt = orc_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int64_t i = 0; i < N * M; ++i) {
        int64_t n = i / M, m = i % M;
        uint8_t vis = 1;
        if (!(skip_diag && n == m)) {
            f3 d;
            float len;
            orc_vis_ray(src + 3 * n, snk + 3 * m, cull, &d, &len);
            f3 o = mk3(src[3 * n], src[3 * n + 1], src[3 * n + 2]);
            for (int64_t t = 0; t < T; ++t) {
                if (orc_hit_packed(d, len, o, tris + 12 * t, cull, eps)) { vis = 0; break; }
            }
        }
        mask[i] = vis;
    }
}

/* ---------------------------------------------------------------------------
 * Uniform-grid acceleration (CPU).  Any-hit visibility is an OR over the
 * triangles, so a traversal that visits every cell a segment passes through
 * returns exactly the brute-force mask.  Triangle boxes are padded by `pad`
 * and the walk is done in FP64, so the set of visited cells is a superset of
 * the cells containing any hit point found by the FP32 test.
 * ------------------------------------------------------------------------- */
typedef struct {
    double org[3];
    double cell;
    int dims[3];
    int64_t *start; /* ncells + 1 */
    int32_t *tri;   /* refs */
    const float *tris;
    int64_t T;
} orc_grid;

static void tri_box(const float *tri, double lo[3], double hi[3]) {
    for (int k = 0; k < 3; ++k) {
        double a = tri[k], b = (double)tri[k] + (double)tri[4 + k], c = (double)tri[k] + (double)tri[8 + k];
        lo[k] = fmin(a, fmin(b, c));
        hi[k] = fmax(a, fmax(b, c));
    }
}

void *orc_grid_build(const float *tris, int64_t T, double cell, double pad) {
    orc_grid *g = (orc_grid *)calloc(1, sizeof(orc_grid));
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t t = 0; t < T; ++t) {
        double a[3], b[3];
        tri_box(tris + 12 * t, a, b);
        for (int k = 0; k < 3; ++k) { lo[k] = fmin(lo[k], a[k]); hi[k] = fmax(hi[k], b[k]); }
    }
    if (T == 0) { for (int k = 0; k < 3; ++k) { lo[k] = 0; hi[k] = 1; } }
    g->cell = cell;
    for (int k = 0; k < 3; ++k) {
        g->org[k] = lo[k] - 2 * pad;
        int d = (int)ceil((hi[k] + 2 * pad - g->org[k]) / cell);
        g->dims[k] = d < 1 ? 1 : d;
    }
    int64_t nc = (int64_t)g->dims[0] * g->dims[1] * g->dims[2];
    g->start = (int64_t *)calloc((size_t)nc + 1, sizeof(int64_t));
    int pass;
    int64_t *cursor = NULL;
    for (pass = 0; pass < 2; ++pass) {
        for (int64_t t = 0; t < T; ++t) {
            double a[3], b[3];
            int i0[3], i1[3];
            tri_box(tris + 12 * t, a, b);
            for (int k = 0; k < 3; ++k) {
                i0[k] = (int)floor((a[k] - pad - g->org[k]) / cell);
                i1[k] = (int)floor((b[k] + pad - g->org[k]) / cell);
                if (i0[k] < 0) i0[k] = 0;
                if (i1[k] > g->dims[k] - 1) i1[k] = g->dims[k] - 1;
            }
            for (int z = i0[2]; z <= i1[2]; ++z)
                for (int y = i0[1]; y <= i1[1]; ++y)
                    for (int x = i0[0]; x <= i1[0]; ++x) {
                        int64_t c = ((int64_t)z * g->dims[1] + y) * g->dims[0] + x;
                        if (pass == 0) g->start[c + 1]++;
                        else g->tri[cursor[c]++] = (int32_t)t;
                    }
        }
        if (pass == 0) {
            for (int64_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
            g->tri = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->start[nc] + 1));
            cursor = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
            memcpy(cursor, g->start, sizeof(int64_t) * (size_t)nc);
        }
    }
    free(cursor);
    g->tris = tris;
    g->T = T;
    return g;
}

void orc_grid_free(void *h) {
    orc_grid *g = (orc_grid *)h;
    if (!g) return;
    free(g->start);
    free(g->tri);
    free(g);
}

void orc_grid_info(void *h, double *org_cell, int32_t *dims, int64_t *n_refs) {
    orc_grid *g = (orc_grid *)h;
    for (int k = 0; k < 3; ++k) { org_cell[k] = g->org[k]; dims[k] = g->dims[k]; }
    org_cell[3] = g->cell;
    *n_refs = g->start[(int64_t)g->dims[0] * g->dims[1] * g->dims[2]];
}

/* Any-hit walk of the segment o -> o + len*d through the grid (Amanatides-Woo
 * in FP64, on the FP64 difference of the end points).  Returns 1 if blocked. */
static int orc_grid_blocked(const orc_grid *g, const float *po, const float *pe, f3 d, float len,
                            int cull, float eps, int64_t *tests) {
    f3 o = mk3(po[0], po[1], po[2]);
    double O[3] = {po[0], po[1], po[2]};
    double D[3] = {(double)pe[0] - po[0], (double)pe[1] - po[1], (double)pe[2] - po[2]};
    double t0 = 0.0, t1 = 1.0;
    double gmax[3];
    for (int k = 0; k < 3; ++k) {
        gmax[k] = g->org[k] + g->dims[k] * g->cell;
        if (D[k] == 0.0) {
            if (O[k] < g->org[k] || O[k] > gmax[k]) return 0;
        } else {
            double ta = (g->org[k] - O[k]) / D[k], tb = (gmax[k] - O[k]) / D[k];
            if (ta > tb) { double s = ta; ta = tb; tb = s; }
            if (ta > t0) t0 = ta;
            if (tb < t1) t1 = tb;
        }
    }
    if (t0 > t1) return 0;
    int idx[3], step[3];
    double tmax[3], tdel[3];
    for (int k = 0; k < 3; ++k) {
        double p = O[k] + t0 * D[k];
        int i = (int)floor((p - g->org[k]) / g->cell);
        if (i < 0) i = 0;
        if (i > g->dims[k] - 1) i = g->dims[k] - 1;
        idx[k] = i;
        if (D[k] > 0) {
            step[k] = 1;
            tmax[k] = (g->org[k] + (i + 1) * g->cell - O[k]) / D[k];
            tdel[k] = g->cell / D[k];
        } else if (D[k] < 0) {
            step[k] = -1;
            tmax[k] = (g->org[k] + i * g->cell - O[k]) / D[k];
            tdel[k] = -g->cell / D[k];
        } else {
            step[k] = 0;
            tmax[k] = INFINITY;
            tdel[k] = INFINITY;
        }
    }
    for (;;) {
        int64_t c = ((int64_t)idx[2] * g->dims[1] + idx[1]) * g->dims[0] + idx[0];
        for (int64_t r = g->start[c]; r < g->start[c + 1]; ++r) {
            if (tests) ++*tests;
            if (orc_hit_packed(d, len, o, g->tris + 12 * (int64_t)g->tri[r], cull, eps)) return 1;
        }
        int k = (tmax[0] < tmax[1]) ? (tmax[0] < tmax[2] ? 0 : 2) : (tmax[1] < tmax[2] ? 1 : 2);
        if (tmax[k] > t1) return 0;
        idx[k] += step[k];
        if (idx[k] < 0 || idx[k] >= g->dims[k]) return 0;
        tmax[k] += tdel[k];
    }
}

void orc_mask_grid(void *h, const float *src, int64_t N, const float *snk, int64_t M, int skip_diag,
                   int cull, float eps, uint8_t *mask, int nthreads) {
    const orc_grid *g = (const orc_grid *)h;
    int nt = orc_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int64_t i = 0; i < N * M; ++i) {
        int64_t n = i / M, m = i % M;
        uint8_t vis = 1;
        if (!(skip_diag && n == m)) {
            f3 d;
            float len;
            orc_vis_ray(src + 3 * n, snk + 3 * m, cull, &d, &len);
            vis = !orc_grid_blocked(g, src + 3 * n, snk + 3 * m, d, len, cull, eps, NULL);
        }
        mask[i] = vis;
    }
}

/* ---------------------------------------------------------------------------
 * FP64 field of one pair: em_wave(ray_launch(E, d), ...) from em.cuh:18-120.
 *   d = (end - src)/r; u = normalize(a x d) with a the cartesian axis that
 *   maximises |a x d| (ties as em.cuh:30-38); v = normalize(d x u);
 *   E_L = (E.u)u + (E.v)v;
 *   G = exp(-alpha r)/r * (cos(beta r) - j sin(beta r));
 *   dG = (-alpha - 1/r - j beta) G;   loss = -(1/2pi) dG (n_sink . d);
 *   out = E_L * loss.
 * E and out are complex 3-vectors as 6 doubles (re, im) x (x, y, z).
 * ------------------------------------------------------------------------- */
static void orc_pair_field_one(const float *ps, const float *pe, const double *E, const float *nrm,
                               double alpha, double beta, double *out) {
    double rv[3] = {(double)pe[0] - ps[0], (double)pe[1] - ps[1], (double)pe[2] - ps[2]};
    double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d[3] = {rv[0] / r, rv[1] / r, rv[2] / r};
    /* |x_axis x d| = sqrt(dy^2+dz^2), |y_axis x d| = sqrt(dx^2+dz^2), |z_axis x d| = sqrt(dx^2+dy^2) */
    double xn = sqrt(d[1] * d[1] + d[2] * d[2]);
    double yn = sqrt(d[0] * d[0] + d[2] * d[2]);
    double zn = sqrt(d[0] * d[0] + d[1] * d[1]);
    double u[3] = {0, 0, 0};
    if (xn > yn && xn > zn) {
        u[0] = 0; u[1] = -d[2]; u[2] = d[1];
    } else if (yn >= xn && yn > zn) {
        u[0] = d[2]; u[1] = 0; u[2] = -d[0];
    } else {
        u[0] = -d[1]; u[1] = d[0]; u[2] = 0;
    }
    double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int k = 0; k < 3; ++k) u[k] /= un;
    double v[3] = {d[1] * u[2] - d[2] * u[1], d[2] * u[0] - d[0] * u[2], d[0] * u[1] - d[1] * u[0]};
    double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) v[k] /= vn;
    double eu_re = E[0] * u[0] + E[2] * u[1] + E[4] * u[2];
    double eu_im = E[1] * u[0] + E[3] * u[1] + E[5] * u[2];
    double ev_re = E[0] * v[0] + E[2] * v[1] + E[4] * v[2];
    double ev_im = E[1] * v[0] + E[3] * v[1] + E[5] * v[2];
    double mag = exp(-alpha * r) / r;
    double g_re = mag * cos(beta * r), g_im = -mag * sin(beta * r);
    double a_re = -alpha - 1.0 / r, a_im = -beta;
    double dg_re = a_re * g_re - a_im * g_im, dg_im = a_re * g_im + a_im * g_re;
    double nd = (double)nrm[0] * d[0] + (double)nrm[1] * d[1] + (double)nrm[2] * d[2];
    double front = -1.0 / (2.0 * 3.14159265358979323846);
    double l_re = front * dg_re * nd, l_im = front * dg_im * nd;
    for (int k = 0; k < 3; ++k) {
        double el_re = eu_re * u[k] + ev_re * v[k];
        double el_im = eu_im * u[k] + ev_im * v[k];
        out[2 * k] = el_re * l_re - el_im * l_im;
        out[2 * k + 1] = el_re * l_im + el_im * l_re;
    }
}

/* Per-pair field matrix S[n, m, :] (the reference's scattering network,
 * frequency_domain_models.cu:166-178 layout), zero where mask == 0. */
void orc_pair_field(const float *src, const double *srcE, int64_t N, const float *snk,
                    const float *snk_nrm, int64_t M, const uint8_t *mask, double alpha, double beta,
                    double *out, int nthreads) {
    int nt = orc_threads(nthreads);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < N * M; ++i) {
        int64_t n = i / M, m = i % M;
        double *o = out + 6 * i;
        if (mask && !mask[i]) {
            for (int k = 0; k < 6; ++k) o[k] = 0.0;
            continue;
        }
        orc_pair_field_one(src + 3 * n, snk + 3 * m, srcE + 6 * n, snk_nrm + 3 * m, alpha, beta, o);
    }
}

/* Sink field: out[m, c] = sum_n w[n, c] * S[n, m, c] (w == NULL means 1), the
 * source sum of frequency_domain.py:847-849, and with w the per-component
 * weighting of the one-bounce composition frequency_domain.py:258-260.
 * Visibility is taken from `mask` if given, else traced here (grid handle g or
 * brute force over tris).  counters (optional): [0] visible pairs, [1] tests. */
void orc_sink_field(const float *src, const double *srcE, const double *srcW, int64_t N,
                    const float *snk, const float *snk_nrm, int64_t M, const uint8_t *mask,
                    void *grid, const float *tris, int64_t T, int skip_diag, int cull, float eps,
                    double alpha, double beta, double *out, int64_t *counters, int nthreads) {
    int nt = orc_threads(nthreads);
    int64_t vis_total = 0, tests_total = 0;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt) reduction(+ : vis_total, tests_total)
    for (int64_t m = 0; m < M; ++m) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int64_t n = 0; n < N; ++n) {
            int vis = 1;
            if (mask) {
                vis = mask[n * M + m];
            } else if (!(skip_diag && n == m)) {
                f3 d;
                float len;
                orc_vis_ray(src + 3 * n, snk + 3 * m, cull, &d, &len);
                if (grid) {
                    vis = !orc_grid_blocked((const orc_grid *)grid, src + 3 * n, snk + 3 * m, d, len,
                                            cull, eps, &tests_total);
                } else {
                    f3 o = mk3(src[3 * n], src[3 * n + 1], src[3 * n + 2]);
                    for (int64_t t = 0; t < T; ++t) {
                        ++tests_total;
                        if (orc_hit_packed(d, len, o, tris + 12 * t, cull, eps)) { vis = 0; break; }
                    }
                }
            }
            if (!vis) continue;
            ++vis_total;
            double s[6];
            orc_pair_field_one(src + 3 * n, snk + 3 * m, srcE + 6 * n, snk_nrm + 3 * m, alpha, beta, s);
            if (srcW) {
                const double *w = srcW + 6 * n;
                for (int k = 0; k < 3; ++k) {
                    acc[2 * k] += w[2 * k] * s[2 * k] - w[2 * k + 1] * s[2 * k + 1];
                    acc[2 * k + 1] += w[2 * k] * s[2 * k + 1] + w[2 * k + 1] * s[2 * k];
                }
            } else {
                for (int k = 0; k < 6; ++k) acc[k] += s[k];
            }
        }
        for (int k = 0; k < 6; ++k) out[6 * m + k] = acc[k];
    }
    if (counters) {
        counters[0] = vis_total;
        counters[1] = tests_total;
    }
}

/* FP32 ray set-up exported for tests (direction and length of each pair). */
void orc_rays(const float *src, int64_t N, const float *snk, int64_t M, float *out4) {
    for (int64_t i = 0; i < N * M; ++i) {
        f3 d;
        float len;
        orc_ray(src + 3 * (i / M), snk + 3 * (i % M), &d, &len);
        out4[4 * i] = d.x; out4[4 * i + 1] = d.y; out4[4 * i + 2] = d.z; out4[4 * i + 3] = len;
    }
}

/* Single ray/triangle test exported for known-answer tests. */
int orc_hit_one(const float *d, float len, const float *o, const float *tri12, int cull, float eps) {
    return orc_hit_packed(mk3(d[0], d[1], d[2]), len, mk3(o[0], o[1], o[2]), tri12, cull, eps);
}

int orc_max_threads(void) { return orc_threads(0); }
