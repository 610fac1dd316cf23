// lyem_paths.cu -- the numba engine's field products.
//
// The numba engine of LyceanEM-Python lists every unblocked path as a row of
// 1-based indices into one point array (sources 1..N, sinks N+1..N+M,
// scatter points after them; 0 = no point): [n, m] or [n, m, 0] for a direct
// path, [n, p, m] for one bounce, [n, p, q, m] for two
// (lyceanem/raycasting/rayfunctions.py:2681-2955).  freqdomainkernal
// (lyceanem/electromagnetics/empropagation.py:1083-1265) evaluates a row as
//   ray = w_a0 (an electric source) or (w_a0 x d_01) / eta_a0 (a magnetic one)
//   for i = 0 .. cols-2:
//     if i > 0:            ray = P(n_{a_i}) ray      (tangential projection)
//     if a_{i+1} != 0:     ray = w_{a_{i+1}} (.) P(d_{a_i a_{i+1}}) ray
//   ray *= L(a0 -> a1) * prod_{i >= 1, a_{i+1} != 0} L(a_i -> a_{i+1})
// with P(x) f = f - (f.x^) x^ (sourcelaunchtransformGPU, :179-258), the
// segment loss L of lossy_propagation (:769-801), the same as em_wave's
// (lyceanem/src/em.cuh:64-120), and adds it to network[source, sink] where
// the sink is the row's last non-zero index (targettingindex, :3395-3430).
// Two details of the reference are kept: a zero index read as a point takes
// the LAST point of the array (Python's index -1), which happens for the
// projection step of rows shorter than the index width; and the projection
// at a_i runs for every i >= 1, so with scattering enabled (3 columns) a
// direct path is also projected onto the plane normal to the sink's normal.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyem.h"
#include "lyem_device.cuh"
#include "lyem_internal.cuh"

namespace lyem {
namespace {

struct C3 {
    float re[3], im[3];
};

// f - (f . x^) x^ for a unit or non-unit x (zero x leaves f unchanged)
__device__ __forceinline__ void project(C3& f, float x, float y, float z) {
    const float n2 = x * x + y * y + z * z;
    if (!(n2 > 0.f)) return;
    const float inv = 1.0f / sqrtf(n2);
    const float u[3] = {x * inv, y * inv, z * inv};
    const float dre = f.re[0] * u[0] + f.re[1] * u[1] + f.re[2] * u[2];
    const float dim = f.im[0] * u[0] + f.im[1] * u[1] + f.im[2] * u[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f.re[k] -= dre * u[k];
        f.im[k] -= dim * u[k];
    }
}

// segment loss -(1/2pi) (n_b . d) (-alpha - 1/r - j beta) exp(-(alpha + j beta) r) / r, phase in FP64
__device__ __forceinline__ void seg_loss(const float* a, const float* b, const float* nb, float alpha, float beta_f,
                                         double beta_d, float& lre, float& lim) {
    const Ray r = make_ray(a[0], a[1], a[2], b[0], b[1], b[2]);
    const double rl = path_length_fp64(a[0], a[1], a[2], b[0], b[1], b[2], r.len);
    float s, c;
    sincosf(reduced_phase(beta_d, rl), &s, &c);
    const float inv_r = 1.0f / r.len;
    const float mag = expf(-alpha * r.len) * inv_r;
    const float g_re = mag * c, g_im = -mag * s;
    const float a_re = -alpha - inv_r, a_im = -beta_f;
    const float nd = nb[0] * r.dx + nb[1] * r.dy + nb[2] * r.dz;
    const float front = -0.15915494309189535f * nd;
    lre = front * (a_re * g_re - a_im * g_im);
    lim = front * (a_re * g_im + a_im * g_re);
}

__global__ void tangential_project_kernel(float* __restrict__ v, const float* __restrict__ nrm, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        C3 f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            f.re[k] = v[6 * i + 2 * k];
            f.im[k] = v[6 * i + 2 * k + 1];
        }
        project(f, nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            v[6 * i + 2 * k] = f.re[k];
            v[6 * i + 2 * k + 1] = f.im[k];
        }
    }
}

struct PathParams {
    const int32_t* paths;
    long long n_paths;
    int cols;
    const float* pos;
    const float* nrm;
    const float* w;           // [n_pts, 6]
    const uint8_t* magnetic;  // [n_pts] or nullptr
    const float* impedance;   // [n_pts] or nullptr
    long long n_pts, n_src, n_snk;
    float alpha, beta_f;
    double beta_d;
    double* out;  // [n_src, n_snk, 3, 2]
    unsigned int* err;
};

__global__ void path_field_kernel(const PathParams p) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < p.n_paths;
         r += (long long)gridDim.x * blockDim.x) {
        const int32_t* row = p.paths + r * p.cols;
        // checks: indices within 0..n_pts, a source first, a sink last
        bool bad = false;
        int last = 0;
        for (int i = 0; i < p.cols; ++i) {
            const int v = row[i];
            if (v < 0 || v > p.n_pts) bad = true;
            if (v != 0) last = v;
        }
        const long long src = (long long)row[0] - 1;
        const long long snk = (long long)last - p.n_src - 1;
        if (bad || src < 0 || src >= p.n_src || row[1] == 0 || snk < 0 || snk >= p.n_snk) {
            atomicOr(p.err, 2u);
            continue;
        }
        auto pt = [&](int v) -> long long {  // 1-based index to row, 0 -> last point (Python's -1)
            return v > 0 ? (long long)v - 1 : p.n_pts - 1;
        };
        const long long a0 = pt(row[0]), a1 = pt(row[1]);
        C3 f;
        const float* wa = p.w + 6 * a0;
        if (p.magnetic && p.magnetic[a0]) {
            const Ray d = make_ray(p.pos[3 * a0], p.pos[3 * a0 + 1], p.pos[3 * a0 + 2], p.pos[3 * a1],
                                   p.pos[3 * a1 + 1], p.pos[3 * a1 + 2]);
            const float dd[3] = {d.dx, d.dy, d.dz};
            const float inv_eta = p.impedance ? 1.0f / p.impedance[a0] : 1.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
                f.re[k] = (wa[2 * k1] * dd[k2] - wa[2 * k2] * dd[k1]) * inv_eta;
                f.im[k] = (wa[2 * k1 + 1] * dd[k2] - wa[2 * k2 + 1] * dd[k1]) * inv_eta;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                f.re[k] = wa[2 * k];
                f.im[k] = wa[2 * k + 1];
            }
        }
        float lre = 1.f, lim = 0.f;
        for (int i = 0; i + 1 < p.cols; ++i) {
            const long long ai = pt(row[i]);
            if (i > 0) project(f, p.nrm[3 * ai], p.nrm[3 * ai + 1], p.nrm[3 * ai + 2]);
            if (row[i + 1] != 0) {
                const long long b = pt(row[i + 1]);
                const float* pa = p.pos + 3 * ai;
                const float* pb = p.pos + 3 * b;
                const Ray d = make_ray(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2]);
                project(f, d.dx, d.dy, d.dz);
                const float* wb = p.w + 6 * b;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float xr = f.re[k] * wb[2 * k] - f.im[k] * wb[2 * k + 1];
                    const float xi = f.re[k] * wb[2 * k + 1] + f.im[k] * wb[2 * k];
                    f.re[k] = xr;
                    f.im[k] = xi;
                }
                float sr, si;
                seg_loss(pa, pb, p.nrm + 3 * b, p.alpha, p.beta_f, p.beta_d, sr, si);
                const float nr = lre * sr - lim * si;
                lim = lre * si + lim * sr;
                lre = nr;
            }
        }
        double* o = p.out + (src * p.n_snk + snk) * 6;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicAdd(o + 2 * k, (double)(f.re[k] * lre - f.im[k] * lim));
            atomicAdd(o + 2 * k + 1, (double)(f.re[k] * lim + f.im[k] * lre));
        }
    }
}

// Time-domain form of the same row walk (timedomainkernal,
// lyceanem/electromagnetics/empropagation.py:1346-1560): real magnitudes
// (the real parts of the weights, the same projections), |loss| of the
// segments, and the arrival time = path length / c + the imaginary parts of
// the x weights of the source and of every later point ("time delays").  The
// path length adds, for i >= 1, the distance from a_i to the point of index
// a_{i+1} even when that index is 0 (then the last point), as the reference does.
__global__ void path_time_kernel(const PathParams p, double* amp, double* arrival, int32_t* pair) {
    const double kC = 299792458.0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < p.n_paths;
         r += (long long)gridDim.x * blockDim.x) {
        const int32_t* row = p.paths + r * p.cols;
        bool bad = false;
        int last = 0;
        for (int i = 0; i < p.cols; ++i) {
            const int v = row[i];
            if (v < 0 || v > p.n_pts) bad = true;
            if (v != 0) last = v;
        }
        const long long src = (long long)row[0] - 1;
        const long long snk = (long long)last - p.n_src - 1;
        if (bad || src < 0 || src >= p.n_src || row[1] == 0 || snk < 0 || snk >= p.n_snk) {
            atomicOr(p.err, 2u);
            pair[2 * r] = -1;
            pair[2 * r + 1] = -1;
            continue;
        }
        auto pt = [&](int v) -> long long { return v > 0 ? (long long)v - 1 : p.n_pts - 1; };
        const long long a0 = pt(row[0]), a1 = pt(row[1]);
        float f[3];
        const float* wa = p.w + 6 * a0;
        double delay = (double)wa[1];
        if (p.magnetic && p.magnetic[a0]) {
            const Ray d = make_ray(p.pos[3 * a0], p.pos[3 * a0 + 1], p.pos[3 * a0 + 2], p.pos[3 * a1],
                                   p.pos[3 * a1 + 1], p.pos[3 * a1 + 2]);
            const float dd[3] = {d.dx, d.dy, d.dz};
            const float inv_eta = p.impedance ? 1.0f / p.impedance[a0] : 1.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
                f[k] = (wa[2 * k1] * dd[k2] - wa[2 * k2] * dd[k1]) * inv_eta;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) f[k] = wa[2 * k];
        }
        float mag = 1.f;
        double length = 0.0;
        for (int i = 0; i + 1 < p.cols; ++i) {
            const long long ai = pt(row[i]);
            const long long bi = pt(row[i + 1]);
            const float* pa = p.pos + 3 * ai;
            const float* pb = p.pos + 3 * bi;
            if (i > 0) {
                C3 g;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    g.re[k] = f[k];
                    g.im[k] = 0.f;
                }
                project(g, p.nrm[3 * ai], p.nrm[3 * ai + 1], p.nrm[3 * ai + 2]);
#pragma unroll
                for (int k = 0; k < 3; ++k) f[k] = g.re[k];
            }
            if (ai != bi) {  // the same point twice (two 0 indices read as the last point) adds nothing
                const Ray d = make_ray(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2]);
                if (d.len > 0.f) length += path_length_fp64(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], d.len);
            }
            if (row[i + 1] != 0) {
                const Ray d = make_ray(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2]);
                C3 g;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    g.re[k] = f[k];
                    g.im[k] = 0.f;
                }
                project(g, d.dx, d.dy, d.dz);
                const float* wb = p.w + 6 * bi;
#pragma unroll
                for (int k = 0; k < 3; ++k) f[k] = g.re[k] * wb[2 * k];
                delay += (double)wb[1];
                float sr, si;
                seg_loss(pa, pb, p.nrm + 3 * bi, p.alpha, p.beta_f, p.beta_d, sr, si);
                mag *= sqrtf(sr * sr + si * si);
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) amp[3 * r + k] = (double)(f[k] * mag);
        arrival[r] = length / kC + delay;
        pair[2 * r] = (int32_t)src;
        pair[2 * r + 1] = (int32_t)snk;
    }
}

unsigned grid_for(long long n) { return capped_blocks(n, 256, 16); }

}  // namespace
}  // namespace lyem

using namespace lyem;

extern "C" {

LYEM_API int lyem_tangential_project(float* d_vec, const float* d_normals, int64_t n, void* stream) {
    if (n < 0) return LYEM_ERR_INVALID;
    if (n == 0) return LYEM_OK;
    if (!d_vec || !d_normals) return LYEM_ERR_INVALID;
    tangential_project_kernel<<<grid_for(n), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(d_vec, d_normals, n);
    note_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        record_cuda_error(e);
        return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

LYEM_API int lyem_path_field(const int32_t* d_paths, int64_t n_paths, int32_t n_cols, const float* d_pos,
                             const float* d_nrm, const float* d_w, const uint8_t* d_magnetic, const float* d_impedance,
                             int64_t n_pts, int64_t n_src, int64_t n_snk, double alpha, double beta, double* d_out,
                             void* stream) {
    if (n_paths < 0 || n_cols < 2 || n_cols > 16 || n_pts < 0 || n_src < 0 || n_snk < 0) return LYEM_ERR_INVALID;
    if (n_paths == 0) return LYEM_OK;
    if (!d_paths || !d_pos || !d_nrm || !d_w || !d_out || n_pts == 0) return LYEM_ERR_INVALID;
    if (n_pts >= (1LL << 31) || n_src + n_snk > n_pts) return LYEM_ERR_INVALID;
    if (((uintptr_t)d_out & 7u) || ((uintptr_t)d_w & 7u)) return LYEM_ERR_INVALID;
    PathParams p;
    p.paths = d_paths;
    p.n_paths = n_paths;
    p.cols = n_cols;
    p.pos = d_pos;
    p.nrm = d_nrm;
    p.w = d_w;
    p.magnetic = d_magnetic;
    p.impedance = d_impedance;
    p.n_pts = n_pts;
    p.n_src = n_src;
    p.n_snk = n_snk;
    p.alpha = (float)alpha;
    p.beta_f = (float)beta;
    p.beta_d = beta;
    p.out = d_out;
    p.err = device_error_word();
    path_field_kernel<<<grid_for(n_paths), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(p);
    note_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        record_cuda_error(e);
        return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

LYEM_API int lyem_path_time(const int32_t* d_paths, int64_t n_paths, int32_t n_cols, const float* d_pos,
                            const float* d_nrm, const float* d_w, const uint8_t* d_magnetic, const float* d_impedance,
                            int64_t n_pts, int64_t n_src, int64_t n_snk, double alpha, double beta, double* d_amp,
                            double* d_arrival, int32_t* d_pair, void* stream) {
    if (n_paths < 0 || n_cols < 2 || n_cols > 16 || n_pts < 0 || n_src < 0 || n_snk < 0) return LYEM_ERR_INVALID;
    if (n_paths == 0) return LYEM_OK;
    if (!d_paths || !d_pos || !d_nrm || !d_w || !d_amp || !d_arrival || !d_pair || n_pts == 0)
        return LYEM_ERR_INVALID;
    if (n_pts >= (1LL << 31) || n_src + n_snk > n_pts) return LYEM_ERR_INVALID;
    if (((uintptr_t)d_amp & 7u) || ((uintptr_t)d_arrival & 7u) || ((uintptr_t)d_w & 7u)) return LYEM_ERR_INVALID;
    PathParams p;
    p.paths = d_paths;
    p.n_paths = n_paths;
    p.cols = n_cols;
    p.pos = d_pos;
    p.nrm = d_nrm;
    p.w = d_w;
    p.magnetic = d_magnetic;
    p.impedance = d_impedance;
    p.n_pts = n_pts;
    p.n_src = n_src;
    p.n_snk = n_snk;
    p.alpha = (float)alpha;
    p.beta_f = (float)beta;
    p.beta_d = beta;
    p.out = nullptr;
    p.err = device_error_word();
    path_time_kernel<<<grid_for(n_paths), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(p, d_amp, d_arrival,
                                                                                           d_pair);
    note_launches(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        record_cuda_error(e);
        return LYEM_ERR_CUDA;
    }
    return LYEM_OK;
}

}  // extern "C"
