// lyem_grid.cu -- GPU build of the uniform grid used by the DDA stage, and of
// the y-z bins of the reference's tile structure.
//
// Steps (all on the device, no host loop over triangles or cells):
//   1. per-triangle padded box -> range of covered cells -> reference count;
//   2. exclusive scan of the counts (offsets per triangle, 64-bit total);
//   3. emit one (cell, triangle) key/value pair per reference, in triangle order;
//   4. stable LSD radix sort of the pairs by cell (8-bit digits), so the
//      triangles of a cell stay in ascending order and the build is deterministic;
//   5. cell ranges by binary search of the sorted keys;
//   6. gather the packed triangles into cell order (contiguous float4 loads
//      for the traversal);
//   7. per cell, its triangles split in two children at the cell's centre, each
//      child's box within the cell and ref range (one 64-byte record per cell
//      step of the traversal); steps 6 and 7 are one pass per cell.
// This replaces the reference's vertex binning with device asserts, its
// O(cells^2) single-block offset computation and its atomicCAS slot
// insertion (lyceanem/src/terrain_acceleration_build.cuh:30-205, 287-431) and
// the host prefix sum of lyceanem/src/frequency_domain_models.cu:118-123.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "lyem_device.cuh"
#include "lyem_grid.cuh"
#include "lyem_internal.cuh"

namespace lyem {

// ------------------------------------------------------------------ bounds
__global__ void tris_bounds_kernel(const float4* __restrict__ tris, long long n, float* bounds6) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        float4 v0 = tris[3 * t], e1 = tris[3 * t + 1], e2 = tris[3 * t + 2];
        float a[3] = {v0.x, v0.y, v0.z};
        float b[3] = {v0.x + e1.x, v0.y + e1.y, v0.z + e1.z};
        float c[3] = {v0.x + e2.x, v0.y + e2.y, v0.z + e2.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], fminf(a[k], fminf(b[k], c[k])));
            hi[k] = fmaxf(hi[k], fmaxf(a[k], fmaxf(b[k], c[k])));
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_down_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_down_sync(0xffffffffu, hi[k], o));
        }
    }
    __shared__ float s[6][32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        for (int k = 0; k < 3; ++k) { s[k][w] = lo[k]; s[3 + k][w] = hi[k]; }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int nw = blockDim.x >> 5;
        float v = s[threadIdx.x][0];
        for (int i = 1; i < nw; ++i) v = threadIdx.x < 3 ? fminf(v, s[threadIdx.x][i]) : fmaxf(v, s[threadIdx.x][i]);
        // order-preserving integer encoding for float atomics
        int bits = __float_as_int(v);
        int key = bits >= 0 ? bits : (bits ^ 0x7fffffff);
        if (threadIdx.x < 3) atomicMin(reinterpret_cast<int*>(bounds6) + threadIdx.x, key);
        else atomicMax(reinterpret_cast<int*>(bounds6) + threadIdx.x, key);
    }
}

__global__ void bounds_init_kernel(float* bounds6) {
    int i = threadIdx.x;
    if (i < 6) {
        float v = i < 3 ? INFINITY : -INFINITY;
        int bits = __float_as_int(v);
        reinterpret_cast<int*>(bounds6)[i] = bits >= 0 ? bits : (bits ^ 0x7fffffff);
    }
}

__global__ void bounds_decode_kernel(float* bounds6) {
    int i = threadIdx.x;
    if (i < 6) {
        int key = reinterpret_cast<int*>(bounds6)[i];
        int bits = key >= 0 ? key : (key ^ 0x7fffffff);
        bounds6[i] = __int_as_float(bits);
    }
}

cudaError_t launch_tris_bounds(const float4* tris, long long n_tris, float* bounds6, cudaStream_t stream) {
    bounds_init_kernel<<<1, 32, 0, stream>>>(bounds6); note_launches(1);
    const unsigned blocks = capped_blocks(n_tris, 256, 8);
    tris_bounds_kernel<<<blocks, 256, 0, stream>>>(tris, n_tris, bounds6); note_launches(1);
    bounds_decode_kernel<<<1, 32, 0, stream>>>(bounds6); note_launches(1);
    return cudaGetLastError();
}

// --------------------------------------------------------- cell coverage
__device__ __forceinline__ void covered_range(const BinSpec& b, const float4* tris, long long t, int i0[3],
                                              int i1[3]) {
    float4 v0 = tris[3 * t], e1 = tris[3 * t + 1], e2 = tris[3 * t + 2];
    float a[3] = {v0.x, v0.y, v0.z};
    float e[3] = {e1.x, e1.y, e1.z};
    float f[3] = {e2.x, e2.y, e2.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int c = b.comp[k];
        float p = a[c], q = a[c] + e[c], r = a[c] + f[c];
        float lo = fminf(p, fminf(q, r)) - b.pad, hi = fmaxf(p, fmaxf(q, r)) + b.pad;
        float fl = floorf((lo - b.org[k]) * b.inv_cell), fh = floorf((hi - b.org[k]) * b.inv_cell);
        // clamp in float first so huge or NaN coordinates cannot overflow the int conversion
        fl = fminf(fmaxf(fl, 0.f), (float)(b.dims[k] - 1));
        fh = fminf(fmaxf(fh, 0.f), (float)(b.dims[k] - 1));
        if (!(fl == fl)) fl = 0.f;
        if (!(fh == fh)) fh = 0.f;
        i0[k] = (int)fl;
        i1[k] = (int)fh;
        if (i1[k] < i0[k]) i1[k] = i0[k];
    }
}

__global__ void count_refs_kernel(BinSpec b, const float4* __restrict__ tris, long long n, int* counts,
                                  unsigned long long* total) {
    unsigned long long local = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i0[3], i1[3];
        covered_range(b, tris, t, i0, i1);
        long long c = (long long)(i1[0] - i0[0] + 1) * (i1[1] - i0[1] + 1) * (i1[2] - i0[2] + 1);
        counts[t] = c > 0x7fffffffLL ? 0x7fffffff : (int)c;
        local += (unsigned long long)c;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(total, local);
}

__global__ void emit_refs_kernel(BinSpec b, const float4* __restrict__ tris, long long n,
                                 const int* __restrict__ offsets, int* keys, int* vals) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i0[3], i1[3];
        covered_range(b, tris, t, i0, i1);
        int o = offsets[t];
        for (int z = i0[2]; z <= i1[2]; ++z)
            for (int y = i0[1]; y <= i1[1]; ++y)
                for (int x = i0[0]; x <= i1[0]; ++x) {
                    keys[o] = (z * b.dims[1] + y) * b.dims[0] + x;
                    vals[o] = (int)t;
                    ++o;
                }
    }
}

// ----------------------------------------------------------------- scan
// Exclusive scan of int32 in 1024-element blocks, recursive over block sums.
constexpr int kScanBlock = 1024;

__global__ void scan_block_kernel(const int* __restrict__ in, int* out, long long n, int* block_sums) {
    __shared__ int warp_tot[8];
    const long long base = (long long)blockIdx.x * kScanBlock;
    const int tid = threadIdx.x;  // 256 threads x 4 items
    int v[4];
    int run = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        long long i = base + 4 * tid + j;
        v[j] = i < n ? in[i] : 0;
        run += v[j];
    }
    // inclusive scan of per-thread totals across the block
    int x = run;
    const int lane = tid & 31, w = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < 8 ? warp_tot[lane] : 0;
        for (int o = 1; o < 8; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < 8) warp_tot[lane] = t;
    }
    __syncthreads();
    int excl = x - run + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        long long i = base + 4 * tid + j;
        if (i < n) out[i] = excl;
        excl += v[j];
    }
    if (tid == 255 && block_sums) block_sums[blockIdx.x] = warp_tot[7];
}

__global__ void add_block_offsets_kernel(int* out, long long n, const int* __restrict__ block_offsets) {
    const long long base = (long long)blockIdx.x * kScanBlock;
    const int add = block_offsets[blockIdx.x];
    for (int j = threadIdx.x; j < kScanBlock; j += blockDim.x) {
        long long i = base + j;
        if (i < n) out[i] += add;
    }
}

size_t scan_workspace_ints(long long n) {
    size_t total = 0;
    while (n > 1) {
        long long nb = (n + kScanBlock - 1) / kScanBlock;
        total += (size_t)nb * 2 + 64;
        n = nb;
    }
    return total + 64;
}

// out = exclusive_scan(in); ws must hold scan_workspace_ints(n) ints.
cudaError_t exclusive_scan(const int* in, int* out, long long n, int* ws, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    long long nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 1) {
        scan_block_kernel<<<1, 256, 0, stream>>>(in, out, n, nullptr); note_launches(1);
        return cudaGetLastError();
    }
    int* sums = ws;
    int* sums_scanned = ws + nb + 32;
    int* rest = sums_scanned + nb + 32;
    scan_block_kernel<<<(unsigned)nb, 256, 0, stream>>>(in, out, n, sums); note_launches(1);
    cudaError_t e = exclusive_scan(sums, sums_scanned, nb, rest, stream);
    if (e != cudaSuccess) return e;
    add_block_offsets_kernel<<<(unsigned)nb, 256, 0, stream>>>(out, n, sums_scanned); note_launches(1);
    return cudaGetLastError();
}

// ----------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__global__ void radix_hist_kernel(const int* __restrict__ keys, long long n, int shift, int* hist, int nblocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        long long idx = base + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void radix_scatter_kernel(const int* __restrict__ kin, const int* __restrict__ vin, int* kout, int* vout,
                                     long long n, int shift, const int* __restrict__ hist_scanned, int nblocks) {
    __shared__ int base[256];
    __shared__ int wcnt[kSortThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    base[tid] = hist_scanned[(long long)tid * nblocks + blockIdx.x];
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        const long long idx = (long long)blockIdx.x * kSortTile + r * kSortThreads + tid;
        const bool valid = idx < n;
        int key = 0, val = 0, d = 0;
        if (valid) {
            key = kin[idx];
            val = vin[idx];
            d = (key >> shift) & 255;
        }
#pragma unroll
        for (int j = 0; j < kSortThreads / 32; ++j) wcnt[j][tid] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 256 + lane);
        const int rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int off = base[d] + rank;
            for (int j = 0; j < w; ++j) off += wcnt[j][d];
            kout[off] = key;
            vout[off] = val;
        }
        __syncthreads();
        int s = 0;
#pragma unroll
        for (int j = 0; j < kSortThreads / 32; ++j) s += wcnt[j][tid];
        base[tid] += s;
        __syncthreads();
    }
}

// Stable sort of (key, value) by key in [0, key_limit).  Sorted output ends
// in (k0, v0) or (k1, v1); returns which through *in_first.
cudaError_t radix_sort_pairs(int* k0, int* v0, int* k1, int* v1, long long n, int key_limit, int* hist,
                             int* hist_scanned, int* scan_ws, bool* in_first, cudaStream_t stream) {
    int bits = 0;
    while (bits < 31 && (1LL << bits) < (long long)key_limit) ++bits;
    const int passes = (bits + 7) / 8;
    const int nblocks = (int)((n + kSortTile - 1) / kSortTile);
    int *ki = k0, *vi = v0, *ko = k1, *vo = v1;
    for (int p = 0; p < passes; ++p) {
        radix_hist_kernel<<<nblocks, kSortThreads, 0, stream>>>(ki, n, 8 * p, hist, nblocks); note_launches(1);
        cudaError_t e = exclusive_scan(hist, hist_scanned, 256LL * nblocks, scan_ws, stream);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<nblocks, kSortThreads, 0, stream>>>(ki, vi, ko, vo, n, 8 * p, hist_scanned, nblocks); note_launches(1);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    *in_first = (ki == k0);
    return cudaGetLastError();
}

__global__ void cell_start_kernel(const int* __restrict__ keys, long long n, long long ncells, int* cell_start) {
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c <= ncells;
         c += (long long)gridDim.x * blockDim.x) {
        long long lo = 0, hi = n;
        while (lo < hi) {
            long long mid = (lo + hi) >> 1;
            if (keys[mid] < c) lo = mid + 1;
            else hi = mid;
        }
        cell_start[c] = (int)lo;
    }
}

__global__ void gather_tris_kernel(const float4* __restrict__ tris, const int* __restrict__ vals, long long n,
                                   float4* out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / 3;
        int c = (int)(i - 3 * r);
        out[i] = tris[3 * (long long)vals[r] + c];
    }
}

// Cell table of the traversal and the cell-ordered triangles, one thread per
// cell.  A cell's triangles are split by an axis-aligned plane (surface-area
// cost, below) into two children, A (centroid below) then B, each
// kept in the (ascending) triangle order of the sorted refs, and the record of
// cell c is four float4:
//   (loA.xyz, first ref) (hiA.xyz, first ref of B) (loB.xyz, first ref of B) (hiB.xyz, end ref)
// (refs as int bits), [lo, hi] of a child being the union of the padded boxes of
// its triangles (vertices and pad exactly as covered_range computes them),
// clipped to the cell widened by two pads.  A segment whose exact path misses a
// child's box cannot hit a triangle of that child inside the cell (a hit point
// lies in its triangle's box and in the cell, at least a pad inside the clipped
// box), and a hit outside the cell is found in the cell that holds it.  Empty
// children get lo = +inf, hi = -inf.  Non-finite triangle coordinates are
// ignored by fminf/fmaxf: such triangles never pass the ray-triangle test.
__device__ __forceinline__ void tri_box(const BinSpec& b, float4 v0, float4 e1, float4 e2, float lo[3], float hi[3]) {
    const float a[3] = {v0.x, v0.y, v0.z}, e[3] = {e1.x, e1.y, e1.z}, f[3] = {e2.x, e2.y, e2.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float p = a[k], q = a[k] + e[k], s = a[k] + f[k];
        lo[k] = fminf(lo[k], fminf(p, fminf(q, s)) - b.pad);
        hi[k] = fmaxf(hi[k], fmaxf(p, fmaxf(q, s)) + b.pad);
    }
}

__device__ __forceinline__ float tri_centroid(float4 v0, float4 e1, float4 e2, int k) {
    const float a[3] = {v0.x, v0.y, v0.z}, e[3] = {e1.x, e1.y, e1.z}, f[3] = {e2.x, e2.y, e2.z};
    return a[k] + (e[k] + f[k]) * (1.f / 3.f);
}

__global__ void cell_fill_kernel(BinSpec b, const float4* __restrict__ tris, const int* __restrict__ vals,
                                 const int* __restrict__ cell_start, long long ncells, float4* __restrict__ cell_tris,
                                 float4* __restrict__ box) {
    const long long plane = (long long)b.dims[0] * b.dims[1];
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncells;
         c += (long long)gridDim.x * blockDim.x) {
        const int q0 = cell_start[c], q1 = cell_start[c + 1];
        const long long iz = c / plane, rem = c - iz * plane, iy = rem / b.dims[0], ix = rem - iy * b.dims[0];
        const float ci[3] = {(float)ix, (float)iy, (float)iz};
        // split: of the planes at k/8 of the cell (k = 1..7) on each axis, the one
        // with the least surface-area cost (the clipped child boxes' areas times
        // their triangle counts, a ray's chance of entering a box being about
        // proportional to its area); a triangle goes to child A when its centroid
        // lies below the plane.  Visibility does not depend on the split.
        int ax = 0;
        float mid = b.org[0] + (ci[0] + 0.5f) * b.cell;
        if (q1 - q0 > 1) {
            float best = INFINITY;
            for (int a = 0; a < 3; ++a) {
                for (int k = 1; k < 8; ++k) {
                    const float plane = b.org[a] + (ci[a] + 0.125f * (float)k) * b.cell;
                    float lo[2][3], hi[2][3];
                    int n[2] = {0, 0};
#pragma unroll
                    for (int h = 0; h < 2; ++h)
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            lo[h][d] = INFINITY;
                            hi[h][d] = -INFINITY;
                        }
                    for (int r = q0; r < q1; ++r) {
                        const float4* t = tris + 3 * (long long)vals[r];
                        const float4 v0 = t[0], e1 = t[1], e2 = t[2];
                        const int h = tri_centroid(v0, e1, e2, a) < plane ? 0 : 1;
                        ++n[h];
                        tri_box(b, v0, e1, e2, lo[h], hi[h]);
                    }
                    float cost = 0.f;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (!n[h]) continue;
                        float ext[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            const float c0 = b.org[d] + ci[d] * b.cell;
                            ext[d] = fmaxf(fminf(hi[h][d], c0 + b.cell + 2.f * b.pad) -
                                               fmaxf(lo[h][d], c0 - 2.f * b.pad), 0.f);
                        }
                        cost += (ext[0] * ext[1] + ext[1] * ext[2] + ext[2] * ext[0]) * (float)n[h];
                    }
                    if (cost < best) {
                        best = cost;
                        ax = a;
                        mid = plane;
                    }
                }
            }
        }
        int na = 0;
        for (int r = q0; r < q1; ++r) {
            const float4* t = tris + 3 * (long long)vals[r];
            na += tri_centroid(t[0], t[1], t[2], ax) < mid ? 1 : 0;
        }
        float loA[3] = {INFINITY, INFINITY, INFINITY}, hiA[3] = {-INFINITY, -INFINITY, -INFINITY};
        float loB[3] = {INFINITY, INFINITY, INFINITY}, hiB[3] = {-INFINITY, -INFINITY, -INFINITY};
        int ia = q0, ib = q0 + na;
        for (int r = q0; r < q1; ++r) {
            const float4* t = tris + 3 * (long long)vals[r];
            const float4 v0 = t[0], e1 = t[1], e2 = t[2];
            const bool in_a = tri_centroid(v0, e1, e2, ax) < mid;
            const int o = in_a ? ia++ : ib++;
            cell_tris[3 * (long long)o] = v0;
            cell_tris[3 * (long long)o + 1] = e1;
            cell_tris[3 * (long long)o + 2] = e2;
            if (in_a) tri_box(b, v0, e1, e2, loA, hiA);
            else tri_box(b, v0, e1, e2, loB, hiB);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c0 = b.org[k] + ci[k] * b.cell;
            const float clo = c0 - 2.f * b.pad, chi = c0 + b.cell + 2.f * b.pad;
            loA[k] = fmaxf(loA[k], clo);
            hiA[k] = fminf(hiA[k], chi);
            loB[k] = fmaxf(loB[k], clo);
            hiB[k] = fminf(hiB[k], chi);
        }
        const int qm = q0 + na;
        box[4 * c] = make_float4(loA[0], loA[1], loA[2], __int_as_float(q0));
        box[4 * c + 1] = make_float4(hiA[0], hiA[1], hiA[2], __int_as_float(qm));
        box[4 * c + 2] = make_float4(loB[0], loB[1], loB[2], __int_as_float(qm));
        box[4 * c + 3] = make_float4(hiB[0], hiB[1], hiB[2], __int_as_float(q1));
    }
}

__global__ void gather_index_kernel(const int* __restrict__ tri_index, const int* __restrict__ vals, long long n,
                                    int* out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n;
         i += (long long)gridDim.x * blockDim.x) {
        long long r = i / 3;
        int c = (int)(i - 3 * r);
        out[i] = tri_index[3 * (long long)vals[r] + c];
    }
}

// ------------------------------------------------------- spatial order
// Morton (Z-order) sort of a point set: consecutive entries of the order are
// close in space, so a warp or block given consecutive points traces coherent rays.
__global__ void points_bounds_kernel(const float* __restrict__ pts, long long n, float* bounds6) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float v = pts[3 * i + k];
            lo[k] = fminf(lo[k], v);
            hi[k] = fmaxf(hi[k], v);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_down_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_down_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 6; ++k) {
            float v = k < 3 ? lo[k] : hi[k - 3];
            int bits = __float_as_int(v);
            int key = bits >= 0 ? bits : (bits ^ 0x7fffffff);
            if (k < 3) atomicMin(reinterpret_cast<int*>(bounds6) + k, key);
            else atomicMax(reinterpret_cast<int*>(bounds6) + k, key);
        }
    }
}

__device__ __forceinline__ unsigned spread10(unsigned x) {
    x &= 1023u;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void morton_kernel(const float* __restrict__ pts, long long n, const float* __restrict__ bounds6,
                              int* keys, int* vals) {
    float lo[3], sc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = bounds6[k];
        float ext = bounds6[3 + k] - lo[k];
        sc[k] = ext > 0.f ? 1023.f / ext : 0.f;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float q = (pts[3 * i + k] - lo[k]) * sc[k];
            q = fminf(fmaxf(q, 0.f), 1023.f);
            if (!(q == q)) q = 0.f;
            c[k] = (unsigned)q;
        }
        keys[i] = (int)(spread10(c[0]) | (spread10(c[1]) << 1) | (spread10(c[2]) << 2));
        vals[i] = (int)i;
    }
}

// Direction tiles: elevation el in [-pi/2, pi/2] and azimuth az in [-pi, pi]
// of each point seen from c are cut into square tiles of edge `tile` radians
// (offset by 1/8 tile); the key orders tiles by (elevation band, azimuth
// tile) and points within a tile by 6-bit (elevation, azimuth) positions.
// nb * na < 2^18 keeps keys below 2^30.
__global__ void direction_key_kernel(const float* __restrict__ pts, long long n, float cx, float cy, float cz,
                                     float tile, int nb, int na, int* keys, int* vals) {
    const float kPi = 3.14159265358979f;
    const float inv = 1.f / tile;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float dx = pts[3 * i] - cx, dy = pts[3 * i + 1] - cy, dz = pts[3 * i + 2] - cz;
        const float fe = (atan2f(dz, hypotf(dx, dy)) + 0.5f * kPi) * inv + 0.125f;
        const float fa = (atan2f(dy, dx) + kPi) * inv + 0.125f;
        int key = 0;
        if (fe == fe && fa == fa) {
            const float be = fminf(fmaxf(floorf(fe), 0.f), (float)(nb - 1));
            const float ba = fminf(fmaxf(floorf(fa), 0.f), (float)(na - 1));
            const int qe = (int)fminf(fmaxf((fe - be) * 64.f, 0.f), 63.f);
            const int qa = (int)fminf(fmaxf((fa - ba) * 64.f, 0.f), 63.f);
            key = ((((int)be * na + (int)ba) << 12) | (qe << 6) | qa);
        }
        keys[i] = key;
        vals[i] = (int)i;
    }
}

cudaError_t direction_order(const float* pts, long long n, const float* centre3, int* order, void* ws,
                            cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    int* k0 = static_cast<int*>(ws) + 64;
    int* v0 = k0 + n + 64;
    int* k1 = v0 + n + 64;
    int* v1 = k1 + n + 64;
    const long long nblocks = (n + kSortTile - 1) / kSortTile;
    int* hist = v1 + n + 64;
    int* hist_scanned = hist + 256 * nblocks + 64;
    int* scan_ws = hist_scanned + 256 * nblocks + 64;
    const unsigned b = capped_blocks(n, 256, 8);
    // tiles of about 16 points if the set were an even elevation-azimuth grid (n points over pi x 2 pi)
    const double kPi = 3.14159265358979323846;
    const double tile = std::max(0.009, 4.0 * std::sqrt(2.0 * kPi * kPi / (double)n));
    const int nb = (int)std::ceil(kPi / tile) + 2, na = (int)std::ceil(2.0 * kPi / tile) + 2;
    direction_key_kernel<<<b, 256, 0, stream>>>(pts, n, centre3[0], centre3[1], centre3[2], (float)tile,
                                                          nb, na, k0, v0);
    note_launches(1);
    bool first = true;
    cudaError_t e = radix_sort_pairs(k0, v0, k1, v1, n, 1 << 30, hist, hist_scanned, scan_ws, &first, stream);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(order, first ? v0 : v1, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, stream);
}

size_t spatial_order_workspace_bytes(long long n) {
    const long long nblocks = (n + kSortTile - 1) / kSortTile;
    size_t ints = 64 + (size_t)4 * (n + 64) + (size_t)2 * (256 * nblocks + 64) + scan_workspace_ints(256 * nblocks);
    return ints * sizeof(int) + 256;
}

cudaError_t spatial_order(const float* pts, long long n, int* order, void* ws, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    float* bounds = static_cast<float*>(ws);
    int* k0 = static_cast<int*>(ws) + 64;
    int* v0 = k0 + n + 64;
    int* k1 = v0 + n + 64;
    int* v1 = k1 + n + 64;
    const long long nblocks = (n + kSortTile - 1) / kSortTile;
    int* hist = v1 + n + 64;
    int* hist_scanned = hist + 256 * nblocks + 64;
    int* scan_ws = hist_scanned + 256 * nblocks + 64;
    bounds_init_kernel<<<1, 32, 0, stream>>>(bounds); note_launches(1);
    const unsigned b = capped_blocks(n, 256, 8);
    points_bounds_kernel<<<b, 256, 0, stream>>>(pts, n, bounds); note_launches(1);
    bounds_decode_kernel<<<1, 32, 0, stream>>>(bounds); note_launches(1);
    morton_kernel<<<b, 256, 0, stream>>>(pts, n, bounds, k0, v0); note_launches(1);
    bool first = true;
    cudaError_t e = radix_sort_pairs(k0, v0, k1, v1, n, 1 << 30, hist, hist_scanned, scan_ws, &first, stream);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(order, first ? v0 : v1, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, stream);
}

static unsigned grid_blocks(long long n, int threads) { return capped_blocks(n, threads, 32); }

// --------------------------------------------------------------- phases
size_t grid_count_workspace_bytes(long long n_tris) {
    return (size_t)(n_tris + 1 + 64) * sizeof(int) + scan_workspace_ints(n_tris + 1) * sizeof(int) + 256;
}

cudaError_t grid_count(const BinSpec& b, const float4* tris, long long n_tris, int* tri_offsets,
                       unsigned long long* total, void* ws, cudaStream_t stream) {
    int* counts = static_cast<int*>(ws);
    int* scan_ws = counts + n_tris + 1 + 64;
    cudaError_t e = cudaMemsetAsync(total, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(counts + n_tris, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    if (n_tris > 0) { count_refs_kernel<<<grid_blocks(n_tris, 256), 256, 0, stream>>>(b, tris, n_tris, counts, total); note_launches(1); }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return exclusive_scan(counts, tri_offsets, n_tris + 1, scan_ws, stream);
}

size_t grid_fill_workspace_bytes(long long n_refs, long long n_cells) {
    (void)n_cells;
    const long long nblocks = (n_refs + kSortTile - 1) / kSortTile;
    size_t ints = (size_t)4 * (n_refs + 64) + (size_t)2 * (256 * nblocks + 64) + scan_workspace_ints(256 * nblocks);
    return ints * sizeof(int) + 256;
}

// Sorted (cell, triangle) pairs; *vals_out points into ws.
cudaError_t grid_sort(const BinSpec& b, const float4* tris, long long n_tris, const int* tri_offsets,
                      long long n_refs, int* cell_start, const int** vals_out, void* ws, cudaStream_t stream) {
    int* k0 = static_cast<int*>(ws);
    int* v0 = k0 + n_refs + 64;
    int* k1 = v0 + n_refs + 64;
    int* v1 = k1 + n_refs + 64;
    const long long nblocks = (n_refs + kSortTile - 1) / kSortTile;
    int* hist = v1 + n_refs + 64;
    int* hist_scanned = hist + 256 * nblocks + 64;
    int* scan_ws = hist_scanned + 256 * nblocks + 64;
    const long long ncells = (long long)b.dims[0] * b.dims[1] * b.dims[2];
    if (n_refs > 0) { emit_refs_kernel<<<grid_blocks(n_tris, 256), 256, 0, stream>>>(b, tris, n_tris, tri_offsets, k0, v0); note_launches(1); }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bool first = true;
    if (n_refs > 0) {
        e = radix_sort_pairs(k0, v0, k1, v1, n_refs, (int)ncells, hist, hist_scanned, scan_ws, &first, stream);
        if (e != cudaSuccess) return e;
    }
    const int* keys = first ? k0 : k1;
    *vals_out = first ? v0 : v1;
    cell_start_kernel<<<grid_blocks(ncells + 1, 256), 256, 0, stream>>>(keys, n_refs, ncells, cell_start); note_launches(1);
    return cudaGetLastError();
}

cudaError_t grid_fill(const BinSpec& b, const float4* tris, long long n_tris, const int* tri_offsets, long long n_refs,
                      int* cell_start, float4* cell_tris, float4* cell_box, void* ws, cudaStream_t stream) {
    const int* vals = nullptr;
    cudaError_t e = grid_sort(b, tris, n_tris, tri_offsets, n_refs, cell_start, &vals, ws, stream);
    if (e != cudaSuccess) return e;
    const long long ncells = (long long)b.dims[0] * b.dims[1] * b.dims[2];
    if (cell_box) {
        cell_fill_kernel<<<grid_blocks(ncells, 128), 128, 0, stream>>>(b, tris, vals, cell_start, ncells, cell_tris,
                                                                      cell_box);
        note_launches(1);
    } else if (n_refs > 0) {
        gather_tris_kernel<<<grid_blocks(3 * n_refs, 256), 256, 0, stream>>>(tris, vals, n_refs, cell_tris);
        note_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t bin_fill_index(const BinSpec& b, const float4* tris, long long n_tris, const int* tri_offsets,
                           long long n_refs, const int* tri_index, int* cell_start, int* out_index, void* ws,
                           cudaStream_t stream) {
    const int* vals = nullptr;
    cudaError_t e = grid_sort(b, tris, n_tris, tri_offsets, n_refs, cell_start, &vals, ws, stream);
    if (e != cudaSuccess) return e;
    if (n_refs > 0)
        gather_index_kernel<<<grid_blocks(3 * n_refs, 256), 256, 0, stream>>>(tri_index, vals, n_refs, out_index); note_launches(1);
    return cudaGetLastError();
}

}  // namespace lyem
