// lyem_grid.cuh -- binning specification and grid-build entry points (lyem_grid.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace lyem {

// A box of dims[0] x dims[1] x dims[2] cubic cells starting at org.  Axis k of
// the box measures coordinate comp[k] of the triangles (0 = x, 1 = y, 2 = z);
// cell id = (i2 * dims[1] + i1) * dims[0] + i0.  The 3-D traversal grid uses
// comp = (0, 1, 2); the reference's y-z tile bins use comp = (2, 1, 0) with
// dims = (nz, ny, 1), which gives its cell id iy * nz + iz.
struct BinSpec {
    float org[3];
    float cell, inv_cell;
    int dims[3];
    int comp[3];
    float pad;
};

size_t scan_workspace_ints(long long n);
cudaError_t exclusive_scan(const int* in, int* out, long long n, int* ws, cudaStream_t stream);

size_t spatial_order_workspace_bytes(long long n);
cudaError_t spatial_order(const float* pts, long long n, int* order, void* ws, cudaStream_t stream);
// Z-order of the points' directions from centre3 (workspace as spatial_order).
cudaError_t direction_order(const float* pts, long long n, const float* centre3, int* order, void* ws,
                            cudaStream_t stream);

size_t grid_count_workspace_bytes(long long n_tris);
cudaError_t grid_count(const BinSpec& b, const float4* tris, long long n_tris, int* tri_offsets,
                       unsigned long long* total, void* ws, cudaStream_t stream);

size_t grid_fill_workspace_bytes(long long n_refs, long long n_cells);
// Also writes the traversal's cell table cell_box[4 * ncells] (3-D grids only):
// per cell two children (its triangles split by a plane of least surface-area cost), each with the
// union of its padded triangle boxes (the boxes the binning used) clipped to the
// cell widened by two pads, and its ref range (see cell_fill_kernel).
cudaError_t grid_fill(const BinSpec& b, const float4* tris, long long n_tris, const int* tri_offsets, long long n_refs,
                      int* cell_start, float4* cell_tris, float4* cell_box, void* ws, cudaStream_t stream);
cudaError_t bin_fill_index(const BinSpec& b, const float4* tris, long long n_tris, const int* tri_offsets,
                           long long n_refs, const int* tri_index, int* cell_start, int* out_index, void* ws,
                           cudaStream_t stream);

}  // namespace lyem
