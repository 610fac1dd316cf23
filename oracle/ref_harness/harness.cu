// harness.cu -- runs the reference's own device functions on chosen inputs.
//
// TEST INFRASTRUCTURE ONLY: compiled (by build_ref.py, where the reference tree
// is mounted) against the reference's headers into oracle/_ref/*.cubin, loaded
// on a GPU by run_ref.py to produce golden vectors that pin the oracle.
//
// The kernel below calls the reference's points_to_rays, hit and em_wave
// (lyceanem/src/raycasting.cuh:19-95, lyceanem/src/em.cuh:18-120) for every
// (source, sink) pair exactly as raycast_brute_force / intersection_brute_force
// do (lyceanem/src/raycasting_brute_force.cuh:19-88): edges formed per test from
// the indexed vertices, the pair skip rule on `flag`, no early exit.  It omits
// only the brute-force kernel's shared-memory triangle tile, which every
// thread rewrites without a barrier (raycasting_brute_force.cuh:36-43).
#include "raycasting.cuh"
#include "em.cuh"
// Also puts the reference's own set_values and raycast_brute_force kernels
// (lyceanem/src/raycasting.cuh:97-108, raycasting_brute_force.cuh:68-88) into
// the cubin, so that time_ref.py can launch them as raycast_wrapper_brute_force
// does (<<<32, 512>>>, raycasting_brute_force.cuh:152-170) and time them.
#include "raycasting_brute_force.cuh"

extern "C" __global__ void ref_pairs(float3* source, float3* end, float4* ray, int source_num, int end_num, int flag,
                                     float3* tri_vertex, int3* triangle_index, int tri_num, PointData* points,
                                     float wave_length, float2 alpha_beta, unsigned char* vis_out,
                                     complex_float3* field_out) {
    const int n_pairs = source_num * end_num;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pairs; i += blockDim.x * gridDim.x) {
        points_to_rays(i, source, end, ray, source_num, end_num, flag);
        const int c = i / end_num, d = i % end_num;
        bool blocked = false;
        if (flag || c != d) {
            const float4 r = ray[i];
            for (int t = 0; t < tri_num; ++t) {
                const int3 idx = triangle_index[t];
                const bool b = hit(make_float3(r.x, r.y, r.z), r.w, source[c], tri_vertex[idx.y] - tri_vertex[idx.x],
                                   tri_vertex[idx.z] - tri_vertex[idx.x], tri_vertex[idx.x]);
                blocked = b ? true : blocked;
            }
        }
        vis_out[i] = blocked ? 0 : 1;
        complex_float3 f;
        f.x = make_cuFloatComplex(0.f, 0.f);
        f.y = f.x;
        f.z = f.x;
        if (!blocked) f = em_wave(alpha_beta, ray[i], points[c], points[d + source_num], wave_length);
        field_out[i] = f;
    }
}
