// lyem_walk.cuh -- one segment's any-hit walk through the uniform grid, shared
// by the pair-stage kernels (lyem_stage.cu) and the batched kernel (lyem_batch.cu).
// Amanatides-Woo; boundary crossings are recomputed from the cell index, so no
// error accumulates; triangles are stored contiguously per cell (float4 loads).
// Entering a cell reads its 32-byte record (box of its triangles, ref range)
// and skips the cell's triangles when the segment misses the box.
// GP is any parameter block with the grid fields of StageParams (g0, g1, cell,
// inv_cell, dims, cell_box, cell_tris, eps).
#pragma once
#include "lyem_device.cuh"
#include "lyem_internal.cuh"

namespace lyem {

struct Walk {
    float ox, oy, oz;
    Ray r;
    float ix, iy, iz, t1;
    int cx, cy, cz, q, q1, guard;
};

// True when the segment certainly misses box [lo, hi]: slab test over the
// parameter range [0, len] (a cell's own range is a part of it).  The computed
// slab parameters carry relative errors of a few units of 2^-24, so the box
// counts as missed only when the entry parameter exceeds the exit parameter by
// more than 2^-19 of it; NaN parameters never make a miss.  An axis the segment
// is parallel to (direction component 0) has the finite stand-in +-2^100 for
// 1/D (walk_setup), so its slab parameters are 0 or of magnitude 2^100 |L - O|:
// outside the slab the box is missed, inside it the slab cuts nothing, and a
// segment within about 2^-100 t of a face can be counted as missing the box.
// That is safe: a box is the union of its triangles' boxes padded by `pad`
// (clipped to the cell widened by two pads), so every hit point lies at least
// a pad inside it, and 2^-100 t is far below any pad.
__device__ __forceinline__ bool box_missed(const Walk& w, float4 lo, float4 hi) {
    float tmin = 0.f, tmax = w.r.len;
#define LYEM_BOX(O, INV, L, H)                                        \
    {                                                                 \
        const float ta = (L - O) * INV, tb = (H - O) * INV;           \
        tmin = fmaxf(tmin, fminf(ta, tb));                            \
        tmax = fminf(tmax, fmaxf(ta, tb));                            \
    }
    LYEM_BOX(w.ox, w.ix, lo.x, hi.x)
    LYEM_BOX(w.oy, w.iy, lo.y, hi.y)
    LYEM_BOX(w.oz, w.iz, lo.z, hi.z)
#undef LYEM_BOX
    return __fmul_rn(tmin, 1.f - 0x1p-19f) > tmax;
}

// Enters cell c: the ref range of the children whose boxes the segment may
// cross (child A's refs come first, then B's, so the union is one range).
template <class GP>
__device__ __forceinline__ void walk_enter(const GP& p, Walk& w, int c) {
    const float4* rec = p.cell_box + 4 * (long long)c;
    int q, qm, q1;
    {
        const float4 loA = __ldg(rec), hiA = __ldg(rec + 1);
        q = __float_as_int(loA.w);
        qm = __float_as_int(hiA.w);
        if (q < qm && box_missed(w, loA, hiA)) q = qm;
    }
    {
        const float4 loB = __ldg(rec + 2), hiB = __ldg(rec + 3);
        q1 = __float_as_int(hiB.w);
        if (qm < q1 && box_missed(w, loB, hiB)) q1 = qm;
    }
    w.q = q;
    w.q1 = q < q1 ? q1 : q;
}

// The segment o -> e of a walk (origin and visibility ray of the mode); enough for walk_test_ref.
template <bool CULL>
__device__ __forceinline__ void walk_ray(Walk& w, float ox, float oy, float oz, float ex, float ey, float ez) {
    w.ox = ox; w.oy = oy; w.oz = oz;
    w.r = vis_ray<CULL>(ox, oy, oz, ex, ey, ez);
}

// Enters the grid along the segment set by walk_ray; false if it misses the grid box.
template <class GP>
__device__ __forceinline__ bool walk_setup(const GP& p, Walk& w) {
    const float ox = w.ox, oy = w.oy, oz = w.oz;
    float t0 = 0.f;
    w.t1 = w.r.len;
    bool miss = false;
#define LYEM_SLAB(D, O, G0, G1, INV)                       \
    if (D == 0.f) {                                        \
        INV = copysignf(0x1p100f, D);                      \
        if (O < G0 || O > G1) miss = true;                 \
    } else {                                               \
        INV = 1.0f / D;                                    \
        float ta = (G0 - O) * INV, tb = (G1 - O) * INV;    \
        t0 = fmaxf(t0, fminf(ta, tb));                     \
        w.t1 = fminf(w.t1, fmaxf(ta, tb));                 \
    }
    LYEM_SLAB(w.r.dx, ox, p.g0[0], p.g1[0], w.ix)
    LYEM_SLAB(w.r.dy, oy, p.g0[1], p.g1[1], w.iy)
    LYEM_SLAB(w.r.dz, oz, p.g0[2], p.g1[2], w.iz)
#undef LYEM_SLAB
    if (miss || !(t0 <= w.t1)) return false;
    w.cx = min(max((int)floorf((ox + t0 * w.r.dx - p.g0[0]) * p.inv_cell), 0), p.dims[0] - 1);
    w.cy = min(max((int)floorf((oy + t0 * w.r.dy - p.g0[1]) * p.inv_cell), 0), p.dims[1] - 1);
    w.cz = min(max((int)floorf((oz + t0 * w.r.dz - p.g0[2]) * p.inv_cell), 0), p.dims[2] - 1);
    w.guard = p.dims[0] + p.dims[1] + p.dims[2] + 2;
    walk_enter(p, w, (w.cz * p.dims[1] + w.cy) * p.dims[0] + w.cx);
    return true;
}

// Starts the walk of segment o -> e; false if the segment misses the grid box.
template <bool CULL, class GP>
__device__ __forceinline__ bool walk_begin(const GP& p, Walk& w, float ox, float oy, float oz, float ex,
                                           float ey, float ez) {
    walk_ray<CULL>(w, ox, oy, oz, ex, ey, ez);
    return walk_setup(p, w);
}

// Tests triangle q of the current cell and advances q; true on a hit.
template <bool CULL, class GP>
__device__ __forceinline__ bool walk_test(const GP& p, Walk& w) {
    const float4* t = p.cell_tris + 3 * (long long)w.q;
    const float4 v0 = __ldg(t), e1 = __ldg(t + 1), e2 = __ldg(t + 2);
    ++w.q;
    return hit_full<CULL>(w.r, w.ox, w.oy, w.oz, v0, e1, e2, p.eps);
}

// Cell-order reference of the triangle of o's cell whose centroid is nearest
// to point o relative to the triangle's size (squared distance over squared
// longest edge), if o lies within that size of it; -1 otherwise (o off every
// triangle of its cell, outside the grid box, or its cell empty).  Called by
// all 32 lanes of a warp with the same o; every lane gets the same answer.  A
// ray leaving a point that lies on (or just off) a surface is most often
// blocked by that surface's own triangle, so the walk tries this one first.
template <class GP>
__device__ __forceinline__ int warp_nearest_ref(const GP& p, float ox, float oy, float oz) {
    int q0 = 0, q1 = 0;
    const float fx = (ox - p.g0[0]) * p.inv_cell, fy = (oy - p.g0[1]) * p.inv_cell, fz = (oz - p.g0[2]) * p.inv_cell;
    if (fx >= 0.f && fy >= 0.f && fz >= 0.f && fx < (float)p.dims[0] && fy < (float)p.dims[1] &&
        fz < (float)p.dims[2]) {
        const int c = ((int)fz * p.dims[1] + (int)fy) * p.dims[0] + (int)fx;
        q0 = __float_as_int(__ldg(&p.cell_box[4 * (long long)c].w));
        q1 = __float_as_int(__ldg(&p.cell_box[4 * (long long)c + 3].w));
    }
    const int lane = threadIdx.x & 31;
    float best = __int_as_float(0x7f800000);
    int ref = -1;
    for (int r = q0 + lane; r < q1; r += 32) {
        const float4* t = p.cell_tris + 3 * (long long)r;
        const float4 v0 = __ldg(t), e1 = __ldg(t + 1), e2 = __ldg(t + 2);
        const float cx = v0.x + (e1.x + e2.x) * (1.f / 3.f) - ox;
        const float cy = v0.y + (e1.y + e2.y) * (1.f / 3.f) - oy;
        const float cz = v0.z + (e1.z + e2.z) * (1.f / 3.f) - oz;
        const float fx = e2.x - e1.x, fy = e2.y - e1.y, fz = e2.z - e1.z;
        const float l2 = fmaxf(fmaxf(e1.x * e1.x + e1.y * e1.y + e1.z * e1.z, e2.x * e2.x + e2.y * e2.y + e2.z * e2.z),
                               fx * fx + fy * fy + fz * fz);
        const float d2 = cx * cx + cy * cy + cz * cz;
        if (d2 < l2 && d2 < best * l2) {  // d2 / l2 < best, without a division
            best = d2 / l2;
            ref = r;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float b2 = __shfl_xor_sync(0xffffffffu, best, o);
        const int r2 = __shfl_xor_sync(0xffffffffu, ref, o);
        if (b2 < best || (b2 == best && r2 > ref)) {  // ties: any fixed rule, the same in every lane
            best = b2;
            ref = r2;
        }
    }
    return ref;
}

// Tests the walk's segment against cell-order reference q (any triangle of the
// scene: a hit there blocks the segment just as one found by the walk).
template <bool CULL, class GP>
__device__ __forceinline__ bool walk_test_ref(const GP& p, const Walk& w, int q) {
    const float4* t = p.cell_tris + 3 * (long long)q;
    return hit_full<CULL>(w.r, w.ox, w.oy, w.oz, __ldg(t), __ldg(t + 1), __ldg(t + 2), p.eps);
}

// Enters the grid along the segment set by walk_ray at parameter `from` (a point
// inside the segment that an earlier partial walk stopped at); false if the rest
// of the segment misses the grid box.  The cell of the restart point is walked
// again, so every cell the segment crosses beyond `from` is visited.
template <class GP>
__device__ __forceinline__ bool walk_setup_from(const GP& p, Walk& w, float from) {
    const float ox = w.ox, oy = w.oy, oz = w.oz;
    float t0 = from;
    w.t1 = w.r.len;
    bool miss = false;
#define LYEM_SLAB(D, O, G0, G1, INV)                       \
    if (D == 0.f) {                                        \
        INV = copysignf(0x1p100f, D);                      \
        if (O < G0 || O > G1) miss = true;                 \
    } else {                                               \
        INV = 1.0f / D;                                    \
        float ta = (G0 - O) * INV, tb = (G1 - O) * INV;    \
        t0 = fmaxf(t0, fminf(ta, tb));                     \
        w.t1 = fminf(w.t1, fmaxf(ta, tb));                 \
    }
    LYEM_SLAB(w.r.dx, ox, p.g0[0], p.g1[0], w.ix)
    LYEM_SLAB(w.r.dy, oy, p.g0[1], p.g1[1], w.iy)
    LYEM_SLAB(w.r.dz, oz, p.g0[2], p.g1[2], w.iz)
#undef LYEM_SLAB
    if (miss || !(t0 <= w.t1)) return false;
    w.cx = min(max((int)floorf((ox + t0 * w.r.dx - p.g0[0]) * p.inv_cell), 0), p.dims[0] - 1);
    w.cy = min(max((int)floorf((oy + t0 * w.r.dy - p.g0[1]) * p.inv_cell), 0), p.dims[1] - 1);
    w.cz = min(max((int)floorf((oz + t0 * w.r.dz - p.g0[2]) * p.inv_cell), 0), p.dims[2] - 1);
    w.guard = p.dims[0] + p.dims[1] + p.dims[2] + 2;
    walk_enter(p, w, (w.cz * p.dims[1] + w.cy) * p.dims[0] + w.cx);
    return true;
}

// Parameters of the next crossing of a cell boundary along each axis (the
// boundary ahead of the current cell, recomputed from the cell index; +inf for
// an axis the segment is parallel to).
template <class GP>
__device__ __forceinline__ void next_crossings(const GP& p, const Walk& w, float& tx, float& ty, float& tz) {
    const float kInf = __int_as_float(0x7f800000);
    const float cell = p.cell;
    tx = (p.g0[0] + (float)(w.cx + (w.r.dx > 0.f ? 1 : 0)) * cell - w.ox) * w.ix;
    ty = (p.g0[1] + (float)(w.cy + (w.r.dy > 0.f ? 1 : 0)) * cell - w.oy) * w.iy;
    tz = (p.g0[2] + (float)(w.cz + (w.r.dz > 0.f ? 1 : 0)) * cell - w.oz) * w.iz;
    if (w.r.dx == 0.f) tx = kInf;
    if (w.r.dy == 0.f) ty = kInf;
    if (w.r.dz == 0.f) tz = kInf;
}

// Crosses the nearest cell boundary unless the crossing lies at or beyond
// parameter `stop`: 0 = the segment or the grid ends there, 1 = the next cell
// was entered, 2 = stopped before a crossing at or beyond `stop`.
template <class GP>
__device__ __forceinline__ int walk_step_until(const GP& p, Walk& w, float stop, unsigned int* err) {
    float tx, ty, tz;
    next_crossings(p, w, tx, ty, tz);
    const float tc = fminf(tx, fminf(ty, tz));
    if (tc > w.t1) return 0;
    if (tc >= stop) return 2;
    bool done;
    if (tx <= ty && tx <= tz) {
        w.cx += w.r.dx > 0.f ? 1 : -1;
        done = w.cx < 0 || w.cx >= p.dims[0];
    } else if (ty <= tz) {
        w.cy += w.r.dy > 0.f ? 1 : -1;
        done = w.cy < 0 || w.cy >= p.dims[1];
    } else {
        w.cz += w.r.dz > 0.f ? 1 : -1;
        done = w.cz < 0 || w.cz >= p.dims[2];
    }
    if (--w.guard < 0) {  // a monotone walk visits at most dims[0] + dims[1] + dims[2] cells
        if (err) atomicOr(err, 2u);
        done = true;
    }
    if (done) return 0;
    walk_enter(p, w, (w.cz * p.dims[1] + w.cy) * p.dims[0] + w.cx);
    return 1;
}

// Crosses the nearest cell boundary; false when the segment or the grid ends there.
template <class GP>
__device__ __forceinline__ bool walk_step(const GP& p, Walk& w, unsigned int* err) {
    float tx, ty, tz;
    next_crossings(p, w, tx, ty, tz);
    bool done;
    if (tx <= ty && tx <= tz) {
        w.cx += w.r.dx > 0.f ? 1 : -1;
        done = tx > w.t1 || w.cx < 0 || w.cx >= p.dims[0];
    } else if (ty <= tz) {
        w.cy += w.r.dy > 0.f ? 1 : -1;
        done = ty > w.t1 || w.cy < 0 || w.cy >= p.dims[1];
    } else {
        w.cz += w.r.dz > 0.f ? 1 : -1;
        done = tz > w.t1 || w.cz < 0 || w.cz >= p.dims[2];
    }
    if (--w.guard < 0) {  // a monotone walk visits at most dims[0] + dims[1] + dims[2] cells
        if (err) atomicOr(err, 2u);
        done = true;
    }
    if (done) return false;
    walk_enter(p, w, (w.cz * p.dims[1] + w.cy) * p.dims[0] + w.cx);
    return true;
}

}  // namespace lyem
