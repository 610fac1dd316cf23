// Host check of the culling test's decisions after the determinant
// (lyem_device.cuh): the guard bands on u and v followed by cull_tail, which
// decides without the reciprocal where the outcome is certain, must give the
// reference's decision (cull_tail_exact: F = rn(1/A), U, V, t rounded as in
// lyceanem/src/raycasting.cuh:44-66) on every input.  Test infrastructure:
// compiled for the host by tests/test_cull_decisions.py with
// -ffp-contract=off, so every host operation is one IEEE binary32 rounding.
//
//   cull_decisions <n_cases> <seed>   prints "cases mismatches fast_fraction"
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "lyem_device.cuh"

namespace {

uint64_t g_state = 0x9e3779b97f4a7c15ull;
uint64_t next_u64() {  // splitmix64
    uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
double uni() { return (double)(next_u64() >> 11) * 0x1p-53; }
int pick(int n) { return (int)(next_u64() % (uint64_t)n); }

// a value near x: x itself, a few ulps away, or a relative offset of 2^-k
float near(float x) {
    switch (pick(4)) {
        case 0:
            return x;
        case 1: {
            float y = x;
            const int steps = pick(9) - 4;
            for (int i = 0; i < (steps < 0 ? -steps : steps); ++i)
                y = std::nextafter(y, steps < 0 ? -INFINITY : INFINITY);
            return y;
        }
        case 2:
            return (float)((double)x * (1.0 + std::ldexp(uni() - 0.5, -(14 + pick(14)))));
        default:
            return (float)((double)x * (1.0 + 0.1 * (uni() - 0.5)));
    }
}

// a ratio in the test's natural range, concentrated at the decision boundaries
double ratio(double edge_hi) {
    switch (pick(6)) {
        case 0: return uni() * edge_hi;
        case 1: return edge_hi * (1.0 + std::ldexp(uni() - 0.5, -(16 + pick(12))));
        case 2: return std::ldexp(uni() - 0.5, -(16 + pick(14)));
        case 3: return -uni();
        case 4: return edge_hi * (1.0 + uni());
        default: return uni() * 2.0 - 0.5;
    }
}

}  // namespace

int main(int argc, char** argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    g_state ^= argc > 2 ? (uint64_t)atoll(argv[2]) : 1ull;
    long long mismatches = 0, fast = 0;
    for (long long i = 0; i < n; ++i) {
        const int ek = pick(8);
        const float eps = ek == 0 ? (float)std::ldexp(uni() + 0.5, -(10 + pick(40))) : ek == 1 ? 0.f
                                                                                     : (pick(2) ? 1e-6f : 1e-7f);
        // determinant: at or just above eps, or any exponent; with eps = 0 also zero, -0 and subnormal
        float A = pick(4) == 0 ? near(eps) : (float)std::ldexp(uni() + 0.5, pick(120) - 60);
        if (eps == 0.f && pick(4) == 0) {
            const int z = pick(3);
            A = z == 0 ? 0.f : z == 1 ? -0.f : (float)std::ldexp(uni() + 0.5, -(127 + pick(22)));
        }
        if (!(A >= eps)) A = eps;
        const float len = pick(5) == 0 ? near(2.f * eps) : (float)std::ldexp(uni() + 0.5, pick(40) - 20);
        const double ru = ratio(1.0);
        const double rv = pick(2) ? ratio(1.0) : (1.0 - ru) * (1.0 + std::ldexp(uni() - 0.5, -(16 + pick(12))));
        const float u = near((float)(ru * A)), v = near((float)(rv * A));
        const double L = (double)len - 2.0 * eps;
        double rt;
        switch (pick(5)) {
            case 0: rt = 2.0 * eps; break;
            case 1: rt = L; break;
            case 2: rt = 4.0 * eps; break;
            case 3: rt = -uni() * L; break;
            default: rt = uni() * L * 1.2;
        }
        const float w = near((float)(rt * A));
        // the kernel's sequence: guard bands on u and v, then cull_tail
        const float aneg = A * -0x1p-20f, ahi = std::fmaf(A, 0x1p-19f, A);
        bool ours;
        if (u < aneg || u > ahi || v < aneg || v > ahi) {
            ours = false;
        } else {
            ours = lyem::cull_tail(A, u, v, w, len, eps, ahi);
            const float Lr = len - 2.f * eps;
            fast += (A >= 0x1p-90f && A <= 0x1p90f && Lr >= 0x1p-20f && Lr <= 0x1p30f) ? 1 : 0;
        }
        const bool ref = lyem::cull_tail_exact(A, u, v, w, len, eps);
        if (ours != ref) {
            if (mismatches < 10)
                std::printf("mismatch A=%a u=%a v=%a w=%a len=%a eps=%a ours=%d ref=%d\n", A, u, v, w, len, eps, ours,
                            ref);
            ++mismatches;
        }
    }
    std::printf("%lld %lld %.4f\n", n, mismatches, (double)fast / (double)n);
    return mismatches ? 1 : 0;
}
