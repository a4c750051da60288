// Linear index -> (i, j, k) inside a staged tile region without integer
// division instructions.
//
// The tile kernels walk their regions (staged padded region, derivative
// boxes, interior points) with a flat index q split by the region's runtime
// extents.  A runtime `q / n` compiles to a reciprocal estimate plus
// corrections, about 20 instructions; the tiles split one such index per
// point for each of the 24 fields.  With m = ceil(2^31 / n), fixed once per
// tile, floor(q / n) = floor(2q * m / 2^32): one shift and one high multiply.
// Exact for q * n < 2^31 (the rounding-up of m adds at most q / 2^31 to
// q / n, below the 1/n gap to the next integer); regions here are under
// 2^13 points with extents under 32.
#pragma once
#include <stdint.h>

namespace dgb {

struct DivBy {
    int n;
    uint32_t m;
    __device__ __forceinline__ explicit DivBy(int n_)
        : n(n_), m((0x80000000u + (uint32_t)n_ - 1u) / (uint32_t)n_) {}
    __device__ __forceinline__ int div(int q) const { return (int)__umulhi((uint32_t)q << 1, m); }
};

// q = i + a.n * (j + b.n * k)
__device__ __forceinline__ void split3(int q, const DivBy &a, const DivBy &b, int &i, int &j, int &k)
{
    const int r = a.div(q);
    i = q - r * a.n;
    k = b.div(r);
    j = r - k * b.n;
}

}  // namespace dgb
