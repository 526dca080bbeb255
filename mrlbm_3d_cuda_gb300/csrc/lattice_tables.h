// D3Q27 velocity set, shared by host and device code.
//
// The direction ORDER is a format shared with the reference
// (MRLBM_3D/src/core/D3Q27/latticeProperties.cuh:12-21): 27-bit direction masks, the
// BCFLUID octant tags and the population halo faces all index directions by it, so it is
// kept identical.  q = 0 rest; 1-6 faces; 7-18 edges; 19-26 corners.
#pragma once

#if defined(__CUDACC__)
#define MRLBM_HD __host__ __device__
#else
#define MRLBM_HD
#endif

namespace mrlbm {

constexpr int kQ = 27;
constexpr int kCx[kQ] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
constexpr int kCy[kQ] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
constexpr int kCz[kQ] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
constexpr int kOpp[kQ] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25};

// Device-usable accessors: the tables packed 2 bits per direction into 64-bit constants
// (constexpr arrays cannot be indexed by a runtime value in device code).
constexpr unsigned long long pack2(const int (&c)[kQ]) {
    unsigned long long v = 0;
    for (int q = 0; q < kQ; ++q) v |= (unsigned long long)(c[q] + 1) << (2 * q);
    return v;
}
constexpr unsigned long long kCxBits = pack2(kCx);
constexpr unsigned long long kCyBits = pack2(kCy);
constexpr unsigned long long kCzBits = pack2(kCz);
MRLBM_HD constexpr int cxq(int q) { return (int)((kCxBits >> (2 * q)) & 3ull) - 1; }
MRLBM_HD constexpr int cyq(int q) { return (int)((kCyBits >> (2 * q)) & 3ull) - 1; }
MRLBM_HD constexpr int czq(int q) { return (int)((kCzBits >> (2 * q)) & 3ull) - 1; }
MRLBM_HD constexpr int oppq(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }

// Weights 8/27, 2/27, 1/54, 1/216 by |c|^2 = 0, 1, 2, 3 (rounded to float like `real`).
constexpr float kW0 = (float)(8.0 / 27.0);
constexpr float kW1 = (float)(2.0 / 27.0);
constexpr float kW2 = (float)(1.0 / 54.0);
constexpr float kW3 = (float)(1.0 / 216.0);
constexpr float kCs2 = (float)(1.0 / 3.0);

MRLBM_HD constexpr float weight(int q) {
    return q == 0 ? kW0 : (q <= 6 ? kW1 : (q <= 18 ? kW2 : kW3));
}

}  // namespace mrlbm
