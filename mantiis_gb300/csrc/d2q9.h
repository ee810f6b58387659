// D2Q9 lattice constants shared by host and device code.
//
// Direction numbering, opposites and weights are the reference's
// (include/utils.hpp:50-70, include/coreLB.hpp:83):
//   c_q = (0,0),(1,0),(0,1),(-1,0),(0,-1),(1,1),(-1,1),(-1,-1),(1,-1)
//   opp = 0,3,4,1,2,7,8,5,6 ; w = 4/9, 1/9 x4, 1/36 x4
// They are a fixed convention of the D2Q9 model and of the boundary tables,
// so they must match the reference exactly.
#pragma once

#if defined(__CUDACC__)
#define MGPU_HD __host__ __device__ __forceinline__
#define MGPU_CONST __constant__
#else
#define MGPU_HD inline
#define MGPU_CONST
#endif

namespace d2q9
{
constexpr int Q = 9;
constexpr int CX[Q] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr int CY[Q] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
constexpr int OPP[Q] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
constexpr double W[Q] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                         1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
// Shan-Chen interaction weights (include/globalParameters.hpp:122)
constexpr double WF[Q] = {0.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0,
                          1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0};

// the same numbers as functions, usable in device code (folded to constants
// when q is a compile-time index)
MGPU_HD constexpr int cx(int q) { return (q == 1 || q == 5 || q == 8) ? 1 : ((q == 3 || q == 6 || q == 7) ? -1 : 0); }
MGPU_HD constexpr int cy(int q) { return (q == 2 || q == 5 || q == 6) ? 1 : ((q == 4 || q == 7 || q == 8) ? -1 : 0); }
MGPU_HD constexpr int opp(int q) { return q == 0 ? 0 : (q < 5 ? (q + 1) % 4 + 1 : (q - 3) % 4 + 5); }
MGPU_HD constexpr double w(int q) { return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0); }
MGPU_HD constexpr double wf(int q) { return q == 0 ? 0.0 : (q < 5 ? 1.0 / 3.0 : 1.0 / 12.0); }
} // namespace d2q9
