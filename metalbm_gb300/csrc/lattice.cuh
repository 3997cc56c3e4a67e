// Compile-time lattice tables for D2Q9, D3Q19 and D3Q27.
//
// The velocity order must be the reference's, because a population's index is
// part of the storage layout the drop-in boundary exchanges with metaLBM
// (Lattice.h:189-199, 579-598, 658-687): index 0 is the rest population, then
// the faceQ populations with c_x = -1, the faceQ with c_x = +1, then c_x = 0.
// Weights are the reference's ratios (Lattice.h:203-205, 602-607, 691-698),
// evaluated in double at compile time exactly as (T)a / (T)b.
//
// Everything is a constexpr function of compile-time indices: inside the
// fully unrolled population loops of the kernels the values fold into
// immediates, so the tables cost no memory traffic at all.
#pragma once

namespace mlbm {

enum : int { LAT_D2Q9 = 0, LAT_D3Q19 = 1, LAT_D3Q27 = 2 };

template <int LAT>
struct Lattice;

template <>
struct Lattice<LAT_D2Q9> {
  static constexpr int D = 2, Q = 9, faceQ = 3;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[9][3] = {{0, 0, 0}, {-1, 1, 0}, {-1, 0, 0}, {-1, -1, 0}, {1, -1, 0},
                             {1, 0, 0}, {1, 1, 0},  {0, -1, 0}, {0, 1, 0}};
    return t[q][d];
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 4.0 / 9.0 : ((q == 2 || q == 5 || q == 7 || q == 8) ? 1.0 / 9.0 : 1.0 / 36.0);
  }
};

template <>
struct Lattice<LAT_D3Q19> {
  static constexpr int D = 3, Q = 19, faceQ = 5;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[19][3] = {{0, 0, 0},   {-1, 0, 0}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1},
                              {-1, 0, 1},  {1, 0, 0},  {1, 1, 0},   {1, -1, 0}, {1, 0, 1},
                              {1, 0, -1},  {0, -1, 0}, {0, 0, -1},  {0, -1, -1}, {0, -1, 1},
                              {0, 1, 0},   {0, 0, 1},  {0, 1, 1},   {0, 1, -1}};
    return t[q][d];
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 1.0 / 3.0
                  : ((q == 1 || q == 6 || q == 11 || q == 12 || q == 15 || q == 16) ? 1.0 / 18.0
                                                                                     : 1.0 / 36.0);
  }
};

template <>
struct Lattice<LAT_D3Q27> {
  static constexpr int D = 3, Q = 27, faceQ = 9;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[27][3] = {
        {0, 0, 0},   {-1, 0, 0},  {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1},  {-1, -1, -1},
        {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},  {1, 0, 0},  {1, 1, 0},   {1, -1, 0},  {1, 0, 1},
        {1, 0, -1},  {1, 1, 1},   {1, 1, -1},  {1, -1, 1}, {1, -1, -1}, {0, -1, 0},  {0, 0, -1},
        {0, -1, -1}, {0, -1, 1},  {0, 1, 0},   {0, 0, 1},  {0, 1, 1},   {0, 1, -1}};
    return t[q][d];
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 8.0 / 27.0
           : (q == 1 || q == 10 || q == 19 || q == 20 || q == 23 || q == 24) ? 2.0 / 27.0
           : (q >= 6 && q <= 9) || (q >= 15 && q <= 18) ? 1.0 / 216.0
                                                        : 1.0 / 54.0;
  }
};

// Index of the population with velocity -c_q.
template <int LAT>
__host__ __device__ constexpr int opposite(int q) {
  using L = Lattice<LAT>;
  for (int p = 0; p < L::Q; ++p)
    if (L::c(p, 0) == -L::c(q, 0) && L::c(p, 1) == -L::c(q, 1) && L::c(p, 2) == -L::c(q, 2))
      return p;
  return -1;
}

// Populations are processed as (q, opposite(q)) pairs: q runs over the rest
// population and the faceQ populations with c_x = -1, plus, for the c_x = 0
// block, the members whose first nonzero component is negative.
template <int LAT>
__host__ __device__ constexpr bool is_pair_leader(int q) {
  using L = Lattice<LAT>;
  if (q == 0) return false;
  for (int d = 0; d < 3; ++d) {
    if (L::c(q, d) < 0) return true;
    if (L::c(q, d) > 0) return false;
  }
  return false;
}

}  // namespace mlbm
