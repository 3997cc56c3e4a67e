// Compile-time lattice tables for D2Q9, D3Q19, D3Q27, D3Q15, D2Q13 and D3Q33.
//
// The velocity order must be the reference's, because a population's index is
// part of the storage layout the drop-in boundary exchanges with metaLBM
// (Lattice.h:146-210, 214-288, 461-533, 536-612, 615-703, 707-802): index 0 is
// the rest population, then the populations with c_x < 0, those with
// c_x > 0, then c_x = 0, each group in the reference's order. Weights are the
// reference's expressions ((T)a / (T)b, or the decimal literals of D3Q33),
// evaluated in double at compile time exactly as the reference does.
//
// R is the lattice's reach (the largest |c_d|: the reference's halo width)
// and ics its 1/c_s^2 (inv_cs2): 3 for every lattice but D3Q33, whose
// c_s^2 = 0.4156023517935171 makes ics the rounded quotient (T)1 / cs2.
//
// Everything is a constexpr function of compile-time indices: inside the
// fully unrolled population loops of the kernels the values fold into
// immediates, so the tables cost no memory traffic at all.
#pragma once

namespace mlbm {

enum : int { LAT_D2Q9 = 0, LAT_D3Q19 = 1, LAT_D3Q27 = 2, LAT_D3Q15 = 3, LAT_D2Q13 = 4, LAT_D3Q33 = 5 };

// the most populations of any lattice (D3Q33)
constexpr int kMaxQ = 33;

template <int LAT>
struct Lattice;

template <>
struct Lattice<LAT_D2Q9> {
  static constexpr int D = 2, Q = 9, faceQ = 3, R = 1;
  static constexpr double ics = 3.0;
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
  static constexpr int D = 3, Q = 19, faceQ = 5, R = 1;
  static constexpr double ics = 3.0;
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
  static constexpr int D = 3, Q = 27, faceQ = 9, R = 1;
  static constexpr double ics = 3.0;
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

template <>
struct Lattice<LAT_D3Q15> {
  static constexpr int D = 3, Q = 15, faceQ = 5, R = 1;
  static constexpr double ics = 3.0;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[15][3] = {{0, 0, 0},   {-1, 0, 0}, {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1},
                              {-1, 1, 1},  {1, 0, 0},  {1, 1, 1},    {1, 1, -1},  {1, -1, 1},
                              {1, -1, -1}, {0, -1, 0}, {0, 0, -1},   {0, 1, 0},   {0, 0, 1}};
    return t[q][d];
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 2.0 / 9.0
           : (q == 1 || q == 6 || q >= 11) ? 1.0 / 9.0
                                           : 1.0 / 72.0;
  }
};

template <>
struct Lattice<LAT_D2Q13> {
  static constexpr int D = 2, Q = 13, faceQ = 4, R = 2;
  static constexpr double ics = 3.0;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[13][3] = {{0, 0, 0},  {-1, 0, 0}, {-1, -1, 0}, {-1, 1, 0}, {-2, 0, 0},
                              {1, 0, 0},  {1, -1, 0}, {1, 1, 0},   {2, 0, 0},  {0, -1, 0},
                              {0, 1, 0},  {0, -2, 0}, {0, 2, 0}};
    return t[q][d];
  }
  __host__ __device__ static constexpr double w(int q) {
    return q == 0 ? 1.0 / 2.0
           : (q == 1 || q == 5 || q == 9 || q == 10) ? 4.0 / 45.0
           : (q == 4 || q == 8 || q == 11 || q == 12) ? 1.0 / 360.0
                                                     : 1.0 / 30.0;
  }
};

template <>
struct Lattice<LAT_D3Q33> {
  static constexpr int D = 3, Q = 33, faceQ = 10, R = 2;
  static constexpr double ics = 1.0 / 0.4156023517935171;
  __host__ __device__ static constexpr int c(int q, int d) {
    constexpr int t[33][3] = {
        {0, 0, 0},   {-1, 0, 0},  {-1, -1, 0},  {-1, 1, 0},  {-1, 0, -1}, {-1, 0, 1},  {-1, -1, -1},
        {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},   {-2, 0, 0},  {1, 0, 0},   {1, 1, 0},   {1, -1, 0},
        {1, 0, 1},   {1, 0, -1},  {1, 1, 1},    {1, 1, -1},  {1, -1, 1},  {1, -1, -1}, {2, 0, 0},
        {0, -1, 0},  {0, 0, -1},  {0, -1, -1},  {0, -1, 1},  {0, 1, 0},   {0, 0, 1},   {0, 1, 1},
        {0, 1, -1},  {0, 2, 0},   {0, -2, 0},   {0, 0, 2},   {0, 0, -2}};
    return t[q][d];
  }
  // classes 0..4 of the weights w0..w4 in population order
  __host__ __device__ static constexpr double w(int q) {
    constexpr int cls[33] = {0, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 1, 2, 2, 2, 2, 3,
                             3, 3, 3, 4, 1, 1, 2, 2, 1, 1, 2, 2, 4, 4, 4, 4};
    constexpr double v[5] = {0.177627658370520295649084, 0.103315974899246818673111,
                             0.000513472406731114352456, 0.021333928148672240120078,
                             0.004273899693974583187026};
    return v[cls[q]];
  }
};

// Constants of Equilibrium<TruncationMa3> (Equilibrium.h:14-33) formed as the
// reference forms them: Power<T, n>::Do(inv_cs2) is the left-folded product
// (Helpers.h:93-113) and 0.5 * Power<T, 2> its first factor.
template <int LAT>
struct EqConst {
  static constexpr double ics = Lattice<LAT>::ics;
  static constexpr double p2 = ics * ics;
  static constexpr double p3 = ics * ics * ics;
  static constexpr double p4 = ics * ics * ics * ics;
  static constexpr double half_p2 = 0.5 * p2;
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
