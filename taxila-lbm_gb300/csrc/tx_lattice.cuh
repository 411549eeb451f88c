// Lattice constants of D2Q9 and D3Q19 as compile-time functions.
//
// Direction order, velocities, weights, the MRT transform M^T and diag(M M^T)
// are those of DiscretizationSetup_D3Q19 (src/lbm/lbm_discretization_d3q19.F90:
// 64-232) and DiscretizationSetUp_D2Q9 (src/lbm/lbm_discretization_d2q9.F90:
// 53-144); the order has to be the reference's because populations cross the
// C ABI in the reference's layout and the MRT moment order fixes rounding.
// Everything here is constexpr so that kernels unrolled with sfor<> fold
// zero and unit MRT coefficients away at compile time.
#pragma once
#include <type_traits>

namespace tx {

template <int B, int E, class F>
__host__ __device__ __forceinline__ void sfor(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    sfor<B + 1, E>(f);
  }
}

template <int D>
struct Lat;

template <>
struct Lat<3> {
  static constexpr int ND = 3;
  static constexpr int Q = 19;
  static constexpr int NAXIS = 6;  // directions 1..6 are the axis links
  __host__ __device__ static constexpr int c(int n, int d) {
    const int cx[19] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0};
    const int cy[19] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1};
    const int cz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    return d == 0 ? cx[n] : (d == 1 ? cy[n] : cz[n]);
  }
  __host__ __device__ static constexpr double w(int n) {
    return n == 0 ? 1.0 / 3.0 : (n <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
  }
  // mt(i, k) = M^T(i, k): value of moment k's basis vector at direction i
  __host__ __device__ static constexpr int mt(int i, int k) {
    const signed char m[19][19] = {
        {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
        {-30, -11, -11, -11, -11, -11, -11, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8},
        {12, -4, -4, -4, -4, -4, -4, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
        {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0},
        {0, -4, 0, 4, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0},
        {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1},
        {0, 0, -4, 0, 4, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1},
        {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
        {0, 0, 0, 0, 0, -4, 4, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
        {0, 2, -1, 2, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
        {0, -4, 2, -4, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
        {0, 0, 1, 0, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
        {0, 0, -2, 0, -2, 2, 2, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, -1, -1, 1, 1, 0, 0, 0, 0, 1, -1, -1, 1},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, -1, -1, 1, 1}};
    return m[k][i];
  }
  __host__ __device__ static constexpr int mmt(int k) {
    const int v[19] = {19, 2394, 252, 10, 40, 10, 40, 10, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8};
    return v[k];
  }
};

template <>
struct Lat<2> {
  static constexpr int ND = 2;
  static constexpr int Q = 9;
  static constexpr int NAXIS = 4;
  __host__ __device__ static constexpr int c(int n, int d) {
    const int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    const int cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    return d == 0 ? cx[n] : (d == 1 ? cy[n] : 0);
  }
  __host__ __device__ static constexpr double w(int n) {
    return n == 0 ? 4.0 / 9.0 : (n <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
  }
  __host__ __device__ static constexpr int mt(int i, int k) {
    const signed char m[9][9] = {{1, 1, 1, 1, 1, 1, 1, 1, 1},   {-4, -1, -1, -1, -1, 2, 2, 2, 2},
                                 {4, -2, -2, -2, -2, 1, 1, 1, 1}, {0, 1, 0, -1, 0, 1, -1, -1, 1},
                                 {0, -2, 0, 2, 0, 1, -1, -1, 1},  {0, 0, 1, 0, -1, 1, 1, -1, -1},
                                 {0, 0, -2, 0, 2, 1, 1, -1, -1},  {0, 1, -1, 1, -1, 0, 0, 0, 0},
                                 {0, 0, 0, 0, 0, 1, -1, 1, -1}};
    return m[k][i];
  }
  __host__ __device__ static constexpr int mmt(int k) {
    const int v[9] = {9, 36, 36, 6, 12, 6, 12, 4, 4};
    return v[k];
  }
};

// the direction with all velocity components negated (disc%opposites)
template <int D>
__host__ __device__ constexpr int opp(int n) {
  int r = 0;
  for (int m = 0; m < Lat<D>::Q; ++m) {
    bool ok = true;
    for (int d = 0; d < D; ++d) ok = ok && (Lat<D>::c(m, d) == -Lat<D>::c(n, d));
    if (ok) r = m;
  }
  return r;
}

// MRT rate index map of DiscretizationSetupRelax_D3Q19 (:234-263) / _D2Q9
// (:147-166): which of s_c, s_e, s_e2, s_q, s_nu, s_pi, s_m relaxes moment k
enum { R_C = 0, R_E, R_E2, R_Q, R_NU, R_PI, R_M };
template <int D>
__host__ __device__ constexpr int rate_of(int k) {
  if (D == 3) {
    const int r[19] = {R_C, R_E, R_E2, R_C, R_Q, R_C, R_Q, R_C, R_Q, R_NU,
                       R_PI, R_NU, R_PI, R_NU, R_NU, R_NU, R_M, R_M, R_M};
    return r[k];
  } else {
    const int r[9] = {R_C, R_E, R_E2, R_C, R_Q, R_C, R_Q, R_NU, R_NU};
    return r[k];
  }
}

// Direction pairs (n, opp(n)) with n < opp(n), in increasing n: pair p's n.
template <int D>
__host__ __device__ constexpr int npairs() {
  return (Lat<D>::Q - 1) / 2;
}
template <int D>
__host__ __device__ constexpr int pair_n(int p) {
  int k = 0;
  for (int n = 1; n < Lat<D>::Q; ++n)
    if (n < opp<D>(n)) {
      if (k == p) return n;
      ++k;
    }
  return -1;
}

// Parity of MRT moment k under c -> -c: even (mt(n,k) = mt(opp(n),k)) or odd
// (mt(n,k) = -mt(opp(n),k), zero at rest).  Every moment of both bases is one
// or the other.
template <int D>
__host__ __device__ constexpr bool moment_even(int k) {
  for (int n = 1; n < Lat<D>::Q; ++n)
    if (Lat<D>::mt(n, k) != Lat<D>::mt(opp<D>(n), k)) return false;
  return true;
}
template <int D>
__host__ __device__ constexpr bool moment_odd(int k) {
  if (Lat<D>::mt(0, k) != 0) return false;
  for (int n = 1; n < Lat<D>::Q; ++n)
    if (Lat<D>::mt(n, k) != -Lat<D>::mt(opp<D>(n), k)) return false;
  return true;
}

// The moments relaxed at s_nu (the traceless second moments): even, zero at rest.
template <int D>
__host__ __device__ constexpr unsigned stress_mask() {
  unsigned b = 0u;
  for (int k = 0; k < Lat<D>::Q; ++k)
    if (rate_of<D>(k) == R_NU) b |= 1u << k;
  return b;
}
template <int D>
__host__ __device__ constexpr bool stress_even_traceless() {
  for (int k = 0; k < Lat<D>::Q; ++k)
    if (rate_of<D>(k) == R_NU && (!moment_even<D>(k) || Lat<D>::mt(0, k) != 0)) return false;
  return true;
}
template <int D>
__host__ __device__ constexpr bool moments_have_parity() {
  for (int k = 0; k < Lat<D>::Q; ++k)
    if (!moment_even<D>(k) && !moment_odd<D>(k)) return false;
  return true;
}
static_assert(stress_even_traceless<3>() && stress_even_traceless<2>(), "s_nu moments must be even and traceless");

// 9 w_n for the direction classes, exactly (axis, diagonal): 1/2, 1/4 in D3Q19;
// 1, 1/4 in D2Q9.
template <int D>
__host__ __device__ constexpr double nine_w(int n) {
  return n <= Lat<D>::NAXIS ? (D == 3 ? 0.5 : 1.0) : 0.25;
}

// Bilinear form of an s_nu moment over direction pairs: the moment k of the
// pair values 9 w_n (c_n.a)(c_n.b) is sum_de stress_coef(k, d, e) a_d b_e,
// stress_coef(k, d, e) = sum over pairs of mt(n, k) 9 w_n c_n,d c_n,e.
template <int D>
__host__ __device__ constexpr double stress_coef(int k, int d, int e) {
  double acc = 0.0;
  for (int p = 0; p < npairs<D>(); ++p) {
    const int n = pair_n<D>(p);
    acc += Lat<D>::mt(n, k) * nine_w<D>(n) * Lat<D>::c(n, d) * Lat<D>::c(n, e);
  }
  return acc;
}

// The s_nu moments see no constant per direction class: over the axis pairs
// and over the diagonal pairs the coefficients mt(n, k) sum to zero.
template <int D>
__host__ __device__ constexpr bool stress_class_free() {
  for (int k = 0; k < Lat<D>::Q; ++k) {
    if (rate_of<D>(k) != R_NU) continue;
    int axis = 0, diag = 0;
    for (int p = 0; p < npairs<D>(); ++p) {
      const int n = pair_n<D>(p);
      if (n <= Lat<D>::NAXIS)
        axis += Lat<D>::mt(n, k);
      else
        diag += Lat<D>::mt(n, k);
    }
    if (axis != 0 || diag != 0) return false;
  }
  return true;
}
static_assert(stress_class_free<3>() && stress_class_free<2>(), "s_nu moments must vanish on class constants");

// The direction with velocity (x, y, z), -1 if none.
template <int D>
__host__ __device__ constexpr int dir_of(int x, int y, int z) {
  for (int n = 0; n < Lat<D>::Q; ++n)
    if (Lat<D>::c(n, 0) == x && Lat<D>::c(n, 1) == y && (D == 3 ? Lat<D>::c(n, 2) : 0) == z) return n;
  return -1;
}
template <int D>
__host__ __device__ constexpr int axis_dir(int d) {
  return dir_of<D>(d == 0 ? 1 : 0, d == 1 ? 1 : 0, d == 2 ? 1 : 0);
}
// The direction e_a + s e_b (a != b, s = +-1).
template <int D>
__host__ __device__ constexpr int diag_dir(int a, int b, int s) {
  int v[3] = {0, 0, 0};
  v[a] = 1;
  v[b] = s;
  return dir_of<D>(v[0], v[1], v[2]);
}

// An s_nu moment k is a quadratic form of the velocity: mt(n, k) =
// sum_de stress_b(k, d, e) c_n,d c_n,e, with the diagonal from the axis
// directions and the off-diagonal from the diagonal directions.
template <int D>
__host__ __device__ constexpr double stress_b(int k, int d, int e) {
  if (d == e) return Lat<D>::mt(axis_dir<D>(d), k);
  return 0.5 * (Lat<D>::mt(diag_dir<D>(d, e, 1), k) - Lat<D>::mt(axis_dir<D>(d), k) - Lat<D>::mt(axis_dir<D>(e), k));
}
template <int D>
__host__ __device__ constexpr bool stress_quadratic() {
  for (int k = 0; k < Lat<D>::Q; ++k) {
    if (rate_of<D>(k) != R_NU) continue;
    for (int n = 0; n < Lat<D>::Q; ++n) {
      double q = 0.0;
      for (int d = 0; d < D; ++d)
        for (int e = 0; e < D; ++e) q += stress_b<D>(k, d, e) * Lat<D>::c(n, d) * Lat<D>::c(n, e);
      if (q != Lat<D>::mt(n, k)) return false;
    }
  }
  return true;
}
static_assert(stress_quadratic<3>() && stress_quadratic<2>(), "s_nu moments must be quadratic forms of c");

}  // namespace tx
