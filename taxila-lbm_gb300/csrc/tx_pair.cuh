// Paired-site step kernels of the FP32-arithmetic forms (FP32 or FP16
// population storage).
//
// One thread updates two consecutive cells in storage order (c0 even, c0 + 1)
// of a lattice with an even site count: usually x-neighbours of one row, at
// odd nx one pair in two rows spans a row end.  Every per-site quantity of the collision is a V2, the value at
// both sites, and every V2 operation is one packed FP32x2 instruction of
// sm_100+ (FADD2 / FMUL2 / FFMA2), so the collision costs half the FP32
// instructions per site.  The two sites' populations of one direction are
// adjacent in memory: they load with one 8-byte (FP32) or 4-byte (FP16) load,
// and the rest population and the pushes along y and z store with one.  Site
// indices, neighbourhoods and stream offsets are formed once per pair.
//
// k_step_pair takes the pairs whose pore sites are all "simple": not on a
// Dirichlet-class face and, when the fluid-fluid force is on, with every
// gradient-stencil neighbour pore (the bulk gradient).  k_step_rest runs the
// per-site step (step_site) on the pore sites of every other pair.  Each pore
// slot of the next state has exactly one writer, so the two launches are
// independent.  The per-site arithmetic is the fast form of step_site, in the
// same expression shapes; only the FMA contractions differ.
#pragma once
#include "tx_kernels.cuh"

// Resident 128-thread blocks per SM that ptxas must make room for in
// k_step_pair (168 registers): each thread carries two sites, so three
// blocks keep more sites in flight than four of step_site.  For two
// components this spills a little; measured on GB300 at 128^3 it is faster
// than two blocks without spills (FP16 storage: 0.128 against 0.153 ms).
#ifndef TX_PAIR_MIN_BLOCKS_S1
#define TX_PAIR_MIN_BLOCKS_S1 3
#endif
#ifndef TX_PAIR_MIN_BLOCKS_S2
#define TX_PAIR_MIN_BLOCKS_S2 3
#endif
#define TX_PAIR_MIN_BLOCKS(S) ((S) == 1 ? TX_PAIR_MIN_BLOCKS_S1 : TX_PAIR_MIN_BLOCKS_S2)

namespace tx {

// c_n . v over the nonzero components of c_n (no zero start: the first term seeds)
template <int D, int n>
__device__ __forceinline__ V2 cdot2(const V2 v[D]) {
  V2 acc{0.f, 0.f};
  bool first = true;
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    constexpr int c = Lat<D>::c(n, d);
    if constexpr (c != 0) {
      if (first)
        acc = c > 0 ? v[d] : -v[d];
      else
        acc = c > 0 ? acc + v[d] : acc - v[d];
      first = false;
    }
  });
  return acc;
}

// ---------------------------------------------------------- storage pairs
// Whether k_step_pair prefetches the pair's population lines into L1 before
// computing the forces.
#ifndef TX_PAIR_PREFETCH
#define TX_PAIR_PREFETCH 1
#endif
// Pairs per thread of k_step_pair (its grid covers the pairs this many times
// over).  One is fastest on GB300: at 128^3 two pairs per thread with the next
// pair's lines prefetched took 0.140 ms (FP16 storage) and 0.157 ms (FP32)
// against 0.129 and 0.141 ms, and four pairs 0.149 and 0.172 ms.
#ifndef TX_PAIR_PER_THREAD
#define TX_PAIR_PER_THREAD 1
#endif
__device__ __forceinline__ void prefetch_l1(const void* p) {
#if defined(__CUDA_ARCH__)
  asm volatile("prefetch.L1 [%0];" ::"l"(p));
#else
  (void)p;
#endif
}

// Two floats to FP16, rounded toward zero, a in the low half (one cvt.rz.f16x2.f32).
__device__ __forceinline__ uint32_t pack_half2_rz(float a, float b) {
#if defined(__CUDA_ARCH__)
  uint32_t u;
  asm("cvt.rz.f16x2.f32 %0, %1, %2;" : "=r"(u) : "f"(b), "f"(a));
  return u;
#else
  const __half ha = __float2half_rz(a), hb = __float2half_rz(b);
  uint16_t la, lb;
  memcpy(&la, &ha, 2);
  memcpy(&lb, &hb, 2);
  return (uint32_t)la | ((uint32_t)lb << 16);
#endif
}

// Population deviations of the two sites at p (p at an even cell of one stream).
template <class T>
__device__ __forceinline__ V2 ld_pair(const T* p, Scl<float> sc) {
  if constexpr (std::is_same<T, __half>::value) {
    const __half2 h = __ldg(reinterpret_cast<const __half2*>(p));
    const float2 f = __half22float2(h);
    return V2{f.x, f.y} * v2(sc.inv);
  } else {
    const float2 f = __ldg(reinterpret_cast<const float2*>(p));
    return V2{f.x, f.y};
  }
}

// The stored values of the two sites at p as floats, the FP16 storage scale
// not divided out (sums of them are scaled once).
template <class T>
__device__ __forceinline__ V2 ld_pair_raw(const T* p) {
  if constexpr (std::is_same<T, __half>::value) {
    const float2 f = __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
    return V2{f.x, f.y};
  } else {
    const float2 f = __ldg(reinterpret_cast<const float2*>(p));
    return V2{f.x, f.y};
  }
}

// Both sites' values to the adjacent slots at p (FP16: stochastic rounding
// with the per-site dithers d0, d1, exactly as st_dev_sr rounds each).
template <class T>
__device__ __forceinline__ void st_pair(T* p, V2 v, Scl<float> sc, uint32_t d0, uint32_t d1) {
  if constexpr (std::is_same<T, __half>::value) {
    const V2 s = v * v2(sc.s);
    const float a = __uint_as_float(__float_as_uint(s.x) + d0);
    const float b = __uint_as_float(__float_as_uint(s.y) + d1);
    *reinterpret_cast<uint32_t*>(p) = pack_half2_rz(a, b);
  } else {
    *reinterpret_cast<float2*>(p) = make_float2(v.x, v.y);
  }
}

// One site's value (lane k of v) at p.
template <class T>
__device__ __forceinline__ void st_one(T* p, float v, Scl<float> sc, uint32_t d) {
  st_dev_sr_s<T, float>(p, v, sc, d);
}

// Both sites' values to two separate slots (a push along x): one scale
// multiply and one FP16 pack for the two, each half stored where it goes;
// w0 / w1 say whether each is stored.
template <class T>
__device__ __forceinline__ void st_two(T* p0, T* p1, V2 v, Scl<float> sc, uint32_t d0, uint32_t d1, bool w0 = true,
                                       bool w1 = true) {
  if constexpr (std::is_same<T, __half>::value) {
    const V2 s = v * v2(sc.s);
    const uint32_t u = pack_half2_rz(__uint_as_float(__float_as_uint(s.x) + d0),
                                     __uint_as_float(__float_as_uint(s.y) + d1));
    if (w0) *reinterpret_cast<uint16_t*>(p0) = (uint16_t)(u & 0xffffu);
    if (w1) *reinterpret_cast<uint16_t*>(p1) = (uint16_t)(u >> 16);
  } else {
    if (w0) *p0 = v.x;
    if (w1) *p1 = v.y;
  }
}

// ------------------------------------------------------------- predicates
// A pore site the paired kernel can update: not on a Dirichlet-class face and,
// with the fluid-fluid force on, every gradient-stencil neighbour pore.
template <int D, int ISO>
__device__ __forceinline__ bool pair_simple_site(const StepArgs& a, const PhysT<float>& P, uint32_t links, int x, int y,
                                                 int z) {
  if (any_dirichlet<D>(a.g, a.faces, x, y, z)) return false;
  if (!P.ff_on) return true;
  constexpr int RB = stencil_reach<D, ISO>();
  return stencil_is_links<D, ISO>() ? ((links | 1u) & (all_links<D>() | 1u)) == (all_links<D>() | 1u)
         : RB == 2                ? (links & kBoxPore2) != 0u
                                  : (links & kBoxPore3) != 0u;
}

// 1: the pair goes to k_step_pair; 0: to k_step_rest; -1: no pore site.
// The two cells of pair i: c0 = 2 i and c0 + 1, with their coordinates.
struct PairSites {
  unsigned c0;
  int x0, y0, z0, x1, y1, z1;
  __device__ __forceinline__ bool same_row() const { return x1 == x0 + 1; }
};
__device__ __forceinline__ PairSites pair_sites(const Geo& g, unsigned i) {
  PairSites ps;
  ps.c0 = 2u * i;
  const unsigned nx = (unsigned)g.nx, ny = (unsigned)g.ny;
  unsigned row = ps.c0 / nx;
  ps.x0 = (int)(ps.c0 - row * nx);
  ps.y0 = (int)(row % ny);
  ps.z0 = (int)(row / ny);
  if (ps.x0 + 1 < g.nx) {
    ps.x1 = ps.x0 + 1;
    ps.y1 = ps.y0;
    ps.z1 = ps.z0;
  } else {
    ++row;
    ps.x1 = 0;
    ps.y1 = (int)(row % ny);
    ps.z1 = (int)(row / ny);
  }
  return ps;
}

template <int D, int ISO>
__device__ __forceinline__ int pair_class(const StepArgs& a, const PhysT<float>& P, uint32_t l0, uint32_t l1,
                                          const PairSites& ps) {
  const bool p0 = (l0 & 1u) != 0u, p1 = (l1 & 1u) != 0u;
  if (!p0 && !p1) return -1;
  if (!ps.same_row()) return 0;  // spans a row end (odd nx): the per-site kernel
  const bool s0 = !p0 || pair_simple_site<D, ISO>(a, P, l0, ps.x0, ps.y0, ps.z0);
  const bool s1 = !p1 || pair_simple_site<D, ISO>(a, P, l1, ps.x1, ps.y1, ps.z1);
  return (s0 && s1) ? 1 : 0;
}

// --------------------------------------------------------------- the pair
// The pair of this thread in a one-dimensional launch over the pairs.
__device__ __forceinline__ bool pair_of(const Geo& g, PairSites& ps) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((long long)2 * i >= g.n) return false;
  ps = pair_sites(g, i);
  return true;
}

// The value of field src (rho, or psi with the EOS on) at the two cells
// (x0 + ex, x0 + 1 + ex) of row (ey, ez), per component.  With nx even, ex
// even lands on an aligned pair of cells (one 16-byte load for two
// components); ex odd takes each cell's own load.
template <int D, int S, int RCH, int ex, int ey, int ez>
__device__ __forceinline__ void field_pair(const Hood<D, RCH>& h0, const Hood<D, RCH>& h1, const float* src, V2 v[S]) {
  const unsigned c = h0.template at<ex, ey, ez>();
  if constexpr (S == 2 && (ex % 2 == 0)) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(src) + (c >> 1));
    v[0] = V2{t.x, t.z};
    v[1] = V2{t.y, t.w};
  } else if constexpr (S == 2) {
    const float2 a = __ldg(reinterpret_cast<const float2*>(src) + c);
    const float2 b = __ldg(reinterpret_cast<const float2*>(src) + h1.template at<ex, ey, ez>());
    v[0] = V2{a.x, b.x};
    v[1] = V2{a.y, b.y};
  } else {
    const unsigned c1 = h1.template at<ex, ey, ez>();
#pragma unroll
    for (int m = 0; m < S; ++m) v[m] = V2{__ldg(src + (size_t)c * S + m), __ldg(src + (size_t)c1 * S + m)};
  }
}

// The fluid-fluid force of both sites of a pair on a lattice with an even nx
// whose pore sites see only pore stencil neighbours (cell_forces' bulk
// gradient on V2 values): F -= psi(x) c0 sum_k g_mk grad_k, with
// grad = sum over opposite stencil terms of w e (psi(x + e) - psi(x - e)).
template <int D, int S, int ISO, int RCH>
__device__ __forceinline__ void pair_ff_bulk(const Hood<D, RCH>& h0, const Hood<D, RCH>& h1, const PhysT<float>& P,
                                             const float* src, const V2 mult[S], V2 F[S][D]) {
  V2 gr[S][D];
  bool seen[D] = {};
  constexpr int NT = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  sfor<0, NT>([&](auto tt) {
    constexpr int t = decltype(tt)::value;
    constexpr FFTerm T = ffterm<D>(t);
    if constexpr (T.level <= ISO && t < ff_opp<D>(t)) {
      constexpr int ex = T.e[0], ey = T.e[1], ez = T.e[2], tw = T.w;
      V2 vp[S], vm[S];
      field_pair<D, S, RCH, ex, ey, ez>(h0, h1, src, vp);
      field_pair<D, S, RCH, -ex, -ey, -ez>(h0, h1, src, vm);
      sfor<0, D>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        constexpr int e = d == 0 ? ex : (d == 1 ? ey : ez);
        if constexpr (e != 0) {
          const V2 coef = v2(float(e) * P.ffwq[d][tw]);
#pragma unroll
          for (int m = 0; m < S; ++m) gr[m][d] = seen[d] ? fma2(coef, vp[m] - vm[m], gr[m][d]) : coef * (vp[m] - vm[m]);
          seen[d] = true;
        }
      });
    }
  });
#pragma unroll
  for (int d = 0; d < D; ++d)
#pragma unroll
    for (int m = 0; m < S; ++m) {
      V2 acc = v2(P.c0g[m][0]) * gr[0][d];
#pragma unroll
      for (int k = 1; k < S; ++k) acc = fma2(v2(P.c0g[m][k]), gr[k][d], acc);
      F[m][d] = F[m][d] - mult[m] * acc;
    }
}

// Collision and push of one component of a simple pair.  FULL (pair_full):
// both sites pore with every link pore (no bounceback), in one row of an
// even-nx lattice, so the pushes need no selects; the caller takes FULL only
// when every active lane of the warp is full.
template <int D, int S, bool MRT, bool FULL, class T, int RCH>
struct PairPush {
  using L = Lat<D>;
  static constexpr int Q = L::Q;
  T* fout;
  unsigned N, c0;
  uint32_t l0, l1;
  bool p0, p1;
  Hood<D, RCH> h0, h1;
  uint32_t seed0;  // the pair's stochastic-rounding seed (FP16)
  Scl<float> sc;

  template <int n>
  __device__ __forceinline__ void operator()(std::integral_constant<int, n>, int m, V2 v) const {
    constexpr int o = opp<D>(n);
    const uint32_t k = (uint32_t)(m * Q + n);
    // FP16: both sites' 13-bit dithers from one multiply-shift product of the
    // pair's seed (bits 31..19 and 18..6; both fields of the product of a
    // uniform seed and an odd multiplier are uniform, so each rounding stays unbiased)
    uint32_t d0 = 0u, d1 = 0u;
    if constexpr (std::is_same<T, __half>::value) {
      const uint32_t prod = seed0 * (mix32(k + 1u) | 1u);
      d0 = prod >> 19;
      d1 = (prod >> 6) & 0x1fffu;
    }
    T* const sn = fout + (size_t)k * N;
    if constexpr (n == 0) {
      if (FULL || (p0 && p1)) {
        st_pair<T>(sn + c0, v, sc, d0, d1);
      } else {
        st_two<T>(sn + c0, sn + c0 + 1, v, sc, d0, d1, p0, p1);
      }
    } else {
      constexpr int cx = L::c(n, 0), cy = L::c(n, 1), cz = D == 3 ? L::c(n, 2) : 0;
      if constexpr (FULL) {
        if constexpr (cx == 0) {
          st_pair<T>(sn + h0.template at<0, cy, cz>(), v, sc, d0, d1);
        } else {
          st_two<T>(sn + h0.template at<cx, cy, cz>(), sn + h1.template at<cx, cy, cz>(), v, sc, d0, d1);
        }
      } else {
        T* const so = fout + (size_t)(m * Q + o) * N;
        const bool q0 = ((l0 >> n) & 1u) != 0u, q1 = ((l1 >> n) & 1u) != 0u;
        st_two<T>(q0 ? sn + h0.template at<cx, cy, cz>() : so + c0, q1 ? sn + h1.template at<cx, cy, cz>() : so + c0 + 1,
                  v, sc, d0, d1, p0, p1);
      }
    }
  }
};

// Fast-form collision of step_site (see there) of component m on V2 values,
// with the pushes.
template <int D>
struct VecD {
  V2 v[D];
};
template <int D, int S, bool MRT, bool FULL, class T, int RCH>
__device__ __forceinline__ void pair_collide_m(const PairPush<D, S, MRT, FULL, T, RCH> push,
                                                      const PhysT<float>& P, const T* fin, unsigned N, unsigned c0,
                                                      int m, V2 r, V2 rd, VecD<D> Fm_, VecD<D> up_) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  constexpr int NP = npairs<D>();
  V2 F[S][D], up[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    F[m][d] = Fm_.v[d];
    up[d] = up_.v[d];
  }
  V2 usqr = up[0] * up[0];
#pragma unroll
  for (int d = 1; d < D; ++d) usqr = fma2(up[d], up[d], usqr);
  const V2 cu_axis = v2(float(1.5 * L::w(1))) * usqr, cu_diag = v2(float(1.5 * L::w(Q - 1))) * usqr;
  V2 Bo[NP], WBe[NP];
  sfor<0, NP>([&](auto pp) {
    constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
    constexpr double w = L::w(n);
    const V2 ud = cdot2<D, n>(up);
    Bo[p] = v2(float(3 * w)) * ud;
    WBe[p] = fma2(v2(float(4.5 * w)) * ud, ud, -(n <= L::NAXIS ? cu_axis : cu_diag));
  });
  const V2 WB0 = v2(D == 3 ? -0.5f : float(-2.0 / 3.0)) * usqr;
  {
    const V2 WA0 = v2(P.WAc[m][0]), WA1 = v2(P.WAc[m][1]), WA2 = v2(P.WAc[m][2]);
    const V2 cA0 = v2(P.cA[m][0]), cA1 = v2(P.cA[m][1]), cA2 = v2(P.cA[m][2]);
    const V2 s0 = v2(P.s0[m]);
    const float kf = P.kfac[m];
    const float keepf = P.keep[m];
    const V2 keep = v2(std::is_same<T, __half>::value ? keepf * push.sc.inv : keepf);
    V2 Fu = F[m][0] * up[0], kF[D];
#pragma unroll
    for (int d = 1; d < D; ++d) Fu = fma2(F[m][d], up[d], Fu);
#pragma unroll
    for (int d = 0; d < D; ++d) kF[d] = v2(kf) * F[m][d];
    const V2 kFu = v2(kf) * Fu;
    const V2 G = fma2(s0, r, -kFu);
    const unsigned spec = P.spec_mask[m];
    const T* fm = fin + (size_t)m * Q * N + c0;
    // the stored value (storage scale not divided out: keep carries it)
    auto pop = [&](auto nn) -> V2 { return ld_pair_raw<T>(fm + (size_t)decltype(nn)::value * N); };
    const V2 E0 = WA0 + WB0;
    // rest direction: g'_0 = keep g_0 + X0
    const V2 X0 = s0 * fma2(WA0, rd, fma2(WB0, r, cA0)) - E0 * kFu;
    auto pair_terms = [&](auto pp, V2& pe, V2& po) {
      constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
      const V2 WA = n <= L::NAXIS ? WA1 : WA2;
      const V2 Ae = WA + WBe[p];
      const V2 h = cdot2<D, n>(kF);
      const V2 De = fma2(WA, rd, fma2(WBe[p], r, n <= L::NAXIS ? cA1 : cA2));
      pe = fma2(s0, De, fma2(Bo[p], h, -(Ae * kFu)));
      po = fma2(Bo[p], G, Ae * h);
    };
    if (spec == 0u && keepf == 0.f) {
      // s0 = 1 (tau = 1): the relaxed populations are the forced equilibrium
      push(std::integral_constant<int, 0>{}, m, X0);
      sfor<0, NP>([&](auto pp) {
        constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
        V2 pe, po;
        pair_terms(pp, pe, po);
        push(std::integral_constant<int, n>{}, m, pe + po);
        push(std::integral_constant<int, nb>{}, m, pe - po);
      });
    } else if (spec == 0u) {
      // every moment relaxes at s0 (BGK)
      push(std::integral_constant<int, 0>{}, m, fma2(keep, pop(std::integral_constant<int, 0>{}), X0));
      sfor<0, NP>([&](auto pp) {
        constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
        V2 pe, po;
        pair_terms(pp, pe, po);
        push(std::integral_constant<int, n>{}, m, fma2(keep, pop(std::integral_constant<int, n>{}), pe + po));
        push(std::integral_constant<int, nb>{}, m, fma2(keep, pop(std::integral_constant<int, nb>{}), pe - po));
      });
    } else if (spec == stress_mask<D>()) {
      // s_nu != s0, every other rate s0: pair sums of the non-equilibrium
      // part, the s_nu moments' corrections, then each pair relaxed
      V2 F3[D];
#pragma unroll
      for (int d = 0; d < D; ++d) F3[d] = v2(3.f) * F[m][d];
      const V2 hFu2 = v2(3.f) * Fu;
      const V2 inv = v2(std::is_same<T, __half>::value ? push.sc.inv : 1.f);
      // the s_nu moments of the pair sums of the non-equilibrium part,
      // S_p = g_n + g_n~ - 2 De - Ae (3 F.u) + Bo c_n.(3 F), accumulated pair by pair
      V2 ck[Q];
      bool seen[Q] = {};
      sfor<0, NP>([&](auto pp) {
        constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
        const V2 WA = n <= L::NAXIS ? WA1 : WA2;
        const V2 Ae = WA + WBe[p];
        const V2 t2 = cdot2<D, n>(F3);
        const V2 gs = (pop(std::integral_constant<int, n>{}) + pop(std::integral_constant<int, nb>{})) * inv;
        const V2 De = fma2(WA, rd, fma2(WBe[p], r, n <= L::NAXIS ? cA1 : cA2));
        const V2 Sp = fma2(Bo[p], t2, fma2(v2(-2.f), De, gs) - Ae * hFu2);
        sfor<0, Q>([&](auto kk) {
          constexpr int kq = decltype(kk)::value;
          if constexpr (rate_of<D>(kq) == R_NU) {
            constexpr int v = L::mt(n, kq);
            if constexpr (v != 0) {
              if (!seen[kq])
                ck[kq] = v == 1 ? Sp : (v == -1 ? -Sp : v2(float(v)) * Sp);
              else
                ck[kq] = v == 1 ? ck[kq] + Sp : (v == -1 ? ck[kq] - Sp : fma2(v2(float(v)), Sp, ck[kq]));
              seen[kq] = true;
            }
          }
        });
      });
      sfor<0, Q>([&](auto kk) {
        constexpr int kq = decltype(kk)::value;
        if constexpr (rate_of<D>(kq) == R_NU) ck[kq] = v2(P.dspec[m][kq]) * ck[kq];
      });
      const bool k0 = keepf == 0.f;
      push(std::integral_constant<int, 0>{}, m, k0 ? X0 : fma2(keep, pop(std::integral_constant<int, 0>{}), X0));
      sfor<0, NP>([&](auto pp) {
        constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
        V2 pe, po;
        pair_terms(pp, pe, po);
        sfor<0, Q>([&](auto kk) {
          constexpr int kq = decltype(kk)::value;
          if constexpr (rate_of<D>(kq) == R_NU) {
            constexpr int v = L::mt(n, kq);
            if constexpr (v == 1) pe = pe - ck[kq];
            else if constexpr (v == -1) pe = pe + ck[kq];
            else if constexpr (v != 0) pe = fma2(v2(float(-v)), ck[kq], pe);
          }
        });
        if (k0) {
          push(std::integral_constant<int, n>{}, m, pe + po);
          push(std::integral_constant<int, nb>{}, m, pe - po);
        } else {
          push(std::integral_constant<int, n>{}, m, fma2(keep, pop(std::integral_constant<int, n>{}), pe + po));
          push(std::integral_constant<int, nb>{}, m, fma2(keep, pop(std::integral_constant<int, nb>{}), pe - po));
        }
      });
    } else if constexpr (MRT) {
      // general rate pattern: relax every moment at s0, then correct each
      // moment whose rate differs by dspec_k times its projection of the
      // deviation from the forced equilibrium
      V2 fo[Q], dfi[Q];
      // the deviations themselves (pop is the stored value, keep carries the scale)
      const V2 inv = v2(std::is_same<T, __half>::value ? push.sc.inv : 1.f);
      const V2 g0 = pop(std::integral_constant<int, 0>{});
      fo[0] = fma2(keep, g0, X0);
      const V2 hFu = v2(1.5f) * Fu;
      V2 hF[D];
#pragma unroll
      for (int d = 0; d < D; ++d) hF[d] = v2(1.5f) * F[m][d];
      dfi[0] = g0 * inv - fma2(WA0, rd, fma2(WB0, r, cA0)) - E0 * hFu;
      sfor<0, NP>([&](auto pp) {
        constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
        V2 pe, po;
        pair_terms(pp, pe, po);
        const V2 sn_ = pop(std::integral_constant<int, n>{}), sb_ = pop(std::integral_constant<int, nb>{});
        fo[n] = fma2(keep, sn_, pe + po);
        fo[nb] = fma2(keep, sb_, pe - po);
        const V2 gn = sn_ * inv, gb = sb_ * inv;
        const V2 WA = n <= L::NAXIS ? WA1 : WA2;
        const V2 t = cdot2<D, n>(hF);
        const V2 En = WA + WBe[p] + Bo[p], Eb = WA + WBe[p] - Bo[p];
        const V2 De = fma2(WA, rd, fma2(WBe[p], r, n <= L::NAXIS ? cA1 : cA2));
        dfi[n] = fma2(En, t - hFu, gn - fma2(Bo[p], r, De));
        dfi[nb] = gb - fma2(Bo[p], -r, De) - Eb * (t + hFu);
      });
      sfor<0, Q>([&](auto kk) {
        constexpr int kq = decltype(kk)::value;
        if (spec & (1u << kq)) {
          V2 md{0.f, 0.f};
          sfor<0, Q>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            constexpr int v = L::mt(i, kq);
            if constexpr (v == 1) md = md + dfi[i];
            else if constexpr (v == -1) md = md - dfi[i];
            else if constexpr (v != 0) md = fma2(v2(float(v)), dfi[i], md);
          });
          const V2 ck = v2(P.dspec[m][kq]) * md;
          sfor<0, Q>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            constexpr int v = L::mt(i, kq);
            if constexpr (v == 1) fo[i] = fo[i] - ck;
            else if constexpr (v == -1) fo[i] = fo[i] + ck;
            else if constexpr (v != 0) fo[i] = fma2(v2(float(-v)), ck, fo[i]);
          });
        }
      });
      sfor<0, Q>([&](auto nn) { push(nn, m, fo[decltype(nn)::value]); });
    }
  }
}

template <int D, int S, bool MRT, bool FULL, class T, int RCH>
__device__ __forceinline__ void pair_collide(const PairPush<D, S, MRT, FULL, T, RCH>& push, const PhysT<float>& P,
                                             const T* fin, unsigned N, unsigned c0, const V2 rc[S], const V2 rcd[S],
                                             const V2 F[S][D], const V2 up[D]) {
  VecD<D> u;
#pragma unroll
  for (int d = 0; d < D; ++d) u.v[d] = up[d];
#pragma unroll
  for (int m = 0; m < S; ++m) {
    VecD<D> f;
#pragma unroll
    for (int d = 0; d < D; ++d) f.v[d] = F[m][d];
    pair_collide_m<D, S, MRT, FULL, T, RCH>(push, P, fin, N, c0, m, rc[m], rcd[m], f, u);
  }
}

// One simple pair: forces per site, moments and collision on V2.
template <int D, int S, int ISO, bool MRT, class T>
__device__ __forceinline__ void step_pair(const StepArgs& a, const PairSites& ps, uint32_t l0, uint32_t l1,
                                          bool warp_full) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  constexpr int RCH = stencil_reach<D, ISO>();
  const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
  const unsigned N = (unsigned)a.g.n;
  const unsigned c0 = ps.c0;
  const bool p0 = (l0 & 1u) != 0u, p1 = (l1 & 1u) != 0u;
  // the pair lies in one row (pair_class): x0 + 1, y0, z0
  const Hood<D, RCH> h0(a.g, ps.x0, ps.y0, ps.z0), h1(a.g, ps.x0 + 1, ps.y0, ps.z0);
  const Scl<float> sc = scl_of(P);
  uint32_t seed0 = 0;
  if constexpr (std::is_same<T, __half>::value) {
    const uint32_t st = 0x9E3779B9u * ((a.steps_ptr ? __ldg(a.steps_ptr) : a.step) + 1u);
    seed0 = mix32(c0 ^ st);  // one seed per pair (PairPush draws both sites' dithers from it)
  }
#if TX_PAIR_PREFETCH
  // ask for the pair's population lines now, so that they arrive in L1 while
  // the forces are computed (a hint: no register waits for it)
  {
    const T* fin0 = reinterpret_cast<const T*>(a.fin) + c0;
#pragma unroll
    for (int k = 0; k < S * Q; ++k) prefetch_l1(fin0 + (size_t)k * N);
  }
#endif
  // forcing density of both sites, then each site's forces (step_site's cell_forces)
  const float* rho = reinterpret_cast<const float*>(a.rho);
  float rfd0[S], rfd1[S], rf0[S], rf1[S];
  if constexpr (S == 2) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(rho) + (c0 >> 1));
    rfd0[0] = t.x;
    rfd0[1] = t.y;
    rfd1[0] = t.z;
    rfd1[1] = t.w;
  } else {
#pragma unroll
    for (int m = 0; m < S; ++m) {
      rfd0[m] = __ldg(rho + (size_t)c0 * S + m);
      rfd1[m] = __ldg(rho + (size_t)(c0 + 1) * S + m);
    }
  }
#pragma unroll
  for (int m = 0; m < S; ++m) {
    rf0[m] = P.rho0[m] + rfd0[m];
    rf1[m] = P.rho0[m] + rfd1[m];
  }
  float F0[S][D], F1[S][D];
#pragma unroll
  for (int m = 0; m < S; ++m)
#pragma unroll
    for (int d = 0; d < D; ++d) F0[m][d] = F1[m][d] = 0.f;
  const float* psi = reinterpret_cast<const float*>(a.psi);
  // with an even nx the fluid-fluid force of both sites comes from one pass
  // over aligned cell pairs (pair_ff_bulk); otherwise each site's cell_forces
  const bool pair_ff = (a.g.nx & 1) == 0;
  if (pair_ff) {
    if (p0) cell_forces<D, S, ISO, false, RCH, float, float, true, false>(h0, l0, P, a.mask, rho, psi, a.g.n, rfd0, rf0, F0);
    if (p1) cell_forces<D, S, ISO, false, RCH, float, float, true, false>(h1, l1, P, a.mask, rho, psi, a.g.n, rfd1, rf1, F1);
  } else {
    if (p0) cell_forces<D, S, ISO, false, RCH, float, float, true>(h0, l0, P, a.mask, rho, psi, a.g.n, rfd0, rf0, F0);
    if (p1) cell_forces<D, S, ISO, false, RCH, float, float, true>(h1, l1, P, a.mask, rho, psi, a.g.n, rfd1, rf1, F1);
  }
  V2 F[S][D], rc[S], rcd[S];
#pragma unroll
  for (int m = 0; m < S; ++m) {
    rc[m] = V2{rf0[m], rf1[m]};
    rcd[m] = V2{rfd0[m], rfd1[m]};
#pragma unroll
    for (int d = 0; d < D; ++d) F[m][d] = V2{F0[m][d], F1[m][d]};
  }
  if (pair_ff && P.ff_on) {
    // psi(x) (EOS on) or rho(x) scales the force; wall lanes are discarded
    V2 mult[S];
    if (P.eos_on) {
      V2 self[S];
      field_pair<D, S, RCH, 0, 0, 0>(h0, h1, psi, self);
#pragma unroll
      for (int m = 0; m < S; ++m) mult[m] = self[m];
    } else {
#pragma unroll
      for (int m = 0; m < S; ++m) mult[m] = rc[m];
    }
    pair_ff_bulk<D, S, ISO, RCH>(h0, h1, P, P.eos_on ? psi : rho, mult, F);
  }
  // moments: flux of each component from pair differences, common velocity
  const T* fin = reinterpret_cast<const T*>(a.fin);
  V2 up[D];
  {
    V2 num[D], den = v2(0.f);
#pragma unroll
    for (int d = 0; d < D; ++d) num[d] = v2(0.f);
#pragma unroll
    for (int m = 0; m < S; ++m) {
      V2 j[D];
      bool seen[D] = {};
      const T* fm = fin + (size_t)m * Q * N + c0;
      sfor<0, npairs<D>()>([&](auto pp) {
        constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
        const V2 dlt = ld_pair_raw<T>(fm + (size_t)n * N) - ld_pair_raw<T>(fm + (size_t)nb * N);
        sfor<0, D>([&](auto dd) {
          constexpr int d = decltype(dd)::value;
          constexpr int c = L::c(n, d);
          if constexpr (c != 0) {
            const V2 t = c == 1 ? dlt : (c == -1 ? -dlt : v2(float(c)) * dlt);
            j[d] = seen[d] ? j[d] + t : t;
            seen[d] = true;
          }
        });
      });
      if constexpr (std::is_same<T, __half>::value) {
        // the storage scale out of the sums
        const V2 inv = v2(sc.inv);
#pragma unroll
        for (int d = 0; d < D; ++d) j[d] = j[d] * inv;
      }
      const V2 mm = v2(P.mmot[m]);
#pragma unroll
      for (int d = 0; d < D; ++d) num[d] = fma2(fma2(v2(0.5f), F[m][d], j[d]), mm, num[d]);
      den = fma2(rc[m], mm, den);
    }
    const V2 inv{__frcp_rn(den.x), __frcp_rn(den.y)};
#pragma unroll
    for (int d = 0; d < D; ++d) up[d] = num[d] * inv;
  }
  T* fout = reinterpret_cast<T*>(a.fout);
  if (warp_full) {
    const PairPush<D, S, MRT, true, T, RCH> push{fout, N, c0, l0, l1, p0, p1, h0, h1, seed0, sc};
    pair_collide<D, S, MRT, true, T, RCH>(push, P, fin, N, c0, rc, rcd, F, up);
  } else {
    const PairPush<D, S, MRT, false, T, RCH> push{fout, N, c0, l0, l1, p0, p1, h0, h1, seed0, sc};
    pair_collide<D, S, MRT, false, T, RCH>(push, P, fin, N, c0, rc, rcd, F, up);
  }
}

// Whether a pair of k_step_pair (one row) goes the bounceback-free way (see
// PairPush): both sites pore with every link pore, on a lattice with an even
// nx (so that the y and z neighbours' pair slots are aligned for one store).
template <int D>
__device__ __forceinline__ bool pair_full(const Geo& g, const PairSites& ps, uint32_t l0, uint32_t l1) {
  constexpr uint32_t all = all_links<D>() | 1u;
  return (g.nx & 1) == 0 && (l0 & all) == all && (l1 & all) == all;
}

// k_step_pair / k_step_rest / k_count_rest: one thread per pair, 1-D grid.
// k_step_pair: each thread takes TX_PAIR_PER_THREAD pairs, one grid apart;
// with more than one it asks for the next pair's population lines before
// updating the current one.
template <int D, int S, int ISO, bool MRT, class T>
__global__ void __launch_bounds__(128, TX_PAIR_MIN_BLOCKS(S)) k_step_pair(StepArgs a_in) {
  const StepArgs a = a_in;
  const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
  const unsigned stride = gridDim.x * blockDim.x;
  const unsigned npairs = (unsigned)(a.g.n / 2);
  constexpr int Q = Lat<D>::Q;
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int r = 0; r < TX_PAIR_PER_THREAD; ++r, i += stride) {
    if (r + 1 < TX_PAIR_PER_THREAD && i + stride < npairs) {
      const T* nxt = reinterpret_cast<const T*>(a.fin) + 2u * (i + stride);
#pragma unroll
      for (int k = 0; k < S * Q; ++k) prefetch_l1(nxt + (size_t)k * (size_t)a.g.n);
    }
    bool run = false, full = false;
    uint2 ll = make_uint2(0u, 0u);
    PairSites ps{};
    if (i < npairs) {
      ps = pair_sites(a.g, i);
      ll = __ldg(reinterpret_cast<const uint2*>(a.links) + (ps.c0 >> 1));
      run = pair_class<D, ISO>(a, P, ll.x, ll.y, ps) == 1;
      full = pair_full<D>(a.g, ps, ll.x, ll.y);
    }
    // every lane votes, so that the vote is uniform over the warp's running lanes
    const bool warp_full = __all_sync(0xffffffffu, full || !run);
    if (run) step_pair<D, S, ISO, MRT, T>(a, ps, ll.x, ll.y, warp_full);
  }
}

template <int D, int S, int ISO, bool MRT, class T>
__global__ void __launch_bounds__(128, TX_STEP_MIN_BLOCKS(S, float, MRT)) k_step_rest(StepArgs a_in) {
  const StepArgs a = a_in;
  PairSites ps;
  if (!pair_of(a.g, ps)) return;
  const uint2 ll = __ldg(reinterpret_cast<const uint2*>(a.links) + (ps.c0 >> 1));
  const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
  if (pair_class<D, ISO>(a, P, ll.x, ll.y, ps) != 0) return;
  step_site<D, S, ISO, MRT, false, T, float, float>(a, ps.x0, ps.y0, ps.z0);
  step_site<D, S, ISO, MRT, false, T, float, float>(a, ps.x1, ps.y1, ps.z1);
}

// Pairs that need the per-site kernel (the count decides whether k_step_rest runs).
template <int D, int ISO>
__global__ void __launch_bounds__(256) k_count_rest(StepArgs a_in, unsigned* count) {
  const StepArgs a = a_in;
  PairSites ps;
  if (!pair_of(a.g, ps)) return;
  const uint2 ll = __ldg(reinterpret_cast<const uint2*>(a.links) + (ps.c0 >> 1));
  const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
  if (pair_class<D, ISO>(a, P, ll.x, ll.y, ps) == 0) atomicAdd(count, 1u);
}

}  // namespace tx
