// CUDA kernels of the Shan-Chen flow step (sm_103a).
//
// Device state between steps is the reference's fi after FlowApplyBCs (the
// post-stream, post-boundary populations) in SoA layout f[(m*Q + n)*N + cell],
// cell = x + nx*(y + ny*z), plus the density used for forcing, rho[cell*S + m].
// One step of LBMRun2 (src/lbm/lbm.F90:283-363) is two launches:
//
//   k_step     per pore site: forces (fluid-solid, body, Shan-Chen), flux and
//              common velocity (FlowUpdateFlux), equilibrium, forcing prefactor
//              and BGK/MRT collision (FlowCollision), then push-streaming with
//              bounceback folded in (FlowStream + FlowBounceback): population n
//              goes to x + c_n, or back to x as opp(n) when x + c_n is a wall
//              (periodic axes wrap; non-periodic faces are ghost walls).
//   k_density  per pore site of the pushed populations: Dirichlet density
//              faces (BCApplyDirichletNode) and the forcing density
//              (DistributionCalcDensity + BCApplyDirichletToRho).
//
// The forces and velocity of a step are recomputed at the start of the next
// k_step from (f, rho), so they are the values the reference stores between
// steps.  Template parameters:
//   D      2 (D2Q9) or 3 (D3Q19)        S    number of components
//   ISO    isotropy order 4, 8, 10      MRT  MRT (true) or BGK (false)
//   EXACT  reference operation order: no FMA (its translation unit is built
//          with --fmad=false), IEEE divides, the reference's expression shapes
//   T      population storage type (double holds f; float holds f - w_n*rho0_m
//          and half (f - w_n*rho0_m) * storage scale, the deviation from a
//          per-component rest density, with the forcing density stored as
//          rho - rho0_m)
//   R      arithmetic type              RT   storage type of rho
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include <cmath>
#include <cstring>

#include "../../include/taxila_gb300.h"

// Resident 128-thread blocks per SM that ptxas must make room for in the
// float-arithmetic k_step: 4 (128 registers a thread) for two components, 6
// (80 registers, no spills) for one.  The FP64 form is bound by the FP64 pipe
// and keeps its full register budget.
#ifndef TX_FLOAT_MIN_BLOCKS
#define TX_FLOAT_MIN_BLOCKS 4
#endif
#ifndef TX_FLOAT_MIN_BLOCKS_S1
#define TX_FLOAT_MIN_BLOCKS_S1 6
#endif
// FP64 step kernels without the general MRT rate path fit 168 registers
// without spills: 3 blocks of 128 threads per SM
#ifndef TX_F64_MIN_BLOCKS
#define TX_F64_MIN_BLOCKS 3
#endif
#define TX_STEP_MIN_BLOCKS(S, R, GENERAL) \
  (sizeof(R) == 4 ? ((S) == 1 ? TX_FLOAT_MIN_BLOCKS_S1 : TX_FLOAT_MIN_BLOCKS) : ((GENERAL) ? 1 : TX_F64_MIN_BLOCKS))

#include "tx_ff_stencil.cuh"
#include "tx_lattice.cuh"

namespace tx {

constexpr int MAXC = 4;
constexpr int MAXMIN = 16;

struct Geo {
  int nx, ny, nz;
  int per[3];
  long long n;
};

// Parameters in the arithmetic type R of the kernels that read them (the
// handle keeps an FP64 and an FP32 copy on the device).
template <class R>
struct PhysT {
  R tau[MAXC], inv_tau[MAXC], cs2[MAXC], inv_cs2[MAXC], dk[MAXC], mm[MAXC], mmot[MAXC];
  R g[MAXC][MAXC];
  R gw[MAXMIN + 1][MAXC];  // row = mineral id (row 0 unused)
  R gvt[3];
  R ffw[12];
  R c0, fs_w_axis, fs_w_diag;
  R srate[MAXC][19];       // MRT rate of moment k
  R srate_mmt[MAXC][19];   // rate / diag(M M^T)
  R rho0[MAXC];            // rest density of the deviation storage (0 in the FP64 form)
  R sscale, inv_sscale;    // FP16 storage scale of the deviations (1 otherwise)
  // equilibrium constants: feq_n = rho W~_n (A_n + B_n) with A_0 = A0, A_n = An
  // (= 1/mm), and cA = (W~_n A_n - w_n) rho0 for the rest, axis and diagonal
  // classes, evaluated exactly on the host (zero for unit molecular mass)
  R A0[MAXC], An[MAXC], cA[MAXC][3];
  // non-ideal EOS: psi(rho) replaces rho in the fluid-fluid force when eos_on
  // (coefficients: SC rho0 | thermo psi0, rho0 | PR a, b, T, alpha)
  int eos_on;
  int eos[MAXC];
  R eos_c[MAXC][4];
  // fast form: relax every moment at s0, then correct the moments whose rate
  // differs (bit k of spec_mask) by dspec = (rate_k - s0) / diag(M M^T)_k
  R s0[MAXC];
  R dspec[MAXC][19];
  R inv_ws_full[3];        // 1 / weight sum of a gradient stencil with every neighbour pore
  unsigned spec_mask[MAXC];
  // fast-form constants folded on the host: W~A per direction class (rest,
  // axis, diagonal), 1 - s0, 3 - 1.5 s0, c0 g[m][k], ffw[w] / ws_full[d]
  R WAc[MAXC][3], keep[MAXC], kfac[MAXC];
  R c0g[MAXC][MAXC];
  R ffwq[3][12];
  int ff_on, fs_on, body_on;
  // every component has the same W~A (equal molecular masses): the FP64 fast
  // form computes the equilibrium weights E_n once per site
  int wa_shared;
  // two components coupled only to each other (g_11 = g_22 = 0)
  int ff_cross;
  // every component has the same mm s_c: it cancels from the common velocity
  int mmot_shared;
};
using Phys = PhysT<double>;

template <class R, class Src>
inline void convert_phys(const PhysT<Src>& a, PhysT<R>* b) {
  auto cp = [](const Src* x, R* y, int n) { for (int i = 0; i < n; ++i) y[i] = R(x[i]); };
  cp(a.tau, b->tau, MAXC); cp(a.inv_tau, b->inv_tau, MAXC); cp(a.cs2, b->cs2, MAXC); cp(a.inv_cs2, b->inv_cs2, MAXC);
  cp(a.dk, b->dk, MAXC); cp(a.mm, b->mm, MAXC); cp(a.mmot, b->mmot, MAXC);
  cp(&a.g[0][0], &b->g[0][0], MAXC * MAXC); cp(&a.gw[0][0], &b->gw[0][0], (MAXMIN + 1) * MAXC);
  cp(a.gvt, b->gvt, 3); cp(a.ffw, b->ffw, 12);
  b->c0 = R(a.c0); b->fs_w_axis = R(a.fs_w_axis); b->fs_w_diag = R(a.fs_w_diag);
  cp(&a.srate[0][0], &b->srate[0][0], MAXC * 19); cp(&a.srate_mmt[0][0], &b->srate_mmt[0][0], MAXC * 19);
  cp(a.rho0, b->rho0, MAXC);
  cp(a.A0, b->A0, MAXC); cp(a.An, b->An, MAXC); cp(&a.cA[0][0], &b->cA[0][0], MAXC * 3);
  b->eos_on = a.eos_on;
  for (int m = 0; m < MAXC; ++m) b->eos[m] = a.eos[m];
  cp(&a.eos_c[0][0], &b->eos_c[0][0], MAXC * 4);
  b->sscale = R(a.sscale);
  b->inv_sscale = R(a.inv_sscale);
  cp(a.s0, b->s0, MAXC); cp(&a.dspec[0][0], &b->dspec[0][0], MAXC * 19); cp(a.inv_ws_full, b->inv_ws_full, 3);
  for (int m = 0; m < MAXC; ++m) b->spec_mask[m] = a.spec_mask[m];
  cp(&a.WAc[0][0], &b->WAc[0][0], MAXC * 3); cp(a.keep, b->keep, MAXC); cp(a.kfac, b->kfac, MAXC);
  cp(&a.c0g[0][0], &b->c0g[0][0], MAXC * MAXC); cp(&a.ffwq[0][0], &b->ffwq[0][0], 36);
  b->ff_on = a.ff_on; b->fs_on = a.fs_on; b->body_on = a.body_on;
  b->wa_shared = a.wa_shared; b->ff_cross = a.ff_cross; b->mmot_shared = a.mmot_shared;
}

// Classes of the exterior BC kinds, as bc%flags holds them next to
// flow%bc_flags (FlowParseBC, lbm_flow.F90:1031-1309; include/lbm_definitions.h:30-35).
enum : int { kClsNone = 0, kClsRefl = 2, kClsDir = 3, kClsNeu = 4, kClsVel = 5 };
__host__ __device__ constexpr int bc_class(int kind) {
  return kind == TX_BC_REFLECTING ? kClsRefl
         : (kind == TX_BC_DENSITY || kind == TX_BC_PRESSURE || kind == TX_BC_PRESSURE_INLET ||
            kind == TX_BC_PRESSURE_OUTLET)
             ? kClsDir
         : (kind == TX_BC_FLUX || kind == TX_BC_MOMENTUM || kind == TX_BC_FLUX_INLET || kind == TX_BC_FLUX_OUTLET)
             ? kClsNeu
         : kind == TX_BC_VELOCITY ? kClsVel
                                  : kClsNone;
}

struct Faces {
  int on[6];              // Dirichlet, Neumann or velocity class: the node density is re-summed
                          // after the corrections (BCUpdateRho, lbm_bc.F90:436-611)
  int dir[6];             // Dirichlet class: the face value is the forcing density of the node
                          // (BCApplyDirichletToRho, lbm_bc.F90:252-434)
  int cls[6];             // kCls* per face XM..ZP
  const double* vals[6];  // [k * area + node], k = d * S + m: the reference's (s, ndims) block
                          // per node; nodes in natural order of the tangential axes
  int order[4];           // BCApply's class sequence (first appearance over XM..ZP, lbm_bc.F90:781-807)
  int norder;
  int post;               // 1: every node correction runs in k_faces (some face is not Dirichlet)
};

// FlowUpdateDensityFromPressure (lbm_flow.F90:2235-2263): component densities
// of pressure p at mass fraction rho1frac (one or two components), in the
// reference's operation order.  g21 = components(2)%gf(1).
__host__ __device__ inline void density_from_pressure(int S, double c0, double g21, double pressure, double rho1frac,
                                                      double* rho) {
  const double eps = 1.e-10;
  if (S == 1) {
    rho[0] = pressure * 3.0;
  } else if (rho1frac < eps) {
    rho[0] = 0.0;
    rho[1] = pressure * 3.0;
  } else if (rho1frac > 1 - eps) {
    rho[0] = pressure * 3.0;
    rho[1] = 0.0;
  } else {
    const double alpha = 1.0 / (1.0 / rho1frac - 1.0);
    rho[0] = (-((1.0 + alpha) / 3.0) + sqrt((1.0 + alpha) / 3.0 * (1.0 + alpha) / 3.0 + 4. * c0 * g21 * alpha * pressure)) /
             (2 * c0 * g21);
    rho[1] = rho[0] / alpha;
  }
}

// The deviation storage of a lattice for the natural-order conversions.
struct Shift {
  double rho0[MAXC];
  double scale;
};
inline Shift shift_of(const PhysT<double>& P) {
  Shift s{};
  for (int m = 0; m < MAXC; ++m) s.rho0[m] = P.rho0[m];
  s.scale = P.sscale;
  return s;
}

struct StepArgs {
  const void* fin;
  void* fout;
  void* rho;                // RT [cell * S + m]
  const uint8_t* mask;      // 0 pore, 1..16 mineral, 255 other wall
  const uint32_t* links;    // link mask of every site (k_links)
  const void* phys;         // device PhysT<R> of the kernels' arithmetic type
  Geo g;
  Faces faces;
  void* psi;                // RT [cell * S + m]: psi(rho) when the EOS is on, else unused
  // step count of this lattice: seeds the stochastic rounding of FP16 stores.
  // Handles pass it by value; batches pass steps_ptr, a per-lattice device
  // counter that the density pass advances (so replayed graphs see it move).
  unsigned step;
  const unsigned* steps_ptr;
  // FP32-arithmetic forms on lattices with an even site count (tx_pair.cuh): pairs
  // that need the per-site kernel k_step_rest (-1: not counted, run it)
  int rest;
};

// psi(rho) of one component: EOSApply_Rho / _SC / _Thermo / _PR
// (lbm_eos.F90:183-350) in the reference's expression shapes; R = 1 in PR.
// A negative PR radicand gives NaN here (the reference stops with an error).
template <class R>
__host__ __device__ __forceinline__ R eos_psi(int type, const R c[4], R gmm, R c0, R rho) {
  if (type == TX_EOS_SC) return c[0] * (R(1.) - exp(-rho / c[0]));
  if (type == TX_EOS_THERMO) return c[0] * exp(-c[1] / rho);
  if (type == TX_EOS_PR) {
    const R a = c[0], b = c[1], T = c[2], alpha = c[3];
    const R br = b * rho;
    const R tmp = R(2.) * (rho * T / (R(1.) - br) - (a * alpha) * (rho * rho) / (R(1.) + R(2.) * b * rho - br * br) - rho / R(3.)) /
                  (c0 * gmm);
    return sqrt(tmp);
  }
  return rho;
}

// ----------------------------------------------------------------- storage
template <class T>
struct St;
template <>
struct St<double> {
  __device__ static __forceinline__ double ld(const double* p) { return __ldg(p); }
  __device__ static __forceinline__ void st(double* p, double v) { *p = v; }
};
template <>
struct St<float> {
  __device__ static __forceinline__ float ld(const float* p) { return __ldg(p); }
  __device__ static __forceinline__ void st(float* p, float v) { *p = v; }
};
template <>
struct St<__half> {
  __device__ static __forceinline__ float ld(const __half* p) { return __half2float(__ldg(p)); }
  __device__ static __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
};
template <class T>
constexpr bool kShifted = !std::is_same<T, double>::value;

// Population deviation f - w_n rho0 at p (the FP16 form divides the storage scale out).
template <class T, class R>
__device__ __forceinline__ R ld_dev(const T* p, const PhysT<R>& P) {
  if constexpr (std::is_same<T, __half>::value)
    return R(St<T>::ld(p)) * P.inv_sscale;
  else
    return R(St<T>::ld(p));
}
template <class T, class R>
__device__ __forceinline__ void st_dev(T* p, R v, const PhysT<R>& P) {
  if constexpr (std::is_same<T, __half>::value)
    St<T>::st(p, v * P.sscale);
  else
    St<T>::st(p, v);
}

// The fast forms' 1/x: in FP32 the correctly rounded reciprocal (no general
// division path); in FP64 the division 1/x, which measured fewer FP64
// instructions per site than __drcp_rn (412 against 427) in k_step.
__device__ __forceinline__ double rcp_rn(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }

// The FP16 storage scale and its inverse, read from the parameter block once
// per thread: the compiler cannot tell that population stores leave the
// parameter block alone, so a field read after a store is read again.
template <class R>
struct Scl {
  R s, inv;
};
template <class R>
__device__ __forceinline__ Scl<R> scl_of(const PhysT<R>& P) {
  return Scl<R>{P.sscale, P.inv_sscale};
}
template <class T, class R>
__device__ __forceinline__ R ld_dev_s(const T* p, Scl<R> sc) {
  if constexpr (std::is_same<T, __half>::value)
    return R(St<T>::ld(p)) * sc.inv;
  else
    return R(St<T>::ld(p));
}

// 32-bit integer finaliser (the "lowbias32" constants of C. Wellons' hash
// prospector): a well-mixed hash of the site, direction and step.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352dU;
  h ^= h >> 15;
  h *= 0x846ca68bU;
  h ^= h >> 16;
  return h;
}

// FP16 store with stochastic rounding: the 13 FP32 mantissa bits that FP16
// drops are rounded up with probability equal to their value (a 13-bit
// dither added to the bit pattern, then truncation toward zero).
// Round-to-nearest of slowly varying fields makes the same error every step
// and biases steady states; a dither that changes with the step does not.
// The dither of population k at a site is the top 13 bits of seed * M_k,
// where seed is a hash of the site and the step and M_k a fixed odd
// multiplier per population (multiply-shift hashing: one multiply per store).
// Other storage types store as st_dev.
__host__ __device__ __forceinline__ uint32_t sr_dither(uint32_t seed, uint32_t k) {
  return (seed * (mix32(k + 1u) | 1u)) >> 19;
}
template <class T, class R>
__device__ __forceinline__ void st_dev_sr_s(T* p, R v, Scl<R> sc, uint32_t dither) {
  if constexpr (std::is_same<T, __half>::value) {
    const float x = float(v * sc.s);
    const uint32_t b = __float_as_uint(x) + dither;
    *p = __float2half_rz(__uint_as_float(b));
  } else {
    St<T>::st(p, v);
  }
}
template <class T, class R>
__device__ __forceinline__ void st_dev_sr(T* p, R v, const PhysT<R>& P, uint32_t dither) {
  st_dev_sr_s<T, R>(p, v, scl_of(P), dither);
}

// The forcing density is stored component-fastest, rho[cell * S + m], so that
// one vector load brings every component of a neighbour.
template <int S, class RT, class R>
__device__ __forceinline__ void rho_at(const RT* rho, unsigned cell, R v[S]) {
  if constexpr (S == 2 && std::is_same<RT, double>::value) {
    const double2 t = __ldg(reinterpret_cast<const double2*>(rho) + cell);
    v[0] = R(t.x);
    v[1] = R(t.y);
  } else if constexpr (S == 2 && std::is_same<RT, float>::value) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(rho) + cell);
    v[0] = R(t.x);
    v[1] = R(t.y);
  } else {
#pragma unroll
    for (int m = 0; m < S; ++m) v[m] = R(__ldg(rho + (size_t)cell * S + m));
  }
}

// --------------------------------------------------------------- geometry
// Neighbourhood of one site within RCH lattice units.  The linear index of
// (x+dx, y+dy, z+dz) is ox[dx] + oy[dy] + oz[dz] (32-bit: tx_create checks
// N < 2^31); bit d+RCH of in_a is clear when coordinate a + d leaves a
// non-periodic axis (the ghost walls of WallsSetGhostNodesD3/D2,
// lbm_walls.F90:179-231).  Periodic extents are >= 3 >= RCH, so one wrap
// suffices; offsets past a non-periodic face are clamped into the lattice so
// that every index stays a valid address.
template <int D, int RCH>
struct Hood {
  static constexpr int RZ = D == 3 ? RCH : 0;
  int ox[2 * RCH + 1], oy[2 * RCH + 1], oz[2 * RZ + 1];
  unsigned in_x, in_y, in_z;

  // coordinate c + d of a site coordinate c in [0, n): wrapped on a periodic
  // axis (n >= 3 >= |d| there), clamped into the lattice otherwise (then the
  // in-bit is clear and the value only keeps addresses valid)
  template <int d, int B>
  __device__ static __forceinline__ int wrap(int c, int n, int per, unsigned& in) {
    constexpr unsigned bit = 1u << B;  // in-bit of offset d
    if constexpr (d == 0) {
      in |= bit;
      return c;
    } else if constexpr (d > 0) {
      const int w = c + d;
      const bool out = w >= n;
      in |= (!out || per) ? bit : 0u;
      return out ? (per ? w - n : n - 1) : w;
    } else {
      const int w = c + d;
      const bool out = w < 0;
      in |= (!out || per) ? bit : 0u;
      return out ? (per ? w + n : 0) : w;
    }
  }
  template <int i>
  __device__ __forceinline__ void fill(const Geo& g, int x, int y, int z) {
    if constexpr (i < 2 * RCH + 1) {
      ox[i] = wrap<i - RCH, i>(x, g.nx, g.per[0], in_x);
      oy[i] = g.nx * wrap<i - RCH, i>(y, g.ny, g.per[1], in_y);
      if constexpr (i < 2 * RZ + 1) oz[i] = g.nx * g.ny * wrap<i - RZ, i>(z, g.nz, g.per[2], in_z);
      fill<i + 1>(g, x, y, z);
    }
  }
  __device__ __forceinline__ Hood(const Geo& g, int x, int y, int z) {
    in_x = in_y = in_z = 0u;
    fill<0>(g, x, y, z);
  }
  template <int dx, int dy, int dz>
  __device__ __forceinline__ unsigned at() const {
    static_assert(dx >= -RCH && dx <= RCH && dy >= -RCH && dy <= RCH && dz >= -RZ && dz <= RZ, "offset beyond reach");
    return (unsigned)(ox[dx + RCH] + oy[dy + RCH] + oz[dz + RZ]);
  }
  template <int dx, int dy, int dz>
  __device__ __forceinline__ bool inside() const {
    return ((in_x >> (dx + RCH)) & (in_y >> (dy + RCH)) & (in_z >> (dz + RZ)) & 1u) != 0u;
  }
};

// Link mask of a site (k_links): bit 0 set when the site is pore space, bit n
// (1..Q-1) when x + c_n is a pore site inside the lattice or across a
// periodic face.  Push streaming, bounceback and the nearest-neighbour
// stencil terms read it instead of the wall mask.
template <int D>
__host__ __device__ constexpr int link_of(int ex, int ey, int ez) {
  int r = -1;
  for (int n = 1; n < Lat<D>::Q; ++n)
    if (Lat<D>::c(n, 0) == ex && Lat<D>::c(n, 1) == ey && (D == 3 ? Lat<D>::c(n, 2) : 0) == ez) r = n;
  return r;
}

template <int D>
__host__ __device__ constexpr uint32_t all_links() {
  return ((1u << Lat<D>::Q) - 1u) & ~1u;
}

// Link-mask bits above the links: every site of the box of reach 2 (3)
// around the site is pore space inside the lattice or across a periodic face,
// so that the isotropy-8 (-10) gradient stencil sees only pore neighbours.
constexpr uint32_t kBoxPore2 = 1u << 31;
constexpr uint32_t kBoxPore3 = 1u << 30;

// pore test of the site at offset (dx, dy, dz): a link bit for lattice links,
// the wall mask for the longer stencil offsets
template <int D, int RCH, int dx, int dy, int dz>
__device__ __forceinline__ bool pore_at(const Hood<D, RCH>& h, uint32_t links, const uint8_t* mask) {
  constexpr int n = link_of<D>(dx, dy, dz);
  if constexpr (n > 0) {
    return ((links >> n) & 1u) != 0u;
  } else {
    const bool in = h.template inside<dx, dy, dz>();
    const bool pore = __ldg(mask + h.template at<dx, dy, dz>()) == 0;
    return in & pore;
  }
}

// Site of this thread in a (x-tile, y-tile, z) launch grid; false when outside.
__device__ __forceinline__ bool site_of(const Geo& g, int& x, int& y, int& z, long long& idx) {
  x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  z = (int)blockIdx.z;
  if (x >= g.nx || y >= g.ny || z >= g.nz) return false;
  idx = (long long)x + (long long)g.nx * ((long long)y + (long long)g.ny * (long long)z);
  return true;
}

__device__ __forceinline__ bool on_face(const Geo& g, int f, int x, int y, int z) {
  const int a = f >> 1;
  const int c = a == 0 ? x : (a == 1 ? y : z);
  const int n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
  return (f & 1) ? c == n - 1 : c == 0;
}

// bit f set <=> face f re-sums its node densities (constant-index reads only)
__device__ __forceinline__ unsigned face_bits(const Faces& fc) {
  return (fc.on[0] ? 1u : 0u) | (fc.on[1] ? 2u : 0u) | (fc.on[2] ? 4u : 0u) | (fc.on[3] ? 8u : 0u) |
         (fc.on[4] ? 16u : 0u) | (fc.on[5] ? 32u : 0u);
}
// bit f set <=> face f is of the Dirichlet class
__device__ __forceinline__ unsigned dir_bits(const Faces& fc) {
  return (fc.dir[0] ? 1u : 0u) | (fc.dir[1] ? 2u : 0u) | (fc.dir[2] ? 4u : 0u) | (fc.dir[3] ? 8u : 0u) |
         (fc.dir[4] ? 16u : 0u) | (fc.dir[5] ? 32u : 0u);
}
// bit f set <=> face f carries a node correction of some class
__device__ __forceinline__ unsigned active_bits(const Faces& fc) {
  unsigned b = 0u;
#pragma unroll
  for (int f = 0; f < 6; ++f) b |= fc.cls[f] != kClsNone ? (1u << f) : 0u;
  return b;
}

// bit f set <=> (x, y, z) lies on face f
__device__ __forceinline__ unsigned site_faces(const Geo& g, int x, int y, int z) {
  return (x == 0 ? 1u : 0u) | (x == g.nx - 1 ? 2u : 0u) | (y == 0 ? 4u : 0u) | (y == g.ny - 1 ? 8u : 0u) |
         (z == 0 ? 16u : 0u) | (z == g.nz - 1 ? 32u : 0u);
}

template <int D>
__device__ __forceinline__ long long face_node(const Geo& g, int f, int x, int y, int z) {
  const int a = f >> 1;
  if (D == 2) return a == 0 ? y : x;
  if (a == 0) return y + (long long)g.ny * z;
  if (a == 1) return x + (long long)g.nx * z;
  return x + (long long)g.nx * y;
}

template <int D>
__device__ __forceinline__ long long face_area(const Geo& g, int f) {
  const int a = f >> 1;
  if (D == 2) return a == 0 ? g.ny : g.nx;
  if (a == 0) return (long long)g.ny * g.nz;
  if (a == 1) return (long long)g.nx * g.nz;
  return (long long)g.nx * g.ny;
}

template <int D>
__device__ __forceinline__ bool any_dirichlet(const Geo& g, const Faces& fc, int x, int y, int z) {
  const unsigned keep = D == 3 ? 63u : 15u;
  return (face_bits(fc) & site_faces(g, x, y, z) & keep) != 0u;
}

template <int D>
__host__ __device__ constexpr FFTerm ffterm(int t) {
  return D == 3 ? ff_d3(t) : ff_d2(t);
}

// the stencil term with the opposite offset, weight and level (-1: none)
template <int D>
__host__ __device__ constexpr int ff_opp(int t) {
  const FFTerm a = ffterm<D>(t);
  const int nt = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  for (int u = 0; u < nt; ++u) {
    const FFTerm b = ffterm<D>(u);
    if (b.e[0] == -a.e[0] && b.e[1] == -a.e[1] && b.e[2] == -a.e[2] && b.w == a.w && b.level == a.level) return u;
  }
  return -1;
}

template <int D, int ISO>
__host__ __device__ constexpr bool stencil_symmetric() {
  const int nt = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  for (int t = 0; t < nt; ++t)
    if (ffterm<D>(t).level <= ISO && ff_opp<D>(t) < 0) return false;
  return true;
}

// Reach of the isotropy-ISO gradient stencil (at least one lattice link).
template <int D, int ISO>
__host__ __device__ constexpr int stencil_reach() {
  int r = 1;
  const int nt = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  for (int t = 0; t < nt; ++t) {
    const FFTerm T = ffterm<D>(t);
    if (T.level > ISO) continue;
    for (int d = 0; d < 3; ++d) {
      const int e = T.e[d] < 0 ? -T.e[d] : T.e[d];
      r = e > r ? e : r;
      for (int k = 0; k < T.naux; ++k) {
        const int q = T.aux[k][d] < 0 ? -T.aux[k][d] : T.aux[k][d];
        r = q > r ? q : r;
      }
    }
  }
  return r;
}

// True when every term of the isotropy-ISO stencil is a plain lattice link
// (isotropy 4): the link mask then decides all of them.
template <int D, int ISO>
__host__ __device__ constexpr bool stencil_is_links() {
  const int nt = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  for (int t = 0; t < nt; ++t) {
    const FFTerm T = ffterm<D>(t);
    if (T.level > ISO) continue;
    if (T.naux > 0 || link_of<D>(T.e[0], T.e[1], T.e[2]) < 0) return false;
  }
  return true;
}

// Weight sum of axis d of the isotropy-ISO stencil with every neighbour pore.
template <int D>
inline double full_weight_sum(int iso, const double ffw[12], int d) {
  const int nt = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
  double ws = 0.0;
  for (int t = 0; t < nt; ++t) {
    const FFTerm T = ffterm<D>(t);
    if (T.level <= iso) ws += ffw[T.w] * (double)(T.e[d] * T.e[d]);
  }
  return ws;
}

// One term of the wall-aware psi gradient: the neighbour x + e must be pore
// space and, for long links, the path cells must satisfy the term's truth
// table.  EXACT sums the normalising weights in the reference's order; the
// fast form counts them per weight class and multiplies once (wc).
template <int D, int S, int ISO, bool EXACT, int TI, int RCH, class R, class RT>
__device__ __forceinline__ void ff_term(const Hood<D, RCH>& h, uint32_t links, const PhysT<R>& P, const uint8_t* mask,
                                        const RT* rho, long long N, const R rfd[S], R gr[S][D], R ws[D], int wc[12][D]) {
  constexpr FFTerm T = ffterm<D>(TI);
  if constexpr (T.level <= ISO) {
    constexpr int ex = T.e[0], ey = T.e[1], ez = T.e[2];
    bool ok = pore_at<D, RCH, ex, ey, ez>(h, links, mask);
    if constexpr (T.naux > 0) {
      unsigned bits = 0;
      if constexpr (T.naux > 0) bits |= pore_at<D, RCH, T.aux[0][0], T.aux[0][1], T.aux[0][2]>(h, links, mask) ? 1u : 0u;
      if constexpr (T.naux > 1) bits |= pore_at<D, RCH, T.aux[1][0], T.aux[1][1], T.aux[1][2]>(h, links, mask) ? 2u : 0u;
      if constexpr (T.naux > 2) bits |= pore_at<D, RCH, T.aux[2][0], T.aux[2][1], T.aux[2][2]>(h, links, mask) ? 4u : 0u;
      if constexpr (T.naux > 3) bits |= pore_at<D, RCH, T.aux[3][0], T.aux[3][1], T.aux[3][2]>(h, links, mask) ? 8u : 0u;
      ok = ok && ((T.truth >> bits) & 1u);
    }
    if (ok) {
      constexpr int tw = T.w;
      const unsigned pi = h.template at<ex, ey, ez>();
      R dif[S];
      rho_at<S>(rho, pi, dif);
#pragma unroll
      for (int m = 0; m < S; ++m) dif[m] = dif[m] - rfd[m];
      sfor<0, D>([&](auto dd) {
        constexpr int d = decltype(dd)::value;
        constexpr int e = d == 0 ? ex : (d == 1 ? ey : ez);
        if constexpr (e != 0) {
          const R coef = R(e) * P.ffw[tw];
#pragma unroll
          for (int m = 0; m < S; ++m) gr[m][d] = gr[m][d] + coef * dif[m];
          if constexpr (EXACT)
            ws[d] = ws[d] + P.ffw[tw] * R(e * e);
          else
            wc[tw][d] += e * e;
        }
      });
    }
  }
}

// ------------------------------------------------------------------ forces
// FlowCalcForces (lbm_flow.F90:760-808) for one pore site: zero, then
// fluid-solid (lbm_forcing.F90:1326-1421), body (:1440-1496) and the
// wall-aware Shan-Chen term (:51-958 / :960-1299), in that order.
// rfd: stored forcing density of the site (rho - rho0); rf: rho itself;
// psi: the psi(rho) field when the EOS is on (then the fluid-fluid force
// differentiates psi and scales by psi(x), FlowCalcForces lbm_flow.F90:790-806).
// BULK_ONLY: the caller guarantees that every stencil neighbour is pore
// whenever the fluid-fluid force is on (the general wall-aware gradient is
// then not compiled in).
// FF = false: fluid-solid and body forces only (the caller adds the
// fluid-fluid force).
template <int D, int S, int ISO, bool EXACT, int RCH, class R, class RT, bool BULK_ONLY = false, bool FF = true>
__device__ __forceinline__ void cell_forces(const Hood<D, RCH>& h, uint32_t links, const PhysT<R>& P,
                                            const uint8_t* mask, const RT* rho, const RT* psi, long long N,
                                            const R rfd[S], const R rf[S], R F[S][D]) {
  using L = Lat<D>;
#pragma unroll
  for (int m = 0; m < S; ++m)
#pragma unroll
    for (int d = 0; d < D; ++d) F[m][d] = EXACT ? R(0) : R(-0.0);

  // only links that end on a wall can carry a fluid-solid force
  const uint32_t walled = ~links & all_links<D>();
  if (P.fs_on && walled) {
    sfor<1, L::Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      constexpr int cx = L::c(n, 0), cy = L::c(n, 1), cz = D == 3 ? L::c(n, 2) : 0;
      if ((walled >> n) & 1u) {
        const int mk = h.template inside<cx, cy, cz>() ? (int)__ldg(mask + h.template at<cx, cy, cz>()) : 255;
        if (mk >= 1 && mk <= MAXMIN) {
          const R wgt = R(n <= L::NAXIS ? P.fs_w_axis : P.fs_w_diag);
          sfor<0, D>([&](auto dd) {
            constexpr int d = decltype(dd)::value;
            constexpr int c = L::c(n, d);
            if constexpr (c != 0) {
#pragma unroll
              for (int m = 0; m < S; ++m) {
                const R t = wgt * rf[m] * R(P.gw[mk][m]);
                F[m][d] = c > 0 ? F[m][d] - t : F[m][d] + t;
              }
            }
          });
        }
      }
    });
  }
  if (P.body_on) {
#pragma unroll
    for (int m = 0; m < S; ++m)
#pragma unroll
      for (int d = 0; d < D; ++d) F[m][d] = F[m][d] + R(P.gvt[d]) * R(P.mm[m]) * rf[m];
  }
  if (!FF || !P.ff_on) return;
  // the differentiated field, its value at x and the force's scale factor
  const RT* src = P.eos_on ? psi : rho;
  R selfv[S], mult[S];
  if (P.eos_on) {
    rho_at<S>(psi, h.template at<0, 0, 0>(), selfv);
#pragma unroll
    for (int m = 0; m < S; ++m) mult[m] = selfv[m];
  } else {
#pragma unroll
    for (int m = 0; m < S; ++m) {
      selfv[m] = rfd[m];
      mult[m] = rf[m];
    }
  }
  if constexpr (!EXACT) {
    // every stencil neighbour pore: the weight sums are constant and the
    // psi(x) terms cancel, so grad = sum_k w_k e_k psi(x + e_k)
    constexpr int RB = stencil_reach<D, ISO>();
    const bool bulk = stencil_is_links<D, ISO>() ? ((links | 1u) & (all_links<D>() | 1u)) == (all_links<D>() | 1u)
                      : RB == 2                ? (links & kBoxPore2) != 0u
                                               : (links & kBoxPore3) != 0u;
    if (bulk) {
      // opposite stencil terms pair up: w e (psi(x + e) - psi(x - e))
      static_assert(stencil_symmetric<D, ISO>(), "every stencil term needs its opposite");
      R gr[S][D];
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int m = 0; m < S; ++m) gr[m][d] = R(-0.0);
      constexpr int NT = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
      sfor<0, NT>([&](auto tt) {
        constexpr int t = decltype(tt)::value;
        constexpr FFTerm T = ffterm<D>(t);
        if constexpr (T.level <= ISO && t < ff_opp<D>(t)) {
          constexpr int ex = T.e[0], ey = T.e[1], ez = T.e[2], tw = T.w;
          R vp[S], vm[S];
          rho_at<S>(src, h.template at<ex, ey, ez>(), vp);
          rho_at<S>(src, h.template at<-ex, -ey, -ez>(), vm);
          R dv[S];
#pragma unroll
          for (int m = 0; m < S; ++m) dv[m] = vp[m] - vm[m];
          sfor<0, D>([&](auto dd) {
            constexpr int d = decltype(dd)::value;
            constexpr int e = d == 0 ? ex : (d == 1 ? ey : ez);
            if constexpr (e != 0) {
              const R coef = R(e) * P.ffwq[d][tw];
#pragma unroll
              for (int m = 0; m < S; ++m) gr[m][d] = gr[m][d] + coef * dv[m];
            }
          });
        }
      });
      // F -= psi(x) c0 sum_k g_mk grad_k (the weight sum is folded into ffwq);
      // with two components coupled only to each other, the one cross term
      if (S == 2 && std::is_same<R, double>::value && P.ff_cross) {
#pragma unroll
        for (int m = 0; m < S; ++m) {
          const R fac = mult[m] * P.c0g[m][S - 1 - m];
#pragma unroll
          for (int d = 0; d < D; ++d) F[m][d] = F[m][d] - fac * gr[S - 1 - m][d];
        }
        return;
      }
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int m = 0; m < S; ++m) {
          R acc = R(-0.0);
#pragma unroll
          for (int k = 0; k < S; ++k) acc = acc + P.c0g[m][k] * gr[k][d];
          F[m][d] = F[m][d] - mult[m] * acc;
        }
      return;
    }
  }
  if constexpr (BULK_ONLY) return;
  {
    R gr[S][D];
    R ws[D];
    int wc[12][D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ws[d] = R(0);
#pragma unroll
      for (int w = 0; w < 12; ++w) wc[w][d] = 0;
#pragma unroll
      for (int m = 0; m < S; ++m) gr[m][d] = R(0);
    }
    constexpr int NT = D == 3 ? FF_D3_COUNT : FF_D2_COUNT;
    sfor<0, NT>([&](auto tt) {
      ff_term<D, S, ISO, EXACT, decltype(tt)::value, RCH, R, RT>(h, links, P, mask, src, N, selfv, gr, ws, wc);
    });
    if constexpr (!EXACT) {
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int w = 1; w < 12; ++w) ws[d] = ws[d] + P.ffw[w] * R(wc[w][d]);
    }
    const R eps = R((double)1.e-12f);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (ws[d] > eps) {
        R q[S];
        if constexpr (EXACT) {
#pragma unroll
          for (int m = 0; m < S; ++m) q[m] = gr[m][d] / ws[d];
        } else {
          const R inv = R(1) / ws[d];
#pragma unroll
          for (int m = 0; m < S; ++m) q[m] = gr[m][d] * inv;
        }
#pragma unroll
        for (int m = 0; m < S; ++m) {
          R acc = R(0);
#pragma unroll
          for (int k = 0; k < S; ++k) acc = acc + R(P.g[m][k]) * q[k];
          F[m][d] = F[m][d] - R(P.c0) * mult[m] * acc;
        }
      }
    }
  }
}

// Load the site's population deviations f - w_n rho0 (f itself in the FP64 form).
template <int D, int S, class T, class R>
__device__ __forceinline__ void load_pops(const T* f, long long N, unsigned c, const PhysT<R>& P,
                                          R fv[S][Lat<D>::Q]) {
  using L = Lat<D>;
#pragma unroll
  for (int m = 0; m < S; ++m)
    sfor<0, L::Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      fv[m][n] = ld_dev<T, R>(f + ((long long)(m * L::Q + n)) * N + c, P);
    });
}

template <int D, int S, class R>
__device__ __forceinline__ R pop_sum(const R fv[S][Lat<D>::Q], int m) {
  R acc = R(0);
  sfor<0, Lat<D>::Q>([&](auto nn) { acc = acc + fv[m][decltype(nn)::value]; });
  return acc;
}

// sum_n f c_n,d in direction order (DistributionCalcFluxD3/D2,
// lbm_distribution_function.F90:451-508); zero terms add nothing
template <int D, int S, class R>
__device__ __forceinline__ R pop_flux(const R fv[S][Lat<D>::Q], int m, int d0) {
  R acc = R(0);
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    if (d == d0) {
      sfor<0, Lat<D>::Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        constexpr int c = Lat<D>::c(n, d);
        if constexpr (c > 0) acc = acc + fv[m][n];
        if constexpr (c < 0) acc = acc - fv[m][n];
      });
    }
  });
  return acc;
}

// c_n . v over the nonzero components of c_n.  Sums start from -0.0, which
// x + -0.0 = x for every x lets the compiler drop: the fast forms use these.
template <int D, int n, class R>
__device__ __forceinline__ R cdot_z(const R v[D]) {
  R acc = R(-0.0);
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    constexpr int c = Lat<D>::c(n, d);
    if constexpr (c > 0) acc = acc + v[d];
    if constexpr (c < 0) acc = acc - v[d];
  });
  return acc;
}

// The bilinear form stress_coef(k, ., .) of s_nu moment k at (a, b); the two
// off-diagonal terms of a symmetric coefficient share one multiplication.
template <int D, int k, class R>
__device__ __forceinline__ R stress_form(const R a[D], const R b[D]) {
  R acc = R(-0.0);
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    sfor<d, D>([&](auto ee) {
      constexpr int e = decltype(ee)::value;
      constexpr double Cde = stress_coef<D>(k, d, e), Ced = stress_coef<D>(k, e, d);
      if constexpr (d == e) {
        if constexpr (Cde != 0.0) acc = acc + R(Cde) * (a[d] * b[d]);
      } else if constexpr (Cde == Ced) {
        if constexpr (Cde != 0.0) acc = acc + R(Cde) * (a[d] * b[e] + a[e] * b[d]);
      } else {
        if constexpr (Cde != 0.0) acc = acc + R(Cde) * (a[d] * b[e]);
        if constexpr (Ced != 0.0) acc = acc + R(Ced) * (a[e] * b[d]);
      }
    });
  });
  return acc;
}

// sum_p c_n,d v_p over the direction pairs (v_p = f_n - f_opp(n) gives the flux)
template <int D, class R>
__device__ __forceinline__ void pair_axis_sums(const R v[npairs<D>()], R j[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) j[d] = R(-0.0);
  sfor<0, npairs<D>()>([&](auto pp) {
    constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
    sfor<0, D>([&](auto dd) {
      constexpr int d = decltype(dd)::value;
      constexpr int c = Lat<D>::c(n, d);
      if constexpr (c == 1) j[d] = j[d] + v[p];
      if constexpr (c == -1) j[d] = j[d] - v[p];
    });
  });
}

// The pair (index p of pair_n) of direction n, and the axis pairs (a, b) of
// the diagonal directions: ab 0 = (x, y), 1 = (x, z), 2 = (y, z).
template <int D>
__host__ __device__ constexpr int pair_of(int n) {
  for (int p = 0; p < npairs<D>(); ++p)
    if (pair_n<D>(p) == n || opp<D>(pair_n<D>(p)) == n) return p;
  return -1;
}
__host__ __device__ constexpr int ab_a(int ab) { return ab == 2 ? 1 : 0; }
__host__ __device__ constexpr int ab_b(int ab) { return ab == 0 ? 1 : 2; }
template <int D>
__host__ __device__ constexpr int n_ab() { return D == 3 ? 3 : 1; }

// sum over the s_nu moments k of coef(k) ck[k], coef a compile-time function
// of k given by CF::at (zero and unit coefficients cost nothing).
template <int D, class CF, class R>
__device__ __forceinline__ R snu_lincomb(const R ck[Lat<D>::Q]) {
  R acc = R(-0.0);
  sfor<0, Lat<D>::Q>([&](auto kk) {
    constexpr int k = decltype(kk)::value;
    if constexpr (rate_of<D>(k) == R_NU) {
      constexpr double c = CF::at(k);
      if constexpr (c == 1.0) acc = acc + ck[k];
      else if constexpr (c == -1.0) acc = acc - ck[k];
      else if constexpr (c != 0.0) acc = acc + R(c) * ck[k];
    }
  });
  return acc;
}
template <int D, int d>
struct SnuAxis {  // B_k(d, d): the correction of the axis pair along d
  static constexpr double at(int k) { return stress_b<D>(k, d, d); }
};
template <int D, int ab>
struct SnuDiagSum {  // B_k(a, a) + B_k(b, b)
  static constexpr double at(int k) { return stress_b<D>(k, ab_a(ab), ab_a(ab)) + stress_b<D>(k, ab_b(ab), ab_b(ab)); }
};
template <int D, int ab>
struct SnuDiagOff {  // 2 B_k(a, b)
  static constexpr double at(int k) { return 2.0 * stress_b<D>(k, ab_a(ab), ab_b(ab)); }
};

// Fast-form flux of one component from pair differences f_n - f_opp(n).
template <int D, class R>
__device__ __forceinline__ void pop_flux_pairs(const R f[Lat<D>::Q], R j[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) j[d] = R(-0.0);
  sfor<0, npairs<D>()>([&](auto pp) {
    constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
    const R dlt = f[n] - f[nb];
    sfor<0, D>([&](auto dd) {
      constexpr int d = decltype(dd)::value;
      constexpr int c = Lat<D>::c(n, d);
      if constexpr (c == 1) j[d] = j[d] + dlt;
      if constexpr (c == -1) j[d] = j[d] - dlt;
      if constexpr (c > 1 || c < -1) j[d] = j[d] + R(c) * dlt;
    });
  });
}

// Density of the collision (Dirichlet nodes re-summed as in BCUpdateRho,
// lbm_bc.F90:436-611) and the common velocity of FlowUpdateUED3/D2
// (lbm_flow.F90:494-574) from the post-stream population deviations and the forces.
template <int D, int S, bool EXACT, class R>
__device__ __forceinline__ void cell_velocity(const StepArgs& a, const PhysT<R>& P, int x, int y, int z,
                                              const R fv[S][Lat<D>::Q], const R rf[S], const R F[S][D], R rc[S],
                                              R up[D]) {
  const bool dn = any_dirichlet<D>(a.g, a.faces, x, y, z);
#pragma unroll
  for (int m = 0; m < S; ++m) rc[m] = dn ? P.rho0[m] + pop_sum<D, S, R>(fv, m) : rf[m];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    R num = R(0), den = R(0);
#pragma unroll
    for (int m = 0; m < S; ++m) {
      const R ue = pop_flux<D, S, R>(fv, m, d) + R(.5) * F[m][d];
      num = num + ue * R(P.mmot[m]);
    }
#pragma unroll
    for (int m = 0; m < S; ++m) den = den + rc[m] * R(P.mmot[m]);
    if constexpr (EXACT)
      up[d] = num / den;
    else
      up[d] = num * (R(1) / den);
  }
}

// Moments of a pore site from its post-stream populations: forces from the
// forcing density, then cell_velocity.
template <int D, int S, int ISO, bool EXACT, class R, class RT>
__device__ __forceinline__ void cell_moments(const StepArgs& a, const PhysT<R>& P, int x, int y, int z, long long idx,
                                             const R fv[S][Lat<D>::Q], R rc[S], R rf[S], R F[S][D], R up[D]) {
  const RT* rho = reinterpret_cast<const RT*>(a.rho);
  R rfd[S];
  rho_at<S>(rho, (unsigned)idx, rfd);
#pragma unroll
  for (int m = 0; m < S; ++m) rf[m] = P.rho0[m] + rfd[m];
  const Hood<D, stencil_reach<D, ISO>()> h(a.g, x, y, z);
  cell_forces<D, S, ISO, EXACT>(h, __ldg(a.links + idx), P, a.mask, rho, reinterpret_cast<const RT*>(a.psi), a.g.n,
                                rfd, rf, F);
  cell_velocity<D, S, EXACT, R>(a, P, x, y, z, fv, rf, F, rc, up);
}

// Equilibrium (DiscretizationEquilf_D3Q19, lbm_discretization_d3q19.F90:265-305;
// _D2Q9, lbm_discretization_d2q9.F90:168-205) and forcing prefactor
// (FlowFiBarEqPrefactor, lbm_flow.F90:836-851) of component m, direction n.
template <int D, int n, bool EXACT, class R>
__device__ __forceinline__ void feq_pf(const PhysT<R>& P, int m, R r, const R u[D], R usqr, const R Fm[D], R& feq, R& pf) {
  using L = Lat<D>;
  const R cs2 = R(P.cs2[m]), dk = R(P.dk[m]);
  R udote = R(0);
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    constexpr int c = L::c(n, d);
    if constexpr (c > 0) udote = udote + u[d];
    if constexpr (c < 0) udote = udote - u[d];
  });
  if constexpr (n == 0) {
    if constexpr (D == 3)
      feq = r * (dk - usqr / R(2.));
    else
      feq = r * ((R(1.) + dk * R(5.)) / R(6.) - R(2.) * usqr / R(3.));
  } else if constexpr (EXACT) {
    feq = R(L::w(n)) * r *
          (R(1.5) * (R(1.) - dk) + udote / cs2 + udote * udote / (R(2.) * cs2 * cs2) - usqr / (R(2.) * cs2));
  } else {
    const R ic = R(P.inv_cs2[m]);
    feq = R(L::w(n)) * r * (R(1.5) * (R(1.) - dk) + udote * ic + R(0.5) * udote * udote * ic * ic - R(0.5) * usqr * ic);
  }
  R acc = R(0);
  sfor<0, D>([&](auto dd) {
    constexpr int d = decltype(dd)::value;
    acc = acc + Fm[d] * (R(L::c(n, d)) - u[d]);
  });
  if constexpr (EXACT)
    pf = acc / (r * cs2);
  else
    pf = acc * (R(1) / (r * cs2));
}

// ------------------------------------------------------------------ step
// One pore site of the step: forces, moments, collision, push.  The kernels
// copy their StepArgs parameter into a local and pass references to that copy.
template <int D, int S, int ISO, bool MRT, bool EXACT, class T, class R, class RT>
__device__ __forceinline__ void step_site(const StepArgs& a, int x, int y, int z) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * (long long)z);
  const unsigned c = (unsigned)idx;  // N < 2^31
  const uint32_t links = __ldg(a.links + c);
  if (!(links & 1u)) return;  // wall site
  const long long N = a.g.n;
  const Hood<D, stencil_reach<D, ISO>()> h(a.g, x, y, z);
  const Scl<R> sc = scl_of(P);
  // stochastic-rounding seed of this site and step (FP16 storage only)
  uint32_t sr_seed = 0;
  if constexpr (std::is_same<T, __half>::value)
    sr_seed = mix32(c ^ (0x9E3779B9u * ((a.steps_ptr ? __ldg(a.steps_ptr) : a.step) + 1u)));

  // forces first (they need only rho and the wall layout)
  R rfd[S], rf[S], F[S][D];
  {
    const RT* rho = reinterpret_cast<const RT*>(a.rho);
    rho_at<S>(rho, c, rfd);
#pragma unroll
    for (int m = 0; m < S; ++m) rf[m] = P.rho0[m] + rfd[m];
    cell_forces<D, S, ISO, EXACT>(h, links, P, a.mask, rho, reinterpret_cast<const RT*>(a.psi), N, rfd, rf, F);
  }
  const T* fin = reinterpret_cast<const T*>(a.fin);
  // moments pass, one component's populations at a time; rcd = rc - rho0
  R rc[S], rcd[S], up[D];
  {
    const bool dn = any_dirichlet<D>(a.g, a.faces, x, y, z);
    R jm[S][D];
    // FP64 fast form with every component's mm s_c equal (P.mmot_shared): that
    // factor cancels from the common velocity, u = (sum_m j_m + F_m / 2) / sum_m rho_m,
    // and the components' pair differences are summed before the axis sums
    constexpr bool kShare = !EXACT && !kShifted<T>;
    const bool share = kShare && P.mmot_shared;
    R jp[npairs<D>()];
#pragma unroll
    for (int m = 0; m < S; ++m) {
      R f1[1][Q];
      sfor<0, Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        f1[0][n] = ld_dev_s<T, R>(fin + ((long long)(m * Q + n)) * N + c, sc);
      });
      if constexpr (EXACT) {
#pragma unroll
        for (int d = 0; d < D; ++d) jm[m][d] = pop_flux<D, 1, R>(f1, 0, d);
      } else if constexpr (kShare) {
        if (share) {
          sfor<0, npairs<D>()>([&](auto pp) {
            constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
            const R dlt = f1[0][n] - f1[0][nb];
            jp[p] = m == 0 ? dlt : jp[p] + dlt;
          });
        } else {
          pop_flux_pairs<D, R>(f1[0], jm[m]);
        }
      } else {
        pop_flux_pairs<D, R>(f1[0], jm[m]);
      }
      rcd[m] = dn ? pop_sum<D, 1, R>(f1, 0) : rfd[m];
      rc[m] = dn ? P.rho0[m] + rcd[m] : rf[m];
    }
    if (share) {
      R den = R(-0.0), J[D];
#pragma unroll
      for (int m = 0; m < S; ++m) den = den + rc[m];
      const R inv = rcp_rn(den);
      pair_axis_sums<D, R>(jp, J);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        R Fs = R(-0.0);
#pragma unroll
        for (int m = 0; m < S; ++m) Fs = Fs + F[m][d];
        up[d] = (J[d] + R(.5) * Fs) * inv;
      }
    } else {
    R den = EXACT ? R(0) : R(-0.0);
#pragma unroll
    for (int m = 0; m < S; ++m) den = den + rc[m] * R(P.mmot[m]);
    const R inv = EXACT ? R(0) : rcp_rn(den);  // fast form: one correctly rounded reciprocal
#pragma unroll
    for (int d = 0; d < D; ++d) {
      R num = EXACT ? R(0) : R(-0.0);
#pragma unroll
      for (int m = 0; m < S; ++m) num = num + (jm[m][d] + R(.5) * F[m][d]) * R(P.mmot[m]);
      if constexpr (EXACT)
        up[d] = num / den;
      else
        up[d] = num * inv;
    }
    }
  }
  R usqr = EXACT ? R(0) : R(-0.0);
#pragma unroll
  for (int d = 0; d < D; ++d) usqr = usqr + up[d] * up[d];

  T* fout = reinterpret_cast<T*>(a.fout);
  // push (DistributionStreamD3/D2 + DistributionBouncebackD3/D2): to x + c_n,
  // or back to x as opp(n) when link n ends on a wall
  auto push = [&](auto nn, int m, R v) {
    constexpr int n = decltype(nn)::value;
    constexpr int o = opp<D>(n);
    T* dst;
    if constexpr (n == 0) {
      dst = fout + (long long)(m * Q) * N + c;
    } else {
      constexpr int cx = L::c(n, 0), cy = L::c(n, 1), cz = D == 3 ? L::c(n, 2) : 0;
      const bool pore = ((links >> n) & 1u) != 0u;
      T* const base = fout + (long long)(m * Q + (pore ? n : o)) * N;
      dst = base + (pore ? h.template at<cx, cy, cz>() : c);
    }
    st_dev_sr_s<T, R>(dst, v, sc, sr_dither(sr_seed, (uint32_t)(m * Q + n)));
  };

  if constexpr (EXACT) {
  #pragma unroll
    for (int m = 0; m < S; ++m) {
      R f[Q];
      {
        R fv1[1][Q];
        load_pops<D, 1, T, R>(fin + (long long)m * Q * N, N, c, P, fv1);
  #pragma unroll
        for (int n = 0; n < Q; ++n) f[n] = fv1[0][n];
      }
      if constexpr (!MRT) {
        // RelaxationCollideSRT (lbm_relaxation.F90:171-180) then f += P feq, one direction at a time
        sfor<0, Q>([&](auto nn) {
          constexpr int n = decltype(nn)::value;
          R feq, pf;
          feq_pf<D, n, EXACT, R>(P, m, rc[m], up, usqr, F[m], feq, pf);
          const R fb = (R(1.) - R(.5) * pf) * feq;
          const R v = f[n] - (f[n] - fb) / R(P.tau[m]);
          push(nn, m, v + pf * feq);
        });
      } else {
        // RelaxationCollideMRT (lbm_relaxation.F90:182-200): coef_k from the
        // pre-collision differences, then each f_i subtracts coef_k mt(i,k) in k order
        R dfi[Q], pfeq[Q];
        sfor<0, Q>([&](auto nn) {
          constexpr int n = decltype(nn)::value;
          R feq, pf;
          feq_pf<D, n, EXACT, R>(P, m, rc[m], up, usqr, F[m], feq, pf);
          dfi[n] = f[n] - (R(1.) - R(.5) * pf) * feq;
          pfeq[n] = pf * feq;
        });
        R coef[Q];
        sfor<0, Q>([&](auto kk) {
          constexpr int k = decltype(kk)::value;
          R md = R(0);
          sfor<0, Q>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            constexpr int v = L::mt(i, k);
            if constexpr (v == 1) md = md + dfi[i];
            else if constexpr (v == -1) md = md - dfi[i];
            else if constexpr (v != 0) md = md + R(v) * dfi[i];
          });
          coef[k] = R(P.srate[m][k]) * md / R(L::mmt(k));
        });
        sfor<0, Q>([&](auto ii) {
          constexpr int i = decltype(ii)::value;
          R v = f[i];
          sfor<0, Q>([&](auto kk) {
            constexpr int k = decltype(kk)::value;
            constexpr int c = L::mt(i, k);
            if constexpr (c == 1) v = v - coef[k];
            else if constexpr (c == -1) v = v + coef[k];
            else if constexpr (c != 0) v = v - coef[k] * R(c);
          });
          push(ii, m, v + pfeq[i]);
        });
      }
    }
  } else if constexpr (!kShifted<T>) {
    // Fast form, FP64 (plain storage), with c_s^2 = 1/3 and E_n = W~_n (A_m,n + B_n)
    // (W~_0 = 1, B_n the velocity terms):
    //   feq_n   = rho E_n
    //   P feq_n = 3 E_n (F.c_n - F.u)          (He forcing)
    //   f'_n    = (1 - s0) f_n + E_n (G + c_n.kF),  G = s0 rho - k F.u,  k = 3 - 1.5 s0,
    // i.e. f - s0 (f - feq + P feq / 2) + P feq, every moment relaxed at s0;
    // moments whose MRT rate differs from s0 are corrected afterwards.
    // Directions come in pairs (n, n~ = opp(n)); with t = c_n.u and, per
    // direction class, WAu = W~A - 1.5 w u^2,
    //   E_n = WAu + t (3w + 4.5w t),   E_n~ = WAu - t (3w - 4.5w t),
    // two FMAs each, and the pair relaxes to E_n (G + h) and E_n~ (G - h) with
    // h = c_n.kF.  E depends on the component only through W~A = w/mm (d_k at
    // rest): it is computed for the first component, and a component with
    // another molecular mass shifts it by the difference of W~A
    // (P.wa_shared: none does).
    constexpr int NP = npairs<D>();
    R En[NP], Eb[NP], E0;
    {
      E0 = P.WAc[0][0] + (D == 3 ? R(-0.5) * usqr : R(-2.0 / 3.0) * usqr);
      const R WAu1 = P.WAc[0][1] - R(1.5 * L::w(1)) * usqr, WAu2 = P.WAc[0][2] - R(1.5 * L::w(Q - 1)) * usqr;
      sfor<0, NP>([&](auto pp) {
        constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
        constexpr double w = L::w(n);
        const R t = cdot_z<D, n>(up);
        const R WAu = n <= L::NAXIS ? WAu1 : WAu2;
        En[p] = t * (R(3 * w) + R(4.5 * w) * t) + WAu;
        Eb[p] = WAu - t * (R(3 * w) - R(4.5 * w) * t);
      });
    }
#pragma unroll
    for (int m = 0; m < S; ++m) {
      if (m > 0 && !P.wa_shared) {
        const R d0 = P.WAc[m][0] - P.WAc[m - 1][0], d1 = P.WAc[m][1] - P.WAc[m - 1][1],
                d2 = P.WAc[m][2] - P.WAc[m - 1][2];
        E0 = E0 + d0;
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
          En[p] = En[p] + (n <= L::NAXIS ? d1 : d2);
          Eb[p] = Eb[p] + (n <= L::NAXIS ? d1 : d2);
        });
      }
      const R r = rc[m];
      const R s0 = P.s0[m];
      const R k = P.kfac[m];
      const R keep = P.keep[m];
      R Fu = R(-0.0), kF[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        Fu = Fu + F[m][d] * up[d];
        kF[d] = k * F[m][d];
      }
      const R G = s0 * r - k * Fu;
      const unsigned spec = P.spec_mask[m];
      const T* fm = fin + (long long)m * Q * N;
      auto pop = [&](auto nn) -> R {
        constexpr int n = decltype(nn)::value;
        return ld_dev_s<T, R>(fm + (long long)n * N + c, sc);
      };
      const R X0 = E0 * G;
      if (spec == 0u && keep == R(0)) {
        // s0 = 1 (tau = 1): the relaxed populations are the forced equilibrium
        push(std::integral_constant<int, 0>{}, m, X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          const R h = cdot_z<D, n>(kF);
          push(std::integral_constant<int, n>{}, m, En[p] * (G + h));
          push(std::integral_constant<int, nb>{}, m, Eb[p] * (G - h));
        });
      } else if (spec == 0u) {
        // every moment relaxes at s0 (BGK): one pair at a time
        push(std::integral_constant<int, 0>{}, m, keep * pop(std::integral_constant<int, 0>{}) + X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          const R h = cdot_z<D, n>(kF);
          push(std::integral_constant<int, n>{}, m, keep * pop(std::integral_constant<int, n>{}) + En[p] * (G + h));
          push(std::integral_constant<int, nb>{}, m, keep * pop(std::integral_constant<int, nb>{}) + Eb[p] * (G - h));
        });
      } else if (spec == stress_mask<D>()) {
        // s_nu != s0, every other rate s0: the corrections ck = dspec md_k come
        // from the s_nu moments md_k of the pair sums of the non-equilibrium
        // part, S_p = f_n + f_n~ - (E_n + E_n~)(r + 1.5 F.u) + (E_n - E_n~) c_n.1.5F.
        // With E_n + E_n~ = 2 WAu + 9w t^2 and E_n - E_n~ = 6w t, the class
        // constants WAu drop out of these moments (stress_class_free), so
        //   md_k = M_k(f_n + f_n~) + T_k(u, F - (r + 1.5 F.u) u),
        // T_k the bilinear form stress_coef.  Each pair is then relaxed and
        // pushed less its correction.
        R ck[Q];
        {
          R gs[NP];
          sfor<0, NP>([&](auto pp) {
            constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
            gs[p] = pop(std::integral_constant<int, n>{}) + pop(std::integral_constant<int, nb>{});
          });
          const R Xh = r + R(1.5) * Fu;
          R vF[D];
#pragma unroll
          for (int d = 0; d < D; ++d) vF[d] = F[m][d] - Xh * up[d];
          // each s_nu moment is a quadratic form B_k of c (stress_b): over the
          // axis pairs B_k(d, d), over the two diagonal pairs of axes (a, b)
          // B_k(a, a) + B_k(b, b) times their sum and 2 B_k(a, b) times their difference
          R sg[n_ab<D>()], dg[n_ab<D>()];
          sfor<0, n_ab<D>()>([&](auto ii) {
            constexpr int ab = decltype(ii)::value;
            constexpr int pp = pair_of<D>(diag_dir<D>(ab_a(ab), ab_b(ab), 1));
            constexpr int pm = pair_of<D>(diag_dir<D>(ab_a(ab), ab_b(ab), -1));
            sg[ab] = gs[pp] + gs[pm];
            dg[ab] = gs[pp] - gs[pm];
          });
          sfor<0, Q>([&](auto kk) {
            constexpr int kq = decltype(kk)::value;
            if constexpr (rate_of<D>(kq) == R_NU) {
              R md = R(-0.0);
              sfor<0, D>([&](auto dd) {
                constexpr int d = decltype(dd)::value;
                constexpr double c = stress_b<D>(kq, d, d);
                if constexpr (c == 1.0) md = md + gs[pair_of<D>(axis_dir<D>(d))];
                else if constexpr (c == -1.0) md = md - gs[pair_of<D>(axis_dir<D>(d))];
                else if constexpr (c != 0.0) md = md + R(c) * gs[pair_of<D>(axis_dir<D>(d))];
              });
              sfor<0, n_ab<D>()>([&](auto ii) {
                constexpr int ab = decltype(ii)::value;
                constexpr double cs = SnuDiagSum<D, ab>::at(kq), cd = SnuDiagOff<D, ab>::at(kq);
                if constexpr (cs == 1.0) md = md + sg[ab];
                else if constexpr (cs == -1.0) md = md - sg[ab];
                else if constexpr (cs != 0.0) md = md + R(cs) * sg[ab];
                if constexpr (cd == 1.0) md = md + dg[ab];
                else if constexpr (cd == -1.0) md = md - dg[ab];
                else if constexpr (cd != 0.0) md = md + R(cd) * dg[ab];
              });
              md = md + stress_form<D, kq, R>(up, vF);
              ck[kq] = P.dspec[m][kq] * md;
            }
          });
        }
        // the correction of each pair, sum_k ck_k mt(n, k): B(d, d) on the axis
        // pairs; on a diagonal pair e_a + s e_b, (B(a, a) + B(b, b)) + s 2 B(a, b)
        R cax[D], csum[n_ab<D>()], coff[n_ab<D>()];
        sfor<0, D>([&](auto dd) {
          constexpr int d = decltype(dd)::value;
          cax[d] = snu_lincomb<D, SnuAxis<D, d>, R>(ck);
        });
        sfor<0, n_ab<D>()>([&](auto ii) {
          constexpr int ab = decltype(ii)::value;
          csum[ab] = snu_lincomb<D, SnuDiagSum<D, ab>, R>(ck);
          coff[ab] = snu_lincomb<D, SnuDiagOff<D, ab>, R>(ck);
        });
        const bool k0 = keep == R(0);
        push(std::integral_constant<int, 0>{}, m, k0 ? X0 : keep * pop(std::integral_constant<int, 0>{}) + X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          R corr;
          if constexpr (n <= L::NAXIS) {
            constexpr int d = L::c(n, 0) != 0 ? 0 : (L::c(n, 1) != 0 ? 1 : 2);
            corr = cax[d];
          } else {
            constexpr int a = L::c(n, 0) != 0 ? 0 : 1;
            constexpr int b = (a == 0 && L::c(n, 1) != 0) ? 1 : 2;
            constexpr int ab = a == 0 ? (b == 1 ? 0 : 1) : 2;
            constexpr int sgn = L::c(n, a) * L::c(n, b);
            corr = sgn > 0 ? csum[ab] + coff[ab] : csum[ab] - coff[ab];
          }
          const R h = cdot_z<D, n>(kF);
          const R vn = En[p] * (G + h) - corr, vb = Eb[p] * (G - h) - corr;
          if (k0) {
            push(std::integral_constant<int, n>{}, m, vn);
            push(std::integral_constant<int, nb>{}, m, vb);
          } else {
            push(std::integral_constant<int, n>{}, m, keep * pop(std::integral_constant<int, n>{}) + vn);
            push(std::integral_constant<int, nb>{}, m, keep * pop(std::integral_constant<int, nb>{}) + vb);
          }
        });
      } else if constexpr (MRT) {
        // General rate pattern, compiled into the MRT kernels only (the host
        // runs the others when every component is BGK-like or s_nu-only):
        // relax every moment at s0, then correct each moment k whose rate
        // differs by dspec_k times its projection of the deviation from the
        // forced equilibrium, f - E_n (r + 1.5 F.u - 1.5 F.c_n)
        R fo[Q], dfi[Q];
        const R hFu = R(1.5) * Fu;
        R hF[D];
#pragma unroll
        for (int d = 0; d < D; ++d) hF[d] = R(1.5) * F[m][d];
        {
          const R g0 = pop(std::integral_constant<int, 0>{});
          fo[0] = keep * g0 + X0;
          dfi[0] = g0 - E0 * (r + hFu);
        }
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          const R h = cdot_z<D, n>(kF), t = cdot_z<D, n>(hF);
          const R gn = pop(std::integral_constant<int, n>{}), gb = pop(std::integral_constant<int, nb>{});
          fo[n] = keep * gn + En[p] * (G + h);
          fo[nb] = keep * gb + Eb[p] * (G - h);
          dfi[n] = gn - En[p] * (r + hFu - t);
          dfi[nb] = gb - Eb[p] * (r + hFu + t);
        });
        sfor<0, Q>([&](auto kk) {
          constexpr int kq = decltype(kk)::value;
          if (spec & (1u << kq)) {
            R md = R(-0.0);
            sfor<0, Q>([&](auto ii) {
              constexpr int i = decltype(ii)::value;
              constexpr int v = L::mt(i, kq);
              if constexpr (v == 1) md = md + dfi[i];
              else if constexpr (v == -1) md = md - dfi[i];
              else if constexpr (v != 0) md = md + R(v) * dfi[i];
            });
            const R ckq = P.dspec[m][kq] * md;
            sfor<0, Q>([&](auto ii) {
              constexpr int i = decltype(ii)::value;
              constexpr int v = L::mt(i, kq);
              if constexpr (v == 1) fo[i] = fo[i] - ckq;
              else if constexpr (v == -1) fo[i] = fo[i] + ckq;
              else if constexpr (v != 0) fo[i] = fo[i] - ckq * R(v);
            });
          }
        });
        sfor<0, Q>([&](auto nn) { push(nn, m, fo[decltype(nn)::value]); });
      }
    }
  } else {
    // Fast form of the FP32-arithmetic forms, with c_s^2 = 1/3 and E_n = W~_n (A_m,n + B_n) (W~_0 = 1):
    //   feq_n   = rho E_n                      (B_n holds the velocity terms)
    //   P feq_n = 3 E_n (F.c_n - F.u)          (He forcing)
    //   f'_n    = (1 - s0) f_n + s0 feq_n + (3 - 1.5 s0) E_n (F.c_n - F.u),
    // i.e. f - s0 (f - feq + P feq / 2) + P feq, every moment relaxed at s0;
    // moments whose MRT rate differs from s0 are corrected afterwards.
    // Everything is computed on deviations from the rest state, g = f - w rho0:
    // g'_n = (1 - s0) g_n + s0 dE_n + k E_n (F.c_n - F.u)
    // with dE_n = feq_n - w_n rho0 = W~A (rho - rho0) + W~B rho + (W~A - w) rho0,
    // so that FP32 arithmetic keeps the precision of the small deviations.
    // WB_n = W~_n B_n is shared by the components.
    //
    // Directions come in pairs (n, n~ = opp(n)).  With ud = c_n.u, the velocity
    // terms split into an even and an odd part, WB_n = WBe + Bo and
    // WB_n~ = WBe - Bo (WBe = 4.5 w ud^2 - 1.5 w u^2, Bo = 3 w ud), and with
    // h = c_n.kF the relaxed pair is
    //   g'_n = keep g_n + Pe + Po,   g'_n~ = keep g_n~ + Pe - Po,
    //   Pe = s0 De + Bo h - Ae kFu,  Po = Bo G + Ae h,  G = s0 rho - kFu,
    // where Ae = W~A + WBe and De = W~A (rho - rho0) + WBe rho + cA.  Moments relaxed at s_nu != s0 (the
    // traceless second moments, even in c) correct Pe through the pair sums of
    // the non-equilibrium part, S_p = dfi_n + dfi_n~.  Other rate patterns take
    // the general path below.
    constexpr int NP = npairs<D>();
    const R cu_axis = R(1.5 * L::w(1)) * usqr, cu_diag = R(1.5 * L::w(Q - 1)) * usqr;
    R Bo[NP], WBe[NP];
    sfor<0, NP>([&](auto pp) {
      constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
      constexpr double w = L::w(n);
      const R ud = cdot_z<D, n>(up);
      Bo[p] = R(3 * w) * ud;
      WBe[p] = R(4.5 * w) * ud * ud - (n <= L::NAXIS ? cu_axis : cu_diag);
    });
    const R WB0 = D == 3 ? R(-0.5) * usqr : R(-2.0 / 3.0) * usqr;
#pragma unroll
    for (int m = 0; m < S; ++m) {
      const R r = rc[m], rd = rcd[m];
      // W~A per direction class (rest, axis, diagonal) and its offset from w
      const R WA0 = P.WAc[m][0], WA1 = P.WAc[m][1], WA2 = P.WAc[m][2];
      const R cA0 = P.cA[m][0], cA1 = P.cA[m][1], cA2 = P.cA[m][2];
      const R s0 = P.s0[m];
      const R k = P.kfac[m];
      const R keep = P.keep[m];
      R Fu = R(-0.0), kF[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        Fu = Fu + F[m][d] * up[d];
        kF[d] = k * F[m][d];
      }
      const R kFu = k * Fu;
      const R G = s0 * r - kFu;
      const unsigned spec = P.spec_mask[m];
      const T* fm = fin + (long long)m * Q * N;
      auto pop = [&](auto nn) -> R {
        constexpr int n = decltype(nn)::value;
        return ld_dev_s<T, R>(fm + (long long)n * N + c, sc);
      };
      const R E0 = WA0 + WB0;
      // rest direction: g'_0 = keep g_0 + X0
      const R X0 = s0 * (WA0 * rd + (WB0 * r + cA0)) - E0 * kFu;
      // the even and odd parts of pair p
      auto pair_terms = [&](auto pp, R& pe, R& po) {
        constexpr int p = decltype(pp)::value, n = pair_n<D>(p);
        const R WA = n <= L::NAXIS ? WA1 : WA2;
        const R Ae = WA + WBe[p];
        const R h = cdot_z<D, n>(kF);
        const R De = WA * rd + (WBe[p] * r + (n <= L::NAXIS ? cA1 : cA2));
        pe = s0 * De + (Bo[p] * h - Ae * kFu);
        po = Bo[p] * G + Ae * h;
      };
      if (spec == 0u && keep == R(0)) {
        // s0 = 1 (tau = 1): the relaxed populations are the forced equilibrium
        push(std::integral_constant<int, 0>{}, m, X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
          R pe, po;
          pair_terms(pp, pe, po);
          push(std::integral_constant<int, n>{}, m, pe + po);
          push(std::integral_constant<int, nb>{}, m, pe - po);
        });
      } else if (spec == 0u) {
        // every moment relaxes at s0 (BGK): one pair at a time
        push(std::integral_constant<int, 0>{}, m, keep * pop(std::integral_constant<int, 0>{}) + X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
          R pe, po;
          pair_terms(pp, pe, po);
          push(std::integral_constant<int, n>{}, m, keep * pop(std::integral_constant<int, n>{}) + (pe + po));
          push(std::integral_constant<int, nb>{}, m, keep * pop(std::integral_constant<int, nb>{}) + (pe - po));
        });
      } else if (spec == stress_mask<D>()) {
        // s_nu != s0, every other rate s0: the s_nu moments of the pair sums
        // of the non-equilibrium part, S_p = g_n + g_n~ - 2 De - Ae (3 F.u) +
        // Bo c_n.(3 F), give the corrections ck; then each pair is relaxed
        // and pushed with its correction.
        R ck[Q];
        {
          // pass 1: the pair sums of the non-equilibrium part, then their s_nu moments
          R F3[D];
#pragma unroll
          for (int d = 0; d < D; ++d) F3[d] = R(3) * F[m][d];
          const R hFu2 = R(3) * Fu;
          R Sp[NP];
          sfor<0, NP>([&](auto pp) {
            constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
            const R WA = n <= L::NAXIS ? WA1 : WA2;
            const R Ae = WA + WBe[p];
            const R t2 = cdot_z<D, n>(F3);
            const R gs = pop(std::integral_constant<int, n>{}) + pop(std::integral_constant<int, nb>{});
            const R De = WA * rd + (WBe[p] * r + (n <= L::NAXIS ? cA1 : cA2));
            Sp[p] = (gs - R(2) * De) - Ae * hFu2 + Bo[p] * t2;
          });
          sfor<0, Q>([&](auto kk) {
            constexpr int kq = decltype(kk)::value;
            if constexpr (rate_of<D>(kq) == R_NU) {
              R md = R(-0.0);
              sfor<0, NP>([&](auto pp) {
                constexpr int p = decltype(pp)::value;
                constexpr int v = L::mt(pair_n<D>(p), kq);
                if constexpr (v == 1) md = md + Sp[p];
                else if constexpr (v == -1) md = md - Sp[p];
                else if constexpr (v != 0) md = md + R(v) * Sp[p];
              });
              ck[kq] = P.dspec[m][kq] * md;
            }
          });
        }
        const bool k0 = keep == R(0);
        push(std::integral_constant<int, 0>{}, m, k0 ? X0 : keep * pop(std::integral_constant<int, 0>{}) + X0);
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          R pe, po;
          pair_terms(pp, pe, po);
          sfor<0, Q>([&](auto kk) {
            constexpr int kq = decltype(kk)::value;
            if constexpr (rate_of<D>(kq) == R_NU) {
              constexpr int v = L::mt(n, kq);
              if constexpr (v == 1) pe = pe - ck[kq];
              else if constexpr (v == -1) pe = pe + ck[kq];
              else if constexpr (v != 0) pe = pe - R(v) * ck[kq];
            }
          });
          if (k0) {
            push(std::integral_constant<int, n>{}, m, pe + po);
            push(std::integral_constant<int, nb>{}, m, pe - po);
          } else {
            push(std::integral_constant<int, n>{}, m, keep * pop(std::integral_constant<int, n>{}) + (pe + po));
            push(std::integral_constant<int, nb>{}, m, keep * pop(std::integral_constant<int, nb>{}) + (pe - po));
          }
        });
      } else if constexpr (MRT) {
        // General rate pattern, compiled into the MRT kernels only (the host
        // runs the others when every component is BGK-like or s_nu-only):
        // relax every moment at s0, then correct each
        // moment k whose rate differs by dspec_k times its projection of the
        // deviation from the forced equilibrium, g - dE_n + 1.5 E_n (F.c_n - F.u)
        R fo[Q], dfi[Q];
        fo[0] = keep * pop(std::integral_constant<int, 0>{}) + X0;
        const R hFu = R(1.5) * Fu;
        R hF[D];
#pragma unroll
        for (int d = 0; d < D; ++d) hF[d] = R(1.5) * F[m][d];
        {
          const R g0 = pop(std::integral_constant<int, 0>{});
          dfi[0] = g0 - (WA0 * rd + (WB0 * r + cA0)) - E0 * hFu;
        }
        sfor<0, NP>([&](auto pp) {
          constexpr int p = decltype(pp)::value, n = pair_n<D>(p), nb = opp<D>(n);
          R pe, po;
          pair_terms(pp, pe, po);
          const R gn = pop(std::integral_constant<int, n>{}), gb = pop(std::integral_constant<int, nb>{});
          fo[n] = keep * gn + (pe + po);
          fo[nb] = keep * gb + (pe - po);
          const R WA = n <= L::NAXIS ? WA1 : WA2;
          const R t = cdot_z<D, n>(hF);
          const R En = WA + WBe[p] + Bo[p], Eb = WA + WBe[p] - Bo[p];
          const R De = WA * rd + (WBe[p] * r + (n <= L::NAXIS ? cA1 : cA2));
          dfi[n] = gn - (De + Bo[p] * r) + En * (t - hFu);
          dfi[nb] = gb - (De - Bo[p] * r) - Eb * (t + hFu);
        });
        sfor<0, Q>([&](auto kk) {
          constexpr int kq = decltype(kk)::value;
          if (spec & (1u << kq)) {
            R md = R(-0.0);
            sfor<0, Q>([&](auto ii) {
              constexpr int i = decltype(ii)::value;
              constexpr int v = L::mt(i, kq);
              if constexpr (v == 1) md = md + dfi[i];
              else if constexpr (v == -1) md = md - dfi[i];
              else if constexpr (v != 0) md = md + R(v) * dfi[i];
            });
            const R ck = P.dspec[m][kq] * md;
            sfor<0, Q>([&](auto ii) {
              constexpr int i = decltype(ii)::value;
              constexpr int v = L::mt(i, kq);
              if constexpr (v == 1) fo[i] = fo[i] - ck;
              else if constexpr (v == -1) fo[i] = fo[i] + ck;
              else if constexpr (v != 0) fo[i] = fo[i] - ck * R(v);
            });
          }
        });
        sfor<0, Q>([&](auto nn) { push(nn, m, fo[decltype(nn)::value]); });
      }
    }
  }
}

template <int D, int S, int ISO, bool MRT, bool EXACT, class T, class R, class RT>
__global__ void __launch_bounds__(128, TX_STEP_MIN_BLOCKS(S, R, MRT || EXACT)) k_step(StepArgs a_in) {
  const StepArgs a = a_in;  // local copy: helpers never address the kernel parameter
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  step_site<D, S, ISO, MRT, EXACT, T, R, RT>(a, x, y, z);
}

// Link masks of every site from the wall mask (see link_of).
template <int D>
__global__ void __launch_bounds__(256) k_links(const uint8_t* mask, Geo g, uint32_t* links) {
  using L = Lat<D>;
  int x, y, z;
  long long idx;
  if (!site_of(g, x, y, z, idx)) return;
  const Hood<D, 1> h(g, x, y, z);
  uint32_t b = __ldg(mask + idx) == 0 ? 1u : 0u;
  sfor<1, L::Q>([&](auto nn) {
    constexpr int n = decltype(nn)::value;
    constexpr int cx = L::c(n, 0), cy = L::c(n, 1), cz = D == 3 ? L::c(n, 2) : 0;
    const bool in = h.template inside<cx, cy, cz>();
    const bool pore = __ldg(mask + h.template at<cx, cy, cz>()) == 0;
    b |= (in & pore) ? (1u << n) : 0u;
  });
  // the whole box of reach 2 (and, in 2D, 3) pore: the bulk gradient of isotropy 8 (10)
  if (b & 1u) {
    const Hood<D, 3> h3(g, x, y, z);
    bool box2 = true, box3 = true;
    constexpr int RZ = D == 3 ? 2 : 0;
    for (int dz = -RZ; dz <= RZ; ++dz)
      for (int dy = -3; dy <= 3; ++dy)
        for (int dx = -3; dx <= 3; ++dx) {
          const bool in = ((h3.in_x >> (dx + 3)) & (h3.in_y >> (dy + 3)) & (h3.in_z >> (dz + (D == 3 ? 3 : 0))) & 1u) != 0u;
          const unsigned off = (unsigned)(h3.ox[dx + 3] + h3.oy[dy + 3] + h3.oz[dz + (D == 3 ? 3 : 0)]);
          const bool ok = in && __ldg(mask + off) == 0;
          const bool r2 = dx >= -2 && dx <= 2 && dy >= -2 && dy <= 2;
          if (r2) box2 = box2 && ok;
          if (D == 2) box3 = box3 && ok;
        }
    if (box2) b |= kBoxPore2;
    if (D == 2 && box3) b |= kBoxPore3;
  }
  links[idx] = b;
}

// -------------------------------------------------- Dirichlet density node
// BCApplyDirichletNode (lbm_bc.F90:1273-1333) in the local frame of
// DiscSetLocalDirections (lbm_discretization_d3q19.F90:566-714; d2q9:372-434):
// normal axis a, inward sign sg, tangential axes in CARDINAL order.
template <int D, int S, class R>
__device__ __forceinline__ void dirichlet_node(int f, const R pv[S], R fv[S][Lat<D>::Q]) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const int a = f >> 1;
  const int sg = (f & 1) == 0 ? 1 : -1;
  int tang[2];
  int nt;
  if (D == 3) {
    tang[0] = a == 0 ? 1 : (a == 1 ? 2 : 0);
    tang[1] = a == 0 ? 2 : (a == 1 ? 0 : 1);
    nt = 2;
  } else {
    tang[0] = a == 0 ? 1 : 0;
    tang[1] = 0;
    nt = 1;
  }
  R wsn = R(0);
  for (int n = 1; n < Q; ++n)
    if (sg * L::c(n, a) == 1) wsn = wsn + R(L::w(n));
#pragma unroll
  for (int m = 0; m < S; ++m) {
    R Qv[3] = {R(0), R(0), R(0)};
    R sum = R(0);
    for (int n = 0; n < Q; ++n) sum = sum + fv[m][n];
    Qv[a] = R(sg) * (pv[m] - sum) / wsn;
    for (int p = 0; p < nt; ++p) {
      const int t = tang[p];
      R mom = R(0), wst = R(0);
      for (int n = 1; n < Q; ++n) {
        mom = mom + fv[m][n] * R(L::c(n, t));
        if (sg * L::c(n, a) == 1 && L::c(n, t) != 0) wst = wst + R(L::w(n));
      }
      Qv[t] = -(mom / wst);
    }
    for (int n = 1; n < Q; ++n) {
      if (sg * L::c(n, a) != 1) continue;
      R cq = R(0);
      for (int d = 0; d < D; ++d) cq = cq + R(L::c(n, d)) * Qv[d];
      fv[m][n] = fv[m][n] + R(L::w(n)) * cq;
    }
  }
}

// ------------------------------------------------------------ V2 arithmetic
// Two FP32 lanes (two sites, or two consecutive cells) computed with the
// packed FP32x2 instructions of sm_100+.
struct V2 {
  float x, y;
};
__host__ __device__ __forceinline__ V2 v2(float a) { return V2{a, a}; }
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float2 f2_(V2 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ V2 v2_(float2 a) { return V2{a.x, a.y}; }
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return v2_(__fadd2_rn(f2_(a), f2_(b))); }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return v2_(__fadd2_rn(f2_(a), make_float2(-b.x, -b.y))); }
__device__ __forceinline__ V2 operator*(V2 a, V2 b) { return v2_(__fmul2_rn(f2_(a), f2_(b))); }
__device__ __forceinline__ V2 fma2(V2 a, V2 b, V2 c) { return v2_(__ffma2_rn(f2_(a), f2_(b), f2_(c))); }
#else
inline V2 operator+(V2 a, V2 b) { return V2{a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return V2{a.x - b.x, a.y - b.y}; }
inline V2 operator*(V2 a, V2 b) { return V2{a.x * b.x, a.y * b.y}; }
inline V2 fma2(V2 a, V2 b, V2 c) { return V2{__builtin_fmaf(a.x, b.x, c.x), __builtin_fmaf(a.y, b.y, c.y)}; }
#endif
__host__ __device__ __forceinline__ V2 operator-(V2 a) { return V2{-a.x, -a.y}; }

// -------------------------------------------------------------- density
// mode 0 (after a step): forcing density = the face value on Dirichlet-class
// face nodes (BCApplyDirichletToRho, lbm_bc.F90:252-434; the last such face in
// XM..ZP order wins), the sum of populations elsewhere.  With only Dirichlet
// faces the node corrections run here too (BCApplyDirichletD3/D2,
// lbm_bc.F90:1091-1271); otherwise k_faces applies every class in order.
// mode 1 (FlowUpdateMoments at init, lbm_flow.F90:466-478): plain sums.
template <int D, int S, class T, class R, class RT>
__device__ __forceinline__ void density_site(const StepArgs& a, int x, int y, int z, int mode) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * (long long)z);
  const unsigned c = (unsigned)idx;  // N < 2^31
  if (__ldg(a.mask + c) != 0) return;
  const long long N = a.g.n;
  RT* rho = reinterpret_cast<RT*>(a.rho);
  T* fcur = reinterpret_cast<T*>(a.fout);
  const unsigned keep = D == 3 ? 63u : 15u;
  const unsigned dhit = mode == 0 ? dir_bits(a.faces) & site_faces(a.g, x, y, z) & keep : 0u;
  if (dhit && a.faces.post) {
    // corrections follow in k_faces: here only the face value as forcing density
    R rf[S];
    sfor<0, 2 * D>([&](auto ff) {
      constexpr int f = decltype(ff)::value;
      if (dhit & (1u << f)) {
        const long long area = face_area<D>(a.g, f), node = face_node<D>(a.g, f, x, y, z);
#pragma unroll
        for (int m = 0; m < S; ++m) rf[m] = R(a.faces.vals[f][(long long)m * area + node]);
      }
    });
#pragma unroll
    for (int m = 0; m < S; ++m) {
      rho[(size_t)c * S + m] = RT(kShifted<T> ? rf[m] - P.rho0[m] : rf[m]);
      if (P.eos_on)
        reinterpret_cast<RT*>(a.psi)[(size_t)c * S + m] = RT(eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, rf[m]));
    }
    return;
  }
  if (!dhit) {
    // stored as rho - rho0 = sum_n (f_n - w_n rho0)
#pragma unroll
    for (int m = 0; m < S; ++m) {
      R acc = R(0);
      sfor<0, Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        acc = acc + ld_dev<T, R>(fcur + (long long)(m * Q + n) * N + c, P);
      });
      rho[(size_t)c * S + m] = RT(acc);
      if (P.eos_on)
        reinterpret_cast<RT*>(a.psi)[(size_t)c * S + m] =
            RT(eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, P.rho0[m] + acc));
    }
    return;
  }
  // Dirichlet nodes work on the populations themselves
  R fv[S][Q];
  load_pops<D, S, T, R>(fcur, N, c, P, fv);
  if constexpr (kShifted<T>) {
#pragma unroll
    for (int m = 0; m < S; ++m)
      sfor<0, Q>([&](auto nn) { fv[m][decltype(nn)::value] += R(L::w(decltype(nn)::value)) * P.rho0[m]; });
  }
  R rf[S];
  sfor<0, 2 * D>([&](auto ff) {
    constexpr int f = decltype(ff)::value;
    if (dhit & (1u << f)) {
      const long long area = face_area<D>(a.g, f), node = face_node<D>(a.g, f, x, y, z);
      const double* vals = a.faces.vals[f];
      R pv[S];
#pragma unroll
      for (int m = 0; m < S; ++m) pv[m] = R(vals[(long long)m * area + node]);
      dirichlet_node<D, S, R>(f, pv, fv);
#pragma unroll
      for (int m = 0; m < S; ++m) rf[m] = pv[m];
    }
  });
#pragma unroll
  for (int m = 0; m < S; ++m) {
    rho[(size_t)c * S + m] = RT(kShifted<T> ? rf[m] - P.rho0[m] : rf[m]);
    if (P.eos_on)
      reinterpret_cast<RT*>(a.psi)[(size_t)c * S + m] = RT(eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, rf[m]));
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      R v = fv[m][n];
      if constexpr (kShifted<T>) v = v - R(L::w(n)) * P.rho0[m];
      st_dev<T, R>(fcur + (long long)(m * Q + n) * N + c, v, P);
    });
  }
}

template <int D, int S, class T, class R, class RT>
__global__ void __launch_bounds__(256) k_density(StepArgs a_in, int mode) {
  const StepArgs a = a_in;  // local copy: helpers never address the kernel parameter
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  density_site<D, S, T, R, RT>(a, x, y, z, mode);
}

// The density pass with 16-byte loads: VW = 16 / sizeof(T) consecutive sites
// per thread (lattices with N a multiple of VW, so that every load is
// aligned).  The pass streams every population once; wide loads keep more
// bytes in flight per instruction.  Groups with a site on a Dirichlet face
// take density_site, site by site; the sums are density_site's, in the same
// order.
template <class T, class R>
__device__ __forceinline__ R from_dev(T v, const PhysT<R>& P) {
  if constexpr (std::is_same<T, __half>::value)
    return R(__half2float(v)) * P.inv_sscale;
  else
    return R(v);
}

// the VW sites from c0: with VEC, 16-byte loads (c0 and N multiples of VW);
// otherwise element loads of the cnt <= VW sites that exist
template <int D, int S, class T, class R, class RT, bool VEC = true>
__device__ __forceinline__ void density_group(const StepArgs& a, long long c0, int mode, int cnt = 16 / (int)sizeof(T)) {
  constexpr int VW = 16 / (int)sizeof(T);
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const long long N = a.g.n;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const unsigned keep = D == 3 ? 63u : 15u;
  if (mode == 0 && (dir_bits(a.faces) & keep)) {
    bool face = false;
#pragma unroll
    for (int v = 0; v < VW; ++v) {
      if (v >= cnt) break;
      const long long c = c0 + v;
      const int x = (int)(c % a.g.nx), y = (int)((c / a.g.nx) % a.g.ny), z = (int)(c / ((long long)a.g.nx * a.g.ny));
      face |= (dir_bits(a.faces) & site_faces(a.g, x, y, z) & keep) != 0u;
    }
    if (face) {
      for (int v = 0; v < cnt; ++v) {
        const long long c = c0 + v;
        const int x = (int)(c % a.g.nx), y = (int)((c / a.g.nx) % a.g.ny), z = (int)(c / ((long long)a.g.nx * a.g.ny));
        density_site<D, S, T, R, RT>(a, x, y, z, mode);
      }
      return;
    }
  }
  bool pore[VW];
  bool any = false;
#pragma unroll
  for (int v = 0; v < VW; ++v) {
    pore[v] = v < cnt && __ldg(a.mask + c0 + (v < cnt ? v : 0)) == 0;
    any |= pore[v];
  }
  if (!any) return;
  const T* fcur = reinterpret_cast<const T*>(a.fout);
  RT* rho = reinterpret_cast<RT*>(a.rho);
  if constexpr (VEC && !std::is_same<T, double>::value) {
    // FP32 arithmetic: the stored values of two cells per packed add, the FP16
    // storage scale applied once to each sum; with two components and every
    // site pore, each two sites' densities leave in one 16-byte store
    float sum[S][VW];
#pragma unroll
    for (int m = 0; m < S; ++m) {
      V2 acc2[VW / 2];
#pragma unroll
      for (int v = 0; v < VW / 2; ++v) acc2[v] = v2(0.f);
      sfor<0, Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        const uint4 w = __ldg(reinterpret_cast<const uint4*>(fcur + (long long)(m * Q + n) * N + c0));
        uint32_t wd[4];
        memcpy(wd, &w, 16);
#pragma unroll
        for (int v = 0; v < VW / 2; ++v) {
          float2 f;
          if constexpr (std::is_same<T, __half>::value) {
            __half2 h;
            memcpy(&h, &wd[v], 4);
            f = __half22float2(h);
          } else {
            memcpy(&f, &wd[2 * v], 8);
          }
          acc2[v] = acc2[v] + V2{f.x, f.y};
        }
      });
      const float inv = std::is_same<T, __half>::value ? float(P.inv_sscale) : 1.f;
#pragma unroll
      for (int v = 0; v < VW / 2; ++v) {
        sum[m][2 * v] = acc2[v].x * inv;
        sum[m][2 * v + 1] = acc2[v].y * inv;
      }
    }
    bool all = true;
#pragma unroll
    for (int v = 0; v < VW; ++v) all = all && pore[v];
    if (S == 2 && all && !P.eos_on) {
#pragma unroll
      for (int v = 0; v < VW; v += 2)
        *reinterpret_cast<float4*>(rho + (size_t)(c0 + v) * S) =
            make_float4(sum[0][v], sum[S - 1][v], sum[0][v + 1], sum[S - 1][v + 1]);
    } else {
#pragma unroll
      for (int v = 0; v < VW; ++v) {
        if (!pore[v]) continue;
#pragma unroll
        for (int m = 0; m < S; ++m) {
          rho[(size_t)(c0 + v) * S + m] = RT(sum[m][v]);
          if (P.eos_on)
            reinterpret_cast<RT*>(a.psi)[(size_t)(c0 + v) * S + m] =
                RT(eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, P.rho0[m] + R(sum[m][v])));
        }
      }
    }
    return;
  }
#pragma unroll
  for (int m = 0; m < S; ++m) {
    R acc[VW];
#pragma unroll
    for (int v = 0; v < VW; ++v) acc[v] = R(0);
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      const T* src = fcur + (long long)(m * Q + n) * N + c0;
      if constexpr (VEC) {
        const uint4 w = __ldg(reinterpret_cast<const uint4*>(src));
        T vals[VW];
        memcpy(vals, &w, 16);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc[v] = acc[v] + from_dev<T, R>(vals[v], P);
      } else {
#pragma unroll
        for (int v = 0; v < VW; ++v)
          if (v < cnt) acc[v] = acc[v] + from_dev<T, R>(__ldg(src + v), P);
      }
    });
#pragma unroll
    for (int v = 0; v < VW; ++v) {
      if (!pore[v]) continue;
      rho[(size_t)(c0 + v) * S + m] = RT(acc[v]);
      if (P.eos_on)
        reinterpret_cast<RT*>(a.psi)[(size_t)(c0 + v) * S + m] =
            RT(eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, P.rho0[m] + acc[v]));
    }
  }
}

template <int D, int S, class T, class R, class RT>
__global__ void __launch_bounds__(256) k_density_vec(StepArgs a_in, int mode) {
  constexpr int VW = 16 / (int)sizeof(T);
  const StepArgs a = a_in;
  const long long c0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * VW;
  if (c0 < a.g.n) density_group<D, S, T, R, RT>(a, c0, mode);
}

// ------------------------------------------------ Neumann and velocity nodes
// BCApplyNeumannNode (lbm_bc.F90:1533-1593): v is the node's (s, ndims)
// momentum block, F the node's forces (FlowCalcRhoForces of this step).
template <int D, int S, class R>
__device__ __forceinline__ void neumann_node(int f, const R v[S * D], const R F[S][D], R fv[S][Lat<D>::Q]) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const int a = f >> 1;
  const int sg = (f & 1) == 0 ? 1 : -1;
#pragma unroll
  for (int m = 0; m < S; ++m) {
    R Qv[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int p = 0; p < D; ++p) {
      R mom = R(0), ws = R(0);
#pragma unroll
      for (int n = 1; n < Q; ++n) {
        const int cp = L::c(n, p);
        if (cp > 0) mom = mom + fv[m][n];
        if (cp < 0) mom = mom - fv[m][n];
        if (sg * L::c(n, a) == 1 && cp != 0) ws = ws + R(L::w(n));
      }
      Qv[p] = (v[p * S + m] - F[m][p] / R(2) - mom) / ws;
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
      if (sg * L::c(n, a) != 1) continue;
      R cq = R(0);
      for (int d = 0; d < D; ++d) cq = cq + R(L::c(n, d)) * Qv[d];
      fv[m][n] = fv[m][n] + R(L::w(n)) * cq;
    }
  }
}

// BCApplyVelocityNode (lbm_bc.F90:1793-1865): every component is driven to
// the velocity in v's first row (entries d * S); tangential axes in CARDINAL order.
template <int D, int S, class R>
__device__ __forceinline__ void velocity_node(int f, const R v[S * D], const R F[S][D], R fv[S][Lat<D>::Q]) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const int a = f >> 1;
  const int sg = (f & 1) == 0 ? 1 : -1;
  int tang[2];
  int nt;
  if (D == 3) {
    tang[0] = a == 0 ? 1 : (a == 1 ? 2 : 0);
    tang[1] = a == 0 ? 2 : (a == 1 ? 0 : 1);
    nt = 2;
  } else {
    tang[0] = a == 0 ? 1 : 0;
    tang[1] = 0;
    nt = 1;
  }
#pragma unroll
  for (int m = 0; m < S; ++m) {
    R Qv[3] = {R(0), R(0), R(0)};
    R momn = R(0), wsn = R(0);
#pragma unroll
    for (int n = 1; n < Q; ++n) {
      const int ca = L::c(n, a);
      if (ca > 0) momn = momn + fv[m][n];
      if (ca < 0) momn = momn - fv[m][n];
      if (sg * ca == 1) wsn = wsn + R(L::w(n));
    }
    R sum = R(0);
#pragma unroll
    for (int n = 0; n < Q; ++n) sum = sum + fv[m][n];
    const R un = v[a * S];
    Qv[a] = (sum * un - momn - F[m][a] / R(2)) / (R(1) - R(sg) * un) / wsn;
    const R rh = sum + wsn * Qv[a] * R(sg);
    for (int p = 0; p < nt; ++p) {
      const int t = tang[p];
      R mom = R(0), ws = R(0);
#pragma unroll
      for (int n = 1; n < Q; ++n) {
        const int ct = L::c(n, t);
        if (ct > 0) mom = mom + fv[m][n];
        if (ct < 0) mom = mom - fv[m][n];
        if (sg * L::c(n, a) == 1 && ct != 0) ws = ws + R(L::w(n));
      }
      Qv[t] = (rh * v[t * S] - F[m][t] / R(2) - mom) / ws;
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
      if (sg * L::c(n, a) != 1) continue;
      R cq = R(0);
      for (int d = 0; d < D; ++d) cq = cq + R(L::c(n, d)) * Qv[d];
      fv[m][n] = fv[m][n] + R(L::w(n)) * cq;
    }
  }
}

// BCApplyReflectingD3/D2 (lbm_bc.F90:825-1073) at a node of face FC, as
// written: each incoming population n takes, in p order, the value of every p
// with the same tangential components and the opposite normal one.  On the
// XM face in 3D the reference compares n's x component with p's z component
// (lbm_bc.F90:851); that comparison is kept.
template <int D, int S, int FC, class R>
__device__ __forceinline__ void reflect_node(R fv[S][Lat<D>::Q]) {
  using L = Lat<D>;
  constexpr int a = FC >> 1, sg = (FC & 1) == 0 ? 1 : -1;
  constexpr int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  constexpr int b3 = (D == 3 && FC == 0) ? 2 : a;
  sfor<1, L::Q>([&](auto nn) {
    constexpr int n = decltype(nn)::value;
    if constexpr (sg * L::c(n, a) > 0) {
      sfor<1, L::Q>([&](auto pp) {
        constexpr int q = decltype(pp)::value;
        constexpr bool same2 = D == 2 ? true : L::c(n, t2) == L::c(q, t2);
        if constexpr (L::c(n, t1) == L::c(q, t1) && same2 && L::c(n, a) == -L::c(q, b3)) {
#pragma unroll
          for (int m = 0; m < S; ++m) fv[m][n] = fv[m][q];
        }
      });
    }
  });
}

// -------------------------------------------------------------- face pass
// BCApply (lbm_bc.F90:781-807) after the density pass, for lattices with a
// face that is not of the Dirichlet class: at each pore face node, the
// classes in BCApply's order, each over the node's faces in XM..ZP order.
// The forces of Neumann and velocity nodes are the ones FlowCalcRhoForces
// computes from this step's forcing density (the next collision's forces).
template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__device__ __forceinline__ void face_site(const StepArgs& a, int x, int y, int z) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const unsigned c = (unsigned)x + (unsigned)a.g.nx * ((unsigned)y + (unsigned)a.g.ny * (unsigned)z);
  if (__ldg(a.mask + c) != 0) return;
  const unsigned keep = D == 3 ? 63u : 15u;
  const unsigned hit = active_bits(a.faces) & site_faces(a.g, x, y, z) & keep;
  if (!hit) return;
  const long long N = a.g.n;
  T* fcur = reinterpret_cast<T*>(a.fout);
  R fv[S][Q];
  load_pops<D, S, T, R>(fcur, N, c, P, fv);
  if constexpr (kShifted<T>) {
#pragma unroll
    for (int m = 0; m < S; ++m)
      sfor<0, Q>([&](auto nn) { fv[m][decltype(nn)::value] += R(L::w(decltype(nn)::value)) * P.rho0[m]; });
  }
  R F[S][D];
  bool need_f = false;
#pragma unroll
  for (int f = 0; f < 2 * D; ++f)
    need_f |= ((hit >> f) & 1u) && (a.faces.cls[f] == kClsNeu || a.faces.cls[f] == kClsVel);
  if (need_f) {
    const RT* rho = reinterpret_cast<const RT*>(a.rho);
    const Hood<D, stencil_reach<D, ISO>()> h(a.g, x, y, z);
    R rfd[S], rf[S];
    rho_at<S>(rho, c, rfd);
#pragma unroll
    for (int m = 0; m < S; ++m) rf[m] = P.rho0[m] + rfd[m];
    cell_forces<D, S, ISO, EXACT>(h, __ldg(a.links + c), P, a.mask, rho, reinterpret_cast<const RT*>(a.psi), N, rfd,
                                  rf, F);
  } else {
#pragma unroll
    for (int m = 0; m < S; ++m)
#pragma unroll
      for (int d = 0; d < D; ++d) F[m][d] = R(0);
  }
  for (int i = 0; i < a.faces.norder; ++i) {
    const int cls = a.faces.order[i];
    sfor<0, 2 * D>([&](auto ff) {
      constexpr int f = decltype(ff)::value;
      if (!((hit >> f) & 1u) || a.faces.cls[f] != cls) return;
      if (cls == kClsRefl) {
        reflect_node<D, S, f, R>(fv);
        return;
      }
      const long long area = face_area<D>(a.g, f), node = face_node<D>(a.g, f, x, y, z);
      R v[S * D];
#pragma unroll
      for (int k = 0; k < S * D; ++k) v[k] = R(a.faces.vals[f][(long long)k * area + node]);
      if (cls == kClsDir)
        dirichlet_node<D, S, R>(f, v, fv);
      else if (cls == kClsNeu)
        neumann_node<D, S, R>(f, v, F, fv);
      else
        velocity_node<D, S, R>(f, v, F, fv);
    });
  }
#pragma unroll
  for (int m = 0; m < S; ++m)
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      R w = fv[m][n];
      if constexpr (kShifted<T>) w = w - R(L::w(n)) * P.rho0[m];
      st_dev<T, R>(fcur + (long long)(m * Q + n) * N + c, w, P);
    });
}

// The face nodes of a lattice: faces with a node correction, each node once
// (by the first of its faces in XM..ZP order).
struct FaceShell {
  int nf;
  int face[6];
  long long start[7];
};

template <int D>
__device__ __forceinline__ bool shell_site(const Geo& g, const FaceShell& sh, long long t, int& x, int& y, int& z) {
  if (t >= sh.start[sh.nf]) return false;
  int i = 0;
  while (i + 1 < sh.nf && t >= sh.start[i + 1]) ++i;
  const int f = sh.face[i];
  const long long q = t - sh.start[i];
  const int a = f >> 1;
  const int fixed = (f & 1) ? (a == 0 ? g.nx : (a == 1 ? g.ny : g.nz)) - 1 : 0;
  if (D == 2) {
    x = a == 0 ? fixed : (int)q;
    y = a == 0 ? (int)q : fixed;
    z = 0;
  } else if (a == 0) {
    x = fixed; y = (int)(q % g.ny); z = (int)(q / g.ny);
  } else if (a == 1) {
    y = fixed; x = (int)(q % g.nx); z = (int)(q / g.nx);
  } else {
    z = fixed; x = (int)(q % g.nx); y = (int)(q / g.nx);
  }
  for (int j = 0; j < i; ++j)
    if (on_face(g, sh.face[j], x, y, z)) return false;
  return true;
}

template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_faces(StepArgs a_in, FaceShell sh) {
  const StepArgs a = a_in;
  int x, y, z;
  if (!shell_site<D>(a.g, sh, (long long)blockIdx.x * blockDim.x + threadIdx.x, x, y, z)) return;
  face_site<D, S, ISO, EXACT, T, R, RT>(a, x, y, z);
}

// ------------------------------------------------------- pressure outlets
// FlowUpdateBCPressureOutletD3/D2 (lbm_flow.F90:2020-2233), two components:
// before a step's boundary pass, the outlet face values become the densities
// of the face pressure at the mass fraction of the neighbour inside (of the
// node itself when that neighbour is a wall).  rho_a there is the previous
// step's: the population sum on re-summed face nodes, the forcing density
// elsewhere.  Reads the state (fin) and the forcing density; writes face f.
template <int D, int S, class T, class R, class RT>
__device__ __forceinline__ void outlet_node(const StepArgs& a, int f, double* vals, double pressure, double c0,
                                            double g21, long long q) {
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const long long area = face_area<D>(a.g, f);
  if (q >= area) return;
  const int ax = f >> 1;
  const int ext = ax == 0 ? a.g.nx : (ax == 1 ? a.g.ny : a.g.nz);
  const int fixed = (f & 1) ? ext - 1 : 0;
  int x, y, z;
  if (D == 2) {
    x = ax == 0 ? fixed : (int)q;
    y = ax == 0 ? (int)q : fixed;
    z = 0;
  } else if (ax == 0) {
    x = fixed; y = (int)(q % a.g.ny); z = (int)(q / a.g.ny);
  } else if (ax == 1) {
    y = fixed; x = (int)(q % a.g.nx); z = (int)(q / a.g.nx);
  } else {
    z = fixed; x = (int)(q % a.g.nx); y = (int)(q / a.g.nx);
  }
  const unsigned c = (unsigned)x + (unsigned)a.g.nx * ((unsigned)y + (unsigned)a.g.ny * (unsigned)z);
  if (__ldg(a.mask + c) != 0) return;
  int nb[3] = {x, y, z};
  nb[ax] += (f & 1) ? -1 : 1;
  unsigned src = c;
  int sx = x, sy = y, sz = z;
  if (nb[ax] >= 0 && nb[ax] < ext) {
    const unsigned cn = (unsigned)nb[0] + (unsigned)a.g.nx * ((unsigned)nb[1] + (unsigned)a.g.ny * (unsigned)nb[2]);
    if (__ldg(a.mask + cn) == 0) {
      src = cn;
      sx = nb[0]; sy = nb[1]; sz = nb[2];
    }
  }
  double r[S];
  const unsigned keep = D == 3 ? 63u : 15u;
  if (face_bits(a.faces) & site_faces(a.g, sx, sy, sz) & keep) {
    R fv[S][Lat<D>::Q];
    load_pops<D, S, T, R>(reinterpret_cast<const T*>(a.fin), a.g.n, src, P, fv);
#pragma unroll
    for (int m = 0; m < S; ++m) r[m] = double(P.rho0[m]) + double(pop_sum<D, S, R>(fv, m));
  } else {
    R rfd[S];
    rho_at<S>(reinterpret_cast<const RT*>(a.rho), src, rfd);
#pragma unroll
    for (int m = 0; m < S; ++m) r[m] = double(P.rho0[m]) + double(rfd[m]);
  }
  double tot = 0.0;
#pragma unroll
  for (int m = 0; m < S; ++m) tot = tot + r[m];
  double out[2] = {0.0, 0.0};
  density_from_pressure(S, c0, g21, pressure, r[0] / tot, out);
  vals[q] = out[0];
  if (S > 1) vals[area + q] = out[1];
}

template <int D, int S, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_outlet(StepArgs a_in, int f, double* vals, double pressure, double c0,
                                                double g21) {
  const StepArgs a = a_in;
  outlet_node<D, S, T, R, RT>(a, f, vals, pressure, c0, g21, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// -------------------------------------------------------------------- init
// FlowFiInit (lbm_flow.F90:923-934): forces from the initial density, the
// equilibrium at the initial velocity, f = (1 - P/2) feq (FlowFeqBarD3/D2).
// uic is [(m*D + d) * N + cell]; rho holds the initial density.
template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__device__ __forceinline__ void init_site(const StepArgs& a, int x, int y, int z, const double* uic) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * (long long)z);
  if (__ldg(a.mask + idx) != 0) return;
  const long long N = a.g.n;
  const RT* rho = reinterpret_cast<const RT*>(a.rho);
  R rfd[S], rf[S], F[S][D];
  rho_at<S>(rho, (unsigned)idx, rfd);
#pragma unroll
  for (int m = 0; m < S; ++m) rf[m] = P.rho0[m] + rfd[m];
  {
    const Hood<D, stencil_reach<D, ISO>()> h(a.g, x, y, z);
    cell_forces<D, S, ISO, EXACT>(h, __ldg(a.links + idx), P, a.mask, rho, reinterpret_cast<const RT*>(a.psi), N,
                                  rfd, rf, F);
  }
  T* fout = reinterpret_cast<T*>(a.fout);
#pragma unroll
  for (int m = 0; m < S; ++m) {
    R u[D];
    R usqr = R(0);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      u[d] = uic ? R(uic[(long long)(m * D + d) * N + idx]) : R(0);
      usqr = usqr + u[d] * u[d];
    }
    if constexpr (EXACT) {
      sfor<0, Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        R feq, pf;
        feq_pf<D, n, EXACT, R>(P, m, rf[m], u, usqr, F[m], feq, pf);
        St<T>::st(fout + (long long)(m * Q + n) * N + idx, (R(1.) - R(0.5) * pf) * feq);
      });
    } else if constexpr (!kShifted<T>) {
      // FP64 fast form: (1 - P/2) feq_n = E_n (rho + 1.5 F.u - 1.5 F.c_n), with the
      // pair weights E_n, E_n~ of step_site (two FMAs each)
      const R WAu1 = P.WAc[m][1] - R(1.5 * L::w(1)) * usqr, WAu2 = P.WAc[m][2] - R(1.5 * L::w(Q - 1)) * usqr;
      R Fu = R(-0.0), hF[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        Fu = Fu + F[m][d] * u[d];
        hF[d] = R(1.5) * F[m][d];
      }
      const R Y = rf[m] + R(1.5) * Fu;
      const R E0 = P.WAc[m][0] + (D == 3 ? R(-0.5) * usqr : R(-2.0 / 3.0) * usqr);
      St<T>::st(fout + (long long)(m * Q) * N + idx, E0 * Y);
      sfor<0, npairs<D>()>([&](auto pp) {
        constexpr int n = pair_n<D>(decltype(pp)::value), nb = opp<D>(n);
        constexpr double w = L::w(n);
        const R t = cdot_z<D, n>(u), h = cdot_z<D, n>(hF);
        const R WAu = n <= L::NAXIS ? WAu1 : WAu2;
        const R En = t * (R(3 * w) + R(4.5 * w) * t) + WAu, Eb = WAu - t * (R(3 * w) - R(4.5 * w) * t);
        St<T>::st(fout + (long long)(m * Q + n) * N + idx, En * (Y - h));
        St<T>::st(fout + (long long)(m * Q + nb) * N + idx, Eb * (Y + h));
      });
    } else {
      // the FP32-arithmetic forms: the deviation (1 - P/2) feq - w rho0 = dE_n - 1.5 E_n (F.c_n - F.u),
      // as in step_site
      const R A0 = P.A0[m], An = P.An[m];
      R Fu = R(0);
#pragma unroll
      for (int d = 0; d < D; ++d) Fu = Fu + F[m][d] * u[d];
      sfor<0, Q>([&](auto nn) {
        constexpr int n = decltype(nn)::value;
        constexpr double w = L::w(n);
        R ud = R(0), Fc = R(0);
        sfor<0, D>([&](auto dd) {
          constexpr int d = decltype(dd)::value;
          constexpr int cc = L::c(n, d);
          if constexpr (cc > 0) {
            ud = ud + u[d];
            Fc = Fc + F[m][d];
          }
          if constexpr (cc < 0) {
            ud = ud - u[d];
            Fc = Fc - F[m][d];
          }
        });
        R WA, WB, cA;
        if constexpr (n == 0) {
          WA = A0;
          WB = D == 3 ? R(-0.5) * usqr : R(-2.0 / 3.0) * usqr;
          cA = P.cA[m][0];
        } else {
          WA = R(w) * An;
          WB = ud * (R(3 * w) + R(4.5 * w) * ud) - R(1.5 * w) * usqr;
          cA = P.cA[m][n <= L::NAXIS ? 1 : 2];
        }
        const R dE = WA * rfd[m] + WB * rf[m] + cA;
        const R v = dE - R(1.5) * (WA + WB) * (Fc - Fu);
        st_dev<T, R>(fout + (long long)(m * Q + n) * N + idx, v, P);
      });
    }
  }
}

template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_init(StepArgs a_in, const double* uic) {
  const StepArgs a = a_in;  // local copy: helpers never address the kernel parameter
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  init_site<D, S, ISO, EXACT, T, R, RT>(a, x, y, z, uic);
}

// -------------------------------------------------------------- downloads
// Fields of the current state in natural order (component fastest).
// what: 2 rho, 3 flux (common velocity), 4 forces, 5 prs, 6 velt, 7 rhot
// (FlowUpdateDiagnosticsD3/D2, lbm_flow.F90:654-758, for psi = rho).
template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__device__ __forceinline__ void moments_site(const StepArgs& a, int x, int y, int z, int what, double* out) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
  const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * (long long)z);
  const bool wall = __ldg(a.mask + idx) != 0;
  const int dof = (what == 2 || what == 12) ? S : (what == 3 || what == 4) ? S * D : (what == 6 ? D : 1);
  if (wall) {
    for (int q = 0; q < dof; ++q) out[idx * dof + q] = 0.0;
    return;
  }
  const long long N = a.g.n;
  R fv[S][Q];
  if (what == 2) {
    // the density needs neither forces nor velocity: the forcing density, or
    // the population sum on re-summed face nodes (as cell_velocity forms rc)
    const bool dn = any_dirichlet<D>(a.g, a.faces, x, y, z);
    R rfd[S];
    rho_at<S>(reinterpret_cast<const RT*>(a.rho), (unsigned)idx, rfd);
    if (dn) load_pops<D, S, T, R>(reinterpret_cast<const T*>(a.fin), N, (unsigned)idx, P, fv);
    for (int m = 0; m < S; ++m) {
      const R sum = dn ? pop_sum<D, S, R>(fv, m) : rfd[m];
      if constexpr (kShifted<T>)
        out[idx * S + m] = double(P.rho0[m]) + double(sum);  // keeps the digits of the deviation
      else
        out[idx * S + m] = double(P.rho0[m] + sum);
    }
    return;
  }
  load_pops<D, S, T, R>(reinterpret_cast<const T*>(a.fin), N, (unsigned)idx, P, fv);
  R rc[S], rf[S], F[S][D], up[D];
  cell_moments<D, S, ISO, EXACT, R, RT>(a, P, x, y, z, idx, fv, rc, rf, F, up);
  if (what == 2) {
    if constexpr (kShifted<T>) {
      // rho0 + (rho - rho0) in FP64, so that the stored deviation keeps its digits
      const bool dn = any_dirichlet<D>(a.g, a.faces, x, y, z);
      R rfd[S];
      rho_at<S>(reinterpret_cast<const RT*>(a.rho), (unsigned)idx, rfd);
      for (int m = 0; m < S; ++m)
        out[idx * S + m] = double(P.rho0[m]) + double(dn ? pop_sum<D, S, R>(fv, m) : rfd[m]);
    } else {
      for (int m = 0; m < S; ++m) out[idx * S + m] = double(rc[m]);
    }
  } else if (what == 3 || what == 4) {
    for (int d = 0; d < D; ++d)
      for (int m = 0; m < S; ++m) out[(idx * D + d) * S + m] = double(what == 3 ? up[d] : F[m][d]);
  } else {
    R rt = R(0);
    for (int m = 0; m < S; ++m) rt = rt + rc[m] * R(P.mm[m]);
    if (what == 7) {
      out[idx] = double(rt);
    } else if (what == 5 || what == 12) {
      // FlowUpdateDiagnosticsD3/D2: psi = EOS(rho) when the EOS is on
      R ps[S];
      for (int m = 0; m < S; ++m) ps[m] = P.eos_on ? eos_psi<R>(P.eos[m], P.eos_c[m], P.g[m][m], P.c0, rc[m]) : rc[m];
      if (what == 12) {
        for (int m = 0; m < S; ++m) out[idx * S + m] = double(ps[m]);
        return;
      }
      R pr = rt / R(3.);
      if (S > 1 || P.eos_on) {
        for (int m = 0; m < S; ++m) {
          R acc = R(0);
          for (int k = 0; k < S; ++k) acc = acc + R(P.g[m][k]) * ps[k];
          pr = pr + R(P.c0) / R(2.) * ps[m] * acc;
        }
      }
      out[idx] = double(pr);
    } else {
      for (int d = 0; d < D; ++d) {
        R acc = R(0);
        for (int m = 0; m < S; ++m) acc = acc + (pop_flux<D, S, R>(fv, m, d) + R(.5) * F[m][d]) * R(P.mm[m]);
        out[idx * D + d] = double(acc / rt);
      }
    }
  }
}

template <int D, int S, int ISO, bool EXACT, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_moments(StepArgs a_in, int what, double* out) {
  const StepArgs a = a_in;  // local copy: helpers never address the kernel parameter
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  moments_site<D, S, ISO, EXACT, T, R, RT>(a, x, y, z, what, out);
}

// Running maximum of |(old - cur) / cur| (DistributionCalcDeltaNorm) over a
// sequence of values, with the FP64 division only for values that may reach
// it: a single-precision screen (|old - cur| and |cur| rounded to float,
// against the maximum less 2^-10, which covers the roundings) passes every
// value that can, and every value whose magnitudes leave float's normal range
// or whose running maximum lies outside [1e-30, 1e30].  The result is the
// exact maximum of the FP64 quotients; zero and NaN quotients never raise it.
struct NormMax {
  double mx = 0.0;
  float thr = 0.f;  // float(mx) (1 - 2^-10), or 0 (screen off)
  __host__ __device__ __forceinline__ void add(double o, double c) {
    constexpr float kMin = 1.17549435e-38f, kMax = 3.40282347e38f;
    if (c == 0.0) return;
    const double a = fabs(o - c), b = fabs(c);
    if (a == 0.0) return;
    const float af = (float)a, bf = (float)b;
    if ((af >= kMin && af <= kMax) && (bf >= kMin && bf <= kMax) && !(af > thr * bf)) return;
    const double v = a / b;
    if (v > mx) {
      mx = v;
      thr = (mx >= 1e-30 && mx < 1e30) ? (float)mx * (1.f - 0.0009765625f) : 0.f;
    }
  }
};

// Natural-order populations <-> SoA state (the shift and the FP16 scale are
// applied in FP64).  Wall cells read and write as zero; with mask = null
// (lattices with specular walls, whose wall cells hold populations) every
// cell's populations pass through.  A block moves kNatTile consecutive sites
// through shared memory, so that both the SoA side (one row per population)
// and the natural side (s*Q consecutive values per site) are read and written
// in whole lines.
constexpr int kNatTile = 64;

template <int D, int S, class T, class R>
__global__ void __launch_bounds__(256) k_pops_to_natural(const T* f, const uint8_t* mask, long long N, Shift sh,
                                                         double* out) {
  constexpr int Q = Lat<D>::Q, SQ = S * Q;
  __shared__ double tile[kNatTile * SQ];
  const long long c0 = (long long)blockIdx.x * kNatTile;
  const int cnt = (int)(N - c0 < kNatTile ? N - c0 : kNatTile);
  for (int i = threadIdx.x; i < SQ * kNatTile; i += blockDim.x) {
    const int q = i / kNatTile, v = i - q * kNatTile;  // q = m * Q + n, the SoA row
    if (v >= cnt) continue;
    const long long idx = c0 + v;
    const int m = q / Q, n = q - m * Q;
    double x = 0.0;
    if (!(mask && __ldg(mask + idx) != 0)) {
      x = double(St<T>::ld(f + (long long)q * N + idx));
      if constexpr (kShifted<T>) x = x / sh.scale + Lat<D>::w(n) * sh.rho0[m];
    }
    tile[v * SQ + n * S + m] = x;
  }
  __syncthreads();
  double* o = out + c0 * SQ;
  for (int i = threadIdx.x; i < cnt * SQ; i += blockDim.x) o[i] = tile[i];
}

template <int D, int S, class T, class R>
__global__ void __launch_bounds__(256) k_pops_from_natural(const double* in, const uint8_t* mask, long long N, Shift sh,
                                                           T* f) {
  constexpr int Q = Lat<D>::Q, SQ = S * Q;
  __shared__ double tile[kNatTile * SQ];
  const long long c0 = (long long)blockIdx.x * kNatTile;
  const int cnt = (int)(N - c0 < kNatTile ? N - c0 : kNatTile);
  const double* src = in + c0 * SQ;
  for (int i = threadIdx.x; i < cnt * SQ; i += blockDim.x) tile[i] = src[i];
  __syncthreads();
  for (int i = threadIdx.x; i < SQ * kNatTile; i += blockDim.x) {
    const int q = i / kNatTile, v = i - q * kNatTile;
    if (v >= cnt) continue;
    const long long idx = c0 + v;
    const int m = q / Q, n = q - m * Q;
    const bool wall = mask && __ldg(mask + idx) != 0;
    double x = wall ? 0.0 : tile[v * SQ + n * S + m];
    if constexpr (kShifted<T>) x = wall ? 0.0 : (x - Lat<D>::w(n) * sh.rho0[m]) * sh.scale;
    if constexpr (std::is_same<T, double>::value)
      f[(long long)q * N + idx] = x;
    else
      St<T>::st(f + (long long)q * N + idx, R(x));
  }
}

}  // namespace tx
