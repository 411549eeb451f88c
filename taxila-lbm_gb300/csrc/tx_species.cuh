// Passive species transport (LBM_Transport_module, src/lbm/lbm_transport.F90).
//
// Each species is a distribution on the flow's lattice that feels no force
// and no boundary condition but bounceback: per step it collides toward an
// equilibrium built from its own concentration and its own flux (the
// reference passes the flux array, not a velocity, to the equilibrium,
// TransportUpdateFeq, :363-378), streams and bounces back
// (TransportReactWithWalls without a reactive matrix, :461-477).  The species
// relax with d_k = 0 (RelaxationCreate, lbm_relaxation.F90:80, is not
// overridden for species).  TransportCollisionD3 collides pore cells;
// TransportCollisionD2 collides cells with walls > 0 (:450), so in 2D the
// species are streamed and bounced back without collision, as the reference
// does.
//
// State between steps: g[(sp*Q + n)*N + cell] after stream and bounceback;
// the concentration and flux of the next collision are the sums of those
// populations (TransportUpdateMoments, :312-318), so one kernel per step does
// the whole transport part of LBMRun2's loop body (lbm.F90:290-370).
#pragma once
#include "tx_kernels.cuh"

namespace tx {

// Relaxation of one species: SRT 1/tau or the MRT rates of its moments.
template <class R>
struct SpecieRelax {
  R tau, inv_tau;
  R srate[19];             // MRT rate of moment k
  R s0;                    // fast form: base rate, and corrections for the others
  R dspec[19];             // (rate_k - s0) / diag(M M^T)_k
  unsigned spec_mask;
};

template <class R>
struct SpeciesPhysT {
  SpecieRelax<R> sp[MAXC];
  R sscale, inv_sscale;    // FP16 storage scale (1 otherwise)
};

struct SpeciesArgs {
  const void* gin;
  void* gout;
  const uint32_t* links;
  const uint8_t* mask;
  const void* phys;        // device SpeciesPhysT<R>
  Geo g;
  int ns;
};

template <class T, class R>
__device__ __forceinline__ R ld_sp(const T* p, const SpeciesPhysT<R>& P) {
  if constexpr (std::is_same<T, __half>::value)
    return R(St<T>::ld(p)) * P.inv_sscale;
  else
    return R(St<T>::ld(p));
}
template <class T, class R>
__device__ __forceinline__ void st_sp(T* p, R v, const SpeciesPhysT<R>& P) {
  if constexpr (std::is_same<T, __half>::value)
    St<T>::st(p, v * P.sscale);
  else
    St<T>::st(p, v);
}

// Species equilibrium of direction n with d_k = 0 and the flux J as the
// velocity: DiscretizationEquilf_D3Q19 (lbm_discretization_d3q19.F90:265-305)
// / _D2Q9 (lbm_discretization_d2q9.F90:168-205) in the exact form's operation
// order.
template <int D, int n, class R>
__device__ __forceinline__ R species_feq_exact(R r, const R J[D], R usqr) {
  using L = Lat<D>;
  const R cs2 = R(1.0 / 3.0), dk = R(0.);
  if constexpr (n == 0) {
    if constexpr (D == 3)
      return r * (dk - usqr / R(2.));
    else
      return r * ((R(1.) + dk * R(5.)) / R(6.) - R(2.) * usqr / R(3.));
  } else {
    R udote = R(0);
    sfor<0, D>([&](auto dd) {
      constexpr int d = decltype(dd)::value;
      constexpr int c = L::c(n, d);
      if constexpr (c > 0) udote = udote + J[d];
      if constexpr (c < 0) udote = udote - J[d];
    });
    return R(L::w(n)) * r *
           (R(1.5) * (R(1.) - dk) + udote / cs2 + udote * udote / (R(2.) * cs2 * cs2) - usqr / (R(2.) * cs2));
  }
}

template <int D, bool MRT, bool EXACT, class T, class R>
__device__ __forceinline__ void species_site(const SpeciesArgs& a, int x, int y, int z) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const SpeciesPhysT<R>& P = *reinterpret_cast<const SpeciesPhysT<R>*>(a.phys);
  const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * (long long)z);
  const unsigned c = (unsigned)idx;
  const uint32_t links = __ldg(a.links + c);
  if (!(links & 1u)) return;  // wall cells hold no species populations
  const long long N = a.g.n;
  const Hood<D, 1> h(a.g, x, y, z);
  const T* gin = reinterpret_cast<const T*>(a.gin);
  T* gout = reinterpret_cast<T*>(a.gout);
  for (int s = 0; s < a.ns; ++s) {
    const SpecieRelax<R>& sr = P.sp[s];
    R g[Q];
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      g[n] = ld_sp<T, R>(gin + (long long)(s * Q + n) * N + c, P);
    });
    if constexpr (D == 3) {
      // concentration and flux in DistributionCalcDensity/Flux order
      R r = R(0), J[D];
      sfor<0, Q>([&](auto nn) { r = r + g[decltype(nn)::value]; });
      {
        R gv[1][Q];
#pragma unroll
        for (int n = 0; n < Q; ++n) gv[0][n] = g[n];
#pragma unroll
        for (int d = 0; d < D; ++d) J[d] = pop_flux<D, 1, R>(gv, 0, d);
      }
      R usqr = R(0);
#pragma unroll
      for (int d = 0; d < D; ++d) usqr = usqr + J[d] * J[d];
      if constexpr (EXACT) {
        R feq[Q];
        sfor<0, Q>([&](auto nn) { feq[decltype(nn)::value] = species_feq_exact<D, decltype(nn)::value, R>(r, J, usqr); });
        if constexpr (!MRT) {
#pragma unroll
          for (int n = 0; n < Q; ++n) g[n] = g[n] - (g[n] - feq[n]) / sr.tau;
        } else {
          R dfi[Q];
#pragma unroll
          for (int n = 0; n < Q; ++n) dfi[n] = g[n] - feq[n];
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
            const R coef = sr.srate[k] * md / R(L::mmt(k));
            sfor<0, Q>([&](auto ii) {
              constexpr int i = decltype(ii)::value;
              constexpr int v = L::mt(i, k);
              if constexpr (v == 1) g[i] = g[i] - coef;
              else if constexpr (v == -1) g[i] = g[i] + coef;
              else if constexpr (v != 0) g[i] = g[i] - coef * R(v);
            });
          });
        }
      } else {
        // feq_n = r W~_n (A_n + B_n) with A_0 = 0, A_n = 1.5 (d_k = 0)
        const R cu_axis = R(1.5 * L::w(1)) * usqr, cu_diag = R(1.5 * L::w(Q - 1)) * usqr;
        R feq[Q];
        sfor<0, Q>([&](auto nn) {
          constexpr int n = decltype(nn)::value;
          if constexpr (n == 0) {
            feq[0] = r * (R(-0.5) * usqr);
          } else {
            R ud = R(0);
            sfor<0, D>([&](auto dd) {
              constexpr int d = decltype(dd)::value;
              constexpr int cc = L::c(n, d);
              if constexpr (cc > 0) ud = ud + J[d];
              if constexpr (cc < 0) ud = ud - J[d];
            });
            constexpr double w = L::w(n);
            feq[n] = r * (R(1.5 * w) + ud * (R(3 * w) + R(4.5 * w) * ud) - (n <= L::NAXIS ? cu_axis : cu_diag));
          }
        });
        R fo[Q];
        const R keep = R(1) - sr.s0;
#pragma unroll
        for (int n = 0; n < Q; ++n) fo[n] = keep * g[n] + sr.s0 * feq[n];
        if (MRT && sr.spec_mask) {
          sfor<0, Q>([&](auto kk) {
            constexpr int k = decltype(kk)::value;
            if (sr.spec_mask & (1u << k)) {
              R md = R(0);
              sfor<0, Q>([&](auto ii) {
                constexpr int i = decltype(ii)::value;
                constexpr int v = L::mt(i, k);
                if constexpr (v == 1) md = md + (g[i] - feq[i]);
                else if constexpr (v == -1) md = md - (g[i] - feq[i]);
                else if constexpr (v != 0) md = md + R(v) * (g[i] - feq[i]);
              });
              const R ck = sr.dspec[k] * md;
              sfor<0, Q>([&](auto ii) {
                constexpr int i = decltype(ii)::value;
                constexpr int v = L::mt(i, k);
                if constexpr (v == 1) fo[i] = fo[i] - ck;
                else if constexpr (v == -1) fo[i] = fo[i] + ck;
                else if constexpr (v != 0) fo[i] = fo[i] - ck * R(v);
              });
            }
          });
        }
#pragma unroll
        for (int n = 0; n < Q; ++n) g[n] = fo[n];
      }
    }
    // push with bounceback, as the flow
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      constexpr int o = opp<D>(n);
      T* dst;
      if constexpr (n == 0) {
        dst = gout + (long long)(s * Q) * N + c;
      } else {
        constexpr int cx = L::c(n, 0), cy = L::c(n, 1), cz = D == 3 ? L::c(n, 2) : 0;
        const bool pore = ((links >> n) & 1u) != 0u;
        T* const base = gout + (long long)(s * Q + (pore ? n : o)) * N;
        dst = base + (pore ? h.template at<cx, cy, cz>() : c);
      }
      st_sp<T, R>(dst, g[n], P);
    });
  }
}

template <int D, bool MRT, bool EXACT, class T, class R>
__global__ void __launch_bounds__(128) k_species(SpeciesArgs a_in) {
  const SpeciesArgs a = a_in;
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  species_site<D, MRT, EXACT, T, R>(a, x, y, z);
}

// TransportFiInit (lbm_transport.F90:320-334): g = geq of the initial
// concentration and flux ([(cell*D + d)*ns + sp], natural order) on pore
// cells, 0 elsewhere.
template <int D, class T, class R>
__global__ void __launch_bounds__(128) k_species_init(SpeciesArgs a_in, const double* conc, const double* flux) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const SpeciesArgs a = a_in;
  const SpeciesPhysT<R>& P = *reinterpret_cast<const SpeciesPhysT<R>*>(a.phys);
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  const bool pore = __ldg(a.mask + idx) == 0;
  T* gout = reinterpret_cast<T*>(a.gout);
  for (int s = 0; s < a.ns; ++s) {
    R r = pore ? R(conc[idx * a.ns + s]) : R(0), J[D], usqr = R(0);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      J[d] = (pore && flux) ? R(flux[(idx * D + d) * a.ns + s]) : R(0);
      usqr = usqr + J[d] * J[d];
    }
    sfor<0, Q>([&](auto nn) {
      constexpr int n = decltype(nn)::value;
      const R v = pore ? species_feq_exact<D, n, R>(r, J, usqr) : R(0);
      st_sp<T, R>(gout + (long long)(s * Q + n) * a.g.n + idx, v, P);
    });
  }
}

// TransportCollisionD2 collides the cells with walls > 0 (lbm_transport.F90:450)
// toward the equilibrium of their moments, which are zero on walls, so their
// equilibrium is zero too.  Wall cells hold populations only next to specular
// walls; this is their collision there, in the operation order of the exact
// form (SRT g - (g - 0) / tau; MRT with the differences g - 0), in place in
// a.gout, before the specular exceptions read them.
template <int D, bool MRT, class T, class R>
__global__ void __launch_bounds__(128) k_species_wall_collide(SpeciesArgs a_in) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const SpeciesArgs a = a_in;
  const SpeciesPhysT<R>& P = *reinterpret_cast<const SpeciesPhysT<R>*>(a.phys);
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  if (__ldg(a.mask + idx) == 0) return;
  T* g0 = reinterpret_cast<T*>(a.gout);
  for (int s = 0; s < a.ns; ++s) {
    const SpecieRelax<R>& sr = P.sp[s];
    R g[Q];
#pragma unroll
    for (int n = 0; n < Q; ++n) g[n] = ld_sp<T, R>(g0 + (long long)(s * Q + n) * a.g.n + idx, P);
    if constexpr (!MRT) {
#pragma unroll
      for (int n = 0; n < Q; ++n) g[n] = g[n] - (g[n] - R(0)) / sr.tau;
    } else {
      R dfi[Q];
#pragma unroll
      for (int n = 0; n < Q; ++n) dfi[n] = g[n] - R(0);
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
        const R coef = sr.srate[k] * md / R(L::mmt(k));
        sfor<0, Q>([&](auto ii) {
          constexpr int i = decltype(ii)::value;
          constexpr int v = L::mt(i, k);
          if constexpr (v == 1) g[i] = g[i] - coef;
          else if constexpr (v == -1) g[i] = g[i] + coef;
          else if constexpr (v != 0) g[i] = g[i] - coef * R(v);
        });
      });
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) st_sp<T, R>(g0 + (long long)(s * Q + n) * a.g.n + idx, g[n], P);
  }
}

// Species fields in natural order: what 9 populations, 10 concentration,
// 11 flux (zero on walls, as TransportUpdateMoments).  With a.mask null every
// cell's populations are read (wall cells hold populations next to specular
// walls); the moments need the mask.
template <int D, class T, class R>
__global__ void __launch_bounds__(128) k_species_fields(SpeciesArgs a_in, int what, double* out) {
  using L = Lat<D>;
  constexpr int Q = L::Q;
  const SpeciesArgs a = a_in;
  const SpeciesPhysT<R>& P = *reinterpret_cast<const SpeciesPhysT<R>*>(a.phys);
  int x, y, z;
  long long idx;
  if (!site_of(a.g, x, y, z, idx)) return;
  const bool pore = !a.mask || __ldg(a.mask + idx) == 0;
  const T* gin = reinterpret_cast<const T*>(a.gin);
  const int ns = a.ns;
  for (int s = 0; s < ns; ++s) {
    double g[Q];
    for (int n = 0; n < Q; ++n) {
      g[n] = pore ? double(ld_sp<T, R>(gin + (long long)(s * Q + n) * a.g.n + idx, P)) : 0.0;
      if (what == 9) out[(idx * Q + n) * ns + s] = g[n];
    }
    if (what == 10) {
      double r = 0.0;
      for (int n = 0; n < Q; ++n) r = r + g[n];
      out[idx * ns + s] = r;
    } else if (what == 11) {
      for (int d = 0; d < D; ++d) {
        double j = 0.0;
        for (int n = 0; n < Q; ++n) {
          const int cc = L::c(n, d);
          if (cc > 0) j = j + g[n];
          if (cc < 0) j = j - g[n];
        }
        out[(idx * D + d) * ns + s] = j;
      }
    }
  }
}

}  // namespace tx
