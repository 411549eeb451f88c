// Host-side parameter handling of the flow step: validation of tx_params,
// translation into the kernels' parameter block, and the wall-code mapping.
// Plain C++ (no CUDA calls), shared by the C ABI and the host emulation of
// the kernels.
#pragma once
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/taxila_gb300.h"
#include "tx_kernels.cuh"
#include "tx_species.cuh"

namespace tx {

// Component counts compiled into the library.
constexpr int kMaxBuiltComponents = 2;

inline int validate(const tx_params* p, std::string* why) {
  auto bad = [&](const std::string& s) {
    *why = s;
    return TX_ERR_ARG;
  };
  if (p->discretization != TX_D3Q19 && p->discretization != TX_D2Q9) return bad("discretization must be TX_D3Q19 or TX_D2Q9");
  const int D = p->discretization == TX_D3Q19 ? 3 : 2;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1) return bad("lattice sizes must be >= 1");
  if (D == 2 && p->nz != 1) return bad("D2Q9 needs nz = 1");
  if ((long long)p->nx * p->ny * p->nz >= (1ll << 31)) return bad("lattices of 2^31 sites or more are not supported");
  if (p->nz > 65535) return bad("nz must be <= 65535");
  if (p->ncomponents < 1 || p->ncomponents > TX_MAX_COMPONENTS) return bad("ncomponents out of range");
  if (p->ncomponents > kMaxBuiltComponents)
    return bad("ncomponents > " + std::to_string(kMaxBuiltComponents) + " is not built into this library");
  if (p->nminerals < 0 || p->nminerals > TX_MAX_MINERALS) return bad("nminerals out of range");
  if (p->relaxation_mode != TX_RELAX_SRT && p->relaxation_mode != TX_RELAX_MRT) return bad("relaxation_mode must be 0 or 1");
  if (!(p->isotropy_order == 4 || p->isotropy_order == 8 || (D == 2 && p->isotropy_order == 10)))
    return bad(D == 3 ? "isotropy_order must be 4 or 8 for D3Q19 (the reference errors on 10)"
                      : "isotropy_order must be 4, 8 or 10");
  if (p->precision < TX_PREC_F64 || p->precision > TX_PREC_F32_F16) return bad("unknown precision form");
  if (p->exact && p->precision != TX_PREC_F64) return bad("exact operation order exists for the FP64 form only");
  if (!(p->storage_scale >= 0.0) || !std::isfinite(p->storage_scale) || p->storage_scale > 1e30)
    return bad("storage_scale must be finite and >= 0");
  for (int a = 0; a < D; ++a) {
    const int lo = p->bc_flags[2 * a], hi = p->bc_flags[2 * a + 1];
    if ((lo == TX_BC_PERIODIC) != (hi == TX_BC_PERIODIC)) return bad("periodic faces must come in pairs");
    const int ext = a == 0 ? p->nx : (a == 1 ? p->ny : p->nz);
    if (lo == TX_BC_PERIODIC && ext < 3) return bad("periodic axes need at least 3 sites");
  }
  // exterior BCs with the reference's own restrictions (FlowParseBC, FlowSetUpBCs,
  // FlowApplyBCs, FlowUpdateDensityFromPressure in lbm_flow.F90)
  bool has_po = false, has_fo = false;
  for (int f = 0; f < 2 * D; ++f) {
    const int v = p->bc_flags[f], S = p->ncomponents;
    const std::string face = "face " + std::to_string(f + 1) + ": ";
    if (v != TX_BC_NULL && v != TX_BC_PERIODIC && bc_class(v) == kClsNone) return bad(face + "unknown BC kind");
    if ((v == TX_BC_PRESSURE || v == TX_BC_FLUX) && S != 1)
      return bad(face + "pressure and flux BCs are single-component BCs (use the _inlet forms)");
    if ((v == TX_BC_PRESSURE_INLET || v == TX_BC_PRESSURE_OUTLET) && S > 2)
      return bad(face + "Invalid number of components for flow");
    if (v == TX_BC_FLUX_INLET && S > 2) return bad(face + "BC flux inlet only implemented for 1 or 2 components.");
    if (v == TX_BC_REFLECTING && D == 2 && f == 0)
      return bad(face + "reflecting XM face of D2Q9: the reference reads ci(p, Z) past its direction table there");
    for (int k = 0; k < 3 * TX_MAX_COMPONENTS; ++k)
      if (!std::isfinite(p->bc_data[f][k])) return bad(face + "bc_data must be finite");
    has_po |= v == TX_BC_PRESSURE_OUTLET;
    has_fo |= v == TX_BC_FLUX_OUTLET;
  }
  if (has_po && p->ncomponents != 1 && (std::fabs(p->g[0][0]) > 1e-10 || p->use_nonideal_eos))
    return bad("Pressure outlet not implemented for non-ideal EOS or g11 or g22 /= 0");
  if (has_po && has_fo)
    return bad("pressure and flux outlets together: the reference's flux-outlet update writes its values into the "
               "pressure-outlet faces");
  if (p->use_nonideal_eos) {
    for (int m = 0; m < p->ncomponents; ++m) {
      const int t = p->eos[m];
      if (t < TX_EOS_RHO || t > TX_EOS_PR) return bad("Invalid EOS type");
      if (t == TX_EOS_SC && !(p->eos_coef[m][0] != 0.0)) return bad("EOS sc: rho0 must be nonzero");
      if (t == TX_EOS_PR && (!(p->eos_coef[m][0] > 0.0) || !(p->eos_coef[m][1] > 0.0) || !(p->eos_coef[m][2] > 0.0) ||
                             p->g[m][m] == 0.0))
        return bad("EOS pr: a, b and T must be > 0 and the self coupling g_mm nonzero");
    }
  }
  if (p->nspecies < 0 || p->nspecies > TX_MAX_COMPONENTS) return bad("nspecies out of range");
  if (p->nspecies > 0) {
    if (p->species_relaxation_mode != TX_RELAX_SRT && p->species_relaxation_mode != TX_RELAX_MRT)
      return bad("species_relaxation_mode must be 0 or 1");
    for (int s = 0; s < p->nspecies; ++s)
      if (p->species_relaxation_mode == TX_RELAX_SRT && !(p->species_tau[s] > 0.0)) return bad("species tau must be > 0");
  }
  for (int m = 0; m < p->ncomponents; ++m) {
    if (!std::isfinite(p->rho0[m])) return bad("rho0 must be finite");
    if (p->relaxation_mode == TX_RELAX_SRT && !(p->tau[m] > 0.0)) return bad("tau must be > 0");
    if (!(p->mm[m] > 0.0)) return bad("molecular masses must be > 0");
  }
  return TX_OK;
}

inline void fill_phys_impl(const tx_params& p, int D, int S, int Q, Phys& P) {
  std::memset(&P, 0, sizeof(P));
  for (int m = 0; m < S; ++m) {
    P.tau[m] = p.tau[m];
    P.inv_tau[m] = 1.0 / p.tau[m];
    P.cs2[m] = 1.0 / 3.0;                     // lbm_relaxation.F90:82
    P.inv_cs2[m] = 3.0;
    P.dk[m] = 1. - 2. / (3. * p.mm[m]);        // lbm_component.F90:158
    P.mm[m] = p.mm[m];
    const double s_c = p.relaxation_mode == TX_RELAX_SRT ? 1.0 / p.tau[m] : p.s_c[m];  // lbm_relaxation.F90:133
    P.mmot[m] = p.mm[m] * s_c;
    for (int k = 0; k < S; ++k) P.g[m][k] = p.g[m][k];
    const double rates[7] = {p.s_c[m], p.s_e[m], p.s_e2[m], p.s_q[m], p.s_nu[m], p.s_pi[m], p.s_m[m]};
    for (int k = 0; k < Q; ++k) {
      const int r = D == 3 ? rate_of<3>(k) : rate_of<2>(k);
      const int mmt = D == 3 ? Lat<3>::mmt(k) : Lat<2>::mmt(k);
      P.srate[m][k] = rates[r];
      P.srate_mmt[m][k] = rates[r] / mmt;
    }
    // fast form: base rate = the rate most moments share (1/tau for BGK)
    if (p.relaxation_mode == TX_RELAX_SRT) {
      P.s0[m] = 1.0 / p.tau[m];
      P.spec_mask[m] = 0u;
    } else {
      int best = 0, best_count = -1;
      for (int k = 0; k < Q; ++k) {
        int c = 0;
        for (int j = 0; j < Q; ++j) c += P.srate[m][j] == P.srate[m][k];
        if (c > best_count) { best_count = c; best = k; }
      }
      P.s0[m] = P.srate[m][best];
      P.spec_mask[m] = 0u;
      for (int k = 0; k < Q; ++k) {
        if (P.srate[m][k] == P.s0[m]) continue;
        const int mmt = D == 3 ? Lat<3>::mmt(k) : Lat<2>::mmt(k);
        P.spec_mask[m] |= 1u << k;
        P.dspec[m][k] = (P.srate[m][k] - P.s0[m]) / mmt;
      }
    }
  }
  for (int q = 0; q < p.nminerals; ++q)
    for (int m = 0; m < S; ++m) P.gw[q + 1][m] = p.gw[q][m];
  for (int d = 0; d < 3; ++d) P.gvt[d] = p.gvt[d];
  // isotropy weights (lbm_discretization_d3q19.F90:199-230, d2q9:119-142)
  const int iso = p.isotropy_order;
  double* w = P.ffw;
  if (D == 3) {
    if (iso == 4) { w[1] = 1.0 / 6.0; w[2] = 1.0 / 12.0; }
    if (iso == 8) {
      w[1] = 4.0 / 45.0; w[2] = 1.0 / 21.0; w[3] = 2.0 / 105.0; w[4] = 5.0 / 504.0;
      w[5] = 1.0 / 315.0; w[6] = 1.0 / 630.0; w[8] = 1.0 / 5040.0;
    }
  } else {
    if (iso == 4) { w[1] = 1.0 / 3.0; w[2] = 1.0 / 12.0; }
    if (iso == 8) { w[1] = 4.0 / 21.0; w[2] = 4.0 / 45.0; w[4] = 1.0 / 60.0; w[5] = 2.0 / 315.0; w[8] = 1.0 / 5040.0; }
    if (iso == 10) {
      w[1] = 262.0 / 1785.0; w[2] = 93.0 / 1190.0; w[4] = 7.0 / 340.0; w[5] = 6.0 / 595.0;
      w[8] = 9.0 / 9520.0; w[9] = 2.0 / 5355.0; w[10] = 1.0 / 7140.0;
    }
  }
  for (int d = 0; d < D; ++d) {
    const double ws = D == 3 ? full_weight_sum<3>(iso, P.ffw, d) : full_weight_sum<2>(iso, P.ffw, d);
    P.inv_ws_full[d] = ws > 0.0 ? 1.0 / ws : 0.0;
  }
  P.c0 = 6.0;  // disc%c_0
  // fluid-solid weights 1./6., 1./12. (D3) and 1./3., 1./12. (D2): default-REAL literals
  if (p.literal_kind == 8) {
    P.fs_w_axis = D == 3 ? 1.0 / 6.0 : 1.0 / 3.0;
    P.fs_w_diag = 1.0 / 12.0;
  } else {
    P.fs_w_axis = D == 3 ? (double)(1.0f / 6.0f) : (double)(1.0f / 3.0f);
    P.fs_w_diag = (double)(1.0f / 12.0f);
  }
  const double eps15 = (double)1.e-15f;
  for (int m = 0; m < S; ++m)
    for (int k = 0; k < S; ++k)
      if (std::fabs(p.g[m][k]) > eps15) P.ff_on = 1;
  for (int q = 0; q < p.nminerals; ++q)
    for (int m = 0; m < S; ++m)
      if (std::fabs(p.gw[q][m]) > eps15) P.fs_on = 1;
  P.body_on = p.body_forces != 0;
  for (int m = 0; m < S; ++m) P.rho0[m] = p.precision == TX_PREC_F64 ? 0.0 : p.rho0[m];
  P.sscale = p.precision == TX_PREC_F32_F16 && p.storage_scale > 0.0 ? p.storage_scale : 1.0;
  // non-ideal EOS (EOSSetFromOptions_*, lbm_eos.F90:90-300); PR keeps a, b, T, alpha(T)
  P.eos_on = p.use_nonideal_eos ? 1 : 0;
  for (int m = 0; m < S; ++m) {
    P.eos[m] = p.use_nonideal_eos ? p.eos[m] : TX_EOS_RHO;
    for (int k = 0; k < 4; ++k) P.eos_c[m][k] = p.eos_coef[m][k];
    if (P.eos[m] == TX_EOS_PR) {
      const double a = p.eos_coef[m][0], b = p.eos_coef[m][1], T = p.eos_coef[m][2], om = p.eos_coef[m][3];
      // the Fortran source spells these constants as default-kind (single
      // precision) literals: they enter the double expressions rounded to float
      const double Tc = a / b * double(0.0778f) / double(0.45724f) / 1.;
      const double t =
          1. + (double(0.37464f) + double(1.54226f) * om - double(0.26992f) * (om * om)) * (1. - std::sqrt(T / Tc));
      P.eos_c[m][3] = t * t;
    }
  }
  for (int m = 0; m < S; ++m) {
    const double mm = p.mm[m], rel = (mm - 1.0) / mm;  // 0 for unit mass
    P.A0[m] = D == 3 ? P.dk[m] : (1.0 + 5.0 * P.dk[m]) / 6.0;
    P.An[m] = 1.0 / mm;  // 1.5 (1 - dk)
    P.cA[m][0] = (D == 3 ? 2.0 / 3.0 : 5.0 / 9.0) * rel * P.rho0[m];
    P.cA[m][1] = -(D == 3 ? 1.0 / 18.0 : 1.0 / 9.0) * rel * P.rho0[m];
    P.cA[m][2] = -(1.0 / 36.0) * rel * P.rho0[m];
    P.WAc[m][0] = P.A0[m];
    P.WAc[m][1] = (D == 3 ? Lat<3>::w(1) : Lat<2>::w(1)) * P.An[m];
    P.WAc[m][2] = (D == 3 ? Lat<3>::w(18) : Lat<2>::w(8)) * P.An[m];
    P.keep[m] = 1.0 - P.s0[m];
    P.kfac[m] = 3.0 - 1.5 * P.s0[m];
    for (int k = 0; k < S; ++k) P.c0g[m][k] = P.c0 * P.g[m][k];
  }
  for (int d = 0; d < D; ++d)
    for (int w = 0; w < 12; ++w) P.ffwq[d][w] = P.ffw[w] * P.inv_ws_full[d];
  P.inv_sscale = 1.0 / P.sscale;
  P.wa_shared = 1;
  for (int m = 1; m < S; ++m)
    for (int q = 0; q < 3; ++q)
      if (P.WAc[m][q] != P.WAc[0][q]) P.wa_shared = 0;
  P.ff_cross = S == 2 && P.c0g[0][0] == 0.0 && P.c0g[1][1] == 0.0;
  P.mmot_shared = 1;
  for (int m = 1; m < S; ++m)
    if (P.mmot[m] != P.mmot[0]) P.mmot_shared = 0;
}

// Whether the fast MRT step needs its general rate path: some component has
// moments with a rate other than s0 beyond the s_nu set.  Otherwise the
// kernels compiled without that path run (fewer registers).
inline bool needs_general_rates(const tx_params& p) {
  if (p.relaxation_mode != TX_RELAX_MRT) return false;
  const int D = p.discretization == TX_D3Q19 ? 3 : 2, S = p.ncomponents, Q = D == 3 ? 19 : 9;
  Phys ph;
  fill_phys_impl(p, D, S, Q, ph);
  const unsigned nu = D == 3 ? stress_mask<3>() : stress_mask<2>();
  for (int m = 0; m < S; ++m)
    if (ph.spec_mask[m] != 0u && ph.spec_mask[m] != nu) return true;
  return false;
}

// ------------------------------------------------------------ exterior BCs
inline long long face_area_of(int D, int nx, int ny, int nz, int f) {
  const int a = f / 2;
  if (D == 2) return a == 0 ? ny : nx;
  return a == 0 ? (long long)ny * nz : (a == 1 ? (long long)nx * nz : (long long)nx * ny);
}

// FlowSetUpBCsD3/D2 (lbm_flow.F90:1311-1956): the values of every node of
// face f, in the reference's (s, ndims) block v[d * S + m] (zero elsewhere).
inline void face_node_values(const tx_params& p, int D, int f, double c0, double* v) {
  const int S = p.ncomponents, a = f / 2;
  const bool plus = (f % 2) == 1;
  const double* bd = p.bc_data[f];
  for (int k = 0; k < S * D; ++k) v[k] = 0.0;
  switch (p.bc_flags[f]) {
    case TX_BC_DENSITY:
      for (int m = 0; m < S; ++m) v[m] = bd[m];
      break;
    case TX_BC_PRESSURE:
    case TX_BC_PRESSURE_INLET: {
      double dens[2] = {0.0, 0.0};
      density_from_pressure(S, c0, S > 1 ? p.g[1][0] : 0.0, bd[0], bd[1], dens);
      for (int m = 0; m < S; ++m) v[m] = dens[m];
      break;
    }
    case TX_BC_PRESSURE_OUTLET:
      v[0] = bd[0];
      break;
    case TX_BC_MOMENTUM:
      for (int m = 0; m < S; ++m)
        for (int d = 0; d < D; ++d) v[d * S + m] = bd[m * D + d];
      break;
    case TX_BC_FLUX:
    case TX_BC_FLUX_INLET:
      if (S == 1) {
        v[a * S] = plus ? -bd[0] : bd[0];
      } else {  // two components: no sign change on the plus faces, as written
        v[a * S] = bd[0] * bd[1];
        v[a * S + 1] = bd[0] * (1.0 - bd[1]);
      }
      break;
    case TX_BC_FLUX_OUTLET:
      v[a * S] = plus ? -bd[0] : bd[0];
      break;
    case TX_BC_VELOCITY:
      for (int d = 0; d < D; ++d) v[d * S] = bd[d];
      break;
  }
}

// Face flags, classes and BCApply's class order (lbm_bc.F90:781-807); vals
// pointers are left to the caller.
inline void setup_faces(const tx_params& p, int D, Faces* fc) {
  std::memset(fc, 0, sizeof(*fc));
  bool seen[8] = {false};
  for (int f = 0; f < 6; ++f) {
    const int cls = f < 2 * D ? bc_class(p.bc_flags[f]) : kClsNone;
    fc->cls[f] = cls;
    fc->on[f] = cls == kClsDir || cls == kClsNeu || cls == kClsVel;
    fc->dir[f] = cls == kClsDir;
    if (cls != kClsDir && cls != kClsNone) fc->post = 1;
    if (cls != kClsNone && !seen[cls]) {
      seen[cls] = true;
      fc->order[fc->norder++] = cls;
    }
  }
}

// Whether a face needs node values on the device.
inline bool face_has_values(const tx_params& p, int D, int f) {
  if (f >= 2 * D) return false;
  const int cls = bc_class(p.bc_flags[f]);
  return cls == kClsDir || cls == kClsNeu || cls == kClsVel;
}

// Two-component pressure outlets refresh their values every step.
inline bool has_outlet_update(const tx_params& p, int D) {
  if (p.ncomponents == 1) return false;
  for (int f = 0; f < 2 * D; ++f)
    if (p.bc_flags[f] == TX_BC_PRESSURE_OUTLET) return true;
  return false;
}

// The face-pass grid: faces with a node correction, in XM..ZP order.
inline FaceShell face_shell(const tx_params& p, int D, int nx, int ny, int nz) {
  FaceShell sh{};
  sh.start[0] = 0;
  for (int f = 0; f < 2 * D; ++f) {
    if (bc_class(p.bc_flags[f]) == kClsNone) continue;
    sh.face[sh.nf] = f;
    sh.start[sh.nf + 1] = sh.start[sh.nf] + face_area_of(D, nx, ny, nz, f);
    ++sh.nf;
  }
  return sh;
}

// Species relaxation (SpecieSetFromOptions, lbm_species.F90:111-133; the
// MRT rate map of DiscretizationSetupRelax) and the fast form's base rate.
inline void fill_species_phys(const tx_params& p, int D, SpeciesPhysT<double>& P) {
  std::memset(&P, 0, sizeof(P));
  const int Q = D == 3 ? 19 : 9;
  P.sscale = p.precision == TX_PREC_F32_F16 && p.storage_scale > 0.0 ? p.storage_scale : 1.0;
  P.inv_sscale = 1.0 / P.sscale;
  for (int s = 0; s < p.nspecies; ++s) {
    SpecieRelax<double>& r = P.sp[s];
    r.tau = p.species_tau[s];
    r.inv_tau = 1.0 / p.species_tau[s];
    for (int k = 0; k < Q; ++k) r.srate[k] = p.species_rates[s][D == 3 ? rate_of<3>(k) : rate_of<2>(k)];
    if (p.species_relaxation_mode == TX_RELAX_SRT) {
      r.s0 = 1.0 / p.species_tau[s];
    } else {
      int best = 0, best_count = -1;
      for (int k = 0; k < Q; ++k) {
        int c = 0;
        for (int j = 0; j < Q; ++j) c += r.srate[j] == r.srate[k];
        if (c > best_count) { best_count = c; best = k; }
      }
      r.s0 = r.srate[best];
      for (int k = 0; k < Q; ++k) {
        if (r.srate[k] == r.s0) continue;
        r.spec_mask |= 1u << k;
        r.dspec[k] = (r.srate[k] - r.s0) / (D == 3 ? Lat<3>::mmt(k) : Lat<2>::mmt(k));
      }
    }
  }
}

template <class R>
inline void convert_species(const SpeciesPhysT<double>& a, SpeciesPhysT<R>* b) {
  for (int s = 0; s < MAXC; ++s) {
    b->sp[s].tau = R(a.sp[s].tau);
    b->sp[s].inv_tau = R(a.sp[s].inv_tau);
    b->sp[s].s0 = R(a.sp[s].s0);
    b->sp[s].spec_mask = a.sp[s].spec_mask;
    for (int k = 0; k < 19; ++k) {
      b->sp[s].srate[k] = R(a.sp[s].srate[k]);
      b->sp[s].dspec[k] = R(a.sp[s].dspec[k]);
    }
  }
  b->sscale = R(a.sscale);
  b->inv_sscale = R(a.inv_sscale);
}

// Reference wall value (lbm_walls.F90:151-177) -> device mask code:
// 0 pore, 1..nminerals mineral, 255 any other wall (codes >= 998, unknown
// minerals, and the specular codes 900-902 where the caller resolves their
// routes: specular_ok; 902 is a plain wall in 2D).  Returns false, with the
// reason, for values the device path rejects: negative or non-finite values,
// and specular codes elsewhere.
inline bool wall_code(double v, int nminerals, uint8_t* code, const char** why, int D = 3, bool specular_ok = false) {
  if (v == 0.0) {
    *code = 0;
    return true;
  }
  if (!(v > 0.0) || !std::isfinite(v)) {
    *why = "wall codes must be 0 (pore) or positive";
    return false;
  }
  if ((v == 900.0 || v == 901.0 || (v == 902.0 && D == 3)) && !specular_ok) {
    *why = "specular (no-stick) wall codes 900-902 need a single-lattice FP64 handle";
    return false;
  }
  const int mineral = v < 998.0 ? (int)v : 0;
  *code = (mineral >= 1 && mineral <= nminerals) ? (uint8_t)mineral : (uint8_t)255;
  return true;
}

}  // namespace tx
