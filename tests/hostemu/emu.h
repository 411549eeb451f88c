// Host emulation of the flow step: the kernels of tx_kernels.cuh run one
// thread at a time on the CPU, with the parameter translation and launch
// shapes of the C ABI (tx_abi.cu).  Test infrastructure: a sanitizer build
// checks every index the kernels form, and the results are compared with the
// oracle on the CPU.
#pragma once
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tx_host_params.h"
#include "tx_pair.cuh"
#include "tx_specular.cuh"

namespace emu {

using namespace tx;

struct Case {
  tx_params p;
  int nsteps = 0;
  int from_fi = 0;            // 0: tx_upload_state + tx_init, 1: tx_upload_fi + tx_init
  std::vector<double> walls;  // [N]
  std::vector<double> init;   // rho [N*S] or fi [N*S*Q], natural order
  std::vector<double> conc;   // species concentrations [N*ns] (empty: no species)
};

struct Result {
  std::vector<double> fi, rho, flux, forces;  // natural order, as tx_download
  std::vector<double> sfi, srho, sflux;       // species fields (when the case has species)
};

// the library's launch3 shape, walked block by block and thread by thread
template <class F>
void launch3(const Geo& g, int threads, F&& f) {
  int bx = ((g.nx + 31) / 32) * 32;
  if (bx > 128) bx = 128;
  if (bx > threads) bx = threads;
  int by = threads / bx;
  if (by < 1) by = 1;
  blockDim = dim3{(unsigned)bx, (unsigned)by, 1};
  gridDim = dim3{(unsigned)((g.nx + bx - 1) / bx), (unsigned)((g.ny + by - 1) / by), (unsigned)g.nz};
  for (unsigned bz = 0; bz < gridDim.z; ++bz)
    for (unsigned byy = 0; byy < gridDim.y; ++byy)
      for (unsigned bxx = 0; bxx < gridDim.x; ++bxx)
        for (unsigned ty = 0; ty < blockDim.y; ++ty)
          for (unsigned tx_ = 0; tx_ < blockDim.x; ++tx_) {
            blockIdx = dim3{bxx, byy, bz};
            threadIdx = dim3{tx_, ty, 0};
            f();
          }
}

template <class F>
void launch1(long long n, int bs, F&& f) {
  blockDim = dim3{(unsigned)bs, 1, 1};
  gridDim = dim3{(unsigned)((n + bs - 1) / bs), 1, 1};
  for (unsigned b = 0; b < gridDim.x; ++b)
    for (int t = 0; t < bs; ++t) {
      blockIdx = dim3{b, 0, 0};
      threadIdx = dim3{(unsigned)t, 0, 0};
      f();
    }
}

// The library's natural-order conversions move tiles of sites through shared
// memory with a barrier between the two halves, which a one-thread-at-a-time
// walk cannot run; here they are plain loops with the same arithmetic (the GPU
// tests compare every download of the kernels with the oracle).
template <int D, int S, class T, class R>
void pops_from_natural(const double* in, const uint8_t* mask, long long N, Shift sh, T* f) {
  constexpr int Q = Lat<D>::Q;
  for (long long idx = 0; idx < N; ++idx)
    for (int n = 0; n < Q; ++n)
      for (int m = 0; m < S; ++m) {
        const bool wall = mask && mask[idx] != 0;
        double x = wall ? 0.0 : in[(idx * Q + n) * S + m];
        if constexpr (kShifted<T>) x = wall ? 0.0 : (x - Lat<D>::w(n) * sh.rho0[m]) * sh.scale;
        if constexpr (std::is_same<T, double>::value)
          f[(long long)(m * Q + n) * N + idx] = x;
        else
          St<T>::st(f + (long long)(m * Q + n) * N + idx, R(x));
      }
}
template <int D, int S, class T, class R>
void pops_to_natural(const T* f, const uint8_t* mask, long long N, Shift sh, double* out) {
  constexpr int Q = Lat<D>::Q;
  for (long long idx = 0; idx < N; ++idx)
    for (int n = 0; n < Q; ++n)
      for (int m = 0; m < S; ++m) {
        double x = 0.0;
        if (!(mask && mask[idx] != 0)) {
          x = double(St<T>::ld(f + (long long)(m * Q + n) * N + idx));
          if constexpr (kShifted<T>) x = x / sh.scale + Lat<D>::w(n) * sh.rho0[m];
        }
        out[(idx * Q + n) * S + m] = x;
      }
}

template <int D, int S, int ISO, bool MRT, bool EXACT, class T, class R, class RT>
std::string run(const Case& c, Result& out) {
  constexpr int Q = Lat<D>::Q;
  const tx_params& p = c.p;
  Geo g{};
  g.nx = p.nx;
  g.ny = p.ny;
  g.nz = D == 3 ? p.nz : 1;
  for (int a = 0; a < 3; ++a) g.per[a] = a < D ? p.bc_flags[2 * a] == TX_BC_PERIODIC : 1;
  g.n = (long long)g.nx * g.ny * g.nz;
  const long long N = g.n;

  Phys ph{};
  fill_phys_impl(p, D, S, Q, ph);
  PhysT<R> P{};
  if constexpr (std::is_same<R, double>::value)
    P = ph;
  else
    convert_phys(ph, &P);

  // specular walls (as tx_upload_walls)
  bool spec = false;
  for (long long i = 0; i < N; ++i) spec = spec || specular_axis(c.walls[(size_t)i], D) >= 0;
  std::vector<uint8_t> mask((size_t)N);
  for (long long i = 0; i < N; ++i) {
    const char* why = nullptr;
    if (!wall_code(c.walls[(size_t)i], p.nminerals, &mask[(size_t)i], &why, D, spec)) return why;
  }
  SpecRoutes routes, sroutes;  // the flow's, and the species' (no BCPreStream copies)
  if (spec) {
    const int nn[3] = {g.nx, g.ny, g.nz};
    std::vector<long long> init_nz;  // wall slots with uploaded content
    if (c.from_fi)
      for (long long i = 0; i < N; ++i)
        if (mask[(size_t)i] != 0)
          for (int n = 0; n < Q; ++n)
            for (int m = 0; m < S; ++m)
              if (c.init[(size_t)((i * Q + n) * S + m)] != 0.0) {
                init_nz.push_back((long long)n * N + i);
                break;
              }
    bool pre[6];
    for (int f = 0; f < 6; ++f) pre[f] = face_has_values(p, D, f);
    std::string why = specular_routes(c.walls.data(), D, nn, g.per, pre, &init_nz, false, &routes);
    if (why.empty() && p.nspecies > 0) {
      const bool none[6] = {false, false, false, false, false, false};
      const bool mix = D == 2 && p.species_relaxation_mode == TX_RELAX_MRT;
      why = specular_routes(c.walls.data(), D, nn, g.per, none, nullptr, mix, &sroutes);
    }
    if (!why.empty()) return why;
  }
  const long long ne = (long long)routes.dst.size();
  std::vector<T> spec_tmp((size_t)(ne * S + 1));
  const uint8_t* pop_mask = spec ? nullptr : mask.data();
  int spec_fresh = 2, spec_fresh_sp = 2;
  std::vector<uint32_t> links((size_t)N);
  launch3(g, 256, [&] { k_links<D>(mask.data(), g, links.data()); });

  std::vector<T> f0((size_t)N * S * Q), f1((size_t)N * S * Q);
  std::memset(f0.data(), 0, f0.size() * sizeof(T));
  std::memset(f1.data(), 0, f1.size() * sizeof(T));
  std::vector<RT> rho((size_t)N * S, RT(0));
  std::vector<RT> psi(p.use_nonideal_eos ? (size_t)N * S : 0, RT(0));
  std::vector<double> facevals[6];
  Faces faces{};
  setup_faces(p, D, &faces);
  const FaceShell shell = face_shell(p, D, g.nx, g.ny, g.nz);
  for (int f = 0; f < 2 * D; ++f) {
    if (!face_has_values(p, D, f)) continue;
    const long long area = face_area_of(D, g.nx, g.ny, g.nz, f);
    double nv[3 * TX_MAX_COMPONENTS];
    face_node_values(p, D, f, ph.c0, nv);
    facevals[f].resize((size_t)area * S * D);
    for (int k = 0; k < S * D; ++k)
      for (long long q = 0; q < area; ++q) facevals[f][(size_t)(k * area + q)] = nv[k];
    faces.vals[f] = facevals[f].data();
  }

  T* buf[2] = {f0.data(), f1.data()};
  int cur = 0;
  unsigned step = 0;
  // the paired step of the FP32-arithmetic forms on lattices with an even site count
  constexpr bool kPairForm = !EXACT && std::is_same<R, float>::value;
  const bool paired = kPairForm && N % 2 == 0;
  int rest = -1;
  auto args = [&](int in, int o) {
    StepArgs a{};
    a.fin = buf[in];
    a.fout = buf[o];
    a.rho = rho.data();
    a.psi = psi.empty() ? nullptr : psi.data();
    a.mask = mask.data();
    a.links = links.data();
    a.phys = &P;
    a.g = g;
    a.faces = faces;
    a.step = step;
    a.rest = rest;
    return a;
  };
  if constexpr (kPairForm) {
    if (paired) {
      unsigned cnt = 0;
      const StepArgs a = args(cur, cur);
      launch1(N / 2, 256, [&] { k_count_rest<D, ISO>(a, &cnt); });
      rest = (int)cnt;
    }
  }
  const Shift sh = shift_of(ph);
  if (c.from_fi) {
    pops_from_natural<D, S, T, R>(c.init.data(), pop_mask, N, sh, buf[cur]);
  } else {
    for (long long i = 0; i < N; ++i)
      for (int m = 0; m < S; ++m)
        rho[(size_t)(i * S + m)] = RT(mask[(size_t)i] == 0 ? c.init[(size_t)(i * S + m)] - ph.rho0[m] : 0.0);
    if (!psi.empty())
      for (long long i = 0; i < N; ++i)
        if (mask[(size_t)i] == 0)
          for (int m = 0; m < S; ++m)
            psi[(size_t)(i * S + m)] =
                RT(eos_psi<double>(ph.eos[m], ph.eos_c[m], ph.g[m][m], ph.c0, c.init[(size_t)(i * S + m)]));
    const StepArgs a = args(cur, cur);
    launch3(g, 128, [&] { k_init<D, S, ISO, EXACT, T, R, RT>(a, nullptr); });
    if (spec) launch1(N, 256, [&] { k_spec_clear_walls<D, T>(buf[cur], mask.data(), N, S, sh); });  // empty wall cells
  }
  // the density pass as the library launches it (16-byte loads when N allows)
  auto density = [&](const StepArgs& a, int mode) {
    constexpr int VW = 16 / (int)sizeof(T);
    if (N % VW == 0)
      launch1(N / VW, 256, [&] { k_density_vec<D, S, T, R, RT>(a, mode); });
    else
      launch3(g, 256, [&] { k_density<D, S, T, R, RT>(a, mode); });
  };
  density(args(cur, cur), 1);
  // species: as tx_create / tx_upload_species / tx_init / tx_step
  const int NS = c.conc.empty() ? 0 : p.nspecies;
  SpeciesPhysT<double> sp{};
  fill_species_phys(p, D, sp);
  SpeciesPhysT<R> spR{};
  if constexpr (std::is_same<R, double>::value)
    spR = sp;
  else
    convert_species(sp, &spR);
  std::vector<T> g0((size_t)N * (NS ? NS : 1) * Q), g1(g0.size());
  std::memset(g0.data(), 0, g0.size() * sizeof(T));
  std::memset(g1.data(), 0, g1.size() * sizeof(T));
  T* gbuf[2] = {g0.data(), g1.data()};
  int gcur = 0;
  auto sargs = [&](int in, int o) {
    SpeciesArgs a{};
    a.gin = gbuf[in];
    a.gout = gbuf[o];
    a.links = links.data();
    a.mask = mask.data();
    a.phys = &spR;
    a.g = g;
    a.ns = NS;
    return a;
  };
  if (NS) {
    const SpeciesArgs a = sargs(gcur, gcur);
    launch3(g, 128, [&] { k_species_init<D, T, R>(a, c.conc.data(), nullptr); });
  }
  for (int t = 0; t < c.nsteps; ++t) {
    const StepArgs a = args(cur, 1 - cur);
    if (has_outlet_update(p, D))
      for (int f = 0; f < 2 * D; ++f)
        if (p.bc_flags[f] == TX_BC_PRESSURE_OUTLET)
          launch1(face_area_of(D, g.nx, g.ny, g.nz, f), 128, [&] {
            k_outlet<D, S, T, R, RT>(a, f, facevals[f].data(), p.bc_data[f][0], ph.c0, p.g[1][0]);
          });
    if (paired) {
      // the library's paired step: k_step_pair, then k_step_rest when pairs need it
      launch1((N / 2 + TX_PAIR_PER_THREAD - 1) / TX_PAIR_PER_THREAD, 128, [&] { k_step_pair<D, S, ISO, MRT, T>(a); });
      if (a.rest != 0) launch1(N / 2, 128, [&] { k_step_rest<D, S, ISO, MRT, T>(a); });
    } else {
      launch3(g, 128, [&] { k_step<D, S, ISO, MRT, EXACT, T, R, RT>(a); });
    }
    if (spec) {
      // the library's specular-wall pass: empty the wall slots of a fresh buffer,
      // then gather and scatter the exceptions to the ordinary push
      T* fo = buf[1 - cur];
      if (spec_fresh > 0) {
        launch1(N, 256, [&] { k_spec_clear_walls<D, T>(fo, mask.data(), N, S, sh); });
        --spec_fresh;
      }
      if (ne) {
        launch1(ne, 256, [&] { k_spec_gather<D, T>(buf[cur], fo, routes.src.data(), routes.dst.data(), ne, S, N, sh, spec_tmp.data()); });
        launch1(ne, 256, [&] { k_spec_scatter<T>(fo, routes.dst.data(), ne, S, (long long)Q * N, spec_tmp.data()); });
      }
    }
    density(a, 0);
    if (faces.post) launch1(shell.start[shell.nf], 128, [&] { k_faces<D, S, ISO, EXACT, T, R, RT>(a, shell); });
    cur = 1 - cur;
    ++step;
    if (NS) {
      const SpeciesArgs sa = sargs(gcur, 1 - gcur);
      if (p.species_relaxation_mode == TX_RELAX_MRT)
        launch3(g, 128, [&] { k_species<D, true, EXACT, T, R>(sa); });
      else
        launch3(g, 128, [&] { k_species<D, false, EXACT, T, R>(sa); });
      if (spec) {
        // the species stream and bounce back as the flow does, through their own
        // exception list (their storage has no rest state)
        Shift ssh{};
        ssh.scale = 1.0;
        if (D == 2) {
          // the reference's 2D transport collides wall cells, which hold populations here
          SpeciesArgs wa = sargs(gcur, gcur);
          if (p.species_relaxation_mode == TX_RELAX_MRT)
            launch3(g, 128, [&] { k_species_wall_collide<D, true, T, R>(wa); });
          else
            launch3(g, 128, [&] { k_species_wall_collide<D, false, T, R>(wa); });
        }
        T* go = gbuf[1 - gcur];
        if (spec_fresh_sp > 0) {
          launch1(N, 256, [&] { k_spec_clear_walls<D, T>(go, mask.data(), N, NS, ssh); });
          --spec_fresh_sp;
        }
        const long long nes = (long long)sroutes.dst.size();
        if (nes) {
          std::vector<T> stmp((size_t)(nes * NS + 1));
          launch1(nes, 256, [&] { k_spec_gather<D, T>(gbuf[gcur], go, sroutes.src.data(), sroutes.dst.data(), nes, NS, N, ssh, stmp.data()); });
          launch1(nes, 256, [&] { k_spec_scatter<T>(go, sroutes.dst.data(), nes, NS, (long long)Q * N, stmp.data()); });
        }
      }
      gcur = 1 - gcur;
    }
  }
  if (NS) {
    const SpeciesArgs sa = sargs(gcur, gcur);
    out.sfi.assign((size_t)N * NS * Q, 0.0);
    out.srho.assign((size_t)N * NS, 0.0);
    out.sflux.assign((size_t)N * NS * D, 0.0);
    SpeciesArgs sa9 = sa;
    if (spec) sa9.mask = nullptr;  // wall cells' populations too
    launch3(g, 128, [&] { k_species_fields<D, T, R>(sa9, 9, out.sfi.data()); });
    launch3(g, 128, [&] { k_species_fields<D, T, R>(sa, 10, out.srho.data()); });
    launch3(g, 128, [&] { k_species_fields<D, T, R>(sa, 11, out.sflux.data()); });
  }
  out.fi.assign((size_t)N * S * Q, 0.0);
  pops_to_natural<D, S, T, R>(buf[cur], pop_mask, N, sh, out.fi.data());
  const StepArgs a = args(cur, cur);
  out.rho.assign((size_t)N * S, 0.0);
  out.flux.assign((size_t)N * S * D, 0.0);
  out.forces.assign((size_t)N * S * D, 0.0);
  launch3(g, 128, [&] { k_moments<D, S, ISO, EXACT, T, R, RT>(a, 2, out.rho.data()); });
  launch3(g, 128, [&] { k_moments<D, S, ISO, EXACT, T, R, RT>(a, 3, out.flux.data()); });
  launch3(g, 128, [&] { k_moments<D, S, ISO, EXACT, T, R, RT>(a, 4, out.forces.data()); });
  return "";
}

// one entry per compiled combination; returns false when none matches
bool dispatch_d3_iso4(const Case& c, Result& out, std::string* err);
bool dispatch_d3_iso8(const Case& c, Result& out, std::string* err);
bool dispatch_d2(const Case& c, Result& out, std::string* err);
bool dispatch_forms(const Case& c, Result& out, std::string* err);

}  // namespace emu

// selects run<...> when the case's parameters match the combination
#define EMU_TRY(D_, S_, ISO_, MRT_, EXACT_, PREC_, T_, R_, RT_)                                          \
  if (c.p.ncomponents == S_ && c.p.isotropy_order == ISO_ && (c.p.relaxation_mode == TX_RELAX_MRT) == MRT_ && \
      (c.p.exact != 0) == EXACT_ && c.p.precision == PREC_) {                                          \
    *err = run<D_, S_, ISO_, MRT_, EXACT_, T_, R_, RT_>(c, out);                                       \
    return true;                                                                                       \
  }
