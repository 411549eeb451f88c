// emu <case.bin> <result.bin>: one flow run of the host emulation.
//
// case.bin:   tx_params (raw struct) | int32 nsteps | int32 from_fi |
//             walls [N] f64 | rho [N*S] or fi [N*S*Q] f64 (natural order) |
//             species concentrations [N*ns] f64 when params.nspecies > 0
// result.bin: fi [N*S*Q] | rho [N*S] | flux [N*D*S] | forces [N*D*S], then
//             species gi [N*ns*Q] | concentration [N*ns] | flux [N*D*ns], f64
// Exit status 0 on success, 2 for parameters the library rejects (message on
// stderr), 3 when the combination is not compiled into the emulation.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>

#include "emu.h"

using namespace emu;

static bool read_all(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

// emu norm: NormMax (the delta norm's screened running maximum) against the
// plain maximum of every FP64 quotient, on seeded sequences that mix ordinary
// values with zeros, ties, tiny and huge magnitudes, subnormals, NaN and inf.
static int norm_selftest() {
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> e(-320, 300), pick(0, 15);
  const double inf = std::numeric_limits<double>::infinity(), qnan = std::numeric_limits<double>::quiet_NaN();
  int bad = 0;
  for (int trial = 0; trial < 4000; ++trial) {
    const int n = 1 + (int)(g() % 400);
    const int mode = trial % 4;
    NormMax acc;
    double ref = 0.0;
    for (int i = 0; i < n; ++i) {
      double c, o;
      const int k = pick(g);
      if (mode == 0) {  // a converging field: relative changes around 1e-7 .. 1e-3
        c = 1.0 + u(g);
        o = c * (1.0 + u(g) * std::pow(10.0, -3 - (int)(g() % 5)));
      } else if (mode == 1) {  // magnitudes over the whole double range
        c = u(g) * std::ldexp(1.0, e(g));
        o = u(g) * std::ldexp(1.0, e(g));
      } else if (mode == 2) {  // near-ties of the quotient
        c = 1.0 + u(g);
        o = c * (1.0 + 1e-6 * (1.0 + 1e-9 * u(g)));
      } else {  // specials
        c = k == 0 ? 0.0 : k == 1 ? qnan : k == 2 ? inf : k == 3 ? 4.9e-324 : k == 4 ? 1e-310 : u(g) * 1e-30;
        o = k == 5 ? c : k == 6 ? qnan : k == 7 ? -inf : k == 8 ? 1e308 : u(g);
      }
      acc.add(o, c);
      const double v = c != 0.0 ? std::fabs((o - c) / c) : 0.0;
      if (v > ref) ref = v;
    }
    uint64_t a, b;
    std::memcpy(&a, &acc.mx, 8);
    std::memcpy(&b, &ref, 8);
    if (a != b) {
      if (bad < 5) fprintf(stderr, "trial %d mode %d: screened %.17g, plain %.17g\n", trial, mode, acc.mx, ref);
      ++bad;
    }
  }
  if (bad) fprintf(stderr, "%d of 4000 sequences differ\n", bad);
  return bad ? 1 : 0;
}

// emu lattice D iso: the library's lattice tables as it compiles them (Lat<D>)
// and as fill_phys_impl sets them up (isotropy weights, MRT rate of every
// moment with the seven rates told apart), one JSON object.
static int lattice_dump(int D, int iso) {
  tx_params p;
  std::memset(&p, 0, sizeof(p));
  p.discretization = D == 3 ? TX_D3Q19 : TX_D2Q9;
  p.nx = p.ny = p.nz = 4;
  p.ncomponents = 1;
  p.relaxation_mode = TX_RELAX_MRT;
  p.isotropy_order = iso;
  p.tau[0] = 1.0;
  p.mm[0] = 1.0;
  p.s_c[0] = 1.01; p.s_e[0] = 1.02; p.s_e2[0] = 1.03; p.s_q[0] = 1.04;
  p.s_nu[0] = 1.05; p.s_pi[0] = 1.06; p.s_m[0] = 1.07;
  const int Q = D == 3 ? 19 : 9;
  Phys P{};
  fill_phys_impl(p, D, 1, Q, P);
  auto c = [&](int n, int a) { return D == 3 ? Lat<3>::c(n, a) : Lat<2>::c(n, a); };
  auto w = [&](int n) { return D == 3 ? Lat<3>::w(n) : Lat<2>::w(n); };
  auto mt = [&](int i, int k) { return D == 3 ? Lat<3>::mt(i, k) : Lat<2>::mt(i, k); };
  auto mmt = [&](int k) { return D == 3 ? Lat<3>::mmt(k) : Lat<2>::mmt(k); };
  printf("{\"ci\": [");
  for (int n = 0; n < Q; ++n) printf("%s[%d, %d, %d]", n ? ", " : "", c(n, 0), c(n, 1), c(n, 2));
  printf("], \"w\": [");
  for (int n = 0; n < Q; ++n) printf("%s%.17g", n ? ", " : "", w(n));
  printf("], \"mt\": [");
  for (int i = 0; i < Q; ++i) {
    printf("%s[", i ? ", " : "");
    for (int k = 0; k < Q; ++k) printf("%s%d", k ? ", " : "", mt(i, k));
    printf("]");
  }
  printf("], \"mmt\": [");
  for (int k = 0; k < Q; ++k) printf("%s%d", k ? ", " : "", mmt(k));
  printf("], \"rate\": [");
  for (int k = 0; k < Q; ++k) printf("%s%.17g", k ? ", " : "", P.srate[0][k]);
  printf("], \"ffw\": [");
  for (int i = 0; i < 12; ++i) printf("%s%.17g", i ? ", " : "", P.ffw[i]);
  printf("]}\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 2 && std::strcmp(argv[1], "norm") == 0) return norm_selftest();
  if (argc == 4 && std::strcmp(argv[1], "lattice") == 0) return lattice_dump(std::atoi(argv[2]), std::atoi(argv[3]));
  if (argc != 3) {
    fprintf(stderr, "usage: emu case.bin result.bin\n");
    return 1;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 1;
  Case c;
  int32_t hdr[2];
  if (!read_all(f, &c.p, sizeof(c.p)) || !read_all(f, hdr, sizeof(hdr))) return 1;
  c.nsteps = hdr[0];
  c.from_fi = hdr[1];
  std::string why;
  const int rc = validate(&c.p, &why);
  if (rc) {
    fprintf(stderr, "%s\n", why.c_str());
    return 2;
  }
  const int D = c.p.discretization == TX_D3Q19 ? 3 : 2, S = c.p.ncomponents, Q = D == 3 ? 19 : 9;
  const long long N = (long long)c.p.nx * c.p.ny * (D == 3 ? c.p.nz : 1);
  c.walls.resize((size_t)N);
  c.init.resize((size_t)(N * S * (c.from_fi ? Q : 1)));
  if (!read_all(f, c.walls.data(), c.walls.size() * 8) || !read_all(f, c.init.data(), c.init.size() * 8)) return 1;
  if (c.p.nspecies > 0) {
    c.conc.resize((size_t)(N * c.p.nspecies));
    if (!read_all(f, c.conc.data(), c.conc.size() * 8)) return 1;
  }
  fclose(f);

  Result r;
  std::string err;
  const bool found = D == 3 ? (dispatch_d3_iso4(c, r, &err) || dispatch_d3_iso8(c, r, &err) || dispatch_forms(c, r, &err))
                            : (dispatch_d2(c, r, &err) || dispatch_forms(c, r, &err));
  if (!found) {
    fprintf(stderr, "combination not compiled into the emulation\n");
    return 3;
  }
  if (!err.empty()) {
    fprintf(stderr, "%s\n", err.c_str());
    return 2;
  }
  FILE* o = fopen(argv[2], "wb");
  if (!o) return 1;
  for (const std::vector<double>* v : {&r.fi, &r.rho, &r.flux, &r.forces, &r.sfi, &r.srho, &r.sflux})
    if (!v->empty()) fwrite(v->data(), 8, v->size(), o);
  fclose(o);
  return 0;
}
