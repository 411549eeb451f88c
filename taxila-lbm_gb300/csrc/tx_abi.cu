// C ABI of the GB300 Shan-Chen step (include/taxila_gb300.h): handle, device
// memory, parameter translation and kernel dispatch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/taxila_gb300.h"
#include "tx_dispatch.h"
#include "tx_specular.cuh"

using namespace tx;

// error text of the calling thread's last failed call without a handle
// (tx_create, tx_step_static, batch creation): one string per host thread, so
// failing calls on several threads at once do not race
static thread_local std::string g_create_error;

struct tx_handle {
  tx_params p{};
  int D = 3, S = 1, Q = 19;
  Geo g{};
  Phys ph{};
  Phys* d_phys = nullptr;     // device copy of ph
  PhysT<float>* d_phys32 = nullptr;  // FP32 copy for the reduced-precision forms
  Faces faces{};
  FaceShell shell{};          // face nodes of the face pass (faces.post)
  bool outlet = false;        // two-component pressure outlets refresh every step
  KernelSet ks{};
  cudaStream_t stream = nullptr;
  size_t pop_bytes = 0;       // bytes of one population element
  void* f[2] = {nullptr, nullptr};
  int cur = 0;                // f[cur] holds the current state
  unsigned steps_done = 0;    // steps since tx_init (seeds FP16 stochastic rounding)
  void* rho = nullptr;        // forcing density
  void* psi = nullptr;        // psi(rho) when the EOS is on
  size_t rho_bytes = 0;
  uint8_t* mask = nullptr;
  uint32_t* links = nullptr;  // link masks (k_links), rebuilt with every wall upload
  double* faceval[6] = {nullptr};
  long long face_n[6] = {0};
  double* stage = nullptr;    // natural-order staging buffer (largest field)
  double* old_rho = nullptr;
  double* old_fi = nullptr;
  double* uic = nullptr;
  unsigned long long* red = nullptr;  // [0] max bits, [1] non-finite count
  unsigned long long* red_host = nullptr;  // pinned copy of red (the per-step norm's read-back)
  double* cons = nullptr;     // conservation-sum partials and per-population totals (first tx_conservation)
  std::vector<uint8_t> host_mask;
  // specular walls (codes 900-902, FP64 forms): exceptions to the ordinary push
  // (tx_specular.cuh), resolved at wall upload; wall cells then hold populations
  bool spec = false;
  std::vector<double> spec_walls;  // the uploaded wall values, for re-resolving at tx_upload_fi
  // the flow's exceptions, and the species' (no BCPreStream copies: their
  // transport applies no boundary condition; 2D MRT: wall cells' slots mix)
  SpecList spec_fl, spec_sp;
  void* spec_tmp = nullptr;       // [exception][component], storage type, shared
  int spec_fresh = 0;              // steps whose output buffer still needs its wall slots cleared
  int spec_fresh_sp = 0;           // the same for the species buffers
  // passive species (transport): populations, parameters, initial state
  int NS = 0;
  SpeciesSet ss{};
  void* sg[2] = {nullptr, nullptr};  // species populations (ping-pong)
  int gcur = 0;
  void* d_sphys = nullptr;    // SpeciesPhysT of the arithmetic type
  double* sconc = nullptr;    // uploaded initial concentration and flux
  double* sflux = nullptr;
  bool have_species = false;
  bool have_walls = false, have_state = false, have_fi = false, inited = false;
  int rest_pairs = -1;        // pairs for k_step_rest (paired FP32-arithmetic forms; counted at wall upload)
  bool timing = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double t_step_ms = 0.0, t_density_ms = 0.0;
  long long n_step_launch = 0, n_density_launch = 0, n_face_launch = 0;
  std::string err;
};

namespace {

int fail(tx_handle* h, int code, const std::string& msg) {
  if (h)
    h->err = msg;
  else
    g_create_error = msg;
  return code;
}

#define TX_CUDA(h, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(h, TX_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

int check_launch(tx_handle* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, TX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return TX_OK;
}

// The wall mask the natural-order conversions zero wall cells with; with
// specular walls wall cells hold populations, which pass through.
const uint8_t* pop_mask(const tx_handle* h) { return h->spec ? nullptr : h->mask; }

void free_spec(tx_handle* h) {
  for (SpecList* l : {&h->spec_fl, &h->spec_sp}) {
    cudaFree(l->dst);
    cudaFree(l->src);
    *l = SpecList{};
  }
  cudaFree(h->spec_tmp);
  h->spec_tmp = nullptr;
}

// Resolves the specular-wall routes of the uploaded walls (init_nz: wall slots
// with non-zero initial content) and puts the exception list on the device.
int upload_spec_routes(tx_handle* h, const std::vector<long long>* init_nz) {
  SpecRoutes r, rs;
  const int n[3] = {h->g.nx, h->g.ny, h->g.nz};
  bool pre[6];
  const bool none[6] = {false, false, false, false, false, false};
  for (int f = 0; f < 6; ++f) pre[f] = face_has_values(h->p, h->D, f);
  std::string why = specular_routes(h->spec_walls.data(), h->D, n, h->g.per, pre, init_nz, false, &r);
  if (why.empty() && h->NS > 0) {
    // the species start from their equilibrium (empty wall cells); in 2D under
    // MRT their wall cells' collision mixes the cells' slots
    const bool mix = h->D == 2 && h->p.species_relaxation_mode == TX_RELAX_MRT;
    why = specular_routes(h->spec_walls.data(), h->D, n, h->g.per, none, nullptr, mix, &rs);
  }
  if (!why.empty()) return fail(h, TX_ERR_ARG, why);
  free_spec(h);
  const long long tmp_n = std::max((long long)r.dst.size() * h->S, (long long)rs.dst.size() * h->NS);
  if (tmp_n > 0) TX_CUDA(h, cudaMalloc(&h->spec_tmp, (size_t)tmp_n * h->pop_bytes));
  for (auto [l, rr] : {std::make_pair(&h->spec_fl, &r), std::make_pair(&h->spec_sp, &rs)}) {
    const long long ne = (long long)rr->dst.size();
    if (ne == 0) continue;
    TX_CUDA(h, cudaMalloc(&l->dst, (size_t)ne * sizeof(long long)));
    TX_CUDA(h, cudaMalloc(&l->src, (size_t)ne * sizeof(long long)));
    l->n = ne;
    TX_CUDA(h, cudaMemcpy(l->dst, rr->dst.data(), (size_t)ne * sizeof(long long), cudaMemcpyHostToDevice));
    TX_CUDA(h, cudaMemcpy(l->src, rr->src.data(), (size_t)ne * sizeof(long long), cudaMemcpyHostToDevice));
  }
  return TX_OK;
}

// After the step kernels (push with ordinary bounceback), before the density
// pass: the specular-wall exceptions, for the ncomp components of state
// buffers fin -> fout (the flow's, or the species', which stream and bounce
// back alike; sh: their storage's rest state and scale).  The output buffer's
// wall slots are emptied on the first two steps after an upload or init
// (fresh), so that wall slots no exception writes are empty in both state buffers.
// fin null: only empty the wall cells of fout.
template <int D, class T>
void spec_launch(tx_handle* h, const SpecList& L, const void* fin, void* fout, int ncomp, const Shift& sh, int& fresh) {
  T* fo = static_cast<T*>(fout);
  const long long N = h->g.n;
  if (fresh > 0) {
    k_spec_clear_walls<D, T><<<(unsigned)((N + 255) / 256), 256, 0, h->stream>>>(fo, h->mask, N, ncomp, sh);
    --fresh;
  }
  const long long ne = L.n;
  if (ne == 0 || !fin) return;
  const unsigned grid = (unsigned)((ne + 255) / 256);
  T* tmp = static_cast<T*>(h->spec_tmp);
  k_spec_gather<D, T><<<grid, 256, 0, h->stream>>>(static_cast<const T*>(fin), fo, L.src, L.dst, ne, ncomp, N, sh, tmp);
  k_spec_scatter<T><<<grid, 256, 0, h->stream>>>(fo, L.dst, ne, ncomp, (long long)h->Q * N, tmp);
}
template <int D>
void spec_apply_d(tx_handle* h, const SpecList& L, const void* fin, void* fout, int ncomp, const Shift& sh, int& fresh) {
  if (h->p.precision == TX_PREC_F64)
    spec_launch<D, double>(h, L, fin, fout, ncomp, sh, fresh);
  else if (h->p.precision == TX_PREC_F32)
    spec_launch<D, float>(h, L, fin, fout, ncomp, sh, fresh);
  else
    spec_launch<D, __half>(h, L, fin, fout, ncomp, sh, fresh);
}
void spec_apply(tx_handle* h, const SpecList& L, const void* fin, void* fout, int ncomp, const Shift& sh, int& fresh) {
  if (h->D == 3)
    spec_apply_d<3>(h, L, fin, fout, ncomp, sh, fresh);
  else
    spec_apply_d<2>(h, L, fin, fout, ncomp, sh, fresh);
}
// the species kernels' arguments: populations read from state in, written to state out
SpeciesArgs species_args(tx_handle* h, int in, int out) {
  SpeciesArgs a{};
  a.gin = h->sg[in];
  a.gout = h->sg[out];
  a.links = h->links;
  a.mask = h->mask;
  a.phys = h->d_sphys;
  a.g = h->g;
  a.ns = h->NS;
  return a;
}
// the species' storage has no rest state
Shift species_shift() {
  Shift sh{};
  sh.scale = 1.0;
  return sh;
}
void spec_pass(tx_handle* h, int in, int out) {
  spec_apply(h, h->spec_fl, h->f[in], h->f[out], h->S, shift_of(h->ph), h->spec_fresh);
}
void spec_pass_species(tx_handle* h, int in, int out) {
  // in 2D the reference collides wall cells, which hold populations here
  if (h->D == 2) h->ss.wall_collide(species_args(h, in, in), h->stream);
  spec_apply(h, h->spec_sp, h->sg[in], h->sg[out], h->NS, species_shift(), h->spec_fresh_sp);
}

// Reference wall values -> device mask codes on the device (the rules of
// wall_code): flags[0] counts values the library refuses (negative or not
// finite), flags[1] counts specular codes, whose routes the host resolves.
__global__ void __launch_bounds__(256) k_wall_codes(const double* walls, long long N, int nminerals, int D,
                                                    uint8_t* mask, unsigned* flags) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double v = walls[i];
  uint8_t code = 255;
  if (v == 0.0) {
    code = 0;
  } else if (!(v > 0.0) || !isfinite(v)) {
    atomicAdd(&flags[0], 1u);
  } else if (specular_axis(v, D) >= 0) {
    atomicAdd(&flags[1], 1u);
  } else if (v < 998.0) {
    const int mineral = (int)v;
    if (mineral >= 1 && mineral <= nminerals) code = (uint8_t)mineral;
  }
  mask[i] = code;
}

// The forcing density from natural-order densities (component fastest, the
// device layout too): rho - rho0 on pore cells, zero on walls.
template <class RT>
__global__ void __launch_bounds__(256) k_rho_from_natural(const double* rho, const uint8_t* mask, long long N, int S,
                                                          Shift sh, RT* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * S) return;
  const long long c = i / S;
  const int m = (int)(i - c * S);
  out[i] = RT(mask[c] == 0 ? rho[i] - sh.rho0[m] : 0.0);
}

// link masks from the device wall mask (after every change of the mask)
int update_links(tx_handle* h) {
  const Launch3 l = launch3(h->g, 256);
  if (h->D == 3)
    k_links<3><<<l.grid, l.block, 0, h->stream>>>(h->mask, h->g, h->links);
  else
    k_links<2><<<l.grid, l.block, 0, h->stream>>>(h->mask, h->g, h->links);
  return check_launch(h, "k_links");
}

StepArgs args(tx_handle* h, int in, int out) {
  StepArgs a{};
  a.fin = h->f[in];
  a.fout = h->f[out];
  a.rho = h->rho;
  a.psi = h->psi;
  a.mask = h->mask;
  a.links = h->links;
  a.phys = h->p.precision == TX_PREC_F64 ? (const void*)h->d_phys : (const void*)h->d_phys32;
  a.g = h->g;
  a.faces = h->faces;
  a.step = h->steps_done;
  a.rest = h->rest_pairs;
  return a;
}

// Pairs of the paired step that need the per-site kernel (none: it is not launched).
int count_rest_pairs(tx_handle* h) {
  h->rest_pairs = -1;
  if (!h->ks.paired(h->g)) return TX_OK;
  unsigned* cnt = reinterpret_cast<unsigned*>(h->red);
  TX_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned), h->stream));
  h->ks.count_rest(args(h, h->cur, h->cur), cnt, h->stream);
  const int rc = check_launch(h, "k_count_rest");
  if (rc) return rc;
  unsigned n = 0;
  TX_CUDA(h, cudaMemcpyAsync(&n, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
  TX_CUDA(h, cudaStreamSynchronize(h->stream));
  h->rest_pairs = (int)n;
  return TX_OK;
}

long long field_dof(const tx_handle* h, int field) {
  if (h->NS == 0 && field >= TX_FIELD_SPECIES_FI && field <= TX_FIELD_SPECIES_FLUX) return -1;
  switch (field) {
    case TX_FIELD_SPECIES_FI: return (long long)h->NS * h->Q;
    case TX_FIELD_SPECIES_RHO: return h->NS;
    case TX_FIELD_SPECIES_FLUX: return (long long)h->NS * h->D;
    case TX_FIELD_FI: return (long long)h->S * h->Q;
    case TX_FIELD_RHO:
    case TX_FIELD_PSI: return h->S;
    case TX_FIELD_FLUX:
    case TX_FIELD_FORCES: return (long long)h->S * h->D;
    case TX_FIELD_PRS:
    case TX_FIELD_RHOT:
    case TX_FIELD_WALLS: return 1;
    case TX_FIELD_VELT: return h->D;
  }
  return -1;
}

}  // namespace

namespace tx {
bool select_species(const tx_params* p, SpeciesSet* ss);
int validate_params(const tx_params* p, std::string* why);
void fill_phys_from(const tx_params& p, int D, int S, int Q, Phys* out);
bool select_kernels(const tx_params* p, KernelSet* ks, bool any_rates = false);
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace tx

namespace {

void fill_phys(tx_handle* h) { fill_phys_impl(h->p, h->D, h->S, h->Q, h->ph); }

// max |(old - cur) / cur| over the field (DistributionCalcDeltaNorm), and old <- cur
// (NormMax screens the FP64 divisions).  mask (with dof values per cell): the
// field is read in place, and walls read as zero.
__global__ void k_delta_norm(const double* cur, double* old, long long n, unsigned long long* red,
                             const uint8_t* mask = nullptr, int dof = 1) {
  NormMax acc;
  unsigned long long bad = 0;
  const bool small = n <= 0xffffffffLL;  // the cell index by a 32-bit division
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long cell = !mask ? 0 : small ? (long long)((unsigned)i / (unsigned)dof) : i / dof;
    const double c = mask && mask[cell] != 0 ? 0.0 : cur[i];
    if (!isfinite(c)) ++bad;
    acc.add(old[i], c);
    old[i] = c;
  }
  double mx = acc.mx;
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&red[0], (unsigned long long)__double_as_longlong(mx));
    if (bad) atomicAdd(&red[1], bad);
  }
}

// Conservation sums, first pass.  Thread t < span adds the elements t,
// t + span, t + 2 span, ... of a natural-order field of n elements in FP64.
// span is a multiple of the field's dof, so every element a thread visits is
// the same degree of freedom (t mod dof), and consecutive threads read
// consecutive elements.
__global__ void k_dof_partials(const double* x, long long n, long long span, double* part) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= span) return;
  double s = 0.0;
  for (long long e = t; e < n; e += span) s += x[e];
  part[t] = s;
}

// Second pass: one warp per degree of freedom k sums part[k + dof * j] over
// j < span / dof, lane l taking j = l, l + 32, ...; the lanes combine by a
// fixed xor-shuffle tree, so the sum is the same on every run.
__global__ void k_dof_reduce(const double* part, long long span, int dof, double* sums) {
  const int k = blockIdx.x, lane = threadIdx.x;
  const long long per = span / dof;
  double s = 0.0;
  for (long long j = lane; j < per; j += 32) s += part[k + (long long)dof * j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sums[k] = s;
}

constexpr int kConsBlocks = 304, kConsThreads = 256;
constexpr long long kConsSpanMax = (long long)kConsBlocks * kConsThreads;

int sync_stream(tx_handle* h) {
  TX_CUDA(h, cudaStreamSynchronize(h->stream));
  return TX_OK;
}

// populations of state cur -> natural order staging
int stage_field(tx_handle* h, int field) {
  const long long N = h->g.n;
  if (field >= TX_FIELD_SPECIES_FI && field <= TX_FIELD_SPECIES_FLUX) {
    SpeciesArgs sa = species_args(h, h->gcur, h->gcur);
    if (h->spec && field == TX_FIELD_SPECIES_FI) sa.mask = nullptr;  // wall cells' populations too
    h->ss.fields(sa, field, h->stage, h->stream);
  } else if (field == TX_FIELD_FI) {
    h->ks.to_natural(h->f[h->cur], pop_mask(h), N, shift_of(h->ph), h->stage, h->stream);
  } else if (field == TX_FIELD_WALLS) {
    return TX_ERR_ARG;
  } else {
    const int what = field == TX_FIELD_RHO ? 2 : field == TX_FIELD_FLUX ? 3 : field == TX_FIELD_FORCES ? 4
                   : field == TX_FIELD_PRS ? 5 : field == TX_FIELD_VELT ? 6 : field == TX_FIELD_PSI ? 12 : 7;
    h->ks.moments(args(h, h->cur, h->cur), what, h->stage, h->stream);
  }
  return check_launch(h, "download kernel");
}

}  // namespace

namespace tx {
int validate_params(const tx_params* p, std::string* why) { return validate(p, why); }
void fill_phys_from(const tx_params& p, int D, int S, int Q, Phys* out) { fill_phys_impl(p, D, S, Q, *out); }
bool select_species(const tx_params* p, SpeciesSet* ss) {
  using Fn = bool (*)(bool, SpeciesSet*);
  static const Fn table[4][2] = {{species_d3_exact, species_d2_exact}, {species_d3_f64, species_d2_f64},
                                 {species_d3_f32, species_d2_f32}, {species_d3_f16, species_d2_f16}};
  const int form = p->precision == TX_PREC_F64 ? (p->exact ? 0 : 1) : (p->precision == TX_PREC_F32 ? 2 : 3);
  return table[form][p->discretization == TX_D3Q19 ? 0 : 1](p->species_relaxation_mode == TX_RELAX_MRT, ss);
}

bool select_kernels(const tx_params* p, KernelSet* ks, bool any_rates) {
  // the fast forms compile the general MRT rate path into the MRT kernels
  // only; lattices whose rates do not need it run the leaner kernels
  const bool mrt = p->relaxation_mode == TX_RELAX_MRT && (p->exact || any_rates || needs_general_rates(*p));
  using Fn = bool (*)(int, int, bool, KernelSet*);
  // [form][dimension 3/2][components 1/2]; form 0 exact FP64, 1 FP64, 2 FP32, 3 FP32/FP16
  static const Fn table[4][2][2] = {
      {{kernels_d3_exact_s1, kernels_d3_exact_s2}, {kernels_d2_exact_s1, kernels_d2_exact_s2}},
      {{kernels_d3_f64_s1, kernels_d3_f64_s2}, {kernels_d2_f64_s1, kernels_d2_f64_s2}},
      {{kernels_d3_f32_s1, kernels_d3_f32_s2}, {kernels_d2_f32_s1, kernels_d2_f32_s2}},
      {{kernels_d3_f16_s1, kernels_d3_f16_s2}, {kernels_d2_f16_s1, kernels_d2_f16_s2}}};
  const int form = p->precision == TX_PREC_F64 ? (p->exact ? 0 : 1) : (p->precision == TX_PREC_F32 ? 2 : 3);
  const int D = p->discretization == TX_D3Q19 ? 3 : 2;
  return table[form][D == 3 ? 0 : 1][p->ncomponents - 1](p->ncomponents, p->isotropy_order, mrt, ks);
}
}  // namespace tx

extern "C" {

int tx_params_default(tx_params* p) {
  if (!p) return TX_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->discretization = TX_D3Q19;
  p->nx = p->ny = p->nz = 1;
  p->ncomponents = 1;
  p->nminerals = 1;
  p->relaxation_mode = TX_RELAX_SRT;
  p->isotropy_order = 4;
  for (int m = 0; m < TX_MAX_COMPONENTS; ++m) {
    p->tau[m] = 1.0;
    p->s_c[m] = p->s_e[m] = p->s_e2[m] = p->s_q[m] = p->s_nu[m] = p->s_pi[m] = p->s_m[m] = 1.0;
    p->mm[m] = 1.0;
  }
  p->literal_kind = 4;
  p->precision = TX_PREC_F64;
  for (int m = 0; m < TX_MAX_COMPONENTS; ++m) p->rho0[m] = 0.0;
  p->storage_scale = 1.0;
  p->nspecies = 0;
  p->species_relaxation_mode = TX_RELAX_SRT;
  for (int m = 0; m < TX_MAX_COMPONENTS; ++m) {
    p->species_tau[m] = 1.0;
    for (int k = 0; k < 7; ++k) p->species_rates[m][k] = 1.0;
  }
  return TX_OK;
}

const char* tx_last_error(const tx_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int tx_create(const tx_params* p, tx_handle** out) {
  if (!p || !out) return fail(nullptr, TX_ERR_ARG, "null argument");
  *out = nullptr;
  std::string why;
  int rc = validate(p, &why);
  if (rc) return fail(nullptr, rc, why);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(nullptr, TX_ERR_NODEVICE, "no CUDA device");
  tx_handle* h = new tx_handle();
  h->p = *p;
  h->D = p->discretization == TX_D3Q19 ? 3 : 2;
  h->S = p->ncomponents;
  h->Q = h->D == 3 ? 19 : 9;
  h->g.nx = p->nx;
  h->g.ny = p->ny;
  h->g.nz = h->D == 3 ? p->nz : 1;
  for (int a = 0; a < 3; ++a) h->g.per[a] = a < h->D ? p->bc_flags[2 * a] == TX_BC_PERIODIC : 1;
  h->g.n = (long long)h->g.nx * h->g.ny * h->g.nz;
  fill_phys(h);
  const bool ok = select_kernels(p, &h->ks);
  if (!ok) {
    delete h;
    return fail(nullptr, TX_ERR_ARG, "no kernel built for this parameter combination");
  }
  const long long N = h->g.n;
  h->pop_bytes = p->precision == TX_PREC_F64 ? 8 : (p->precision == TX_PREC_F32 ? 4 : 2);
  h->rho_bytes = p->precision == TX_PREC_F64 ? 8 : 4;
  auto cleanup = [&](const std::string& msg, int code) {
    tx_destroy(h);
    return fail(nullptr, code, msg);
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup("cudaStreamCreate failed", TX_ERR_CUDA);
  const size_t popb = (size_t)N * h->S * h->Q * h->pop_bytes;
  h->NS = p->nspecies;
  const size_t stageb = (size_t)N * (h->S > h->NS ? h->S : h->NS) * h->Q * sizeof(double);
  if (cudaMalloc(&h->f[0], popb) != cudaSuccess || cudaMalloc(&h->f[1], popb) != cudaSuccess ||
      cudaMalloc(&h->rho, (size_t)N * h->S * h->rho_bytes) != cudaSuccess ||
      (p->use_nonideal_eos && cudaMalloc(&h->psi, (size_t)N * h->S * h->rho_bytes) != cudaSuccess) ||
      cudaMalloc(&h->mask, (size_t)N) != cudaSuccess || cudaMalloc(&h->links, (size_t)N * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&h->stage, stageb) != cudaSuccess ||
      cudaMalloc(&h->red, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&h->red_host, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&h->d_phys, sizeof(Phys)) != cudaSuccess ||
      cudaMalloc(&h->d_phys32, sizeof(PhysT<float>)) != cudaSuccess)
    return cleanup("device allocation failed", TX_ERR_NOMEM);
  PhysT<float> ph32{};
  convert_phys(h->ph, &ph32);
  if (cudaMemcpy(h->d_phys, &h->ph, sizeof(Phys), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->d_phys32, &ph32, sizeof(ph32), cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup("parameter upload failed", TX_ERR_CUDA);
  cudaMemsetAsync(h->f[0], 0, popb, h->stream);
  cudaMemsetAsync(h->f[1], 0, popb, h->stream);
  if (h->NS > 0) {
    if (!select_species(p, &h->ss)) return cleanup("no species kernel built for this form", TX_ERR_ARG);
    const size_t gb = (size_t)N * h->NS * h->Q * h->pop_bytes;
    SpeciesPhysT<double> sp{};
    fill_species_phys(*p, h->D, sp);
    SpeciesPhysT<float> sp32{};
    convert_species(sp, &sp32);
    const bool f64 = p->precision == TX_PREC_F64;
    const size_t spb = f64 ? sizeof(sp) : sizeof(sp32);
    if (cudaMalloc(&h->sg[0], gb) != cudaSuccess || cudaMalloc(&h->sg[1], gb) != cudaSuccess ||
        cudaMalloc(&h->d_sphys, spb) != cudaSuccess)
      return cleanup("device allocation failed", TX_ERR_NOMEM);
    if (cudaMemcpy(h->d_sphys, f64 ? (const void*)&sp : (const void*)&sp32, spb, cudaMemcpyHostToDevice) != cudaSuccess)
      return cleanup("species parameter upload failed", TX_ERR_CUDA);
    cudaMemsetAsync(h->sg[0], 0, gb, h->stream);
    cudaMemsetAsync(h->sg[1], 0, gb, h->stream);
  }
  cudaMemsetAsync(h->rho, 0, (size_t)N * h->S * h->rho_bytes, h->stream);
  cudaMemsetAsync(h->mask, 0, (size_t)N, h->stream);
  h->host_mask.assign((size_t)N, 0);
  if (update_links(h) != TX_OK) {
    const std::string why = h->err;
    return cleanup(why, TX_ERR_CUDA);
  }
  // exterior faces (FlowSetUpBCsD3/D2, lbm_flow.F90:1311-1956): the same values at
  // every node of a face, the reference's (s, ndims) block per node
  setup_faces(*p, h->D, &h->faces);
  h->shell = face_shell(*p, h->D, h->g.nx, h->g.ny, h->g.nz);
  h->outlet = has_outlet_update(*p, h->D);
  const int nbcs = h->S * h->D;
  for (int f = 0; f < 2 * h->D; ++f) {
    if (!face_has_values(*p, h->D, f)) continue;
    const long long area = face_area_of(h->D, h->g.nx, h->g.ny, h->g.nz, f);
    h->face_n[f] = area;
    double nv[3 * TX_MAX_COMPONENTS];
    face_node_values(*p, h->D, f, h->ph.c0, nv);
    std::vector<double> v((size_t)area * nbcs);
    for (int k = 0; k < nbcs; ++k)
      for (long long q = 0; q < area; ++q) v[(size_t)k * area + q] = nv[k];
    if (cudaMalloc(&h->faceval[f], v.size() * sizeof(double)) != cudaSuccess) return cleanup("device allocation failed", TX_ERR_NOMEM);
    if (cudaMemcpy(h->faceval[f], v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      return cleanup("face value upload failed", TX_ERR_CUDA);
    h->faces.vals[f] = h->faceval[f];
  }
  for (int i = 0; i < 4; ++i) cudaEventCreate(&h->ev[i]);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return cleanup("stream sync failed", TX_ERR_CUDA);
  if (count_rest_pairs(h) != TX_OK) {
    const std::string why = h->err;
    return cleanup(why, TX_ERR_CUDA);
  }
  *out = h;
  return TX_OK;
}

int tx_destroy(tx_handle* h) {
  if (!h) return TX_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->f[0]);
  cudaFree(h->f[1]);
  cudaFree(h->rho);
  cudaFree(h->psi);
  cudaFree(h->mask);
  cudaFree(h->links);
  cudaFree(h->stage);
  cudaFree(h->sg[0]);
  cudaFree(h->sg[1]);
  cudaFree(h->d_sphys);
  cudaFree(h->sconc);
  cudaFree(h->sflux);
  cudaFree(h->old_rho);
  cudaFree(h->old_fi);
  cudaFree(h->uic);
  cudaFree(h->red);
  cudaFreeHost(h->red_host);
  cudaFree(h->cons);
  free_spec(h);
  cudaFree(h->d_phys);
  cudaFree(h->d_phys32);
  for (int f = 0; f < 6; ++f) cudaFree(h->faceval[f]);
  for (int i = 0; i < 4; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return TX_OK;
}

int tx_upload_walls(tx_handle* h, const double* walls) {
  if (!h || !walls) return TX_ERR_ARG;
  const long long N = h->g.n;
  // codes on the device, into the staging area (the walls, then the new mask),
  // so that a refused upload leaves the handle's walls as they were
  double* dw = h->stage;
  uint8_t* dmask = reinterpret_cast<uint8_t*>(h->stage + N);
  unsigned* flags = reinterpret_cast<unsigned*>(h->red);
  TX_CUDA(h, cudaMemcpyAsync(dw, walls, (size_t)N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TX_CUDA(h, cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned), h->stream));
  k_wall_codes<<<(unsigned)((N + 255) / 256), 256, 0, h->stream>>>(dw, N, h->p.nminerals, h->D, dmask, flags);
  int rc0 = check_launch(h, "k_wall_codes");
  if (rc0) return rc0;
  unsigned fl[2] = {0u, 0u};
  TX_CUDA(h, cudaMemcpyAsync(fl, flags, sizeof(fl), cudaMemcpyDeviceToHost, h->stream));
  rc0 = sync_stream(h);
  if (rc0) return rc0;
  if (fl[0]) return fail(h, TX_ERR_ARG, "wall codes must be 0 (pore) or positive");
  const bool spec = fl[1] != 0;
  if (!spec) {
    TX_CUDA(h, cudaMemcpyAsync(h->mask, dmask, (size_t)N, cudaMemcpyDeviceToDevice, h->stream));
    TX_CUDA(h, cudaMemcpyAsync(h->host_mask.data(), dmask, (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    free_spec(h);
    h->spec_walls.clear();
    h->spec = false;
    h->spec_fresh = h->spec_fresh_sp = 2;
    int rc = update_links(h);
    if (rc != TX_OK) return rc;
    rc = count_rest_pairs(h);
    if (rc != TX_OK) return rc;
    h->have_walls = true;
    return sync_stream(h);
  }
  // specular walls: codes and routes on the host
  std::vector<uint8_t> mask((size_t)N);
  for (long long i = 0; i < N; ++i) {
    const char* why = nullptr;
    if (!wall_code(walls[i], h->p.nminerals, &mask[(size_t)i], &why, h->D, spec)) return fail(h, TX_ERR_ARG, why);
  }
  if (spec) {
    std::vector<double> prev(walls, walls + N);
    h->spec_walls.swap(prev);
    const int rc = upload_spec_routes(h, nullptr);
    if (rc != TX_OK) {
      h->spec_walls.swap(prev);  // a refused geometry leaves the handle as it was
      return rc;
    }
  } else {
    free_spec(h);
    h->spec_walls.clear();
  }
  h->spec = spec;
  h->spec_fresh = h->spec_fresh_sp = 2;
  h->host_mask.swap(mask);
  TX_CUDA(h, cudaMemcpyAsync(h->mask, h->host_mask.data(), (size_t)N, cudaMemcpyHostToDevice, h->stream));
  int rc = update_links(h);
  if (rc != TX_OK) return rc;
  rc = count_rest_pairs(h);
  if (rc != TX_OK) return rc;
  h->have_walls = true;
  return sync_stream(h);
}

int tx_upload_state(tx_handle* h, const double* rho, const double* u) {
  if (!h || !rho) return TX_ERR_ARG;
  const long long N = h->g.n;
  const int S = h->S, D = h->D;
  // rho - rho0 on the device: natural order (component fastest, the device
  // layout too), zero on walls
  TX_CUDA(h, cudaMemcpyAsync(h->stage, rho, (size_t)N * S * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  const unsigned grid = (unsigned)((N * S + 255) / 256);
  if (h->rho_bytes == 8)
    k_rho_from_natural<double><<<grid, 256, 0, h->stream>>>(h->stage, h->mask, N, S, shift_of(h->ph),
                                                            static_cast<double*>(h->rho));
  else
    k_rho_from_natural<float><<<grid, 256, 0, h->stream>>>(h->stage, h->mask, N, S, shift_of(h->ph),
                                                           static_cast<float*>(h->rho));
  int rc0 = check_launch(h, "k_rho_from_natural");
  if (rc0) return rc0;
  TX_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->psi) {
    // psi(rho) of the initial density, for the forces of FlowFiInit
    std::vector<double> ps((size_t)N * S, 0.0);
    for (long long i = 0; i < N; ++i)
      if (h->host_mask[(size_t)i] == 0)
        for (int m = 0; m < S; ++m)
          ps[(size_t)(i * S + m)] = eos_psi<double>(h->ph.eos[m], h->ph.eos_c[m], h->ph.g[m][m], h->ph.c0, rho[i * S + m]);
    if (h->rho_bytes == 8) {
      TX_CUDA(h, cudaMemcpyAsync(h->psi, ps.data(), ps.size() * 8, cudaMemcpyHostToDevice, h->stream));
      TX_CUDA(h, cudaStreamSynchronize(h->stream));
    } else {
      std::vector<float> pf(ps.begin(), ps.end());
      TX_CUDA(h, cudaMemcpyAsync(h->psi, pf.data(), pf.size() * 4, cudaMemcpyHostToDevice, h->stream));
      TX_CUDA(h, cudaStreamSynchronize(h->stream));
    }
  }
  cudaFree(h->uic);
  h->uic = nullptr;
  if (u) {
    std::vector<double> ut((size_t)N * S * D);
    for (long long i = 0; i < N; ++i)
      for (int d = 0; d < D; ++d)
        for (int m = 0; m < S; ++m) ut[((size_t)(m * D + d)) * N + i] = u[(i * D + d) * S + m];
    double* fresh = nullptr;  // the handle keeps the pointer only once the allocation succeeded
    TX_CUDA(h, cudaMalloc(&fresh, ut.size() * sizeof(double)));
    h->uic = fresh;
    TX_CUDA(h, cudaMemcpy(h->uic, ut.data(), ut.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  h->have_state = true;
  h->have_fi = false;
  h->inited = false;
  return TX_OK;
}

int tx_upload_species(tx_handle* h, const double* conc, const double* flux) {
  if (!h || !conc) return TX_ERR_ARG;
  if (h->NS == 0) return fail(h, TX_ERR_STATE, "the handle was created with nspecies = 0");
  const long long N = h->g.n;
  const size_t cb = (size_t)N * h->NS * sizeof(double), fb = cb * h->D;
  if (!h->sconc) {
    double* fresh = nullptr;  // the handle keeps the pointer only once the allocation succeeded
    TX_CUDA(h, cudaMalloc(&fresh, cb));
    h->sconc = fresh;
  }
  TX_CUDA(h, cudaMemcpyAsync(h->sconc, conc, cb, cudaMemcpyHostToDevice, h->stream));
  cudaFree(h->sflux);
  h->sflux = nullptr;
  if (flux) {
    double* fresh = nullptr;
    TX_CUDA(h, cudaMalloc(&fresh, fb));
    h->sflux = fresh;
    TX_CUDA(h, cudaMemcpyAsync(h->sflux, flux, fb, cudaMemcpyHostToDevice, h->stream));
  }
  h->have_species = true;
  h->inited = false;
  return sync_stream(h);
}

int tx_upload_fi(tx_handle* h, const double* fi) {
  if (!h || !fi) return TX_ERR_ARG;
  const long long N = h->g.n;
  const size_t bytes = (size_t)N * h->S * h->Q * sizeof(double);
  if (h->spec) {
    // populations uploaded into wall cells travel on like those the sweep leaves there
    std::vector<long long> nz;
    for (int n = 0; n < h->Q; ++n)
      for (long long i = 0; i < N; ++i) {
        if (h->host_mask[(size_t)i] == 0) continue;
        bool any = false;
        for (int m = 0; m < h->S; ++m) any = any || fi[(i * h->Q + n) * h->S + m] != 0.0;
        if (any) nz.push_back((long long)n * N + i);
      }
    const int rc = upload_spec_routes(h, nz.empty() ? nullptr : &nz);
    if (rc != TX_OK) return rc;
  }
  TX_CUDA(h, cudaMemcpyAsync(h->stage, fi, bytes, cudaMemcpyHostToDevice, h->stream));
  h->ks.from_natural(h->stage, pop_mask(h), N, shift_of(h->ph), h->f[h->cur], h->stream);
  int rc = check_launch(h, "k_pops_from_natural");
  if (rc) return rc;
  h->have_fi = true;
  h->have_state = false;
  h->inited = false;
  return sync_stream(h);
}

int tx_upload_bc_values(tx_handle* h, int32_t face, const double* vals) {
  if (!h || !vals) return TX_ERR_ARG;
  const int f = face - 1;
  if (f < 0 || f >= 2 * h->D || !h->faceval[f]) return fail(h, TX_ERR_ARG, "face carries no boundary values");
  const long long area = h->face_n[f];
  const int nbcs = h->S * h->D;
  std::vector<double> v((size_t)area * nbcs);
  for (long long q = 0; q < area; ++q)
    for (int k = 0; k < nbcs; ++k) v[(size_t)k * area + q] = vals[q * nbcs + k];
  TX_CUDA(h, cudaMemcpy(h->faceval[f], v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
  return TX_OK;
}

int tx_init(tx_handle* h) {
  if (!h) return TX_ERR_ARG;
  if (!h->have_walls) return fail(h, TX_ERR_STATE, "tx_upload_walls must come before tx_init");
  if (!h->have_state && !h->have_fi) return fail(h, TX_ERR_STATE, "tx_upload_state or tx_upload_fi must come before tx_init");
  if (!h->have_fi) {
    // FlowFiInit: the state buffer becomes (1 - P/2) feq of the initial moments
    if (h->spec) {
      // wall cells start empty (the reference's VecSet(fi, 0))
      int once = 1;
      spec_apply(h, h->spec_fl, nullptr, h->f[h->cur], h->S, shift_of(h->ph), once);
    }
    h->ks.init(args(h, h->cur, h->cur), h->uic, h->stream);
    int rc = check_launch(h, "k_init");
    if (rc) return rc;
  }
  h->spec_fresh = h->spec_fresh_sp = 2;
  // FlowUpdateMoments: the forcing density is the plain population sum
  h->ks.density(args(h, h->cur, h->cur), 1, h->stream);
  int rc = check_launch(h, "k_density");
  if (rc) return rc;
  if (h->NS > 0 && h->have_species) {
    // TransportFiInit; TransportUpdateMoments happens in the next collision
    h->ss.init(species_args(h, h->gcur, h->gcur), h->sconc, h->sflux, h->stream);
    rc = check_launch(h, "k_species_init");
    if (rc) return rc;
  }
  rc = sync_stream(h);
  if (rc) return rc;
  cudaFree(h->uic);
  h->uic = nullptr;
  h->steps_done = 0;
  h->inited = true;
  return TX_OK;
}

int tx_step(tx_handle* h, int32_t nsteps) {
  if (!h) return TX_ERR_ARG;
  if (!h->inited) return fail(h, TX_ERR_STATE, "tx_init must come before tx_step");
  if (nsteps < 0) return fail(h, TX_ERR_ARG, "nsteps must be >= 0");
  for (int t = 0; t < nsteps; ++t) {
    const int nxt = 1 - h->cur;
    StepArgs a = args(h, h->cur, nxt);
    if (h->outlet) {
      // FlowApplyBCs' pressure-outlet refresh (lbm_flow.F90:1964-1978), from the state
      for (int f = 0; f < 2 * h->D; ++f)
        if (h->p.bc_flags[f] == TX_BC_PRESSURE_OUTLET) {
          h->ks.outlet(a, f, h->faceval[f], h->p.bc_data[f][0], h->ph.c0, h->p.g[1][0], h->stream);
          ++h->n_face_launch;
        }
    }
    if (h->timing) cudaEventRecord(h->ev[0], h->stream);
    h->ks.step(a, h->stream);
    if (h->spec) spec_pass(h, h->cur, nxt);
    if (h->timing) cudaEventRecord(h->ev[1], h->stream);
    h->ks.density(a, 0, h->stream);
    if (h->faces.post) {
      h->ks.faces(a, h->shell, h->stream);
      ++h->n_face_launch;
    }
    if (h->timing) cudaEventRecord(h->ev[2], h->stream);
    if (h->NS > 0 && h->have_species) {
      h->ss.step(species_args(h, h->gcur, 1 - h->gcur), h->stream);
      if (h->spec) spec_pass_species(h, h->gcur, 1 - h->gcur);
      h->gcur = 1 - h->gcur;
    }
    int rc = check_launch(h, "k_step/k_density");
    if (rc) return rc;
    h->cur = nxt;
    h->steps_done++;
    h->n_step_launch++;
    h->n_density_launch++;
    if (h->timing) {
      TX_CUDA(h, cudaEventSynchronize(h->ev[2]));
      float a_ms = 0.f, b_ms = 0.f;
      cudaEventElapsedTime(&a_ms, h->ev[0], h->ev[1]);
      cudaEventElapsedTime(&b_ms, h->ev[1], h->ev[2]);
      h->t_step_ms += a_ms;
      h->t_density_ms += b_ms;
    }
  }
  return TX_OK;
}

int tx_step_species(tx_handle* h, int32_t nsteps) {
  if (!h) return TX_ERR_ARG;
  if (!h->inited) return fail(h, TX_ERR_STATE, "tx_init must come before tx_step_species");
  if (nsteps < 0) return fail(h, TX_ERR_ARG, "nsteps must be >= 0");
  if (h->NS == 0 || !h->have_species) return fail(h, TX_ERR_STATE, "the handle holds no species state");
  for (int t = 0; t < nsteps; ++t) {
    // the species part of tx_step alone: the flow state and its step count stay as they are
    h->ss.step(species_args(h, h->gcur, 1 - h->gcur), h->stream);
    if (h->spec) spec_pass_species(h, h->gcur, 1 - h->gcur);
    h->gcur = 1 - h->gcur;
    const int rc = check_launch(h, "k_species");
    if (rc) return rc;
  }
  return TX_OK;
}

int tx_sync(tx_handle* h) {
  if (!h) return TX_ERR_ARG;
  return sync_stream(h);
}

int64_t tx_field_size(const tx_handle* h, int32_t field) {
  if (!h) return -1;
  const long long dof = field_dof(h, field);
  return dof < 0 ? -1 : dof * h->g.n;
}

int tx_download(tx_handle* h, int32_t field, double* out) {
  if (!h || !out) return TX_ERR_ARG;
  const long long dof = field_dof(h, field);
  if (dof < 0) return fail(h, TX_ERR_ARG, "unknown field");
  const long long N = h->g.n;
  if (field == TX_FIELD_WALLS) {
    // the uploaded codes are kept on the host in mask form (with specular
    // walls, as uploaded); report them as the reference walls vector
    if (h->spec) {
      std::memcpy(out, h->spec_walls.data(), (size_t)N * sizeof(double));
      return TX_OK;
    }
    for (long long i = 0; i < N; ++i) {
      const uint8_t c = h->host_mask[(size_t)i];
      out[i] = c == 255 ? 999.0 : (double)c;
    }
    return TX_OK;
  }
  if (!h->inited) return fail(h, TX_ERR_STATE, "tx_init must come before tx_download");
  int rc = stage_field(h, field);
  if (rc) return rc;
  TX_CUDA(h, cudaMemcpyAsync(out, h->stage, (size_t)(N * dof) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync_stream(h);
}

int tx_delta_norm(tx_handle* h, int32_t field, double* norm) {
  if (!h || !norm) return TX_ERR_ARG;
  if (field != TX_FIELD_RHO && field != TX_FIELD_FI) return fail(h, TX_ERR_ARG, "delta norm over rho or fi only");
  if (!h->inited) return fail(h, TX_ERR_STATE, "tx_init must come before tx_delta_norm");
  const long long n = tx_field_size(h, field);
  double*& old = field == TX_FIELD_RHO ? h->old_rho : h->old_fi;
  if (!old) {
    double* fresh = nullptr;  // the handle keeps the pointer only once the allocation succeeded
    TX_CUDA(h, cudaMalloc(&fresh, (size_t)n * sizeof(double)));
    old = fresh;
    TX_CUDA(h, cudaMemsetAsync(old, 0, (size_t)n * sizeof(double), h->stream));
  }
  // In the FP64 form without face nodes that re-sum their density, the
  // density field is the stored forcing density itself (zero on walls)
  bool in_place = field == TX_FIELD_RHO && h->p.precision == TX_PREC_F64;
  for (int f = 0; f < 6; ++f) in_place = in_place && !h->faces.on[f];
  int rc = in_place ? TX_OK : stage_field(h, field);
  if (rc) return rc;
  TX_CUDA(h, cudaMemsetAsync(h->red, 0, 2 * sizeof(unsigned long long), h->stream));
  if (in_place)
    k_delta_norm<<<1216, 256, 0, h->stream>>>(static_cast<const double*>(h->rho), old, n, h->red, h->mask, h->S);
  else
    k_delta_norm<<<1216, 256, 0, h->stream>>>(h->stage, old, n, h->red);
  rc = check_launch(h, "k_delta_norm");
  if (rc) return rc;
  unsigned long long* r = h->red_host;
  TX_CUDA(h, cudaMemcpyAsync(r, h->red, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  rc = sync_stream(h);
  if (rc) return rc;
  double v;
  std::memcpy(&v, &r[0], sizeof(v));
  *norm = v;
  if (r[1]) return fail(h, TX_ERR_NONFINITE, "non-finite values in the field (" + std::to_string(r[1]) + " sites)");
  return TX_OK;
}

int tx_conservation(tx_handle* h, double* out) {
  if (!h || !out) return TX_ERR_ARG;
  if (!h->inited) return fail(h, TX_ERR_STATE, "tx_init must come before tx_conservation");
  const int dof = h->S * h->Q;
  const long long n = h->g.n * dof;
  const long long span = (kConsSpanMax / dof) * dof;
  if (!h->cons) {
    double* fresh = nullptr;  // the handle keeps the pointer only once the allocation succeeded
    TX_CUDA(h, cudaMalloc(&fresh, (size_t)(kConsSpanMax + 128) * sizeof(double)));
    h->cons = fresh;
  }
  int rc = stage_field(h, TX_FIELD_FI);
  if (rc) return rc;
  double* sums_d = h->cons + kConsSpanMax;
  k_dof_partials<<<kConsBlocks, kConsThreads, 0, h->stream>>>(h->stage, n, span, h->cons);
  rc = check_launch(h, "k_dof_partials");
  if (rc) return rc;
  k_dof_reduce<<<dof, 32, 0, h->stream>>>(h->cons, span, dof, sums_d);
  rc = check_launch(h, "k_dof_reduce");
  if (rc) return rc;
  double sums[TX_MAX_COMPONENTS * 19];
  TX_CUDA(h, cudaMemcpyAsync(sums, sums_d, (size_t)dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  rc = sync_stream(h);
  if (rc) return rc;
  // natural order: population n of component m is dof n * S + m
  bool finite = true;
  for (int m = 0; m < h->S; ++m) {
    double mass = 0.0;
    for (int q = 0; q < h->Q; ++q) mass += sums[q * h->S + m];
    out[m] = mass;
    finite = finite && std::isfinite(mass);
    for (int d = 0; d < h->D; ++d) {
      double mom = 0.0;
      for (int q = 0; q < h->Q; ++q) {
        const int c = h->D == 3 ? Lat<3>::c(q, d) : Lat<2>::c(q, d);
        if (c) mom += c * sums[q * h->S + m];
      }
      out[h->S + m * h->D + d] = mom;
      finite = finite && std::isfinite(mom);
    }
  }
  if (!finite) return fail(h, TX_ERR_NONFINITE, "non-finite populations in the conservation sums");
  return TX_OK;
}

/* ------------------------------------------------------- instrumentation */
int tx_set_timing(tx_handle* h, int32_t on) {
  if (!h) return TX_ERR_ARG;
  h->timing = on != 0;
  h->t_step_ms = h->t_density_ms = 0.0;
  h->n_step_launch = h->n_density_launch = h->n_face_launch = 0;
  return TX_OK;
}

int tx_get_timing(tx_handle* h, double* ms_step, double* ms_density, int64_t* launches) {
  if (!h) return TX_ERR_ARG;
  if (ms_step) *ms_step = h->t_step_ms;
  if (ms_density) *ms_density = h->t_density_ms;
  if (launches) *launches = h->n_step_launch + h->n_density_launch + h->n_face_launch;
  return TX_OK;
}

void* tx_get_stream(tx_handle* h) { return h ? (void*)h->stream : nullptr; }

const char* tx_kernel_name(const tx_handle* h) { return h ? h->ks.name : ""; }

}  // extern "C"
