// Batch engine: many lattices of one kernel form on one GPU (tx_batch_* in
// include/taxila_gb300.h).
//
// Each lattice owns its device buffers (two population buffers, forcing
// density, wall mask, link masks, the velocity of the previous probe, density
// faces and a parameter block), allocated stream-ordered from the device's
// default memory pool so that lattices join and leave without a device-wide
// synchronisation.  The host keeps a slot list; every change of it rewrites
// the lattice descriptors and the tile table in device memory.  The persistent
// grid and the device addresses of those tables do not change, so the
// captured K-step graph stays valid across joins and leaves and is only
// re-captured when a table has to grow or the tile shape changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/taxila_gb300.h"
#include "tx_dispatch.h"

using namespace tx;

namespace tx {
bool select_kernels(const tx_params* p, KernelSet* ks, bool any_rates = false);
bool select_species(const tx_params* p, SpeciesSet* ss);
void set_global_error(const std::string& msg);
}

namespace {

struct Lattice {
  int id = 0;
  tx_params p{};
  int D = 3, S = 1, Q = 19;
  Geo g{};
  Phys ph{};
  void* f[2] = {nullptr, nullptr};
  void* rho = nullptr;
  void* psi = nullptr;        // psi(rho) when the EOS is on
  uint8_t* mask = nullptr;
  uint32_t* links = nullptr;
  double* uold = nullptr;
  unsigned* steps_dev = nullptr;  // device step counter (FP16 stochastic-rounding seed)
  double* faceval[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  void* phys = nullptr;       // PhysT<R> of the batch's arithmetic type
  Faces faces{};
  FaceShell shell{};          // face nodes of the face pass (faces.post)
  void* sg[2] = {nullptr, nullptr};  // species populations
  void* sphys = nullptr;             // SpeciesPhysT<R>
  int NS = 0;
  long long bytes = 0;
  long long steps = 0;
  bool paired = false;        // the paired step (FP32-arithmetic forms, even site count)
  int rest = -1;              // its pairs for the per-site kernel
};

size_t pop_bytes(int precision) { return precision == TX_PREC_F64 ? 8 : (precision == TX_PREC_F32 ? 4 : 2); }
size_t rho_bytes(int precision) { return precision == TX_PREC_F64 ? 8 : 4; }

long long face_area(const tx_params& p, int D, int f) {
  const int a = f / 2;
  if (D == 2) return a == 0 ? p.ny : p.nx;
  return a == 0 ? (long long)p.ny * p.nz : a == 1 ? (long long)p.nx * p.nz : (long long)p.nx * p.ny;
}

long long lattice_bytes(const tx_params& p) {
  const int D = p.discretization == TX_D3Q19 ? 3 : 2, Q = D == 3 ? 19 : 9, S = p.ncomponents;
  const long long N = (long long)p.nx * p.ny * (D == 3 ? p.nz : 1);
  long long b = 2 * N * S * Q * (long long)pop_bytes(p.precision) +
                N * S * (long long)rho_bytes(p.precision) * (p.use_nonideal_eos ? 2 : 1) + N +
                4 * N + 8LL * D * N + (long long)sizeof(Phys);
  for (int f = 0; f < 2 * D; ++f)
    if (face_has_values(p, D, f)) b += face_area(p, D, f) * S * D * 8;
  if (p.nspecies > 0) b += 2 * N * p.nspecies * Q * (long long)pop_bytes(p.precision) + (long long)sizeof(SpeciesPhysT<double>);
  return b;
}

}  // namespace

struct tx_batch {
  tx_params form{};
  KernelSet ks{};
  SpeciesSet ss{};
  int D = 3, S = 1, Q = 19;
  cudaStream_t stream = nullptr;
  int sm_count = 1;
  std::vector<Lattice*> slots;  // active lattices, in table order
  int next_id = 1;
  long long budget = 0, in_use = 0;
  // device tables
  LatDesc* d_lats = nullptr;
  int lat_cap = 0;
  int4* d_tiles = nullptr;
  ProbePart* d_parts = nullptr;
  int tile_cap = 0;
  int* d_ntiles = nullptr;
  ProbePart* d_res = nullptr;
  int ntiles = 0;
  int2* d_ltiles = nullptr;  // the density pass's linear tiles
  int ltile_cap = 0;
  int* d_nltiles = nullptr;
  int2* d_ftiles = nullptr;  // face-pass tiles
  int ftile_cap = 0;
  int* d_nftiles = nullptr;
  int4* d_otiles = nullptr;  // outlet-refresh tiles
  int otile_cap = 0;
  int* d_notiles = nullptr;
  int4* d_stiles = nullptr;  // step tiles: per-site, pair and per-site-of-pairs
  int stile_cap = 0;
  int* d_nstiles = nullptr;
  int4* d_ptiles = nullptr;
  int ptile_cap = 0;
  int* d_nptiles = nullptr;
  int4* d_rtiles = nullptr;
  int rtile_cap = 0;
  int* d_nrtiles = nullptr;
  unsigned* d_count = nullptr;  // pair count of a joining lattice
  bool need_faces = false, need_outlets = false;  // launched once a lattice needs them
  bool tables_ok = true;  // false after a failed rebuild_tables: launches and probes refuse until one succeeds
  // launch shape
  int bx = 32, by = 4, bz = 1, blocks_per_sm = 4;
  // graph
  int graph_steps = 20;
  cudaGraphExec_t exec = nullptr;
  int flip = 0;
  std::string err;
};

namespace {

// One block per lattice slot: its tiles' partials in a fixed order.
__global__ void __launch_bounds__(256) k_probe_reduce(const LatDesc* lats, int nlat, const ProbePart* parts,
                                                      ProbePart* out) {
  constexpr int NV = 6 + MAXC;  // du, umax, usum x/y/z, npore, mass per component
  __shared__ double red[256][NV];
  const int l = blockIdx.x;
  if (l >= nlat) return;
  const int t0 = lats[l].tile_begin, tn = lats[l].tile_count;
  double v[NV];
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int t = (int)threadIdx.x; t < tn; t += blockDim.x) {
    const ProbePart p = parts[t0 + t];
    v[0] = fmax(v[0], p.du);
    v[1] = fmax(v[1], p.umax);
    for (int d = 0; d < 3; ++d) v[2 + d] += p.usum[d];
    v[5] += p.npore;
    for (int m = 0; m < MAXC; ++m) v[6 + m] += p.mass[m];
  }
  for (int k = 0; k < NV; ++k) red[threadIdx.x][k] = v[k];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      red[threadIdx.x][0] = fmax(red[threadIdx.x][0], red[threadIdx.x + s][0]);
      red[threadIdx.x][1] = fmax(red[threadIdx.x][1], red[threadIdx.x + s][1]);
      for (int k = 2; k < NV; ++k) red[threadIdx.x][k] += red[threadIdx.x + s][k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ProbePart r{};
    r.du = red[0][0];
    r.umax = red[0][1];
    for (int d = 0; d < 3; ++d) r.usum[d] = red[0][2 + d];
    r.npore = red[0][5];
    for (int m = 0; m < MAXC; ++m) r.mass[m] = red[0][6 + m];
    out[l] = r;
  }
}


int bfail(tx_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

#define TX_BCUDA(b, call)                                                                                  \
  do {                                                                                                     \
    const cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return bfail(b, TX_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

void drop_graph(tx_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

int grid_of(const tx_batch* b) { return b->sm_count * b->blocks_per_sm; }

BatchArgs bargs(const tx_batch* b) {
  BatchArgs a{};
  a.lats = b->d_lats;
  a.tiles = b->d_tiles;
  a.ntiles = b->d_ntiles;
  a.parts = b->d_parts;
  a.ltiles = b->d_ltiles;
  a.nltiles = b->d_nltiles;
  a.ftiles = b->d_ftiles;
  a.nftiles = b->d_nftiles;
  a.otiles = b->d_otiles;
  a.notiles = b->d_notiles;
  a.stiles = b->d_stiles;
  a.nstiles = b->d_nstiles;
  a.ptiles = b->d_ptiles;
  a.nptiles = b->d_nptiles;
  a.rtiles = b->d_rtiles;
  a.nrtiles = b->d_nrtiles;
  return a;
}

StepArgs lattice_args(const tx_batch* b, const Lattice* L, int in, int out) {
  StepArgs a{};
  a.fin = L->f[in];
  a.fout = L->f[out];
  a.rho = L->rho;
  a.psi = L->psi;
  a.mask = L->mask;
  a.links = L->links;
  a.phys = L->phys;
  a.g = L->g;
  a.faces = L->faces;
  a.steps_ptr = L->steps_dev;
  a.rest = L->rest;
  (void)b;
  return a;
}

// Grows a device table to hold n entries (dropping the graph, whose launches
// name the old address); entries are rewritten by the caller.
template <class E>
int grow_table(tx_batch* b, E** ptr, int* cap, int n);

template <class E>
int grow_table(tx_batch* b, E** ptr, int* cap, int n) {
  if (n <= *cap) return TX_OK;
  const int c = std::max(n, 2 * *cap);
  drop_graph(b);
  if (*ptr) cudaFreeAsync(*ptr, b->stream);
  *ptr = nullptr;
  *cap = 0;
  TX_BCUDA(b, cudaMallocAsync((void**)ptr, (size_t)c * sizeof(E), b->stream));
  *cap = c;
  return TX_OK;
}

// Rewrites the descriptors and the tile table of the active lattices.
int rebuild_tables(tx_batch* b) {
  b->tables_ok = false;
  std::vector<LatDesc> descs;
  std::vector<int4> tiles;
  std::vector<int2> ltiles, ftiles;
  std::vector<int4> otiles, stiles, ptiles, rtiles;
  const long long run = 128LL * (long long)(16 / pop_bytes(b->form.precision));  // sites per density tile
  for (size_t s = 0; s < b->slots.size(); ++s) {
    Lattice* L = b->slots[s];
    LatDesc d{};
    d.a = lattice_args(b, L, 0, 1);
    d.uold = L->uold;
    d.sg0 = L->sg[0];
    d.sg1 = L->sg[1];
    d.sphys = L->sphys;
    d.ns = L->NS;
    d.tile_begin = (int)tiles.size();
    for (int z = 0; z < L->g.nz; z += b->bz)
      for (int y = 0; y < L->g.ny; y += b->by)
        for (int x = 0; x < L->g.nx; x += b->bx) tiles.push_back(make_int4((int)s, x, y, z));
    d.tile_count = (int)tiles.size() - d.tile_begin;
    if (L->paired) {
      for (long long i0 = 0; 2 * i0 < L->g.n; i0 += 128 * kPairTileRuns) {
        ptiles.push_back(make_int4((int)s, (int)i0, 0, 0));
        if (L->rest != 0) rtiles.push_back(make_int4((int)s, (int)i0, 0, 0));
      }
    } else {
      stiles.insert(stiles.end(), tiles.begin() + d.tile_begin, tiles.end());
    }
    d.ltile_begin = (int)ltiles.size();
    for (long long c0 = 0; c0 < L->g.n; c0 += run) ltiles.push_back(make_int2((int)s, (int)c0));
    d.shell = L->shell;
    d.c0 = L->ph.c0;
    d.g21 = L->S > 1 ? L->p.g[1][0] : 0.0;
    for (int f = 0; f < 6; ++f) d.outlet_p[f] = L->p.bc_data[f][0];
    if (L->faces.post)
      for (long long q0 = 0; q0 < L->shell.start[L->shell.nf]; q0 += 128) ftiles.push_back(make_int2((int)s, (int)q0));
    if (has_outlet_update(L->p, L->D))
      for (int f = 0; f < 2 * L->D; ++f)
        if (L->p.bc_flags[f] == TX_BC_PRESSURE_OUTLET)
          for (long long q0 = 0; q0 < face_area(L->p, L->D, f); q0 += 128) otiles.push_back(make_int4((int)s, f, (int)q0, 0));
    descs.push_back(d);
  }
  const int nl = (int)descs.size(), nt = (int)tiles.size(), nlt = (int)ltiles.size();
  const int nft = (int)ftiles.size(), nov = (int)otiles.size();
  if (nl > b->lat_cap) {
    const int cap = std::max(nl, 2 * b->lat_cap);
    drop_graph(b);
    if (b->d_lats) cudaFreeAsync(b->d_lats, b->stream);
    if (b->d_res) cudaFreeAsync(b->d_res, b->stream);
    b->d_lats = nullptr;
    b->d_res = nullptr;
    b->lat_cap = 0;
    TX_BCUDA(b, cudaMallocAsync(&b->d_lats, (size_t)cap * sizeof(LatDesc), b->stream));
    TX_BCUDA(b, cudaMallocAsync(&b->d_res, (size_t)cap * sizeof(ProbePart), b->stream));
    b->lat_cap = cap;
  }
  if (nt > b->tile_cap) {
    const int cap = std::max(nt, 2 * b->tile_cap);
    drop_graph(b);
    if (b->d_tiles) cudaFreeAsync(b->d_tiles, b->stream);
    if (b->d_parts) cudaFreeAsync(b->d_parts, b->stream);
    b->d_tiles = nullptr;
    b->d_parts = nullptr;
    b->tile_cap = 0;
    TX_BCUDA(b, cudaMallocAsync(&b->d_tiles, (size_t)cap * sizeof(int4), b->stream));
    TX_BCUDA(b, cudaMallocAsync(&b->d_parts, (size_t)cap * sizeof(ProbePart), b->stream));
    b->tile_cap = cap;
  }
  if (nlt > b->ltile_cap) {
    const int cap = std::max(nlt, 2 * b->ltile_cap);
    drop_graph(b);
    if (b->d_ltiles) cudaFreeAsync(b->d_ltiles, b->stream);
    b->d_ltiles = nullptr;
    b->ltile_cap = 0;
    TX_BCUDA(b, cudaMallocAsync(&b->d_ltiles, (size_t)cap * sizeof(int2), b->stream));
    b->ltile_cap = cap;
  }
  if (nft > b->ftile_cap) {
    const int cap = std::max(nft, 2 * b->ftile_cap);
    drop_graph(b);
    if (b->d_ftiles) cudaFreeAsync(b->d_ftiles, b->stream);
    b->d_ftiles = nullptr;
    b->ftile_cap = 0;
    TX_BCUDA(b, cudaMallocAsync(&b->d_ftiles, (size_t)cap * sizeof(int2), b->stream));
    b->ftile_cap = cap;
  }
  if (nov > b->otile_cap) {
    const int cap = std::max(nov, 2 * b->otile_cap);
    drop_graph(b);
    if (b->d_otiles) cudaFreeAsync(b->d_otiles, b->stream);
    b->d_otiles = nullptr;
    b->otile_cap = 0;
    TX_BCUDA(b, cudaMallocAsync(&b->d_otiles, (size_t)cap * sizeof(int4), b->stream));
    b->otile_cap = cap;
  }
  // the step's tables
  {
    const int ns = (int)stiles.size(), np = (int)ptiles.size(), nr = (int)rtiles.size();
    int rc = grow_table(b, &b->d_stiles, &b->stile_cap, ns);
    if (!rc) rc = grow_table(b, &b->d_ptiles, &b->ptile_cap, np);
    if (!rc) rc = grow_table(b, &b->d_rtiles, &b->rtile_cap, nr);
    if (rc) return rc;
    if (ns) TX_BCUDA(b, cudaMemcpyAsync(b->d_stiles, stiles.data(), (size_t)ns * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    if (np) TX_BCUDA(b, cudaMemcpyAsync(b->d_ptiles, ptiles.data(), (size_t)np * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    if (nr) TX_BCUDA(b, cudaMemcpyAsync(b->d_rtiles, rtiles.data(), (size_t)nr * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    TX_BCUDA(b, cudaMemcpyAsync(b->d_nstiles, &ns, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    TX_BCUDA(b, cudaMemcpyAsync(b->d_nptiles, &np, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    TX_BCUDA(b, cudaMemcpyAsync(b->d_nrtiles, &nr, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    // the counts are copied from the stack: wait for them before it goes
    TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  }
  if (nft) TX_BCUDA(b, cudaMemcpyAsync(b->d_ftiles, ftiles.data(), (size_t)nft * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  if (nov) TX_BCUDA(b, cudaMemcpyAsync(b->d_otiles, otiles.data(), (size_t)nov * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
  TX_BCUDA(b, cudaMemcpyAsync(b->d_nftiles, &nft, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  TX_BCUDA(b, cudaMemcpyAsync(b->d_notiles, &nov, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if (nl) TX_BCUDA(b, cudaMemcpyAsync(b->d_lats, descs.data(), (size_t)nl * sizeof(LatDesc), cudaMemcpyHostToDevice, b->stream));
  if (nlt) TX_BCUDA(b, cudaMemcpyAsync(b->d_ltiles, ltiles.data(), (size_t)nlt * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  TX_BCUDA(b, cudaMemcpyAsync(b->d_nltiles, &nlt, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if (nt) TX_BCUDA(b, cudaMemcpyAsync(b->d_tiles, tiles.data(), (size_t)nt * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
  TX_BCUDA(b, cudaMemcpyAsync(b->d_ntiles, &nt, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  // the host vectors die with this call: the copies must have left them
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  b->ntiles = nt;
  b->tables_ok = true;
  return TX_OK;
}

int launch_step(tx_batch* b, int flip) {
  const dim3 blk((unsigned)b->bx, (unsigned)b->by, (unsigned)b->bz);
  const BatchArgs a = bargs(b);
  if (b->need_outlets) b->ks.outlet_tiles(a, flip, grid_of(b), blk, b->stream);
  b->ks.step_tiles(a, flip, grid_of(b), blk, b->stream);
  b->ks.density_tiles(a, flip, grid_of(b), blk, b->stream);
  if (b->need_faces) b->ks.faces_tiles(a, flip, grid_of(b), blk, b->stream);
  if (b->form.nspecies > 0) b->ss.step_tiles(a, flip, grid_of(b), blk, b->stream);
  TX_BCUDA(b, cudaGetLastError());
  return TX_OK;
}

int capture_graph(tx_batch* b) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  TX_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = TX_OK;
  for (int s = 0; s < b->graph_steps && rc == TX_OK; ++s) rc = launch_step(b, s & 1);
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bfail(b, TX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  const cudaError_t ei = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    b->exec = nullptr;
    return bfail(b, TX_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
  }
  return TX_OK;
}

void free_lattice(tx_batch* b, Lattice* L) {
  cudaStream_t s = b->stream;
  for (void* p : {(void*)L->f[0], (void*)L->f[1], L->rho, L->psi, (void*)L->mask, (void*)L->links, (void*)L->uold, L->phys,
                  L->sg[0], L->sg[1], L->sphys, (void*)L->steps_dev})
    if (p) cudaFreeAsync(p, s);
  for (int f = 0; f < 6; ++f)
    if (L->faceval[f]) cudaFreeAsync(L->faceval[f], s);
  b->in_use -= L->bytes;
  delete L;
}

int stage(tx_batch* b, const Lattice* L, int field, double* out) {
  const long long N = L->g.n;
  if (field >= TX_FIELD_SPECIES_FI && field <= TX_FIELD_SPECIES_FLUX) {
    SpeciesArgs a{};
    a.gin = L->sg[b->flip];
    a.gout = L->sg[b->flip];
    a.links = L->links;
    a.mask = L->mask;
    a.phys = L->sphys;
    a.g = L->g;
    a.ns = L->NS;
    b->ss.fields(a, field, out, b->stream);
  } else if (field == TX_FIELD_FI) {
    b->ks.to_natural(L->f[b->flip], L->mask, N, shift_of(L->ph), out, b->stream);
  } else {
    const int what = field == TX_FIELD_RHO ? 2 : field == TX_FIELD_FLUX ? 3 : field == TX_FIELD_FORCES ? 4
                   : field == TX_FIELD_PRS ? 5 : field == TX_FIELD_VELT ? 6 : field == TX_FIELD_PSI ? 12 : 7;
    b->ks.moments(lattice_args(b, L, b->flip, b->flip), what, out, b->stream);
  }
  TX_BCUDA(b, cudaGetLastError());
  return TX_OK;
}

long long field_dof(const Lattice* L, int field) {
  if (L->NS == 0 && field >= TX_FIELD_SPECIES_FI && field <= TX_FIELD_SPECIES_FLUX) return -1;
  switch (field) {
    case TX_FIELD_SPECIES_FI: return (long long)L->NS * L->Q;
    case TX_FIELD_SPECIES_RHO: return L->NS;
    case TX_FIELD_SPECIES_FLUX: return (long long)L->NS * L->D;
    case TX_FIELD_FI: return (long long)L->S * L->Q;
    case TX_FIELD_RHO:
    case TX_FIELD_PSI: return L->S;
    case TX_FIELD_FLUX:
    case TX_FIELD_FORCES: return (long long)L->S * L->D;
    case TX_FIELD_PRS:
    case TX_FIELD_RHOT: return 1;
    case TX_FIELD_VELT: return L->D;
  }
  return -1;
}

}  // namespace

extern "C" {

int tx_batch_create(const tx_params* form, int64_t hbm_budget_bytes, tx_batch** out) {
  if (!form || !out) return TX_ERR_ARG;
  *out = nullptr;
  tx_params f = *form;
  if (f.exact) {
    tx::set_global_error("batches run the fast forms only (exact must be 0)");
    return TX_ERR_ARG;
  }
  // the geometry of the form is irrelevant: validate it on a small lattice
  f.nx = f.ny = 4;
  f.nz = f.discretization == TX_D3Q19 ? 4 : 1;
  std::string why;
  const int rc = tx::validate(&f, &why);
  if (rc) {
    tx::set_global_error(why);
    return rc;
  }
  tx_batch* b = new tx_batch();
  b->form = f;
  b->D = f.discretization == TX_D3Q19 ? 3 : 2;
  b->S = f.ncomponents;
  b->Q = b->D == 3 ? 19 : 9;
  b->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : 0;
  // lattices added later may carry any MRT rates
  if (!select_kernels(&f, &b->ks, true) || (f.nspecies > 0 && !select_species(&f, &b->ss))) {
    delete b;
    tx::set_global_error("no kernel built for this parameter combination");
    return TX_ERR_ARG;
  }
  if (b->D == 2) {
    b->bx = 32;
    b->by = 4;
    b->bz = 1;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&b->d_ntiles, sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_nltiles, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&b->d_nftiles, sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_notiles, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&b->d_nstiles, sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_nptiles, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&b->d_nrtiles, sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_count, sizeof(unsigned)) != cudaSuccess) {
    tx::set_global_error("CUDA device setup failed");
    tx_batch_destroy(b);
    return TX_ERR_NODEVICE;
  }
  cudaMemset(b->d_ntiles, 0, sizeof(int));
  cudaMemset(b->d_nltiles, 0, sizeof(int));
  cudaMemset(b->d_nftiles, 0, sizeof(int));
  cudaMemset(b->d_notiles, 0, sizeof(int));
  cudaMemset(b->d_nstiles, 0, sizeof(int));
  cudaMemset(b->d_nptiles, 0, sizeof(int));
  cudaMemset(b->d_nrtiles, 0, sizeof(int));
  *out = b;
  return TX_OK;
}

int tx_batch_destroy(tx_batch* b) {
  if (!b) return TX_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (Lattice* L : b->slots) free_lattice(b, L);
  b->slots.clear();
  for (void* p : {(void*)b->d_lats, (void*)b->d_tiles, (void*)b->d_parts, (void*)b->d_res, (void*)b->d_ltiles,
                 (void*)b->d_ftiles, (void*)b->d_otiles, (void*)b->d_stiles, (void*)b->d_ptiles, (void*)b->d_rtiles})
    if (p) cudaFreeAsync(p, b->stream);
  if (b->stream) cudaStreamSynchronize(b->stream);
  cudaFree(b->d_ntiles);
  cudaFree(b->d_nltiles);
  cudaFree(b->d_nftiles);
  cudaFree(b->d_notiles);
  cudaFree(b->d_nstiles);
  cudaFree(b->d_nptiles);
  cudaFree(b->d_nrtiles);
  cudaFree(b->d_count);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return TX_OK;
}

const char* tx_batch_last_error(const tx_batch* b) { return b ? b->err.c_str() : tx_last_error(nullptr); }

int64_t tx_batch_lattice_bytes(const tx_params* p) { return p ? lattice_bytes(*p) : -1; }
int64_t tx_batch_bytes_in_use(const tx_batch* b) { return b ? b->in_use : -1; }
int32_t tx_batch_count(const tx_batch* b) { return b ? (int32_t)b->slots.size() : -1; }
void* tx_batch_stream(tx_batch* b) { return b ? (void*)b->stream : nullptr; }

int tx_batch_add(tx_batch* b, const tx_params* p, const double* walls, const double* rho, const double* u,
                 const double* conc, int32_t* id) {
  if (!b || !p || !walls || !rho || !id) return TX_ERR_ARG;
  if (p->nspecies > 0 && !conc) return bfail(b, TX_ERR_ARG, "the lattice has species: conc is required");
  std::string why;
  int rc = tx::validate(p, &why);
  if (rc) return bfail(b, rc, why);
  const tx_params& f = b->form;
  if (p->discretization != f.discretization || p->ncomponents != f.ncomponents ||
      p->relaxation_mode != f.relaxation_mode || p->isotropy_order != f.isotropy_order ||
      p->precision != f.precision || p->exact || p->nspecies != f.nspecies ||
      (p->nspecies > 0 && p->species_relaxation_mode != f.species_relaxation_mode))
    return bfail(b, TX_ERR_ARG, "lattice parameters do not match the batch's kernel form");
  const long long bytes = lattice_bytes(*p);
  if (b->budget && b->in_use + bytes > b->budget)
    return bfail(b, TX_ERR_NOMEM, "lattice needs " + std::to_string(bytes) + " bytes; " +
                                      std::to_string(b->budget - b->in_use) + " left in the budget");
  Lattice* L = new Lattice();
  L->p = *p;
  L->D = b->D;
  L->S = b->S;
  L->Q = b->Q;
  L->g.nx = p->nx;
  L->g.ny = p->ny;
  L->g.nz = b->D == 3 ? p->nz : 1;
  for (int a = 0; a < 3; ++a) L->g.per[a] = a < b->D ? p->bc_flags[2 * a] == TX_BC_PERIODIC : 1;
  L->g.n = (long long)L->g.nx * L->g.ny * L->g.nz;
  const long long N = L->g.n;
  const int S = b->S, Q = b->Q, D = b->D;
  fill_phys_impl(*p, D, S, Q, L->ph);

  // host-side preparation first, so that a bad argument allocates nothing
  std::vector<uint8_t> mask((size_t)N);
  for (long long i = 0; i < N; ++i) {
    const char* w = nullptr;
    if (!wall_code(walls[i], p->nminerals, &mask[(size_t)i], &w, D)) {
      delete L;
      return bfail(b, TX_ERR_ARG, w);
    }
  }
  std::vector<double> rt((size_t)N * S);
  for (long long i = 0; i < N; ++i)
    for (int m = 0; m < S; ++m) rt[(size_t)(i * S + m)] = mask[(size_t)i] == 0 ? rho[i * S + m] - L->ph.rho0[m] : 0.0;
  std::vector<float> rt32;
  if (rho_bytes(p->precision) == 4) rt32.assign(rt.begin(), rt.end());
  // psi(rho) of the initial density for the forces of FlowFiInit
  std::vector<double> ps;
  std::vector<float> ps32;
  if (p->use_nonideal_eos) {
    ps.assign((size_t)N * S, 0.0);
    for (long long i = 0; i < N; ++i)
      if (mask[(size_t)i] == 0)
        for (int m = 0; m < S; ++m)
          ps[(size_t)(i * S + m)] = eos_psi<double>(L->ph.eos[m], L->ph.eos_c[m], L->ph.g[m][m], L->ph.c0, rho[i * S + m]);
    if (rho_bytes(p->precision) == 4) ps32.assign(ps.begin(), ps.end());
  }
  std::vector<double> ut;
  if (u) {
    ut.resize((size_t)N * S * D);
    for (long long i = 0; i < N; ++i)
      for (int d = 0; d < D; ++d)
        for (int m = 0; m < S; ++m) ut[((size_t)(m * D + d)) * N + i] = u[(i * D + d) * S + m];
  }
  PhysT<float> ph32{};
  convert_phys(L->ph, &ph32);

  cudaStream_t st = b->stream;
  const size_t popb = (size_t)N * S * Q * pop_bytes(p->precision);
  const size_t physb = p->precision == TX_PREC_F64 ? sizeof(Phys) : sizeof(PhysT<float>);
  double* uic = nullptr;
  auto undo = [&](const std::string& msg, int code) {
    if (uic) cudaFreeAsync(uic, st);
    free_lattice(b, L);  // subtracts L->bytes, which is still 0
    cudaStreamSynchronize(st);
    return bfail(b, code, msg);
  };
#define TX_BALLOC(ptr, sz)                                                   \
  if (cudaMallocAsync((void**)&(ptr), (sz), st) != cudaSuccess) {           \
    cudaGetLastError();                                                     \
    return undo("device allocation failed", TX_ERR_NOMEM);                  \
  }
  TX_BALLOC(L->f[0], popb);
  TX_BALLOC(L->f[1], popb);
  TX_BALLOC(L->rho, (size_t)N * S * rho_bytes(p->precision));
  if (p->use_nonideal_eos) TX_BALLOC(L->psi, (size_t)N * S * rho_bytes(p->precision));
  TX_BALLOC(L->mask, (size_t)N);
  TX_BALLOC(L->links, (size_t)N * sizeof(uint32_t));
  TX_BALLOC(L->uold, (size_t)N * D * sizeof(double));
  TX_BALLOC(L->steps_dev, sizeof(unsigned));
  TX_BALLOC(L->phys, physb);
  setup_faces(*p, D, &L->faces);
  L->shell = face_shell(*p, D, L->g.nx, L->g.ny, L->g.nz);
  for (int fc = 0; fc < 2 * D; ++fc) {
    if (!face_has_values(*p, D, fc)) continue;
    const long long area = face_area(*p, D, fc);
    double nv[3 * TX_MAX_COMPONENTS];
    face_node_values(*p, D, fc, L->ph.c0, nv);
    std::vector<double> v((size_t)area * S * D);
    for (int k = 0; k < S * D; ++k)
      for (long long q = 0; q < area; ++q) v[(size_t)(k * area + q)] = nv[k];
    TX_BALLOC(L->faceval[fc], v.size() * sizeof(double));
    if (cudaMemcpyAsync(L->faceval[fc], v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return undo("face upload failed", TX_ERR_CUDA);
    L->faces.vals[fc] = L->faceval[fc];
  }
  if (u) TX_BALLOC(uic, ut.size() * sizeof(double));
  // species: populations, parameters and the initial concentration
  double* sconc = nullptr;
  SpeciesPhysT<double> sp{};
  SpeciesPhysT<float> sp32{};
  const size_t spb = p->precision == TX_PREC_F64 ? sizeof(sp) : sizeof(sp32);
  const size_t gb = (size_t)N * p->nspecies * Q * pop_bytes(p->precision);
  if (p->nspecies > 0) {
    L->NS = p->nspecies;
    fill_species_phys(*p, D, sp);
    convert_species(sp, &sp32);
    TX_BALLOC(L->sg[0], gb);
    TX_BALLOC(L->sg[1], gb);
    TX_BALLOC(L->sphys, spb);
    TX_BALLOC(sconc, (size_t)N * p->nspecies * sizeof(double));
  }
#undef TX_BALLOC
  const void* phsrc = p->precision == TX_PREC_F64 ? (const void*)&L->ph : (const void*)&ph32;
  bool ok = cudaMemcpyAsync(L->phys, phsrc, physb, cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(L->mask, mask.data(), (size_t)N, cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemsetAsync(L->f[0], 0, popb, st) == cudaSuccess && cudaMemsetAsync(L->f[1], 0, popb, st) == cudaSuccess &&
            cudaMemsetAsync(L->uold, 0, (size_t)N * D * sizeof(double), st) == cudaSuccess &&
            cudaMemsetAsync(L->steps_dev, 0, sizeof(unsigned), st) == cudaSuccess;
  if (ok)
    ok = rt32.empty() ? cudaMemcpyAsync(L->rho, rt.data(), rt.size() * 8, cudaMemcpyHostToDevice, st) == cudaSuccess
                      : cudaMemcpyAsync(L->rho, rt32.data(), rt32.size() * 4, cudaMemcpyHostToDevice, st) == cudaSuccess;
  if (ok && uic) ok = cudaMemcpyAsync(uic, ut.data(), ut.size() * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess;
  if (ok && L->psi)
    ok = ps32.empty() ? cudaMemcpyAsync(L->psi, ps.data(), ps.size() * 8, cudaMemcpyHostToDevice, st) == cudaSuccess
                      : cudaMemcpyAsync(L->psi, ps32.data(), ps32.size() * 4, cudaMemcpyHostToDevice, st) == cudaSuccess;
  if (ok && L->NS > 0)
    ok = cudaMemcpyAsync(L->sphys, p->precision == TX_PREC_F64 ? (const void*)&sp : (const void*)&sp32, spb,
                         cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaMemsetAsync(L->sg[0], 0, gb, st) == cudaSuccess && cudaMemsetAsync(L->sg[1], 0, gb, st) == cudaSuccess &&
         cudaMemcpyAsync(sconc, conc, (size_t)N * L->NS * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess;
  if (!ok) {
    if (sconc) cudaFreeAsync(sconc, st);
    return undo("state upload failed", TX_ERR_CUDA);
  }
  {
    const Launch3 l = launch3(L->g, 256);
    if (D == 3)
      k_links<3><<<l.grid, l.block, 0, st>>>(L->mask, L->g, L->links);
    else
      k_links<2><<<l.grid, l.block, 0, st>>>(L->mask, L->g, L->links);
  }
  // the paired step and its pairs for the per-site kernel
  L->paired = b->ks.paired(L->g);
  L->rest = -1;
  if (L->paired) {
    unsigned n = 0;
    const bool okc = cudaMemsetAsync(b->d_count, 0, sizeof(unsigned), st) == cudaSuccess &&
                     (b->ks.count_rest(lattice_args(b, L, b->flip, b->flip), b->d_count, st),
                      cudaGetLastError() == cudaSuccess) &&
                     cudaMemcpyAsync(&n, b->d_count, sizeof(unsigned), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                     cudaStreamSynchronize(st) == cudaSuccess;
    if (!okc) {
      if (sconc) cudaFreeAsync(sconc, st);
      return undo("pair count failed", TX_ERR_CUDA);
    }
    L->rest = (int)n;
  }
  // FlowFiInit + FlowUpdateMoments into the buffer that holds the state at the batch's flip
  const StepArgs a = lattice_args(b, L, b->flip, b->flip);
  b->ks.init(a, uic, st);
  b->ks.density(a, 1, st);
  if (L->NS > 0) {
    // TransportFiInit into the species buffer of the batch's flip
    SpeciesArgs sa{};
    sa.gin = L->sg[b->flip];
    sa.gout = L->sg[b->flip];
    sa.links = L->links;
    sa.mask = L->mask;
    sa.phys = L->sphys;
    sa.g = L->g;
    sa.ns = L->NS;
    b->ss.init(sa, sconc, nullptr, st);
  }
  const cudaError_t e = cudaGetLastError();
  const cudaError_t es = cudaStreamSynchronize(st);  // the host staging vectors die with this call
  if (e != cudaSuccess || es != cudaSuccess)
    return undo(std::string("lattice init: ") + cudaGetErrorString(e != cudaSuccess ? e : es), TX_ERR_CUDA);
  if (uic) cudaFreeAsync(uic, st);
  if (sconc) cudaFreeAsync(sconc, st);
  L->bytes = bytes;
  b->in_use += bytes;
  L->id = b->next_id++;
  b->slots.push_back(L);
  // the face pass and the outlet refresh join the step (and its graph) with
  // the first lattice that needs them, and stay
  const bool nf = b->need_faces || L->faces.post, no = b->need_outlets || has_outlet_update(*p, D);
  if (nf != b->need_faces || no != b->need_outlets) drop_graph(b);
  b->need_faces = nf;
  b->need_outlets = no;
  rc = rebuild_tables(b);
  if (rc) return rc;
  *id = L->id;
  return TX_OK;
}

int tx_batch_remove(tx_batch* b, int32_t id) {
  if (!b) return TX_ERR_ARG;
  for (size_t s = 0; s < b->slots.size(); ++s) {
    if (b->slots[s]->id != id) continue;
    Lattice* L = b->slots[s];
    b->slots.erase(b->slots.begin() + (long)s);
    const int rc = rebuild_tables(b);  // the device tables stop naming the lattice before its memory goes
    free_lattice(b, L);
    return rc;
  }
  return bfail(b, TX_ERR_ARG, "no lattice with id " + std::to_string(id));
}

int tx_batch_sync(tx_batch* b) {
  if (!b) return TX_ERR_ARG;
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  return TX_OK;
}

int tx_batch_step(tx_batch* b, int32_t nsteps) {
  const int rc = tx_batch_launch(b, nsteps);
  return rc ? rc : tx_batch_sync(b);
}

int tx_batch_launch(tx_batch* b, int32_t nsteps) {
  if (!b) return TX_ERR_ARG;
  if (nsteps < 0) return bfail(b, TX_ERR_ARG, "nsteps must be >= 0");
  if (b->slots.empty() || nsteps == 0) return TX_OK;
  if (!b->tables_ok) return bfail(b, TX_ERR_STATE, "the batch's device tables were not rebuilt after the last change (see the error it returned)");
  int left = nsteps;
  while (left > 0) {
    if (b->graph_steps > 0 && b->flip == 0 && left >= b->graph_steps) {
      if (!b->exec) {
        const int rc = capture_graph(b);
        if (rc) return rc;
      }
      TX_BCUDA(b, cudaGraphLaunch(b->exec, b->stream));
      left -= b->graph_steps;
    } else {
      const int rc = launch_step(b, b->flip);
      if (rc) return rc;
      b->flip ^= 1;
      --left;
    }
  }
  for (Lattice* L : b->slots) L->steps += nsteps;
  return TX_OK;
}

int tx_batch_probe(tx_batch* b, int32_t cap, tx_probe* out, int32_t* n) {
  if (!b || !n || (cap > 0 && !out)) return TX_ERR_ARG;
  const int nl = (int)b->slots.size();
  *n = nl;
  if (!nl) return TX_OK;
  if (!b->tables_ok) return bfail(b, TX_ERR_STATE, "the batch's device tables were not rebuilt after the last change (see the error it returned)");
  const dim3 blk((unsigned)b->bx, (unsigned)b->by, (unsigned)b->bz);
  b->ks.probe_tiles(bargs(b), b->flip, grid_of(b), blk, b->stream);
  k_probe_reduce<<<nl, 256, 0, b->stream>>>(b->d_lats, nl, b->d_parts, b->d_res);
  TX_BCUDA(b, cudaGetLastError());
  std::vector<ProbePart> res((size_t)nl);
  TX_BCUDA(b, cudaMemcpyAsync(res.data(), b->d_res, (size_t)nl * sizeof(ProbePart), cudaMemcpyDeviceToHost, b->stream));
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  for (int s = 0; s < nl && s < cap; ++s) {
    tx_probe& o = out[s];
    std::memset(&o, 0, sizeof(o));
    o.id = b->slots[(size_t)s]->id;
    o.du_max = res[(size_t)s].du;
    o.u_max = res[(size_t)s].umax;
    for (int d = 0; d < 3; ++d) o.u_sum[d] = res[(size_t)s].usum[d];
    o.pore_sites = (int64_t)res[(size_t)s].npore;
    o.steps = b->slots[(size_t)s]->steps;
    for (int m = 0; m < TX_MAX_COMPONENTS && m < MAXC; ++m) o.mass[m] = res[(size_t)s].mass[m];
  }
  return TX_OK;
}

int tx_batch_download(tx_batch* b, int32_t id, int32_t field, double* out) {
  if (!b || !out) return TX_ERR_ARG;
  const Lattice* L = nullptr;
  for (const Lattice* c : b->slots)
    if (c->id == id) L = c;
  if (!L) return bfail(b, TX_ERR_ARG, "no lattice with id " + std::to_string(id));
  if (field == TX_FIELD_WALLS) return bfail(b, TX_ERR_ARG, "walls are not kept on the host in a batch");
  const long long dof = field_dof(L, field);
  if (dof < 0) return bfail(b, TX_ERR_ARG, "unknown field");
  const size_t bytes = (size_t)(dof * L->g.n) * sizeof(double);
  double* d = nullptr;
  TX_BCUDA(b, cudaMallocAsync((void**)&d, bytes, b->stream));
  int rc = stage(b, L, field, d);
  if (rc == TX_OK) {
    const cudaError_t e1 = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, b->stream);
    if (e1 != cudaSuccess) rc = bfail(b, TX_ERR_CUDA, cudaGetErrorString(e1));
  }
  cudaFreeAsync(d, b->stream);
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  return rc;
}

int tx_batch_set_tiles(tx_batch* b, int32_t bx, int32_t by, int32_t bz, int32_t blocks_per_sm) {
  if (!b) return TX_ERR_ARG;
  if (bx < 1 || by < 1 || bz < 1 || bx * by * bz != 128 || (b->D == 2 && bz != 1) || blocks_per_sm < 1 ||
      blocks_per_sm > 32)
    return bfail(b, TX_ERR_ARG, "tiles must hold 128 threads (bz = 1 in 2D) and 1..32 blocks per SM");
  const bool same = bx == b->bx && by == b->by && bz == b->bz && blocks_per_sm == b->blocks_per_sm;
  if (same) return TX_OK;
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  drop_graph(b);
  b->bx = bx;
  b->by = by;
  b->bz = bz;
  b->blocks_per_sm = blocks_per_sm;
  return rebuild_tables(b);
}

int tx_batch_set_graph(tx_batch* b, int32_t steps_per_graph) {
  if (!b) return TX_ERR_ARG;
  if (steps_per_graph < 0 || steps_per_graph == 1 || (steps_per_graph & 1))
    return bfail(b, TX_ERR_ARG, "steps per graph must be 0 or an even number >= 2");
  TX_BCUDA(b, cudaStreamSynchronize(b->stream));
  drop_graph(b);
  b->graph_steps = steps_per_graph;
  return TX_OK;
}

int tx_batch_tune(tx_batch* b, int32_t steps_per_trial, int32_t* chosen) {
  if (!b || steps_per_trial < 1) return TX_ERR_ARG;
  if (b->slots.empty()) return bfail(b, TX_ERR_STATE, "tune needs lattices in the batch");
  if (!b->tables_ok) return bfail(b, TX_ERR_STATE, "the batch's device tables were not rebuilt after the last change (see the error it returned)");
  struct Cand {
    int bx, by, bz, bps;
  };
  std::vector<Cand> cands;
  const int shapes3[][3] = {{128, 1, 1}, {64, 2, 1}, {32, 4, 1}, {32, 2, 2}, {16, 8, 1}, {16, 4, 2}};
  const int shapes2[][3] = {{128, 1, 1}, {64, 2, 1}, {32, 4, 1}, {16, 8, 1}};
  const int nshape = b->D == 3 ? 6 : 4;
  for (int s = 0; s < nshape; ++s)
    for (int bps : {4, 8}) {
      const int* sh = b->D == 3 ? shapes3[s] : shapes2[s];
      cands.push_back({sh[0], sh[1], sh[2], bps});
    }
  cudaEvent_t e0, e1;
  TX_BCUDA(b, cudaEventCreate(&e0));
  TX_BCUDA(b, cudaEventCreate(&e1));
  float best = 1e30f;
  Cand win = cands[0];
  int rc = TX_OK;
  for (const Cand& c : cands) {
    rc = tx_batch_set_tiles(b, c.bx, c.by, c.bz, c.bps);
    if (rc) break;
    rc = launch_step(b, b->flip);  // untimed warm-up
    if (rc) break;
    b->flip ^= 1;
    cudaEventRecord(e0, b->stream);
    for (int s = 0; s < steps_per_trial && rc == TX_OK; ++s) {
      rc = launch_step(b, b->flip);
      b->flip ^= 1;
    }
    cudaEventRecord(e1, b->stream);
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = bfail(b, TX_ERR_CUDA, "tune timing failed");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    for (Lattice* L : b->slots) L->steps += steps_per_trial + 1;
    if (ms < best) {
      best = ms;
      win = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  rc = tx_batch_set_tiles(b, win.bx, win.by, win.bz, win.bps);
  if (rc) return rc;
  if (chosen) {
    chosen[0] = win.bx;
    chosen[1] = win.by;
    chosen[2] = win.bz;
    chosen[3] = win.bps;
  }
  return TX_OK;
}

}  // extern "C"
