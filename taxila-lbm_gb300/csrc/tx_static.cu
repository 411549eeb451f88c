// tx_step_static: the flow step for callers that cannot allocate device memory.
//
// Some hosts of this library own every byte of device memory themselves, for
// example an application that pre-allocates one arena at start-up and forbids
// later cudaMalloc calls, or a plugin that is handed device buffers by its
// host.  Such callers can still run the step: they pass their own device
// arrays for the inputs (walls, populations) and the output (populations), and
// all working storage of the step (wall mask, forcing density, parameters,
// density-face values and the two ping-pong population buffers) lives in one
// file-scope device array, tx_static_scratch, of TX_STATIC_SCRATCH_BYTES.
// Every GPU that loads the library holds that array until the process exits.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (the host-side name is only a stand-in and must never be
// passed to a kernel) and keeps it for the life of the process; make that
// first call before any stream capture.  A cudaDeviceReset unloads the
// library's device code, so the kept address is stale afterwards: do not call
// tx_step_static on a device after resetting it in the same process.  All
// calls share the one array and leave its contents behind: each call clears
// what has to start at zero, and calls whose GPU work overlaps (two streams,
// two host threads) race on it.  A call that fails after queueing work waits
// for that work before it returns, so a retry never overlaps it.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/taxila_gb300.h"
#include "tx_dispatch.h"

using namespace tx;

namespace {

static __device__ __align__(256) unsigned char tx_static_scratch[TX_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};
}  // namespace

namespace tx {
void set_global_error(const std::string& msg);
}

namespace {

// errors of tx_step_static are reported through tx_last_error(NULL)
int static_fail(int code, const std::string& msg) {
  tx::set_global_error(msg);
  return code;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// walls (reference codes, natural order) -> mask; records a bad code (the
// specular codes too: 900, 901 and, in 3D, 902; in 2D 902 is a plain wall)
__global__ void k_static_mask(const double* walls, long long n, int nminerals, int D, uint8_t* mask, unsigned* bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = walls[i];
  uint8_t code;
  if (v == 0.0) {
    code = 0;
  } else if (!(v > 0.0) || v == 900.0 || v == 901.0 || (v == 902.0 && D == 3) || !isfinite(v)) {
    atomicOr(bad, 1u);
    code = 255;
  } else {
    const int mineral = (int)v;
    code = (v < 998.0 && mineral >= 1 && mineral <= nminerals) ? (uint8_t)mineral : (uint8_t)255;
  }
  mask[i] = code;
}

__global__ void k_static_fill(double* p, long long n, double v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace

// Parameter translation shared with tx_abi.cu.
namespace tx {
int validate_params(const tx_params* p, std::string* why);
void fill_phys_from(const tx_params& p, int D, int S, int Q, Phys* out);
bool select_kernels(const tx_params* p, KernelSet* ks, bool any_rates = false);
}  // namespace tx

extern "C" int tx_step_static(const tx_params* p, const double* walls, const double* fi_in, double* fi_out,
                              int32_t nsteps, void* stream_ptr) {
  if (!p || !walls || !fi_in || !fi_out) return static_fail(TX_ERR_ARG, "null argument");
  if (nsteps < 0) return static_fail(TX_ERR_ARG, "nsteps must be >= 0");
  std::string why;
  int rc = validate_params(p, &why);
  if (rc) return static_fail(rc, why);
  if (p->precision != TX_PREC_F64) return static_fail(TX_ERR_ARG, "tx_step_static runs the FP64 form only");
  if (p->nspecies != 0) return static_fail(TX_ERR_ARG, "tx_step_static runs the flow only (nspecies must be 0)");
  KernelSet ks{};
  if (!select_kernels(p, &ks)) return static_fail(TX_ERR_ARG, "no kernel built for this parameter combination");

  const int D = p->discretization == TX_D3Q19 ? 3 : 2;
  const int S = p->ncomponents, Q = D == 3 ? 19 : 9;
  Geo g{};
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = D == 3 ? p->nz : 1;
  for (int a = 0; a < 3; ++a) g.per[a] = a < D ? p->bc_flags[2 * a] == TX_BC_PERIODIC : 1;
  g.n = (long long)g.nx * g.ny * g.nz;
  const long long N = g.n;

  // carve the scratch array: parameters | mask | links | rho | face values | populations A | populations B | flag
  long long area[6] = {0, 0, 0, 0, 0, 0};
  for (int f = 0; f < 2 * D; ++f)
    if (face_has_values(*p, D, f)) area[f] = face_area_of(D, g.nx, g.ny, g.nz, f);
  size_t off = 0;
  const size_t o_phys = off;
  off = align256(off + sizeof(Phys));
  const size_t o_mask = off;
  off = align256(off + (size_t)N);
  const size_t o_links = off;
  off = align256(off + (size_t)N * sizeof(uint32_t));
  const size_t o_rho = off;
  off = align256(off + (size_t)N * S * sizeof(double));
  const size_t o_psi = off;
  if (p->use_nonideal_eos) off = align256(off + (size_t)N * S * sizeof(double));
  size_t o_face[6];
  for (int f = 0; f < 6; ++f) {
    o_face[f] = off;
    off = align256(off + (size_t)area[f] * S * D * sizeof(double));
  }
  const size_t pop_bytes = (size_t)N * S * Q * sizeof(double);
  const size_t o_pa = off;
  off = align256(off + pop_bytes);
  const size_t o_pb = off;
  off = align256(off + pop_bytes);
  const size_t o_flag = off;
  off = align256(off + sizeof(unsigned));
  if (off > (size_t)TX_STATIC_SCRATCH_BYTES)
    return static_fail(TX_ERR_ARG, "lattice needs " + std::to_string(off) + " bytes of working storage; "
                                   "tx_step_static has " + std::to_string((long long)TX_STATIC_SCRATCH_BYTES) +
                                   " (use tx_create for larger lattices)");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return static_fail(TX_ERR_NODEVICE, "no current CUDA device");
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_scratch_addr[dev]) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, tx_static_scratch);
      if (e != cudaSuccess || !ptr)
        return static_fail(TX_ERR_CUDA, std::string("cudaGetSymbolAddress(tx_static_scratch): ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = (unsigned char*)ptr;
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream_ptr;

  Phys ph{};
  fill_phys_from(*p, D, S, Q, &ph);
  Phys* d_phys = (Phys*)(base + o_phys);
  uint8_t* mask = base + o_mask;
  uint32_t* links = (uint32_t*)(base + o_links);
  double* rho = (double*)(base + o_rho);
  double* pa = (double*)(base + o_pa);
  double* pb = (double*)(base + o_pb);
  unsigned* flag = (unsigned*)(base + o_flag);

  // on an error after work was queued, wait for that work (ignoring the
  // result) before returning, so that no kernel still writes the static area
  // when the caller retries
#define TX_SCHK(call)                                                                 \
  do {                                                                                \
    const cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                          \
      (void)cudaStreamSynchronize(st);                                                \
      return static_fail(TX_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    }                                                                                 \
  } while (0)

  // what must start at zero: the flag, the density and the second population buffer
  TX_SCHK(cudaMemcpyAsync(d_phys, &ph, sizeof(Phys), cudaMemcpyHostToDevice, st));
  TX_SCHK(cudaMemsetAsync(flag, 0, sizeof(unsigned), st));
  TX_SCHK(cudaMemsetAsync(rho, 0, (size_t)N * S * sizeof(double), st));
  TX_SCHK(cudaMemsetAsync(pb, 0, pop_bytes, st));
  k_static_mask<<<grid_for(N, 256), 256, 0, st>>>(walls, N, p->nminerals, D, mask, flag);
  {
    const Launch3 l = launch3(g, 256);
    if (D == 3)
      k_links<3><<<l.grid, l.block, 0, st>>>(mask, g, links);
    else
      k_links<2><<<l.grid, l.block, 0, st>>>(mask, g, links);
  }
  Faces faces{};
  setup_faces(*p, D, &faces);
  for (int f = 0; f < 2 * D; ++f) {
    if (!area[f]) continue;
    double* v = (double*)(base + o_face[f]);
    double nv[3 * TX_MAX_COMPONENTS];
    face_node_values(*p, D, f, ph.c0, nv);
    for (int k = 0; k < S * D; ++k)
      k_static_fill<<<grid_for(area[f], 256), 256, 0, st>>>(v + (long long)k * area[f], area[f], nv[k]);
    faces.vals[f] = v;
  }
  TX_SCHK(cudaGetLastError());
  // reject bad wall codes before any step touches fi_out
  {
    unsigned bad = 0;
    TX_SCHK(cudaMemcpyAsync(&bad, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    TX_SCHK(cudaStreamSynchronize(st));
    if (bad) return static_fail(TX_ERR_ARG, "wall codes must be 0 or positive; specular codes 900-902 are not supported");
  }

  StepArgs a{};
  a.rho = rho;
  a.psi = p->use_nonideal_eos ? (void*)(base + o_psi) : nullptr;
  a.mask = mask;
  a.links = links;
  a.phys = d_phys;
  a.g = g;
  a.faces = faces;
  // restart from fi_in exactly like tx_upload_fi + tx_init (FlowUpdateMoments: plain sums)
  ks.from_natural(fi_in, mask, N, shift_of(ph), pa, st);
  a.fin = pa;
  a.fout = pa;
  ks.density(a, 1, st);
  double* cur = pa;
  double* nxt = pb;
  const FaceShell shell = face_shell(*p, D, g.nx, g.ny, g.nz);
  const bool outlet = has_outlet_update(*p, D);
  for (int t = 0; t < nsteps; ++t) {
    a.fin = cur;
    a.fout = nxt;
    if (outlet)
      for (int f = 0; f < 2 * D; ++f)
        if (p->bc_flags[f] == TX_BC_PRESSURE_OUTLET)
          ks.outlet(a, f, (double*)(base + o_face[f]), p->bc_data[f][0], ph.c0, p->g[1][0], st);
    ks.step(a, st);
    ks.density(a, 0, st);
    if (faces.post) ks.faces(a, shell, st);
    double* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  ks.to_natural(cur, mask, N, shift_of(ph), fi_out, st);
  TX_SCHK(cudaGetLastError());
  TX_SCHK(cudaStreamSynchronize(st));
#undef TX_SCHK
  return TX_OK;
}
