// Kernel tables: one KernelSet per (dimension, components, isotropy, MRT,
// exactness, storage form); built by the tx_inst_*.cu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tx_batch.cuh"
#include "tx_host_params.h"
#include "tx_kernels.cuh"
#include "tx_pair.cuh"
#include "tx_species.cuh"

namespace tx {

struct KernelSet {
  void (*step)(const StepArgs&, cudaStream_t);
  void (*density)(const StepArgs&, int mode, cudaStream_t);
  void (*init)(const StepArgs&, const double* uic, cudaStream_t);
  void (*moments)(const StepArgs&, int what, double* out, cudaStream_t);
  void (*to_natural)(const void* f, const uint8_t* mask, long long N, Shift sh, double* out, cudaStream_t);
  void (*from_natural)(const double* in, const uint8_t* mask, long long N, Shift sh, void* f, cudaStream_t);
  // batched (persistent, tile-table) kernels; no-ops in the exact FP64 form
  void (*step_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);
  void (*density_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);
  void (*probe_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);
  // exterior BCs beyond Dirichlet faces: the face pass after k_density, and the
  // per-step refresh of one two-component pressure-outlet face before k_step
  void (*faces)(const StepArgs&, const FaceShell&, cudaStream_t);
  void (*outlet)(const StepArgs&, int face, double* vals, double pressure, double c0, double g21, cudaStream_t);
  // their batched forms (no-ops in the exact form)
  void (*faces_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);
  void (*outlet_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);
  // paired-site step (FP32-arithmetic forms, even site count): whether a lattice takes
  // it, and how many of its pairs need the per-site kernel (counted into *count)
  bool (*paired)(const Geo&);
  void (*count_rest)(const StepArgs&, unsigned* count, cudaStream_t);
  const char* name;
};

// Passive-species kernels of one (dimension, form); built by the s1 units.
struct SpeciesSet {
  void (*step)(const SpeciesArgs&, cudaStream_t);
  void (*init)(const SpeciesArgs&, const double* conc, const double* flux, cudaStream_t);
  void (*fields)(const SpeciesArgs&, int what, double* out, cudaStream_t);
  void (*step_tiles)(const BatchArgs&, int flip, int grid, dim3 block, cudaStream_t);  // no-op in the exact form
  void (*wall_collide)(const SpeciesArgs&, cudaStream_t);  // 2D with specular walls: collide wall cells in gout
};
bool species_d3_exact(bool mrt, SpeciesSet* ss);
bool species_d2_exact(bool mrt, SpeciesSet* ss);
bool species_d3_f64(bool mrt, SpeciesSet* ss);
bool species_d2_f64(bool mrt, SpeciesSet* ss);
bool species_d3_f32(bool mrt, SpeciesSet* ss);
bool species_d2_f32(bool mrt, SpeciesSet* ss);
bool species_d3_f16(bool mrt, SpeciesSet* ss);
bool species_d2_f16(bool mrt, SpeciesSet* ss);

bool kernels_d3_exact_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_exact_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_exact_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_exact_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f64_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f64_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f64_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f64_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f32_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f32_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f32_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f32_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f16_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d3_f16_s2(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f16_s1(int S, int ISO, bool MRT, KernelSet* ks);
bool kernels_d2_f16_s2(int S, int ISO, bool MRT, KernelSet* ks);

inline unsigned grid_for(long long n, int block) { return (unsigned)((n + block - 1) / block); }

// Lattice kernels run on an (x-tile, y-tile, z) grid of `threads` threads per
// block: x tiles of up to 128 sites (a multiple of 32), the rest of the block in y.
struct Launch3 {
  dim3 grid, block;
};
inline Launch3 launch3(const Geo& g, int threads);
// the launch of the paired kernels: one-dimensional, `per` pairs per thread
inline Launch3 launch_pairs(const Geo& g, int threads, int per = 1) {
  Launch3 l;
  l.block = dim3((unsigned)threads, 1, 1);
  l.grid = dim3(grid_for(g.n / 2, threads * per), 1, 1);
  return l;
}
inline Launch3 launch3(const Geo& g, int threads) {
  int bx = ((g.nx + 31) / 32) * 32;
  if (bx > 128) bx = 128;
  if (bx > threads) bx = threads;
  int by = threads / bx;
  if (by < 1) by = 1;
  Launch3 l;
  l.block = dim3((unsigned)bx, (unsigned)by, 1);
  l.grid = dim3((unsigned)((g.nx + bx - 1) / bx), (unsigned)((g.ny + by - 1) / by), (unsigned)g.nz);
  return l;
}

}  // namespace tx

// Instantiates the launchers of one storage/arithmetic form for one dimension.
#define TX_FORM_LAUNCHERS(D, S, ISO, MRT, EXACT, T, R, RT) TX_FORM_LAUNCHERS_(D, S, ISO, MRT, EXACT, T, R, RT)
#define TX_FORM_LAUNCHERS_(D, S, ISO, MRT, EXACT, T, R, RT)                                                  \
  struct L_##S##_##ISO##_##MRT {                                                                             \
    static constexpr bool kPairForm = !EXACT && std::is_same<R, float>::value;                                \
    static bool paired(const Geo& g) { return kPairForm && g.n % 2 == 0; }                                    \
    static void step(const StepArgs& a, cudaStream_t s) {                                                     \
      if constexpr (kPairForm) {                                                                              \
        if (paired(a.g)) {                                                                                    \
          const Launch3 lp = launch_pairs(a.g, 128, TX_PAIR_PER_THREAD), l = launch_pairs(a.g, 128);         \
          k_step_pair<D, S, ISO, MRT, T><<<lp.grid, lp.block, 0, s>>>(a);                                     \
          if (a.rest != 0) k_step_rest<D, S, ISO, MRT, T><<<l.grid, l.block, 0, s>>>(a);                      \
          return;                                                                                             \
        }                                                                                                     \
      }                                                                                                       \
      k_step<D, S, ISO, MRT, EXACT, T, R, RT><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a);                        \
    }                                                                                                         \
    static void count_rest(const StepArgs& a, unsigned* count, cudaStream_t s) {                              \
      if constexpr (kPairForm) {                                                                              \
        const Launch3 l = launch_pairs(a.g, 256);                                                             \
        if (paired(a.g)) k_count_rest<D, ISO><<<l.grid, l.block, 0, s>>>(a, count);                           \
      }                                                                                                       \
    }                                                                                                         \
    static void density(const StepArgs& a, int mode, cudaStream_t s) {                                        \
      constexpr int VW = 16 / (int)sizeof(T);                                                                 \
      if (a.g.n % VW == 0)                                                                                    \
        k_density_vec<D, S, T, R, RT><<<grid_for(a.g.n / VW, 256), 256, 0, s>>>(a, mode);                     \
      else                                                                                                    \
        k_density<D, S, T, R, RT><<<launch3(a.g, 256).grid, launch3(a.g, 256).block, 0, s>>>(a, mode);        \
    }                                                                                                         \
    static void init(const StepArgs& a, const double* u, cudaStream_t s) {                                    \
      k_init<D, S, ISO, EXACT, T, R, RT><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a, u);                          \
    }                                                                                                         \
    static void moments(const StepArgs& a, int what, double* out, cudaStream_t s) {                           \
      k_moments<D, S, ISO, EXACT, T, R, RT><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a, what, out);               \
    }                                                                                                         \
    static void to_nat(const void* f, const uint8_t* m, long long N, Shift sh, double* o, cudaStream_t s) {   \
      k_pops_to_natural<D, S, T, R><<<grid_for(N, kNatTile), 256, 0, s>>>(reinterpret_cast<const T*>(f), m, N, sh, o); \
    }                                                                                                         \
    static void from_nat(const double* i, const uint8_t* m, long long N, Shift sh, void* f, cudaStream_t s) { \
      k_pops_from_natural<D, S, T, R><<<grid_for(N, kNatTile), 256, 0, s>>>(i, m, N, sh, reinterpret_cast<T*>(f)); \
    }                                                                                                         \
    static void step_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {                \
      if constexpr (!EXACT) k_step_tiles<D, S, ISO, MRT, T, R, RT><<<grid, blk, 0, s>>>(b, flip);             \
      if constexpr (kPairForm) {                                                                              \
        k_step_pair_tiles<D, S, ISO, MRT, T><<<grid, blk, 0, s>>>(b, flip);                                   \
        k_step_rest_tiles<D, S, ISO, MRT, T><<<grid, blk, 0, s>>>(b, flip);                                   \
      }                                                                                                       \
    }                                                                                                         \
    static void density_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {             \
      if constexpr (!EXACT) k_density_tiles<D, S, T, R, RT><<<grid, blk, 0, s>>>(b, flip);                    \
    }                                                                                                         \
    static void probe_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {               \
      if constexpr (!EXACT) k_probe_tiles<D, S, ISO, T, R, RT><<<grid, blk, 0, s>>>(b, flip);                 \
    }                                                                                                         \
    static void faces(const StepArgs& a, const FaceShell& sh, cudaStream_t s) {                               \
      const long long n = sh.start[sh.nf];                                                                    \
      if (n > 0) k_faces<D, S, ISO, EXACT, T, R, RT><<<grid_for(n, 128), 128, 0, s>>>(a, sh);                 \
    }                                                                                                         \
    static void outlet(const StepArgs& a, int f, double* v, double p, double c0, double g21, cudaStream_t s) { \
      const long long n = face_area_of(D, a.g.nx, a.g.ny, a.g.nz, f);                                         \
      k_outlet<D, S, T, R, RT><<<grid_for(n, 128), 128, 0, s>>>(a, f, v, p, c0, g21);                         \
    }                                                                                                         \
    static void faces_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {               \
      if constexpr (!EXACT) k_faces_tiles<D, S, ISO, T, R, RT><<<grid, blk, 0, s>>>(b, flip);                 \
    }                                                                                                         \
    static void outlet_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {              \
      if constexpr (!EXACT) k_outlet_tiles<D, S, T, R, RT><<<grid, blk, 0, s>>>(b, flip);                     \
    }                                                                                                         \
  };

#define TX_FORM_CASE(S, ISO, MRT) TX_FORM_CASE_(S, ISO, MRT)
#define TX_FORM_CASE_(S, ISO, MRT)                                                                               \
  if (s == S && iso == ISO && mrt == MRT) {                                                                    \
    *ks = KernelSet{&L_##S##_##ISO##_##MRT::step,   &L_##S##_##ISO##_##MRT::density,                           \
                    &L_##S##_##ISO##_##MRT::init,   &L_##S##_##ISO##_##MRT::moments,                           \
                    &L_##S##_##ISO##_##MRT::to_nat, &L_##S##_##ISO##_##MRT::from_nat,                          \
                    &L_##S##_##ISO##_##MRT::step_tiles, &L_##S##_##ISO##_##MRT::density_tiles,                 \
                    &L_##S##_##ISO##_##MRT::probe_tiles, &L_##S##_##ISO##_##MRT::faces,                        \
                    &L_##S##_##ISO##_##MRT::outlet, &L_##S##_##ISO##_##MRT::faces_tiles,                          \
                    &L_##S##_##ISO##_##MRT::outlet_tiles,                                                         \
                    &L_##S##_##ISO##_##MRT::paired, &L_##S##_##ISO##_##MRT::count_rest,                          \
                    MRT ? #S "c iso" #ISO " rates:any" : #S "c iso" #ISO " rates:bgk/s_nu"};                    \
    return true;                                                                                               \
  }
