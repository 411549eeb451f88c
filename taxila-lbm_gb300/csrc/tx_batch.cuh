// Batched flow step: many independent lattices advanced by one persistent
// launch per kernel.
//
// The lattices of a batch share one kernel form (dimension, components,
// isotropy, relaxation, storage) but each has its own size, walls, physical
// parameters and boundary faces.  A tile table lists (lattice, tile origin)
// for every tile of every active lattice; a tile is one thread block
// (bx, by, bz).  A fixed grid of persistent blocks walks the table, so the
// launch configuration never changes when lattices join or leave: the table
// and its length live in device memory, which is what lets the host capture
// the step loop once in a CUDA graph and keep replaying it while the table is
// rewritten between replays.
//
// Every site is updated by the same per-site functions as the single-lattice
// kernels (step_site, density_site), so a lattice's populations do not depend
// on the tile shape, on the other lattices or on the launch.
//
// All lattices of a batch step in lockstep.  flip selects the ping-pong
// buffer: at flip 0 a lattice's state is in LatDesc::a.fin, at flip 1 in
// LatDesc::a.fout.
#pragma once
#include "tx_kernels.cuh"
#include "tx_pair.cuh"
#include "tx_species.cuh"

namespace tx {

struct LatDesc {
  StepArgs a;         // fin: state buffer at flip 0; fout: the other buffer
  double* uold;       // velocity at the previous probe, [d * N + cell]
  int tile_begin;     // this lattice's tiles in the table
  int tile_count;
  int ltile_begin;    // its first tile of the density pass's linear table
  // exterior faces beyond Dirichlet ones: the face nodes of the face pass, and
  // the pressure of each two-component pressure outlet (c0, g21 of its update)
  FaceShell shell;
  double outlet_p[6];
  double c0, g21;
  // passive species: populations at flip 0 / the other buffer, parameters
  const void* sg0;
  void* sg1;
  const void* sphys;
  int ns;
};

// per-tile partial of a probe: velocity change and velocity statistics over pore sites
struct ProbePart {
  double du;          // max over sites and axes of |u - u_old|
  double umax;        // max over sites and axes of |u|
  double usum[3];     // sum of u per axis
  double npore;       // pore sites
  double mass[MAXC];  // sum of each component's density
};

struct BatchArgs {
  const LatDesc* lats;
  const int4* tiles;  // (lattice slot, x0, y0, z0)
  const int* ntiles;  // table length (device memory: may change between graph replays)
  ProbePart* parts;   // [tile]
  const int2* ltiles; // density pass: (lattice slot, first site) of runs of 128 x VW sites
  const int* nltiles;
  const int2* ftiles; // face pass: (lattice slot, first shell node) of runs of 128 face nodes
  const int* nftiles;
  const int4* otiles; // outlet refresh: (lattice slot, face, first node, 0) of runs of 128 nodes
  const int* notiles;
  // the step: per-site tiles of the lattices without the paired kernel; pair
  // tiles (lattice slot, first pair: kPairTileRuns runs of 128 pairs) of those with it, and
  // the pair tiles of the lattices that have pairs for the per-site kernel
  const int4* stiles;
  const int* nstiles;
  const int4* ptiles;
  const int* nptiles;
  const int4* rtiles;
  const int* nrtiles;
};

__device__ __forceinline__ StepArgs flipped(const StepArgs& s, int flip) {
  StepArgs a = s;
  if (flip) {
    a.fin = s.fout;
    a.fout = const_cast<void*>(s.fin);
  }
  return a;
}

template <int D, int S, int ISO, bool MRT, class T, class R, class RT>
__global__ void __launch_bounds__(128, TX_STEP_MIN_BLOCKS(S, R, MRT)) k_step_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.nstiles);
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.stiles + t);
    const StepArgs a = flipped(b.lats[tl.x].a, flip);
    const int x = tl.y + (int)threadIdx.x, y = tl.z + (int)threadIdx.y, z = tl.w + (int)threadIdx.z;
    if (x < a.g.nx && y < a.g.ny && z < a.g.nz) step_site<D, S, ISO, MRT, false, T, R, RT>(a, x, y, z);
  }
}

// The paired step of k_step_pair over the pair tiles: runs of
// kPairTileRuns x 128 pairs (lattice slot, first pair) of the lattices with an
// even site count; a thread takes one pair of each run of 128, so the
// lattice's arguments are read once per kPairTileRuns pairs.
constexpr int kPairTileRuns = 4;
template <int D, int S, int ISO, bool MRT, class T>
__global__ void __launch_bounds__(128, TX_PAIR_MIN_BLOCKS(S)) k_step_pair_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.nptiles);
  const int lane = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.ptiles + t);
    const StepArgs a = flipped(b.lats[tl.x].a, flip);
    const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
    for (int r = 0; r < kPairTileRuns; ++r) {
      const unsigned i = (unsigned)tl.y + (unsigned)(128 * r + lane);
      bool run = false, full = false;
      uint2 ll = make_uint2(0u, 0u);
      PairSites ps{};
      if ((long long)2 * i < a.g.n) {
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
}

// The per-site step of the pairs that k_step_pair_tiles leaves (k_step_rest).
template <int D, int S, int ISO, bool MRT, class T>
__global__ void __launch_bounds__(128, TX_STEP_MIN_BLOCKS(S, float, MRT)) k_step_rest_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.nrtiles);
  const int lane = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.rtiles + t);
    const StepArgs a = flipped(b.lats[tl.x].a, flip);
    const PhysT<float>& P = *reinterpret_cast<const PhysT<float>*>(a.phys);
    for (int r = 0; r < kPairTileRuns; ++r) {
      const unsigned i = (unsigned)tl.y + (unsigned)(128 * r + lane);
      if ((long long)2 * i < a.g.n) {
        const PairSites ps = pair_sites(a.g, i);
        const uint2 ll = __ldg(reinterpret_cast<const uint2*>(a.links) + (ps.c0 >> 1));
        if (pair_class<D, ISO>(a, P, ll.x, ll.y, ps) == 0) {
          step_site<D, S, ISO, MRT, false, T, float, float>(a, ps.x0, ps.y0, ps.z0);
          step_site<D, S, ISO, MRT, false, T, float, float>(a, ps.x1, ps.y1, ps.z1);
        }
      }
    }
  }
}

// after k_step_tiles at the same flip: the pushed populations are in a.fout.
// The density pass streams each lattice's sites in order: tiles of 128
// threads x VW consecutive sites, 16-byte loads where the site count allows.
template <int D, int S, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_density_tiles(BatchArgs b, int flip) {
  constexpr int VW = 16 / (int)sizeof(T);
  const int nt = __ldg(b.nltiles);
  const int lane = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int2 tl = __ldg(b.ltiles + t);
    const StepArgs a = flipped(b.lats[tl.x].a, flip);
    const long long N = a.g.n;
    const long long c0 = (long long)tl.y + (long long)lane * VW;
    if (c0 < N) {
      if (N % VW == 0)
        density_group<D, S, T, R, RT, true>(a, c0, 0);
      else
        density_group<D, S, T, R, RT, false>(a, c0, 0, (int)(N - c0 < VW ? N - c0 : VW));
    }
    // the lattice's step counter advances once per step (the step kernel of
    // this step has finished reading it; the next one reads the new value)
    if (t == b.lats[tl.x].ltile_begin && lane == 0 && a.steps_ptr) atomicAdd(const_cast<unsigned*>(a.steps_ptr), 1u);
  }
}

// Face pass after k_density_tiles at the same flip (lattices whose faces are
// not all of the Dirichlet class): face_site at each face node.
template <int D, int S, int ISO, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_faces_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.nftiles);
  const int lane = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int2 tl = __ldg(b.ftiles + t);
    const LatDesc& L = b.lats[tl.x];
    const StepArgs a = flipped(L.a, flip);
    int x, y, z;
    if (shell_site<D>(a.g, L.shell, (long long)tl.y + lane, x, y, z)) face_site<D, S, ISO, false, T, R, RT>(a, x, y, z);
  }
}

// Two-component pressure outlets, before k_step_tiles at the same flip.
template <int D, int S, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_outlet_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.notiles);
  const int lane = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.otiles + t);
    const LatDesc& L = b.lats[tl.x];
    const StepArgs a = flipped(L.a, flip);
    outlet_node<D, S, T, R, RT>(a, tl.y, const_cast<double*>(a.faces.vals[tl.y]), L.outlet_p[tl.y], L.c0, L.g21,
                                (long long)tl.z + lane);
  }
}

// species step of every lattice after the flow step at the same flip
template <int D, bool MRT, class T, class R>
__global__ void __launch_bounds__(128) k_species_tiles(BatchArgs b, int flip) {
  const int nt = __ldg(b.ntiles);
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.tiles + t);
    const LatDesc& L = b.lats[tl.x];
    SpeciesArgs a{};
    a.gin = flip ? L.sg1 : L.sg0;
    a.gout = flip ? const_cast<void*>(L.sg0) : L.sg1;
    a.links = L.a.links;
    a.mask = L.a.mask;
    a.phys = L.sphys;
    a.g = L.a.g;
    a.ns = L.ns;
    const int x = tl.y + (int)threadIdx.x, y = tl.z + (int)threadIdx.y, z = tl.w + (int)threadIdx.z;
    if (a.ns > 0 && x < a.g.nx && y < a.g.ny && z < a.g.nz) species_site<D, MRT, false, T, R>(a, x, y, z);
  }
}

// Velocity of every pore site (the common velocity of FlowUpdateUED3/D2,
// forces included) against the previous probe; one ProbePart per tile,
// reduced in a fixed order so that the result depends only on the lattice.
template <int D, int S, int ISO, class T, class R, class RT>
__global__ void __launch_bounds__(128) k_probe_tiles(BatchArgs b, int flip) {
  constexpr int NV = 6 + S;  // du, umax, usum x/y/z, npore, mass per component
  __shared__ double red[4][NV];
  const int nt = __ldg(b.ntiles);
  const int tid = (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z));
  const int lane = tid & 31, warp = tid >> 5;
  for (int t = blockIdx.x; t < nt; t += gridDim.x) {
    const int4 tl = __ldg(b.tiles + t);
    const LatDesc& L = b.lats[tl.x];
    const StepArgs a = flipped(L.a, flip);
    const int x = tl.y + (int)threadIdx.x, y = tl.z + (int)threadIdx.y, z = tl.w + (int)threadIdx.z;
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    if (x < a.g.nx && y < a.g.ny && z < a.g.nz) {
      const long long idx = (long long)x + (long long)a.g.nx * ((long long)y + (long long)a.g.ny * z);
      if (__ldg(a.mask + idx) == 0) {
        const PhysT<R>& P = *reinterpret_cast<const PhysT<R>*>(a.phys);
        R fv[S][Lat<D>::Q];
        load_pops<D, S, T, R>(reinterpret_cast<const T*>(a.fin), a.g.n, (unsigned)idx, P, fv);
        R rc[S], rf[S], F[S][D], up[D];
        cell_moments<D, S, ISO, false, R, RT>(a, P, x, y, z, idx, fv, rc, rf, F, up);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double u = double(up[d]);
          double* uo = L.uold + (long long)d * a.g.n + idx;
          v[0] = fmax(v[0], fabs(u - *uo));
          v[1] = fmax(v[1], fabs(u));
          v[2 + d] = u;
          *uo = u;
        }
        v[5] = 1.0;
#pragma unroll
        for (int m = 0; m < S; ++m) v[6 + m] = double(rc[m]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v[0] = fmax(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
      v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], o));
#pragma unroll
      for (int k = 2; k < NV; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    if (lane == 0)
      for (int k = 0; k < NV; ++k) red[warp][k] = v[k];
    __syncthreads();
    if (tid == 0) {
      ProbePart p{};
      p.du = fmax(fmax(red[0][0], red[1][0]), fmax(red[2][0], red[3][0]));
      p.umax = fmax(fmax(red[0][1], red[1][1]), fmax(red[2][1], red[3][1]));
      for (int d = 0; d < 3; ++d) p.usum[d] = ((red[0][2 + d] + red[1][2 + d]) + red[2][2 + d]) + red[3][2 + d];
      p.npore = ((red[0][5] + red[1][5]) + red[2][5]) + red[3][5];
      for (int m = 0; m < S; ++m) p.mass[m] = ((red[0][6 + m] + red[1][6 + m]) + red[2][6 + m]) + red[3][6 + m];
      b.parts[t] = p;
    }
    __syncthreads();
  }
}

}  // namespace tx
