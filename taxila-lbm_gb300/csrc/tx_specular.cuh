// Specular ("no-stick") walls, wall codes 900/901/902 (WALL_NORMAL_X/Y/Z).
//
// DistributionBouncebackD3/D2 (src/lbm/lbm_distribution_function.F90:668-784)
// walks the fi-ghosted box in k-j-i order.  An ordinary wall cell W sends each
// population it received, f(n, W), back to W - c_n as opp(n); a specular wall
// normal to axis a sends it to W - c_n,a e_a as reflect_a(n) (only the a
// component of c flips), checking only that coordinate against the owned
// range.  Every wall cell is cleared after its own turn, but a later specular
// wall may write into an earlier wall cell, so wall cells can end a step
// holding populations.  The stream carries those into the neighbours on the
// next step, and a wall cell read later in the sweep passes on what earlier
// walls wrote into it.
//
// The walls never change between uploads, so where each population slot's
// final value comes from is a property of the geometry alone.  The host
// resolves it once per wall upload (specular_routes): for slot (m, T), the
// last event of the sweep that touches it (the write of a wall, or T's own
// clearing) decides its value; a wall's write is the content of the slot it
// reads at its own turn, which is resolved the same way at that earlier time.
// The chain ends at a cleared slot (zero) or at the value the stream brought
// in, i.e. a post-collision population P(n', X').  Most slots resolve to what
// the ordinary push-with-bounceback kernels already write; the others form a
// short list of exceptions, which two small kernels apply after the step
// kernel and before the density pass: k_spec_gather reads every exception's
// source (a pore cell's P sits where the step kernel pushed it; a wall cell's
// content sits in the previous state buffer), then k_spec_scatter writes them,
// so no exception reads a slot another one overwrites.
//
// Passive species stream and bounce back through the same sweep with a list
// of their own: the transport applies no boundary condition (LBMRun2,
// src/lbm/lbm.F90:348-352), so their chains never end at a face's BCPreStream
// copy.  In 2D the transport also collides the wall cells toward a zero
// equilibrium (TransportCollisionD2, src/lbm/lbm_transport.F90:433-458);
// under MRT that mixes a wall cell's slots, and their list then keeps every
// slot of a wall cell that can hold content (cell_mix).
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "tx_kernels.cuh"

namespace tx {

// Wall code of a specular wall: the axis it is normal to, else -1.  In 2D the
// reference knows WALL_NORMAL_X and _Y only; 902 is an ordinary wall there.
__host__ __device__ inline int specular_axis(double v, int D) {
  if (v == 900.0) return 0;
  if (v == 901.0) return 1;
  if (v == 902.0 && D == 3) return 2;
  return -1;
}

// Exceptions to the ordinary push: dst[e] = slot n * N + cell that receives
// another value; src[e] = -1 for zero, else (slot << 1) | 1 for a slot of the
// previous state (a wall cell's content) or (slot << 1) for a slot of the
// state the step kernel just wrote (where it pushed a pore cell's P).
struct SpecRoutes {
  std::vector<long long> dst, src;
};
// an exception list on the device
struct SpecList {
  long long n = 0;
  long long* dst = nullptr;
  long long* src = nullptr;
};

// Resolves every owned slot (see the file comment).  walls: the reference's
// wall values in natural order (x fastest); n: lattice sides (n[2] = 1 in 2D);
// per: periodic axes; prestream: faces XM..ZP whose boundary condition copies
// populations into the ghost layer before the stream (BCPreStream,
// lbm_bc.F90:613-779); init_nz: sorted slots (n * N + cell) of wall cells
// whose initial content is not zero (uploaded populations), or null;
// cell_mix: wall cells are collided, and a collision that mixes their slots
// (the 2D species' MRT toward a zero equilibrium) makes every slot of a wall
// cell live once one of them is.  Returns
// "" or the reason the geometry is refused (a slot whose value would come
// from outside what the reference defines).
//
// A wall slot whose chain ends at another wall cell's content keeps that
// content one step later.  Wall slots that no chain of such moves connects to
// a pore cell's P (or to non-zero initial content) stay zero for ever, as
// they do with ordinary walls alone; their exceptions are dropped, so the
// list stays proportional to the specular walls' neighbourhood.
inline std::string specular_routes(const double* walls, int D, const int n[3], const int per[3], const bool prestream[6],
                                   const std::vector<long long>* init_nz, bool cell_mix, SpecRoutes* out) {
  const int Q = D == 3 ? 19 : 9;
  int c[19][3], opp[19], refl[3][19];
  for (int q = 0; q < Q; ++q)
    for (int a = 0; a < 3; ++a) c[q][a] = D == 3 ? Lat<3>::c(q, a) : Lat<2>::c(q, a);
  for (int q = 0; q < Q; ++q)
    for (int r = 0; r < Q; ++r) {
      if (c[r][0] == -c[q][0] && c[r][1] == -c[q][1] && c[r][2] == -c[q][2]) opp[q] = r;
      for (int a = 0; a < 3; ++a) {
        bool ok = true;
        for (int b = 0; b < 3; ++b) ok = ok && c[r][b] == (b == a ? -c[q][b] : c[q][b]);
        if (ok) refl[a][q] = r;
      }
    }
  // the fi-ghosted box: one ghost layer on each axis of the lattice
  int lo[3], len[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = a < D ? 0 : 1;
    len[a] = a < D ? n[a] + 2 : 1;
  }
  const long long N = (long long)n[0] * n[1] * n[2];
  auto owned = [&](const int x[3]) {
    return x[0] >= 1 && x[0] <= n[0] && x[1] >= 1 && x[1] <= n[1] && x[2] >= 1 && x[2] <= n[2];
  };
  auto pos = [&](const int x[3]) {
    return ((long long)(x[2] - lo[2]) * len[1] + (x[1] - lo[1])) * len[0] + (x[0] - lo[0]);
  };
  // the owned cell a ghost cell copies (all out-of-range axes periodic), else false
  auto wrap = [&](const int x[3], int w[3]) {
    for (int a = 0; a < 3; ++a) {
      w[a] = x[a];
      if (x[a] >= 1 && x[a] <= n[a]) continue;
      if (!per[a]) return false;
      w[a] = ((x[a] - 1) % n[a] + n[a]) % n[a] + 1;
    }
    return true;
  };
  auto cell = [&](const int x[3]) { return (long long)(x[0] - 1) + (long long)n[0] * ((x[1] - 1) + (long long)n[1] * (x[2] - 1)); };
  // WallsSetGhostNodes: ghost cells past a non-periodic face are walls (999)
  auto code = [&](const int x[3]) {
    int w[3];
    return wrap(x, w) ? walls[cell(w)] : 999.0;
  };
  out->dst.clear();
  out->src.clear();
  const long long kInf = 1LL << 62;
  // One z-layer of owned slots (the chains only read the walls, so layers are
  // independent); the error of a refused geometry, else null.
  auto layer = [&](int z, std::vector<long long>& ldst, std::vector<long long>& lsrc) -> const char* {
    for (int y = 1; y <= n[1]; ++y)
      for (int x = 1; x <= n[0]; ++x) {
        const int T0[3] = {x, y, z};
        const double vt = code(T0);
        for (int m = 0; m < Q; ++m) {
          // resolve the final value of slot (m, T0)
          int cm = m, X[3] = {x, y, z};
          long long t = kInf;
          bool zero = false, done = false;
          int sn = -1, S[3] = {0, 0, 0};
          for (int hop = 0; hop < 64 && !done; ++hop) {
            long long best = -1;
            int kind = 0, rn = -1, R[3] = {0, 0, 0};
            const double vx = code(X);
            if (vx > 0.0 && pos(X) < t) {  // the slot's own clearing
              best = pos(X);
              kind = 1;
            }
            if (owned(X)) {  // an ordinary wall at X - c_m sends back opp(m)
              int W[3];
              for (int a = 0; a < 3; ++a) W[a] = X[a] - c[cm][a];
              const double vw = code(W);
              const long long pw = pos(W);
              if (vw > 0.0 && specular_axis(vw, D) < 0 && pw < t && pw > best) {
                best = pw;
                kind = 2;
                rn = opp[cm];
                for (int a = 0; a < 3; ++a) R[a] = W[a];
              }
            }
            for (int a = 0; a < D; ++a) {  // a specular wall at X - c_m,a e_a sends reflect_a(m)
              if (c[cm][a] == 0 || X[a] < 1 || X[a] > n[a]) continue;
              int W[3] = {X[0], X[1], X[2]};
              W[a] -= c[cm][a];
              const long long pw = pos(W);
              if (specular_axis(code(W), D) == a && pw < t && pw > best) {
                best = pw;
                kind = 2;
                rn = refl[a][cm];
                for (int b = 0; b < 3; ++b) R[b] = W[b];
              }
            }
            if (kind == 1) {
              zero = true;
              done = true;
            } else if (kind == 2) {
              cm = rn;
              for (int a = 0; a < 3; ++a) X[a] = R[a];
              t = best;
            } else {
              // no event: the value the stream brought in from X - c_m (a ghost
              // source holds the periodic image's post-collision value)
              for (int a = 0; a < 3; ++a) {
                const int cc = c[cm][a];
                const int lo_a = 1 + (cc < 0 ? cc : 0), hi_a = n[a] + (cc > 0 ? cc : 0);
                if (X[a] < lo_a || X[a] > hi_a) return "specular walls: a population would come from a ghost slot the stream does not write";
              }
              int Sx[3];
              for (int a = 0; a < 3; ++a) Sx[a] = X[a] - c[cm][a];
              done = true;
              if (wrap(Sx, S)) {
                sn = cm;
              } else {
                // a ghost cell past a non-periodic face: cleared by the last
                // bounceback (a 999 wall), unless a face's BCPreStream copied
                // P(m, X) of a face cell X into it (the last such face wins)
                zero = true;
                if (owned(X))
                  for (int f = 0; f < 2 * D; ++f) {
                    const int a = f / 2;
                    const bool minus = f % 2 == 0;
                    if (!prestream[f] || X[a] != (minus ? 1 : n[a]) || !(minus ? c[cm][a] > 0 : c[cm][a] < 0)) continue;
                    zero = false;
                    sn = cm;
                    for (int b = 0; b < 3; ++b) S[b] = X[b];
                  }
              }
            }
          }
          if (!done) return "specular walls: a chain of wall-to-wall moves did not end";
          // what the ordinary push writes into (m, T0): nothing into a wall cell
          // (it stays zero); P(m, T0 - c_m) from a pore neighbour; else T0's own
          // opp(m) bounced back
          bool std_zero = false;
          int stdn = -1, stdX[3] = {x, y, z};
          if (vt != 0.0) {
            std_zero = true;
          } else {
            int Y[3], Yw[3];
            for (int a = 0; a < 3; ++a) Y[a] = T0[a] - c[m][a];
            if (wrap(Y, Yw) && walls[cell(Yw)] == 0.0) {
              stdn = m;
              for (int a = 0; a < 3; ++a) stdX[a] = Yw[a];
            } else {
              stdn = opp[m];
            }
          }
          // (with cell_mix a wall cell's zero slots are listed too: its
          // collision may have written them in place)
          if (zero && std_zero && !cell_mix) continue;
          if (!zero && !std_zero && sn == stdn && S[0] == stdX[0] && S[1] == stdX[1] && S[2] == stdX[2]) continue;
          ldst.push_back((long long)m * N + cell(T0));
          if (zero) {
            lsrc.push_back(-1);
          } else if (walls[cell(S)] != 0.0) {
            lsrc.push_back((((long long)sn * N + cell(S)) << 1) | 1);  // a wall cell's content
          } else {
            // where the step kernel pushed P(sn, S): to S + c_sn when that is pore, else back into S as opp(sn)
            int Y[3], Yw[3];
            for (int a = 0; a < 3; ++a) Y[a] = S[a] + c[sn][a];
            long long slot;
            if (wrap(Y, Yw) && walls[cell(Yw)] == 0.0)
              slot = (long long)sn * N + cell(Yw);
            else
              slot = (long long)opp[sn] * N + cell(S);
            lsrc.push_back(slot << 1);
          }
        }
      }
    return nullptr;
  };
  // The layers run on host threads; their lists are joined in layer order,
  // the order one thread would produce.
  const int nz = n[2];
  const unsigned hw = std::thread::hardware_concurrency();
  const int nt = (int)std::max(1u, std::min(hw ? hw : 1u, (unsigned)std::min(nz, 32)));
  std::vector<std::vector<long long>> ld((size_t)nz), ls((size_t)nz);
  std::vector<const char*> err((size_t)nz, nullptr);
  std::atomic<int> next{0};
  auto run_layers = [&]() {
    for (int z = next.fetch_add(1); z < nz; z = next.fetch_add(1)) err[(size_t)z] = layer(z + 1, ld[(size_t)z], ls[(size_t)z]);
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nt; ++i) pool.emplace_back(run_layers);
  run_layers();
  for (std::thread& t : pool) t.join();
  for (int z = 0; z < nz; ++z)
    if (err[(size_t)z]) return err[(size_t)z];
  for (int z = 0; z < nz; ++z) {
    out->dst.insert(out->dst.end(), ld[(size_t)z].begin(), ld[(size_t)z].end());
    out->src.insert(out->src.end(), ls[(size_t)z].begin(), ls[(size_t)z].end());
  }
  // Keep the exceptions into pore cells, and those into wall slots that a chain
  // of wall-content moves links to a pore cell's P or to non-zero initial content.
  const size_t E = out->dst.size();
  auto is_wall_slot = [&](long long slot) { return walls[slot % N] != 0.0; };
  std::vector<std::pair<long long, size_t>> readers;  // (wall slot read from the previous state, exception)
  std::vector<char> live(E, 0);
  std::vector<size_t> work;
  for (size_t e = 0; e < E; ++e) {
    const long long s = out->src[e];
    if (!is_wall_slot(out->dst[e])) {
      live[e] = 1;
    } else if (s >= 0 && !(s & 1)) {
      live[e] = 1;
      work.push_back(e);
    }
    if (s >= 0 && (s & 1) && is_wall_slot(out->dst[e])) readers.emplace_back(s >> 1, e);
  }
  std::sort(readers.begin(), readers.end());
  auto wake_slot = [&](long long slot) {
    auto it = std::lower_bound(readers.begin(), readers.end(), std::make_pair(slot, (size_t)0));
    for (; it != readers.end() && it->first == slot; ++it)
      if (!live[it->second]) {
        live[it->second] = 1;
        work.push_back(it->second);
      }
  };
  // cell_mix: liveness per wall cell; a live cell keeps the exceptions read
  // from any of its slots and those into all of its slots (the zero ones too)
  std::vector<std::pair<long long, size_t>> writers;  // (wall cell written, exception)
  std::vector<char> cell_live;
  if (cell_mix) {
    cell_live.assign((size_t)N, 0);
    for (size_t e = 0; e < E; ++e)
      if (is_wall_slot(out->dst[e])) writers.emplace_back(out->dst[e] % N, e);
    std::sort(writers.begin(), writers.end());
  }
  auto wake = [&](long long slot) {
    if (!cell_mix) return wake_slot(slot);
    const long long cell = slot % N;
    if (cell_live[(size_t)cell]) return;
    cell_live[(size_t)cell] = 1;
    for (int q = 0; q < Q; ++q) wake_slot((long long)q * N + cell);
    auto it = std::lower_bound(writers.begin(), writers.end(), std::make_pair(cell, (size_t)0));
    for (; it != writers.end() && it->first == cell; ++it) live[it->second] = 1;
  };
  if (init_nz)
    for (long long s : *init_nz) wake(s);
  while (!work.empty()) {
    const size_t e = work.back();
    work.pop_back();
    wake(out->dst[e]);
  }
  size_t k = 0;
  for (size_t e = 0; e < E; ++e)
    if (live[e]) {
      out->dst[k] = out->dst[e];
      out->src[k] = out->src[e];
      ++k;
    }
  out->dst.resize(k);
  out->src.resize(k);
  return "";
}

// The stored value of an empty population slot (f = 0): its deviation
// (0 - w_n rho0_m) times the storage scale in the FP32/FP16 forms, zero in the
// FP64 form (and for species, whose storage has no rest state: sh.rho0 = 0).
template <int D, class T>
__host__ __device__ inline T empty_slot(int m, int n, const Shift& sh) {
  if constexpr (std::is_same<T, double>::value) {
    return 0.0;
  } else {
    const double x = (0.0 - Lat<D>::w(n) * sh.rho0[m]) * sh.scale;
    if constexpr (std::is_same<T, float>::value)
      return (float)x;
    else
      return __float2half_rn((float)x);
  }
}

// Every exception's source value, per component (pops: [(m * Q + n) * N + cell]):
// a copy of the stored value (a slot of the same speed |c|, so of the same
// weight and rest-state offset), or the empty value of the destination slot.
template <int D, class T>
__global__ void __launch_bounds__(256) k_spec_gather(const T* fin, const T* fout, const long long* src,
                                                     const long long* dst, long long ne, int S, long long N, Shift sh,
                                                     T* tmp) {
  constexpr int Q = Lat<D>::Q;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const long long s = src[e];
  for (int m = 0; m < S; ++m) {
    T v;
    if (s >= 0)
      v = ((s & 1) ? fin : fout)[(long long)m * Q * N + (s >> 1)];
    else
      v = empty_slot<D, T>(m, (int)(dst[e] / N), sh);
    tmp[e * S + m] = v;
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_spec_scatter(T* fout, const long long* dst, long long ne, int S, long long QN,
                                                      const T* tmp) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int m = 0; m < S; ++m) fout[(long long)m * QN + dst[e]] = tmp[e * S + m];
}

// Empties every wall cell's slots (after an upload or init, before the state
// buffers have both been written by a step with the routes above).
template <int D, class T>
__global__ void __launch_bounds__(256) k_spec_clear_walls(T* f, const uint8_t* mask, long long N, int S, Shift sh) {
  constexpr int Q = Lat<D>::Q;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || mask[i] == 0) return;
  for (int m = 0; m < S; ++m)
    for (int n = 0; n < Q; ++n) f[(long long)(m * Q + n) * N + i] = empty_slot<D, T>(m, n, sh);
}

}  // namespace tx
