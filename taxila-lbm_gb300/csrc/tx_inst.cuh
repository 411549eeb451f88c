// Body of one tx_inst_*.cu translation unit: the kernel table of one
// (dimension, exactness, storage) combination for one component count, isotropy order and relaxation mode.  The including file defines
// TX_D, TX_S, TX_EXACT, TX_T, TX_R, TX_RT and TX_FN before including this.
#include "tx_dispatch.h"

namespace tx {
namespace {
#define TX_L(ISO, MRT) TX_FORM_LAUNCHERS(TX_D, TX_S, ISO, MRT, TX_EXACT, TX_T, TX_R, TX_RT)
TX_L(4, false)
TX_L(4, true)
TX_L(8, false)
TX_L(8, true)
#if TX_D == 2
TX_L(10, false)
TX_L(10, true)
#endif
#undef TX_L
}  // namespace

#ifdef TX_SPECIES_FN
namespace {
template <bool MRT>
struct SpeciesLaunch {
  static void step(const SpeciesArgs& a, cudaStream_t s) {
    k_species<TX_D, MRT, TX_EXACT, TX_T, TX_R><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a);
  }
  static void init(const SpeciesArgs& a, const double* conc, const double* flux, cudaStream_t s) {
    k_species_init<TX_D, TX_T, TX_R><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a, conc, flux);
  }
  static void fields(const SpeciesArgs& a, int what, double* out, cudaStream_t s) {
    k_species_fields<TX_D, TX_T, TX_R><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a, what, out);
  }
  static void step_tiles(const BatchArgs& b, int flip, int grid, dim3 blk, cudaStream_t s) {
    if constexpr (!TX_EXACT) k_species_tiles<TX_D, MRT, TX_T, TX_R><<<grid, blk, 0, s>>>(b, flip);
  }
  static void wall_collide(const SpeciesArgs& a, cudaStream_t s) {
    k_species_wall_collide<TX_D, MRT, TX_T, TX_R><<<launch3(a.g, 128).grid, launch3(a.g, 128).block, 0, s>>>(a);
  }
};
}  // namespace

bool TX_SPECIES_FN(bool mrt, SpeciesSet* ss) {
  if (mrt)
    *ss = SpeciesSet{&SpeciesLaunch<true>::step, &SpeciesLaunch<true>::init, &SpeciesLaunch<true>::fields,
                     &SpeciesLaunch<true>::step_tiles, &SpeciesLaunch<true>::wall_collide};
  else
    *ss = SpeciesSet{&SpeciesLaunch<false>::step, &SpeciesLaunch<false>::init, &SpeciesLaunch<false>::fields,
                     &SpeciesLaunch<false>::step_tiles, &SpeciesLaunch<false>::wall_collide};
  return true;
}
#endif

bool TX_FN(int s, int iso, bool mrt, KernelSet* ks) {
  TX_FORM_CASE(TX_S, 4, false)
  TX_FORM_CASE(TX_S, 4, true)
  TX_FORM_CASE(TX_S, 8, false)
  TX_FORM_CASE(TX_S, 8, true)
#if TX_D == 2
  TX_FORM_CASE(TX_S, 10, false)
  TX_FORM_CASE(TX_S, 10, true)
#endif
  return false;
}

}  // namespace tx
