// Reduced-precision forms of the host emulation: FP32 arithmetic with FP32
// or FP16 population storage.
#include "emu.h"

namespace emu {
bool dispatch_forms(const Case& c, Result& out, std::string* err) {
  if (c.p.discretization == TX_D3Q19) {
    EMU_TRY(3, 2, 4, true, false, TX_PREC_F32, float, float, float)
    EMU_TRY(3, 2, 4, true, false, TX_PREC_F32_F16, __half, float, float)
    EMU_TRY(3, 1, 4, false, false, TX_PREC_F32, float, float, float)
    EMU_TRY(3, 1, 4, false, false, TX_PREC_F32_F16, __half, float, float)
  } else {
    EMU_TRY(2, 2, 4, false, false, TX_PREC_F32, float, float, float)
  }
  return false;
}
}  // namespace emu
