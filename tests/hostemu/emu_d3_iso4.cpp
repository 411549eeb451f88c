// D3Q19 FP64 combinations of the host emulation, isotropy 4 (exact and fast forms).
#include "emu.h"

namespace emu {
bool dispatch_d3_iso4(const Case& c, Result& out, std::string* err) {
  if (c.p.discretization != TX_D3Q19) return false;
  EMU_TRY(3, 1, 4, false, true, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 1, 4, false, false, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 1, 4, true, true, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 1, 4, true, false, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 2, 4, false, true, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 2, 4, false, false, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 2, 4, true, true, TX_PREC_F64, double, double, double)
  EMU_TRY(3, 2, 4, true, false, TX_PREC_F64, double, double, double)
  return false;
}
}  // namespace emu
