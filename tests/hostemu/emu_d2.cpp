// D2Q9 FP64 combinations of the host emulation (exact and fast forms).
#include "emu.h"

namespace emu {
bool dispatch_d2(const Case& c, Result& out, std::string* err) {
  if (c.p.discretization != TX_D2Q9) return false;
  EMU_TRY(2, 1, 4, false, true, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 1, 4, false, false, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 4, false, true, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 4, false, false, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 8, true, true, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 8, true, false, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 10, true, true, TX_PREC_F64, double, double, double)
  EMU_TRY(2, 2, 10, true, false, TX_PREC_F64, double, double, double)
  return false;
}
}  // namespace emu
