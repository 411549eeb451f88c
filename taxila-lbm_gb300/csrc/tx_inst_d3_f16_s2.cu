// Kernel table: D3, 2 component(s), fast arithmetic, storage __half, arithmetic float.
#define TX_D 3
#define TX_S 2
#define TX_EXACT false
#define TX_T __half
#define TX_R float
#define TX_RT float
#define TX_FN kernels_d3_f16_s2
#include "tx_inst.cuh"
