// Kernel table: D3, 1 component(s), fast arithmetic, storage __half, arithmetic float.
#define TX_D 3
#define TX_S 1
#define TX_EXACT false
#define TX_T __half
#define TX_R float
#define TX_RT float
#define TX_FN kernels_d3_f16_s1
#define TX_SPECIES_FN species_d3_f16
#include "tx_inst.cuh"
