// Kernel table: D2, 2 component(s), fast arithmetic, storage double, arithmetic double.
#define TX_D 2
#define TX_S 2
#define TX_EXACT false
#define TX_T double
#define TX_R double
#define TX_RT double
#define TX_FN kernels_d2_f64_s2
#include "tx_inst.cuh"
