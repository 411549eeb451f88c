// Kernel table: D2, 1 component(s), fast arithmetic, storage double, arithmetic double.
#define TX_D 2
#define TX_S 1
#define TX_EXACT false
#define TX_T double
#define TX_R double
#define TX_RT double
#define TX_FN kernels_d2_f64_s1
#define TX_SPECIES_FN species_d2_f64
#include "tx_inst.cuh"
