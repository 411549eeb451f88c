// Kernel table: D2, 1 component(s), reference operation order (built with --fmad=false), storage double, arithmetic double.
#define TX_D 2
#define TX_S 1
#define TX_EXACT true
#define TX_T double
#define TX_R double
#define TX_RT double
#define TX_FN kernels_d2_exact_s1
#define TX_SPECIES_FN species_d2_exact
#include "tx_inst.cuh"
