// Kernel instantiations for fp16 population storage (D3Q15, D3Q19, D3Q27).
#define LBMG_STORE __half
#define LBMG_OPS_NAME ops_fp16
#include "ops_impl.cuh"
