// Kernel instantiations for fp32 population storage (D3Q15, D3Q19, D3Q27).
#define LBMG_STORE float
#define LBMG_OPS_NAME ops_fp32
#include "ops_impl.cuh"
