// Kernel instantiations for bf16 population storage (D3Q15, D3Q19, D3Q27).
#define LBMG_STORE __nv_bfloat16
#define LBMG_OPS_NAME ops_bf16
#include "ops_impl.cuh"
