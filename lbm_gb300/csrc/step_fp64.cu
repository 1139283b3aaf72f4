// Kernel instantiations for fp64 population storage (D3Q15, D3Q19, D3Q27). Compiled with
// -fmad=false: no multiply-add is fused, so every FP64 operation rounds exactly where the
// reference's does.
#define LBMG_STORE double
#define LBMG_OPS_NAME ops_fp64
#include "ops_impl.cuh"
