// kernels_inst.cu -- one instantiation of the hot-path kernels, selected at compile time:
// PLENS_P = N+1 and PLENS_REAL = double (plain form) or float (mixed form: flux differencing,
// surface fluxes and residual accumulation in FP32; state, metric terms, RK registers, the blend
// and the update in FP64). The build compiles this file once per (P, precision) in parallel.
#include "launch.cuh"

#if !defined(PLENS_P) || !defined(PLENS_REAL) || !defined(PLENS_TABLE)
#error "compile with -DPLENS_P=<N+1> -DPLENS_REAL=<double|float> -DPLENS_TABLE=<function name>"
#endif

namespace plens_gpu {

LaunchTable PLENS_TABLE() { return Launch<PLENS_P, PLENS_REAL>::table(); }

}  // namespace plens_gpu
