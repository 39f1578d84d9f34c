// Compile-time pass kernels, FP32.
#include "fit_ct_impl.cuh"

namespace fit {
template int ct_strided<float>(const float2*, float2*, int, long, long, bool, float, const float2*, cudaStream_t);
template int ct_c2r<float>(const float2*, float*, int, long, float, const float2*, cudaStream_t);
template int ct_r2c<float>(const float*, float2*, int, long, float, const float2*, cudaStream_t);
template int ct_z_full<float>(const float2*, float2*, int, int, int, int, long, const float2*, cudaStream_t);
}  // namespace fit
