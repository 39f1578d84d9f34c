// Compile-time pass kernels, FP64.
#include "fit_ct_impl.cuh"

namespace fit {
template int ct_strided<double>(const double2*, double2*, int, long, long, bool, double, const double2*,
                                cudaStream_t);
template int ct_c2r<double>(const double2*, double*, int, long, double, const double2*, cudaStream_t);
template int ct_r2c<double>(const double*, double2*, int, long, double, const double2*, cudaStream_t);
template int ct_z_full<double>(const double2*, double2*, int, int, int, int, long, const double2*, cudaStream_t);
}  // namespace fit
