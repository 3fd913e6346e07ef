// fft_reg.cu — FP64 and FP32 instantiations of the register engine
// (fft_reg.cuh) and the list of lengths it covers.
#include "fft_reg.cuh"

namespace he4g {

bool fft_reg_supported(int n) {
  switch (n) {
#define HE4G_CASE(N, P, Q) case N:
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
    return true;
  }
  return false;
}

template bool reg_c2r_corr<double>(const Grid&, const FftPlan&, const double2*, double2*, double*, const double*,
                                   double, double, cudaStream_t, bool);
template bool reg_c2r_corr<float>(const Grid&, const FftPlan&, const float2*, float2*, float*, const float*, float,
                                  float, cudaStream_t, bool);
template bool reg_y<double>(const Grid&, const FftPlan&, void* const*, int, int, cudaStream_t, bool);
template bool reg_y<float>(const Grid&, const FftPlan&, void* const*, int, int, cudaStream_t, bool);
template bool reg_z<double>(const Grid&, const FftPlan&, const void*, void* const*, const void* const*, int, double,
                            const void*, const ZExtra&, cudaStream_t, bool);
template bool reg_z<float>(const Grid&, const FftPlan&, const void*, void* const*, const void* const*, int, double,
                           const void*, const ZExtra&, cudaStream_t, bool);
template bool reg_r2c<double>(const Grid&, const FftPlan&, const double2*, int, const double*, const double*, double,
                              double, double2*, cudaStream_t, bool);
template bool reg_r2c<float>(const Grid&, const FftPlan&, const float2*, int, const float*, const float*, float,
                             float, float2*, cudaStream_t, bool);
template bool reg_c2r<double>(const Grid&, const FftPlan&, const double2*, int, const double2*, const double2*,
                              double*, double*, int, const Pot4Args<double>&, cudaStream_t, bool);
template bool reg_c2r<float>(const Grid&, const FftPlan&, const float2*, int, const float2*, const float2*, float*,
                             float*, int, const Pot4Args<float>&, cudaStream_t, bool);

}  // namespace he4g
