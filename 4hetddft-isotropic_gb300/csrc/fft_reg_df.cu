// fft_reg_df.cu — df64 instantiation of the register engine (fft_reg.cuh):
// the 3D FFT convolutions of HE4G_PREC_DF64 in paired-FP32 arithmetic on the
// df64 fields and spectra of that form. Its own translation unit, so that it
// compiles in parallel with the FP64/FP32 one.
#include "fft_reg.cuh"

namespace he4g {

template bool reg_c2r_corr<df64>(const Grid&, const FftPlan&, const df2*, df2*, df64*, const df64*, df64, df64,
                                 cudaStream_t, bool);
template bool reg_y<df64>(const Grid&, const FftPlan&, void* const*, int, int, cudaStream_t, bool);
template bool reg_z<df64>(const Grid&, const FftPlan&, const void*, void* const*, const void* const*, int, double,
                          const void*, const ZExtra&, cudaStream_t, bool);
template bool reg_r2c<df64>(const Grid&, const FftPlan&, const df2*, int, const df64*, const df64*, df64, df64,
                            df2*, cudaStream_t, bool);
template bool reg_c2r<df64>(const Grid&, const FftPlan&, const df2*, int, const df2*, const df2*, df64*, df64*,
                            int, const Pot4Args<df64>&, cudaStream_t, bool);

}  // namespace he4g
