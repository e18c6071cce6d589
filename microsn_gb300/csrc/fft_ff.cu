// Float-float forward transform and interleaving last pass of fft_impl.cuh (FP64 maps
// with mlc_map_set_fft(map, MLC_FFT_F32X2)); the fused convolution is in fft_ff_conv.cu,
// its own unit because its kernels take the longest to compile.  The plain convolution
// has no float-float form.
#include "fft_impl.cuh"

namespace mlc {

template void forward_impl<ff>(mlc_ctx*, const FftPlan2D&, const void*, int, void*);
template bool c2r_interleave_impl<ff, double>(mlc_ctx*, const FftPlan2D&, const void*, long, int, int, void*, unsigned);

}  // namespace mlc
