// Float-float fused convolution (P0-P3) of fft_impl.cuh.
#include "fft_impl.cuh"

namespace mlc {

template void conv_fused_impl<ff>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*, void*, int);

}  // namespace mlc
