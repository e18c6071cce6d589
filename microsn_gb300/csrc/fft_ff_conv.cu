// Float-float fused convolution (P0-P3) of fft_impl.cuh.
#include "fft_impl.cuh"

namespace mlc {

template void conv_fused_impl<ff>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*, void*, int);
template bool profile_spectrum_supported_impl<ff>(const FftPlan2D&);
template void profile_spectrum_impl<ff>(mlc_ctx*, const FftPlan2D&, const double*, int, void*);
template void conv_cached_impl<ff>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);
template void conv_cached_real_impl<ff>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);

}  // namespace mlc
