// FP32 instantiations of the FFT and convolution passes of fft_impl.cuh.
#include "fft_impl.cuh"

namespace mlc {

template void forward_impl<float>(mlc_ctx*, const FftPlan2D&, const void*, int, void*);
template void conv_fused_impl<float>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*, void*, int);
template bool profile_spectrum_supported_impl<float>(const FftPlan2D&);
template void profile_spectrum_impl<float>(mlc_ctx*, const FftPlan2D&, const double*, int, void*);
template void conv_cached_impl<float>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);
template void conv_cached_real_impl<float>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);
template void conv_plain_impl<float>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*);
template bool c2r_interleave_impl<float, float>(mlc_ctx*, const FftPlan2D&, const void*, long, int, int, void*, unsigned);

}  // namespace mlc
