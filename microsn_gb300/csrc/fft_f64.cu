// FP64 instantiations of the FFT and convolution passes of fft_impl.cuh.
#include "fft_impl.cuh"

namespace mlc {

template void forward_impl<double>(mlc_ctx*, const FftPlan2D&, const void*, int, void*);
template void conv_fused_impl<double>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*, void*, int);
template bool profile_spectrum_supported_impl<double>(const FftPlan2D&);
template void profile_spectrum_impl<double>(mlc_ctx*, const FftPlan2D&, const double*, int, void*);
template void conv_cached_impl<double>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);
template void conv_cached_real_impl<double>(mlc_ctx*, const FftPlan2D&, const void*, const void*, void*);
template void conv_plain_impl<double>(mlc_ctx*, const FftPlan2D&, const void*, const double*, int, void*);
template bool c2r_interleave_impl<double, double>(mlc_ctx*, const FftPlan2D&, const void*, long, int, int, void*, unsigned);

}  // namespace mlc
