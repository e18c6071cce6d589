// Float-float inverse row passes with FP32 outputs (FP32 maps with
// mlc_map_set_fft(map, MLC_FFT_F32X2)): the interleaving last pass of a profile group and the
// plain last pass of a single convolution.  The forward transform and P0-P2 are the FP64
// maps' float-float kernels (fft_ff.cu, fft_ff_conv.cu): they read and write float-float
// spectra whatever the pixels' type.
#include "fft_impl.cuh"

namespace mlc {

template bool c2r_interleave_impl<ff, float>(mlc_ctx*, const FftPlan2D&, const void*, long, int, int, void*, unsigned);
template void rows_c2r_impl<ff, float>(mlc_ctx*, const FftPlan2D&, const void*, void*);

}  // namespace mlc
