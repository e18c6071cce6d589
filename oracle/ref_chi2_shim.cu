// Test infrastructure only: the reference's getChi2CPU (chi2/chi2_functions.cuh:150-190)
// behind a C entry, compiled from the reference's sources where they lie into
// oracle/_ref/libmlcref_chi2.so by oracle/Makefile.  Nothing in the product links it.
#include "chi2_functions.cuh"

extern "C" float ref_chi2_cpu(const float* f_obs, const float* df_obs, const float* mu1, const float* mu2, int N,
                              int F, int T) {
  float like = 0.0f;
  getChi2CPU(const_cast<float*>(f_obs), const_cast<float*>(df_obs), const_cast<float*>(mu1),
             const_cast<float*>(mu2), N, F, T, &like);
  return like;
}
