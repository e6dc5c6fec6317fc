/* artful_cuda — the FP32 trace with the reference's rounding.  Built with -fmad=false -prec-div=true
 * -prec-sqrt=true -ftz=false: every float operation rounds once, as the reference's SIMD kernels do
 * (src/software/simd.h:1-5, CMakeLists.txt:54-55), so the frame comes out bit for bit the same. */
#include "lensKernel.cuh"

namespace artf {
cudaError_t launchExact(const TraceLaunch& l) { return launchUniform<float>(l, &l.frame); }
}  // namespace artf
