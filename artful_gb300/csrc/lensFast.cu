/* artful_cuda — the FP32 trace at full speed.  Built with fused multiply-adds and fast division and
 * square roots (-fmad=true -prec-div=false -prec-sqrt=false -ftz=true): within the reference's
 * tolerance, not its bits. */
#include "lensKernel.cuh"

namespace artf {
cudaError_t launchFast(const TraceLaunch& l) { return launchUniform<float>(l, &l.frame); }
}  // namespace artf
