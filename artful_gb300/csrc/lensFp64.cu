/* artful_cuda — the plain FP64 trace: the reference's integrator with every operation in double,
 * from the frame computed in double.  The FP64 GPU oracle the mixed-precision trace is measured against
 * (and, at half step, the discretisation reference). */
#define ARTF_FAST_FP64 1 /* FP64 division and square roots by refined hardware estimates (lensCore.cuh) */
#include "lensKernel.cuh"

namespace artf {
cudaError_t launchFp64(const TraceLaunch& l) { return launchUniform<double>(l, &l.frame64); }
}  // namespace artf
