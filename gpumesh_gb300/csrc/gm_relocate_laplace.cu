// Relocation kernels of the Laplace smoothers (see gm_relocate.cuh).
#include "gm_relocate.cuh"

namespace gm {

cudaError_t launch_relocate_spring(const RelocLaunch& L) { return launch_relocate_smoother<kSmoothSpring>(L); }
cudaError_t launch_relocate_qlaplace(const RelocLaunch& L) { return launch_relocate_smoother<kSmoothQLaplace>(L); }

}  // namespace gm
