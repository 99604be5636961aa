// Relocation kernels of one smoother (see gm_relocate.cuh).
#include "gm_relocate.cuh"

namespace gm {

cudaError_t launch_relocate_spawn(const RelocLaunch& L) { return launch_relocate_smoother<kSmoothSpawn>(L); }

}  // namespace gm
