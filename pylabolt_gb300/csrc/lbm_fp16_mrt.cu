// FP16 shifted storage: the fused step's MRT instantiations (every kernel
// shape, forcing model and phase).
#define LBM_STEP_DEFINITIONS
#include "lbm_aux.cuh"

namespace lbm {

template cudaError_t step_coll<__half, 1>(int, const StepArgs&, Variant, int, cudaStream_t);

}  // namespace lbm
