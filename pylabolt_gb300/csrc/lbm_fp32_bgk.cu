// FP32 shifted storage: the fused step's BGK instantiations (every kernel
// shape, forcing model and phase).
#define LBM_STEP_DEFINITIONS
#include "lbm_aux.cuh"

namespace lbm {

template cudaError_t step_coll<float, 0>(int, const StepArgs&, Variant, int, cudaStream_t);

}  // namespace lbm
