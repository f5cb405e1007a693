// FP64 instantiation of the fused step.  This translation unit is compiled
// with --fmad=false: no multiply-add is contracted, so every FP64 operation
// rounds exactly like the reference CPU kernels (which Numba compiles without
// fast-math) and the results are bit-identical to them.
#define LBM_STEP_DEFINITIONS
#include "lbm_aux.cuh"

namespace lbm {

template cudaError_t step_coll<double, 0>(int, const StepArgs&, Variant, int, cudaStream_t);
template cudaError_t step_coll<double, 1>(int, const StepArgs&, Variant, int, cudaStream_t);

const KernelSet& kernels_fp64() {
  static const KernelSet k = Kernels<double>::make();
  return k;
}

}  // namespace lbm
