// FP32 shifted-storage instantiation of the fused step and its helpers.
#include "lbm_aux.cuh"

namespace lbm {

const KernelSet& kernels_fp32() {
  static const KernelSet k = Kernels<float>::make();
  return k;
}

}  // namespace lbm
