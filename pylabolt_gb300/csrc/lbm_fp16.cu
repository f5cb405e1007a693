// FP16 shifted-storage instantiation of the fused step and its helpers.
#include "lbm_aux.cuh"

namespace lbm {

const KernelSet& kernels_fp16() {
  static const KernelSet k = Kernels<__half>::make();
  return k;
}

}  // namespace lbm
