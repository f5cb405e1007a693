// FP32 shifted-storage instantiation of the kernel set; the fused step's
// BGK and MRT instantiations are in lbm_fp32_bgk.cu and lbm_fp32_mrt.cu.
#include "lbm_aux.cuh"

namespace lbm {

const KernelSet& kernels_fp32() {
  static const KernelSet k = Kernels<float>::make();
  return k;
}

}  // namespace lbm
