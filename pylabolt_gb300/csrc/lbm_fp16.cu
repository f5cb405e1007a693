// FP16 shifted-storage instantiation of the kernel set; the fused step's
// BGK and MRT instantiations are in lbm_fp16_bgk.cu and lbm_fp16_mrt.cu.
#include "lbm_aux.cuh"

namespace lbm {

const KernelSet& kernels_fp16() {
  static const KernelSet k = Kernels<__half>::make();
  return k;
}

}  // namespace lbm
