// Precision-independent helpers (deterministic final reduction, host-order
// <-> device-order node copies).
#include "lbm_aux.cuh"

namespace lbm {

// Sums rows of 8 doubles in two fixed-shape stages (same result every run):
// kFinishBlocks blocks each sum a contiguous range of rows (thread t takes
// rows t, t+256, ... of the range, then a shared-memory tree), and one block
// sums those kFinishBlocks rows the same way.
__global__ void finish_reduce_kernel(const double* __restrict__ partials,
                                     long long nrows, double* out) {
  __shared__ double sh[8][256];
  const long long per = (nrows + gridDim.x - 1) / gridDim.x;
  const long long r0 = blockIdx.x * per;
  const long long r1 = r0 + per < nrows ? r0 + per : nrows;
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x)
#pragma unroll
    for (int c = 0; c < 8; ++c) s[c] += partials[r * 8 + c];
#pragma unroll
  for (int c = 0; c < 8; ++c) sh[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
#pragma unroll
      for (int c = 0; c < 8; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 8) out[blockIdx.x * 8 + threadIdx.x] = sh[threadIdx.x][0];
}

cudaError_t finish_reduce(const double* partials, long long nrows, double* scratch,
                          double* out8, cudaStream_t s) {
  finish_reduce_kernel<<<kFinishBlocks, 256, 0, s>>>(partials, nrows, scratch);
  finish_reduce_kernel<<<1, 256, 0, s>>>(scratch, kFinishBlocks, out8);
  return cudaGetLastError();
}

// layout 0: inner ind = x*ny + y ; 1: padded ind = (x+1)*(ny+2) + (y+1)
__global__ void reorder_kernel(const Geom g, const double* __restrict__ in,
                               double* __restrict__ out, int ncomp, int layout,
                               int to_device) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.nx) return;
  const long long hn = layout == 0 ? (long long)x * g.ny + y
                                   : (long long)(x + 1) * (g.ny + 2) + (y + 1);
  const long long dn = g.node(x, y);
  for (int c = 0; c < ncomp; ++c) {
    if (to_device)
      out[c * g.plane + dn] = in[hn * ncomp + c];
    else
      out[hn * ncomp + c] = in[c * g.plane + dn];
  }
}

cudaError_t reorder(const Geom& g, const double* in, double* out, int ncomp,
                    int layout, int to_device, cudaStream_t s) {
  dim3 grid((g.nx + kStepBlock - 1) / kStepBlock, g.ny);
  reorder_kernel<<<grid, kStepBlock, 0, s>>>(g, in, out, ncomp, layout, to_device);
  return cudaGetLastError();
}

}  // namespace lbm
