// Precision-independent helpers (deterministic final reduction, host-order
// <-> device-order node copies).
#include "lbm_aux.cuh"

namespace lbm {

// Sums rows of 8 doubles in two fixed-shape stages (same result every run):
// kFinishBlocks blocks each sum a contiguous range of rows (thread t takes
// rows t, t+256, ... of the range, then a shared-memory tree), and one block
// sums those kFinishBlocks rows the same way.
__global__ void finish_reduce_kernel(const double* __restrict__ partials,
                                     long long nrows, double* scratch, unsigned* counter,
                                     double* out8) {
  __shared__ double sh[8][256];
  __shared__ bool last;
  // stage 1: block b sums the rows of its contiguous slice into scratch row b
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
  if (threadIdx.x < 8) scratch[blockIdx.x * 8 + threadIdx.x] = sh[threadIdx.x][0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  // stage 2, in the last block to finish: the scratch rows in row order
  __threadfence();
#pragma unroll
  for (int c = 0; c < 8; ++c) s[c] = 0;
  for (int r = threadIdx.x; r < (int)gridDim.x; r += blockDim.x)
#pragma unroll
    for (int c = 0; c < 8; ++c) s[c] += __ldcg(scratch + r * 8 + c);
#pragma unroll
  for (int c = 0; c < 8; ++c) sh[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
#pragma unroll
      for (int c = 0; c < 8; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 8) out8[threadIdx.x] = sh[threadIdx.x][0];
  if (threadIdx.x == 0) *counter = 0u;   // ready for the next reduction
}

cudaError_t finish_reduce(const double* partials, long long nrows, double* scratch,
                          double* out8, cudaStream_t s) {
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kFinishBlocks * 8);
  finish_reduce_kernel<<<kFinishBlocks, 256, 0, s>>>(partials, nrows, scratch, counter, out8);
  return cudaGetLastError();
}

// Host order <-> device order, as a tiled transpose: host arrays are x-major
// (consecutive y contiguous), device planes y-major (consecutive x
// contiguous).  A 32 x 32 tile passes through shared memory, so both sides
// are read and written in contiguous runs; the host side may be the caller's
// pinned buffer itself, read or written over the host link.
// layout 0: inner ind = x*ny + y ; 1: padded ind = (x+1)*(ny+2) + (y+1)
constexpr int kTile = 32, kTileRows = 8;

template <class TI, class TO>
__global__ void __launch_bounds__(kTile * kTileRows)
    reorder_kernel(const Geom g, const TI* __restrict__ in, TO* __restrict__ out,
                   int ncomp, int layout, int to_device, int x_lo, int x_hi) {
  __shared__ double t[kTile][kTile + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = x_lo + blockIdx.x * kTile, y0 = blockIdx.y * kTile;
  const long long hy = layout == 0 ? g.ny : g.ny + 2;   // host stride of x
  const int off = layout == 0 ? 0 : 1;
  for (int c = 0; c < ncomp; ++c) {
    if (to_device) {
      for (int r = ty; r < kTile; r += kTileRows) {   // host rows: x = x0 + r, lanes along y
        const int x = x0 + r, y = y0 + tx;
        if (x < x_hi && y < g.ny) t[r][tx] = double(in[((x + off) * hy + y + off) * ncomp + c]);
      }
      __syncthreads();
      for (int r = ty; r < kTile; r += kTileRows) {   // device rows: y = y0 + r, lanes along x
        const int x = x0 + tx, y = y0 + r;
        if (x < x_hi && y < g.ny) out[c * g.plane + g.node(x, y)] = TO(t[tx][r]);
      }
    } else {
      for (int r = ty; r < kTile; r += kTileRows) {
        const int x = x0 + tx, y = y0 + r;
        if (x < x_hi && y < g.ny) t[r][tx] = double(in[c * g.plane + g.node(x, y)]);
      }
      __syncthreads();
      for (int r = ty; r < kTile; r += kTileRows) {
        const int x = x0 + r, y = y0 + tx;
        if (x < x_hi && y < g.ny) out[((x + off) * hy + y + off) * ncomp + c] = TO(t[tx][r]);
      }
    }
    __syncthreads();
  }
}

// Self-test of the bounded wait: one thread waits on an mbarrier that
// expects one arrival nobody makes.  The wait must give up after limit_ns,
// set kErrWaitTimeout in *err and return; *waited_ns receives how long it
// waited.  The barrier is invalidated before the block exits.
__global__ void bounded_wait_selftest_kernel(int* err, unsigned long long limit_ns,
                                             unsigned long long* waited_ns) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const unsigned long long t0 = global_ns();
  const bool got = mbar_wait_bounded(b, 0, err, limit_ns);
  *waited_ns = global_ns() - t0;
  if (got) atomicExch(err, 0);
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
}

cudaError_t bounded_wait_selftest(int* err, double limit_s, unsigned long long* waited_ns,
                                  cudaStream_t s) {
  bounded_wait_selftest_kernel<<<1, 32, 0, s>>>(err, (unsigned long long)(limit_s * 1e9), waited_ns);
  return cudaGetLastError();
}

template <class TI, class TO>
static cudaError_t reorder_launch(const Geom& g, const TI* in, TO* out, int ncomp, int layout,
                                  int to_device, int x_lo, int x_hi, cudaStream_t s) {
  if (x_lo < 0 || x_hi > g.nx || x_lo >= x_hi) return cudaErrorInvalidValue;
  dim3 grid((x_hi - x_lo + kTile - 1) / kTile, (g.ny + kTile - 1) / kTile);
  reorder_kernel<TI, TO><<<grid, dim3(kTile, kTileRows), 0, s>>>(g, in, out, ncomp, layout,
                                                                 to_device, x_lo, x_hi);
  return cudaGetLastError();
}

cudaError_t reorder(const Geom& g, const double* in, double* out, int ncomp,
                    int layout, int to_device, cudaStream_t s) {
  return reorder_launch(g, in, out, ncomp, layout, to_device, 0, g.nx, s);
}

cudaError_t reorder_cols(const Geom& g, const double* in, double* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s) {
  return reorder_launch(g, in, out, ncomp, layout, to_device, x_lo, x_hi, s);
}

cudaError_t reorder_cols(const Geom& g, const float* in, double* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s) {
  return reorder_launch(g, in, out, ncomp, layout, to_device, x_lo, x_hi, s);
}

cudaError_t reorder_cols(const Geom& g, const double* in, float* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s) {
  return reorder_launch(g, in, out, ncomp, layout, to_device, x_lo, x_hi, s);
}

cudaError_t reorder_cols(const Geom& g, const float* in, float* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s) {
  return reorder_launch(g, in, out, ncomp, layout, to_device, x_lo, x_hi, s);
}

}  // namespace lbm
