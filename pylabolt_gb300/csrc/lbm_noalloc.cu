// lbm_conservation_noalloc: mass and momentum sums of a population array
// that the caller owns, computed without allocating any device memory.
//
// Why it exists: some callers of this library cannot allocate device memory.
// Examples are in-situ analysis code embedded in a larger solver that hands
// out all device memory from its own pool, and monitoring loops that cannot
// afford cudaMalloc's implicit device synchronisation.  This entry point
// takes device pointers to its input and output and keeps its scratch (one
// partial-sum row per grid row plus the second reduction stage) in a fixed,
// file-scope device array instead of allocating it.
//
// The device address of that array is looked up once per device, on the
// first call with that device current, and kept for the life of the process;
// a cudaDeviceReset of the device makes it stale (the header says so).
//
// The scratch array below is part of the library image: every GPU that loads
// liblbm_gb300.so holds it (about 0.5 MB) until the process exits.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "lbm_gb300.h"
#include "lbm_internal.h"

namespace {

constexpr int kNoAllocMaxRows = LBM_NOALLOC_MAX_ROWS;   // largest ny accepted
constexpr int kStage2Blocks = 64;                        // second-stage rows
constexpr int kCols = 8;                                 // doubles per partial row

// Partial sums: rows [0, ny) of the first stage, then kStage2Blocks rows of
// the second stage.  Each call overwrites every row it later reads, so nothing
// has to be cleared between calls.
static __device__ __align__(256) double g_noalloc_scratch[(kNoAllocMaxRows + kStage2Blocks) * kCols];

// Device address of g_noalloc_scratch per device ordinal (host code cannot use
// the symbol's name as a device pointer).
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int fail(int code, const std::string& msg) {
  lbm::record_error(msg);   // reported by lbm_last_error()
  return code;
}

__host__ __device__ constexpr double wk(int k) {
  return k == 0 ? 4.0 / 9.0 : (k <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
}
__host__ __device__ constexpr int cxk(int k) {
  return (k == 1 || k == 5 || k == 8) ? 1 : ((k == 3 || k == 6 || k == 7) ? -1 : 0);
}
__host__ __device__ constexpr int cyk(int k) {
  return (k == 2 || k == 5 || k == 6) ? 1 : ((k == 4 || k == 7 || k == 8) ? -1 : 0);
}

template <int PREC>
__device__ __forceinline__ double load_f(const void* pop, long long i, int k, double inv_scale) {
  if (PREC == LBM_FP64) return static_cast<const double*>(pop)[i];
  if (PREC == LBM_FP32_SHIFTED) return double(static_cast<const float*>(pop)[i]) + wk(k);
  return double(__half2float(static_cast<const __half*>(pop)[i])) * inv_scale + wk(k);
}

// Stage 1: one block per grid row, fixed summation order.
template <int PREC>
__global__ void row_sums_kernel(LbmPopView v, double inv_scale, double* scratch) {
  const int y = blockIdx.x;
  double s[3] = {0, 0, 0};
  for (int x = threadIdx.x; x < v.nx; x += blockDim.x) {
    const long long n = (long long)y * v.pitch + x;
    if (v.exclude && v.exclude[n]) continue;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double f = load_f<PREC>(v.pop, k * v.plane + n, k, inv_scale);
      s[0] += f;
      s[1] += cxk(k) * f;
      s[2] += cyk(k) * f;
    }
  }
  __shared__ double sh[3][256];
  for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < kCols) scratch[(long long)y * kCols + threadIdx.x] = threadIdx.x < 3 ? sh[threadIdx.x][0] : 0.0;
}

// Stages 2 and 3: sum `nrows` rows into gridDim.x rows (fixed order).
__global__ void rows_reduce_kernel(const double* in, int nrows, double* out, int ncols_out) {
  __shared__ double sh[3][256];
  const int per = (nrows + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * per;
  const int r1 = r0 + per < nrows ? r0 + per : nrows;
  double s[3] = {0, 0, 0};
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    for (int c = 0; c < 3; ++c) s[c] += in[(long long)r * kCols + c];
  for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < ncols_out) out[(long long)blockIdx.x * ncols_out + threadIdx.x] = threadIdx.x < 3 ? sh[threadIdx.x][0] : 0.0;
}

// One-time set-up per device (with that device current): the device address
// of the scratch array.
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(LBM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<double*>(g_scratch_addr[dev]);
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_conservation_noalloc(const LbmPopView* view, double* out_device, void* stream) {
  if (!view || !view->pop || !out_device)
    return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: null argument");
  const LbmPopView& v = *view;
  if (v.precision < LBM_FP64 || v.precision > LBM_FP16_SHIFTED)
    return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: unknown precision");
  if (v.nx < 1 || v.ny < 1 || v.pitch < v.nx || v.plane < (long long)v.ny * v.pitch)
    return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: need nx, ny >= 1, pitch >= nx, plane >= ny*pitch");
  if (v.ny > kNoAllocMaxRows)
    return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: ny = " + std::to_string(v.ny) +
                                 " exceeds the " + std::to_string(kNoAllocMaxRows) +
                                 " rows of its fixed scratch; use lbm_conservation on a handle");
  if (v.precision == LBM_FP16_SHIFTED && !(v.fp16_scale > 0.0))
    return fail(LBM_ERR_ARG, "lbm_conservation_noalloc: fp16_scale must be > 0");
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double inv_scale = v.precision == LBM_FP16_SHIFTED ? 1.0 / v.fp16_scale : 1.0;
  if (v.precision == LBM_FP64)
    row_sums_kernel<LBM_FP64><<<v.ny, 256, 0, s>>>(v, inv_scale, scratch);
  else if (v.precision == LBM_FP32_SHIFTED)
    row_sums_kernel<LBM_FP32_SHIFTED><<<v.ny, 256, 0, s>>>(v, inv_scale, scratch);
  else
    row_sums_kernel<LBM_FP16_SHIFTED><<<v.ny, 256, 0, s>>>(v, inv_scale, scratch);
  double* stage2 = scratch + (long long)kNoAllocMaxRows * kCols;
  rows_reduce_kernel<<<kStage2Blocks, 256, 0, s>>>(scratch, v.ny, stage2, kCols);
  rows_reduce_kernel<<<1, 256, 0, s>>>(stage2, kStage2Blocks, out_device, 3);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}

}  // extern "C"
