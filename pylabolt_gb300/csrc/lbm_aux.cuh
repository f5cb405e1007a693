// Auxiliary kernels of one storage precision (conversions, conservation sums)
// and the KernelSet that bundles them with the fused step kernel.
#pragma once
#include <utility>

#include "lbm_adjoint.cuh"
#include "lbm_force.cuh"
#include "lbm_moving.cuh"

namespace lbm {

constexpr int kStepBlock = 256;

template <class S>
__global__ void convert_kernel(const Geom g, const Params p, S* f, double* f64,
                               int dir, int aa_state) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.nx) return;
  const long long n = g.node(x, y);
  const bool solid = g.cls[n] == 2;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const long long i = k * g.plane + n;
    const double w = Store<S>::shifted ? Wk(k) : 0.0;
    if (dir == 0) {
      const long long src = aa_post_index(g.plane, g.pitch, aa_state, n, k);
      f64[i] = solid ? 0.0 : double(Store<S>::ld(f, src, p)) + w;
    } else {
      Store<S>::st(f, i, typename Store<S>::T(solid ? 0.0 : f64[i] - w), p);
    }
  }
}

template <class T>
__global__ void moments_to_f64_kernel(const Geom g, const T* mr, const T* mx,
                                      const T* my, double* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.nx) return;
  const long long n = g.node(x, y);
  out[n] = double(mr[n]);
  out[g.plane + n] = double(mx[n]);
  out[2 * g.plane + n] = double(my[n]);
}

template <class T>
__global__ void body_from_f64_kernel(const Geom g, const double* in, T* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.nx) return;
  const long long n = g.node(x, y);
  out[n] = T(in[n]);
  out[g.plane + n] = T(in[g.plane + n]);
}

// One block per row; fixed summation order -> deterministic.
template <class S>
__global__ void conservation_kernel(const Geom g, const Params p, const S* f,
                                    double* partials, int aa_state) {
  const int y = blockIdx.x;
  double s[3] = {0, 0, 0};
  for (int x = threadIdx.x; x < g.nx; x += blockDim.x) {
    const long long n = g.node(x, y);
    if (g.cls[n] == 2) continue;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double v = double(Store<S>::ld(f, aa_post_index(g.plane, g.pitch, aa_state, n, k), p)) +
                       (Store<S>::shifted ? Wk(k) : 0.0);
      s[0] += v;
      s[1] += CXk(k) * v;
      s[2] += CYk(k) * v;
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
  if (threadIdx.x < 8)
    partials[(long long)y * 8 + threadIdx.x] = threadIdx.x < 3 ? sh[threadIdx.x][0] : 0.0;
}

// ---------------------------------------------------------------------------
template <class S, int COLL>
cudaError_t step_coll(int forc, const StepArgs& a, Variant v, int sms, cudaStream_t s);

template <class S>
struct Kernels {
  using T = typename Store<S>::T;
  static dim3 node_grid(const Geom& g) {
    return dim3((g.nx + kStepBlock - 1) / kStepBlock, g.ny);
  }
  // The scalar kernel with or without the residual's code.
  template <int COLL, int FORC, bool RES>
  static cudaError_t scalar(const StepArgs& a, Variant v, dim3 grid, cudaStream_t s) {
    if (a.rho_dyn_out) {   // moving obstacles: the scalar kernel's MOV instantiations
      if (v.stages == 0)
        step_kernel<S, COLL, FORC, 0, true, RES><<<grid, v.block, 0, s>>>(a);
      else if (v.stages == 1 && v.block <= 256)
        step_kernel<S, COLL, FORC, 1, true, RES><<<grid, v.block, 0, s>>>(a);
      else if (v.stages == 2 && v.block <= 256)
        step_kernel<S, COLL, FORC, 2, true, RES><<<grid, v.block, 0, s>>>(a);
      else
        return cudaErrorInvalidValue;
      return cudaGetLastError();
    }
    if (v.stages == 1 || v.stages == 2) {
      if (v.block > 256) return cudaErrorInvalidValue;
      if (v.stages == 1)
        step_kernel<S, COLL, FORC, 1, false, RES><<<grid, v.block, 0, s>>>(a);
      else
        step_kernel<S, COLL, FORC, 2, false, RES><<<grid, v.block, 0, s>>>(a);
    } else {
      step_kernel<S, COLL, FORC, 0, false, RES><<<grid, v.block, 0, s>>>(a);
    }
    return cudaGetLastError();
  }

  // The node-pair kernel (stages = register cap: 0 none, 1 40, 2 64, 3 32);
  // with moving obstacles (rho_dyn_out) the 40-register shape only.
  template <int COLL, int FORC, bool RES>
  static cudaError_t pair(const StepArgs& a, Variant v, dim3 grid, cudaStream_t s) {
    if constexpr (Store<S>::shifted) {
      if (a.rho_dyn_out) {
        if (v.stages != 1) return cudaErrorInvalidValue;
        step_pair_kernel<S, COLL, FORC, 1, RES, true><<<grid, v.block, 0, s>>>(a);
        return cudaGetLastError();
      }
      switch (v.stages) {
        case 0: step_pair_kernel<S, COLL, FORC, 0, RES><<<grid, v.block, 0, s>>>(a); break;
        case 1: step_pair_kernel<S, COLL, FORC, 1, RES><<<grid, v.block, 0, s>>>(a); break;
        case 2: step_pair_kernel<S, COLL, FORC, 2, RES><<<grid, v.block, 0, s>>>(a); break;
        case 3: step_pair_kernel<S, COLL, FORC, 3, RES><<<grid, v.block, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
      }
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }

  // The AA node-pair kernel, one phase (stages = register cap).
  template <int COLL, int FORC>
  static cudaError_t aa_pair(const StepArgs& a, Variant v, dim3 grid, cudaStream_t s) {
    if constexpr (Store<S>::shifted) {
      if (v.vec != 2) return cudaErrorInvalidValue;
      const bool odd = a.aa == 2;
      switch (v.stages * 2 + (odd ? 1 : 0)) {
        case 0: step_aa_pair_kernel<S, COLL, FORC, 0, false><<<grid, v.block, 0, s>>>(a); break;
        case 1: step_aa_pair_kernel<S, COLL, FORC, 0, true><<<grid, v.block, 0, s>>>(a); break;
        case 2: step_aa_pair_kernel<S, COLL, FORC, 1, false><<<grid, v.block, 0, s>>>(a); break;
        case 3: step_aa_pair_kernel<S, COLL, FORC, 1, true><<<grid, v.block, 0, s>>>(a); break;
        case 4: step_aa_pair_kernel<S, COLL, FORC, 2, false><<<grid, v.block, 0, s>>>(a); break;
        case 5: step_aa_pair_kernel<S, COLL, FORC, 2, true><<<grid, v.block, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
      }
      return cudaGetLastError();
    }
    return cudaErrorInvalidValue;
  }

  // MODE 0: two buffers; 1 / 2: the AA layout's even / odd phase (two pairs
  // of a tile per thread only)
  template <int COLL, int FORC, bool RES, int MODE>
  static cudaError_t tile(const StepArgs& a, Variant v, dim3 grid, cudaStream_t s) {
    if constexpr (Store<S>::shifted) {
      const int smem = v.stages * tile_stage_bytes();
      constexpr int TP = kTileBytes / (2 * sizeof(S));   // pairs of a tile
      // bytes the attribute was last raised to, per device (function
      // attributes belong to each device's copy of the kernel)
      constexpr int kDevices = 64;
      static int configured[kDevices][3] = {};
      if (v.block == TP / 2 || (MODE == 0 && (v.block == TP || v.block == TP / 4))) {
        const int i = v.block == TP ? 0 : (v.block == TP / 2 ? 1 : 2);
        const auto kern = MODE != 0 ? step_tile_pair_kernel<S, COLL, FORC, RES, 2, MODE>
                          : i == 0  ? step_tile_pair_kernel<S, COLL, FORC, RES, 1, MODE>
                          : i == 1  ? step_tile_pair_kernel<S, COLL, FORC, RES, 2, MODE>
                                    : step_tile_pair_kernel<S, COLL, FORC, RES, 4, MODE>;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kDevices || smem > configured[dev][i]) {
          e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
          if (e != cudaSuccess) return e;
          if (dev >= 0 && dev < kDevices) configured[dev][i] = smem;
        }
        kern<<<grid, v.block, smem, s>>>(a, v.stages);
        return cudaGetLastError();
      }
    }
    return cudaErrorInvalidValue;
  }

  template <int COLL, int FORC>
  static cudaError_t step_t(const StepArgs& a, Variant v, int sms, cudaStream_t s) {
    const dim3 grid = step_grid(a.g, v, sms, sizeof(S), (a.flags & F_RESIDUAL) != 0);
    if (a.aa) {   // AA layout: the scalar kernel (capped for shifted storage), one phase
      constexpr int AC = Store<S>::shifted ? (COLL == 0 ? 1 : 2) : 0;
      if constexpr (Store<S>::shifted) {
        if (v.kind == 2) {   // node pairs from shared-memory tiles, in place
          if (v.vec != 2 || v.block != kTileBytes / (4 * (int)sizeof(S)) || v.stages < 1 ||
              v.stages > kMaxTileStages || a.rho_dyn_out)
            return cudaErrorInvalidValue;
          const bool res = (a.flags & F_RESIDUAL) != 0;
          if (a.aa == 1)
            return res ? tile<COLL, FORC, true, 1>(a, v, grid, s) : tile<COLL, FORC, false, 1>(a, v, grid, s);
          return res ? tile<COLL, FORC, true, 2>(a, v, grid, s) : tile<COLL, FORC, false, 2>(a, v, grid, s);
        }
      }
      if (v.block > 256) return cudaErrorInvalidValue;
      if (v.kind == 3) return aa_pair<COLL, FORC>(a, v, grid, s);
      if (v.kind != 0) return cudaErrorInvalidValue;
      if (a.aa == 1)
        step_aa_kernel<S, COLL, FORC, AC, false><<<grid, v.block, 0, s>>>(a);
      else
        step_aa_kernel<S, COLL, FORC, AC, true><<<grid, v.block, 0, s>>>(a);
      return cudaGetLastError();
    }
    if constexpr (Store<S>::shifted) {
      if (v.kind == 3) {   // node pairs (moving obstacles: the 40-register shape)
        if (v.vec != 2 || v.block > 256) return cudaErrorInvalidValue;
        if (a.flags & F_RESIDUAL) return pair<COLL, FORC, true>(a, v, grid, s);
        return pair<COLL, FORC, false>(a, v, grid, s);
      }
      if (v.kind == 2) {   // node pairs from shared-memory tiles (no moving obstacles)
        if (v.vec != 2 || (v.block != kTileBytes / (2 * (int)sizeof(S)) &&
                           v.block != kTileBytes / (4 * (int)sizeof(S)) &&
                           v.block != kTileBytes / (8 * (int)sizeof(S))) ||
            v.stages < 1 || v.stages > kMaxTileStages || a.rho_dyn_out)
          return cudaErrorInvalidValue;
        if (a.flags & F_RESIDUAL) return tile<COLL, FORC, true, 0>(a, v, grid, s);
        return tile<COLL, FORC, false, 0>(a, v, grid, s);
      }
    }
    if (v.kind != 0) return cudaErrorInvalidValue;
    if (a.flags & F_RESIDUAL) return scalar<COLL, FORC, true>(a, v, grid, s);
    return scalar<COLL, FORC, false>(a, v, grid, s);
  }
  static cudaError_t step(int coll, int forc, const StepArgs& a, Variant v, int sms,
                          cudaStream_t s) {
    return coll == 0 ? step_coll<S, 0>(forc, a, v, sms, s) : step_coll<S, 1>(forc, a, v, sms, s);
  }
  static cudaError_t init(const Geom& g, const Params& p, const double* rho,
                          const double* u, void* f, void* mr, void* mx, void* my,
                          int x_lo, int x_hi, cudaStream_t s) {
    if (x_lo < 0 || x_hi > g.nx || x_lo >= x_hi) return cudaErrorInvalidValue;
    const dim3 grid((x_hi - x_lo + kStepBlock - 1) / kStepBlock, g.ny);
    init_kernel<S><<<grid, kStepBlock, 0, s>>>(
        g, p, rho, u, static_cast<S*>(f), static_cast<T*>(mr),
        static_cast<T*>(mx), static_cast<T*>(my), x_lo, x_hi);
    return cudaGetLastError();
  }
  static cudaError_t convert(const Geom& g, const Params& p, void* f,
                             double* f64, int dir, int aa_state, cudaStream_t s) {
    convert_kernel<S><<<node_grid(g), kStepBlock, 0, s>>>(g, p, static_cast<S*>(f),
                                                           f64, dir, aa_state);
    return cudaGetLastError();
  }
  static cudaError_t moments_to_f64(const Geom& g, const void* mr, const void* mx,
                                    const void* my, double* out, cudaStream_t s) {
    moments_to_f64_kernel<T><<<node_grid(g), kStepBlock, 0, s>>>(
        g, static_cast<const T*>(mr), static_cast<const T*>(mx),
        static_cast<const T*>(my), out);
    return cudaGetLastError();
  }
  static cudaError_t body_from_f64(const Geom& g, const double* in, void* out,
                                   cudaStream_t s) {
    body_from_f64_kernel<T><<<node_grid(g), kStepBlock, 0, s>>>(g, in,
                                                                 static_cast<T*>(out));
    return cudaGetLastError();
  }
  static cudaError_t conservation(const Geom& g, const Params& p, const void* f,
                                  double* partials, int aa_state, cudaStream_t s) {
    conservation_kernel<S><<<g.ny, 256, 0, s>>>(g, p, static_cast<const S*>(f), partials,
                                                aa_state);
    return cudaGetLastError();
  }
  template <class U = S>
  static cudaError_t adjoint(int forc, const AdjArgs& a, cudaStream_t s) {
    const dim3 grid = node_grid(a.g);
    if (forc == 0)
      adjoint_kernel<S, 0><<<grid, kStepBlock, 0, s>>>(a);
    else if (forc == 1)
      adjoint_kernel<S, 1><<<grid, kStepBlock, 0, s>>>(a);
    else
      adjoint_kernel<S, 2><<<grid, kStepBlock, 0, s>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t forces(const ForceArgs& a, int ngroups, cudaStream_t s) {
    force_kernel<S><<<ngroups, kForceBlock, 0, s>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t mov_motion(const MovArgs& a, cudaStream_t s) {
    mov_motion_kernel<S><<<1, kMovMaxObstacles, 0, s>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t mov_raster(const MovArgs& a, int side, cudaStream_t s) {
    const dim3 blk(16, 16), grid((side + 15) / 16, (side + 15) / 16);
    mov_raster_kernel<S><<<grid, blk, 0, s>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t mov_classify(const MovArgs& a, int side, cudaStream_t s) {
    const dim3 blk(16, 16), grid((side + 2 + 15) / 16, (side + 2 + 15) / 16);
    mov_classify_kernel<S><<<grid, blk, 0, s>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t mov_force(const MovArgs& a, cudaStream_t s) {
    mov_force_kernel<S><<<kMovForceBlocks, kMovForceThreads, 0, s>>>(a);
    mov_force_finish_kernel<S><<<1, kMovForceBlocks, 0, s>>>(a);
    return cudaGetLastError();
  }
  static KernelSet make() {
    KernelSet k;
    k.elem_bytes = sizeof(S);
    k.compute_bytes = sizeof(T);
    k.step = &step;
    if constexpr (Store<S>::shifted) {
      // kind 2: node pairs from shared-memory tiles {2, threads, stages}
      // (TP threads: one pair of a tile each, TP / 2: two, TP / 4: four);
      // kind 0: {threads, register cap: 0 none, 1 32, 2 40};
      // kind 3: node pairs {2 nodes per thread, threads, register cap: 0 none,
      // 1 40, 2 64, 3 32}
      // The first candidate runs the untuned first step and is kept with
      // LBM_TUNE=0: the one that measured fastest for the storage at
      // 8192x2048 (FP32 node pairs, FP16 node-pair tiles).
      constexpr int TP = kTileBytes / (2 * sizeof(S));
      const Variant vs[] = {{2, 2, TP / 2, 2}, {2, 2, TP / 2, 3}, {2, 2, TP, 2},
                            {2, 2, TP / 4, 2}, {0, 1, 128, 0}, {0, 1, 256, 0}, {0, 1, 128, 1},
                            {0, 1, 256, 1}, {0, 1, 128, 2}, {0, 1, 256, 2}, {3, 2, 128, 0},
                            {3, 2, 256, 0}, {3, 2, 128, 1}, {3, 2, 256, 2}, {3, 2, 128, 3}};
      k.nvariants = 15;
      for (int i = 0; i < 15; ++i) k.variants[i] = vs[i];
      if (sizeof(S) == 4) std::swap(k.variants[0], k.variants[12]);
    } else {
      const Variant vs[] = {{0, 1, 128, 0}, {0, 1, 256, 0}, {0, 1, 512, 0}};
      k.nvariants = 3;
      for (int i = 0; i < 3; ++i) k.variants[i] = vs[i];
    }
    k.init = &init;
    k.convert = &convert;
    k.moments_to_f64 = &moments_to_f64;
    k.body_from_f64 = &body_from_f64;
    k.conservation = &conservation;
    k.forces = &forces;
    k.mov_motion = &mov_motion;
    k.mov_raster = &mov_raster;
    k.mov_classify = &mov_classify;
    k.mov_force = &mov_force;
    if constexpr (sizeof(S) >= 4)
      k.adjoint = &adjoint<S>;
    else
      k.adjoint = nullptr;
    return k;
  }
};

// One collision model's fused steps for storage S, defined (LBM_STEP_DEFINITIONS)
// and instantiated only in the units that compile them: lbm_fp64.cu for FP64,
// lbm_<storage>_{bgk,mrt}.cu for shifted storage, compiled in parallel.
#ifdef LBM_STEP_DEFINITIONS
template <class S, int COLL>
cudaError_t step_coll(int forc, const StepArgs& a, Variant v, int sms, cudaStream_t s) {
  if (forc == 0) return Kernels<S>::template step_t<COLL, 0>(a, v, sms, s);
  if (forc == 1) return Kernels<S>::template step_t<COLL, 1>(a, v, sms, s);
  return Kernels<S>::template step_t<COLL, 2>(a, v, sms, s);
}
#endif

}  // namespace lbm
