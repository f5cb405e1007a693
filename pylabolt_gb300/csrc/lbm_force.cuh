// Momentum-exchange force and torque on obstacles and wall boundary elements.
//
// The reference evaluates, after a time step, for every link (node x,
// direction k_out towards a solid or a wall, k_in its opposite)
//     value = pop[x, k_out] c_{k_out} - pop_new[x, k_in] c_{k_in}
// with pop the post-collision populations of the step and pop_new the
// populations after streaming and boundaries
// (pylabolt/parallel/cpu/force_torque_kernels.py:11-90 for obstacles, with the
// torque r x value about the obstacle's reference point; :96-141 for wall
// boundary elements).  Here the device state after step t is pop = p_t, and
// pop_new at a boundary node is what the next step's pull computes from the
// node's link record, so the same link evaluation is reused.  Right after
// initialisation both are the stored populations (the reference initialises
// pop = pop_new = f_eq).  In the AA layout p_t and the link values are read
// where the phase left them (aa_post_index, special_link_aa).
//
// One block per group, a fixed-stride walk over the group's links and a fixed
// shared-memory tree: the sums are deterministic; they are formed in FP64 for
// every storage.
#pragma once
#include "lbm_kernels.cuh"

namespace lbm {

template <class S>
__device__ __forceinline__ typename Store<S>::T incoming_k(const Geom& g, const Params& p,
                                                          const S* __restrict__ f, long long n,
                                                          int r, const typename Store<S>::T* side,
                                                          int k) {
  switch (k) {
    case 1: return special_link<1, S>(g, p, f, n, r, side);
    case 2: return special_link<2, S>(g, p, f, n, r, side);
    case 3: return special_link<3, S>(g, p, f, n, r, side);
    case 4: return special_link<4, S>(g, p, f, n, r, side);
    case 5: return special_link<5, S>(g, p, f, n, r, side);
    case 6: return special_link<6, S>(g, p, f, n, r, side);
    case 7: return special_link<7, S>(g, p, f, n, r, side);
    case 8: return special_link<8, S>(g, p, f, n, r, side);
    default: return Store<S>::ld(f, n, p);
  }
}

// The same for the AA layout: ODD = the coming step is an odd phase.
template <class S, bool ODD>
__device__ __forceinline__ typename Store<S>::T incoming_k_aa(const Geom& g, const Params& p,
                                                             const S* __restrict__ f, long long n,
                                                             int r, const typename Store<S>::T* side,
                                                             int k) {
  switch (k) {
    case 1: return special_link_aa<1, S, ODD>(g, p, f, n, r, side);
    case 2: return special_link_aa<2, S, ODD>(g, p, f, n, r, side);
    case 3: return special_link_aa<3, S, ODD>(g, p, f, n, r, side);
    case 4: return special_link_aa<4, S, ODD>(g, p, f, n, r, side);
    case 5: return special_link_aa<5, S, ODD>(g, p, f, n, r, side);
    case 6: return special_link_aa<6, S, ODD>(g, p, f, n, r, side);
    case 7: return special_link_aa<7, S, ODD>(g, p, f, n, r, side);
    case 8: return special_link_aa<8, S, ODD>(g, p, f, n, r, side);
    default: return Store<S>::ld(f, n, p);
  }
}

constexpr int kForceBlock = 256;

template <class S>
__global__ void __launch_bounds__(kForceBlock) force_kernel(const ForceArgs a) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  __shared__ double red[3][kForceBlock];
  const int grp = blockIdx.x;
  const S* __restrict__ f = static_cast<const S*>(a.pop);
  const T* side = static_cast<const T*>(a.side);
  double sx = 0.0, sy = 0.0, st = 0.0;
  for (int i = a.gstart[grp] + threadIdx.x; i < a.gstart[grp + 1]; i += kForceBlock) {
    const long long n = a.node[i];
    const int ko = a.kk[2 * i], ki = a.kk[2 * i + 1];
    double fo = double(Store<S>::ld(f, aa_post_index(a.g.plane, a.g.pitch, a.aa_state, n, ko), a.p));
    double fi;
    if (a.nopull)
      fi = double(Store<S>::ld(f, ki * a.g.plane + n, a.p));
    else if (a.aa_state == 1)   // AA, after an even phase: the next step is odd
      fi = double(incoming_k_aa<S, true>(a.g, a.p, f, n, a.rec[i], side, ki));
    else if (a.aa_state == 2)
      fi = double(incoming_k_aa<S, false>(a.g, a.p, f, n, a.rec[i], side, ki));
    else
      fi = double(incoming_k<S>(a.g, a.p, f, n, a.rec[i], side, ki));
    if (SH) {  // shifted storage holds f - w
      fo += Wk(ko);
      fi += Wk(ki);
    }
    const double vx = fo * double(CXk(ko)) - fi * double(CXk(ki));
    const double vy = fo * double(CYk(ko)) - fi * double(CYk(ki));
    sx += vx;
    sy += vy;
    st += a.arm[2 * i] * vy - a.arm[2 * i + 1] * vx;
  }
  red[0][threadIdx.x] = sx;
  red[1][threadIdx.x] = sy;
  red[2][threadIdx.x] = st;
  __syncthreads();
#pragma unroll
  for (int h = kForceBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 3) a.out[grp * 3 + threadIdx.x] = red[threadIdx.x][0];
}

}  // namespace lbm
