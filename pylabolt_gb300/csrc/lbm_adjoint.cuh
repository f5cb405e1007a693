// Discrete adjoint of the fused fluidLB step (BGK, Guo forcing none / linear /
// second order; links PULL, ZERO, BB, MBB).
//
// Notation: f^t = incoming populations of step t (the reference's pop_new
// after step t-1), p_t = C(f^t) the post-collision populations (device state),
// f^{t+1} = S(p_t) stream + boundary links.  a^t = dL/df^t.
//
// One reverse step t (this kernel, one thread per node n):
//   1. recompute f^t(n) from p_{t-1} exactly as the forward step pulls it;
//   2. A = S^T a^{t+1}: the transpose of the pull, i.e. the adjoints of the
//      nodes/directions that read p_t(n)_m -- node n + c_m for a bulk node,
//      the recorded reader and/or the node itself (bounce-back) for a
//      boundary node;
//   3. a^t(n) = J_C(f^t(n))^T A (reverse mode through rho, u, f_eq and the
//      Guo source) plus, for moving-wall links, the dependence of
//      f^{t+1}(n)_k on rho^t(n), plus at t = T the loss term dL/du^T;
//   4. accumulates dL/dF(n) (body-force field), dL/domega and dL/du_wall.
#pragma once
#include "lbm_kernels.cuh"

// Resident 256-thread blocks per SM asked of ptxas.  The kernel is latency
// bound: 4 blocks (64 registers, no spills) for the FP32 adjoint; the FP64
// adjoint spills below 128 registers, so 2.
#ifndef LBM_ADJ_MIN_BLOCKS
#define LBM_ADJ_MIN_BLOCKS 4
#endif

namespace lbm {

template <class S, int FORC>
__global__ void __launch_bounds__(256, sizeof(typename Store<S>::T) == 4 ? LBM_ADJ_MIN_BLOCKS : 2)
    adjoint_kernel(const AdjArgs a) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  const Geom& g = a.g;
  const Params& p = a.p;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  T red[3] = {0, 0, 0};
  // this warp's running sums, fetched before the node's loads so that the
  // read-modify-write at the end costs no extra memory round trip
  const int lane = threadIdx.x & 31;
  const long long slot = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * (blockDim.x >> 5) +
                         (threadIdx.x >> 5);
  double run[3] = {0, 0, 0};
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 3; ++i) run[i] = a.gpart[slot * 4 + i];
  }
  if (x < g.nx) {
    const long long n = g.node(x, y);
    const int cls = g.cls[n];
    if (cls < 2) {
      const S* __restrict__ fin = static_cast<const S*>(a.fprev);
      const T* __restrict__ an = static_cast<const T*>(a.a_next);
      T* __restrict__ ac = static_cast<T*>(a.a_cur);
      const int r = cls == 1 ? g.recmap[n] : -1;
      T gF0 = T(0), gF1 = T(0);   // running dL/dF of this node, fetched early
      if (a.gF) {
        const T* gF = static_cast<const T*>(a.gF);
        gF0 = gF[n];
        gF1 = gF[g.plane + n];
      }
      // ---- 1. f^t(n): physical deviations g (shifted) or f (FP64)
      T f[9];
      if (a.nopull) {
#pragma unroll
        for (int k = 0; k < 9; ++k) f[k] = Store<S>::ld(fin, k * g.plane + n, p);
      } else if (cls == 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k)
          f[k] = Store<S>::ld(fin, k * g.plane + n - CYk(k) * g.pitch - CXk(k), p);
      } else {
        const T* side = static_cast<const T*>(a.side_prev);
        f[0] = Store<S>::ld(fin, n, p);
        f[1] = special_link<1, S>(g, p, fin, n, r, side);
        f[2] = special_link<2, S>(g, p, fin, n, r, side);
        f[3] = special_link<3, S>(g, p, fin, n, r, side);
        f[4] = special_link<4, S>(g, p, fin, n, r, side);
        f[5] = special_link<5, S>(g, p, fin, n, r, side);
        f[6] = special_link<6, S>(g, p, fin, n, r, side);
        f[7] = special_link<7, S>(g, p, fin, n, r, side);
        f[8] = special_link<8, S>(g, p, fin, n, r, side);
      }
      // ---- forward quantities
      T rho, drho, jx, jy;
      moments<SH>(f, rho, drho, jx, jy);
      // FP32 constants come pre-converted (an FP64 -> FP32 conversion per
      // thread would run on GB300's slow FP64 pipe)
      const T i2 = SH ? T(p.f_i2) : T(p.inv_cs_2), i4 = SH ? T(p.f_i4) : T(p.inv_cs_4);
      const T om = SH ? T(p.f_omega) : T(p.omega), omh = SH ? T(p.f_homh) : T(p.one_m_half_omega);
      T Fx = T(0), Fy = T(0), dFx = T(0), dFy = T(0);  // dF = dF/drho
      if (FORC != 0) {
        if (a.body) {
          const T* body = static_cast<const T*>(a.body);
          Fx = body[n];
          Fy = body[g.plane + n];
        } else {
          dFx = SH ? T(p.f_gx) : T(p.gx);
          dFy = SH ? T(p.f_gy) : T(p.gy);
          Fx = rho * dFx;
          Fy = rho * dFy;
        }
      }
      const T inv_rho = T(1) / rho;
      const T ux = (jx + T(0.5) * Fx) * inv_rho;
      const T uy = (jy + T(0.5) * Fy) * inv_rho;
      const T u2 = ux * ux + uy * uy;
      // ---- 2. A = S^T a^{t+1}
      T A[9];
#pragma unroll
      for (int m = 0; m < 9; ++m) A[m] = T(0);
      if (an) {
        if (cls == 0) {
#pragma unroll
          for (int m = 0; m < 9; ++m)
            A[m] = an[m * g.plane + n + CYk(m) * g.pitch + CXk(m)];
        } else {
#pragma unroll
          for (int m = 0; m < 9; ++m) {
            const int rdr = a.tr_reader[r * 9 + m];
            T v = rdr >= 0 ? an[m * g.plane + rdr] : T(0);
            if (a.tr_self[r * 9 + m]) v += an[INVk(m) * g.plane + n];
            A[m] = v;
          }
        }
      }
      // ---- 3. reverse mode through the collision, through the moments of A:
      // every sum over k below is sum_k A_k w_k P(c_k) with P of degree <= 2,
      // i.e. a combination of M0 = sum A w, Mc = sum A w c, Mcc = sum A w c c.
      const T w1 = T(1.0 / 9.0), w2 = T(1.0 / 36.0);
      const T d13 = A[1] - A[3], d24 = A[2] - A[4];
      const T s13 = A[1] + A[3], s24 = A[2] + A[4];
      const T s5678 = (A[5] + A[7]) + (A[6] + A[8]);
      const T M0 = T(4.0 / 9.0) * A[0] + w1 * (s13 + s24) + w2 * s5678;
      const T Mx = w1 * d13 + w2 * ((A[5] - A[7]) + (A[8] - A[6]));
      const T My = w1 * d24 + w2 * ((A[5] - A[7]) + (A[6] - A[8]));
      const T Mxx = w1 * s13 + w2 * s5678;
      const T Myy = w1 * s24 + w2 * s5678;
      const T Mxy = w2 * ((A[5] + A[7]) - (A[6] + A[8]));
      const T uMc = ux * Mx + uy * My;
      const T Mccux = Mxx * ux + Mxy * uy, Mccuy = Mxy * ux + Myy * uy;   // Mcc u
      const T uMccu = ux * Mccux + uy * Mccuy;
      // sum_k A_k f_eq,k = rho B,  B = sum_k A_k w_k E_k
      const T Bm1 = -T(0.5) * i2 * u2 * M0 + i2 * uMc + T(0.5) * i4 * uMccu;   // B - M0
      T adj_rho = om * (M0 + Bm1);
      T adj_ux = om * rho * (i2 * Mx + i4 * Mccux - i2 * ux * M0);
      T adj_uy = om * rho * (i2 * My + i4 * Mccuy - i2 * uy * M0);
      T adj_Fx = T(0), adj_Fy = T(0);
      // sum_k A_k (f_eq,k - f_k): in shifted storage f = g + w, so
      // rho B - sum A f = M0 drho + rho (B - M0) - sum A g (no cancellation)
      T sAf = T(0);
#pragma unroll
      for (int k = 0; k < 9; ++k) sAf += A[k] * f[k];
      T g_om = SH ? M0 * drho + rho * Bm1 - sAf : rho * (M0 + Bm1) - sAf;
      if (FORC == 1) {
        const T sAF = i2 * (Mx * Fx + My * Fy);          // sum A Fbar
        g_om -= T(0.5) * sAF;
        adj_Fx += omh * i2 * Mx;
        adj_Fy += omh * i2 * My;
      } else if (FORC == 2) {
        const T uF = ux * Fx + uy * Fy;
        const T MccFx = Mxx * Fx + Mxy * Fy, MccFy = Mxy * Fx + Myy * Fy;
        const T sAF = i2 * (Mx * Fx + My * Fy) - i2 * M0 * uF + i4 * (ux * MccFx + uy * MccFy);
        g_om -= T(0.5) * sAF;
        adj_Fx += omh * (i2 * Mx - i2 * M0 * ux + i4 * Mccux);
        adj_Fy += omh * (i2 * My - i2 * M0 * uy + i4 * Mccuy);
        adj_ux += omh * (-i2 * M0 * Fx + i4 * MccFx);
        adj_uy += omh * (-i2 * M0 * Fy + i4 * MccFy);
      }
      if (a.grad_u) {  // loss term: dL/du^T of this node
        adj_ux += T(a.grad_u[n]);
        adj_uy += T(a.grad_u[g.plane + n]);
      }
      // u = (j + F/2) / rho
      const T adj_jx = adj_ux * inv_rho, adj_jy = adj_uy * inv_rho;
      adj_Fx += T(0.5) * adj_ux * inv_rho;
      adj_Fy += T(0.5) * adj_uy * inv_rho;
      adj_rho -= (adj_ux * ux + adj_uy * uy) * inv_rho;
      if (FORC != 0 && !a.body) adj_rho += adj_Fx * dFx + adj_Fy * dFy;  // F = rho g
      // moving-wall links of this node: f^{t+1}(n)_k = p_t(n)_kbar - 2 w i2 rho^t (c_kbar . u_w)
      T mbb = T(0), guw_x = T(0), guw_y = T(0);
      if (r >= 0 && an) {
        const bool wall = a.wall_rec[r] != 0;
#pragma unroll
        for (int k = 1; k < 9; ++k) {
          if (g.rtype[r * 9 + k] != LINK_MBB) continue;
          const int kb = INVk(k);
          const T coef = -T(2.0 * Wk(kb)) * i2;
          const T ak = an[k * g.plane + n];
          mbb += coef * T(g.rparam[r * 9 + k]) * ak;
          if (wall) {
            guw_x += coef * rho * T(CXk(kb)) * ak;
            guw_y += coef * rho * T(CYk(kb)) * ak;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const T out = (T(1) - om) * A[j] + adj_rho + adj_jx * T(CXk(j)) + adj_jy * T(CYk(j)) + mbb;
        ac[j * g.plane + n] = out;
      }
      if (a.gF) {
        T* gF = static_cast<T*>(a.gF);
        gF[n] = gF0 + adj_Fx;
        gF[g.plane + n] = gF1 + adj_Fy;
      }
      red[0] = g_om;
      red[1] = guw_x;
      red[2] = guw_y;
    }
  }
  // warp sums, accumulated into this warp's slot across reverse steps (fixed
  // slots, so the final sum is deterministic; no block barrier)
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const T v = warp_sum<T>(red[i]);
    if (lane == 0) a.gpart[slot * 4 + i] = run[i] + double(v);
  }
}

}  // namespace lbm
