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

namespace lbm {

template <class S, int FORC>
__global__ void __launch_bounds__(256) adjoint_kernel(const AdjArgs a) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  const Geom& g = a.g;
  const Params& p = a.p;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  T red[3] = {0, 0, 0};
  if (x < g.nx) {
    const long long n = g.node(x, y);
    const int cls = g.cls[n];
    if (cls < 2) {
      const S* __restrict__ fin = static_cast<const S*>(a.fprev);
      const T* __restrict__ an = static_cast<const T*>(a.a_next);
      T* __restrict__ ac = static_cast<T*>(a.a_cur);
      const int r = cls == 1 ? g.recmap[n] : -1;
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
      const T i2 = T(p.inv_cs_2), i4 = T(p.inv_cs_4);
      const T om = T(p.omega), omh = T(p.one_m_half_omega);
      T Fx = T(0), Fy = T(0), dFx = T(0), dFy = T(0);  // dF = dF/drho
      if (FORC != 0) {
        if (a.body) {
          const T* body = static_cast<const T*>(a.body);
          Fx = body[n];
          Fy = body[g.plane + n];
        } else {
          dFx = T(p.gx);
          dFy = T(p.gy);
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
      // ---- 3. reverse mode through the collision
      T adj_rho = T(0), adj_ux = T(0), adj_uy = T(0), adj_Fx = T(0), adj_Fy = T(0);
      T g_om = T(0);
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const T cx = T(CXk(k)), cy = T(CYk(k)), w = T(Wk(k));
        const T cu = cx * ux + cy * uy;
        const T E = T(1) + i2 * cu + T(0.5) * i4 * cu * cu - T(0.5) * i2 * u2;
        const T Ak = A[k];
        // f_eq_k = w rho E ; p_k = f_k + om (f_eq_k - f_k) + omh Fbar_k
        adj_rho += om * Ak * w * E;
        const T dEx = i2 * cx + i4 * cu * cx - i2 * ux;
        const T dEy = i2 * cy + i4 * cu * cy - i2 * uy;
        adj_ux += om * Ak * w * rho * dEx;
        adj_uy += om * Ak * w * rho * dEy;
        // f_eq - f in the stored representation (g_eq - g when shifted)
        const T feq_minus_f = SH ? w * (drho + rho * (E - T(1))) - f[k] : w * rho * E - f[k];
        T Fbar = T(0);
        if (FORC == 1) {
          const T cF = cx * Fx + cy * Fy;
          Fbar = w * i2 * cF;
          adj_Fx += omh * Ak * w * i2 * cx;
          adj_Fy += omh * Ak * w * i2 * cy;
        } else if (FORC == 2) {
          const T cF = cx * Fx + cy * Fy;
          const T ex = (cx - ux) * i2 + cu * cx * i4;
          const T ey = (cy - uy) * i2 + cu * cy * i4;
          Fbar = w * (ex * Fx + ey * Fy);
          adj_Fx += omh * Ak * w * ex;
          adj_Fy += omh * Ak * w * ey;
          // d Fbar / du = w (-i2 F + i4 (c.F) c)
          adj_ux += omh * Ak * w * (-i2 * Fx + i4 * cF * cx);
          adj_uy += omh * Ak * w * (-i2 * Fy + i4 * cF * cy);
        }
        g_om += Ak * (feq_minus_f - T(0.5) * Fbar);
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
        gF[n] += adj_Fx;
        gF[g.plane + n] += adj_Fy;
      }
      red[0] = g_om;
      red[1] = guw_x;
      red[2] = guw_y;
    }
  }
  // block sums, accumulated into this block's slot across reverse steps
  __shared__ double sh[32][3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const T v = warp_sum<T>(red[i]);
    if (lane == 0) sh[wid][i] = double(v);
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w][threadIdx.x];
    a.gpart[((long long)blockIdx.y * gridDim.x + blockIdx.x) * 4 + threadIdx.x] += s;
  }
}

}  // namespace lbm
