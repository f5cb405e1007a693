// Fused D2Q9 fluidLB step for sm_103a: pull-stream + boundary links + moments
// + (BGK | MRT) collision with (none | Guo linear | Guo second order) forcing,
// optional moment output and FP64 residual partial sums, in one launch.
//
// One launch of step_kernel advances the device state from the post-collision
// populations of step t-1 to those of step t.  Relative to the reference's
// Solver.single_time_step (pylabolt/solvers/fluidLB.py:206-253) it performs
// [stream + boundaries of step t-1] followed by [density, force, velocity,
// collide of step t]; the moments it computes are the ones the reference holds
// after step t.  Boundary rules that read moments of step t-1 (moving walls,
// moving solids, anti-bounce-back) read them from a small side array that the
// previous launch wrote for every boundary ("special") node.
//
// Storage:
//   double : f in FP64; arithmetic follows the reference kernels' operation
//            order literally (compile this instantiation with --fmad=false) so
//            results are bit-identical to the reference CPU kernels.
//   float  : g = f - w_i in FP32, FP32 arithmetic (shifted populations).
//   __half : g * scale in FP16, FP32 arithmetic.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "lbm_internal.h"

namespace lbm {

__host__ __device__ constexpr int CXk(int k) {
  return (k == 1 || k == 5 || k == 8) ? 1 : ((k == 3 || k == 6 || k == 7) ? -1 : 0);
}
__host__ __device__ constexpr int CYk(int k) {
  return (k == 2 || k == 5 || k == 6) ? 1 : ((k == 4 || k == 7 || k == 8) ? -1 : 0);
}
__host__ __device__ constexpr int INVk(int k) {
  return k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4) + 1 : ((k - 3) % 4) + 5);
}
// D2Q9 weights 4/9, 1/9, 1/36 (FP64 values of pylabolt/base/lattice.py:54-57)
__host__ __device__ constexpr double Wk(int k) {
  return k == 0 ? 4.0 / 9.0 : (k <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
}
static_assert(INVk(1) == 3 && INVk(2) == 4 && INVk(3) == 1 && INVk(4) == 2 &&
                  INVk(5) == 7 && INVk(6) == 8 && INVk(7) == 5 && INVk(8) == 6,
              "inverse directions");

enum : int { LINK_PULL = 0, LINK_ZERO = 1, LINK_BB = 2, LINK_MBB = 3, LINK_ABB = 4 };

// A*x + B*y for A,B in {-1,0,1}, IEEE-identical to the reference's
// float(A)*x + float(B)*y: a zero coefficient contributes a signed zero that
// does not change a non-zero sum, +-1 products are exact.
template <int A, int B, class T>
__device__ __forceinline__ T lin2(T x, T y) {
  if (A == 0 && B == 0) return T(0);
  if (A == 0) return B > 0 ? y : -y;
  if (B == 0) return A > 0 ? x : -x;
  T ax = A > 0 ? x : -x;
  return B > 0 ? ax + y : ax - y;
}

// ---------------------------------------------------------------------------
// storage traits
template <class S> struct Store;
template <> struct Store<double> {
  using T = double;
  static constexpr bool shifted = false;
  static constexpr bool scaled = false;
  __device__ static __forceinline__ T ldr(const double* __restrict__ p, long long i) { return p[i]; }
  __device__ static __forceinline__ void str(double* __restrict__ p, long long i, T v) { p[i] = v; }
  __device__ static __forceinline__ T ld(const double* __restrict__ p, long long i, const Params&) {
    return p[i];
  }
  __device__ static __forceinline__ void st(double* __restrict__ p, long long i, T v, const Params&) {
    p[i] = v;
  }
};
template <> struct Store<float> {
  using T = float;
  static constexpr bool shifted = true;
  static constexpr bool scaled = false;
  __device__ static __forceinline__ T ldr(const float* __restrict__ p, long long i) { return p[i]; }
  __device__ static __forceinline__ void str(float* __restrict__ p, long long i, T v) { p[i] = v; }
  __device__ static __forceinline__ T ld(const float* __restrict__ p, long long i, const Params&) {
    return p[i];
  }
  __device__ static __forceinline__ void st(float* __restrict__ p, long long i, T v, const Params&) {
    p[i] = v;
  }
};
// FP16 stores g * scale; ldr/str move the stored (scaled) value, ld/st the
// physical g.
template <> struct Store<__half> {
  using T = float;
  static constexpr bool shifted = true;
  static constexpr bool scaled = true;
  __device__ static __forceinline__ T ldr(const __half* __restrict__ p, long long i) {
    return __half2float(p[i]);
  }
  __device__ static __forceinline__ void str(__half* __restrict__ p, long long i, T v) {
    p[i] = __float2half_rn(v);
  }
  __device__ static __forceinline__ T ld(const __half* __restrict__ p, long long i, const Params& q) {
    return __half2float(p[i]) * q.f_inv_scale;
  }
  __device__ static __forceinline__ void st(__half* __restrict__ p, long long i, T v, const Params& q) {
    p[i] = __float2half_rn(v * q.f_scale);
  }
};

// ---------------------------------------------------------------------------
// FP64, reference operation order (collision_kernels.py:5-153,
// compute_fields_kernels.py:5-65, force_field_kernels.py:5-25).
template <int K, int FORC>
__device__ __forceinline__ double bgk_ref_k(double fk, double rho, double ux,
                                            double uy, double hu2, double Fx,
                                            double Fy, const Params& p) {
  constexpr int cx = CXk(K), cy = CYk(K);
  const double cu = lin2<cx, cy>(ux, uy);
  double e;
  if (cx == 0 && cy == 0)
    e = 1.0 - hu2;
  else
    e = ((1.0 + p.inv_cs_2 * cu) + (p.half_inv_cs_4 * cu) * cu) - hu2;
  const double pop_eq = (Wk(K) * rho) * e;
  double out = p.one_m_omega * fk + p.omega * pop_eq;
  if (FORC == 1) {
    if (cx != 0 || cy != 0) {
      const double ft = (Wk(K) * lin2<cx, cy>(Fx, Fy)) * p.inv_cs_2;
      out = out + p.one_m_half_omega * ft;
    }
  } else if (FORC == 2) {
    double const_x, const_y;
    if (cx == 0)
      const_x = (-ux) * p.inv_cs_2;
    else
      const_x = (double(cx) - ux) * p.inv_cs_2 + (cx > 0 ? cu : -cu) * p.inv_cs_4;
    if (cy == 0)
      const_y = (-uy) * p.inv_cs_2;
    else
      const_y = (double(cy) - uy) * p.inv_cs_2 + (cy > 0 ? cu : -cu) * p.inv_cs_4;
    const double ft = Wk(K) * (const_x * Fx + const_y * Fy);
    out = out + p.one_m_half_omega * ft;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Moments.  FP64: reference order.  Shifted: deviation sums.
template <bool SHIFTED, class T>
__device__ __forceinline__ void moments(const T f[9], T& rho, T& drho, T& jx,
                                        T& jy) {
  if (!SHIFTED) {
    T s = f[0];
#pragma unroll
    for (int k = 1; k < 9; ++k) s = s + f[k];
    rho = s;
    drho = s;
    jx = ((((f[1] - f[3]) + f[5]) - f[6]) - f[7]) + f[8];
    jy = ((((f[2] - f[4]) + f[5]) + f[6]) - f[7]) - f[8];
  } else {
    drho = ((f[0] + (f[1] + f[3])) + (f[2] + f[4])) + ((f[5] + f[7]) + (f[6] + f[8]));
    rho = T(1) + drho;
    jx = ((f[1] - f[3]) + (f[5] - f[7])) + (f[8] - f[6]);
    jy = ((f[2] - f[4]) + (f[5] - f[7])) + (f[6] - f[8]);
  }
}

// Shifted BGK: g* = g + omega (g_eq - g) + (1 - omega/2) Fbar, with
// g_eq = w (drho + rho (3 cu + 4.5 cu^2 - 1.5 u^2)).
template <int K, int FORC, class T>
__device__ __forceinline__ T bgk_shift_k(T gk, T rho, T drho, T ux, T uy,
                                         T u2, T Fx, T Fy, T omega, T omh) {
  constexpr int cx = CXk(K), cy = CYk(K);
  const T w = T(Wk(K));
  const T cu = lin2<cx, cy>(ux, uy);
  const T geq = w * (drho + rho * (T(3) * cu + T(4.5) * cu * cu - T(1.5) * u2));
  T out = gk + omega * (geq - gk);
  if (FORC == 1) {
    if (cx != 0 || cy != 0) out += omh * (w * T(3) * lin2<cx, cy>(Fx, Fy));
  } else if (FORC == 2) {
    const T ex = (T(cx) - ux) * T(3) + T(9) * cu * T(cx);
    const T ey = (T(cy) - uy) * T(3) + T(9) * cu * T(cy);
    out += omh * (w * (ex * Fx + ey * Fy));
  }
  return out;
}

// Shifted BGK on stored values G = scale * g (scale 1 for FP32 storage),
// written over the opposite-direction pairs (k, kbar): with
// A = drho - 1.5 rho u^2 and C = 3 rho (c_k . u), the equilibrium deviations are
// g_eq,k = w (A + 1.5 C (c_k . u) + C) and g_eq,kbar = w (A + 1.5 C (c_k . u) - C).
// The update is g* = g + omega d with d = g_eq - g: adding the small
// relaxation term to g rounds far less than (1 - omega) g + omega g_eq, whose
// two large products drift the FP32 state over long runs.
//
// Exact conservation.  In exact arithmetic sum_k d_k = 0 and sum_k c_k d_k =
// F/2 (the half-force shift of u).  Their FP32 values differ by a few units
// in the last place of g_eq, and as the flow changes slowly the same defect
// repeats every step: mass and momentum drift linearly in time (the 8192x2048
// cylinder reaches 3.4e-5 relative velocity error against FP64 after 10^4
// steps).  So the diagonal pairs (5,7), (6,8) are relaxed as computed, the
// axis pairs (1,3), (2,4) keep their computed sum but take the difference that
// makes the x / y momentum change exactly F/2, and d_0 is minus the sum of the
// others: the FP32 relaxation then conserves what the stored populations hold
// (error 1.3e-7 after 10^4 steps, flat in time).  The adjustments are of the
// size of the rounding defect, so the scheme is the same to first order.
//
// FP16 storage skips this (PROJ = false): its storage rounding, not the
// arithmetic, sets its error.
//
// The Guo source (times 1 - omega/2) is split the same way into its even and
// odd parts.
template <int FORC, bool PROJ>
__device__ __forceinline__ void bgk_shift_pairs(float G[9], float rho, float drho, float ux,
                                                float uy, float Fx, float Fy, const Params& p,
                                                float om) {
  const float A = drho - 1.5f * rho * (ux * ux + uy * uy);
  const float r3 = 3.f * rho;
  const float cus[4] = {ux, uy, ux + uy, uy - ux};
  const int ks[4] = {1, 2, 5, 6};
  const int kbs[4] = {3, 4, 7, 8};
  if (!PROJ) {
    G[0] = fmaf(om, fmaf(p.f_wsc[0], A, -G[0]), G[0]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float q = p.f_wsc[j < 2 ? 1 : 2];
      const float C = r3 * cus[j];
      const float S = A + 1.5f * C * cus[j];
      G[ks[j]] = fmaf(om, fmaf(q, S + C, -G[ks[j]]), G[ks[j]]);
      G[kbs[j]] = fmaf(om, fmaf(q, S - C, -G[kbs[j]]), G[kbs[j]]);
    }
  } else {
    float m = 0.f, sx = 0.f, sy = 0.f;   // sums of the diagonal relaxation terms
#pragma unroll
    for (int j = 2; j < 4; ++j) {
      const float q = p.f_wsc[2];
      const float C = r3 * cus[j];
      const float S = A + 1.5f * C * cus[j];
      const float dk = fmaf(q, S + C, -G[ks[j]]);
      const float dkb = fmaf(q, S - C, -G[kbs[j]]);
      m += dk + dkb;
      const float df = dk - dkb;          // (5,7): c = (1,1); (6,8): c = (-1,1)
      sx += j == 2 ? df : -df;
      sy += df;
      G[ks[j]] = fmaf(om, dk, G[ks[j]]);
      G[kbs[j]] = fmaf(om, dkb, G[kbs[j]]);
    }
    // exact momentum changes of the relaxation: scale F / 2
    const float hx = FORC != 0 ? 0.5f * p.f_scale * Fx : 0.f;
    const float hy = FORC != 0 ? 0.5f * p.f_scale * Fy : 0.f;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float q = p.f_wsc[1];
      const float C = r3 * cus[j];
      const float S = A + 1.5f * C * cus[j];
      const float sum = fmaf(q, S + C, -G[ks[j]]) + fmaf(q, S - C, -G[kbs[j]]);
      const float dif = (j == 0 ? hx - sx : hy - sy);
      m += sum;
      G[ks[j]] = fmaf(om, 0.5f * (sum + dif), G[ks[j]]);
      G[kbs[j]] = fmaf(om, 0.5f * (sum - dif), G[kbs[j]]);
    }
    G[0] = fmaf(om, -m, G[0]);
  }
  if (FORC != 0) {
    const float cfs[4] = {Fx, Fy, Fx + Fy, Fy - Fx};
    const float uF = ux * Fx + uy * Fy;
    // (1 - omega/2) w scale; recomputed when omega comes from a map
    const float hs = om == p.f_omega ? 1.f : (1.f - 0.5f * om) / (1.f - 0.5f * p.f_omega);
    if (FORC == 2) G[0] += hs * p.f_omh[0] * (-3.f * uF);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float h = hs * p.f_omh[j < 2 ? 1 : 2];
      const float O = 3.f * cfs[j];
      const float E = FORC == 2 ? 9.f * cus[j] * cfs[j] - 3.f * uF : 0.f;
      G[ks[j]] += h * (E + O);
      G[kbs[j]] += h * (E - O);
    }
  }
}

// MRT (project definition; the reference declares MRT without a kernel,
// pylabolt/base/collision_operator.py:136-165).  Moment basis M of
// collision_operator.py:147-157, S = diag(1, s_e, s_eps, 1, s_q, 1, s_q, s_nu,
// s_nu), equilibrium moments M f_eq and Guo source moments M Fbar in closed form
// for general inv_cs_2 (i2) / inv_cs_4 (i4).  Works on f (FP64) or on
// g = f - w (shifted; M w = (1,-2,1,0,...)).
template <int FORC, bool SHIFTED, class T>
__device__ __forceinline__ void mrt_collide(T f[9], T rho, T drho, T ux, T uy,
                                            T Fx, T Fy, const Params& p) {
  const T i2 = T(p.inv_cs_2), i4 = T(p.inv_cs_4);
  const T s_e = T(p.s_e), s_eps = T(p.s_eps), s_q = T(p.s_q), s_nu = T(p.s_nu);
  const T a14 = f[1] + f[2] + f[3] + f[4];
  const T a58 = f[5] + f[6] + f[7] + f[8];
  T m[9];
  m[0] = f[0] + a14 + a58;
  m[1] = T(-4) * f[0] - a14 + T(2) * a58;
  m[2] = T(4) * f[0] - T(2) * a14 + a58;
  m[3] = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
  m[4] = T(-2) * f[1] + T(2) * f[3] + f[5] - f[6] - f[7] + f[8];
  m[5] = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
  m[6] = T(-2) * f[2] + T(2) * f[4] + f[5] + f[6] - f[7] - f[8];
  m[7] = f[1] - f[2] + f[3] - f[4];
  m[8] = f[5] - f[6] + f[7] - f[8];
  const T u2 = ux * ux + uy * uy;
  const T third_i2 = i2 / T(3), ninth_i4 = i4 / T(9);
  T meq[9];
  // equilibrium moments; shifted form subtracts M w = (1, -2, 1, 0, ...)
  // shifted: rho_eq - 1 = drho - ..., never (1 + drho) - 1, which would round
  // the mass deviation to the FP32 spacing of 1
  meq[0] = (SHIFTED ? drho : rho) - rho * ((T(3) * i2 - i4) / T(6)) * u2;
  meq[1] = SHIFTED ? (T(-2) * drho + rho * i2 * u2) : rho * (i2 * u2 - T(2));
  meq[2] = SHIFTED ? (drho - rho * ((T(3) * i2 + i4) / T(6)) * u2)
                   : rho - rho * ((T(3) * i2 + i4) / T(6)) * u2;
  meq[3] = third_i2 * rho * ux;
  meq[4] = -meq[3];
  meq[5] = third_i2 * rho * uy;
  meq[6] = -meq[5];
  meq[7] = ninth_i4 * rho * (ux * ux - uy * uy);
  meq[8] = ninth_i4 * rho * ux * uy;
  T mf[9] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
  if (FORC != 0) {
    mf[3] = third_i2 * Fx;
    mf[4] = -mf[3];
    mf[5] = third_i2 * Fy;
    mf[6] = -mf[5];
  }
  if (FORC == 2) {
    const T uF = Fx * ux + Fy * uy;
    mf[0] = -((T(3) * i2 - i4) / T(3)) * uF;
    mf[1] = T(2) * i2 * uF;
    mf[2] = -((T(3) * i2 + i4) / T(3)) * uF;
    mf[7] = T(2) * ninth_i4 * (Fx * ux - Fy * uy);
    mf[8] = ninth_i4 * (Fx * uy + Fy * ux);
  }
  const T S[9] = {T(1), s_e, s_eps, T(1), s_q, T(1), s_q, s_nu, s_nu};
  T a[9];
  const T inv_norm[9] = {T(1) / T(9), T(1) / T(36), T(1) / T(36), T(1) / T(6),
                         T(1) / T(12), T(1) / T(6), T(1) / T(12), T(1) / T(4),
                         T(1) / T(4)};
#pragma unroll
  for (int i = 0; i < 9; ++i)
    a[i] = (m[i] - S[i] * (m[i] - meq[i]) + (T(1) - T(0.5) * S[i]) * mf[i]) * inv_norm[i];
  // f = M^T diag(1/|row|^2) m*
  const T b = a[0] - a[1] - T(2) * a[2];
  const T c = a[0] + T(2) * a[1] + a[2];
  f[0] = a[0] - T(4) * a[1] + T(4) * a[2];
  f[1] = b + a[3] - T(2) * a[4] + a[7];
  f[2] = b + a[5] - T(2) * a[6] - a[7];
  f[3] = b - a[3] + T(2) * a[4] + a[7];
  f[4] = b - a[5] + T(2) * a[6] - a[7];
  f[5] = c + a[3] + a[4] + a[5] + a[6] + a[8];
  f[6] = c - a[3] - a[4] + a[5] + a[6] - a[8];
  f[7] = c - a[3] - a[4] - a[5] - a[6] + a[8];
  f[8] = c + a[3] + a[4] - a[5] - a[6] - a[8];
}

// ---------------------------------------------------------------------------
// Incoming population of direction K at a boundary node (record r).
template <int K, class S>
__device__ __forceinline__ typename Store<S>::T special_link(
    const Geom& g, const Params& p, const S* __restrict__ fin, long long n, int r,
    const typename Store<S>::T* __restrict__ side) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  constexpr int KB = INVk(K);
  const int li = r * 9 + K;
  const int type = g.rtype[li];
  if (type == LINK_PULL) return Store<S>::ld(fin, K * g.plane + g.rsrc[li], p);
  if (type == LINK_ZERO) return SH ? T(-Wk(K)) : T(0);
  const T raw = Store<S>::ld(fin, KB * g.plane + n, p);
  if (type == LINK_BB) return raw;
  if (type == LINK_MBB) {
    // streaming_kernels.py:41-47 / fluid_boundary_kernels.py:54-62:
    // raw - 2 w rho inv_cs_2 (c_kbar . u)
    const T rho = side[3 * r];
    if (!SH)
      return raw - ((T(2.0 * Wk(KB)) * rho) * T(p.inv_cs_2)) * T(g.rparam[li]);
    return raw - (T(2.0 * Wk(KB)) * rho * T(3)) * g.rpf[li].x;
  }
  // LINK_ABB -- fluid_boundary_kernels.py:100-152
  const int ra = g.raux[li];
  const T ux = side[3 * r + 1], uy = side[3 * r + 2];
  const T uex = ux + T(0.5) * (ux - side[3 * ra + 1]);
  const T uey = uy + T(0.5) * (uy - side[3 * ra + 2]);
  const T u2 = uex * uex + uey * uey;
  const T cu = lin2<CXk(KB), CYk(KB)>(uex, uey);
  T rho_w;
  if constexpr (SH)
    rho_w = g.rpf[li].x;
  else
    rho_w = g.rparam[li];
  if (!SH) {
    const T temp = (T(2.0 * Wk(KB)) * rho_w) *
                   ((T(1) + (T(p.half_inv_cs_4) * cu) * cu) - T(p.half_inv_cs_2) * u2);
    return -raw + temp;
  }
  // rho_w - 1 is formed in FP64 (on the host, rpf.y): rounding rho_w itself
  // to FP32 would shift the imposed density difference by up to 6e-8
  // absolute.
  const T drho_w = g.rpf[li].y;
  return -raw + T(2.0 * Wk(KB)) * (drho_w + rho_w * (T(4.5) * cu * cu - T(1.5) * u2));
}

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// MRT on shifted storage in delta form: G* = G + M^-1 dm, in stored units
// G = scale * g, with the D2Q9 constants (inv_cs_2 = 3, inv_cs_4 = 9; the
// shifted paths always use them).  dm = -S (m - meq) + (1 - S/2) mf on the
// non-conserved moments e, eps, qx, qy, pxx, pxy, and the exact changes of
// the conserved ones: 0 for rho and F for j (meq_j + mf_j / 2 = rho u + F/2 =
// j + F).  Reconstructing G* whole rounds at the scale of G and, as the flow
// changes slowly, the same mass / momentum defect repeats every step (1e-4
// relative velocity drift in 10^4 steps); the correction M^-1 dm is small and
// so is its rounding.  Same moments as mrt_collide, specialised: no
// divisions, no conserved-moment work.
template <int FORC>
__device__ __forceinline__ void mrt_shifted(float G[9], float rho, float drho, float ux,
                                            float uy, float Fx, float Fy, const Params& p) {
  const float sc = p.f_scale;
  const float a13 = G[1] + G[3], a24 = G[2] + G[4];
  const float a14 = a13 + a24;
  const float a57 = G[5] + G[7], a68 = G[6] + G[8];
  const float a58 = a57 + a68;
  const float d57 = G[5] - G[7], d68 = G[6] - G[8];
  const float m_e = fmaf(-4.f, G[0], fmaf(2.f, a58, -a14));
  const float m_eps = fmaf(4.f, G[0], fmaf(-2.f, a14, a58));
  const float m_qx = fmaf(-2.f, G[1] - G[3], d57 - d68);
  const float m_qy = fmaf(-2.f, G[2] - G[4], d57 + d68);
  const float m_xx = a13 - a24;
  const float m_xy = a57 - a68;
  const float rs = rho * sc;
  const float r3u2 = 3.f * rs * (ux * ux + uy * uy);
  const float dr = drho * sc;
  const float eq_e = fmaf(-2.f, dr, r3u2);
  const float eq_eps = dr - r3u2;
  const float eq_qx = -rs * ux, eq_qy = -rs * uy;
  const float eq_xx = rs * (ux * ux - uy * uy), eq_xy = rs * ux * uy;
  float da_e = p.f_mrt_s[0] * (m_e - eq_e);
  float da_eps = p.f_mrt_s[1] * (m_eps - eq_eps);
  float da_qx = p.f_mrt_s[2] * (m_qx - eq_qx);
  float da_qy = p.f_mrt_s[2] * (m_qy - eq_qy);
  float da_xx = p.f_mrt_s[3] * (m_xx - eq_xx);
  float da_xy = p.f_mrt_s[3] * (m_xy - eq_xy);
  float da_jx = 0.f, da_jy = 0.f;
  if (FORC != 0) {
    const float fx = sc * Fx, fy = sc * Fy;
    da_jx = fx * (1.f / 6.f);
    da_jy = fy * (1.f / 6.f);
    da_qx = fmaf(p.f_mrt_h[2], -fx, da_qx);
    da_qy = fmaf(p.f_mrt_h[2], -fy, da_qy);
    if (FORC == 2) {
      const float uF = ux * fx + uy * fy;
      da_e = fmaf(p.f_mrt_h[0], 6.f * uF, da_e);
      da_eps = fmaf(p.f_mrt_h[1], -6.f * uF, da_eps);
      da_xx = fmaf(p.f_mrt_h[3], 2.f * (fx * ux - fy * uy), da_xx);
      da_xy = fmaf(p.f_mrt_h[3], fx * uy + fy * ux, da_xy);
    }
  }
  // G* - G = M^T diag(1/|row|^2) dm
  const float b = fmaf(-2.f, da_eps, -da_e);
  const float c = fmaf(2.f, da_e, da_eps);
  G[0] += 4.f * (da_eps - da_e);
  const float x1 = fmaf(-2.f, da_qx, da_jx), y1 = fmaf(-2.f, da_qy, da_jy);
  G[1] += (b + x1) + da_xx;
  G[3] += (b - x1) + da_xx;
  G[2] += (b + y1) - da_xx;
  G[4] += (b - y1) - da_xx;
  const float x2 = da_jx + da_qx, y2 = da_jy + da_qy;
  G[5] += c + (x2 + y2) + da_xy;
  G[6] += c + (y2 - x2) - da_xy;
  G[7] += c - (x2 + y2) + da_xy;
  G[8] += c + (x2 - y2) - da_xy;
}

// Moments, force, velocity and collision of one node: f holds the incoming
// populations (f, or g = f - w when shifted) and receives the post-collision
// ones.
// `seg` is the node's 32-node row segment (y * nseg + x / 32), used to read a
// per-segment relaxation rate when the case has one (batched cases).
template <class S, int COLL, int FORC>
__device__ __forceinline__ void node_update(typename Store<S>::T f[9], const StepArgs& a,
                                            long long n, typename Store<S>::T& rho,
                                            typename Store<S>::T& ux,
                                            typename Store<S>::T& uy, int seg) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  const Params& p = a.p;
  T drho, jx, jy;
  moments<SH>(f, rho, drho, jx, jy);
  if constexpr (Store<S>::scaled) {
    // f holds G = scale * g: rescale the moments only
    drho *= p.f_inv_scale;
    jx *= p.f_inv_scale;
    jy *= p.f_inv_scale;
    rho = T(1) + drho;
  }
  T Fx = T(0), Fy = T(0);
  if (FORC != 0) {
    if (a.body) {
      const T* body = static_cast<const T*>(a.body);
      Fx = body[n];
      Fy = body[a.g.plane + n];
    } else if constexpr (SH) {
      Fx = rho * p.f_gx;
      Fy = rho * p.f_gy;
    } else {
      Fx = rho * T(p.gx);
      Fy = rho * T(p.gy);
    }
  }
  if constexpr (!SH) {
    // compute_fields_kernels.py:61-65
    const T inv_density = T(1) / (rho + T(p.eps));
    ux = jx * inv_density + (T(0.5) * Fx) * inv_density;
    uy = jy * inv_density + (T(0.5) * Fy) * inv_density;
  } else {
    const T inv_density = __frcp_rn(rho);
    ux = (jx + T(0.5) * Fx) * inv_density;
    uy = (jy + T(0.5) * Fy) * inv_density;
  }
  if constexpr (COLL == 1 && SH) {
    mrt_shifted<FORC>(f, rho, drho, ux, uy, Fx, Fy, p);
  } else if constexpr (COLL == 1) {
    mrt_collide<FORC, false>(f, rho, drho, ux, uy, Fx, Fy, p);
  } else if constexpr (!SH) {
    const T hu2 = T(p.half_inv_cs_2) * (ux * ux + uy * uy);
    f[0] = bgk_ref_k<0, FORC>(f[0], rho, ux, uy, hu2, Fx, Fy, p);
    f[1] = bgk_ref_k<1, FORC>(f[1], rho, ux, uy, hu2, Fx, Fy, p);
    f[2] = bgk_ref_k<2, FORC>(f[2], rho, ux, uy, hu2, Fx, Fy, p);
    f[3] = bgk_ref_k<3, FORC>(f[3], rho, ux, uy, hu2, Fx, Fy, p);
    f[4] = bgk_ref_k<4, FORC>(f[4], rho, ux, uy, hu2, Fx, Fy, p);
    f[5] = bgk_ref_k<5, FORC>(f[5], rho, ux, uy, hu2, Fx, Fy, p);
    f[6] = bgk_ref_k<6, FORC>(f[6], rho, ux, uy, hu2, Fx, Fy, p);
    f[7] = bgk_ref_k<7, FORC>(f[7], rho, ux, uy, hu2, Fx, Fy, p);
    f[8] = bgk_ref_k<8, FORC>(f[8], rho, ux, uy, hu2, Fx, Fy, p);
  } else {
    const float om = a.omega_seg ? a.omega_seg[seg] : p.f_omega;
    bgk_shift_pairs<FORC, !Store<S>::scaled>(f, rho, drho, ux, uy, Fx, Fy, p, om);
  }
}

// Incoming populations of a boundary node from its link record.
template <class S>
__device__ __forceinline__ void special_links(typename Store<S>::T f[9], const StepArgs& a,
                                              const S* __restrict__ fin, long long n, int r) {
  using T = typename Store<S>::T;
  const T* side = static_cast<const T*>(a.side_in);
  f[1] = special_link<1, S>(a.g, a.p, fin, n, r, side);
  f[2] = special_link<2, S>(a.g, a.p, fin, n, r, side);
  f[3] = special_link<3, S>(a.g, a.p, fin, n, r, side);
  f[4] = special_link<4, S>(a.g, a.p, fin, n, r, side);
  f[5] = special_link<5, S>(a.g, a.p, fin, n, r, side);
  f[6] = special_link<6, S>(a.g, a.p, fin, n, r, side);
  f[7] = special_link<7, S>(a.g, a.p, fin, n, r, side);
  f[8] = special_link<8, S>(a.g, a.p, fin, n, r, side);
  if constexpr (Store<S>::scaled) {
#pragma unroll
    for (int k = 1; k < 9; ++k) f[k] *= a.p.f_scale;
  }
}

// lin2 with run-time coefficients in {-1, 0, 1} (same IEEE result).
template <class T>
__device__ __forceinline__ T lin2r(int A, int B, T x, T y) {
  if (A == 0 && B == 0) return T(0);
  if (A == 0) return B > 0 ? y : -y;
  if (B == 0) return A > 0 ? x : -x;
  const T ax = A > 0 ? x : -x;
  return B > 0 ? ax + y : ax - y;
}

// Incoming populations of a node next to a moving obstacle (class 4): pull,
// or moving-solid bounce-back from a source the obstacle covers
// (streaming_kernels.py:41-47; rho of this node from the previous step).
template <class S>
__device__ __forceinline__ void dynamic_links(typename Store<S>::T f[9], const StepArgs& a,
                                              const S* __restrict__ fin, int ni) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  const Geom& g = a.g;
  const Params& p = a.p;
  const T* us = static_cast<const T*>(a.us);
  const T rho = static_cast<const T*>(a.rho_dyn_in)[ni];
#pragma unroll
  for (int k = 1; k < 9; ++k) {
    const int src = ni - CYk(k) * g.pitch - CXk(k);
    const int kb = INVk(k);
    T v;
    if (a.dsolid[src]) {
      const T raw = Store<S>::ld(fin + kb * g.plane, ni, p);
      const T cu = lin2r<T>(CXk(kb), CYk(kb), us[src], us[g.plane + src]);
      v = SH ? raw - (T(2.0 * Wk(kb)) * rho * T(3)) * cu
             : raw - ((T(2.0 * Wk(kb)) * rho) * T(p.inv_cs_2)) * cu;
    } else {
      v = Store<S>::ld(fin + k * g.plane, src, p);
    }
    f[k] = Store<S>::scaled ? v * p.f_scale : v;
  }
}

// Side data, moment output and residual terms of one updated node.  The
// residual terms are formed in the compute type T (FP32 for shifted storage:
// GB300's FP64 rate is a small fraction of its FP32 rate) and summed in FP64
// per block.
// The residual's previous-step fields of node n.
template <class T>
__device__ __forceinline__ void load_old(const StepArgs& a, long long n, T o[3]) {
  o[0] = static_cast<const T*>(a.rho_old)[n];
  o[1] = static_cast<const T*>(a.ux_old)[n];
  o[2] = static_cast<const T*>(a.uy_old)[n];
}

// RES: residual terms when the step's flags ask (RES_FLAG), never (RES_OFF),
// or always with the previous-step fields already loaded in `pre` (RES_ON:
// the scalar kernel's residual instantiation issues those loads with the
// populations', so that their latency overlaps).
enum { RES_FLAG = 0, RES_OFF = 1, RES_ON = 2 };

template <class T, int RES = RES_FLAG>
__device__ __forceinline__ void node_outputs(const StepArgs& a, long long n, int r, T rho,
                                             T ux, T uy, T red[7], const T* pre = nullptr) {
  if (r >= 0) {
    T* side = static_cast<T*>(a.side_out);
    side[3 * r] = rho;
    side[3 * r + 1] = ux;
    side[3 * r + 2] = uy;
  }
  if (a.flags & F_MOMENTS) {
    static_cast<T*>(a.rho)[n] = rho;
    static_cast<T*>(a.ux)[n] = ux;
    static_cast<T*>(a.uy)[n] = uy;
  }
  if (RES == RES_ON || (RES == RES_FLAG && (a.flags & F_RESIDUAL))) {
    // compute_residues_kernels.py:6-73: sums over fluid nodes
    T o[3];
    if (RES == RES_ON) {
      o[0] = pre[0];
      o[1] = pre[1];
      o[2] = pre[2];
    } else {
      load_old<T>(a, n, o);
    }
    const T v[3] = {rho, ux, uy};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T d = v[c] - o[c];
      red[2 * c] += d * d;
      red[2 * c + 1] += o[c] * o[c];
    }
    red[6] += (isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2])) ? T(0) : T(1);
    static_cast<T*>(a.rho_new)[n] = rho;
    static_cast<T*>(a.ux_new)[n] = ux;
    static_cast<T*>(a.uy_new)[n] = uy;
  }
}

// Warp sums of eight values in 9 shuffles instead of 8 x 5: a butterfly in
// which every level halves the values a lane carries (4, 2, 1, then two
// levels on the last one).  Lane l returns the warp sum of value
// (l >> 2) & 7.  The pairing is fixed, so the sums are deterministic.
template <class R>
__device__ __forceinline__ R warp_sum8(const R v[8]) {
  const int lane = threadIdx.x & 31;
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  R a4[4], a2[2];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const R send = b4 ? v[i] : v[i + 4];
    const R keep = b4 ? v[i + 4] : v[i];
    a4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const R send = b3 ? a4[i] : a4[i + 2];
    const R keep = b3 ? a4[i + 2] : a4[i];
    a2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  R c = (b2 ? a2[1] : a2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? a2[0] : a2[1], 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  return c;
}

template <class T>
__device__ __forceinline__ void block_residual(const StepArgs& a, T red[7]) {
  __shared__ double sh[16][8];   // one row per warp: blocks of at most 512 threads
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const T v[8] = {red[0], red[1], red[2], red[3], red[4], red[5], red[6], T(0)};
  const T s = warp_sum8<T>(v);
  if ((lane & 3) == 0) sh[wid][(lane >> 2) & 7] = double(s);
  __syncthreads();
  if (threadIdx.x < 8) {
    double t = 0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) t += sh[w][threadIdx.x];
    a.partials[((long long)blockIdx.y * gridDim.x + blockIdx.x) * 8 + threadIdx.x] = t;
  }
}

// ---------------------------------------------------------------------------
// One node of the scalar kernel.  MOV: the case has moving obstacles
// (class-4 nodes, the density kept for their bounce-back).
template <class S, int COLL, int FORC, bool MOV, bool RES>
__device__ __forceinline__ void step_node(const StepArgs& a, int x, int y,
                                          typename Store<S>::T red[7]) {
  using T = typename Store<S>::T;
  const Geom& g = a.g;
  // 32-bit node index (plane < 2^31 is checked at create).  The bulk pulls
  // and the stores address from this node's element of plane 0 with
  // warp-uniform 64-bit offsets (k * plane - c_k . (1, pitch)): one 64-bit add
  // per access.
  const int ni = (y + 1) * g.pitch + x;
  const long long n = ni;
  const S* __restrict__ fin = static_cast<const S*>(a.fin);
  S* __restrict__ fout = static_cast<S*>(a.fout);
  const S* __restrict__ fn = fin + ni;
  S* __restrict__ on = fout + ni;
  int cls = 0;
  const bool seg = g.segflag[y * g.nseg + (x >> 5)] != 0;
  if (seg) cls = g.cls[ni];
  if (cls == 2) return;
  T old[3];
  if (RES) load_old<T>(a, n, old);
  T f[9];
  int r = -1;
  if (cls == 1) r = g.recmap[ni];
  if (a.flags & F_NOPULL) {
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = Store<S>::ldr(fn, k * g.plane);
  } else if (cls == 0) {
#pragma unroll
    for (int k = 0; k < 9; ++k)
      f[k] = Store<S>::ldr(fn, k * g.plane - (long long)(CYk(k) * g.pitch + CXk(k)));
  } else if (MOV && cls == 4) {
    f[0] = Store<S>::ldr(fin, ni);
    dynamic_links<S>(f, a, fin, ni);
  } else {
    f[0] = Store<S>::ldr(fin, n);
    special_links<S>(f, a, fin, n, r);
  }
  T rho, ux, uy;
  node_update<S, COLL, FORC>(f, a, n, rho, ux, uy, y * g.nseg + (x >> 5));
#pragma unroll
  for (int k = 0; k < 9; ++k) Store<S>::str(on, k * g.plane, f[k]);
  // density of every node of a flagged segment: the segments around a
  // moving obstacle are flagged a step before their nodes can enter class 4,
  // whose bounce-back then reads it
  if (MOV && seg) static_cast<T*>(a.rho_dyn_out)[ni] = rho;
  node_outputs<T, RES ? RES_ON : RES_OFF>(a, n, r, rho, ux, uy, red, old);
}

// Scalar kernel: one node per thread.  Used for FP64 (whose cost is its FP64
// arithmetic, not memory) and as an autotuner candidate.
// CAP = 1 asks for 8 resident blocks of 256 threads (at most 32 registers),
// CAP = 2 for 6 (at most 40 registers; for the MRT collision).  MOV = true:
// the case has moving obstacles (a separate instantiation, so that cases
// without them run the plain body).  RES: the step evaluates the residual
// (F_RESIDUAL); the plain instantiation carries none of its code.
template <class S, int COLL, int FORC, int CAP, bool MOV, bool RES>
__global__ void __launch_bounds__(CAP ? 256 : 512, CAP == 1 ? 8 : (CAP == 2 ? 6 : 1))
    step_kernel(const StepArgs a) {
  using T = typename Store<S>::T;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  T red[7] = {0, 0, 0, 0, 0, 0, 0};
  if (x < a.g.nx) step_node<S, COLL, FORC, MOV, RES>(a, x, y, red);
  if (RES) block_residual<decltype(red[0] + 0)>(a, red);
}

// ---------------------------------------------------------------------------
// AA layout: one population array updated in place (pylabolt_gb300 layout
// LBM_POP_AA).  With off(k) = c_ky * pitch + c_kx:
//   even phase  reads  f_k = A[n][k]                 (the incoming values)
//               writes A[n][kbar] = p_k               (own node, swapped)
//   odd phase   reads  f_k = A[n - off(k)][kbar]      (neighbour's swapped slot)
//               writes A[n + off(k)][k] = p_k         (pushed to the neighbour)
// Every location a thread writes is one only it reads, so the update is in
// place without races.  Link records see the same values as the pull kernel:
//   even  PULL from s: A[s + off(k)][k]   bounce-back raw p_kbar: A[n - off(k)][kbar]
//   odd   PULL from s: A[s][kbar]         bounce-back raw p_kbar: A[n][k]
// (the first step after initialisation reads A[n][k] for every node, like
// the pull kernel's no-pull step).  Pushes beyond the domain edges land in
// the padding rows / columns (pitch >= nx + 2) or the guard rows; the host
// rejects PULL sources whose even-phase location another node would
// overwrite (zero_gradient).
template <int K, class S, bool ODD>
__device__ __forceinline__ typename Store<S>::T special_link_aa(
    const Geom& g, const Params& p, const S* __restrict__ A, long long n, int r,
    const typename Store<S>::T* __restrict__ side) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  constexpr int KB = INVk(K);
  const long long off = (long long)CYk(K) * g.pitch + CXk(K);
  const int li = r * 9 + K;
  const int type = g.rtype[li];
  if (type == LINK_PULL) {
    const long long s = g.rsrc[li];
    return ODD ? Store<S>::ld(A, KB * g.plane + s, p) : Store<S>::ld(A, K * g.plane + s + off, p);
  }
  if (type == LINK_ZERO) return SH ? T(-Wk(K)) : T(0);
  const T raw = ODD ? Store<S>::ld(A, K * g.plane + n, p) : Store<S>::ld(A, KB * g.plane + n - off, p);
  if (type == LINK_BB) return raw;
  if (type == LINK_MBB) {
    const T rho = side[3 * r];
    if (!SH)
      return raw - ((T(2.0 * Wk(KB)) * rho) * T(p.inv_cs_2)) * T(g.rparam[li]);
    return raw - (T(2.0 * Wk(KB)) * rho * T(3)) * g.rpf[li].x;
  }
  const int ra = g.raux[li];
  const T ux = side[3 * r + 1], uy = side[3 * r + 2];
  const T uex = ux + T(0.5) * (ux - side[3 * ra + 1]);
  const T uey = uy + T(0.5) * (uy - side[3 * ra + 2]);
  const T u2 = uex * uex + uey * uey;
  const T cu = lin2<CXk(KB), CYk(KB)>(uex, uey);
  T rho_w;
  if constexpr (SH)
    rho_w = g.rpf[li].x;
  else
    rho_w = g.rparam[li];
  if (!SH) {
    const T temp = (T(2.0 * Wk(KB)) * rho_w) *
                   ((T(1) + (T(p.half_inv_cs_4) * cu) * cu) - T(p.half_inv_cs_2) * u2);
    return -raw + temp;
  }
  const T drho_w = g.rpf[li].y;
  return -raw + T(2.0 * Wk(KB)) * (drho_w + rho_w * (T(4.5) * cu * cu - T(1.5) * u2));
}

template <class S, bool ODD>
__device__ __forceinline__ void special_links_aa(typename Store<S>::T f[9], const StepArgs& a,
                                                 const S* __restrict__ A, long long n, int r) {
  using T = typename Store<S>::T;
  const T* side = static_cast<const T*>(a.side_in);
  f[1] = special_link_aa<1, S, ODD>(a.g, a.p, A, n, r, side);
  f[2] = special_link_aa<2, S, ODD>(a.g, a.p, A, n, r, side);
  f[3] = special_link_aa<3, S, ODD>(a.g, a.p, A, n, r, side);
  f[4] = special_link_aa<4, S, ODD>(a.g, a.p, A, n, r, side);
  f[5] = special_link_aa<5, S, ODD>(a.g, a.p, A, n, r, side);
  f[6] = special_link_aa<6, S, ODD>(a.g, a.p, A, n, r, side);
  f[7] = special_link_aa<7, S, ODD>(a.g, a.p, A, n, r, side);
  f[8] = special_link_aa<8, S, ODD>(a.g, a.p, A, n, r, side);
  if constexpr (Store<S>::scaled) {
#pragma unroll
    for (int k = 1; k < 9; ++k) f[k] *= a.p.f_scale;
  }
}

// One node of the AA kernel (either phase).
template <class S, int COLL, int FORC, bool ODD>
__device__ __forceinline__ void aa_node(const StepArgs& a, int x, int y,
                                        typename Store<S>::T red[7]) {
  using T = typename Store<S>::T;
  const Geom& g = a.g;
  const int ni = (y + 1) * g.pitch + x;
  const long long n = ni;
  S* A = static_cast<S*>(a.fout);   // == a.fin
  S* An = A + ni;                   // this node's element of plane 0 (uniform offsets below)
  int cls = 0;
  if (g.segflag[y * g.nseg + (x >> 5)]) cls = g.cls[ni];
  if (cls == 2) return;
  T f[9];
  int r = -1;
  if (cls == 1) r = g.recmap[ni];
  if (!ODD && ((a.flags & F_NOPULL) || cls == 0)) {
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = Store<S>::ldr(An, k * g.plane);
  } else if (ODD && cls == 0) {
#pragma unroll
    for (int k = 0; k < 9; ++k)
      f[k] = Store<S>::ldr(An, INVk(k) * g.plane - (long long)(CYk(k) * g.pitch + CXk(k)));
  } else {
    f[0] = Store<S>::ldr(A, ni);
    special_links_aa<S, ODD>(f, a, A, n, r);
  }
  T rho, ux, uy;
  node_update<S, COLL, FORC>(f, a, n, rho, ux, uy, y * g.nseg + (x >> 5));
  if (!ODD) {
#pragma unroll
    for (int k = 0; k < 9; ++k) Store<S>::str(An, INVk(k) * g.plane, f[k]);
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k)
      Store<S>::str(An, k * g.plane + (long long)(CYk(k) * g.pitch + CXk(k)), f[k]);
  }
  node_outputs<T>(a, n, r, rho, ux, uy, red);
}

template <class S, int COLL, int FORC, int CAP, bool ODD>
__global__ void __launch_bounds__(CAP ? 256 : 512, CAP == 1 ? 8 : (CAP == 2 ? 6 : 1))
    step_aa_kernel(const StepArgs a) {
  using T = typename Store<S>::T;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  T red[7] = {0, 0, 0, 0, 0, 0, 0};
  if (x < a.g.nx) aa_node<S, COLL, FORC, ODD>(a, x, y, red);
  if (a.flags & F_RESIDUAL) block_residual<decltype(red[0] + 0)>(a, red);
}

// ---------------------------------------------------------------------------
// Node pairs: one thread updates nodes (x0, y) and (x0 + 1, y), x0 even, and
// moves every population plane as one aligned word holding both nodes (two
// halves for FP16 storage, two floats for FP32).  A direction with c_kx = 0
// reads the word at x0 of its source row y - c_ky.  c_kx = +1 needs the
// values at (x0 - 1, x0): the upper half of the word at x0 - 2 and the lower
// half of the word at x0; c_kx = -1 needs (x0 + 1, x0 + 2): the upper half
// of the word at x0 and the lower half of the word at x0 + 2.  The extra
// word is a neighbouring thread's own word, so it comes from L1.  This halves
// the per-node cost of addressing, class checks, loads, stores and the
// float -> half packing, which bound the one-node-per-thread FP16 step (it
// issues as many instructions per node as the FP32 one for half the bytes).
//
// A pair whose 32-node row segment holds any boundary, solid or padding node
// (segflag) takes the per-node scalar path for both nodes, so link records
// are handled exactly as by step_kernel.  On a no-pull step a bulk pair reads
// its own slots as aligned words.
template <class S> struct PairIO;
template <> struct PairIO<__half> {
  using W = uint32_t;
  __device__ static __forceinline__ W ld(const W* __restrict__ p, long long i) { return p[i]; }
  // upper value of word a, lower value of word b
  __device__ static __forceinline__ W mid(W a, W b) { return __byte_perm(a, b, 0x5432); }
  __device__ static __forceinline__ void unpack(W w, float& lo, float& hi) {
    __half2 h;
    memcpy(&h, &w, 4);
    const float2 t = __half22float2(h);
    lo = t.x;
    hi = t.y;
  }
  __device__ static __forceinline__ W pack(float lo, float hi) {
    const __half2 h = __floats2half2_rn(lo, hi);
    W w;
    memcpy(&w, &h, 4);
    return w;
  }
};
template <> struct PairIO<float> {
  using W = float2;
  __device__ static __forceinline__ W ld(const W* __restrict__ p, long long i) { return p[i]; }
  __device__ static __forceinline__ W mid(W a, W b) { return make_float2(a.y, b.x); }
  __device__ static __forceinline__ void unpack(W w, float& lo, float& hi) {
    lo = w.x;
    hi = w.y;
  }
  __device__ static __forceinline__ W pack(float lo, float hi) { return make_float2(lo, hi); }
};

// Incoming word of direction K for the pair at byte offset `nb` of plane 0:
// the word at nb from `base` (the buffer plus the direction's plane and c_ky
// rows, the same for the whole grid), combined with its neighbour for
// c_kx != 0 (both nodes).
template <class S, int K>
__device__ __forceinline__ typename PairIO<S>::W pair_pull(const char* __restrict__ base, uint32_t nb) {
  using IO = PairIO<S>;
  using W = typename IO::W;
  constexpr int cx = CXk(K);
  const W* p = reinterpret_cast<const W*>(base + nb);
  if (cx == 0) return IO::ld(p, 0);
  if (cx == 1) return IO::mid(IO::ld(p, -1), IO::ld(p, 0));
  return IO::mid(IO::ld(p, 0), IO::ld(p, 1));
}

// Moment output and residual terms of a bulk pair (nodes n, n + 1; n even),
// the two nodes' values moved as one 8-byte word per field (node_outputs does
// the same per node).  o2: the previous residual step's fields (RES).
template <bool RES>
__device__ __forceinline__ void pair_outputs(const StepArgs& a, long long n, float rho0, float ux0,
                                             float uy0, float rho1, float ux1, float uy1,
                                             float red[7], const float2 o2[3]) {
  const float2 v[3] = {make_float2(rho0, rho1), make_float2(ux0, ux1), make_float2(uy0, uy1)};
  if (a.flags & F_MOMENTS) {
    *reinterpret_cast<float2*>(static_cast<float*>(a.rho) + n) = v[0];
    *reinterpret_cast<float2*>(static_cast<float*>(a.ux) + n) = v[1];
    *reinterpret_cast<float2*>(static_cast<float*>(a.uy) + n) = v[2];
  }
  if (RES) {
    // compute_residues_kernels.py:6-73: sums over fluid nodes
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float d0 = v[c].x - o2[c].x, d1 = v[c].y - o2[c].y;
      red[2 * c] += d0 * d0;
      red[2 * c] += d1 * d1;
      red[2 * c + 1] += o2[c].x * o2[c].x;
      red[2 * c + 1] += o2[c].y * o2[c].y;
    }
    red[6] += (isfinite(rho0) && isfinite(ux0) && isfinite(uy0)) ? 0.f : 1.f;
    red[6] += (isfinite(rho1) && isfinite(ux1) && isfinite(uy1)) ? 0.f : 1.f;
    *reinterpret_cast<float2*>(static_cast<float*>(a.rho_new) + n) = v[0];
    *reinterpret_cast<float2*>(static_cast<float*>(a.ux_new) + n) = v[1];
    *reinterpret_cast<float2*>(static_cast<float*>(a.uy_new) + n) = v[2];
  }
}

// Collision, stores and outputs of a bulk pair (nodes n, n + 1) from its
// nine incoming words.
template <class S, int COLL, int FORC, bool RES>
__device__ __forceinline__ void pair_finish(const StepArgs& a, long long n, int seg,
                                            const typename PairIO<S>::W w[9],
                                            const float2 o2[3], float red[7]) {
  using IO = PairIO<S>;
  using W = typename IO::W;
  float f0[9], f1[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) IO::unpack(w[k], f0[k], f1[k]);
  float rho0, ux0, uy0, rho1, ux1, uy1;
  node_update<S, COLL, FORC>(f0, a, n, rho0, ux0, uy0, seg);
  node_update<S, COLL, FORC>(f1, a, n + 1, rho1, ux1, uy1, seg);
  // plane base (the same for the whole grid) + the node's 32-bit byte offset
  char* const fo = static_cast<char*>(a.fout);
  const uint32_t nb = (uint32_t)(n * (long long)sizeof(S));
#pragma unroll
  for (int k = 0; k < 9; ++k) *reinterpret_cast<W*>(fo + a.off_plane[k] + nb) = IO::pack(f0[k], f1[k]);
  pair_outputs<RES>(a, n, rho0, ux0, uy0, rho1, ux1, uy1, red, o2);
}

// One pair of the node-pair kernel (row y, nodes x0 and x0 + 1).  MOV: the
// case has moving obstacles; their nodes and the segments around them are
// flagged, so only the per-node path sees them (and records the densities
// their bounce-back reads).
template <class S, int COLL, int FORC, bool RES, bool MOV = false>
__device__ __forceinline__ void pair_step(const StepArgs& a, int x0, int y, float red[7]) {
  using IO = PairIO<S>;
  using W = typename IO::W;
  const Geom& g = a.g;
  const int seg = y * g.nseg + (x0 >> 5);
  if (g.segflag[seg] != 0) {
    step_node<S, COLL, FORC, MOV, RES>(a, x0, y, red);
    if (x0 + 1 < g.nx) step_node<S, COLL, FORC, MOV, RES>(a, x0 + 1, y, red);
    return;
  }
  // both nodes are bulk nodes: every source is inside the grid
  const int ni = (y + 1) * g.pitch + x0;   // even: pitch and x0 are even
  const long long n = ni;
  const char* const fi = static_cast<const char*>(a.fin);
  const uint32_t nb = (uint32_t)ni * (uint32_t)sizeof(S);   // byte offset in a plane
  // the previous residual step's fields of both nodes (n even: 8-byte words)
  float2 o2[3];
  if (RES) {
    o2[0] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.rho_old) + n);
    o2[1] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.ux_old) + n);
    o2[2] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.uy_old) + n);
  }
  W w[9];
  if (a.flags & F_NOPULL) {   // the stored populations are the incoming ones: own slots
#pragma unroll
    for (int k = 0; k < 9; ++k) w[k] = *reinterpret_cast<const W*>(fi + a.off_plane[k] + nb);
  } else {
    w[0] = pair_pull<S, 0>(fi + a.off_pull[0], nb);
    w[1] = pair_pull<S, 1>(fi + a.off_pull[1], nb);
    w[2] = pair_pull<S, 2>(fi + a.off_pull[2], nb);
    w[3] = pair_pull<S, 3>(fi + a.off_pull[3], nb);
    w[4] = pair_pull<S, 4>(fi + a.off_pull[4], nb);
    w[5] = pair_pull<S, 5>(fi + a.off_pull[5], nb);
    w[6] = pair_pull<S, 6>(fi + a.off_pull[6], nb);
    w[7] = pair_pull<S, 7>(fi + a.off_pull[7], nb);
    w[8] = pair_pull<S, 8>(fi + a.off_pull[8], nb);
  }
  pair_finish<S, COLL, FORC, RES>(a, n, seg, w, o2, red);
}

// CAP = 1 asks for 6 resident blocks of 256 threads (at most 40 registers),
// CAP = 2 for 4 (at most 64), CAP = 3 for 7 (32, with a few spills).  RES: the
// residual instantiation; MOV: the moving-obstacle one (CAP = 1 only).  (Two
// rows per thread, one after the other, ran no faster: 131.8 against 131.5
// GLUPS in FP16, 87.6 against 91.0 in FP32.)
template <class S, int COLL, int FORC, int CAP, bool RES, bool MOV = false>
__global__ void __launch_bounds__(256, CAP == 1 ? 6 : (CAP == 2 ? 4 : (CAP == 3 ? 7 : 1)))
    step_pair_kernel(const StepArgs a) {
  const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  float red[7] = {0, 0, 0, 0, 0, 0, 0};
  if (x0 < a.g.nx) pair_step<S, COLL, FORC, RES, MOV>(a, x0, blockIdx.y, red);
  if (RES) block_residual<float>(a, red);
}

// Node pairs in the AA layout.  Even phase: both nodes' own slots, aligned
// words in and out (plane k in, plane kbar out).  Odd phase: the pull of
// plane kbar from x0 - c_kx as in pair_pull, and pushes to x0 + c_kx of plane
// k: aligned words for c_kx = 0, otherwise one value per node (the two
// targets straddle two words whose other halves belong to the neighbouring
// pairs).  Every slot is still read and written by one node only: the word
// loads of the odd phase also bring in a neighbour's half, which that
// neighbour may rewrite in the same phase, but only the own half is used.
// Flagged segments, and every pair of a no-pull step in the odd phase, take
// aa_node.
template <class S, int COLL, int FORC, int CAP, bool ODD>
__global__ void __launch_bounds__(256, CAP == 1 ? 6 : (CAP == 2 ? 4 : 1))
    step_aa_pair_kernel(const StepArgs a) {
  using IO = PairIO<S>;
  using W = typename IO::W;
  const Geom& g = a.g;
  const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y;
  float red[7] = {0, 0, 0, 0, 0, 0, 0};
  if (x0 < g.nx) {
    const int seg = y * g.nseg + (x0 >> 5);
    if (g.segflag[seg] != 0 || (ODD && (a.flags & F_NOPULL))) {
      aa_node<S, COLL, FORC, ODD>(a, x0, y, red);
      if (x0 + 1 < g.nx) aa_node<S, COLL, FORC, ODD>(a, x0 + 1, y, red);
    } else {
      const int ni = (y + 1) * g.pitch + x0;
      const long long n = ni;
      char* const A = static_cast<char*>(a.fout);
      const uint32_t nb = (uint32_t)ni * (uint32_t)sizeof(S);   // byte offset in a plane
      W w[9];
      if (!ODD) {
#pragma unroll
        for (int k = 0; k < 9; ++k) w[k] = *reinterpret_cast<const W*>(A + a.off_plane[k] + nb);
      } else {
        w[0] = pair_pull<S, 0>(A + a.off_aa_pull[0], nb);
        w[1] = pair_pull<S, 1>(A + a.off_aa_pull[1], nb);
        w[2] = pair_pull<S, 2>(A + a.off_aa_pull[2], nb);
        w[3] = pair_pull<S, 3>(A + a.off_aa_pull[3], nb);
        w[4] = pair_pull<S, 4>(A + a.off_aa_pull[4], nb);
        w[5] = pair_pull<S, 5>(A + a.off_aa_pull[5], nb);
        w[6] = pair_pull<S, 6>(A + a.off_aa_pull[6], nb);
        w[7] = pair_pull<S, 7>(A + a.off_aa_pull[7], nb);
        w[8] = pair_pull<S, 8>(A + a.off_aa_pull[8], nb);
      }
      float f0[9], f1[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) IO::unpack(w[k], f0[k], f1[k]);
      float rho0, ux0, uy0, rho1, ux1, uy1;
      node_update<S, COLL, FORC>(f0, a, n, rho0, ux0, uy0, seg);
      node_update<S, COLL, FORC>(f1, a, n + 1, rho1, ux1, uy1, seg);
      if (!ODD) {
#pragma unroll
        for (int k = 0; k < 9; ++k)
          *reinterpret_cast<W*>(A + a.off_plane[INVk(k)] + nb) = IO::pack(f0[k], f1[k]);
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          char* t = A + a.off_aa_push[k] + nb;
          if (CXk(k) == 0) {   // both targets in one word, c_ky rows away
            *reinterpret_cast<W*>(t) = IO::pack(f0[k], f1[k]);
          } else {
            S* ts = reinterpret_cast<S*>(t);
            Store<S>::str(ts, 0, f0[k]);
            Store<S>::str(ts, 1, f1[k]);
          }
        }
      }
      node_outputs<float, RES_FLAG>(a, n, -1, rho0, ux0, uy0, red);
      node_outputs<float, RES_FLAG>(a, n + 1, -1, rho1, ux1, uy1, red);
    }
  }
  if (a.flags & F_RESIDUAL) block_residual<float>(a, red);
}

// ---------------------------------------------------------------------------
// Shared-memory and bulk-copy helpers (bounded mbarrier waits).
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for `parity` of the barrier; false after ~1 s (then *err is set).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int* err,
                                                  unsigned long long limit_ns = 1000000000ull) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) {
      atomicExch(err, kErrWaitTimeout);
      return false;
    }
  }
  return true;
}

// Persistent node-pair kernel fed by bulk copies (shifted storage).
//
// Work is split into tiles: one row y and TW = kTileBytes / sizeof(S) nodes of
// every population plane.  For a tile, thread 0 copies per direction k the
// source row y - c_ky over [x0 - H, x0 + TW + H) (H: one 16-byte granule of
// halo on each side) into one shared-memory stage with cp.async.bulk, and arms
// the stage's mbarrier with the byte count.  The ring of `stages` stages keeps
// the next tiles' loads in flight while the block works on the current one,
// with no registers holding them.  A thread takes node pairs of the tile: it
// reads the nine incoming words from shared memory (the x shift as in
// pair_pull; aligned own slots on a no-pull step), and the arithmetic and the
// stores are those of the node-pair kernel.  Flagged segments (boundary,
// solid and padding nodes) are left out
// of the tiles: their per-node path (link records, dependent global loads)
// would hold up the warp that refills the ring and, through it, the block.
// After its tiles each block works through its share of the list of flagged
// segments, one node per lane through step_node.  Every mbarrier wait is bounded in
// wall-clock time; on expiry the kernel records kErrWaitTimeout, waits
// (bounded) for its own copies and returns.

// The flagged segments of the kind-2 kernel: block b takes its share of the
// segment list, one segment per warp, one node per lane (step_node, or
// aa_node in the AA layout's phases: MODE 1 even, 2 odd).
template <class S, int COLL, int FORC, bool RES, int MODE>
__device__ __forceinline__ void tile_flagged_segments(const StepArgs& a, float red[7]) {
  const Geom& g = a.g;
  const int f0 = (int)((long long)g.nflag * blockIdx.x / gridDim.x);
  const int f1 = (int)((long long)g.nflag * (blockIdx.x + 1) / gridDim.x);
  for (int i = f0 + (int)(threadIdx.x >> 5); i < f1; i += (int)(blockDim.x >> 5)) {
    const int sg = g.seglist[i];
    const int y = sg / g.nseg;
    const int x = (sg - y * g.nseg) * 32 + (int)(threadIdx.x & 31);
    if (x >= g.nx) continue;
    if constexpr (MODE == 0)
      step_node<S, COLL, FORC, false, RES>(a, x, y, red);
    else
      aa_node<S, COLL, FORC, MODE == 2>(a, x, y, red);
  }
}

// Incoming word of direction K of the pair whose word in direction 0's stage
// row is `row`: aligned (AA even phase: the nodes' own slots), or pulled
// from x - c_kx as in pair_pull.
template <class S, int K, int MODE>
__device__ __forceinline__ typename PairIO<S>::W tile_pull(const typename PairIO<S>::W* row) {
  using IO = PairIO<S>;
  constexpr int cx = MODE == 1 ? 0 : CXk(K);
  if (cx == 0) return row[0];
  if (cx == 1) return IO::mid(row[-1], row[0]);
  return IO::mid(row[0], row[1]);
}

// The node-pair kernel fed by shared-memory tiles, in three modes: MODE 0
// two buffers (fin -> fout), MODE 1 / 2 the AA layout's even / odd phase in
// place (the same slots as step_aa_pair_kernel: the even phase reads a
// node's own slots of plane k and writes plane kbar; the odd phase pulls
// plane kbar from x - c_k and pushes plane k to x + c_k).  In the AA phases
// every slot is read and written by one node only; a tile's copy also brings
// in slots of neighbouring tiles' nodes, which may be rewritten meanwhile,
// but those values are never used.
//
// PPT: pairs of a tile per thread (blocks of TW / (2 PPT) threads); up to 64
// registers a thread.
template <class S, int COLL, int FORC, bool RES, int PPT, int MODE>
__global__ void __launch_bounds__(kTileBytes / (2 * PPT * sizeof(S)), 2048 * PPT * sizeof(S) / kTileBytes)
    step_tile_pair_kernel(const StepArgs a, int stages) {
  static_assert(Store<S>::shifted, "the tile kernel is for shifted storage");
  using IO = PairIO<S>;
  using W = typename IO::W;
  constexpr int TW = kTileBytes / sizeof(S);         // nodes per tile
  constexpr int H = kTmaHaloBytes / sizeof(S);       // halo nodes on each side
  constexpr int RWW = (TW + 2 * H) / 2;              // words of one stage row
  constexpr uint32_t kStageBytes = 9 * (TW + 2 * H) * sizeof(S);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[kMaxTileStages], empty[kMaxTileStages];
  const Geom& g = a.g;
  float red[7] = {0, 0, 0, 0, 0, 0, 0};

  // a no-pull step (the first after initialisation) reads every node's own
  // slots: two buffers run it through the tiles with aligned reads, the AA
  // odd phase per node
  const bool nopull = (a.flags & F_NOPULL) != 0;
  if (MODE == 2 && nopull) {
    const int npr = (g.nx + 1) / 2;
    const long long total = (long long)g.ny * npr;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
      const int y = (int)(q / npr), x0 = 2 * (int)(q % npr);
      if (g.segflag[y * g.nseg + (x0 >> 5)] != 0) continue;   // in the segment list
      aa_node<S, COLL, FORC, true>(a, x0, y, red);
      aa_node<S, COLL, FORC, true>(a, x0 + 1, y, red);
    }
    tile_flagged_segments<S, COLL, FORC, RES, MODE>(a, red);
    if constexpr (RES) block_residual<float>(a, red);
    return;
  }

  // block b takes the contiguous tiles [t0, t1) in row-major order; the
  // consumer cursor (cy, cx) and thread 0's copy cursor (py, px) walk them.
  // A tile's copies span its nodes up to nx rounded up to the copy granule,
  // plus the halo on both sides (at most one halo past a row's end, inside
  // the next row or the guard row).
  const int tpr = (g.nx + TW - 1) / TW;
  const int ntiles = g.ny * tpr;
  const int nxr = (g.nx + H - 1) / H * H;
  const int t0 = (int)((long long)ntiles * blockIdx.x / gridDim.x);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
  const char* src = static_cast<const char*>(MODE == 0 ? a.fin : a.fout);
  const long long* off = MODE == 0 ? (nopull ? a.off_plane : a.off_pull)
                                    : (MODE == 1 ? a.off_plane : a.off_aa_pull);
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), blockDim.x / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int y, int x0, int s) {
    const uint32_t copy = (uint32_t)((min(TW, nxr - x0) + 2 * H) * (int)sizeof(S));
    const uint32_t bar = smem_u32(&full[s]);
    mbar_expect_tx(bar, 9 * copy);
    const uint32_t dst0 = smem_u32(smem_raw + (size_t)s * kStageBytes);
    const char* src0 = src + (g.node(x0, y) - H) * (long long)sizeof(S);
#pragma unroll
    for (int k = 0; k < 9; ++k)
      bulk_g2s(dst0 + k * (uint32_t)(RWW * sizeof(W)), src0 + off[k], copy, bar);
  };
  int cy = t0 / tpr, cx = (t0 - cy * tpr) * TW;
  int py = cy, px = cx, pt = t0;
  if (threadIdx.x == 0) {   // prologue: fill the ring
    for (int s = 0; s < stages && pt < t1; ++s, ++pt) {
      issue(py, px, s);
      px += TW;
      if (px >= g.nx) px = 0, ++py;
    }
  }

  // Each warp walks the tiles on its own: it waits for a stage's copies
  // (full), works on its pairs and releases the stage (empty, one arrival
  // per warp).  Thread 0 refills a stage once every warp has released it, so
  // a warp slowed down holds up no other warp until the ring's other stages
  // are used up.  Waits are bounded and their outcome is made warp-uniform,
  // so a warp leaves the loop as a whole.
  bool ok = true;
  int t = t0, s = 0;
  uint32_t parity = 0;
  for (; t < t1; ++t) {
    // the thread's pairs of this tile: segment flags (and the previous
    // residual step's fields) are loaded before the wait for the stage
    int x0[PPT];
    bool bulk[PPT];
    float2 o2[PPT][3];
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
      x0[p] = cx + 2 * (int)(threadIdx.x + p * blockDim.x);
      bulk[p] = x0[p] < g.nx && g.segflag[cy * g.nseg + (x0[p] >> 5)] == 0;
      if (RES && bulk[p]) {
        const long long n = g.node(x0[p], cy);
        o2[p][0] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.rho_old) + n);
        o2[p][1] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.ux_old) + n);
        o2[p][2] = *reinterpret_cast<const float2*>(static_cast<const float*>(a.uy_old) + n);
      }
    }
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&full[s]), parity, a.err))) {
      ok = false;
      break;
    }
    const W* stage = reinterpret_cast<const W*>(smem_raw + (size_t)s * kStageBytes);
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
      if (!bulk[p]) continue;   // flagged: in the segment list, after the tiles
      const int j = (int)(threadIdx.x + p * blockDim.x);
      const long long n = g.node(x0[p], cy);
      const W* row = stage + H / 2 + j;   // the pair's word in direction 0's row
      W w[9];
      if (MODE == 0 && nopull) {
#pragma unroll
        for (int k = 0; k < 9; ++k) w[k] = row[k * RWW];
      } else {
        w[0] = tile_pull<S, 0, MODE>(row);
        w[1] = tile_pull<S, 1, MODE>(row + 1 * RWW);
        w[2] = tile_pull<S, 2, MODE>(row + 2 * RWW);
        w[3] = tile_pull<S, 3, MODE>(row + 3 * RWW);
        w[4] = tile_pull<S, 4, MODE>(row + 4 * RWW);
        w[5] = tile_pull<S, 5, MODE>(row + 5 * RWW);
        w[6] = tile_pull<S, 6, MODE>(row + 6 * RWW);
        w[7] = tile_pull<S, 7, MODE>(row + 7 * RWW);
        w[8] = tile_pull<S, 8, MODE>(row + 8 * RWW);
      }
      const int seg = cy * g.nseg + (x0[p] >> 5);
      char* const fo = static_cast<char*>(a.fout);
      const uint32_t nb = (uint32_t)n * (uint32_t)sizeof(S);   // byte offset in a plane
      if constexpr (MODE == 0) {
        pair_finish<S, COLL, FORC, RES>(a, n, seg, w, o2[p], red);
      } else {
        float f0[9], f1[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) IO::unpack(w[k], f0[k], f1[k]);
        float rho0, ux0, uy0, rho1, ux1, uy1;
        node_update<S, COLL, FORC>(f0, a, n, rho0, ux0, uy0, seg);
        node_update<S, COLL, FORC>(f1, a, n + 1, rho1, ux1, uy1, seg);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          if (MODE == 1) {   // own slots, plane kbar
            *reinterpret_cast<W*>(fo + a.off_plane[INVk(k)] + nb) = IO::pack(f0[k], f1[k]);
          } else {           // pushes to x + c_k of plane k
            char* tg = fo + a.off_aa_push[k] + nb;
            if (CXk(k) == 0) {
              *reinterpret_cast<W*>(tg) = IO::pack(f0[k], f1[k]);
            } else {
              S* ts = reinterpret_cast<S*>(tg);
              Store<S>::str(ts, 0, f0[k]);
              Store<S>::str(ts, 1, f1[k]);
            }
          }
        }
        pair_outputs<RES>(a, n, rho0, ux0, uy0, rho1, ux1, uy1, red, o2[p]);
      }
    }
    __syncwarp();   // every lane is done reading stage s
    if (lane == 0) mbar_arrive(smem_u32(&empty[s]));
    if (threadIdx.x < 32) {   // warp 0: thread 0 refills stage s with tile pt
      bool got = true;
      if (threadIdx.x == 0 && pt < t1) {
        got = mbar_wait_bounded(smem_u32(&empty[s]), parity, a.err);
        if (got) {
          issue(py, px, s);
          px += TW;
          if (px >= g.nx) px = 0, ++py;
          ++pt;
        }
      }
      if (!__shfl_sync(0xffffffffu, got, 0)) {
        ok = false;
        ++t;   // tile t was consumed
        break;
      }
    }
    cx += TW;
    if (cx >= g.nx) cx = 0, ++cy;
    if (++s == stages) s = 0, parity ^= 1u;
  }
  if (!ok && threadIdx.x == 0) {
    // drain the copies still in flight (tiles t .. pt-1), bounded, so no
    // bulk copy lands in shared memory after the block has left
    for (int j = t - t0; j < pt - t0; ++j) {
      const uint32_t bar = smem_u32(&full[j % stages]);
      const uint32_t par = (uint32_t)((j / stages) & 1);
      const unsigned long long tw0 = global_ns();
      while (!mbar_try_wait(bar, par) && global_ns() - tw0 < 1000000000ull) {
      }
    }
  }
  if (ok) tile_flagged_segments<S, COLL, FORC, RES, MODE>(a, red);
  __syncthreads();
  if constexpr (RES) block_residual<float>(a, red);
}

// ---------------------------------------------------------------------------
// Initial equilibrium -- equilibrium_kernels.py:38-78.  rho/u are FP64 device
// arrays in device order; moments (compute type) receive rho/u on every node
// of the columns x_lo <= x < x_hi.
template <class S>
__global__ void init_kernel(const Geom g, const Params p, const double* __restrict__ rho,
                            const double* __restrict__ u, S* __restrict__ f,
                            typename Store<S>::T* mr, typename Store<S>::T* mx,
                            typename Store<S>::T* my, int x_lo, int x_hi) {
  using T = typename Store<S>::T;
  const int x = x_lo + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= x_hi) return;
  const long long n = g.node(x, y);
  const double r = rho[n], ux = u[n], uy = u[g.plane + n];
  mr[n] = T(r);
  mx[n] = T(ux);
  my[n] = T(uy);
  if (g.cls[n] == 2) {
#pragma unroll
    for (int k = 0; k < 9; ++k) Store<S>::st(f, k * g.plane + n, T(0), p);
    return;
  }
  if constexpr (Store<S>::shifted) {
    // g_eq = f_eq - w without cancellation: w (r e - 1) = w ((r - 1) + r (e - 1)),
    // in FP32 (D2Q9 constants) from r - 1 formed in FP64: GB300's FP64 rate
    // made the FP64 form 2 ms at 8192 x 2048, ten times the memory time, for a
    // value that is rounded to FP32 (or FP16) anyway.
    const float dr = float(r - 1.0), rf = float(r), fx = float(ux), fy = float(uy);
    const float hu2 = 1.5f * (fx * fx + fy * fy);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float cu = lin2r<float>(CXk(k), CYk(k), fx, fy);
      const float em1 = k == 0 ? -hu2 : fmaf(cu, fmaf(4.5f, cu, 3.f), -hu2);
      Store<S>::st(f, k * g.plane + n, T(float(Wk(k)) * fmaf(rf, em1, dr)), p);
    }
  } else {
    // equilibrium_kernels.py:6-35, the reference's operation order
    const double hu2 = p.half_inv_cs_2 * (ux * ux + uy * uy);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int cx = CXk(k), cy = CYk(k);
      double cu = 0.0;
      if (cx != 0 && cy != 0) cu = (cx > 0 ? ux : -ux) + (cy > 0 ? uy : -uy);
      else if (cx != 0) cu = cx > 0 ? ux : -ux;
      else if (cy != 0) cu = cy > 0 ? uy : -uy;
      const double e = (cx == 0 && cy == 0) ? 1.0 - hu2
                                            : ((1.0 + p.inv_cs_2 * cu) + (p.half_inv_cs_4 * cu) * cu) - hu2;
      Store<S>::st(f, k * g.plane + n, T((Wk(k) * r) * e), p);
    }
  }
}

}  // namespace lbm
