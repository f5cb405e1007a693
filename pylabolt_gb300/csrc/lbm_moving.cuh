// Moving circular obstacles (extension: the reference's moving-obstacle path
// cannot run; pylabolt/base/obstacle_operator.py:47-73 calls an undefined
// reconstruct_obstacles and leaves the refill of uncovered nodes as a TODO).
//
// Per step, before the fused step kernel:
//   mov_motion_kernel    the integrator of update_position_velocity
//                        (pylabolt/parallel/cpu/obstacle_kernels.py:386-460)
//                        from the last step's force and torque, and the box of
//                        nodes the move may change;
//   mov_raster_kernel    solid flag, wall velocity v + omega x r and the
//                        reported density / velocity of covered nodes
//                        (construct_circle, obstacle_kernels.py:43-93, or
//                        construct_ellipse :192-241 with the inclination the
//                        rotation has reached); nodes left behind are marked
//                        fresh;
//   mov_classify_kernel  node classes around the obstacle (2 solid, 4 fluid
//                        next to a moving solid, 0 bulk) and the refill of
//                        fresh nodes with f_eq(mean density of their fluid
//                        neighbours, the wall velocity they had);
// after it:
//   mov_force_kernel     momentum exchange on the obstacle
//                        (compute_force_torque_single_phase,
//                        force_torque_kernels.py:11-90) with the bounce-back
//                        the next step applies, summed in a fixed order
//                        (thread g of kMovForceBlocks x kMovForceThreads
//                        takes box nodes g, g + 16384, ..., a shared-memory
//                        tree per block, then mov_force_finish's tree over
//                        the blocks), and the fresh flags cleared.
// Class-4 nodes pull their links at run time in the step kernel
// (dynamic_links): a moving-solid source gives
// pop[x,kbar] - 2 w_kbar rho(x) inv_cs_2 (c_kbar . u_solid)
// (streaming_kernels.py:41-47) with rho(x) of the previous step (rho_dyn).
//
// Index safety: the motion kernel only accepts a box whose one-node border
// lies in [1, nx-2] x [1, ny-2] (so every neighbour read is a grid node), and
// a move of less than one node per step (so the box fits the side x side
// launch the host sizes from the radius); otherwise it records an error and
// leaves the obstacle where it was.
#pragma once
#include "lbm_kernels.cuh"

namespace lbm {

__device__ __forceinline__ long long mov_off(const Geom& g, int k) {
  return (long long)CYk(k) * g.pitch + CXk(k);
}

// f_eq(r, u) of node n into storage, formed in FP64 (init_kernel's FP64 form;
// a refill touches a few nodes per step).
template <class S>
__device__ __forceinline__ void store_feq(const Geom& g, const Params& p, S* f, long long n,
                                          double r, double ux, double uy) {
  using T = typename Store<S>::T;
  const double hu2 = p.half_inv_cs_2 * (ux * ux + uy * uy);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int cx = CXk(k), cy = CYk(k);
    double cu = 0.0;
    if (cx != 0 && cy != 0) cu = (cx > 0 ? ux : -ux) + (cy > 0 ? uy : -uy);
    else if (cx != 0) cu = cx > 0 ? ux : -ux;
    else if (cy != 0) cu = cy > 0 ? uy : -uy;
    if (Store<S>::shifted) {
      // g_eq = f_eq - w computed without cancellation: w ((r - 1) + r (e - 1))
      const double em1 = (cx == 0 && cy == 0) ? -hu2
                                              : (p.inv_cs_2 * cu + (p.half_inv_cs_4 * cu) * cu) - hu2;
      Store<S>::st(f, k * g.plane + n, T(Wk(k) * ((r - 1.0) + r * em1)), p);
    } else {
      const double e = (cx == 0 && cy == 0)
                           ? 1.0 - hu2
                           : ((1.0 + p.inv_cs_2 * cu) + (p.half_inv_cs_4 * cu) * cu) - hu2;
      Store<S>::st(f, k * g.plane + n, T((Wk(k) * r) * e), p);
    }
  }
}

// a.j < 0: no motion, only the box of the current position (set-up).
template <class S>
__global__ void mov_motion_kernel(const MovArgs a) {
  const int j = threadIdx.x;
  if (j >= a.n) return;
  MovObs o = a.obs[j];
  double ncx = o.cx, ncy = o.cy;
  MovObs m = o;
  if (a.j >= 0) {
    const double om_old = o.om, vx_old = o.vx, vy_old = o.vy;
    double tt = 0.0, fx = 0.0, fy = 0.0;
    if (o.calculated) {
      if (o.rotation) {
        m.om = o.om + o.tq / o.inertia;
        tt = o.tq;
      }
      if (o.translation) {
        m.vx = o.vx + (o.fx / o.mass + a.gx);
        m.vy = o.vy + (o.fy / o.mass + a.gy);
        fx = o.fx;
        fy = o.fy;
      }
    }
    if (o.rotation) m.angle = o.angle + (om_old + 0.5 * tt / o.inertia);
    if (o.translation) {
      ncx = o.cx + (vx_old + 0.5 * (fx / o.mass + a.gx));
      ncy = o.cy + (vy_old + 0.5 * (fy / o.mass + a.gy));
    }
  }
  if (!(fabs(ncx - o.cx) < 1.0 && fabs(ncy - o.cy) < 1.0)) {
    atomicExch(a.err, kErrMovSpeed);
    m = o;
    ncx = o.cx;
    ncy = o.cy;
  }
  int bx0 = (int)floor(fmin(o.cx, ncx) - o.r) - 1, bx1 = (int)ceil(fmax(o.cx, ncx) + o.r) + 1;
  int by0 = (int)floor(fmin(o.cy, ncy) - o.r) - 1, by1 = (int)ceil(fmax(o.cy, ncy) + o.r) + 1;
  if (bx0 < 2 || by0 < 2 || bx1 > a.g.nx - 3 || by1 > a.g.ny - 3) {
    atomicExch(a.err, kErrMovBounds);
    m = o;
    ncx = o.cx;
    ncy = o.cy;
    bx0 = (int)floor(o.cx - o.r) - 1;
    bx1 = (int)ceil(o.cx + o.r) + 1;
    by0 = (int)floor(o.cy - o.r) - 1;
    by1 = (int)ceil(o.cy + o.r) + 1;
    // an obstacle registered out of range gets an empty box (the host rejects
    // it; every box kernel returns at once on bx1 < bx0)
    if (bx0 < 2 || by0 < 2 || bx1 > a.g.nx - 3 || by1 > a.g.ny - 3) {
      bx0 = by0 = 2;
      bx1 = by1 = 1;
    }
  }
  m.cx = ncx;
  m.cy = ncy;
  if (m.shape == 1) {   // orientation of the ellipse for this step's raster
    m.cth = cos(m.angle);
    m.sth = sin(m.angle);
  }
  m.bx0 = bx0;
  m.bx1 = bx1;
  m.by0 = by0;
  m.by1 = by1;
  a.obs[j] = m;
}

template <class S>
__global__ void mov_raster_kernel(const MovArgs a) {
  using T = typename Store<S>::T;
  const MovObs& o = a.obs[a.j];
  if (o.bx1 < o.bx0) return;
  const int x = o.bx0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = o.by0 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > o.bx1 || y > o.by1) return;
  const Geom& g = a.g;
  const long long n = g.node(x, y);
  const double rx = (double)x - o.cx, ry = (double)y - o.cy;
  const uint8_t me = (uint8_t)(a.j + 1);
  bool inside;
  if (o.shape == 1) {   // is_ellipse's test in the turned frame (obstacle_kernels.py:151-189)
    const double xp = rx * o.cth + ry * o.sth;
    const double yp = -rx * o.sth + ry * o.cth;
    inside = (xp * xp) / (o.sa * o.sa) + (yp * yp) / (o.sb * o.sb) <= 1.0;
  } else {
    inside = rx * rx + ry * ry <= o.r * o.r;
  }
  if (inside) {
    a.dsolid[n] = me;
    const double ux = o.vx - o.om * ry, uy = o.vy + o.om * rx;
    T* us = static_cast<T*>(a.us);
    us[n] = T(ux);
    us[g.plane + n] = T(uy);
    static_cast<T*>(a.mr)[n] = T(o.density);
    static_cast<T*>(a.mx)[n] = T(ux);
    static_cast<T*>(a.my)[n] = T(uy);
  } else if (a.dsolid[n] == me) {
    a.dsolid[n] = 0;
    a.fresh[n] = 1;
  }
}

template <class S>
__global__ void mov_classify_kernel(const MovArgs a) {
  using T = typename Store<S>::T;
  const MovObs& o = a.obs[a.j];
  if (o.bx1 < o.bx0) return;
  const int x = o.bx0 - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = o.by0 - 1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x > o.bx1 + 1 || y > o.by1 + 1) return;
  const Geom& g = a.g;
  const long long n = g.node(x, y);
  // the region must be static bulk fluid (no boundary record, no static solid)
  if (g.cls[n] == 1) atomicExch(a.err, kErrMovNeighbour);
  a.segflag[y * g.nseg + (x >> 5)] = 1;
  if (a.dsolid[n]) {
    a.cls[n] = 2;
    return;
  }
  bool next_to_solid = false;
#pragma unroll
  for (int k = 1; k < 9; ++k) next_to_solid |= a.dsolid[n + mov_off(g, k)] != 0;
  a.cls[n] = next_to_solid ? 4 : 0;
  if (a.fresh[n]) {
    const T* rd = static_cast<const T*>(a.rho_dyn);
    double sum = 0.0;
    int cnt = 0;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const long long q = n + mov_off(g, k);
      if (a.dsolid[q] == 0 && a.fresh[q] == 0) {
        sum += double(rd[q]);
        ++cnt;
      }
    }
    const double rho = cnt ? sum / cnt : 1.0;
    const T* us = static_cast<const T*>(a.us);
    store_feq<S>(g, a.p, static_cast<S*>(a.pop), n, rho, double(us[n]), double(us[g.plane + n]));
    static_cast<T*>(a.rho_dyn)[n] = T(rho);
  }
}


template <class S>
__global__ void __launch_bounds__(kMovForceThreads) mov_force_kernel(const MovArgs a) {
  using T = typename Store<S>::T;
  constexpr bool SH = Store<S>::shifted;
  const MovObs* ob = a.obs + a.j;
  const int x0 = ob->bx0 - 1, y0 = ob->by0 - 1;
  // an empty box (bx1 < bx0) contributes nothing
  const int W = ob->bx1 < ob->bx0 ? 0 : ob->bx1 - ob->bx0 + 3, H = ob->by1 - ob->by0 + 3;
  const double cx = ob->cx, cy = ob->cy;
  const Geom& g = a.g;
  const Params& p = a.p;
  const S* f = static_cast<const S*>(a.pop);
  const T* us = static_cast<const T*>(a.us);
  const T* rd = static_cast<const T*>(a.rho_dyn);
  const uint8_t me = (uint8_t)(a.j + 1);
  double sx = 0.0, sy = 0.0, st = 0.0;
  const int tid = threadIdx.x;
  for (int i = blockIdx.x * kMovForceThreads + tid; i < W * H;
       i += kMovForceThreads * kMovForceBlocks) {
    const int x = x0 + i / H, y = y0 + i % H;
    const long long n = g.node(x, y);
    if (a.fresh[n]) a.fresh[n] = 0;
    if (a.cls[n] != 4) continue;
    // the obstacle of the first solid neighbour in direction order
    // (compute_obstacle_boundary, obstacle_kernels.py:307-350)
    uint8_t first = 0;
#pragma unroll
    for (int k = 1; k < 9; ++k)
      if (first == 0) first = a.dsolid[n + mov_off(g, k)];
    if (first != me) continue;
    const double rx = (double)x - cx, ry = (double)y - cy;
#pragma unroll
    for (int k = 1; k < 9; ++k) {
      const long long q = n + mov_off(g, k);
      if (a.dsolid[q] == 0) continue;
      const int kb = INVk(k);
      // population k leaves towards the solid; it comes back as kbar
      const T raw = Store<S>::ld(f, k * g.plane + n, p);
      T back;
      if (a.nopull) {
        back = Store<S>::ld(f, kb * g.plane + n, p);
      } else {
        const T cu = lin2r<T>(CXk(k), CYk(k), us[q], us[g.plane + q]);
        const T rho = rd[n];
        back = SH ? raw - (T(2.0 * Wk(k)) * rho * T(3)) * cu
                  : raw - ((T(2.0 * Wk(k)) * rho) * T(p.inv_cs_2)) * cu;
      }
      double fo = double(raw), fb = double(back);
      if (SH) {
        fo += Wk(k);
        fb += Wk(kb);
      }
      const double vx = fo * double(CXk(k)) - fb * double(CXk(kb));
      const double vy = fo * double(CYk(k)) - fb * double(CYk(kb));
      sx += vx;
      sy += vy;
      st += rx * vy - ry * vx;
    }
  }
  __shared__ double red[3][kMovForceThreads];
  red[0][tid] = sx;
  red[1][tid] = sy;
  red[2][tid] = st;
  __syncthreads();
#pragma unroll
  for (int h = kMovForceThreads / 2; h > 0; h >>= 1) {
    if (tid < h)
#pragma unroll
      for (int c = 0; c < 3; ++c) red[c][tid] += red[c][tid + h];
    __syncthreads();
  }
  if (tid < 3) a.part[(a.j * kMovForceBlocks + blockIdx.x) * 3 + tid] = red[tid][0];
}

template <class S>
__global__ void mov_force_finish_kernel(const MovArgs a) {
  __shared__ double red[3][kMovForceBlocks];
  const int t = threadIdx.x;
  for (int c = 0; c < 3; ++c) red[c][t] = a.part[(a.j * kMovForceBlocks + t) * 3 + c];
  __syncthreads();
#pragma unroll
  for (int h = kMovForceBlocks / 2; h > 0; h >>= 1) {
    if (t < h)
#pragma unroll
      for (int c = 0; c < 3; ++c) red[c][t] += red[c][t + h];
    __syncthreads();
  }
  if (t == 0) {
    MovObs* ob = a.obs + a.j;
    ob->fx = red[0][0];
    ob->fy = red[1][0];
    ob->tq = red[2][0];
  }
}

}  // namespace lbm
