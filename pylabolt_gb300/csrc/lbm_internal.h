// Internal interface between the C-ABI layer (lbm_capi.cu) and the kernel
// translation units (lbm_fp64.cu: FP64, built with --fmad=false so it keeps
// the reference's rounding; lbm_lowp.cu: FP32 / FP16 shifted storage).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace lbm {

// Device-side geometry of one case.  Populations are SoA planes of
// (ny+2) rows of `pitch` elements (x fastest); row 0 and row ny+1 are padding
// rows so that vector loads of the rows above/below an edge row stay inside
// the allocation.  Node (x, y) has index n = (y+1)*pitch + x.  `pitch` is a
// multiple of the 512-byte row segment of one warp.
struct Geom {
  int nx, ny, pitch, nseg;   // nseg = ceil(nx/32) warp segments per row
  long long plane;           // elements per population plane = (ny+2)*pitch
  const uint8_t* cls;        // [plane] node class: 0 bulk, 1 special, 2 solid
                             // (3 on padding rows and columns)
  const uint8_t* segflag;    // [ny*nseg] 0: all 32 nodes of the segment bulk
  const int* seglist;        // [nflag] y*nseg + x/32 of every segment flagged at
  int nflag;                 // creation, in order (the kind-2 kernel's boundary work)
  const int* recmap;         // [plane] record index of special nodes
  int nrec;
  const int8_t* rtype;       // [nrec*9] link kind
  const int* rsrc;           // [nrec*9] PULL source node (device index)
  const double* rparam;      // [nrec*9]
  const float2* rpf;         // [nrec*9] FP32 (param, param - 1), rounded from
                             // FP64 on the host: the shifted paths read these,
                             // so that no FP64 conversion runs in the step
  const int* raux;           // [nrec*9] ABB: record index of node x+n
#ifdef __CUDACC__
  __host__ __device__
#endif
  long long node(int x, int y) const { return (long long)(y + 1) * pitch + x; }
};

struct Params {
  double omega, one_m_omega, one_m_half_omega;
  double inv_cs_2, inv_cs_4, half_inv_cs_2, half_inv_cs_4, eps;
  double gx, gy;
  double s_e, s_eps, s_q, s_nu;
  double scale, inv_scale;   // FP16 storage scale
  // FP32 constants of the shifted-storage collision (scale = storage scale)
  float f_omega;             // omega
  float f_wsc[3];            // w * scale for |c|^2 = 0, 1, 2
  float f_omh[3];            // (1 - omega/2) * w * scale for |c|^2 = 0, 1, 2
  float f_gx, f_gy, f_scale, f_inv_scale;
  float f_i2, f_i4, f_homh;  // inv_cs_2, inv_cs_4, 1 - omega/2 of the FP32 paths
  // MRT of the shifted paths, per relaxed moment (e, eps, q, nu):
  // -s / |row|^2 and (1 - s/2) / |row|^2
  float f_mrt_s[4], f_mrt_h[4];
};

enum StepFlags {
  F_NOPULL = 1,      // populations in `fin` already are the incoming ones
  F_MOMENTS = 2,     // write rho/ux/uy
  F_RESIDUAL = 4,    // residual sums against *_old, then *_new <- this step's fields
};

// Arguments of one fused step launch.  `void*` arrays are typed by the
// instantiation: populations in storage type, the rest in compute type.
struct StepArgs {
  Geom g;
  Params p;
  const void* fin;
  void* fout;
  const void* side_in;   // [nrec*3] rho, ux, uy of the previous step
  void* side_out;
  void* rho; void* ux; void* uy;            // [plane] moments
  // residual: fields of the previous residual step are read from *_old and
  // this step's written to *_new (two array sets swapped per residual step: a
  // load and a store of one address in the same pass stall on the in-flight
  // miss in L2)
  const void* rho_old; const void* ux_old; const void* uy_old;
  void* rho_new; void* ux_new; void* uy_new;
  double* partials;      // [nblocks*8] residual partial sums
  const void* body;      // [2*plane] body force or null
  int* err;              // device-visible error word (bounded waits)
  const float* omega_seg;  // [ny*nseg] relaxation rate per 32-node segment, or null
  // moving obstacles (class-4 nodes pull their links at run time)
  const uint8_t* dsolid;   // [plane] 0, or 1 + index of the moving obstacle covering it
  const void* us;          // [2*plane] velocity of moving-solid nodes (compute type)
  // [plane] density of class-4 nodes: of the last step (read) and of this one
  // (written); two buffers swapped with the populations, so that a launch
  // that does not advance the state (autotuner) leaves it untouched
  const void* rho_dyn_in;
  void* rho_dyn_out;
  int aa;                  // 0: two buffers (fin -> fout); AA layout (fin == fout):
                           // 1 even phase, 2 odd phase
  int flags;
  // Byte offsets of direction k from a node's element of plane 0, filled on
  // the host so that the node-pair kernels add a constant per access instead
  // of forming it: the pull source (plane k, row y - c_ky), the plane k of the
  // node itself, the AA odd phase's pull (plane kbar, row y - c_ky) and push
  // (plane k, node + c_k).
  long long off_pull[9], off_plane[9], off_aa_pull[9], off_aa_push[9];
};

// Fills the byte offsets of StepArgs for storage elements of `eb` bytes.
inline void fill_offsets(StepArgs& a, int eb) {
  static const int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
  static const int cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
  static const int inv[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
  const long long P = a.g.plane, R = a.g.pitch;
  for (int k = 0; k < 9; ++k) {
    a.off_pull[k] = (k * P - cy[k] * R) * eb;
    a.off_plane[k] = k * P * eb;
    a.off_aa_pull[k] = (inv[k] * P - cy[k] * R) * eb;
    a.off_aa_push[k] = (k * P + cy[k] * R + cx[k]) * eb;
  }
}

// Arguments of one reverse (adjoint) step; see lbm_adjoint.cuh.
struct AdjArgs {
  Geom g;
  Params p;
  const void* fprev;      // p_{t-1} (storage type): its pull gives f^t
  const void* side_prev;  // rho, u of step t-1 at boundary nodes (compute type)
  const void* a_next;     // a^{t+1} = dL/df^{t+1}, [9][plane] compute type; null at t = T
  void* a_cur;            // a^t out
  const double* grad_u;   // dL/du^T, [2][plane] FP64, only at t = T
  void* gF;               // dL/dF accumulator [2][plane] (compute type) or null
  double* gpart;          // [blocks][4]: dL/domega, dL/du_wall x, y (accumulated)
  const int* tr_reader;   // [nrec*9] node that pulls p_t(n)_m, or -1
  const int8_t* tr_self;  // [nrec*9] 1: n's own link mbar bounces p_t(n)_m back
  const int8_t* wall_rec; // [nrec] 1: the record's MBB links are wall links
  const void* body;       // body force [2][plane] or null (then F = rho g)
  int nopull;             // t = 1: f^1 are the stored populations themselves
};

// Momentum-exchange force sums over link groups (obstacles, wall elements).
// Links are sorted by group; group i owns [gstart[i], gstart[i+1]).
struct ForceArgs {
  Geom g;
  Params p;
  const void* pop;        // post-collision populations p_t (storage type)
  const void* side;       // rho, u of step t at boundary nodes (compute type)
  const long long* node;  // [n] device node index
  const int* rec;         // [n] link record of the node
  const int8_t* kk;       // [2n] k_out, k_in
  const double* arm;      // [2n] lever arm rx, ry
  const int* gstart;      // [ngroups+1]
  int nopull;             // state holds incoming populations (t = 0): f_new = p
  int aa_state;           // AA layout: 1 after an even phase, 2 after an odd one
  double* out;            // [ngroups][3] fx, fy, torque
};

// Where the post-collision population k of node n sits in the AA layout:
// after an even phase in the node's own opposite slot, after an odd phase in
// slot k of the neighbour it moves to; otherwise (two buffers, or the
// incoming populations after initialisation) at the node's slot k.
__host__ __device__ inline long long aa_post_index(long long plane, int pitch, int state,
                                                   long long n, int k) {
  const int cx = (k == 1 || k == 5 || k == 8) ? 1 : ((k == 3 || k == 6 || k == 7) ? -1 : 0);
  const int cy = (k == 2 || k == 5 || k == 6) ? 1 : ((k == 4 || k == 7 || k == 8) ? -1 : 0);
  const int kb = k == 0 ? 0 : (k <= 4 ? ((k + 1) % 4) + 1 : ((k - 3) % 4) + 5);
  if (state == 1) return kb * plane + n;
  if (state == 2) return k * plane + n + (long long)cy * pitch + cx;
  return k * plane + n;
}

// A moving obstacle on the device (FP64 state, see lbm_set_moving_obstacles).
struct MovObs {
  double cx, cy, r, vx, vy, om, angle, mass, inertia, density, fx, fy, tq;
  double sa, sb;            // ellipse semi-axes (shape 1)
  double cth, sth;          // cos, sin of `angle` (ellipse orientation), set by the motion
  int id, calculated, rotation, translation;
  int shape;                // 0 circle, 1 ellipse
  int bx0, by0, bx1, by1;   // nodes the last move may have changed (inclusive)
};

// Arguments of the moving-obstacle kernels.
struct MovArgs {
  Geom g;
  Params p;
  MovObs* obs;
  int n;                    // obstacles
  int j;                    // obstacle of this launch (raster, classify, force)
  double gx, gy;            // gravity of the motion
  uint8_t* dsolid;
  uint8_t* fresh;           // [plane] 1: left by an obstacle this step
  uint8_t* cls;             // writable views of Geom::cls / segflag
  uint8_t* segflag;
  void* us;                 // [2*plane]
  void* rho_dyn;            // [plane] buffer of the current state
  void* pop;                // current state (storage type)
  void* mr; void* mx; void* my;   // moments (solid nodes get rho_s, u_s)
  int nopull;               // force: the state holds incoming populations
  double* part;             // force: per-block partial sums [n][blocks][3]
  int* err;                 // device-visible error word
};

// Launch shape of the fused step.
//   kind 0: scalar kernel, one node per thread
//   kind 2: persistent node-pair kernel fed by bulk copies: tiles of one row
//           segment of kTileBytes per plane, `stages` shared-memory stages,
//           `block` threads (vec = 2)
//   kind 3: node-pair kernel, two nodes per thread along x (vec = 2),
//           `stages` its register cap
struct Variant {
  int kind;
  int vec;
  int block;
  int stages;
};

constexpr int kMaxVariants = 16;     // autotuner candidates per storage at most
constexpr int kTmaRowBytes = 4096;   // row pitch alignment of shifted storage, bytes
constexpr int kTileBytes = 2048;     // tile width of the kind-2 kernel, bytes of one plane row
constexpr int kTmaHaloBytes = 16;    // bulk-copy granule: halo on each side
constexpr int kMaxTileStages = 8;    // shared-memory stages of the kind-2 kernel at most
constexpr int kSmemPerSM = 228 * 1024;   // shared memory of one SM, bytes
constexpr int kErrWaitTimeout = 1;   // err code: an mbarrier wait timed out
constexpr int kErrMovBounds = 2;     // a moving obstacle would leave the allowed region
constexpr int kErrMovSpeed = 3;      // a moving obstacle would move a node or more in a step
constexpr int kErrMovNeighbour = 4;  // a moving obstacle reached a static solid or boundary node
constexpr int kMovMaxObstacles = 32;
constexpr int kMovForceThreads = 256;   // momentum-exchange launch of a moving obstacle
constexpr int kMovForceBlocks = 64;

// Kernels of one storage precision.
struct KernelSet {
  int elem_bytes;        // storage bytes per population value
  int compute_bytes;     // bytes per moment value
  cudaError_t (*step)(int collision, int forcing, const StepArgs& a, Variant v,
                      int sms, cudaStream_t s);
  int nvariants;             // candidate launch shapes for the autotuner
  Variant variants[kMaxVariants];
  // f_eq(rho,u) into storage on fluid nodes (zeros on solids); moments get
  // rho/u on every node.  rho [plane], u [2][plane], FP64, device order.
  cudaError_t (*init)(const Geom& g, const Params& p, const double* rho,
                      const double* u, void* f, void* mr, void* mx, void* my,
                      int x_lo, int x_hi, cudaStream_t s);
  // storage <-> FP64 [9][plane] (dir 0: to FP64, 1: from FP64); solids 0.
  // aa_state (dir 0): where the post-collision values sit (aa_post_index).
  cudaError_t (*convert)(const Geom& g, const Params& p, void* f, double* f64,
                         int dir, int aa_state, cudaStream_t s);
  // moments (compute type) -> FP64 [3][plane]
  cudaError_t (*moments_to_f64)(const Geom& g, const void* mr, const void* mx,
                                const void* my, double* out, cudaStream_t s);
  // FP64 [2][plane] -> compute type [2][plane]
  cudaError_t (*body_from_f64)(const Geom& g, const double* in, void* out,
                               cudaStream_t s);
  // partial sums {sum f, sum cx f, sum cy f} per block row -> partials[ny][8]
  cudaError_t (*conservation)(const Geom& g, const Params& p, const void* f,
                              double* partials, int aa_state, cudaStream_t s);
  // one reverse step (null where the storage has no adjoint)
  cudaError_t (*adjoint)(int forcing, const AdjArgs& a, cudaStream_t s);
  // momentum-exchange sums, one block per group
  cudaError_t (*forces)(const ForceArgs& a, int ngroups, cudaStream_t s);
  // moving obstacles: motion (one thread each), raster and classify (one
  // launch per obstacle over its box, side x side threads), momentum exchange
  cudaError_t (*mov_motion)(const MovArgs& a, cudaStream_t s);
  cudaError_t (*mov_raster)(const MovArgs& a, int side, cudaStream_t s);
  cudaError_t (*mov_classify)(const MovArgs& a, int side, cudaStream_t s);
  cudaError_t (*mov_force)(const MovArgs& a, cudaStream_t s);
};

const KernelSet& kernels_fp64();
const KernelSet& kernels_fp32();
const KernelSet& kernels_fp16();

// Deterministic reduction of `nrows` rows of 8 doubles into out8 (fixed
// order; out8 may be mapped host memory), one launch: `scratch` holds
// kFinishBlocks rows and, after them, a zeroed counter (kFinishScratch
// doubles in all) that tells the last block to finish to sum the rows.
constexpr int kFinishBlocks = 128;
constexpr int kFinishScratch = kFinishBlocks * 8 + 8;
cudaError_t finish_reduce(const double* partials, long long nrows, double* scratch,
                          double* out8, cudaStream_t s);
// Shared memory of one stage of the kind-2 kernel (nine halo-padded row windows).
inline int tile_stage_bytes() { return 9 * (kTileBytes + 2 * kTmaHaloBytes); }
// Number of SMs of the current device (cached by the caller's handle).
// grid of the fused step for variant v (`sms` multiprocessors; res: a
// residual launch).  Kind 2 is persistent: as many blocks as are sure to be
// resident at once -- shared memory per block (stages, the static barriers,
// the residual rows of a residual launch, and the 1 KB the runtime reserves)
// and the 1024 threads per SM its launch bounds guarantee registers for.
inline dim3 step_grid(const Geom& g, Variant v, int sms, int elem_bytes, bool res) {
  if (v.kind == 2) {
    const int tw = kTileBytes / elem_bytes;
    const long long tiles = (long long)g.ny * ((g.nx + tw - 1) / tw);
    const int smem = v.stages * tile_stage_bytes() + 2 * 8 * kMaxTileStages + (res ? 16 * 8 * 8 : 0) + 1024;
    int per_sm = kSmemPerSM / smem;
    if (per_sm * v.block > 1024) per_sm = 1024 / v.block;   // 64 registers a thread
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)sms * per_sm;
    if (blocks > tiles) blocks = tiles;
    return dim3((unsigned)blocks, 1);
  }
  // blocks cover the nodes x < nx of a row, not its padding (the AA layout's
  // rows carry at least one padding column: a whole block more at nx = 8192)
  const long long per_block = (long long)v.block * v.vec;
  return dim3((unsigned)((g.nx + per_block - 1) / per_block), (unsigned)g.ny);
}
// Host-order <-> device-order copies of node data with `ncomp`
// components: host AoS [node][ncomp] in inner (ind = x*ny+y) or padded
// (ind = (x+1)*(ny+2)+(y+1)) order; device SoA [ncomp][plane].
cudaError_t reorder(const Geom& g, const double* in, double* out, int ncomp,
                    int layout, int to_device, cudaStream_t s);
// The same for the columns x_lo <= x < x_hi only; the FP32 forms take FP32
// host-order data (widened exactly on the way in, rounded to nearest on the
// way out) for the single-precision field entry points.
cudaError_t reorder_cols(const Geom& g, const double* in, double* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s);
cudaError_t reorder_cols(const Geom& g, const float* in, double* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s);
cudaError_t reorder_cols(const Geom& g, const double* in, float* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s);
cudaError_t reorder_cols(const Geom& g, const float* in, float* out, int ncomp,
                         int layout, int to_device, int x_lo, int x_hi, cudaStream_t s);

// Launches the bounded-wait self-test kernel (one mbarrier nobody arrives
// at): *err (device-visible) gets kErrWaitTimeout after limit_s, *waited_ns
// (device-visible) the time waited.
cudaError_t bounded_wait_selftest(int* err, double limit_s, unsigned long long* waited_ns,
                                  cudaStream_t s);

// Sets the message lbm_last_error() returns on this thread.
void record_error(const std::string& msg);

}  // namespace lbm
