// C-ABI of liblbm_gb300.so (declarations and documentation: include/lbm_gb300.h).
//
// The handle owns every device allocation of one case.  All arguments are
// validated on the host before any device work: in particular every bulk node
// (a node without a link record) must have its eight neighbours inside the
// grid and fluid, and every link source/aux index must be a valid fluid node,
// so the fused kernel never reads outside its arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "lbm_gb300.h"
#include "lbm_internal.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// 64-bit FNV-1a over n bytes, continuing from h.
uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}
constexpr uint64_t kFnvSeed = 14695981039346656037ull;

#define LBM_CUDA(expr)                                                         \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return fail(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kGraphChunk = 32;   // steps per captured graph (even)
constexpr int kTailGraphs = 4;    // graphs of fewer steps kept (the remainder of a call)
constexpr int kResRing = 8;       // residual steps whose sums stay readable
constexpr int kCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
constexpr int kCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

}  // namespace

namespace lbm {
void record_error(const std::string& msg) { g_err = msg; }
}  // namespace lbm

struct LbmHandle {
  LbmConfig cfg{};
  const lbm::KernelSet* ks = nullptr;
  lbm::Geom g{};
  lbm::Params p{};
  cudaStream_t stream = nullptr;
  // host transfers in column chunks: copies on `xfer`, transposes on `stream`
  static constexpr int kXferChunks = 4;
  cudaStream_t xfer = nullptr;
  cudaEvent_t xev[kXferChunks + 1] = {};
  std::vector<std::pair<void*, size_t>> allocs;   // device allocations and their sizes
  size_t dev_bytes = 0;
  void* pop[2] = {nullptr, nullptr};      // first population plane
  void* pop_raw[2] = {nullptr, nullptr};  // allocation (one guard row each side)
  void* side[2] = {nullptr, nullptr};
  void* mom[3] = {nullptr, nullptr, nullptr};
  void* old[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // two sets of rho, ux, uy
  int old_cur = 0;             // set holding the previous residual step's fields
  void* body = nullptr;
  float* omega_seg = nullptr;  // optional per-segment relaxation rate
  double* partials = nullptr;
  double* red = nullptr;       // device [16]: residual sums, conservation sums
  double* scratch = nullptr;   // device [kFinishScratch]: block sums and the last-block counter
  double* host_red = nullptr;  // pinned [16 + 8 kResRing]: sums; residual ring
  double* host_red_dev = nullptr;   // host_red as the device addresses it
  // The sums of the last kResRing residual steps, each in its own slot of
  // host_red (8 words from word 16 on), with the event recorded after its
  // reduction and its time step (-1: empty): a step's residual can be read
  // while later steps run.
  cudaEvent_t res_ev[kResRing] = {};
  int64_t res_t[kResRing] = {-1, -1, -1, -1, -1, -1, -1, -1};
  int64_t res_seq = 0;
  double* stage = nullptr;     // device FP64 staging
  size_t stage_elems = 0;
  int cur = 0;                 // AA layout: both pop[] are one buffer; cur 0 = next step even
  bool aa = false;             // LBM_POP_AA
  bool initialized = false, nopull = true, has_moments = false, has_residual = false;
  int64_t t = 0, launches = 0;
  cudaGraphExec_t gexec = nullptr;
  int gparity = 0;
  // graphs of 2 .. kGraphChunk - 1 plain steps, by step count and starting
  // buffer parity, the most recent kTailGraphs kept
  struct TailGraph {
    int count = 0, parity = 0;
    cudaGraphExec_t exec = nullptr;
  };
  TailGraph tails[kTailGraphs];
  int tail_next = 0;
  lbm::Variant variant{0, 1, 256, 0};
  lbm::Variant res_variant{0, 1, 256, 0};   // shape of residual steps (tuned on the first)
  bool res_tuned = false;
  int sms = 1;                 // multiprocessors of the device
  bool host_link = false;      // kernels may read / write the caller's pinned buffers directly
  int* err_host = nullptr;     // mapped pinned word the kernels set on a failed wait
  int* err_dev = nullptr;
  bool tuned = false;
  double tune_ms[lbm::kMaxVariants] = {};
  // hashes of what a saved state depends on besides the sizes: node classes,
  // link table and relaxation parameters (lbm_create); the omega map
  uint64_t case_hash = 0, omega_hash = 0;
  double timeout_s = 600.0;
  // host copies kept for the adjoint set-up
  std::vector<uint8_t> h_cls;
  std::vector<LbmNodeLinks> h_links;
  // adjoint workspace (allocated by the first lbm_adjoint_forward)
  struct Adj {
    bool tables = false;
    std::string unsupported;       // non-empty: why the adjoint is unavailable
    int* tr_reader = nullptr;
    int8_t* tr_self = nullptr;
    int8_t* wall_rec = nullptr;
    int64_t T = 0;
    int interval = 0;
    std::vector<void*> ckpt, ckpt_side;
    // two sets of interval-1 recomputed states: the backward recomputes the
    // next segment into one set (on `aux`) while the reverse steps read the other
    std::vector<void*> seg, seg_side;
    cudaStream_t aux = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // fork, join, R[2], A[2]
    void* a[2] = {nullptr, nullptr};
    void* gF = nullptr;
    double* gpart = nullptr;
    double* grad_u = nullptr;      // [2][plane]
    long long nparts = 0;
    bool ready = false;
    // both passes are captured once per (T, interval) plan and replayed
    cudaGraphExec_t fwd_graph = nullptr, bwd_graph = nullptr;
    int64_t graph_T = -1;
    int graph_interval = -1;
  } adj;
  // moving obstacles (lbm_set_moving_obstacles)
  struct Mov {
    int n = 0;
    int side = 0;                    // raster launch covers side x side nodes
    lbm::MovObs* obs = nullptr;      // device state
    std::vector<lbm::MovObs> init;   // registered state (restored by lbm_init_fields)
    uint8_t* dsolid = nullptr;
    uint8_t* fresh = nullptr;
    void* us = nullptr;
    void* rho_dyn[2] = {nullptr, nullptr};   // swapped with the population buffers
    double* part = nullptr;          // momentum-exchange partial sums
    uint8_t* cls_static = nullptr;   // classes / segment flags without moving obstacles
    uint8_t* seg_static = nullptr;
    double gx = 0.0, gy = 0.0;
  } mov;
  // momentum-exchange links (lbm_set_force_links)
  struct Force {
    long long* node = nullptr;
    int* rec = nullptr;
    int8_t* kk = nullptr;
    double* arm = nullptr;
    int* gstart = nullptr;
    double* out = nullptr;
    int ngroups = 0;
    int64_t n = 0;
  } force;

  // frees one allocation of this handle
  void release(void* q) {
    if (!q) return;
    for (auto it = allocs.begin(); it != allocs.end(); ++it)
      if (it->first == q) {
        cudaFree(q);
        dev_bytes -= it->second;
        allocs.erase(it);
        return;
      }
  }

  ~LbmHandle() {
    drop_graphs();
    if (adj.fwd_graph) cudaGraphExecDestroy(adj.fwd_graph);
    if (adj.bwd_graph) cudaGraphExecDestroy(adj.bwd_graph);
    for (cudaEvent_t e : adj.ev)
      if (e) cudaEventDestroy(e);
    if (adj.aux) cudaStreamDestroy(adj.aux);
    for (cudaEvent_t e : xev)
      if (e) cudaEventDestroy(e);
    if (xfer) cudaStreamDestroy(xfer);
    for (auto& a : allocs) cudaFree(a.first);
    for (cudaEvent_t e : res_ev)
      if (e) cudaEventDestroy(e);
    if (host_red) cudaFreeHost(host_red);
    if (err_host) cudaFreeHost(err_host);
    if (stream) cudaStreamDestroy(stream);
  }

  int alloc(void** p, size_t bytes) {
    if (std::getenv("LBM_FAIL_ALLOC"))
      return fail(LBM_ERR_ALLOC, "device allocation refused (LBM_FAIL_ALLOC is set)");
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(LBM_ERR_ALLOC, "cudaMalloc(" + std::to_string(bytes) +
                                     " bytes): " + cudaGetErrorString(e));
    }
    allocs.emplace_back(*p, bytes);
    dev_bytes += bytes;
    return LBM_OK;
  }

  void clear_residuals() {
    has_residual = false;
    for (int64_t& v : res_t) v = -1;
  }
  double* res_slot(int i) const { return host_red + 16 + 8 * i; }

  // Waits for the handle's stream (or, given one, for an event on it).
  int wait(cudaEvent_t ev = nullptr) {
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      cudaError_t e = ev ? cudaEventQuery(ev) : cudaStreamQuery(stream);
      if (e == cudaSuccess) {
        if (err_host && *reinterpret_cast<volatile int*>(err_host) != 0) {
          const int code = *reinterpret_cast<volatile int*>(err_host);
          *err_host = 0;
          if (code == lbm::kErrMovBounds)
            return fail(LBM_ERR_STATE, "a moving obstacle would come within two nodes of the domain edge; "
                                       "it was left where it was");
          if (code == lbm::kErrMovSpeed)
            return fail(LBM_ERR_STATE, "a moving obstacle would move a node or more in one step; "
                                       "it was left where it was");
          if (code == lbm::kErrMovNeighbour)
            return fail(LBM_ERR_STATE, "a moving obstacle reached a boundary node or a static solid");
          return fail(LBM_ERR_TIMEOUT, "a bounded mbarrier wait in the step kernel expired");
        }
        return LBM_OK;
      }
      if (e != cudaErrorNotReady)
        return fail(LBM_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
      double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (el > timeout_s)
        return fail(LBM_ERR_TIMEOUT, "device work did not finish within " +
                                         std::to_string(timeout_s) + " s");
      // spin for the first 1 ms: a yield can hand the core to another
      // runnable thread for a whole time slice on a busy host, a sleep costs
      // ~50 us of timer slack, and a step takes 0.2 ms.  Then yield up to
      // 5 ms, then poll every 200 us.
      if (el < 0.001)
        continue;
      if (el < 0.005)
        std::this_thread::yield();
      else
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
  }

  // The copy stream and events of the chunked host transfers.
  int ensure_xfer() {
    if (xfer) return LBM_OK;
    cudaStream_t st = nullptr;
    LBM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (cudaEvent_t& e : xev) {
      const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      if (r != cudaSuccess) {
        cudaStreamDestroy(st);
        return fail(LBM_ERR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(r));
      }
    }
    xfer = st;
    return LBM_OK;
  }
  // First column of transfer chunk c (c = kXferChunks gives nx): multiples of
  // the 32-column transpose tile.
  int xfer_col(int c) const {
    const int w = ((cfg.nx + kXferChunks - 1) / kXferChunks + 31) / 32 * 32;
    return std::min(cfg.nx, c * w);
  }

  int ensure_stage(size_t elems) {
    if (stage_elems >= elems) return LBM_OK;
    if (stage) {
      LBM_CUDA(cudaStreamSynchronize(stream));
      release(stage);
      stage = nullptr;
      stage_elems = 0;
    }
    int rc = alloc(reinterpret_cast<void**>(&stage), elems * sizeof(double));
    if (rc) return rc;
    stage_elems = elems;
    return LBM_OK;
  }

  // Device address of a caller's pinned (page-locked or registered) host
  // buffer, which the transposing copy kernels then read or write directly
  // over the host link: one pass instead of a copy into a staging buffer and
  // a second pass.  Only where the device can also reach pageable memory
  // (Grace-Blackwell's coherent link), so that any host address it is given
  // stays reachable.  nullptr: stage through a copy.
  template <class P>
  P* host_direct(P* q) const {
    if (!host_link) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return at.type == cudaMemoryTypeHost && at.devicePointer ? static_cast<P*>(at.devicePointer) : nullptr;
  }

  long long host_nodes(int layout) const {
    return layout == LBM_LAYOUT_PADDED ? (long long)(cfg.nx + 2) * (cfg.ny + 2)
                                       : (long long)cfg.nx * cfg.ny;
  }

  // One fused step launch; advance=false leaves the state untouched (the
  // kernel only writes the other population buffer and side array).
  int launch(int flags, bool advance = true) {
    return launch_v(flags, (flags & lbm::F_RESIDUAL) && res_tuned ? res_variant : variant, advance);
  }

  // Shape of residual steps: a residual step runs the scalar kernel's
  // residual instantiation, whose best shape can differ from the plain
  // step's.  Times every scalar candidate on the live state without
  // advancing it (the other population buffer, side array and the residual's
  // output set are written, all rewritten by the real step).
  int tune_residual() {
    res_tuned = true;
    res_variant = variant;
    if (aa || std::getenv("LBM_VARIANT")) return LBM_OK;
    const char* t = std::getenv("LBM_TUNE");
    if (t && t[0] == '0') return LBM_OK;
    cudaEvent_t e0, e1;
    LBM_CUDA(cudaEventCreate(&e0));
    LBM_CUDA(cudaEventCreate(&e1));
    double best = 1e30;
    int rc = LBM_OK;
    for (int pass = 0; pass < 2 && rc == LBM_OK; ++pass)
      for (int i = 0; i < ks->nvariants && rc == LBM_OK; ++i) {
        const lbm::Variant v = ks->variants[i];
        // every kernel has a residual instantiation; moving obstacles take
        // the scalar one or the 40-register pairs
        if (mov.n && !mov_ok(v)) continue;
        if ((rc = launch_v(lbm::F_RESIDUAL, v, false))) break;
        cudaEventRecord(e0, stream);
        for (int r = 0; r < 4 && rc == LBM_OK; ++r) rc = launch_v(lbm::F_RESIDUAL, v, false);
        cudaEventRecord(e1, stream);
        if (rc == LBM_OK) rc = wait();
        float ms = 0.f;
        if (rc == LBM_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms < best) {
          best = ms;
          res_variant = v;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }

  int launch_v(int flags, lbm::Variant v, bool advance) {
    const int rc = launch_bufs(flags, v, pop[cur], pop[cur ^ 1], side[cur], side[cur ^ 1], nullptr,
                               mov.rho_dyn[cur], mov.rho_dyn[cur ^ 1], aa ? (cur == 0 ? 1 : 2) : 0);
    if (rc == LBM_OK && advance) cur ^= 1;
    return rc;
  }

  // One fused step from `fin` / `side_in` into `fout` / `side_out`.
  int launch_bufs(int flags, lbm::Variant v, const void* fin, void* fout, const void* sin,
                  void* sout, cudaStream_t on = nullptr, const void* rdin = nullptr,
                  void* rdout = nullptr, int aa_phase = 0) {
    lbm::StepArgs a;
    a.g = g;
    a.p = p;
    a.fin = fin;
    a.fout = fout;
    a.side_in = sin;
    a.side_out = sout;
    a.rho = mom[0];
    a.ux = mom[1];
    a.uy = mom[2];
    a.rho_old = old[3 * old_cur];
    a.ux_old = old[3 * old_cur + 1];
    a.uy_old = old[3 * old_cur + 2];
    a.rho_new = old[3 * (old_cur ^ 1)];
    a.ux_new = old[3 * (old_cur ^ 1) + 1];
    a.uy_new = old[3 * (old_cur ^ 1) + 2];
    a.partials = partials;
    a.body = body;
    a.err = err_dev;
    a.omega_seg = omega_seg;
    a.dsolid = mov.dsolid;
    a.us = mov.us;
    a.rho_dyn_in = rdin;
    a.rho_dyn_out = rdout;
    a.aa = aa_phase;
    a.flags = flags;
    lbm::fill_offsets(a, ks->elem_bytes);
    LBM_CUDA(ks->step(cfg.collision, cfg.forcing, a, v, sms, on ? on : stream));
    return LBM_OK;
  }

  // Transpose of the link table: for every boundary node s and direction m,
  // the node that pulls p(s)_m (or -1) and whether s itself bounces it back.
  int build_adjoint_tables() {
    if (adj.tables) return adj.unsupported.empty() ? LBM_OK : fail(LBM_ERR_ARG, adj.unsupported);
    adj.tables = true;
    if (cfg.collision != LBM_BGK) adj.unsupported = "adjoint: only BGK collision is supported";
    if (mov.n) adj.unsupported = "adjoint: moving obstacles are not supported";
    if (!ks->adjoint) adj.unsupported = "adjoint: FP64 or FP32-shifted storage is required";
    const int nx = g.nx, ny = g.ny, pitch = g.pitch;
    auto dev = [&](int64_t node) { return (long long)(node % ny + 1) * pitch + node / ny; };
    const int64_t nrec = (int64_t)h_links.size();
    std::unordered_map<long long, int> rec_of;   // device node -> record
    for (int64_t r = 0; r < nrec; ++r) rec_of[dev(h_links[r].node)] = (int)r;
    std::unordered_map<long long, long long> reader;   // (src dev)*9+k -> reader dev
    for (int64_t r = 0; r < nrec && adj.unsupported.empty(); ++r) {
      const LbmNodeLinks& L = h_links[r];
      const long long y = dev(L.node);
      for (int k = 1; k < 9; ++k) {
        if (L.type[k] == LBM_LINK_ABB) {
          adj.unsupported = "adjoint: anti-bounce-back (fixed_pressure) links are not supported";
          break;
        }
        if (L.type[k] != LBM_LINK_PULL) continue;
        const long long key = dev(L.src[k]) * 9 + k;
        if (!reader.emplace(key, y).second) {
          adj.unsupported = "adjoint: a population is pulled by two nodes (zero_gradient) - not supported";
          break;
        }
        // a plain in-grid neighbour must be the standard source
        const long long yx = L.node / ny, yy = L.node % ny;
        const long long sx = yx - kCX[k], sy = yy - kCY[k];
        if (sx >= 0 && sx < nx && sy >= 0 && sy < ny && dev(L.src[k]) != (sy + 1) * pitch + sx) {
          adj.unsupported = "adjoint: a link pulls from a node other than its neighbour - not supported";
          break;
        }
      }
    }
    if (!adj.unsupported.empty()) return fail(LBM_ERR_ARG, adj.unsupported);
    const size_t n9 = 9 * std::max<int64_t>(nrec, 1);
    std::vector<int> trr(n9, -1);
    std::vector<int8_t> trs(n9, 0), wr(std::max<int64_t>(nrec, 1), 0);
    static const int inv[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
    for (int64_t r = 0; r < nrec; ++r) {
      const LbmNodeLinks& L = h_links[r];
      const long long s = dev(L.node);
      const long long sx = L.node / ny, sy = L.node % ny;
      wr[r] = L.wall;
      trr[9 * r] = (int)s;   // the rest population stays at the node
      for (int m = 1; m < 9; ++m) {
        const long long yx = sx + kCX[m], yy = sy + kCY[m];
        long long rd = -1;
        if (yx >= 0 && yx < nx && yy >= 0 && yy < ny && h_cls[(yy + 1) * pitch + yx] == 0) {
          rd = (yy + 1) * pitch + yx;   // bulk neighbour
        } else {
          auto it = reader.find(s * 9 + m);
          if (it != reader.end()) rd = it->second;
        }
        trr[9 * r + m] = (int)rd;
        const int tb = L.type[inv[m]];
        trs[9 * r + m] = (tb == LBM_LINK_BB || tb == LBM_LINK_MBB) ? 1 : 0;
      }
    }
    int rc;
    if ((rc = alloc(reinterpret_cast<void**>(&adj.tr_reader), n9 * sizeof(int))) ||
        (rc = alloc(reinterpret_cast<void**>(&adj.tr_self), n9)) ||
        (rc = alloc(reinterpret_cast<void**>(&adj.wall_rec), wr.size())))
      return rc;
    LBM_CUDA(cudaMemcpyAsync(adj.tr_reader, trr.data(), n9 * sizeof(int), cudaMemcpyHostToDevice, stream));
    LBM_CUDA(cudaMemcpyAsync(adj.tr_self, trs.data(), n9, cudaMemcpyHostToDevice, stream));
    LBM_CUDA(cudaMemcpyAsync(adj.wall_rec, wr.data(), wr.size(), cudaMemcpyHostToDevice, stream));
    return wait();
  }

  // The residual's two sets of previous-step fields, allocated (zero, as
  // after lbm_init_fields) by the first step that asks for a residual: runs
  // without one keep six planes of compute type free.
  int ensure_old() {
    if (old[0]) return LBM_OK;
    const size_t bytes = (size_t)g.plane * ks->compute_bytes;
    for (int i = 0; i < 6; ++i) {
      void* q = nullptr;
      int rc = alloc(&q, bytes);
      if (rc) {
        for (int j = 0; j < i; ++j) {
          release(old[j]);
          old[j] = nullptr;
        }
        return rc;
      }
      old[i] = q;
      LBM_CUDA(cudaMemsetAsync(old[i], 0, bytes, stream));
    }
    old_cur = 0;
    return LBM_OK;
  }

  // Where the post-collision populations of the current state sit
  // (lbm::aa_post_index): 0 two buffers or freshly set, 1 after an even AA
  // phase, 2 after an odd one.
  int aa_state() const { return !aa || nopull ? 0 : (cur == 1 ? 1 : 2); }

  size_t state_bytes() const { return (9 * g.plane + 2 * g.pitch) * (size_t)ks->elem_bytes; }
  size_t side_bytes() const { return 3 * (size_t)std::max(g.nrec, 1) * ks->compute_bytes; }

  // state buffers hold a guard row before plane 0, like pop_raw
  void* state_base(void* raw) const { return static_cast<char*>(raw) + g.pitch * ks->elem_bytes; }

  // Captures the work `enqueue` puts on the stream into an executable graph.
  template <class F>
  int capture(cudaGraphExec_t* out, F&& enqueue) {
    cudaGraph_t graph = nullptr;
    LBM_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue();
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      *out = nullptr;
      return fail(LBM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    return LBM_OK;
  }

  // Kernels that handle moving obstacles (class-4 links on the per-node path,
  // the densities their bounce-back reads): the scalar kernel, and the
  // node-pair kernel's 40-register shape, whose flagged segments take the
  // scalar body.
  bool mov_ok(lbm::Variant v) const {
    return v.kind == 0 || (v.kind == 3 && v.vec == 2 && v.stages == 1);
  }

  // The node-pair tile kernel in the AA layout: shifted storage, two pairs
  // of a tile per thread, 1 to kMaxTileStages stages, no moving obstacles.
  bool aa_tile_ok(lbm::Variant v) const {
    return cfg.precision != LBM_FP64 && !mov.n && v.kind == 2 && v.vec == 2 &&
           v.block == lbm::kTileBytes / (4 * ks->elem_bytes) && v.stages >= 1 &&
           v.stages <= lbm::kMaxTileStages;
  }

  // Register cap of the scalar AA kernel (0 none for FP64; shifted storage:
  // 1 (32 registers) for BGK, 2 (40) for MRT).
  int aa_scalar_cap() const {
    return cfg.precision == LBM_FP64 ? 0 : (cfg.collision == LBM_BGK ? 1 : 2);
  }

  long long nparts_of(lbm::Variant v) const {
    const dim3 gr = lbm::step_grid(g, v, sms, ks->elem_bytes, true);   // residual launches
    return (long long)gr.x * gr.y;
  }

  // Times every candidate launch shape on the current state (without
  // advancing it) and keeps the fastest.
  int autotune() {
    tuned = true;
    if (const char* f = std::getenv("LBM_VARIANT")) {
      int kind = -1, vec = 0, blk = 0, st = 0;
      if (aa && std::sscanf(f, "%d,%d,%d,%d", &kind, &vec, &blk, &st) == 4) {
        if (aa_tile_ok(lbm::Variant{kind, vec, blk, st})) {
          variant = lbm::Variant{kind, vec, blk, st};
          return LBM_OK;
        }
        const bool scalar = kind == 0 && vec == 1;
        const bool pairs = kind == 3 && vec == 2 && cfg.precision != LBM_FP64 && st >= 0 && st <= 2;
        if (!(scalar || pairs) || blk < 32 || blk > 256 || blk % 32)
          return fail(LBM_ERR_ARG, std::string("LBM_VARIANT: the AA layout runs the scalar kernel "
                                               "(0,1,block,cap) or, for shifted storage, the node-pair "
                                               "kernel (3,2,block,cap), 32 <= block <= 256, or the tile "
                                               "kernel (2,2,tile/4 bytes,stages): ") + f);
        if (scalar)
          variant = lbm::Variant{0, 1, blk, aa_scalar_cap()};   // the storage's register cap
        else
          variant = lbm::Variant{3, 2, blk, st};
        return LBM_OK;
      }
      if (std::sscanf(f, "%d,%d,%d,%d", &kind, &vec, &blk, &st) == 4) {
        for (int i = 0; i < ks->nvariants; ++i)
          if (ks->variants[i].kind == kind && ks->variants[i].vec == vec &&
              ks->variants[i].block == blk && ks->variants[i].stages == st) {
            if (mov.n && !mov_ok(ks->variants[i]))
              return fail(LBM_ERR_ARG, "LBM_VARIANT: moving obstacles need the scalar kernel (kind 0) "
                                       "or the node-pair kernel with a 40-register cap (3,2,block,1)");
            variant = ks->variants[i];
            return LBM_OK;
          }
        return fail(LBM_ERR_ARG, std::string("LBM_VARIANT does not name a candidate: ") + f);
      }
    }
    if (aa) return LBM_OK;   // in place: a trial launch would advance the state
    variant = ks->variants[0];
    if (mov.n)
      for (int i = 0; i < ks->nvariants; ++i)
        if (ks->variants[i].kind == 0 && ks->variants[i].stages == 0) {
          variant = ks->variants[i];
          break;
        }
    const char* t = std::getenv("LBM_TUNE");
    if (t && t[0] == '0') return LBM_OK;
    const int flags = 0;
    cudaEvent_t e0, e1;
    LBM_CUDA(cudaEventCreate(&e0));
    LBM_CUDA(cudaEventCreate(&e1));
    double best = 1e30;
    int rc = LBM_OK;
    for (int i = 0; i < ks->nvariants && rc == LBM_OK; ++i) {
      const lbm::Variant v = ks->variants[i];
      if (mov.n && !mov_ok(v)) {   // class-4 links: the scalar kernel or 40-register pairs
        tune_ms[i] = 1e30;
        continue;
      }
      if ((rc = launch_v(flags, v, false))) break;
      cudaEventRecord(e0, stream);
      for (int r = 0; r < 3 && rc == LBM_OK; ++r) rc = launch_v(flags, v, false);
      cudaEventRecord(e1, stream);
      if (rc == LBM_OK) rc = wait();
      float ms = 0.f;
      if (rc == LBM_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
        tune_ms[i] = ms / 3.0;
        if (ms < best) {
          best = ms;
          variant = v;
        }
      }
    }
    // second pass: the three fastest again, 8 launches each, interleaved
    // twice, keeping each one's better mean (one short timing can be off by
    // a clock ramp or a neighbour's burst)
    if (rc == LBM_OK && ks->nvariants > 1) {
      int order[lbm::kMaxVariants];
      for (int i = 0; i < ks->nvariants; ++i) order[i] = i;
      std::sort(order, order + ks->nvariants, [&](int x, int y) { return tune_ms[x] < tune_ms[y]; });
      const int top = std::min(3, ks->nvariants);
      double refined[3] = {1e30, 1e30, 1e30};
      for (int pass = 0; pass < 2 && rc == LBM_OK; ++pass)
        for (int j = 0; j < top && rc == LBM_OK; ++j) {
          const lbm::Variant v = ks->variants[order[j]];
          cudaEventRecord(e0, stream);
          for (int r = 0; r < 8 && rc == LBM_OK; ++r) rc = launch_v(flags, v, false);
          cudaEventRecord(e1, stream);
          if (rc == LBM_OK) rc = wait();
          float ms = 0.f;
          if (rc == LBM_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
            refined[j] = std::min(refined[j], ms / 8.0);
        }
      if (rc == LBM_OK) {
        int bj = 0;
        for (int j = 0; j < top; ++j) {
          tune_ms[order[j]] = refined[j];
          if (refined[j] < refined[bj]) bj = j;
        }
        variant = ks->variants[order[bj]];
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }

  lbm::MovArgs mov_args(int j, int nopull_state) {
    lbm::MovArgs a;
    a.g = g;
    a.p = p;
    a.obs = mov.obs;
    a.n = mov.n;
    a.j = j;
    a.gx = mov.gx;
    a.gy = mov.gy;
    a.dsolid = mov.dsolid;
    a.fresh = mov.fresh;
    a.cls = const_cast<uint8_t*>(g.cls);
    a.segflag = const_cast<uint8_t*>(g.segflag);
    a.us = mov.us;
    a.rho_dyn = mov.rho_dyn[cur];
    a.pop = pop[cur];
    a.mr = mom[0];
    a.mx = mom[1];
    a.my = mom[2];
    a.nopull = nopull_state;
    a.part = mov.part;
    a.err = err_dev;
    return a;
  }

  // Geometry of the moving obstacles for the coming step (motion = false:
  // only place them at their current position, as at initialisation).
  int mov_geometry(bool motion) {
    LBM_CUDA(ks->mov_motion(mov_args(motion ? 0 : -1, 0), stream));
    for (int j = 0; j < mov.n; ++j) LBM_CUDA(ks->mov_raster(mov_args(j, 0), mov.side, stream));
    for (int j = 0; j < mov.n; ++j) LBM_CUDA(ks->mov_classify(mov_args(j, 0), mov.side, stream));
    return LBM_OK;
  }
  int mov_forces(int nopull_state) {
    for (int j = 0; j < mov.n; ++j) LBM_CUDA(ks->mov_force(mov_args(j, nopull_state), stream));
    return LBM_OK;
  }

  // One time step with the moving-obstacle work around the fused step.
  int step_full(int flags) {
    int rc;
    if (mov.n && (rc = mov_geometry(true))) return rc;
    if ((rc = launch(flags))) return rc;
    if (mov.n && (rc = mov_forces(0))) return rc;
    return LBM_OK;
  }

  // Captures `count` plain steps starting from buffer parity `parity` into
  // an executable graph (nothing runs; cur is left as it was).
  int capture_steps(int count, int parity, cudaGraphExec_t* out) {
    cudaGraph_t graph = nullptr;
    *out = nullptr;
    LBM_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int c0 = cur;
    cur = parity;
    int rc = LBM_OK;
    for (int i = 0; i < count && rc == LBM_OK; ++i) rc = step_full(0);
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    cur = c0;
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      *out = nullptr;
      return fail(LBM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    return LBM_OK;
  }

  // The kGraphChunk-step graph, from parity `parity`.
  int capture_graph(int parity) {
    const int rc = capture_steps(kGraphChunk, parity, &gexec);
    if (rc == LBM_OK) gparity = parity;
    return rc;
  }

  // The graph of `count` (2 .. kGraphChunk - 1) plain steps from parity
  // `parity`, captured on first use.
  int tail_graph(int count, int parity, cudaGraphExec_t* out) {
    for (const TailGraph& t : tails)
      if (t.exec && t.count == count && t.parity == parity) {
        *out = t.exec;
        return LBM_OK;
      }
    TailGraph& t = tails[tail_next];
    tail_next = (tail_next + 1) % kTailGraphs;
    if (t.exec) cudaGraphExecDestroy(t.exec);   // freed once a launch in flight ends
    t = TailGraph{};
    const int rc = capture_steps(count, parity, &t.exec);
    if (rc) return rc;
    t.count = count;
    t.parity = parity;
    *out = t.exec;
    return LBM_OK;
  }

  // Graphs hold the kernel arguments and buffer parity of their capture.
  void drop_graphs() {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    for (TailGraph& t : tails) {
      if (t.exec) cudaGraphExecDestroy(t.exec);
      t = TailGraph{};
    }
  }

  // Captures, before a timed call, the graphs an lbm_step(nsteps) from the
  // present state will launch, following the step loop's choices.
  int prepare_graphs(int64_t nsteps) {
    if (std::getenv("LBM_NO_GRAPH") || !tuned || nopull || nsteps < 2) return LBM_OK;
    int64_t plain = nsteps - 1;   // the last step is launched on its own
    int c = cur;
    int rc;
    while (plain > 0) {
      if (plain >= kGraphChunk) {
        if (!gexec && (rc = capture_graph(c))) return rc;
        if (c == gparity) {
          plain -= kGraphChunk;
          continue;
        }
      } else if (plain >= 2) {
        cudaGraphExec_t ex = nullptr;
        return tail_graph((int)plain, c, &ex);
      }
      c ^= 1;
      --plain;
    }
    return LBM_OK;
  }
};

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }

int lbm_create(const LbmConfig* cfg, const uint8_t* node_solid,
               const LbmNodeLinks* links, int64_t nlinks, LbmHandle** out) {
  if (!cfg || !node_solid || !out || (nlinks > 0 && !links) || nlinks < 0)
    return fail(LBM_ERR_ARG, "lbm_create: null argument");
  *out = nullptr;
  const LbmConfig& c = *cfg;
  if (c.nx < 1 || c.ny < 1 || c.ny > 65535 || c.nx > (1 << 26))
    return fail(LBM_ERR_ARG, "lbm_create: grid must satisfy 1 <= nx, 1 <= ny <= 65535");
  if (c.precision < LBM_FP64 || c.precision > LBM_FP16_SHIFTED)
    return fail(LBM_ERR_ARG, "lbm_create: unknown precision");
  if (c.collision != LBM_BGK && c.collision != LBM_MRT)
    return fail(LBM_ERR_ARG, "lbm_create: unknown collision model");
  if (c.forcing < LBM_FORCING_NONE || c.forcing > LBM_GUO_SECOND_ORDER)
    return fail(LBM_ERR_ARG, "lbm_create: unknown forcing model");
  if (!(c.omega > 0.0 && c.omega < 2.0))
    return fail(LBM_ERR_ARG, "lbm_create: omega = 1/tau must lie in (0, 2)");
  if (c.precision == LBM_FP16_SHIFTED && !(c.fp16_scale > 0.0))
    return fail(LBM_ERR_ARG, "lbm_create: fp16_scale must be > 0");
  if (c.layout != LBM_POP_AB && c.layout != LBM_POP_AA)
    return fail(LBM_ERR_ARG, "lbm_create: unknown population layout");
  const bool aa = c.layout == LBM_POP_AA;

  const lbm::KernelSet* ks = c.precision == LBM_FP64 ? &lbm::kernels_fp64()
                             : c.precision == LBM_FP32_SHIFTED ? &lbm::kernels_fp32()
                                                                : &lbm::kernels_fp16();
  const int nx = c.nx, ny = c.ny;
  // rows are multiples of 4096 B for shifted storage (whole 2048-byte tiles
  // of the tile kernel), 512 B for FP64.
  // AA layout (scalar kernel only): 128-byte rows with at least one padding
  // column, which receives the pushes across the x edges.
  const int align = (aa ? 128 : c.precision == LBM_FP64 ? 512 : lbm::kTmaRowBytes) / ks->elem_bytes;
  const int pitch = ((aa ? nx + 1 : nx) + align - 1) / align * align;
  const long long plane = (long long)(ny + 2) * pitch;
  if (plane >= (1LL << 31) / 1)
    return fail(LBM_ERR_ARG, "lbm_create: grid too large (ny*pitch must be < 2^31)");
  const long long nin = (long long)nx * ny;

  // ---- host-side geometry and link table --------------------------------
  auto dnode = [&](long long x, long long y) { return (y + 1) * pitch + x; };
  std::vector<uint8_t> cls(plane, 3);   // 3: padding row / column
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y)
      cls[dnode(x, y)] = node_solid[(long long)x * ny + y] ? 2 : 0;
  std::vector<int> recmap(plane, -1);
  for (int64_t r = 0; r < nlinks; ++r) {
    const int64_t node = links[r].node;
    if (node < 0 || node >= nin)
      return fail(LBM_ERR_ARG, "lbm_create: link record " + std::to_string(r) + " has node out of range");
    const long long dn = dnode(node / ny, node % ny);
    if (cls[dn] == 2)
      return fail(LBM_ERR_ARG, "lbm_create: link record for a solid node " + std::to_string(node));
    if (recmap[dn] >= 0)
      return fail(LBM_ERR_ARG, "lbm_create: node " + std::to_string(node) + " has two link records");
    recmap[dn] = (int)r;
    cls[dn] = 1;
  }
  std::vector<int8_t> rtype(9 * std::max<int64_t>(nlinks, 1), 0);
  std::vector<int> rsrc(9 * std::max<int64_t>(nlinks, 1), 0), raux(9 * std::max<int64_t>(nlinks, 1), 0);
  std::vector<double> rparam(9 * std::max<int64_t>(nlinks, 1), 0.0);
  for (int64_t r = 0; r < nlinks; ++r) {
    const LbmNodeLinks& L = links[r];
    for (int k = 0; k < 9; ++k) {
      const int ty = L.type[k];
      const size_t li = 9 * r + k;
      rtype[li] = (int8_t)ty;
      rparam[li] = L.param[k];
      if (k == 0) continue;  // the rest population is always the node's own
      if (ty == LBM_LINK_PULL) {
        const int64_t s = L.src[k];
        if (s < 0 || s >= nin)
          return fail(LBM_ERR_ARG, "lbm_create: PULL source out of range at node " + std::to_string(L.node));
        const long long ds = dnode(s / ny, s % ny);
        if (cls[ds] == 2)
          return fail(LBM_ERR_ARG, "lbm_create: PULL source is solid at node " + std::to_string(L.node));
        rsrc[li] = (int)ds;
      } else if (ty == LBM_LINK_ABB) {
        const int64_t s = L.aux[k];
        if (s < 0 || s >= nin)
          return fail(LBM_ERR_ARG, "lbm_create: ABB neighbour out of range at node " + std::to_string(L.node));
        const long long ds = dnode(s / ny, s % ny);
        if (recmap[ds] < 0)
          return fail(LBM_ERR_ARG, "lbm_create: ABB neighbour " + std::to_string(s) +
                                       " of node " + std::to_string(L.node) + " has no link record");
        raux[li] = recmap[ds];
      } else if (ty != LBM_LINK_ZERO && ty != LBM_LINK_BB && ty != LBM_LINK_MBB) {
        return fail(LBM_ERR_ARG, "lbm_create: unknown link type at node " + std::to_string(L.node));
      }
    }
  }
  // every bulk node must have in-grid fluid neighbours
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      if (cls[dnode(x, y)] != 0) continue;
      for (int k = 1; k < 9; ++k) {
        const int xs = x - kCX[k], ys = y - kCY[k];
        if (xs < 0 || xs >= nx || ys < 0 || ys >= ny || cls[dnode(xs, ys)] == 2)
          return fail(LBM_ERR_ARG, "lbm_create: node (" + std::to_string(x) + "," +
                                       std::to_string(y) + ") borders the grid edge or a solid but has no link record");
      }
    }
  // AA layout: a thread's in-place reads and writes must not meet another
  // node's.  A non-pull link of direction k reads a slot that the node's
  // neighbour x - c_k would write, so that neighbour must be solid or outside
  // the grid; a pull from s reads a slot that the node s + c_k would write,
  // so that node must be the puller itself, solid or outside the grid.
  if (aa)
    for (int64_t r = 0; r < nlinks; ++r) {
      const LbmNodeLinks& L = links[r];
      const long long x = L.node / ny, y = L.node % ny;
      for (int k = 1; k < 9; ++k) {
        long long tx, ty;
        if (L.type[k] == LBM_LINK_PULL) {
          tx = L.src[k] / ny + kCX[k];
          ty = L.src[k] % ny + kCY[k];
          if (tx == x && ty == y) continue;
        } else if (L.type[k] == LBM_LINK_ZERO) {
          continue;
        } else {
          tx = x - kCX[k];
          ty = y - kCY[k];
        }
        if (tx >= 0 && tx < nx && ty >= 0 && ty < ny && cls[dnode(tx, ty)] != 2)
          return fail(LBM_ERR_ARG, "lbm_create: AA layout: link " + std::to_string(k) + " of node (" +
                                       std::to_string(x) + "," + std::to_string(y) +
                                       ") reads a population another fluid node overwrites in place "
                                       "(zero_gradient or an inner boundary); use the two-buffer layout");
      }
    }
  const int nseg = (nx + 31) / 32;
  std::vector<uint8_t> segflag((size_t)ny * nseg, 0);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x)
      if (cls[dnode(x, y)]) segflag[(size_t)y * nseg + x / 32] = 1;
  std::vector<int> seglist;
  for (size_t i = 0; i < segflag.size(); ++i)
    if (segflag[i]) seglist.push_back((int)i);

  // ---- device --------------------------------------------------------------
  LbmHandle* h = new LbmHandle();
  h->cfg = c;
  h->ks = ks;
  h->h_cls = cls;
  h->h_links.assign(links, links + nlinks);
  {   // field by field: the records' padding bytes are not part of the case
    uint64_t hs = fnv1a(kFnvSeed, cls.data(), cls.size());
    for (const LbmNodeLinks& L : h->h_links) {
      hs = fnv1a(hs, &L.node, sizeof L.node);
      hs = fnv1a(hs, L.src, sizeof L.src);
      hs = fnv1a(hs, L.aux, sizeof L.aux);
      hs = fnv1a(hs, L.param, sizeof L.param);
      hs = fnv1a(hs, L.type, sizeof L.type);
      hs = fnv1a(hs, &L.wall, sizeof L.wall);
    }
    const double rel[] = {c.omega, c.inv_cs_2, c.inv_cs_4, c.eps, c.gravity[0], c.gravity[1],
                          c.mrt_s[0], c.mrt_s[1], c.mrt_s[2], c.mrt_s[3], c.fp16_scale};
    h->case_hash = fnv1a(hs, rel, sizeof rel);
  }
  auto bail = [&](int rc) {
    delete h;
    return rc;
  };
  if (std::getenv("LBM_FAIL_ALLOC")) return bail(fail(LBM_ERR_ALLOC, "device allocation refused (LBM_FAIL_ALLOC is set)"));
  cudaError_t e = cudaSetDevice(c.device);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e)));
  // the handle's stream at the highest priority (the adjoint's recompute
  // stream runs below it)
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  e = cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_hi);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)));

  lbm::Geom& g = h->g;
  g.nx = nx;
  g.ny = ny;
  g.pitch = pitch;
  g.nseg = nseg;
  g.plane = plane;
  g.nrec = (int)nlinks;
  const size_t eb = ks->elem_bytes, cb = ks->compute_bytes;
  const size_t nrec1 = std::max<int64_t>(nlinks, 1);
  void *d_cls, *d_seg, *d_seglist, *d_recmap, *d_rtype, *d_rsrc, *d_rparam, *d_raux, *d_rpf;
  std::vector<float2> rpf(rparam.size());
  for (size_t i = 0; i < rparam.size(); ++i)
    rpf[i] = make_float2((float)rparam[i], (float)(rparam[i] - 1.0));
  int rc;
  if ((rc = h->alloc(&d_cls, plane)) || (rc = h->alloc(&d_seg, segflag.size())) ||
      (rc = h->alloc(&d_seglist, std::max<size_t>(seglist.size(), 1) * sizeof(int))) ||
      (rc = h->alloc(&d_recmap, plane * sizeof(int))) || (rc = h->alloc(&d_rtype, 9 * nrec1)) ||
      (rc = h->alloc(&d_rsrc, 9 * nrec1 * sizeof(int))) ||
      (rc = h->alloc(&d_rparam, 9 * nrec1 * sizeof(double))) ||
      (rc = h->alloc(&d_rpf, 9 * nrec1 * sizeof(float2))) ||
      (rc = h->alloc(&d_raux, 9 * nrec1 * sizeof(int))) ||
      (rc = h->alloc(&h->pop_raw[0], (9 * plane + 2 * pitch) * eb)) ||
      (!aa && (rc = h->alloc(&h->pop_raw[1], (9 * plane + 2 * pitch) * eb))) ||
      (rc = h->alloc(&h->side[0], 3 * nrec1 * cb)) || (rc = h->alloc(&h->side[1], 3 * nrec1 * cb)))
    return bail(rc);
  // one guard row before and after the nine planes
  if (aa) h->pop_raw[1] = h->pop_raw[0];
  h->aa = aa;
  for (int i = 0; i < 2; ++i) h->pop[i] = static_cast<char*>(h->pop_raw[i]) + pitch * eb;
  // rho, ux, uy: three consecutive planes of one allocation (u is read back
  // as a two-component array from ux)
  if ((rc = h->alloc(&h->mom[0], 3 * plane * cb))) return bail(rc);
  h->mom[1] = static_cast<char*>(h->mom[0]) + plane * cb;
  h->mom[2] = static_cast<char*>(h->mom[0]) + 2 * plane * cb;
  e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, c.device);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("device attribute: ") + cudaGetErrorString(e)));
  {
    int pageable = 0, same_va = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c.device) != cudaSuccess ||
        cudaDeviceGetAttribute(&same_va, cudaDevAttrCanUseHostPointerForRegisteredMem, c.device) != cudaSuccess) {
      cudaGetLastError();
      pageable = same_va = 0;
    }
    const char* st = std::getenv("LBM_HOST_DIRECT");
    h->host_link = pageable == 1 && same_va == 1 && st && st[0] == '1';
  }
  e = cudaHostAlloc(reinterpret_cast<void**>(&h->err_host), sizeof(int), cudaHostAllocMapped);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_ALLOC, std::string("cudaHostAlloc: ") + cudaGetErrorString(e)));
  *h->err_host = 0;
  e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->err_dev), h->err_host, 0);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("cudaHostGetDevicePointer: ") + cudaGetErrorString(e)));
  h->variant = ks->variants[0];
  if (aa) {
    // no autotuner (a trial launch would advance the state in place): FP64
    // runs the scalar kernel; FP32 the node-pair kernel, 128 threads under a
    // 40-register cap (86.2 GLUPS at 8192x2048 against 82.8 scalar and 76.3
    // from shared-memory tiles); FP16 the node-pair tile kernel, two pairs of
    // a tile per thread, two stages (139.9 against 125.8 node pairs)
    h->variant = c.precision == LBM_FP64            ? lbm::Variant{0, 1, 128, 0}
                 : c.precision == LBM_FP32_SHIFTED ? lbm::Variant{3, 2, 128, 1}
                                                   : lbm::Variant{2, 2, lbm::kTileBytes / 8, 2};
  }
  long long maxparts = ny;
  for (int i = 0; i < ks->nvariants; ++i) maxparts = std::max(maxparts, h->nparts_of(ks->variants[i]));
  if (aa) {
    maxparts = std::max(maxparts, h->nparts_of(lbm::Variant{0, 1, 32, 0}));   // smallest AA block
    if (c.precision != LBM_FP64)   // the AA tile kernel's largest grid (one stage)
      maxparts = std::max(maxparts, h->nparts_of(lbm::Variant{2, 2, lbm::kTileBytes / (4 * (int)eb), 1}));
  }
  if ((rc = h->alloc(reinterpret_cast<void**>(&h->partials), maxparts * 8 * sizeof(double))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&h->red), 16 * sizeof(double))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&h->scratch), lbm::kFinishScratch * sizeof(double))))
    return bail(rc);
  e = cudaMallocHost(reinterpret_cast<void**>(&h->host_red), (16 + 8 * kResRing) * sizeof(double));
  if (e != cudaSuccess) return bail(fail(LBM_ERR_ALLOC, std::string("cudaMallocHost: ") + cudaGetErrorString(e)));
  // the reductions write their results straight into it
  e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->host_red_dev), h->host_red, 0);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("cudaHostGetDevicePointer: ") + cudaGetErrorString(e)));
  for (cudaEvent_t& ev : h->res_ev)
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      return bail(fail(LBM_ERR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e)));
  if ((e = cudaMemsetAsync(h->scratch, 0, lbm::kFinishScratch * sizeof(double), h->stream)) != cudaSuccess)
    return bail(fail(LBM_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));
  g.cls = (const uint8_t*)d_cls;
  g.segflag = (const uint8_t*)d_seg;
  g.seglist = (const int*)d_seglist;
  g.nflag = (int)seglist.size();
  g.recmap = (const int*)d_recmap;
  g.rtype = (const int8_t*)d_rtype;
  g.rsrc = (const int*)d_rsrc;
  g.rparam = (const double*)d_rparam;
  g.rpf = (const float2*)d_rpf;
  g.raux = (const int*)d_raux;
  auto up = [&](void* d, const void* src, size_t bytes) {
    return cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, h->stream);
  };
  if ((e = up(d_cls, cls.data(), plane)) != cudaSuccess ||
      (e = up(d_seg, segflag.data(), segflag.size())) != cudaSuccess ||
      (!seglist.empty() && (e = up(d_seglist, seglist.data(), seglist.size() * sizeof(int))) != cudaSuccess) ||
      (e = up(d_recmap, recmap.data(), plane * sizeof(int))) != cudaSuccess ||
      (e = up(d_rtype, rtype.data(), rtype.size())) != cudaSuccess ||
      (e = up(d_rsrc, rsrc.data(), rsrc.size() * sizeof(int))) != cudaSuccess ||
      (e = up(d_rparam, rparam.data(), rparam.size() * sizeof(double))) != cudaSuccess ||
      (e = up(d_rpf, rpf.data(), rpf.size() * sizeof(float2))) != cudaSuccess ||
      (e = up(d_raux, raux.data(), raux.size() * sizeof(int))) != cudaSuccess)
    return bail(fail(LBM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e)));
  for (int i = 0; i < 2; ++i) {
    if ((e = cudaMemsetAsync(h->pop_raw[i], 0, (9 * plane + 2 * pitch) * eb, h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(h->side[i], 0, 3 * nrec1 * cb, h->stream)) != cudaSuccess)
      return bail(fail(LBM_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));
  }
  for (int i = 0; i < 3; ++i)
    if ((e = cudaMemsetAsync(h->mom[i], 0, plane * cb, h->stream)) != cudaSuccess)
      return bail(fail(LBM_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));

  lbm::Params& p = h->p;
  p.omega = c.omega;
  p.one_m_omega = 1 - c.omega;
  p.one_m_half_omega = 1 - 0.5 * c.omega;
  const bool fp64 = c.precision == LBM_FP64;
  p.inv_cs_2 = fp64 ? c.inv_cs_2 : 3.0;
  p.inv_cs_4 = fp64 ? c.inv_cs_4 : 9.0;
  p.half_inv_cs_2 = 0.5 * p.inv_cs_2;
  p.half_inv_cs_4 = 0.5 * p.inv_cs_4;
  p.eps = c.eps;
  p.gx = c.forcing ? c.gravity[0] : 0.0;
  p.gy = c.forcing ? c.gravity[1] : 0.0;
  p.s_e = c.mrt_s[0];
  p.s_eps = c.mrt_s[1];
  p.s_q = c.mrt_s[2];
  p.s_nu = c.mrt_s[3];
  p.scale = c.precision == LBM_FP16_SHIFTED ? c.fp16_scale : 1.0;
  p.inv_scale = 1.0 / p.scale;
  {
    const double w[3] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0};
    p.f_omega = (float)c.omega;
    for (int i = 0; i < 3; ++i) {
      p.f_wsc[i] = (float)(w[i] * p.scale);
      p.f_omh[i] = (float)((1.0 - 0.5 * c.omega) * w[i] * p.scale);
    }
    p.f_gx = (float)p.gx;
    p.f_gy = (float)p.gy;
    p.f_scale = (float)p.scale;
    p.f_inv_scale = (float)p.inv_scale;
    p.f_i2 = (float)p.inv_cs_2;
    p.f_i4 = (float)p.inv_cs_4;
    p.f_homh = (float)p.one_m_half_omega;
    const double rates[4] = {c.mrt_s[0], c.mrt_s[1], c.mrt_s[2], c.mrt_s[3]};
    const double norm2[4] = {36.0, 36.0, 12.0, 4.0};   // |row|^2 of e, eps, q, nu
    for (int i = 0; i < 4; ++i) {
      p.f_mrt_s[i] = (float)(-rates[i] / norm2[i]);
      p.f_mrt_h[i] = (float)((1.0 - 0.5 * rates[i]) / norm2[i]);
    }
  }
  if (c.body_force_field) {
    if ((rc = h->alloc(&h->body, 2 * plane * cb))) return bail(rc);
    if ((e = cudaMemsetAsync(h->body, 0, 2 * plane * cb, h->stream)) != cudaSuccess)
      return bail(fail(LBM_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));
  }
  if (const char* to = std::getenv("LBM_SYNC_TIMEOUT_S")) h->timeout_s = std::atof(to);
  if ((rc = h->wait())) return bail(rc);
  *out = h;
  return LBM_OK;
}

int lbm_destroy(LbmHandle* h) {
  if (!h) return fail(LBM_ERR_ARG, "lbm_destroy: null handle");
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
  return LBM_OK;
}

extern "C++" {
// Caller fields in host order (HT = double, or float for single-precision
// cases) to the FP64 device-order stage *ds: rho [plane], u [2][plane].
// *inited: the equilibrium was written chunk by chunk as the columns
// arrived (inner layout, staged, no moving obstacles).
template <class HT>
static int fields_to_stage(LbmHandle* h, const HT* rho, const HT* u, int layout, double** ds_out,
                           bool* inited) {
  const long long nh = h->host_nodes(layout), plane = h->g.plane;
  *inited = false;
  const HT* rd = h->host_direct(rho);
  const HT* ud = h->host_direct(u);
  const bool direct = rd && ud;
  // host-order part of the stage, in doubles (none when read in place)
  const long long hn = direct ? 0 : (3 * nh * (long long)sizeof(HT) + 7) / 8;
  int rc = h->ensure_stage(hn + 3 * plane);
  if (rc) return rc;
  h->initialized = false;   // until the new state is complete
  // device order: rho [plane], u [2][plane]; the transposes write every
  // inner node, the only ones the equilibrium kernel reads
  double* ds = h->stage + hn;
  HT* hs = reinterpret_cast<HT*>(h->stage);   // host order: rho [nh], u [nh][2]
  const int nx = h->cfg.nx;
  // the previous residual step's fields restart from zero; they do not
  // depend on the new fields, so they clear while those are copied
  auto clear_old = [&]() -> int {
    for (int i = 0; i < 6; ++i)
      if (h->old[i]) LBM_CUDA(cudaMemsetAsync(h->old[i], 0, plane * h->ks->compute_bytes, h->stream));
    h->old_cur = 0;
    return LBM_OK;
  };
  if (h->aa) h->cur = 0;   // AA: the first step is an even phase
  // with no moving obstacles the classes are static, so the equilibrium of a
  // chunk of columns can be written as soon as the chunk is transposed
  const bool chunk_init = !h->mov.n;
  if (direct) {   // transposed straight from the caller's pinned buffers
    if ((rc = clear_old())) return rc;
    LBM_CUDA(lbm::reorder_cols(h->g, rd, ds, 1, layout, 1, 0, nx, h->stream));
    LBM_CUDA(lbm::reorder_cols(h->g, ud, ds + plane, 2, layout, 1, 0, nx, h->stream));
  } else if (layout == LBM_LAYOUT_INNER) {
    // column chunks: chunk c is copied on the transfer stream while the
    // handle's stream transposes chunk c - 1 (host order is x-major, so the
    // columns x0 <= x < x1 are one contiguous run of each array)
    if ((rc = h->ensure_xfer())) return rc;
    const long long ny = h->cfg.ny;
    constexpr int NC = LbmHandle::kXferChunks;
    LBM_CUDA(cudaEventRecord(h->xev[NC], h->stream));
    LBM_CUDA(cudaStreamWaitEvent(h->xfer, h->xev[NC], 0));
    if ((rc = clear_old())) return rc;   // after the event: the copies need not wait
    for (int c = 0; c < NC; ++c) {
      const int x0 = h->xfer_col(c), x1 = h->xfer_col(c + 1);
      if (x0 >= x1) continue;
      LBM_CUDA(cudaMemcpyAsync(hs + x0 * ny, rho + x0 * ny, (x1 - x0) * ny * sizeof(HT),
                               cudaMemcpyDefault, h->xfer));
      LBM_CUDA(cudaMemcpyAsync(hs + nh + 2 * x0 * ny, u + 2 * x0 * ny, 2 * (x1 - x0) * ny * sizeof(HT),
                               cudaMemcpyDefault, h->xfer));
      LBM_CUDA(cudaEventRecord(h->xev[c], h->xfer));
      LBM_CUDA(cudaStreamWaitEvent(h->stream, h->xev[c], 0));
      LBM_CUDA(lbm::reorder_cols(h->g, hs, ds, 1, layout, 1, x0, x1, h->stream));
      LBM_CUDA(lbm::reorder_cols(h->g, hs + nh, ds + plane, 2, layout, 1, x0, x1, h->stream));
      if (chunk_init)
        LBM_CUDA(h->ks->init(h->g, h->p, ds, ds + plane, h->pop[h->cur], h->mom[0], h->mom[1],
                             h->mom[2], x0, x1, h->stream));
    }
    *inited = chunk_init;
  } else {
    if ((rc = clear_old())) return rc;
    LBM_CUDA(cudaMemcpyAsync(hs, rho, nh * sizeof(HT), cudaMemcpyDefault, h->stream));
    LBM_CUDA(cudaMemcpyAsync(hs + nh, u, 2 * nh * sizeof(HT), cudaMemcpyDefault, h->stream));
    LBM_CUDA(lbm::reorder_cols(h->g, hs, ds, 1, layout, 1, 0, nx, h->stream));
    LBM_CUDA(lbm::reorder_cols(h->g, hs + nh, ds + plane, 2, layout, 1, 0, nx, h->stream));
  }
  *ds_out = ds;
  return LBM_OK;
}

}  // extern "C++"

static int init_from_stage(LbmHandle* h, double* ds, bool inited);

extern "C++" {
template <class HT>
static int init_fields(LbmHandle* h, const HT* rho, const HT* u, int layout, const char* name) {
  if (!h || !rho || !u) return fail(LBM_ERR_ARG, std::string(name) + ": null argument");
  if (layout != LBM_LAYOUT_INNER && layout != LBM_LAYOUT_PADDED)
    return fail(LBM_ERR_ARG, std::string(name) + ": unknown layout");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  double* ds = nullptr;
  bool inited = false;
  int rc = fields_to_stage(h, rho, u, layout, &ds, &inited);
  return rc ? rc : init_from_stage(h, ds, inited);
}

}  // extern "C++"

int lbm_init_fields(LbmHandle* h, const double* rho, const double* u, int layout) {
  return init_fields(h, rho, u, layout, "lbm_init_fields");
}

int lbm_init_fields_f32(LbmHandle* h, const float* rho, const float* u, int layout) {
  return init_fields(h, rho, u, layout, "lbm_init_fields_f32");
}

// Equilibrium populations from the staged fields, then the step state reset.
static int init_from_stage(LbmHandle* h, double* ds, bool inited) {
  const long long plane = h->g.plane;
  int rc;
  if (h->mov.n) {   // static classes back before f_eq is written (a run may have moved obstacles)
    LBM_CUDA(cudaMemcpyAsync(const_cast<uint8_t*>(h->g.cls), h->mov.cls_static, plane,
                             cudaMemcpyDeviceToDevice, h->stream));
    LBM_CUDA(cudaMemcpyAsync(const_cast<uint8_t*>(h->g.segflag), h->mov.seg_static,
                             (size_t)h->g.ny * h->g.nseg, cudaMemcpyDeviceToDevice, h->stream));
  }
  if (!inited)
    LBM_CUDA(h->ks->init(h->g, h->p, ds, ds + plane, h->pop[h->cur], h->mom[0], h->mom[1],
                         h->mom[2], 0, h->cfg.nx, h->stream));
  if (h->mov.n) {
    // registered obstacle state, static classes, then the obstacles placed,
    // their nodes classified and the t = 0 momentum exchange (the reference
    // computes forces before the first step, fluidLB.py:323-335)
    auto& M = h->mov;
    const size_t cb = h->ks->compute_bytes;
    LBM_CUDA(cudaMemcpyAsync(M.obs, M.init.data(), M.n * sizeof(lbm::MovObs), cudaMemcpyHostToDevice,
                             h->stream));
    LBM_CUDA(cudaMemsetAsync(M.dsolid, 0, plane, h->stream));
    LBM_CUDA(cudaMemsetAsync(M.fresh, 0, plane, h->stream));
    LBM_CUDA(cudaMemcpyAsync(M.rho_dyn[h->cur], h->mom[0], plane * cb, cudaMemcpyDeviceToDevice, h->stream));
    if ((rc = h->mov_geometry(false)) || (rc = h->mov_forces(1))) return rc;
  }
  if ((rc = h->wait())) return rc;
  h->initialized = true;
  h->nopull = true;
  h->has_moments = true;
  h->clear_residuals();
  h->t = 0;
  return LBM_OK;
}

int lbm_set_body_force(LbmHandle* h, const double* force) {
  if (!h || !force) return fail(LBM_ERR_ARG, "lbm_set_body_force: null argument");
  if (!h->body) return fail(LBM_ERR_STATE, "lbm_set_body_force: case was created without body_force_field");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const long long nh = h->host_nodes(LBM_LAYOUT_INNER), plane = h->g.plane;
  int rc = h->ensure_stage(2 * nh + 2 * plane);
  if (rc) return rc;
  double* hs = h->stage;
  double* ds = h->stage + 2 * nh;
  LBM_CUDA(cudaMemcpyAsync(hs, force, 2 * nh * sizeof(double), cudaMemcpyDefault, h->stream));
  LBM_CUDA(cudaMemsetAsync(ds, 0, 2 * plane * sizeof(double), h->stream));
  LBM_CUDA(lbm::reorder(h->g, hs, ds, 2, LBM_LAYOUT_INNER, 1, h->stream));
  LBM_CUDA(h->ks->body_from_f64(h->g, ds, h->body, h->stream));
  return h->wait();
}

int lbm_set_omega_map(LbmHandle* h, const double* omega) {
  if (!h || !omega) return fail(LBM_ERR_ARG, "lbm_set_omega_map: null argument");
  if (h->cfg.precision == LBM_FP64 || h->cfg.collision != LBM_BGK)
    return fail(LBM_ERR_ARG, "lbm_set_omega_map: needs BGK with shifted (FP32/FP16) storage");
  const lbm::Geom& g = h->g;
  const int nx = g.nx, ny = g.ny;
  std::vector<float> seg((size_t)ny * g.nseg, (float)h->cfg.omega);
  std::vector<uint8_t> set((size_t)ny * g.nseg, 0);
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      if (h->h_cls[(long long)(y + 1) * g.pitch + x] >= 2) continue;   // solid
      const double w = omega[(long long)x * ny + y];
      if (!(w > 0.0 && w < 2.0)) return fail(LBM_ERR_ARG, "lbm_set_omega_map: omega must lie in (0, 2)");
      const size_t i = (size_t)y * g.nseg + x / 32;
      if (set[i] && seg[i] != (float)w)
        return fail(LBM_ERR_ARG, "lbm_set_omega_map: omega differs inside the 32-node segment of node (" +
                                     std::to_string(x) + "," + std::to_string(y) + ")");
      seg[i] = (float)w;
      set[i] = 1;
    }
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  if (!h->omega_seg) {
    int rc = h->alloc(reinterpret_cast<void**>(&h->omega_seg), seg.size() * sizeof(float));
    if (rc) return rc;
  }
  LBM_CUDA(cudaMemcpyAsync(h->omega_seg, seg.data(), seg.size() * sizeof(float), cudaMemcpyHostToDevice,
                           h->stream));
  h->omega_hash = fnv1a(kFnvSeed, seg.data(), seg.size() * sizeof(float));
  h->drop_graphs();   // graphs captured earlier hold the old argument
  return h->wait();
}

int lbm_step_ex(LbmHandle* h, int64_t nsteps, int flags) {
  if (!h) return fail(LBM_ERR_ARG, "lbm_step: null handle");
  if (nsteps < 0) return fail(LBM_ERR_ARG, "lbm_step: nsteps < 0");
  if (flags & ~(LBM_STEP_MOMENTS | LBM_STEP_RESIDUAL)) return fail(LBM_ERR_ARG, "lbm_step: unknown flags");
  if (!h->initialized) return fail(LBM_ERR_STATE, "lbm_step: call lbm_init_fields or lbm_set_populations first");
  if (nsteps == 0) return LBM_OK;
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int kflags = (flags & LBM_STEP_MOMENTS ? lbm::F_MOMENTS : 0) |
               (flags & LBM_STEP_RESIDUAL ? lbm::F_RESIDUAL : 0);
  int64_t s = 0;
  int rc;
  if ((flags & LBM_STEP_RESIDUAL) && (rc = h->ensure_old())) return rc;
  auto one = [&](int fl) {
    int r = h->step_full(fl);
    if (r) return r;
    if (fl & lbm::F_RESIDUAL) h->old_cur ^= 1;
    h->nopull = false;
    h->t += 1;
    h->launches += 1;
    return LBM_OK;
  };
  if (h->nopull) {
    if ((rc = one(lbm::F_NOPULL | (nsteps == 1 ? kflags : 0)))) return rc;
    s = 1;
  }
  // tune on the steady (pulling) step, which all later steps use
  if (!h->tuned && !h->nopull && s < nsteps && (rc = h->autotune())) return rc;
  int64_t plain = nsteps - s - (s < nsteps ? 1 : 0);
  const bool graphs = !std::getenv("LBM_NO_GRAPH");
  while (plain > 0) {
    if (plain >= kGraphChunk && graphs) {
      if (!h->gexec && (rc = h->capture_graph(h->cur))) return rc;
      if (h->cur == h->gparity) {
        LBM_CUDA(cudaGraphLaunch(h->gexec, h->stream));
        h->t += kGraphChunk;
        h->launches += kGraphChunk;
        plain -= kGraphChunk;
        continue;
      }
    } else if (plain >= 2 && graphs) {   // the remainder, as one graph of its own
      cudaGraphExec_t ex = nullptr;
      if ((rc = h->tail_graph((int)plain, h->cur, &ex))) return rc;
      LBM_CUDA(cudaGraphLaunch(ex, h->stream));
      h->cur ^= (int)(plain & 1);
      h->t += plain;
      h->launches += plain;
      plain = 0;
      continue;
    }
    if ((rc = one(0))) return rc;
    --plain;
  }
  if (s < nsteps) {
    if ((kflags & lbm::F_RESIDUAL) && !h->res_tuned && h->tuned && (rc = h->tune_residual())) return rc;
    if ((rc = one(kflags))) return rc;
  }
  if (flags & LBM_STEP_MOMENTS) h->has_moments = true;
  if (flags & LBM_STEP_RESIDUAL) {
    const lbm::Variant rv = h->res_tuned ? h->res_variant : h->variant;
    const int slot = (int)(h->res_seq % kResRing);
    LBM_CUDA(lbm::finish_reduce(h->partials, h->nparts_of(rv), h->scratch, h->host_red_dev + 16 + 8 * slot,
                                h->stream));
    LBM_CUDA(cudaEventRecord(h->res_ev[slot], h->stream));
    h->res_t[slot] = h->t;
    h->res_seq += 1;
    h->has_residual = true;
  }
  return LBM_OK;
}

int lbm_step(LbmHandle* h, int64_t nsteps) { return lbm_step_ex(h, nsteps, 0); }

int lbm_adjoint_forward(LbmHandle* h, int64_t nsteps, int interval) {
  if (!h) return fail(LBM_ERR_ARG, "lbm_adjoint_forward: null handle");
  if (nsteps < 1 || interval < 1) return fail(LBM_ERR_ARG, "lbm_adjoint_forward: need nsteps >= 1, interval >= 1");
  if (!h->initialized || !h->nopull || h->t != 0)
    return fail(LBM_ERR_STATE, "lbm_adjoint_forward: call lbm_init_fields first (the pass starts at t = 0)");
  if (h->aa) return fail(LBM_ERR_ARG, "lbm_adjoint_forward: not available with the AA population layout");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int rc = h->build_adjoint_tables();
  if (rc) return rc;
  auto& A = h->adj;
  const int64_t nck = (nsteps + interval - 1) / interval;   // states at t = 0, I, 2I, ...
  // (re)allocate the workspace when the plan changes
  if (!A.ready || A.interval != interval || (int64_t)A.ckpt.size() < nck) {
    for (auto* v : {&A.ckpt, &A.ckpt_side, &A.seg, &A.seg_side})
      for (void* q : *v) h->release(q);
    A.ckpt.assign(nck, nullptr);
    A.ckpt_side.assign(nck, nullptr);
    A.seg.assign(interval > 1 ? 2 * (interval - 1) : 0, nullptr);
    A.seg_side.assign(A.seg.size(), nullptr);
    for (size_t i = 0; i < A.ckpt.size(); ++i)
      if ((rc = h->alloc(&A.ckpt[i], h->state_bytes())) || (rc = h->alloc(&A.ckpt_side[i], h->side_bytes())))
        return rc;
    for (size_t i = 0; i < A.seg.size(); ++i)
      if ((rc = h->alloc(&A.seg[i], h->state_bytes())) || (rc = h->alloc(&A.seg_side[i], h->side_bytes())))
        return rc;
    if (!A.a[0]) {
      const size_t ab = 9 * h->g.plane * (size_t)h->ks->compute_bytes;
      A.nparts = h->nparts_of(lbm::Variant{0, 1, 256, 0}) * 8;   // one row per warp
      if ((rc = h->alloc(&A.a[0], ab)) || (rc = h->alloc(&A.a[1], ab)) ||
          (rc = h->alloc(&A.gF, 2 * h->g.plane * (size_t)h->ks->compute_bytes)) ||
          (rc = h->alloc(reinterpret_cast<void**>(&A.gpart), A.nparts * 4 * sizeof(double))) ||
          (rc = h->alloc(reinterpret_cast<void**>(&A.grad_u), 2 * h->g.plane * sizeof(double))))
        return rc;
      LBM_CUDA(cudaMemsetAsync(A.a[0], 0, ab, h->stream));
      LBM_CUDA(cudaMemsetAsync(A.a[1], 0, ab, h->stream));
      LBM_CUDA(cudaMemsetAsync(A.grad_u, 0, 2 * h->g.plane * sizeof(double), h->stream));
    }
    if (!A.aux) {
      // the recompute stream runs at the lowest priority: the reverse steps on
      // the handle's stream are the critical path
      int lo = 0, hi = 0;
      LBM_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      LBM_CUDA(cudaStreamCreateWithPriority(&A.aux, cudaStreamNonBlocking, lo));
      for (cudaEvent_t& e : A.ev) LBM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    A.interval = interval;
    A.ready = true;
  }
  if (!h->tuned && (rc = h->autotune())) return rc;
  const bool use_graph = !std::getenv("LBM_NO_GRAPH");
  if (use_graph && (A.graph_T != nsteps || A.graph_interval != interval)) {
    if (A.fwd_graph) cudaGraphExecDestroy(A.fwd_graph);
    if (A.bwd_graph) cudaGraphExecDestroy(A.bwd_graph);
    A.fwd_graph = A.bwd_graph = nullptr;
    A.graph_T = nsteps;
    A.graph_interval = interval;
  }
  // the pass starts from buffer 0 so that one captured graph fits every call
  if (h->cur != 0) {
    LBM_CUDA(cudaMemcpyAsync(h->pop[0], h->pop[1], 9 * h->g.plane * h->ks->elem_bytes,
                             cudaMemcpyDeviceToDevice, h->stream));
    h->cur = 0;
  }
  auto enqueue = [&]() -> int {
    // t = 0: the initial populations (read without pulling)
    LBM_CUDA(cudaMemcpyAsync(h->state_base(A.ckpt[0]), h->pop[h->cur], 9 * h->g.plane * h->ks->elem_bytes,
                             cudaMemcpyDeviceToDevice, h->stream));
    for (int64_t t = 1; t <= nsteps; ++t) {
      const int fl = (t == 1 ? lbm::F_NOPULL : 0) | (t == nsteps ? lbm::F_MOMENTS : 0);
      int r = h->launch(fl);
      if (r) return r;
      if (t % interval == 0 && t < nsteps) {
        const int64_t c = t / interval;
        LBM_CUDA(cudaMemcpyAsync(h->state_base(A.ckpt[c]), h->pop[h->cur], 9 * h->g.plane * h->ks->elem_bytes,
                                 cudaMemcpyDeviceToDevice, h->stream));
        LBM_CUDA(cudaMemcpyAsync(A.ckpt_side[c], h->side[h->cur], h->side_bytes(), cudaMemcpyDeviceToDevice,
                                 h->stream));
      }
    }
    return LBM_OK;
  };
  if (use_graph) {
    if (!A.fwd_graph) {
      rc = h->capture(&A.fwd_graph, enqueue);
      h->cur = 0;   // capture only recorded the launches
      if (rc) return rc;
    }
    LBM_CUDA(cudaGraphLaunch(A.fwd_graph, h->stream));
    h->cur = (int)(nsteps & 1);
  } else if ((rc = enqueue())) {
    return rc;
  }
  h->nopull = false;
  h->t = nsteps;
  h->clear_residuals();
  h->launches += nsteps;
  h->has_moments = true;
  A.T = nsteps;
  return h->wait();
}

int lbm_adjoint_backward(LbmHandle* h, const double* grad_u, double* grad_force,
                         double* grad_tau, double* grad_uwall) {
  if (!h || !grad_u) return fail(LBM_ERR_ARG, "lbm_adjoint_backward: null argument");
  auto& A = h->adj;
  if (!A.ready || A.T < 1) return fail(LBM_ERR_STATE, "lbm_adjoint_backward: run lbm_adjoint_forward first");
  if (grad_force && !h->body) return fail(LBM_ERR_STATE, "lbm_adjoint_backward: no body-force field to differentiate");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const lbm::Geom& g = h->g;
  const long long nh = (long long)g.nx * g.ny;
  int rc = h->ensure_stage(2 * nh);
  if (rc) return rc;
  LBM_CUDA(cudaMemcpyAsync(h->stage, grad_u, 2 * nh * sizeof(double), cudaMemcpyDefault, h->stream));
  LBM_CUDA(lbm::reorder(g, h->stage, A.grad_u, 2, LBM_LAYOUT_INNER, 1, h->stream));
  const int I = A.interval;
  const int64_t T = A.T;
  const lbm::Variant plain = h->variant;
  auto enqueue = [&]() -> int {
    LBM_CUDA(cudaMemsetAsync(A.gF, 0, 2 * g.plane * (size_t)h->ks->compute_bytes, h->stream));
    LBM_CUDA(cudaMemsetAsync(A.gpart, 0, A.nparts * 4 * sizeof(double), h->stream));
    int cur_a = 0;
    bool have_next = false;
    const int64_t C = (T - 1) / I;
    cudaEvent_t* const evR = A.ev + 2;
    cudaEvent_t* const evA = A.ev + 4;
    LBM_CUDA(cudaEventRecord(A.ev[0], h->stream));   // fork
    LBM_CUDA(cudaStreamWaitEvent(A.aux, A.ev[0], 0));
    for (int64_t c = C; c >= 0; --c) {
      const int64_t t0 = c * I, t1 = std::min<int64_t>(t0 + I, T);
      const int set = (int)(c & 1);
      void* const* seg = A.seg.data() + set * (I - 1);
      void* const* seg_side = A.seg_side.data() + set * (I - 1);
      // aux: recompute p_{t0+1} .. p_{t1-1} into this segment's set, once the
      // reverse steps of segment c+2 (same set) have read it
      if (c + 2 <= C) LBM_CUDA(cudaStreamWaitEvent(A.aux, evA[set], 0));
      for (int64_t t = t0 + 1; t < t1; ++t) {
        const void* fin = t == t0 + 1 ? h->state_base(A.ckpt[c]) : h->state_base(seg[t - t0 - 2]);
        const void* sin = t == t0 + 1 ? A.ckpt_side[c] : seg_side[t - t0 - 2];
        int r = h->launch_bufs(t == 1 ? lbm::F_NOPULL : 0, plain, fin, h->state_base(seg[t - t0 - 1]), sin,
                               seg_side[t - t0 - 1], A.aux);
        if (r) return r;
      }
      LBM_CUDA(cudaEventRecord(evR[set], A.aux));
      // main: reverse steps t1 .. t0+1 (overlap the recompute of segment c-1)
      LBM_CUDA(cudaStreamWaitEvent(h->stream, evR[set], 0));
      for (int64_t t = t1; t > t0; --t) {
        lbm::AdjArgs a;
        a.g = g;
        a.p = h->p;
        a.fprev = t - 1 == t0 ? h->state_base(A.ckpt[c]) : h->state_base(seg[t - t0 - 2]);
        a.side_prev = t - 1 == t0 ? A.ckpt_side[c] : seg_side[t - t0 - 2];
        a.a_next = have_next ? A.a[cur_a] : nullptr;
        a.a_cur = A.a[cur_a ^ 1];
        a.grad_u = t == T ? A.grad_u : nullptr;
        a.gF = h->body ? A.gF : nullptr;
        a.gpart = A.gpart;
        a.tr_reader = A.tr_reader;
        a.tr_self = A.tr_self;
        a.wall_rec = A.wall_rec;
        a.body = h->body;
        a.nopull = t == 1;
        LBM_CUDA(h->ks->adjoint(h->cfg.forcing, a, h->stream));
        cur_a ^= 1;
        have_next = true;
      }
      LBM_CUDA(cudaEventRecord(evA[set], h->stream));
    }
    LBM_CUDA(cudaEventRecord(A.ev[1], A.aux));   // join
    LBM_CUDA(cudaStreamWaitEvent(h->stream, A.ev[1], 0));
    return LBM_OK;
  };
  if (!std::getenv("LBM_NO_GRAPH")) {
    if (!A.bwd_graph && (rc = h->capture(&A.bwd_graph, enqueue))) return rc;
    LBM_CUDA(cudaGraphLaunch(A.bwd_graph, h->stream));
  } else if ((rc = enqueue())) {
    return rc;
  }
  // parameter gradients: fixed-order sum of the per-block rows on the host
  std::vector<double> part(A.nparts * 4);
  LBM_CUDA(cudaMemcpyAsync(part.data(), A.gpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((rc = h->wait())) return rc;
  if (grad_force) {
    if ((rc = h->ensure_stage(2 * nh + 3 * g.plane))) return rc;
    LBM_CUDA(h->ks->moments_to_f64(g, A.gF, static_cast<char*>(A.gF) + g.plane * h->ks->compute_bytes,
                                   A.gF, h->stage + 2 * nh, h->stream));
    LBM_CUDA(lbm::reorder(g, h->stage + 2 * nh, h->stage, 2, LBM_LAYOUT_INNER, 0, h->stream));
    LBM_CUDA(cudaMemcpyAsync(grad_force, h->stage, 2 * nh * sizeof(double), cudaMemcpyDefault, h->stream));
    if ((rc = h->wait())) return rc;
  }
  double s[3] = {0, 0, 0};
  for (long long b = 0; b < A.nparts; ++b)
    for (int i = 0; i < 3; ++i) s[i] += part[b * 4 + i];
  if (grad_tau) *grad_tau = -s[0] * h->cfg.omega * h->cfg.omega;   // d omega / d tau = -omega^2
  if (grad_uwall) {
    grad_uwall[0] = s[1];
    grad_uwall[1] = s[2];
  }
  return LBM_OK;
}

extern "C++" {
// Moments of the last recorded step into caller fields in host order
// (HT = double, or float for single-precision cases, rounded to nearest).
// The device keeps them as three consecutive planes in the compute type
// (FP64, or FP32 for shifted storage); they are transposed straight from
// there, widened or rounded on the way.
template <class HT, class CT>
static cudaError_t moments_cols(const LbmHandle* h, const CT* mom, HT* rho, HT* u, int layout,
                                int x0, int x1) {
  const long long plane = h->g.plane;
  cudaError_t e = lbm::reorder_cols(h->g, mom, rho, 1, layout, 0, x0, x1, h->stream);
  if (e != cudaSuccess) return e;
  return lbm::reorder_cols(h->g, mom + plane, u, 2, layout, 0, x0, x1, h->stream);
}

template <class HT>
static cudaError_t moments_cols(const LbmHandle* h, HT* rho, HT* u, int layout, int x0, int x1) {
  if (h->ks->compute_bytes == sizeof(float))
    return moments_cols(h, static_cast<const float*>(h->mom[0]), rho, u, layout, x0, x1);
  return moments_cols(h, static_cast<const double*>(h->mom[0]), rho, u, layout, x0, x1);
}

template <class HT>
static int get_moments(LbmHandle* h, HT* rho, HT* u, int layout, const char* name) {
  if (!h || !rho || !u) return fail(LBM_ERR_ARG, std::string(name) + ": null argument");
  if (layout != LBM_LAYOUT_INNER && layout != LBM_LAYOUT_PADDED)
    return fail(LBM_ERR_ARG, std::string(name) + ": unknown layout");
  if (!h->has_moments)
    return fail(LBM_ERR_STATE, std::string(name) + ": no moments recorded (use LBM_STEP_MOMENTS)");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const long long nh = h->host_nodes(layout);
  const int nx = h->cfg.nx;
  HT* rd = layout == LBM_LAYOUT_INNER ? h->host_direct(rho) : nullptr;
  HT* ud = layout == LBM_LAYOUT_INNER ? h->host_direct(u) : nullptr;
  if (rd && ud) {   // transposed straight into the caller's pinned buffers
    LBM_CUDA(moments_cols(h, rd, ud, layout, 0, nx));
    return h->wait();
  }
  const long long hn = (3 * nh * (long long)sizeof(HT) + 7) / 8;   // host-order stage, in doubles
  int rc = h->ensure_stage(hn);
  if (rc) return rc;
  HT* hs = reinterpret_cast<HT*>(h->stage);
  if (layout == LBM_LAYOUT_INNER) {
    // column chunks: chunk c goes to the host on the transfer stream while
    // the handle's stream transposes chunk c + 1
    if ((rc = h->ensure_xfer())) return rc;
    const long long ny = h->cfg.ny;
    constexpr int NC = LbmHandle::kXferChunks;
    for (int c = 0; c < NC; ++c) {
      const int x0 = h->xfer_col(c), x1 = h->xfer_col(c + 1);
      if (x0 >= x1) continue;
      LBM_CUDA(moments_cols(h, hs, hs + nh, layout, x0, x1));
      LBM_CUDA(cudaEventRecord(h->xev[c], h->stream));
      LBM_CUDA(cudaStreamWaitEvent(h->xfer, h->xev[c], 0));
      LBM_CUDA(cudaMemcpyAsync(rho + x0 * ny, hs + x0 * ny, (x1 - x0) * ny * sizeof(HT),
                               cudaMemcpyDefault, h->xfer));
      LBM_CUDA(cudaMemcpyAsync(u + 2 * x0 * ny, hs + nh + 2 * x0 * ny, 2 * (x1 - x0) * ny * sizeof(HT),
                               cudaMemcpyDefault, h->xfer));
    }
    LBM_CUDA(cudaEventRecord(h->xev[NC], h->xfer));
    LBM_CUDA(cudaStreamWaitEvent(h->stream, h->xev[NC], 0));
    return h->wait();
  }
  LBM_CUDA(cudaMemsetAsync(hs, 0, 3 * nh * sizeof(HT), h->stream));   // ghosts of the padded layout
  LBM_CUDA(moments_cols(h, hs, hs + nh, layout, 0, nx));
  LBM_CUDA(cudaMemcpyAsync(rho, hs, nh * sizeof(HT), cudaMemcpyDefault, h->stream));
  LBM_CUDA(cudaMemcpyAsync(u, hs + nh, 2 * nh * sizeof(HT), cudaMemcpyDefault, h->stream));
  return h->wait();
}

}  // extern "C++"

int lbm_get_moments(LbmHandle* h, double* rho, double* u, int layout) {
  return get_moments(h, rho, u, layout, "lbm_get_moments");
}

int lbm_get_moments_f32(LbmHandle* h, float* rho, float* u, int layout) {
  return get_moments(h, rho, u, layout, "lbm_get_moments_f32");
}

namespace {
// {res_rho, res_ux, res_uy} from one residual step's sums (residues.py:204-222)
int residual_of(const LbmHandle* h, const double* s, double out[3], const char* who) {
  for (int c = 0; c < 3; ++c) out[c] = std::sqrt(s[2 * c] / (s[2 * c + 1] + h->cfg.eps));
  if (s[6] > 0)
    return fail(LBM_ERR_NONFINITE, std::string(who) + ": " + std::to_string((long long)s[6]) +
                                       " fluid nodes have non-finite density or velocity");
  return LBM_OK;
}
}  // namespace

int lbm_residual(LbmHandle* h, double out[3]) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_residual: null argument");
  if (!h->has_residual) return fail(LBM_ERR_STATE, "lbm_residual: no residual step recorded (use LBM_STEP_RESIDUAL)");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int rc = h->wait();
  if (rc) return rc;
  return residual_of(h, h->res_slot((int)((h->res_seq - 1) % kResRing)), out, "lbm_residual");
}

int lbm_residual_at(LbmHandle* h, int64_t t, double out[3]) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_residual_at: null argument");
  int slot = -1;
  for (int i = 0; i < kResRing; ++i)
    if (h->res_t[i] == t && t >= 0) slot = i;
  if (slot < 0)
    return fail(LBM_ERR_STATE, "lbm_residual_at: time step " + std::to_string((long long)t) +
                                   " is not one of the last " + std::to_string(kResRing) +
                                   " residual steps since initialisation");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int rc = h->wait(h->res_ev[slot]);   // that step only, not the steps queued after it
  if (rc) return rc;
  return residual_of(h, h->res_slot(slot), out, "lbm_residual_at");
}

int lbm_conservation(LbmHandle* h, double out[3]) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_conservation: null argument");
  if (!h->initialized) return fail(LBM_ERR_STATE, "lbm_conservation: not initialised");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  LBM_CUDA(h->ks->conservation(h->g, h->p, h->pop[h->cur], h->partials, h->aa_state(), h->stream));
  LBM_CUDA(lbm::finish_reduce(h->partials, h->g.ny, h->scratch, h->host_red_dev + 8, h->stream));
  int rc = h->wait();
  if (rc) return rc;
  for (int c = 0; c < 3; ++c) out[c] = h->host_red[8 + c];
  // the residual partial sums were overwritten; the host copy stays valid
  return LBM_OK;
}

int lbm_get_populations(LbmHandle* h, double* pop) {
  if (!h || !pop) return fail(LBM_ERR_ARG, "lbm_get_populations: null argument");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const long long nh = h->host_nodes(LBM_LAYOUT_PADDED), plane = h->g.plane;
  int rc = h->ensure_stage(9 * nh + 9 * plane);
  if (rc) return rc;
  double* hs = h->stage;
  double* ds = h->stage + 9 * nh;
  LBM_CUDA(h->ks->convert(h->g, h->p, h->pop[h->cur], ds, 0, h->aa_state(), h->stream));
  LBM_CUDA(cudaMemsetAsync(hs, 0, 9 * nh * sizeof(double), h->stream));
  LBM_CUDA(lbm::reorder(h->g, ds, hs, 9, LBM_LAYOUT_PADDED, 0, h->stream));
  LBM_CUDA(cudaMemcpyAsync(pop, hs, 9 * nh * sizeof(double), cudaMemcpyDefault, h->stream));
  return h->wait();
}

int lbm_set_populations(LbmHandle* h, const double* pop_new) {
  if (!h || !pop_new) return fail(LBM_ERR_ARG, "lbm_set_populations: null argument");
  if (h->mov.n) return fail(LBM_ERR_STATE, "lbm_set_populations: not supported with moving obstacles");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const long long nh = h->host_nodes(LBM_LAYOUT_PADDED), plane = h->g.plane;
  int rc = h->ensure_stage(9 * nh + 9 * plane);
  if (rc) return rc;
  h->initialized = false;   // until the new state is complete
  double* hs = h->stage;
  double* ds = h->stage + 9 * nh;
  LBM_CUDA(cudaMemcpyAsync(hs, pop_new, 9 * nh * sizeof(double), cudaMemcpyDefault, h->stream));
  LBM_CUDA(cudaMemsetAsync(ds, 0, 9 * plane * sizeof(double), h->stream));
  LBM_CUDA(lbm::reorder(h->g, hs, ds, 9, LBM_LAYOUT_PADDED, 1, h->stream));
  if (h->aa) h->cur = 0;   // AA: the next step is an even phase that reads the set values
  LBM_CUDA(h->ks->convert(h->g, h->p, h->pop[h->cur], ds, 1, 0, h->stream));
  if ((rc = h->wait())) return rc;
  h->initialized = true;
  h->nopull = true;
  return LBM_OK;
}

int lbm_set_force_links(LbmHandle* h, const LbmForceLink* links, int64_t nlinks, int ngroups) {
  if (!h || (nlinks > 0 && !links)) return fail(LBM_ERR_ARG, "lbm_set_force_links: null argument");
  if (nlinks < 0 || ngroups < 0 || (nlinks > 0 && ngroups == 0) || nlinks > (int64_t)INT32_MAX)
    return fail(LBM_ERR_ARG, "lbm_set_force_links: bad link or group count");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const lbm::Geom& g = h->g;
  const int64_t nx = g.nx, ny = g.ny;
  std::unordered_map<int64_t, int> rec_of;   // inner node -> record
  for (size_t r = 0; r < h->h_links.size(); ++r) rec_of[h->h_links[r].node] = (int)r;
  std::vector<int64_t> order(nlinks);
  for (int64_t i = 0; i < nlinks; ++i) {
    const LbmForceLink& L = links[i];
    if (L.group < 0 || L.group >= ngroups)
      return fail(LBM_ERR_ARG, "lbm_set_force_links: link " + std::to_string(i) + " has group out of range");
    if (L.k_out < 0 || L.k_out > 8 || L.k_in < 0 || L.k_in > 8)
      return fail(LBM_ERR_ARG, "lbm_set_force_links: link " + std::to_string(i) + " has a direction out of range");
    if (L.node < 0 || L.node >= nx * ny || !rec_of.count(L.node))
      return fail(LBM_ERR_ARG, "lbm_set_force_links: link " + std::to_string(i) +
                                   " is not on a boundary node of the link table");
    order[i] = i;
  }
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return links[a].group < links[b].group; });
  std::vector<long long> node(nlinks);
  std::vector<int> rec(nlinks), gstart(ngroups + 1, 0);
  std::vector<int8_t> kk(2 * nlinks);
  std::vector<double> arm(2 * nlinks);
  for (int64_t j = 0; j < nlinks; ++j) {
    const LbmForceLink& L = links[order[j]];
    node[j] = (long long)(L.node % ny + 1) * g.pitch + L.node / ny;
    rec[j] = rec_of[L.node];
    kk[2 * j] = L.k_out;
    kk[2 * j + 1] = L.k_in;
    arm[2 * j] = L.rx;
    arm[2 * j + 1] = L.ry;
    ++gstart[L.group + 1];
  }
  for (int q = 0; q < ngroups; ++q) gstart[q + 1] += gstart[q];
  auto& F = h->force;
  for (void* q : {(void*)F.node, (void*)F.rec, (void*)F.kk, (void*)F.arm, (void*)F.gstart, (void*)F.out})
    h->release(q);
  F = LbmHandle::Force{};
  if (ngroups == 0) return LBM_OK;
  const size_t n1 = std::max<int64_t>(nlinks, 1);
  int rc;
  if ((rc = h->alloc(reinterpret_cast<void**>(&F.node), n1 * sizeof(long long))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&F.rec), n1 * sizeof(int))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&F.kk), 2 * n1)) ||
      (rc = h->alloc(reinterpret_cast<void**>(&F.arm), 2 * n1 * sizeof(double))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&F.gstart), (ngroups + 1) * sizeof(int))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&F.out), 3 * (size_t)ngroups * sizeof(double))))
    return rc;
  if (nlinks > 0) {
    LBM_CUDA(cudaMemcpyAsync(F.node, node.data(), nlinks * sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    LBM_CUDA(cudaMemcpyAsync(F.rec, rec.data(), nlinks * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    LBM_CUDA(cudaMemcpyAsync(F.kk, kk.data(), 2 * nlinks, cudaMemcpyHostToDevice, h->stream));
    LBM_CUDA(cudaMemcpyAsync(F.arm, arm.data(), 2 * nlinks * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  }
  LBM_CUDA(cudaMemcpyAsync(F.gstart, gstart.data(), (ngroups + 1) * sizeof(int), cudaMemcpyHostToDevice,
                           h->stream));
  F.ngroups = ngroups;
  F.n = nlinks;
  return h->wait();   // the host vectors go out of scope
}

int lbm_forces(LbmHandle* h, double* out) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_forces: null argument");
  if (!h->initialized) return fail(LBM_ERR_STATE, "lbm_forces: not initialised");
  const auto& F = h->force;
  if (F.ngroups == 0) return LBM_OK;
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  lbm::ForceArgs a;
  a.g = h->g;
  a.p = h->p;
  a.pop = h->pop[h->cur];
  a.side = h->side[h->cur];
  a.node = F.node;
  a.rec = F.rec;
  a.kk = F.kk;
  a.arm = F.arm;
  a.gstart = F.gstart;
  a.nopull = h->nopull ? 1 : 0;
  a.aa_state = h->aa_state();
  a.out = F.out;
  LBM_CUDA(h->ks->forces(a, F.ngroups, h->stream));
  LBM_CUDA(cudaMemcpyAsync(out, F.out, 3 * (size_t)F.ngroups * sizeof(double), cudaMemcpyDefault, h->stream));
  return h->wait();
}

int lbm_set_moving_obstacles(LbmHandle* h, const LbmMovingObstacle* obs, int n,
                             const double gravity[2]) {
  if (!h || (n > 0 && !obs)) return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: null argument");
  if (n < 0 || n > lbm::kMovMaxObstacles)
    return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: 0 to " + std::to_string(lbm::kMovMaxObstacles) +
                                 " obstacles");
  if (h->mov.n) return fail(LBM_ERR_STATE, "lbm_set_moving_obstacles: already set");
  if (h->aa && n > 0)
    return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: not available with the AA population layout");
  if (n == 0) return LBM_OK;
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const lbm::Geom& g = h->g;
  auto& M = h->mov;
  M.init.assign(n, lbm::MovObs{});
  double rmax = 0.0;
  for (int j = 0; j < n; ++j) {
    const LbmMovingObstacle& o = obs[j];
    lbm::MovObs& m = M.init[j];
    if (!(o.radius > 0.0) || !std::isfinite(o.center[0]) || !std::isfinite(o.center[1]))
      return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) + ": bad radius or centre");
    if (o.shape != 0 && o.shape != 1)
      return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) +
                                   ": shape must be 0 (circle) or 1 (ellipse)");
    if (o.shape == 1 && !(o.semi_axes[0] > 0.0 && o.semi_axes[1] > 0.0 &&
                          o.radius >= o.semi_axes[0] && o.radius >= o.semi_axes[1] &&
                          std::isfinite(o.angle)))
      return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) +
                                   ": an ellipse needs semi-axes > 0, radius >= both and a finite angle");
    if (o.calculated && ((o.translation && !(o.mass > 0.0)) || (o.rotation && !(o.inertia > 0.0))))
      return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) + ": mass and inertia must be > 0");
    m.cx = o.center[0];
    m.cy = o.center[1];
    m.r = o.radius;
    m.vx = o.velocity[0];
    m.vy = o.velocity[1];
    m.om = o.omega;
    m.angle = o.angle;
    m.mass = o.mass;
    m.inertia = o.inertia;
    m.density = o.density;
    m.fx = m.fy = m.tq = 0.0;
    m.id = o.id;
    m.calculated = o.calculated;
    m.rotation = o.rotation;
    m.translation = o.translation;
    m.shape = o.shape;
    m.sa = o.shape == 1 ? o.semi_axes[0] : 0.0;
    m.sb = o.shape == 1 ? o.semi_axes[1] : 0.0;
    // the initial box with its border must lie in [1, nx-2] x [1, ny-2] and
    // in static bulk fluid
    const int bx0 = (int)std::floor(m.cx - m.r) - 1, bx1 = (int)std::ceil(m.cx + m.r) + 1;
    const int by0 = (int)std::floor(m.cy - m.r) - 1, by1 = (int)std::ceil(m.cy + m.r) + 1;
    if (bx0 < 2 || by0 < 2 || bx1 > g.nx - 3 || by1 > g.ny - 3)
      return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) +
                                   " must stay two nodes away from the domain edges");
    for (int y = by0 - 1; y <= by1 + 1; ++y)
      for (int x = bx0 - 1; x <= bx1 + 1; ++x)
        if (h->h_cls[g.node(x, y)] != 0)
          return fail(LBM_ERR_ARG, "lbm_set_moving_obstacles: obstacle " + std::to_string(j) +
                                       " starts next to a boundary node or a static solid");
    rmax = std::max(rmax, m.r);
  }
  M.side = 2 * (int)std::ceil(rmax) + 8;
  M.gx = gravity ? gravity[0] : 0.0;
  M.gy = gravity ? gravity[1] : 0.0;
  const size_t plane = g.plane, cb = h->ks->compute_bytes;
  const size_t nseg = (size_t)g.ny * g.nseg;
  int rc;
  if ((rc = h->alloc(reinterpret_cast<void**>(&M.obs), n * sizeof(lbm::MovObs))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&M.dsolid), plane)) ||
      (rc = h->alloc(reinterpret_cast<void**>(&M.fresh), plane)) ||
      (rc = h->alloc(&M.us, 2 * plane * cb)) || (rc = h->alloc(&M.rho_dyn[0], plane * cb)) ||
      (rc = h->alloc(&M.rho_dyn[1], plane * cb)) ||
      (rc = h->alloc(reinterpret_cast<void**>(&M.part), (size_t)n * lbm::kMovForceBlocks * 3 * sizeof(double))) ||
      (rc = h->alloc(reinterpret_cast<void**>(&M.cls_static), plane)) ||
      (rc = h->alloc(reinterpret_cast<void**>(&M.seg_static), nseg)))
    return rc;
  LBM_CUDA(cudaMemsetAsync(M.us, 0, 2 * plane * cb, h->stream));
  LBM_CUDA(cudaMemsetAsync(M.dsolid, 0, plane, h->stream));
  LBM_CUDA(cudaMemsetAsync(M.fresh, 0, plane, h->stream));
  LBM_CUDA(cudaMemcpyAsync(M.cls_static, h->g.cls, plane, cudaMemcpyDeviceToDevice, h->stream));
  LBM_CUDA(cudaMemcpyAsync(M.seg_static, h->g.segflag, nseg, cudaMemcpyDeviceToDevice, h->stream));
  M.n = n;
  // only the scalar kernel serves class-4 nodes: every launch from now on,
  // the no-pull first step included, uses a scalar shape (re-picked among
  // the scalar candidates by the autotuner)
  for (int i = 0; i < h->ks->nvariants; ++i)
    if (h->ks->variants[i].kind == 0 && h->ks->variants[i].stages == 0) {
      h->variant = h->ks->variants[i];
      break;
    }
  h->tuned = false;
  h->res_tuned = false;
  h->drop_graphs();
  // the obstacles are placed by lbm_init_fields, which must come next
  h->initialized = false;
  return h->wait();
}

int lbm_get_moving_obstacles(LbmHandle* h, LbmMovingObstacle* out) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_get_moving_obstacles: null argument");
  auto& M = h->mov;
  if (!M.n) return LBM_OK;
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  std::vector<lbm::MovObs> st(M.n);
  LBM_CUDA(cudaMemcpyAsync(st.data(), M.obs, M.n * sizeof(lbm::MovObs), cudaMemcpyDeviceToHost, h->stream));
  int rc = h->wait();
  if (rc) return rc;
  for (int j = 0; j < M.n; ++j) {
    const lbm::MovObs& m = st[j];
    LbmMovingObstacle& o = out[j];
    o.center[0] = m.cx;
    o.center[1] = m.cy;
    o.radius = m.r;
    o.velocity[0] = m.vx;
    o.velocity[1] = m.vy;
    o.omega = m.om;
    o.angle = m.angle;
    o.mass = m.mass;
    o.inertia = m.inertia;
    o.density = m.density;
    o.force[0] = m.fx;
    o.force[1] = m.fy;
    o.torque = m.tq;
    o.id = m.id;
    o.calculated = m.calculated;
    o.rotation = m.rotation;
    o.translation = m.translation;
    o.shape = m.shape;
    o.semi_axes[0] = m.sa;
    o.semi_axes[1] = m.sb;
    o.reserved = 0;
  }
  return LBM_OK;
}

int lbm_get_node_flags(LbmHandle* h, uint8_t* flags) {
  if (!h || !flags) return fail(LBM_ERR_ARG, "lbm_get_node_flags: null argument");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const lbm::Geom& g = h->g;
  std::vector<uint8_t> ds;
  if (h->mov.n) {
    ds.resize(g.plane);
    LBM_CUDA(cudaMemcpyAsync(ds.data(), h->mov.dsolid, g.plane, cudaMemcpyDeviceToHost, h->stream));
    int rc = h->wait();
    if (rc) return rc;
  }
  for (long long x = 0; x < g.nx; ++x)
    for (long long y = 0; y < g.ny; ++y) {
      const long long n = g.node((int)x, (int)y);
      uint8_t v = h->h_cls[n] == 2 ? 1 : 0;
      if (!ds.empty() && ds[n]) v = (uint8_t)(1 + ds[n]);
      flags[x * g.ny + y] = v;
    }
  return LBM_OK;
}

int lbm_time(LbmHandle* h, int64_t* t) {
  if (!h || !t) return fail(LBM_ERR_ARG, "lbm_time: null argument");
  *t = h->t;
  return LBM_OK;
}

int lbm_kernel_launches(LbmHandle* h, int64_t* n) {
  if (!h || !n) return fail(LBM_ERR_ARG, "lbm_kernel_launches: null argument");
  *n = h->launches;
  return LBM_OK;
}

int lbm_kernel_variant(LbmHandle* h, int out[4]) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_kernel_variant: null argument");
  out[0] = h->variant.kind;
  out[1] = h->variant.vec;
  out[2] = h->variant.block;
  out[3] = h->variant.stages;
  return LBM_OK;
}

int lbm_tuning(LbmHandle* h, double* ms_per_candidate, int* ncandidates) {
  if (!h || !ms_per_candidate || !ncandidates) return fail(LBM_ERR_ARG, "lbm_tuning: null argument");
  *ncandidates = h->ks->nvariants;
  for (int i = 0; i < h->ks->nvariants; ++i) ms_per_candidate[i] = h->tune_ms[i];
  return LBM_OK;
}

int lbm_device_bytes(LbmHandle* h, int64_t* bytes) {
  if (!h || !bytes) return fail(LBM_ERR_ARG, "lbm_device_bytes: null argument");
  *bytes = (int64_t)h->dev_bytes;
  return LBM_OK;
}

int lbm_time_steps(LbmHandle* h, int64_t nsteps, double* ms) {
  if (!h || !ms) return fail(LBM_ERR_ARG, "lbm_time_steps: null argument");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  cudaEvent_t e0, e1;
  LBM_CUDA(cudaEventCreate(&e0));
  LBM_CUDA(cudaEventCreate(&e1));
  // graphs are captured before the timed region (capture runs nothing)
  int rc = h->initialized ? h->prepare_graphs(nsteps) : LBM_OK;
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  cudaError_t e = cudaEventRecord(e0, h->stream);
  if (e == cudaSuccess) {
    rc = lbm_step(h, nsteps);
    if (rc == LBM_OK) e = cudaEventRecord(e1, h->stream);
  }
  if (rc == LBM_OK && e == cudaSuccess) rc = h->wait();
  float f = 0.f;
  if (rc == LBM_OK && e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("events: ") + cudaGetErrorString(e));
  *ms = f;
  return LBM_OK;
}

// ---- step state: save / restore -------------------------------------------
namespace {
struct StateHeader {
  char magic[8];   // "LBMSTATE"
  int32_t version;
  int32_t nx, ny, precision, collision, forcing, layout, pitch, nrec;
  int32_t cur, nopull, has_old, old_cur, mov_n;
  int64_t plane, t;
  uint64_t pop_bytes, side_bytes, old_bytes, mov_bytes;
  uint64_t case_hash, omega_hash;
  // launch shapes of the saving handle (launch shapes round FP32 / FP16
  // arithmetic differently, so a restart keeps them instead of re-tuning)
  int32_t tuned, res_tuned;
  int32_t variant[4], res_variant[4];   // kind, vec, block, stages
};
constexpr int32_t kStateVersion = 4;

// Moving-obstacle part of the state: obstacles, node classes and segment
// flags (they follow the obstacles), solid / refill flags, solid velocity and
// the densities the next step's moving bounce-back reads.
struct MovPart {
  void* p;
  size_t bytes;
};
std::vector<MovPart> mov_parts(LbmHandle* h) {
  auto& M = h->mov;
  const size_t plane = h->g.plane, cb = h->ks->compute_bytes;
  if (!M.n) return {};
  return {{M.obs, M.n * sizeof(lbm::MovObs)},
          {const_cast<uint8_t*>(h->g.cls), plane},
          {const_cast<uint8_t*>(h->g.segflag), (size_t)h->g.ny * h->g.nseg},
          {M.dsolid, plane},
          {M.fresh, plane},
          {M.us, 2 * plane * cb},
          {M.rho_dyn[h->cur], plane * cb}};
}

StateHeader state_header(const LbmHandle* h) {
  StateHeader H;
  std::memset(&H, 0, sizeof H);
  std::memcpy(H.magic, "LBMSTATE", 8);
  H.version = kStateVersion;
  H.nx = h->cfg.nx;
  H.ny = h->cfg.ny;
  H.precision = h->cfg.precision;
  H.collision = h->cfg.collision;
  H.forcing = h->cfg.forcing;
  H.layout = h->cfg.layout;
  H.pitch = h->g.pitch;
  H.nrec = h->g.nrec;
  H.cur = h->cur;
  H.nopull = h->nopull ? 1 : 0;
  H.has_old = h->old[0] ? 1 : 0;
  H.old_cur = h->old_cur;
  H.mov_n = h->mov.n;
  for (const MovPart& m : mov_parts(const_cast<LbmHandle*>(h))) H.mov_bytes += m.bytes;
  H.plane = h->g.plane;
  H.t = h->t;
  H.pop_bytes = h->state_bytes();
  H.side_bytes = h->side_bytes();
  H.old_bytes = H.has_old ? 6 * (uint64_t)h->g.plane * h->ks->compute_bytes : 0;
  H.case_hash = h->case_hash;
  H.omega_hash = h->omega_hash;
  H.tuned = h->tuned ? 1 : 0;
  H.res_tuned = h->res_tuned ? 1 : 0;
  const lbm::Variant* vs[2] = {&h->variant, &h->res_variant};
  int32_t* outs[2] = {H.variant, H.res_variant};
  for (int i = 0; i < 2; ++i) {
    outs[i][0] = vs[i]->kind;
    outs[i][1] = vs[i]->vec;
    outs[i][2] = vs[i]->block;
    outs[i][3] = vs[i]->stages;
  }
  return H;
}

// A saved launch shape, if the handle may run it: one of the storage's
// candidates, or for the AA layout the scalar kernel with 32..256 threads.
bool valid_variant(const LbmHandle* h, const int32_t v[4], lbm::Variant* out) {
  const lbm::Variant w{v[0], v[1], v[2], v[3]};
  if (h->aa) {
    if (h->aa_tile_ok(w)) {
      *out = w;
      return true;
    }
    const bool scalar = w.kind == 0 && w.vec == 1;
    const bool pairs = w.kind == 3 && w.vec == 2 && h->cfg.precision != LBM_FP64 && w.stages >= 0 &&
                       w.stages <= 2;
    if (!(scalar || pairs) || w.block < 32 || w.block > 256 || w.block % 32) return false;
    *out = w;
    return true;
  }
  for (int i = 0; i < h->ks->nvariants; ++i) {
    const lbm::Variant& c = h->ks->variants[i];
    if (c.kind == w.kind && c.vec == w.vec && c.block == w.block && c.stages == w.stages) {
      if (h->mov.n && !h->mov_ok(c)) return false;
      *out = c;
      return true;
    }
  }
  return false;
}
}  // namespace

int lbm_state_size(LbmHandle* h, int64_t* bytes) {
  if (!h || !bytes) return fail(LBM_ERR_ARG, "lbm_state_size: null argument");
  const StateHeader H = state_header(h);
  *bytes = (int64_t)(sizeof(StateHeader) + H.pop_bytes + H.side_bytes + H.old_bytes + H.mov_bytes);
  return LBM_OK;
}

int lbm_save_state(LbmHandle* h, void* out) {
  if (!h || !out) return fail(LBM_ERR_ARG, "lbm_save_state: null argument");
  if (!h->initialized) return fail(LBM_ERR_STATE, "lbm_save_state: not initialised");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const StateHeader H = state_header(h);
  char* o = static_cast<char*>(out);
  std::memcpy(o, &H, sizeof H);
  o += sizeof H;
  LBM_CUDA(cudaMemcpyAsync(o, h->pop_raw[h->cur], H.pop_bytes, cudaMemcpyDeviceToHost, h->stream));
  o += H.pop_bytes;
  LBM_CUDA(cudaMemcpyAsync(o, h->side[h->cur], H.side_bytes, cudaMemcpyDeviceToHost, h->stream));
  o += H.side_bytes;
  for (int i = 0; i < 6 && H.has_old; ++i) {
    const size_t b = H.old_bytes / 6;
    LBM_CUDA(cudaMemcpyAsync(o, h->old[i], b, cudaMemcpyDeviceToHost, h->stream));
    o += b;
  }
  for (const MovPart& m : mov_parts(h)) {
    LBM_CUDA(cudaMemcpyAsync(o, m.p, m.bytes, cudaMemcpyDeviceToHost, h->stream));
    o += m.bytes;
  }
  return h->wait();
}

int lbm_load_state(LbmHandle* h, const void* in) {
  if (!h || !in) return fail(LBM_ERR_ARG, "lbm_load_state: null argument");
  StateHeader H;
  std::memcpy(&H, in, sizeof H);
  if (std::memcmp(H.magic, "LBMSTATE", 8) != 0 || H.version != kStateVersion)
    return fail(LBM_ERR_ARG, "lbm_load_state: not a saved state of this library version");
  const StateHeader M = state_header(h);
  if (H.nx != M.nx || H.ny != M.ny || H.precision != M.precision || H.collision != M.collision ||
      H.forcing != M.forcing || H.layout != M.layout || H.pitch != M.pitch || H.plane != M.plane ||
      H.nrec != M.nrec || H.pop_bytes != M.pop_bytes || H.side_bytes != M.side_bytes ||
      H.mov_n != M.mov_n || H.mov_bytes != M.mov_bytes ||
      H.cur < 0 || H.cur > 1 || H.old_cur < 0 || H.old_cur > 1 ||
      H.old_bytes != (H.has_old ? 6 * (uint64_t)h->g.plane * h->ks->compute_bytes : 0))
    return fail(LBM_ERR_ARG, "lbm_load_state: the state was saved from a case with another grid, "
                             "storage, collision, forcing, layout, link table or moving obstacles");
  if (H.case_hash != M.case_hash || H.omega_hash != M.omega_hash)
    return fail(LBM_ERR_ARG, "lbm_load_state: the state was saved from a case with another "
                             "obstacle layout, link table, relaxation parameters or omega map");
  lbm::Variant v_plain = h->variant, v_res = h->res_variant;
  if ((H.tuned && !valid_variant(h, H.variant, &v_plain)) ||
      (H.res_tuned && !valid_variant(h, H.res_variant, &v_res)))
    return fail(LBM_ERR_ARG, "lbm_load_state: the saved launch shape is not one this handle runs");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int rc;
  if (H.has_old && (rc = h->ensure_old())) return rc;
  h->initialized = false;   // until the state is complete
  h->drop_graphs();   // graphs captured earlier hold the old buffer parity
  h->cur = h->aa ? H.cur : 0;   // AA: the phase; two buffers: restore into buffer 0
  const char* p = static_cast<const char*>(in) + sizeof H;
  LBM_CUDA(cudaMemcpyAsync(h->pop_raw[h->cur], p, H.pop_bytes, cudaMemcpyHostToDevice, h->stream));
  p += H.pop_bytes;
  LBM_CUDA(cudaMemcpyAsync(h->side[h->cur], p, H.side_bytes, cudaMemcpyHostToDevice, h->stream));
  p += H.side_bytes;
  const size_t ob = (size_t)h->g.plane * h->ks->compute_bytes;
  for (int i = 0; i < 6 && h->old[0]; ++i) {
    if (H.has_old) {
      LBM_CUDA(cudaMemcpyAsync(h->old[i], p, ob, cudaMemcpyHostToDevice, h->stream));
      p += ob;
    } else {
      LBM_CUDA(cudaMemsetAsync(h->old[i], 0, ob, h->stream));
    }
  }
  for (const MovPart& m : mov_parts(h)) {   // after cur is set: rho_dyn[cur]
    LBM_CUDA(cudaMemcpyAsync(m.p, p, m.bytes, cudaMemcpyHostToDevice, h->stream));
    p += m.bytes;
  }
  if ((rc = h->wait())) return rc;
  h->old_cur = H.has_old ? H.old_cur : 0;
  h->t = H.t;
  h->nopull = H.nopull != 0;
  // the saved launch shapes continue the run in the same rounding; a shape
  // not yet tuned when the state was saved is tuned by this handle
  if (H.tuned) {
    h->variant = v_plain;
    h->tuned = true;
  }
  if (H.res_tuned) {
    h->res_variant = v_res;
    h->res_tuned = true;
  }
  h->has_moments = false;
  h->clear_residuals();
  h->initialized = true;
  return LBM_OK;
}

int lbm_selftest_bounded_wait(LbmHandle* h, double limit_s, double* waited_s) {
  if (!h || !waited_s) return fail(LBM_ERR_ARG, "lbm_selftest_bounded_wait: null argument");
  if (!(limit_s > 0.0 && limit_s <= 1.0))
    return fail(LBM_ERR_ARG, "lbm_selftest_bounded_wait: limit_s must lie in (0, 1]");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  int rc = h->wait();   // earlier work first: its errors are not the test's
  if (rc) return rc;
  auto* waited = reinterpret_cast<unsigned long long*>(h->red + 15);
  LBM_CUDA(lbm::bounded_wait_selftest(h->err_dev, limit_s, waited, h->stream));
  LBM_CUDA(cudaMemcpyAsync(h->host_red + 15, waited, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  rc = h->wait();
  unsigned long long ns = 0;
  std::memcpy(&ns, h->host_red + 15, sizeof ns);
  *waited_s = ns * 1e-9;
  return rc;
}

int lbm_synchronize(LbmHandle* h, double timeout_s) {
  if (!h) return fail(LBM_ERR_ARG, "lbm_synchronize: null handle");
  LBM_CUDA(cudaSetDevice(h->cfg.device));
  const double keep = h->timeout_s;
  if (timeout_s > 0) h->timeout_s = timeout_s;
  int rc = h->wait();
  h->timeout_s = keep;
  return rc;
}

}  // extern "C"
