/*
 * lbm_gb300.h -- C-ABI of the GB300 fluidLB D2Q9 step (liblbm_gb300.so).
 *
 * The reference (Malyadeep/pylabolt) is pure Python: its hot path is a set of
 * Numba kernels selected by name inside the operator layer.  These entry points
 * replace that layer for one case on one GPU.  Each declaration names the
 * reference code it stands in for.
 *
 * Conventions
 *  - Every call returns an int status (LBM_OK == 0).  lbm_last_error() gives a
 *    message for the last failing call of the calling thread.
 *  - Caller arrays are borrowed for the duration of the call only.  The library
 *    owns all device memory of a handle.  The node, field and population
 *    arrays of lbm_init_fields, lbm_set_body_force, lbm_get_moments,
 *    lbm_get_populations, lbm_set_populations, lbm_forces and
 *    lbm_adjoint_backward may be host memory (pageable or pinned) or device
 *    memory (unified addressing picks the copy direction); device arrays
 *    written by other streams must be complete before the call.
 *  - Node arrays on the host use the reference's inner-node order
 *    ind = x * ny + y (x-major, y fastest), i.e. the padded index
 *    (x+1)*(ny+2)+(y+1) of pylabolt/base/fields.py with the ghost ring removed,
 *    unless a `layout` argument selects the padded form.
 *  - One CUDA stream per handle; a handle is not thread-safe.  Calls that
 *    return data to the host synchronise that stream with a bounded wait
 *    (LBM_ERR_TIMEOUT when it expires).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct LbmHandle LbmHandle;

/* status codes */
#define LBM_OK 0
#define LBM_ERR_ARG 1        /* invalid argument or configuration           */
#define LBM_ERR_CUDA 2       /* a CUDA runtime call failed                   */
#define LBM_ERR_NONFINITE 3  /* the residual pass met a non-finite moment    */
#define LBM_ERR_TIMEOUT 4    /* a bounded device wait expired                */
#define LBM_ERR_STATE 5      /* call out of order (e.g. step before init)    */
#define LBM_ERR_ALLOC 6      /* device allocation failed                     */

/* storage / arithmetic of the populations */
#define LBM_FP64 0           /* f in FP64, reference operation order         */
#define LBM_FP32_SHIFTED 1   /* f - w_i stored in FP32, FP32 arithmetic      */
#define LBM_FP16_SHIFTED 2   /* (f - w_i)*scale stored in FP16, FP32 arithmetic */

/* collision model -- pylabolt/solvers/fluidLB.py:35-40 names */
#define LBM_BGK 0
#define LBM_MRT 1

/* forcing model -- pylabolt/solvers/fluidLB.py:27-33 names */
#define LBM_FORCING_NONE 0
#define LBM_GUO_LINEAR 1
#define LBM_GUO_SECOND_ORDER 2

/* per-direction link kinds of a boundary ("special") node */
#define LBM_LINK_PULL 0   /* f_i(x) <- f*_i(src): plain or periodic-wrapped pull,
                             also the zero_gradient source                      */
#define LBM_LINK_ZERO 1   /* f_i(x) <- 0: pull from a ghost node nobody fills   */
#define LBM_LINK_BB 2     /* f_i(x) <- f*_ibar(x): halfway bounce-back          */
#define LBM_LINK_MBB 3    /* f_i(x) <- f*_ibar(x) - 2 w rho(x) inv_cs_2 param:
                             moving wall / moving solid, param = c_ibar . u_w   */
#define LBM_LINK_ABB 4    /* f_i(x) <- -f*_ibar(x) + 2 w rho_w (1 + ...):
                             anti-bounce-back, param = rho_w, aux = node x+n    */

/* moment layouts for lbm_get_moments / lbm_init_fields */
#define LBM_LAYOUT_INNER 0   /* [nx*ny], ind = x*ny + y                    */
#define LBM_LAYOUT_PADDED 1  /* [(nx+2)*(ny+2)], ind = x*(ny+2) + y, ghosts 0 */

/* population layouts (LbmConfig.layout) */
#define LBM_POP_AB 0   /* two buffers: a step pulls from one, writes the other   */
#define LBM_POP_AA 1   /* one buffer, in place (AA pattern): even steps read and
                          write each node's own slots (swapped), odd steps pull
                          from and push to the neighbours' slots.  Half the
                          population memory.  Not with moving obstacles, the
                          adjoint or zero_gradient links.  Its launch shape
                          is fixed per storage (no autotuner trials: they
                          would advance the state): the scalar kernel for
                          FP64, node pairs for FP32, node-pair tiles for
                          FP16. */

/* flags of lbm_step_ex: what the last step of the call records */
#define LBM_STEP_MOMENTS 1   /* keep rho/u of that step for lbm_get_moments */
#define LBM_STEP_RESIDUAL 2  /* evaluate the residual for lbm_residual      */

typedef struct {
  int32_t nx, ny;          /* inner grid (mesh_dict["grid"])                   */
  int32_t precision;       /* LBM_FP64 / LBM_FP32_SHIFTED / LBM_FP16_SHIFTED   */
  int32_t collision;       /* LBM_BGK / LBM_MRT                                */
  int32_t forcing;         /* LBM_FORCING_NONE / LBM_GUO_*                     */
  int32_t body_force_field;/* 1: per-node force field replaces rho*g           */
  int32_t device;          /* CUDA device ordinal                              */
  int32_t layout;          /* LBM_POP_AB (default) / LBM_POP_AA                */
  double omega;            /* 1/tau, tau = kin_visc*inv_cs_2 + 0.5             */
  double inv_cs_2, inv_cs_4; /* pylabolt/base/lattice.py:41-44 values           */
  double eps;              /* control.float_min (FP64 eps)                     */
  double gravity[2];       /* forcing_dict["gravity"]; zero for forcing None   */
  double mrt_s[4];         /* s_e, s_eps, s_q, s_nu (MRT only)                 */
  double fp16_scale;       /* storage scale of LBM_FP16_SHIFTED (power of 2)   */
} LbmConfig;

/* Links of one boundary node: every node whose nine incoming populations are
 * not all plain in-domain pulls (domain edges, periodic edges, solid
 * neighbours) and every node whose moments an anti-bounce-back link reads. */
typedef struct {
  int64_t node;            /* inner index x*ny + y                          */
  int64_t src[9];          /* PULL: source node (inner index)               */
  int64_t aux[9];          /* ABB: node x+n (inner index; must be listed)   */
  double param[9];         /* MBB: c_ibar . u ; ABB: rho_w                  */
  int8_t type[9];          /* LBM_LINK_*                                    */
  int8_t wall;             /* 1: the MBB links come from a fixed_velocity
                              boundary (their u_w gets a gradient)          */
  int8_t reserved[6];
} LbmNodeLinks;

/* Creates a case on the GPU: geometry, link table and parameters.  Replaces
 * the operator set-up of Solver.__init__/set_backend
 * (pylabolt/solvers/fluidLB.py:109-204: State, CollisionOperator,
 * ForceOperator, StreamingOperator, BoundaryOperator kernel binding).
 * node_solid: [nx*ny] bytes, 1 = solid (pylabolt/base/fields.py `solid`). */
int lbm_create(const LbmConfig* cfg, const uint8_t* node_solid,
               const LbmNodeLinks* links, int64_t nlinks, LbmHandle** out);

/* Sets rho/u and the populations entering the next step to f_eq(rho, u) on
 * fluid nodes; solid nodes keep rho/u as given (reported by lbm_get_moments).
 * Replaces initialize_pop_density_based_second_order
 * (pylabolt/parallel/cpu/equilibrium_kernels.py:38-78) and the initial
 * fields of pylabolt/base/init_fields.py.  rho: [n], u: [n][2] in `layout`.
 * Host arrays are copied into a device staging buffer and transposed there;
 * with LBM_HOST_DIRECT=1 (read at lbm_create) pinned host arrays are read in
 * place by the transposing kernel over the host link, where the device can
 * reach pageable memory (Grace-Blackwell), and lbm_get_moments writes pinned
 * inner-layout arrays the same way.  The values are the same either way. */
int lbm_init_fields(LbmHandle* h, const double* rho, const double* u, int layout);

/* As lbm_init_fields with FP32 fields: a case with "precision": "single"
 * holds state.fields.density/velocity as float32 (pylabolt/base/control.py:36-40,
 * pylabolt/base/fields.py:64-77).  The values are widened exactly, so the
 * state equals lbm_init_fields on the same values as doubles; half the bytes
 * cross the host link. */
int lbm_init_fields_f32(LbmHandle* h, const float* rho, const float* u, int layout);

/* Sets a per-node body force field F[n][2] (inner layout) used instead of
 * rho*g when cfg.body_force_field == 1 (extension: no reference key). */
int lbm_set_body_force(LbmHandle* h, const double* force);

/* Per-node relaxation rate omega [nx*ny] (inner layout), constant inside
 * every 32-node row segment (x / 32) of fluid nodes; replaces cfg.omega for
 * BGK with shifted storage.  Used to advance many cases of different
 * viscosity in one grid (extension: the reference has one omega per run,
 * collision_operator.py:89-91). */
int lbm_set_omega_map(LbmHandle* h, const double* omega);

/* Advances nsteps time steps, each one Solver.single_time_step
 * (pylabolt/solvers/fluidLB.py:206-253: density, force, velocity, collide,
 * periodic wrap, stream, boundaries) as one fused kernel launch.  Runs of
 * steps are replayed from captured CUDA graphs: 32-step chunks and the rest
 * of the call as one graph (the reference captures one step,
 * fluidLB.py:270-287). */
int lbm_step(LbmHandle* h, int64_t nsteps);

/* As lbm_step; the last step also records what `flags` asks for
 * (LBM_STEP_MOMENTS / LBM_STEP_RESIDUAL).  The host loop of Solver.run
 * (fluidLB.py:352-384) calls this on std_out_interval / save_interval steps. */
int lbm_step_ex(LbmHandle* h, int64_t nsteps, int flags);

/* rho/u of the last step recorded with LBM_STEP_MOMENTS: the fields the
 * reference holds in state.fields.density/velocity after that step and writes
 * with InputOutputOperator.write_fields (pylabolt/utils/io_operator.py:158-190).
 * rho: [n], u: [n][2] in `layout`. */
int lbm_get_moments(LbmHandle* h, double* rho, double* u, int layout);

/* As lbm_get_moments into FP32 fields (single-precision cases), each value
 * the FP64 result rounded to nearest; exact for FP32 and FP16 storage, whose
 * moments are FP32 values. */
int lbm_get_moments_f32(LbmHandle* h, float* rho, float* u, int layout);

/* Residuals {res_rho, res_ux, res_uy} of the last LBM_STEP_RESIDUAL step:
 * sqrt(sum (phi-phi_old)^2 / (sum phi_old^2 + eps)) over fluid nodes, phi_old
 * from the previous residual step (zeros at first) -- ResidueOperator,
 * pylabolt/utils/residues.py:171-222.  Returns LBM_ERR_NONFINITE when that
 * pass met a non-finite rho or u. */
int lbm_residual(LbmHandle* h, double out[3]);

/* The same residuals for the residual step that ended at time step t (t as
 * lbm_time reports it), which must be one of the last eight residual steps
 * since initialisation (LBM_ERR_STATE otherwise).  Waits for that step only,
 * not for the steps queued after it: a host loop can read step t's residual
 * while step t+1 runs, as the reference's run loop logs each step's residues
 * (pylabolt/solvers/fluidLB.py:364-375). */
int lbm_residual_at(LbmHandle* h, int64_t t, double out[3]);

/* FP64 sums over fluid nodes of the stored post-collision populations:
 * {sum f, sum cx f, sum cy f} (mass and momentum diagnostics; extension). */
int lbm_conservation(LbmHandle* h, double out[3]);

/* Post-collision populations of the last step (the reference's pop_fluid),
 * FP64 in the padded AoS layout [(nx+2)*(ny+2)][9] of
 * pylabolt/base/fields.py:83-92; ghost and solid nodes are 0. */
int lbm_get_populations(LbmHandle* h, double* pop);

/* Sets the populations entering the next step (the reference's pop_fluid_new)
 * from the padded AoS layout; the next step starts from them directly. */
int lbm_set_populations(LbmHandle* h, const double* pop_new);

/* Forward pass that keeps what lbm_adjoint_backward needs (extension: the
 * reference has no adjoint).  Starts from the fields of the last
 * lbm_init_fields, runs nsteps steps, stores the state every `interval`
 * steps (1 = every step; states in between are recomputed by the backward
 * pass) and records the moments of the last step (lbm_get_moments).
 * Supported: BGK with Guo forcing none/linear/second order; links PULL,
 * ZERO, BB, MBB (no anti-bounce-back, no zero_gradient); FP64 or FP32
 * shifted storage. */
int lbm_adjoint_forward(LbmHandle* h, int64_t nsteps, int interval);

/* Reverse pass of the last lbm_adjoint_forward.  grad_u: dL/du of the last
 * step's velocity, [nx*ny][2] inner layout (FP64).  Outputs (NULL to skip):
 * grad_force [nx*ny][2] = dL/dF of the body-force field, *grad_tau = dL/dtau,
 * grad_uwall[2] = dL/du_w of the fixed_velocity links marked `wall`.  The
 * discrete adjoint of the step kernels' own arithmetic, with
 * checkpoint-and-recompute between stored states. */
int lbm_adjoint_backward(LbmHandle* h, const double* grad_u, double* grad_force,
                         double* grad_tau, double* grad_uwall);

/* One momentum-exchange link: node x, the population k_out leaving x towards
 * a solid node or a wall, and k_in, the population coming back along the
 * opposite direction.  Its contribution to its group (an obstacle or a wall
 * boundary element) is
 *     v = pop[x,k_out] c_{k_out} - pop_new[x,k_in] c_{k_in}
 *     force += v,  torque += rx v_y - ry v_x
 * with pop the post-collision populations of the last step and pop_new the
 * populations after its streaming and boundaries.  (rx, ry) is the lever arm
 * from the group's reference point (minimum image on periodic axes). */
typedef struct {
  int64_t node;            /* inner index x*ny + y; must have a link record */
  int32_t group;           /* 0 .. ngroups-1                                */
  int8_t k_out, k_in;      /* D2Q9 directions, k_in = opposite of k_out     */
  int8_t reserved[2];
  double rx, ry;           /* lever arm (obstacles); 0 for wall elements    */
} LbmForceLink;

/* Registers the momentum-exchange links (replaces the argument set-up of
 * ObstacleOperator / BoundaryOperator force computation,
 * pylabolt/base/obstacle_operator.py:75-114, boundary_operator.py:362-397).
 * A later call replaces the previous set. */
int lbm_set_force_links(LbmHandle* h, const LbmForceLink* links, int64_t nlinks, int ngroups);

/* Force and torque of every group on the current state, FP64:
 * out[g*3 + {0,1,2}] = {fx, fy, torque}.  Replaces
 * compute_force_torque_single_phase and compute_boundary_force_single_phase
 * (pylabolt/parallel/cpu/force_torque_kernels.py:11-141) evaluated after a
 * time step (fluidLB.py:249-253, :361-366); right after lbm_init_fields it
 * gives the t = 0 values (pop = pop_new = f_eq, fluidLB.py:323-335). */
int lbm_forces(LbmHandle* h, double* out);

/* A circular or elliptic obstacle that moves (extension: the reference's moving-obstacle
 * path cannot run, pylabolt/base/obstacle_operator.py:47-73 calls an undefined
 * reconstruct_obstacles).  Each step, before the fused step:
 *   1. motion (update_position_velocity, pylabolt/parallel/cpu/
 *      obstacle_kernels.py:386-460, from the last step's force / torque):
 *      calculated: omega += T/I (rotation), v += F/m + g (translation);
 *      angle += omega_old + T/(2I); center += v_old + (F/m + g)/2;
 *   2. re-rasterisation: (x-cx)^2 + (y-cy)^2 <= r^2 is solid (an ellipse:
 *      its semi-axes at the angle reached, construct_ellipse, obstacle_kernels.py:
 *      192-241), with velocity v + omega x r and the obstacle's density;
 *      nodes it leaves become fluid
 *      and are refilled with f_eq(mean rho of their fluid neighbours, the
 *      wall velocity they had);
 *   3. fluid nodes next to it pull moving-solid bounce-back
 *      pop[x,kbar] - 2 w rho(x) inv_cs_2 (c_kbar . u_solid) at run time
 *      (streaming_kernels.py:41-47);
 * and after it the momentum exchange on the obstacle (force_torque_kernels.py:
 * 11-90) feeds the next motion.  An obstacle must stay two nodes away from
 * the domain edges and from static solids / boundary nodes, and move less
 * than one node per step; a step that would break this fails with
 * LBM_ERR_STATE and leaves the obstacle where it was. */
typedef struct {
  double center[2];        /* position, lattice units                        */
  double radius;           /* circle radius; for an ellipse its semi-major
                              axis (the radius of the box it moves in)      */
  double velocity[2];      /* linear velocity                                */
  double omega;            /* angular velocity                               */
  double angle;            /* inclination (radians); an ellipse's major axis
                              lies at this angle to x and turns with it     */
  double mass, inertia;    /* pi r^2 rho_s and m r^2 / 2 (pi a b rho_s and
                              m (a^2 + b^2) / 4 for an ellipse, obstacle.py) */
  double density;          /* rho_s: the density reported on its nodes       */
  double force[2], torque; /* momentum exchange of the last step (output)    */
  int32_t id;              /* obstacle id: reference order in obstacle_dict  */
  int32_t calculated;      /* 1: velocities follow the force and torque      */
  int32_t rotation, translation;  /* degrees of freedom                      */
  double semi_axes[2];     /* ellipse: semi-major a, semi-minor b            */
  int32_t shape;           /* 0 circle, 1 ellipse                            */
  int32_t reserved;
} LbmMovingObstacle;

/* Registers the moving obstacles (at most 32) and the gravity of their
 * motion; call after lbm_create.  lbm_init_fields must follow before the next
 * step (it places them).  The scalar step kernel or the node-pair kernel's
 * 40-register shape serves a case with moving obstacles. */
int lbm_set_moving_obstacles(LbmHandle* h, const LbmMovingObstacle* obs, int n,
                             const double gravity[2]);

/* Current state of the moving obstacles (position, velocities, force and
 * torque of the last step), in registration order. */
int lbm_get_moving_obstacles(LbmHandle* h, LbmMovingObstacle* out);

/* Node flags of the current geometry, inner layout [nx*ny]: 0 fluid, 1 static
 * solid, 2 + i solid of moving obstacle i (registration order). */
int lbm_get_node_flags(LbmHandle* h, uint8_t* flags);

/* Checkpoint / restart of the step state (extension: the reference reads
 * control_dict["checkpoint_interval"] but writes no checkpoint).  The state
 * is the current population buffer (storage type, guard rows included), the
 * boundary nodes' side array, the residual's previous-step fields when they
 * exist, the time and the layout phase, and with moving obstacles their
 * device state (obstacles, node classes, solid / refill flags, solid velocity,
 * bounce-back densities), behind a versioned header.  A state loads into a
 * handle created with the same configuration, link table and number of moving
 * obstacles (after lbm_init_fields); the run then continues bit for bit. */
int lbm_state_size(LbmHandle* h, int64_t* bytes);
int lbm_save_state(LbmHandle* h, void* out);        /* out: lbm_state_size bytes */
int lbm_load_state(LbmHandle* h, const void* in);

/* Number of completed steps since the last init. */
int lbm_time(LbmHandle* h, int64_t* t);

/* Number of fused step-kernel launches issued since the handle was created. */
int lbm_kernel_launches(LbmHandle* h, int64_t* n);

/* Launch shape of the fused step picked by the autotuner on the first step:
 * out = {kind (0 scalar, 2 node pairs from shared-memory tiles, 3 node pairs),
 * nodes per thread, threads per block, stages (kind 2: shared-memory stages;
 * kinds 0 and 3: register cap)}.  LBM_VARIANT="kind,vec,block,stages"
 * forces one candidate, LBM_TUNE=0 keeps the first.  (Extension: the
 * reference launches every kernel with 256 threads, backend.py:59-75.) */
int lbm_kernel_variant(LbmHandle* h, int out[4]);

/* Per-candidate mean step time (ms) measured by the autotuner; *n receives the
 * number of candidates (at most 16). */
int lbm_tuning(LbmHandle* h, double* ms_per_candidate, int* n);

/* Device bytes held by the handle. */
int lbm_device_bytes(LbmHandle* h, int64_t* bytes);

/* Runs `nsteps` as lbm_step and returns the elapsed device time in
 * milliseconds, measured with CUDA events on the handle's stream. */
int lbm_time_steps(LbmHandle* h, int64_t nsteps, double* ms);

/* Waits (bounded by timeout_s seconds) for all work of the handle. */
int lbm_synchronize(LbmHandle* h, double timeout_s);

/* Self-test of the device-side bounded waits (no counterpart in the
 * reference, which only aborts: pylabolt/base/state.py:121-125).  Runs a
 * kernel that waits on an mbarrier nobody arrives at, with the same bounded
 * wait the pipelined step kernel uses, limited to limit_s (0 < limit_s <= 1).
 * The wait gives up, the kernel sets the handle's error word and returns;
 * the call then reports LBM_ERR_TIMEOUT like a step whose wait expired, with
 * *waited_s the time the kernel waited.  The handle stays usable. */
int lbm_selftest_bounded_wait(LbmHandle* h, double limit_s, double* waited_s);

/* A population array owned by the caller, in device memory: value of node
 * (x, y), direction k at pop[k*plane + y*pitch + x], stored as f (LBM_FP64),
 * g = f - w_k (LBM_FP32_SHIFTED) or g * fp16_scale in IEEE half
 * (LBM_FP16_SHIFTED).  Directions k = 0..8 have (cx, cy) = (0,0), (1,0),
 * (0,1), (-1,0), (0,-1), (1,1), (-1,1), (-1,-1), (1,-1) and weights
 * w_k = 4/9 (k = 0), 1/9 (k = 1..4), 1/36 (k = 5..8). */
typedef struct {
  int32_t precision;
  int32_t nx, ny;
  int32_t reserved;
  int64_t pitch;            /* elements from one row to the next            */
  int64_t plane;            /* elements from one direction to the next      */
  const void* pop;          /* device pointer                               */
  const uint8_t* exclude;   /* device pointer or NULL: [y*pitch + x] != 0
                               leaves the node out (e.g. solid nodes)       */
  double fp16_scale;
} LbmPopView;

#define LBM_NOALLOC_MAX_ROWS 8192

/* No counterpart in the reference.  Same sums as lbm_conservation
 * ({sum f, sum cx f, sum cy f} over the nodes not excluded, FP64), for a
 * population array the caller owns, for callers that cannot allocate device
 * memory: code embedded in a host application that hands out all device
 * memory from its own pool, or monitoring loops that cannot take cudaMalloc's
 * implicit synchronisation.  It allocates nothing: its scratch is a fixed
 * device array inside the library (LBM_NOALLOC_MAX_ROWS + 64 rows of 8
 * doubles, about 0.5 MB, held by every GPU that loads the library until the
 * process exits).  out_device receives 3 doubles; the work is queued on
 * `stream` (a cudaStream_t, NULL for the default stream) and the call returns
 * without waiting.  ny above LBM_NOALLOC_MAX_ROWS is rejected (LBM_ERR_ARG).
 * The first call on each device, with that device current, looks up the
 * scratch array's device address (cudaGetSymbolAddress) and keeps it for the
 * life of the process, so make that first call before any stream capture;
 * after a cudaDeviceReset of that device the kept address is stale and the
 * entry point must not be called again in that process.  All calls share the
 * one scratch array, which keeps the last call's partial sums (each call
 * overwrites every row it reads, so nothing needs clearing): calls whose
 * work overlaps on the GPU (other streams, or other host threads on the same
 * device) race and must be serialised by the caller. */
int lbm_conservation_noalloc(const LbmPopView* view, double* out_device, void* stream);

/* Message of the last failing call on this thread ("" if none). */
const char* lbm_last_error(void);

/* Releases the handle and its device memory. */
int lbm_destroy(LbmHandle* h);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
