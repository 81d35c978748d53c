/*
 * yarnsim.h -- C ABI of the GB300 yarn-level cloth step.
 *
 * One handle (ys_batch) holds any number of cloths of uneven sizes, each a
 * W x L grid of yarn crossings with 5 DOFs per interior crossing (x, y, z and
 * the Eulerian u, v) and 3 per boundary crossing, exactly as the reference's
 * Cloth (src/Cloth.h:40-84). The handle owns every device buffer; callers pass
 * host pointers (copied on the handle's stream) or device pointers (flagged by
 * YS_ON_DEVICE) and never see CUDA or torch types.
 *
 * Reference interface each entry point replaces (paths relative to the
 * reference project root):
 *   ys_batch_create   Cloth::Cloth + Cloth::set_handles + Environment +
 *                     PhysicsCloth::InitMV  (src/Cloth.cpp:3-50, 386-394;
 *                     src/Environment.h:16-21; src/PhysicsCloth.cpp:3-44)
 *   ys_set_state      Cloth::set_ClothState        (src/Cloth.cpp:421-438)
 *   ys_get_state      Cloth::get_ClothState        (src/Cloth.cpp:350-371)
 *   ys_set_wind(s)    Environment::wind            (src/Wind.h:6-17)
 *   ys_assemble       PhysicsCloth::FillMV + the A, b formation of SimStep
 *                     (src/PhysicsCloth.cpp:46-156; src/TrainHelper.cpp:19-20)
 *   ys_export_system  PhysicsCloth::get_SpaM/get_SpaFPos/get_SpaFVel/get_SpaF
 *                     combined into A and b, dense reference layout
 *                     (src/PhysicsCloth.h:72-77, src/MatrixMp.cpp:40-111)
 *   ys_solve          EigenSolver::apply on the assembled system
 *                     (src/Solvers.h:35-52, src/Solvers.cpp:3-31)
 *   ys_step           SimStep (src/TrainHelper.cpp:15-54) and
 *                     SimStep(..., ext_force) (src/TrainHelper.cpp:56-97)
 *   ys_step_tangent(_ext)  the gradient LibTorch's autograd takes through
 *                     SimStep and EigenSolver's backward (src/Solvers.cpp:
 *                     33-58), forward mode, parameters or external force
 *   ys_collider_*     Collision::find_impacts (src/Collision.cpp:184-208),
 *                     Collision::collision_response (src/Collision.cpp:
 *                     73-156) and InelasticProjection's backward
 *                     (src/Collision.cpp:496-682)
 *
 * Error convention: every call returns a ys_status; a cloth whose system or
 * solution is non-finite is reported per cloth (SimStep returning false,
 * src/TrainHelper.cpp:22-48) and left unchanged. Nothing ever exits (a
 * response that does not converge returns YS_ERR_MAXITER where the
 * reference exits the process).
 * Threading: one handle per host thread; calls are ordered on the handle's
 * stream.
 */
#ifndef YARNSIM_H
#define YARNSIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  YS_OK = 0,
  YS_ERR_ARG = 1,        /* invalid argument */
  YS_ERR_CUDA = 2,       /* a CUDA call failed (message via ys_last_error) */
  YS_ERR_NONFINITE = 3,  /* at least one cloth had a non-finite system or solution */
  YS_ERR_MAXITER = 4     /* at least one cloth stopped at the PCG iteration cap */
} ys_status;

/* flags */
#define YS_ON_DEVICE 1 /* pointers are device pointers (else host) */

typedef struct ys_batch ys_batch;

/* Construction parameters of one cloth, in the reference's own units
 * (Cloth(W, L, height, L_, R, yarns, kc, kf, df, mu, S, handle_stiffness,
 * WovenPattern, InitPose), src/Cloth.h:55-60, plus gravity and wind).
 * Yarn material is given per yarn line: warp line j is node row v = j
 * (`length` entries), weft line i is node column u = i (`width` entries);
 * ks = Y*PI*R^2 and kb = B*PI*R^2 (src/Yarn.h:12-16). */
typedef struct {
  int32_t width, length;
  double height, L, R;
  int32_t pose;  /* 0 Upright, 1 Flat  (src/Cloth.cpp:57-59) */
  int32_t weave; /* 0 Plain, 1 Twill, 2 Satin (src/Cloth.cpp:69-92) */
  const double *warp_rho, *warp_Y, *warp_B;
  const double *weft_rho, *weft_Y, *weft_B;
  double kc, kf, df, mu, S, handle_stiffness;
  double G[3];
  double wind_vel[3];
  double wind_density, wind_drag;
  int32_t n_handles;
  const int32_t *handles; /* n_handles (u, v) pairs */
} ys_cloth_desc;

typedef struct {
  double tol;         /* relative residual |r| / |b|; <= 0: DBL_EPSILON (Eigen default) */
  int32_t maxiter;    /* per cloth; < 0: 2 * system dimension (Eigen default) */
  int32_t check_every;/* iterations between convergence checks; <= 0: the batch's default
                         (16, or what ys_autotune chose) */
} ys_solve_opts;

typedef struct {
  int32_t ok;         /* 1 if the step succeeded (SimStep's return value) */
  int32_t cg_iterations;
  double cg_error;    /* sqrt(|r|^2 / |b|^2) at exit */
  int32_t hit_maxiter;
} ys_cloth_stats;

typedef struct {
  int32_t n_cloths;
  int64_t total_nodes;      /* sum of width*length */
  int64_t device_bytes;     /* device memory held by the handle */
} ys_batch_info;

const char *ys_last_error(void);

ys_status ys_batch_create(int32_t n_cloths, const ys_cloth_desc *descs, int32_t device, void *cuda_stream,
                          ys_batch **out);
void ys_batch_destroy(ys_batch *b);
ys_status ys_batch_get_info(const ys_batch *b, ys_batch_info *info);
/* node offset of cloth c inside the batch's node-ordered arrays */
int64_t ys_cloth_node_offset(const ys_batch *b, int32_t c);
/* system dimension of cloth c in the reference's layout: 3*W*L + 2*(W-2)*(L-2) */
int64_t ys_cloth_dim(const ys_batch *b, int32_t c);

/* Node-ordered state of the whole batch (node = offset(c) + u + v*W):
 * lpos, lposfix, lvel: [total_nodes][3]; epos, eposbar, evel: [total_nodes][2].
 * Any pointer may be NULL (that field is left untouched). Host arrays in
 * page-locked memory (cudaMallocHost / cudaHostAlloc / cudaHostRegister) are
 * read or written by the device directly; pageable ones go through a device
 * stage. Either way both calls return once the host arrays are read or
 * filled. */
ys_status ys_set_state(ys_batch *b, const double *lpos, const double *lposfix, const double *lvel,
                       const double *epos, const double *eposbar, const double *evel, int32_t flags);
ys_status ys_get_state(ys_batch *b, double *lpos, double *lposfix, double *lvel, double *epos, double *eposbar,
                       double *evel, int32_t flags);
/* Node normals [total_nodes][3] of the current positions: NodeNorm
 * (src/Cloth.cpp:440-463) of every interior node, as Cloth::UpdateClothUnits
 * leaves them (src/Cloth.cpp:307-348); zero for boundary nodes. */
ys_status ys_get_normals(ys_batch *b, double *normals, int32_t flags);
ys_status ys_set_wind(ys_batch *b, int32_t cloth, const double wind_vel[3]);
/* Wind velocity of every cloth at once: [n_cloths][3] (one copy). */
ys_status ys_set_winds(ys_batch *b, const double *wind_vel, int32_t flags);

/* FillMV + A, b for step size h; ext_force: NULL or [total_nodes][5] (node
 * layout x, y, z, u, v; the u, v entries of boundary nodes are ignored). */
ys_status ys_assemble(ys_batch *b, double h, const double *ext_force, int32_t flags);
/* Dense copy of cloth c's assembled A (dim x dim, row-major) and b (dim), in
 * the reference's DOF order; meant for checks on small cloths. */
ys_status ys_export_system(ys_batch *b, int32_t cloth, double *A, double *rhs);
/* Jacobi-PCG on the assembled systems; the solution stays on the device. */
ys_status ys_solve(ys_batch *b, const ys_solve_opts *opts, ys_cloth_stats *stats);
/* Solution of the last ys_solve in node layout [total_nodes][5]. */
ys_status ys_get_solution(ys_batch *b, double *x, int32_t flags);
/* One SimStep for every cloth: assemble, solve, update. stats: NULL or
 * n_cloths entries (host). */
ys_status ys_step(ys_batch *b, double h, const double *ext_force, int32_t flags, const ys_solve_opts *opts,
                  ys_cloth_stats *stats);
/* Whole-step CUDA graphs (no counterpart in the reference): with enable = 1,
 * ys_step runs as one graph launch -- the assembly kernels, a conditional
 * while node over the PCG iterations (check_every of them per trip, ending
 * when no cloth iterates or at the iteration cap), the check and the update --
 * captured on first use and again when h, the presence of an external force
 * or the solve options change. Results equal the launch-by-launch step bit
 * for bit. Ignored while ys_profile is on. The graph's kernels keep the PCG
 * vectors in L2 through an access-policy window on the handle's own capture
 * stream, for which the first graph build sets this context's persisting-L2
 * limit (cudaLimitPersistingL2CacheSize) to the window's size, at most the
 * device's maximum; the caller's stream is not changed. */
ys_status ys_use_graphs(ys_batch *b, int32_t enable);
/* ys_step through the graph regardless of ys_use_graphs. */
ys_status ys_step_graphed(ys_batch *b, double h, const double *ext_force, int32_t flags, const ys_solve_opts *opts,
                          ys_cloth_stats *stats);
/* Step schedule (no counterpart in the reference). */
typedef struct ys_schedule {
  int32_t graphs;      /* 1: one CUDA graph per step (ys_use_graphs) */
  int32_t check_every; /* PCG iterations between convergence checks (phase PCG) */
  double ms_per_step;  /* measured time of the chosen schedule */
  int32_t pcg;         /* YS_PCG_PHASES or YS_PCG_PERSISTENT */
  int32_t pcg_threads; /* persistent PCG: threads per CTA (128, 256, 512, 1024) */
  int32_t pcg_cluster; /* persistent PCG: CTAs per cloth (1, 2, 4, 8, 16) */
  int32_t producer_threads; /* block size of the record producers and the gather (64, 128, 256) */
} ys_schedule;
/* PCG schedules. Both run Eigen's Jacobi-PCG with the same arithmetic and the
 * same summation order, so they give bit-identical solutions:
 *  - phases: three launches per iteration over every 128-node block of the
 *    batch (SpMV, axpy, direction), convergence checked every check_every
 *    iterations (the default);
 *  - persistent: one launch for the whole solve, a cluster of pcg_cluster CTAs
 *    of pcg_threads threads per cloth, each thread owning one node; needs
 *    width * length <= pcg_threads * pcg_cluster for every cloth. */
enum { YS_PCG_PHASES = 0, YS_PCG_PERSISTENT = 1 };
/* Selects the PCG schedule for every later solve of the batch (steps, tangent
 * and adjoint solves). YS_ERR_ARG if a cloth does not fit the persistent shape
 * or the GPU cannot hold one cluster of it. */
ys_status ys_set_pcg_schedule(ys_batch *b, int32_t pcg, int32_t threads, int32_t cluster);
/* Block size of the element-record producers and the gather (a multiple of
 * 32 up to 256; default 128; the edges use at most 128). Results do not
 * depend on it: one thread per element, nothing shared. */
ys_status ys_set_producer_threads(ys_batch *b, int32_t threads);
/* Times every schedule over `steps` steps of size h without an external force,
 * each from the batch's current state, which is restored afterwards, and makes
 * the fastest the batch's default: graph or launch by launch x (phase PCG with
 * check_every in {2, 4, 8, 16, 32}, or persistent PCG in every cluster shape
 * that holds the largest cloth with at most 4x its nodes), then the producer
 * block sizes 64, 128, 256 under the best of those. All schedules give
 * bit-identical states. */
ys_status ys_autotune(ys_batch *b, double h, const ys_solve_opts *opts, int32_t steps, ys_schedule *best);
/* The schedules the last ys_autotune timed, with their times: copies up to
 * cap of them to out and returns how many there were (-1: null handle). */
int32_t ys_autotune_results(const ys_batch *b, ys_schedule *out, int32_t cap);
/* y = A x with the assembled matrices (node layout [total_nodes][5]). */
ys_status ys_apply_system(ys_batch *b, const double *x, double *y, int32_t flags);
/* y = A x like ys_apply_system, for callers that must not allocate at call
 * time (device memory owned by another allocator; loops that cannot take the
 * synchronisation an allocation may imply). No counterpart in the reference.
 * x and y are DEVICE pointers in node layout [total_nodes][5]; the call is
 * asynchronous on the handle's stream. It allocates nothing and writes no
 * buffer of the batch: its working memory is one static per-device scratch
 * array holding at most 65,536 nodes (YS_ERR_ARG above that). Nothing in the
 * scratch needs to start at zero. Calls that overlap in time on one device
 * share that scratch and race. The first call on a device looks up the
 * scratch's address (the runtime may load the library's device code then);
 * make it before any stream capture begins. x or y that is not memory of the
 * batch's device (or managed memory) gives YS_ERR_ARG and launches nothing.
 * With profiling on (ys_profile) its two launches are counted but timed in
 * no phase: timing would need CUDA events. */
ys_status ys_apply_system_noalloc(ys_batch *b, const double *x, double *y);
/* Waits for the handle's stream. */
ys_status ys_synchronize(ys_batch *b);

/* ---- Forward-mode sensitivities of the step (tangents).
 * Replaces the gradient path of the reference's parameter learning
 * (YarnSimNet* + loss.backward(), src/TrainHeter.h:194-231, through
 * EigenSolver::backward, src/Solvers.h:35-52 / src/Solvers.cpp:33-58): the
 * reference has 8 learned scalars (rho, Y, B of two yarn types, S, mu), so
 * propagating ys_tangent_count() (4) directional derivatives per cloth alongside
 * the state (more directions: a second pass, or copies of the cloth in one
 * batch with their own seeds)
 * gives d(state_t)/d(theta) for every step t of a rollout at the cost of a few
 * extra solves per step, with no stored trajectory. Directions are seeded on
 * the per-line materials (rho, Y, B), the per-cloth S and mu, and/or the
 * initial state; the tangent of every later state is then exact for the
 * discrete step (A dq = db - dA q). */
enum { YS_TANGENT_EXACT = 0, YS_TANGENT_REFERENCE = 1 };
/* Number of tangent directions a step carries (4). */
int32_t ys_tangent_count(void);
/* Allocates the tangent buffers (about 21 KB per node) and zeroes every
 * tangent. mode: YS_TANGENT_EXACT. */
ys_status ys_tangent_enable(ys_batch *b, int32_t mode);
/* Parameter directions, host arrays, NULL = 0: drho, dY, dB
 * [ys_tangent_count()][total lines] with lines ordered cloth by cloth, warp
 * lines (length) then weft lines (width) as in ys_cloth_desc; dS, dmu
 * [ys_tangent_count()][n_cloths]. */
ys_status ys_tangent_seed(ys_batch *b, const double *drho, const double *dY, const double *dB, const double *dS,
                          const double *dmu);
/* State tangents [ys_tangent_count()][total_nodes][3|2] (NULL = 0 on set,
 * skipped on get); flags as ys_set_state. */
ys_status ys_tangent_set_state(ys_batch *b, const double *dlpos, const double *dlvel, const double *depos,
                               const double *deposbar, const double *devel, int32_t flags);
ys_status ys_tangent_get_state(ys_batch *b, double *dlpos, double *dlvel, double *depos, double *deposbar,
                               double *devel, int32_t flags);
/* ys_step, also advancing the first kact tangent directions (0..ys_tangent_count()). */
ys_status ys_step_tangent(ys_batch *b, double h, const double *ext_force, int32_t flags, const ys_solve_opts *opts,
                          int32_t kact, ys_cloth_stats *stats);
/* The same with tangents of the external force: dext_force [kact][total_nodes][5]
 * (ext_force's layout; NULL = 0), so a control force's parameters can be
 * tangent directions (ForceNet's lift and drag, src/TrainEmbed.h:96-163). */
ys_status ys_step_tangent_ext(ys_batch *b, double h, const double *ext_force, const double *dext_force, int32_t flags,
                              const ys_solve_opts *opts, int32_t kact, ys_cloth_stats *stats);

/* ---- Reverse mode: the adjoint of one step.
 * Replaces the backward pass of the reference's loss.backward() through a
 * rollout (src/TrainHeter.h:194-231, src/TrainControl.h:192-231), i.e.
 * EigenSolver's backward (src/Solvers.cpp:33-58) plus autograd through
 * FillMV's force terms, for any number of inputs at a cost independent of
 * their number: per-node control forces at every step, the state, the
 * materials. One call turns dL/d(state after a step) into dL/d(state
 * before it), dL/d(materials) and dL/d(external force of that step):
 *   q_bar from the update's transpose; lambda = A^-T q_bar (YS_TANGENT_EXACT:
 *   the derivative of the discrete step) or A^-1 q_bar
 *   (YS_TANGENT_REFERENCE: what the reference's autograd computes, A, M and
 *   dF/dv held constant); then -lambda^T d(A q - b) / d(state, materials)
 *   by forward-mode directional derivatives of the residual on copies of the
 *   cloths (512 directions per step, 4 per copy), compressed by a colouring
 *   of the nodes (row blocks depend on nodes within grid distance 4).
 * The adjoint owns a workspace batch of `copies` copies of b's cloths
 * (about 25 KB per copied node); 512 / (4 copies) passes per step. */
typedef struct ys_adjoint ys_adjoint;
/* copies: 1..128 (128: one pass per step). b must outlive the adjoint. */
ys_status ys_adjoint_create(ys_batch *b, int32_t mode, int32_t copies, ys_adjoint **out);
void ys_adjoint_destroy(ys_adjoint *a);
/* One step backwards from the state b holds now (the state at the start of
 * the step, as ys_set_state left it; b's state is not changed). h, ext_force
 * and opts as ys_step. gin[5] = dL/d(LPos, LVel, EPos, EVel, EPosBar after the
 * step) in ys_set_state's node layout ([total_nodes][3|2]; NULL = 0);
 * gout[5] receives dL/d(the same, before the step) (NULL = not returned).
 * gparams[5] (NULL entries skipped) receive dL/d rho, dL/d Y, dL/d B per yarn
 * line ([total lines], ys_tangent_seed's order) and dL/d S, dL/d mu per cloth;
 * gext [total_nodes][5] receives dL/d ext_force (0 where the step ignores
 * it). flags: YS_ON_DEVICE for device arrays. stats: the forward solve. */
ys_status ys_adjoint_step(ys_adjoint *a, double h, const double *ext_force, const double *const *gin,
                          double *const *gout, double *const *gparams, double *gext, int32_t flags,
                          const ys_solve_opts *opts, ys_cloth_stats *stats);

/* Kernel accounting (no counterpart in the reference). Kernel classes: */
enum {
  YS_PROF_GEOM = 0,      /* node normals */
  YS_PROF_EDGES = 1,     /* edge records (mass, gravity, stretch, inertia, dM/dt, contact) */
  YS_PROF_BENDS = 2,     /* bend + crimp records */
  YS_PROF_FACES = 3,     /* wind records */
  YS_PROF_GATHER = 4,    /* row blocks from edge/bend/face records + sliding friction */
  YS_PROF_SHEAR = 5,     /* shear records (with jamming) */
  YS_PROF_FINALIZE = 6,  /* shear into row blocks, handles, external force, Jacobi, finite check */
  YS_PROF_PCG_SETUP = 7,
  YS_PROF_SPMV = 8,      /* stencil SpMV q = A p (+ p.q) */
  YS_PROF_AXPY = 9,      /* x, r update (+ r.r, r.z) */
  YS_PROF_DIR = 10,      /* stop test, p update */
  YS_PROF_UPDATE = 11,   /* Cloth::update */
  YS_PROF_MISC = 12,     /* bookkeeping */
  YS_PROF_GNN = 13,      /* learned preconditioner: features, network, G blocks */
  YS_PROF_PREC = 14,     /* learned preconditioner: z = G^T G r */
  YS_PROF_PCG_PERSIST = 15, /* persistent per-cloth PCG (the whole solve in one launch) */
  YS_PROF_KINDS = 16
};
/* enable = 1 brackets every launch with CUDA events on the handle's stream
 * (adds a little host overhead); the totals accumulate until read. */
ys_status ys_profile(ys_batch *b, int32_t enable);
/* ms[YS_PROF_KINDS] summed event time, launches_per_kind[YS_PROF_KINDS] timed
 * launches, total_launches = every kernel launched by the handle (timed or
 * not) since the last reset. Any pointer may be NULL. */
ys_status ys_profile_read(ys_batch *b, double *ms, int64_t *launches_per_kind, int64_t *total_launches,
                          int32_t reset);

/* ---- Continuous collision detection (broad + narrow phase).
 * Replaces Collision::find_impacts (src/Collision.cpp:184-208) over the
 * cloth mesh and one obstacle mesh: the reference's BVH over 18-DOP CCD
 * boxes (src/BVH.cpp, src/CollisionUtil.cpp:3-9), its traversal
 * (src/Collision.cpp:266-326) and comp_face_impacts' vertex-face and
 * edge-edge tests (src/Collision.cpp:210-253, 327-419). The pair list equals
 * the reference's as a set, each pair oriented as the reference reports it;
 * the order is face-major (the reference's depends on its OpenMP threads). */
typedef struct ys_collider ys_collider;
typedef struct {
  int32_t type;      /* 0 vertex-face, 1 edge-edge */
  int32_t nodes[4];  /* cloth node id, or -1 - id for an obstacle node */
  double t;          /* time of coplanarity in [0, 1] of the step */
  double w[4];       /* barycentric weights (Impact::ws) */
  double n[3];       /* contact normal */
  int64_t pair;      /* index of the face pair in the pair list */
} ys_impact;
/* Faces [(W-1)(L-1)*2][3] of a W x L cloth's mesh in the reference's order
 * (src/Cloth.cpp:271-294) and their edges [F][3][2] (edge k joins face nodes
 * k and k+1, oriented as the reference's mesh edges; NULL to skip). */
ys_status ys_cloth_mesh_topology(int32_t width, int32_t length, int32_t *faces, int32_t *face_edges);
/* A collider for a cloth mesh (node ids 0..n_nodes-1) and an obstacle mesh
 * (n_obs_faces may be 0); thickness dilates the boxes (src/BVH.cpp:268-286);
 * ccd = 1: boxes span both positions of the step. The collider keeps up to
 * three host threads (with the calling one, four) for the cloth tree's build
 * and the response's zone projections, until ys_collider_destroy; its calls
 * are not to be made from two host threads at once. */
ys_status ys_collider_create(int32_t n_nodes, int32_t n_faces, const int32_t *faces, const int32_t *face_edges,
                             int32_t n_obs_nodes, int32_t n_obs_faces, const int32_t *obs_faces, double thickness,
                             int32_t ccd, int32_t device, void *cuda_stream, ys_collider **out);
void ys_collider_destroy(ys_collider *c);
/* Positions at the end (x) and start (x_prev) of the step, [n][3] each (host,
 * or device with YS_ON_DEVICE); rebuilds both trees as the reference does for
 * every collision_response call. */
ys_status ys_collider_set_positions(ys_collider *c, const double *x, const double *x_prev, const double *obs_x,
                                    const double *obs_x_prev, int32_t flags);
/* Broad phase; n_pairs receives the count. */
ys_status ys_collider_find_pairs(ys_collider *c, int64_t *n_pairs);
/* pairs [n_pairs][3]: first face, second face, 1 if the second is an obstacle face. */
ys_status ys_collider_get_pairs(ys_collider *c, int32_t *pairs, int64_t cap);
/* Narrow phase over the pair list; n_impacts receives the count. */
ys_status ys_collider_find_impacts(ys_collider *c, int64_t *n_impacts);
ys_status ys_collider_get_impacts(ys_collider *c, ys_impact *impacts, int64_t cap);

/* ---- Impact-zone response: Collision::collision_response
 * (src/Collision.cpp:73-156) over the positions given to
 * ys_collider_set_positions (x after the step, x_prev before it). Rounds of
 * GPU detection (after the first, only face pairs with a face next to an
 * active zone), a greedy independent subset of the impacts sorted by time,
 * impact zones with merging, and the inelastic projection of every zone that
 * gained impacts (NormalOpt, src/Collision.h:139-165), solved exactly on the
 * host (the reference's augmented Lagrangian stops at its tolerances);
 * ties in time are broken by type, nodes, weights and normal. node_mass [n]
 * may be NULL (equal masses, as the reference's MeshMass gives). x_out [n][3]
 * receives the positions after the response; v [n][3] (may be NULL) is
 * updated in place as v + damp (x - x_before) / h when any zone moved.
 * Returns YS_ERR_MAXITER when max_iter rounds (the reference's 100) still
 * found impacts, where the reference exits, or when a zone gathers more than
 * the zone limit (65,536 impacts unless ys_collider_set_max_zone_impacts says
 * otherwise; layers tangled beyond what the response resolves keep merging
 * zones); x_out and v are written as they stand. Zones of up to 64 impacts are
 * projected exactly (least-distance programme through NNLS); larger ones -- a
 * cloth's contact patch on an obstacle chains its impacts into one zone --
 * by Hildreth's iterations on the same programme to 1e-13 relative. */
typedef struct {
  int32_t rounds;      /* rounds that found impacts (the reference's iter) */
  int32_t converged;   /* 1: a round found no impact within max_iter */
  int32_t changed;     /* 1: a zone was projected (velocities updated) */
  int32_t zones;       /* impact zones at the end */
  int32_t infeasible;  /* projections whose constraints had no solution (zone left in place) */
  int32_t zone_overflow; /* 1: stopped at a zone larger than the zone limit */
  int64_t impacts;     /* impacts the zones received, over all rounds */
  int64_t projections; /* zone projections */
  int32_t reverted;    /* projections that would have moved a node by more than 4 x (its displacement in
                          the step + thickness) -- nearly contradictory constraints of a crumpling cloth --
                          and sent the zone back to its positions at the start of the step instead */
  int32_t pad_;
  double detect_ms;    /* host wall time in the detection rounds (uploads, GPU detection, downloads) */
  double zones_ms;     /* host wall time in zone building and projections */
} ys_response_info;
ys_status ys_collider_respond(ys_collider *c, const double *node_mass, double h, double damp, int32_t max_iter,
                              double *x_out, double *v, ys_response_info *info);
/* The zone limit of ys_collider_respond (default 65,536 impacts per zone). */
ys_status ys_collider_set_max_zone_impacts(ys_collider *c, int32_t n);
/* The impacts the zones received, in order (info.impacts of them); the
 * pair field holds the round that found each. */
ys_status ys_collider_response_impacts(ys_collider *c, ys_impact *impacts, int64_t cap);
/* Backward of the last response (InelasticProjection::backward,
 * src/Collision.cpp:496-682, and the velocity update): dl_dx, dl_dv [n][3]
 * (either may be NULL) are the gradients of the outputs; dl_dx_in and
 * dl_dv_in [n][3] receive those of the inputs, dl_dw [impacts][4] and
 * dl_dn [impacts][3] (may be NULL) those of each impact's weights and
 * normal. The gradient of a projection's anchor goes to the zone's positions
 * at that projection, as the reference's autograd sends it. With
 * YS_RESPONSE_GRAD_IMPACTS the weight and normal gradients are carried on
 * into the positions each impact was computed from (collision_test's cubic
 * root, positions at the root, signed distances), and dl_dx_prev [n][3]
 * (may be NULL) receives the part for the step's start positions; the root's
 * derivative is the reference's CubicSolver backward unless
 * YS_RESPONSE_GRAD_EXACT_ROOT is also set (that backward lacks the minus sign
 * of the implicit derivative, src/Solvers.cpp:172-178). */
#define YS_RESPONSE_GRAD_IMPACTS 1
#define YS_RESPONSE_GRAD_EXACT_ROOT 2
ys_status ys_collider_respond_backward(ys_collider *c, const double *dl_dx, const double *dl_dv, int32_t flags,
                                       double *dl_dx_in, double *dl_dv_in, double *dl_dx_prev, double *dl_dw,
                                       double *dl_dn);

/* ---- learned preconditioner (no counterpart in the reference: its solve is
 * Eigen's Jacobi-PCG, src/Solvers.cpp:3-31, which stays the default and the
 * fallback). A graph network over the crossing graph reads each assembled
 * system and emits a factorised sparse approximate inverse M^-1 = G^T G, G
 * block lower triangular over seven blocks of each node: self, left, down,
 * left-down, right-down, left-2, down-2 (5 x 5 blocks; G_i,0 = (I + N_i,0)
 * L_i^-1, G_i,b = N_i,b L_src^-1, L_i the Cholesky factor of node i's
 * diagonal block). The conjugate-gradient iteration keeps FP64 and the same
 * stopping rule |r| <= tol |b|; M^-1 is applied in FP32 with the flexible
 * (Polak-Ribiere) direction update. */
typedef struct ys_gnn ys_gnn;
enum { YS_PREC_JACOBI = 0, YS_PREC_LEARNED = 1 };
/* training objectives: the Kaporin number of G A G^T (stochastic trace), or
 * the distance of N to the blocks of the exact FSAI of the pattern (its
 * minimiser), computed per node from the assembled system (the default) */
enum { YS_GNN_KAPORIN = 0, YS_GNN_FSAI = 1 };
/* number of FP32 parameters (packed: W0 [64][128], b0 [64], 3 x (W [64][320],
 * b [64]), Wh [outputs][64], bh [outputs]) */
int32_t ys_gnn_param_count(void);
/* network outputs per node and blocks of G per node */
void ys_gnn_dims(int32_t *outputs, int32_t *blocks);
ys_status ys_gnn_set_objective(ys_gnn *g, int32_t objective);
/* a network with seeded initial weights (output head zero: the analytic
 * first-order approximate inverse G = (I - E_lower) L^-1) */
ys_status ys_gnn_create(int32_t device, uint64_t seed, ys_gnn **out);
void ys_gnn_destroy(ys_gnn *g);
ys_status ys_gnn_get_params(ys_gnn *g, float *out);
/* also resets the optimiser state */
ys_status ys_gnn_set_params(ys_gnn *g, const float *in);
/* One Adam step (rate lr) on the network's objective over the systems the
 * batch assembled last (its ys_assemble or ys_step); *loss receives the loss
 * before the step. YS_GNN_KAPORIN: loss = log(tr(G A G^T) / n) - (2 / n)
 * log |det G| (n DOFs; the trace from Rademacher probes drawn from seed, the
 * determinant exact). YS_GNN_FSAI: loss = mean over nodes of |N - N*|_F^2,
 * N* the exact FSAI's blocks in the network's parametrisation. */
ys_status ys_gnn_train_step(ys_gnn *g, ys_batch *b, uint64_t seed, float lr, double *loss);
/* Loss and gradient without an update (probes [total_nodes][5] host, or NULL
 * for seeded probes; Kaporin objective only); outputs [total_nodes][outputs]
 * network outputs, gblocks [total_nodes][25 blocks] blocks of G in pattern
 * order (row-major 5 x 5); any output may be NULL. */
ys_status ys_gnn_loss_grad(ys_gnn *g, ys_batch *b, const float *probes, uint64_t seed, double *loss, float *grad,
                           float *outputs, float *gblocks);
/* kind YS_PREC_JACOBI (default) or YS_PREC_LEARNED with network g; the batch
 * borrows g, which must outlive its use. With ys_use_graphs a learned step is
 * one graph launch (the network evaluated inside it when due). */
ys_status ys_set_preconditioner(ys_batch *b, int32_t kind, ys_gnn *g);
/* evaluate the network once per `every` learned solves (default 1) and reuse
 * G in between: a G from an earlier step is still a symmetric positive
 * definite preconditioner, only a less fitted one */
ys_status ys_precond_refresh(ys_batch *b, int32_t every);
/* learned solves so far and how many fell back to Jacobi-PCG */
ys_status ys_precond_info(ys_batch *b, int64_t *solves, int64_t *fallbacks);
/* the last assembled system's raw coefficient slots [159][total_nodes] and
 * right-hand side [5][total_nodes] (host; either may be NULL) */
ys_status ys_get_system_slots(ys_batch *b, double *slots, double *rhs);
/* C [M][N] = A [M][K] B [N][K]^T on the tensor cores (BF16 bits in, FP32
 * out; N a multiple of 64, K of 64): a self-test of the network's GEMM. */
ys_status ys_tc_gemm_bf16(int32_t device, const uint16_t *A, const uint16_t *B, float *C, int32_t M, int32_t N,
                          int32_t K);

#ifdef __cplusplus
}
#endif
#endif
