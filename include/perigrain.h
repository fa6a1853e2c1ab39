/*
 * perigrain.h -- C ABI of the GB300 (sm_103a) PeriDEM time-integration engine.
 *
 * This replaces the in-process boundary of the reference simulator,
 *   template<unsigned dim> void run_timeloop(vector<ParticleN<dim>>& PArr, Timeloop TL,
 *                                            Contact CN, RectWall<dim> Wall)
 * (reference src/particle/timeloop.h:501-502), and the setup/config/output plumbing around it
 * (src/read/load_hdf5.h:42-201, src/read/read_config.h:122-297, timeloop.h:881-1014).
 *
 * Conventions
 *   - Plain C types only; every function returns a pg_status (PG_OK == 0). No exceptions cross
 *     the ABI. pg_last_error() gives a message for the last failing call on this thread.
 *   - Host arrays are in the reference's node order: grain-major (grain g owns global nodes
 *     [grain_node_offset[g], grain_node_offset[g+1])), nodes in the order of `Pos` in all.h5,
 *     vectors row-major (node, component) with `dim` components.
 *   - A handle holds one or more independent simulations ("instances"); grains of one instance
 *     are contiguous. Grains interact only with grains of the same instance. simulate2d/3d
 *     use one instance; the batched ensemble uses hundreds.
 *   - One handle = one CUDA stream on the current device; calls on one handle must come from
 *     one host thread at a time.
 */
#ifndef PERIGRAIN_H
#define PERIGRAIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pg_status {
  PG_OK = 0,
  PG_EINVAL = 1,     /* bad argument or inconsistent setup */
  PG_ENOMEM = 2,     /* device or pinned-host allocation failed */
  PG_ECUDA = 3,      /* a CUDA runtime call failed */
  PG_ENAN = 4,       /* a non-finite position/velocity was detected */
  PG_ETIMEOUT = 5,   /* a bounded device-side wait gave up */
  PG_EIO = 6,        /* file missing, unreadable or malformed */
  PG_ECAPACITY = 7,  /* a fixed-capacity device table overflowed (see pg_last_error) */
  PG_ERANGE = 8,     /* a node left the coordinate range the contact grid can resolve */
  PG_ENODEV = 9      /* no CUDA device / CUDA extension unavailable */
} pg_status;

typedef enum pg_precision {
  PG_FP64 = 0,  /* reference arithmetic: FP64 everywhere, same operation order (parity path) */
  PG_MIXED = 1  /* FP32 bond/contact forces and accumulation; FP64 disp/vel/pos and xi_norm */
} pg_precision;

typedef struct pg_handle pg_handle;

/* Setup of all grains of all instances (the content of data/hdf5/all.h5 for every instance).
 * Reference: ParticleN<dim> (src/particle/particle2.h:29-86), Contact (src/particle/contact.h:43-112),
 * RectWall<dim> (contact.h:114-305), loaded by load_particles/load_contact/load_wall
 * (src/read/load_hdf5.h:42-201). */
typedef struct pg_setup_desc {
  uint32_t dim;          /* 2 or 3 */
  uint32_t n_instances;  /* >= 1 */
  uint32_t n_grains;     /* total over instances */
  uint32_t n_nodes;      /* total over grains */
  const uint32_t* grain_instance;    /* [n_grains] non-decreasing instance id */
  const uint32_t* grain_node_offset; /* [n_grains+1] */
  /* per node, reference order */
  const double* pos;       /* [n_nodes*dim] Pos */
  const double* vol;       /* [n_nodes]     Vol */
  const double* disp;      /* [n_nodes*dim] */
  const double* vel;       /* [n_nodes*dim] */
  const double* acc;       /* [n_nodes*dim] */
  const double* extforce;  /* [n_nodes*dim] */
  /* bonds: CSR over global node index; row i lists the grain-local indices of i's neighbours
   * in NbdArr order (conn2NArr, src/read/load_hdf5.h:28-38). Every bond appears in both rows. */
  const uint64_t* bond_offset; /* [n_nodes+1] */
  const uint32_t* bond_local;  /* [bond_offset[n_nodes]] grain-local neighbour index */
  /* per grain node lists (grain-local indices), CSR over grains */
  const uint32_t* bdry_offset;    /* [n_grains+1] nonlocal boundary nodes (bdry_nodes) */
  const uint32_t* bdry_nodes;
  const uint32_t* clamped_offset; /* [n_grains+1] clamped_nodes */
  const uint32_t* clamped_nodes;
  /* per grain scalars */
  const double* delta;
  const double* rho;
  const double* cnot;
  const double* snot;
  const int32_t* movable;
  const int32_t* breakable;
  const int32_t* stoppable;
  const uint8_t* break_bonds;   /* ParticleN::break_bonds (simulate2d sets 1 for all) */
  const uint32_t* torque_axis;  /* may be NULL when torque is disabled */
  const double* torque_val;     /* may be NULL when torque is disabled */
  /* per instance contact parameters (pairwise/ in all.h5, after config overrides) */
  const double* contact_radius;
  const double* normal_stiffness;
  const double* friction_coefficient;
  const double* damping_ratio;
  /* per instance wall: allow flag, geometry and side speeds in RectWall::lrtb() order:
   * 2D [left, right, top, bottom], 3D [x_min, y_min, z_min, x_max, y_max, z_max]. */
  const int32_t* allow_wall;  /* [n_instances] */
  const double* wall_geom;    /* [n_instances * 2*dim] */
  const double* wall_speed;   /* [n_instances * 2*dim] */
} pg_setup_desc;

/* Run options (Timeloop + Contact flags, src/particle/timeloop.h:62-202, contact.h:85-108). */
typedef struct pg_config {
  double dt;
  int32_t enable_fracture;
  int32_t nl_bdry_only;
  int32_t allow_damping;
  int32_t allow_friction;
  int32_t self_contact;
  int32_t enable_torque;
  int32_t gradient_extforce;
  uint32_t extforce_maxstep;
  int32_t precision;       /* pg_precision */
  int32_t record_pairs;    /* 1: keep a per-step log of (count, hash) of contact pairs */
  uint32_t pair_log_capacity; /* steps kept in the pair log ring (default 1024 when 0) */
  uint32_t first_step;     /* t of the first step taken (1, or resume_ind*modulo + 1) */
  uint32_t max_contacts;   /* per-node contact candidate capacity (default 48 when 0) */
  uint32_t block_size;     /* threads per block of the fused force kernel (0: default 128) */
  int32_t autotune;        /* 1: pick block_size, cells_per_node and contact_skin by timing trial runs */
  uint32_t cells_per_node; /* contact-grid capacity per node (0: 4 in 2D, 8 in 3D) */
  double contact_skin;     /* > 0: keep per-node contact candidate lists built with radius
                              R_c (1 + contact_skin), rebuilt when a node has moved more than
                              0.45 contact_skin R_c since the last build (results are unchanged);
                              0: search the contact grid every step. Default 0.25; autotune
                              also picks it */
  int32_t timeloop;        /* 0: run_timeloop (timeloop.h:501-1015); 1: run_timeloop_worm
                              (timeloop.h:1018-1369): gait clamps of local nodes 0-3, external
                              force in the first of three 1000-step phases only, contact and walls
                              for every movable grain (no stoppable gate), no torque or ramp */
  int32_t node_order;      /* device layout of the nodes inside each grain (pg_node_order); results
                              do not depend on it: the reference's orders -- bond rows, contact
                              candidates, wall reactions, sums over a grain -- are kept through the
                              nodes' original indices, and every output is in the input's order */
} pg_config;

/* Node layout inside each grain on the device. */
typedef enum pg_node_order {
  PG_ORDER_INPUT = 0,   /* as given */
  PG_ORDER_CELL = 1,    /* default: cell-sorted -- strips of one node spacing (sqrt / cbrt of the
                           mean node volume) along y (2D) or z then y (3D), x ascending within a
                           strip, so that consecutive nodes (a warp's 32) are neighbours in space
                           whatever order the mesh generator wrote them in. A grain whose input
                           order is about as local already (mean index distance of bonded nodes
                           at most 1.5x the cell order's) keeps its input order */
  PG_ORDER_CELL_DEGREE = 2, /* the cell order's choice, then a stable sort by bond count (most
                           bonds first), so warp chunks of the bond slab hold nodes of equal degree
                           (less padding, less coalesced neighbour gathers: the autotuner decides) */
  PG_ORDER_SHUFFLE = 3, /* a seeded random order (tests of the order independence) */
  PG_ORDER_CELL_BLOCK_DEGREE = 4 /* the cell order's choice, then a stable sort by bond count (most
                           bonds first) inside consecutive windows of 256 nodes of each grain: warp
                           chunks of nearly equal degree while every node stays within 256 places
                           of its cell-order position (the autotuner decides) */
} pg_node_order;

/* ---- lifecycle ---------------------------------------------------------------------------- */
int pg_version(void);
int pg_device_count(int* count);
const char* pg_status_string(int status);
const char* pg_last_error(void);
void pg_config_default(pg_config* cfg);

/* Make `device` the current CUDA device of the calling thread for subsequent pg_create calls
 * (one process per GPU under torchrun: device = LOCAL_RANK). */
int pg_select_device(int device);
/* Copy the setup to the current CUDA device and build the device layout. */
int pg_create(const pg_setup_desc* setup, const pg_config* cfg, pg_handle** out);
int pg_destroy(pg_handle* h);

/* ---- stepping (timeloop.h:608-879: position update, force loop, velocity update, wall move) */
int pg_step(pg_handle* h, uint32_t nsteps);
int pg_synchronize(pg_handle* h);
/* pg_step bracketed by CUDA events on the handle's stream; *elapsed_ms = device time of the
 * nsteps steps (synchronizes). */
int pg_step_timed(pg_handle* h, uint32_t nsteps, double* elapsed_ms);
/* Index t of the next step to be taken. */
int pg_get_step(pg_handle* h, uint64_t* next_t);

/* ---- state access (host buffers, reference node order) ------------------------------------ */
typedef enum pg_field {
  PG_FIELD_CURRPOS = 0,  /* CurrPos after the last step's position update */
  PG_FIELD_VEL = 1,
  PG_FIELD_ACC = 2,
  PG_FIELD_FORCE = 3,    /* force density of the last step (what tc_*.h5 stores as force) */
  PG_FIELD_DISP = 4,
  PG_FIELD_POS = 5
} pg_field;
/* out: [n_nodes*dim] doubles. Synchronizes the handle's stream. */
int pg_get_field(pg_handle* h, int field, double* out);
/* Overwrite a field (PG_FIELD_DISP/VEL/ACC/POS) -- used by resume and by the
 * reset_partzero_y hook (timeloop.h:629-650). Writing POS keeps the bond reference vectors
 * xi (computed from the positions given at creation) unchanged, as the reference does. */
int pg_set_field(pg_handle* h, int field, const double* in);
/* alive[b] = 1 if bond b (CSR order given at creation) is intact. */
int pg_get_bond_alive(pg_handle* h, uint8_t* alive);
/* Step at which each bond broke (0 = intact), CSR order. */
int pg_get_bond_break_step(pg_handle* h, uint32_t* step);
/* Replace the alive set (resume with enable_fracture: Connectivity reloaded, timeloop.h:530-536). */
int pg_set_bond_alive(pg_handle* h, const uint8_t* alive);
/* Wall reactions of the last step: [n_instances * 2*dim * dim], RectWall::get_reaction() order. */
int pg_get_reaction(pg_handle* h, double* out);
/* Current wall geometry [n_instances * 2*dim] (lrtb order) and override it. */
int pg_get_wall(pg_handle* h, double* out);
int pg_set_wall(pg_handle* h, const double* geom);
/* Grain flags (set_movable_index / set_stoppable_index hooks, timeloop.h:612-627). */
int pg_set_grain_flags(pg_handle* h, uint32_t grain, int32_t movable, int32_t stoppable);

/* ---- asynchronous snapshots (the output step of run_timeloop, timeloop.h:881-1006) --------- */
/* pg_snapshot enqueues, on the handle's stream behind the steps already issued, a copy of the
 * state the tc_/wall_ files hold into device staging, and the copies from there into the
 * caller's buffers on a second stream, so they overlap the steps issued after it. It does not
 * block. pg_wait blocks until those copies are done, fills the items below and returns the
 * device status word read at the snapshot, as pg_synchronize does. One snapshot is in flight
 * per handle: pg_snapshot first completes one that has not been waited for. A null pointer
 * skips its item. Buffers stay owned by the caller and must stay valid until pg_wait returns;
 * page-locked buffers (pg_host_alloc, cudaHostAlloc) receive the copies directly, other memory
 * through a page-locked bounce buffer that pg_wait copies out. Each item equals what the
 * synchronous getter returns after the same steps. */
typedef struct pg_snapshot_desc {
  double* currpos;            /* [n_nodes*dim], as pg_get_field(PG_FIELD_CURRPOS) */
  double* vel;                /* [n_nodes*dim] */
  double* acc;                /* [n_nodes*dim] */
  double* force;              /* [n_nodes*dim], force density */
  double* disp;               /* [n_nodes*dim] */
  uint8_t* bond_alive;        /* [n_bonds], as pg_get_bond_alive */
  double* wall;               /* [n_instances*2*dim], as pg_get_wall */
  double* reaction;           /* [n_instances*2*dim*dim], as pg_get_reaction */
  uint64_t* too_close_events; /* as pg_get_device_status */
  uint64_t* last_step;        /* index of the last step taken before the snapshot */
} pg_snapshot_desc;
int pg_snapshot(pg_handle* h, const pg_snapshot_desc* d);
int pg_wait(pg_handle* h);
/* Page-locked host memory (for snapshot buffers); pg_host_free releases it. */
int pg_host_alloc(size_t bytes, void** out);
int pg_host_free(void* p);

/* ---- diagnostics ---------------------------------------------------------------------------- */
/* Per-step contact-pair log (needs cfg.record_pairs): for the last `n` steps ending at the
 * last completed step, count[k] = number of node pairs that passed the contact test
 * (|x_q - x_p| <= R_c') and hash[k] = wrapping sum of splitmix64((gid_p << 32) | gid_q). */
int pg_get_pair_log(pg_handle* h, uint32_t n, uint64_t* count, uint64_t* hash);
/* Sticky device error word (PG_ECAPACITY/PG_ERANGE/...), 0 if none; also "nodes too close"
 * events (dir_norm == 0 in contact.h:737) counted since creation. */
int pg_get_device_status(pg_handle* h, int32_t* status, uint64_t* too_close_events);
/* Test hook for the failure path of the bounded device waits: presets the arrival count of the
 * cooperative grid build's barrier, so that its next wait cannot complete; the blocks give up
 * after the poll limit (~0.3 s) and the step's status becomes PG_ETIMEOUT. A handle that timed
 * out is halted: grid builds already enqueued return at entry (the barrier's arrival count is
 * stale), and once a status check (pg_synchronize, pg_step_timed, pg_wait, pg_get_device_status)
 * has reported PG_ETIMEOUT, pg_step returns PG_ETIMEOUT without launching (create a new handle).
 * PG_EINVAL without candidate lists or cooperative launch. */
int pg_debug_grid_barrier(pg_handle* h, uint32_t arrivals);
/* Test hook for the FP64 path's integer arithmetic (correctly rounded division, square root,
 * addition, subtraction, multiplication and FP32 -> FP64 conversion on the integer pipe): for host
 * arrays of n doubles (0 <= n <= 2^26) computes out[i] = a[i] / b[i] (op PG_IEEE_DIV),
 * sqrt(|a[i]|) (PG_IEEE_SQRT), a[i] + b[i] (PG_IEEE_ADD), a[i] - b[i] (PG_IEEE_SUB), a[i] * b[i]
 * (PG_IEEE_MUL) or (double)(float)a[i] (PG_IEEE_WIDEN) on the current device with the routines
 * the kernels use, for comparison with IEEE results. PG_EINVAL for another op. */
enum pg_ieee_op { PG_IEEE_DIV = 0, PG_IEEE_SQRT = 1, PG_IEEE_ADD = 2, PG_IEEE_SUB = 3, PG_IEEE_MUL = 4, PG_IEEE_WIDEN = 5 };
int pg_debug_ieee64(int32_t op, const double* a, const double* b, int64_t n, double* out);
/* Launch configuration in use (after autotuning): force-kernel block size, grid cells per node. */
int pg_get_launch_config(pg_handle* h, uint32_t* block_size, uint32_t* cells_per_node);
/* Contact candidate-list skin in use (fraction of R_c; 0: grid search every step). */
int pg_get_contact_skin(pg_handle* h, double* skin);
/* Node layout in use: the pg_node_order asked for (after autotuning), and whether it differs from
 * the input's order (0: the input already was in that order, or PG_ORDER_INPUT). */
int pg_get_node_order(pg_handle* h, int32_t* order, int32_t* permuted);
/* Test hook of the node layout, on the host only (no device needed): validates the setup as
 * pg_create does without a device (bond rows included) and fills perm[i] = the input index of
 * device node i (n_nodes entries) for the pg_node_order `order`, and *permuted = 0 when that is the
 * input order itself. */
int pg_debug_node_order(const pg_setup_desc* s, int32_t order, uint32_t* perm, int32_t* permuted);
/* Number of kernel launches issued by the last pg_step call. */
int pg_get_launch_count(pg_handle* h, uint64_t* launches);
/* Per-kernel device time of the last pg_step call (CUDA events; needs timing enabled). */
int pg_set_timing(pg_handle* h, int32_t enable);
int pg_get_kernel_times(pg_handle* h, double* force_ms, double* total_ms, uint64_t* force_launches);

/* ---- post-processing on the device ---------------------------------------------------------- */
/* The quantities the reference's post-processing scripts compute from the tc_/wall_ files
 * (read_sim_output.py:126-133, :183-232, :305-312; gen_damage_data.py; gen_timestep_data.py),
 * computed from the current state on the device; only the aggregates are copied out. Every
 * pointer may be NULL (not computed). Grain means are over the grain's nodes (numpy `mean(axis=0)`);
 * damage of a node is (deg0 - deg) / deg0 with deg the intact bonds now and deg0 at creation. */
typedef struct pg_post {
  double* grain_mean_vel;     /* [n_grains*dim] particle_mean_vel */
  double* grain_mean_acc;     /* [n_grains*dim] particle_mean_acc */
  double* grain_mean_currpos; /* [n_grains*dim] particle_mean_CurrPos */
  double* grain_force;        /* [n_grains*dim] particle_force: sum of the force density */
  double* grain_damage;       /* [n_grains] mean node damage of the grain */
  double* node_damage;        /* [n_nodes] node damage (the `damage` plot quantity) */
  double* inertial_force;     /* [n_instances*dim] sum of vol * rho * acc (read_force_val f_sum) */
  double* volume_fraction;    /* [n_instances] grain volume / wall box volume (extract_bulk) */
} pg_post;
int pg_postprocess(pg_handle* h, const pg_post* out);

/* ---- gradients ------------------------------------------------------------------------------ */
/* The reference has no gradient path; these entry points differentiate its time step
 * (timeloop.h:608-879, the run_timeloop body) with respect to per-grain parameters.
 *
 * Parameters per grain g, in this order (PG_NPARAM): cnot (bond stiffness, particle2.h:140; it
 * also sets the self-contact stiffness cnot/R_c', contact.h:709-730), normal contact stiffness,
 * damping ratio, friction coefficient. Two grains in contact use the mean of their values; with
 * equal values this is the reference's global Contact parameters (contact.h:43-112), and grain g
 * meets a wall with its own values. The gradient is that of the run with its masks frozen: bond
 * breaks, contact pairs, friction branches (sliding or sticking) and wall contacts stay as the
 * forward pass decided them. Torque (enable_torque) is not differentiated: PG_EINVAL. Every
 * movable grain must be stoppable (the adjoint gathers each contact pair at both nodes).
 *
 * Usage: pg_grad_begin marks the current state as the origin; pg_grad_forward runs n_steps from
 * the origin keeping a checkpoint of the state every checkpoint_every steps; the caller reads the
 * objectives (pg_get_field, pg_get_reaction); pg_grad_backward recomputes each segment from its
 * checkpoint (recording the masks) and runs the reverse steps, leaving the handle at the final
 * state again. Memory: one checkpoint per segment plus one segment of tape. */
#define PG_NPARAM 4
/* Per-grain parameters; any pointer may be NULL (left unchanged). Setting kn, zeta or mu makes
 * the force kernels use the per-grain contact parameters. snot (critical stretch) has no
 * gradient (bond breaks are frozen) but is settable so cnot and snot can follow one modulus. */
int pg_set_grain_params(pg_handle* h, const double* cnot, const double* snot, const double* kn,
                        const double* zeta, const double* mu);
int pg_get_grain_params(pg_handle* h, double* cnot, double* snot, double* kn, double* zeta, double* mu);
/* Mark the current state as the origin of differentiable runs. */
int pg_grad_begin(pg_handle* h);
/* Restore the origin state. */
int pg_grad_reset(pg_handle* h);
/* Masks of a run recorded once and replayed by frozen forwards (finite-difference checks and
 * FP64 reference gradients). */
typedef struct pg_masks pg_masks;
/* From the origin, run n_steps with the handle's own precision, recording the masks of every
 * step (contact entries, wall bits, bond breaks). Leaves the handle at the end of the run. */
int pg_masks_record(pg_handle* h, uint32_t n_steps, pg_masks** out);
void pg_masks_free(pg_masks* m);
/* From the origin, run n_steps keeping a checkpoint every checkpoint_every steps. frozen = NULL:
 * the handle's own step (FP64 or mixed precision); otherwise an FP64 step that replays the
 * masks of `frozen` (recorded from this origin, n_steps <= its length) instead of deciding
 * them. */
int pg_grad_forward(pg_handle* h, uint32_t n_steps, uint32_t checkpoint_every, const pg_masks* frozen);
/* Cotangents of the last forward's final state -- disp_bar, vel_bar [n_nodes*dim] (NULL = 0) and
 * of its last step's wall reactions reaction_bar [n_instances*2*dim*dim] (NULL = 0) -- to
 * grad[n_grains*PG_NPARAM], the gradient with respect to the per-grain parameters. */
int pg_grad_backward(pg_handle* h, const double* disp_bar, const double* vel_bar, const double* reaction_bar,
                     double* grad);
/* Device time of the last pg_grad_forward / pg_grad_backward (CUDA events) and their kernel
 * launch counts. */
int pg_grad_times(pg_handle* h, double* forward_ms, double* backward_ms, uint64_t* forward_launches,
                  uint64_t* backward_launches);

/* ---- setup helpers -------------------------------------------------------------------------- */
/* Bond list of one grain on the GPU: every node pair (i, j), i < j, with
 * sqrt(sum_c (p_j[c] - p_i[c])^2) <= delta, rows in lexicographic order -- the Connectivity the
 * reference's setup writes (exp_dict.py:171-222: itertools.combinations + single_bond, which
 * compares the same FP64 distance). pos: device pointer, n x dim doubles; pairs: device pointer,
 * capacity x 2 uint32. *n_pairs receives the number of pairs (also when it exceeds capacity, then
 * PG_ECAPACITY and the first `capacity` rows are written). Temporary device memory is allocated
 * and freed inside the call. Runs on `stream` (a cudaStream_t, NULL for the default stream) and
 * returns after it completes. pg_bond_last_error() describes a failure. */
int pg_build_bonds(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs,
                   uint64_t capacity, uint64_t* n_pairs, void* stream);
const char* pg_bond_last_error(void);

/* pg_build_bonds without any device allocation, for callers that cannot allocate device memory:
 * allocator or memory-pool hooks (a cudaMalloc there would re-enter the allocator they implement)
 * and hosts that reserve all device memory up front or run under a hard device-memory quota. This
 * entry point has no counterpart in the reference. Same arguments and results as pg_build_bonds;
 * its scratch is a file-scope device array sized for one grain of at most PG_NOALLOC_MAX_NODES
 * nodes (about 1.7 MB, held by every GPU that loads the library until exit); larger n returns
 * PG_EINVAL. Calls share that array, so calls that overlap on the GPU race; each call clears what
 * it needs. The first call on a device looks the array's device address up and caches it for the
 * CUDA context (make that first call before any stream capture; do not call it again on a device
 * after cudaDeviceReset). It returns after `stream` completes. pg_noalloc_last_error() describes
 * a failure. */
#define PG_NOALLOC_MAX_NODES 32768u
int pg_build_bonds_noalloc(const double* pos, uint32_t n, uint32_t dim, double delta, uint32_t* pairs,
                           uint64_t capacity, uint64_t* n_pairs, void* stream);
const char* pg_noalloc_last_error(void);

/* Incircle packing of a simplex mesh: the grain centres and radii the reference's packing
 * generator computes from its mesh (exp_dict.py:1072-1313 get_incenter_mesh_loc; the mesher,
 * gmsh, is the caller's). All arrays are device pointers. */
typedef struct pg_pack_mesh {
  uint32_t dim;               /* 2: triangles, 3: tetrahedra */
  uint32_t n_nodes;
  uint32_t n_elems;
  const double* pos;          /* [n_nodes][dim] */
  const uint32_t* elems;      /* [n_elems][dim + 1] node indices */
  uint32_t n_bdry_nodes;
  const uint32_t* bdry_nodes; /* [n_bdry_nodes] */
  uint32_t n_bdry_edges;      /* 2D boundary segments (used by the maximin pass with gen_bdry) */
  const uint32_t* bdry_edges; /* [n_bdry_edges][2] */
} pg_pack_mesh;

/* Writes the incircle (insphere) of every element -- centres[e], radii[e] for e < n_elems --
 * followed by one circle per mesh node in node order (exp_dict.py:1186-1296):
 *   modify_nodal_circles == 0: interior nodes; centre = the node, radius = min over the node's
 *     elements of |incenter - node| - inradius (2D and 3D);
 *   modify_nodal_circles != 0 (2D only): interior nodes, plus boundary nodes when gen_bdry; the
 *     solution of the reference's per-node maximin problem (the largest circle clear of the
 *     surrounding incircles and, for boundary nodes, of the lines of their boundary edges,
 *     centred in the box of those incircles' centres), reached from the reference's initial guess.
 * centers: [n_elems + n_nodes][dim] doubles, radii: [n_elems + n_nodes]; *n_out receives the number
 * of circles written. *n_unpolished (may be NULL) counts maximin nodes whose exact solve found no
 * tight point (their circle is the ascent's end point). Temporary device memory is allocated and
 * freed inside the call; runs on `stream` and returns after it completes.
 * pg_pack_last_error() describes a failure. */
int pg_pack_incenters(const pg_pack_mesh* mesh, int32_t modify_nodal_circles, int32_t gen_bdry, double* centers,
                      double* radii, uint32_t* n_out, uint32_t* n_unpolished, void* stream);
const char* pg_pack_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PERIGRAIN_H */
