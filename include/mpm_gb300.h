/*
 * mpm_gb300 -- GB300-native (sm_103a) explicit USL step of mpm-2d behind a C
 * ABI.  Plain pointers and sizes only; every entry point returns an int
 * status (MPMG_OK on success) and never exits the process.
 *
 * This is the flat interface the libmpm-compatible entry points of
 * mpm_libmpm.h are built on.  One mpmg_ctx holds one simulation resident in
 * the GPU's memory: particle state in structure-of-arrays form in the
 * caller's original particle order, the background grid, and the scratch the
 * step needs (sort buffers, per-element partial sums, solver vectors).
 *
 * Reference interfaces each call replaces (paths inside neocpp89/mpm-2d):
 *   mpmg_create      mpm_init (libmpm/process_usl.c:68-280) + material_init
 *                    (the material plugins) + bc_validate (the BC plugins), with the
 *                    driver's dt (src/main.c:742)
 *   mpmg_step        the driver loop body (src/main.c:946-977):
 *                    explicit_mpm_step_usl_threaded (process_usl.c:465-592)
 *                    followed by time_varying_loads (loading.c:34-54)
 *   mpmg_get_field   reads of job->particles[] / job->nodes[] (process.h:116-213)
 *   mpmg_destroy     mpm_cleanup (process_usl.c:974-1004)
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stddef.h>
#include <stdio.h>

#if defined(__GNUC__)
#define MPMG_API __attribute__((visibility("default")))
#else
#define MPMG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Values 1..3 match libmpm/exitcodes.h's CXSparse codes where
   the meaning carries over (a failed fluidity solve is EXIT_ERROR_CS_SOL). */
enum mpmg_status {
    MPMG_OK = 0,
    MPMG_ERR_SOLVER = 2,          /* fluidity solve did not converge (EXIT_ERROR_CS_SOL) */
    MPMG_ERR_INVALID = 16,        /* bad argument or configuration */
    MPMG_ERR_CUDA = 17,           /* CUDA runtime error (no GPU, launch failure, ...) */
    MPMG_ERR_NOMEM = 18,          /* device allocation failed */
    MPMG_ERR_UNKNOWN_FIELD = 19,
    MPMG_ERR_UNSUPPORTED = 20,    /* material or boundary condition not implemented */
    MPMG_ERR_DEVICE = 21,         /* a kernel reported an internal error (status word) */
    MPMG_ERR_SCRATCH_LIMIT = 22   /* size exceeds a fixed scratch capacity */
};

/* Material kinds: the reference plugins with a device implementation. */
enum mpmg_material {
    MPMG_ISOLIN = 0,              /* materialsrc/isolin.c */
    MPMG_G_LOCAL_MU2 = 1,         /* materialsrc/g_local_mu2.c */
    MPMG_G_NONLOCAL_MU2 = 2,      /* materialsrc/g_nonlocal_mu2.c */
    MPMG_G_NONLOCAL = 3,          /* materialsrc/g_nonlocal.c */
    MPMG_DP_RI_MT = 4,            /* materialsrc/dp_ri_mt.c */
    MPMG_G_LOCAL_MU2_PLANE_STRAIN = 5,  /* materialsrc/g_local_mu2_plane_strain.c */
    MPMG_G_LOCAL_MU2_TRUE_2D = 6,       /* materialsrc/g_local_mu2_true_2d.c */
    MPMG_G_LOCAL_MU2_EXT = 7,           /* materialsrc/g_local_mu2_ext.c */
    MPMG_G_NONLOCAL_AVG = 8,            /* materialsrc/g_nonlocal_avg.c (and g_nonlocal_bicgstab.c, the same
                                           code): g_nonlocal with the element average of the nodal
                                           fluidity at the particles */
    MPMG_G_LOCAL_MU2_REVERSE = 9        /* materialsrc/g_local_mu2_reverse.c */
};

/* Boundary-condition kinds: the reference plugins with a device implementation. */
enum mpmg_bc {
    MPMG_BOX = 0,                 /* bcsrc/box.c */
    MPMG_SQUARE_SILO = 1          /* bcsrc/square_silo.c */
};

enum mpmg_gravity {
    MPMG_GRAVITY_REFERENCE_RAMP = 0,  /* loading.c: 0 on step 1, then -9.8 t/0.1 up to -9.8 */
    MPMG_GRAVITY_CONSTANT = 1         /* mpmg_config.gravity from step 1 on */
};

/* Arithmetic of the step.  MPMG_PRECISION_FP64 is the reference's (FP64
   everywhere).  MPMG_PRECISION_MIXED keeps particle state, shape functions,
   P2G and G2P contributions and the material update in FP32, and sums nodal
   mass and momentum, updates the momentum and divides by nodal mass in
   float-float arithmetic (an unevaluated sum of two FP32 values: 48
   significant bits, on the FP32 pipe); MPMG_PRECISION_MIXED_F64NODE does
   those nodal sums and the division in FP64 instead (GB300 runs FP64 at 1/64
   of the FP32 rate, so this form's grid update is several times slower).
   Both mixed forms keep particles in element order on the device (read-back
   returns the caller's order) and support isolin, g_local_mu2 and
   g_nonlocal_mu2 (whose material law evaluates in FP64 from the FP32 state,
   and whose fluidity solve stays FP64). */
enum mpmg_precision {
    MPMG_PRECISION_FP64 = 0,
    MPMG_PRECISION_MIXED = 1,
    MPMG_PRECISION_MIXED_F64NODE = 2
};

/* Step scheme.  MPMG_SCHEME_USL is explicit_mpm_step_usl_threaded
   (process_usl.c:465-592).  MPMG_SCHEME_MUSL is
   explicit_mpm_step_musl_threaded (process_usl.c:284-462): after the particles
   move, their updated momentum is mapped to the nodes again with the
   start-of-step shape functions, and the strain rate uses the nodal
   velocities of that second projection (the reference applies its momentum
   boundary conditions only after those velocities are formed, and so does
   this library).  MUSL runs in the FP64 form, for isolin and g_local_mu2. */
enum mpmg_scheme {
    MPMG_SCHEME_USL = 0,
    MPMG_SCHEME_MUSL = 1
};

/* Preconditioner of the fluidity solve (g_nonlocal_mu2, g_nonlocal and
   g_nonlocal_avg).  The reference factorises the assembled matrix
   (g_nonlocal_mu2.c:510-519); this library solves the same system by
   conjugate gradients to mpmg_config.solver_tol.
   MPMG_PRECOND_MULTIGRID: one geometric-multigrid V-cycle on the node lattice
   per iteration (Galerkin coarse operators, FP32 cycle, FP64 outer
   iteration).  It takes 5 to 10 iterations where Jacobi takes hundreds.  It
   is used where a block's share of the grid fits the kernel (up to about
   280 000 nodes on a GB300); larger grids fall back to Jacobi.
   MPMG_PRECOND_JACOBI: diagonal scaling. */
enum mpmg_precond {
    MPMG_PRECOND_MULTIGRID = 0,
    MPMG_PRECOND_JACOBI = 1
};

/* Material parameter slots (mpmg_config.mp).  mpmg_default_params fills the
   reference's compile-time constants for a material kind. */
enum mpmg_mparam {
    MPMG_MP_E = 0, MPMG_MP_NU, MPMG_MP_MU_S, MPMG_MP_MU_2, MPMG_MP_I0,
    MPMG_MP_GRAINS_RHO, MPMG_MP_GRAINS_D, MPMG_MP_A, MPMG_MP_RHO_CRITICAL,
    MPMG_MP_B, MPMG_MP_COHESION,
    MPMG_MP_COUNT = 16
};

typedef struct mpmg_config {
    int Nx, Ny;              /* grid nodes per row and per column (reference: N, N) */
    double h;                /* element edge (reference: len / (N - 1)) */
    double xmax, ymax;       /* element-map inside bounds (reference: 1.0, 1.0) */
    double dt;
    int material;            /* enum mpmg_material */
    double mp[MPMG_MP_COUNT];
    int bc;                  /* enum mpmg_bc */
    double bcf[4];           /* box: x0, y0, width, height; silo: hole radius, open time, wall fraction */
    int bci[4];              /* box: friction bits (1 x, 2 y) for left, bottom, right, top */
    int gravity_mode;        /* enum mpmg_gravity */
    double gravity;          /* constant mode: body force per unit mass along y */
    int store_transients;    /* nonzero: keep x_tt, y_tt, strain rates and nodal
                                momentum/force for read-back (parity tests) */
    double solver_tol;       /* fluidity PCG relative residual (default 1e-10) */
    int solver_maxit;        /* fluidity PCG iteration cap (default 20000) */
    int device;              /* CUDA device ordinal */
    int solver_warm_start;   /* nonzero: start the fluidity PCG from the previous
                                step's nodal fluidity instead of zero (rows that
                                no element touches start at zero either way, as
                                the reference's direct solve gives zero there).
                                Off by default: with it on, a step's result also
                                depends on the previous solve's rounding, so a run
                                restarted from a state file (which carries no
                                solver state) no longer continues bit for bit;
                                on the 835 996-particle silo it saves about 5 % of
                                the iterations. */
    int precision;           /* enum mpmg_precision */
    int scheme;              /* enum mpmg_scheme */
    int solver_precond;      /* enum mpmg_precond (default multigrid) */
} mpmg_config;

typedef struct mpmg_ctx mpmg_ctx;

/* Fills mp[MPMG_MP_COUNT] with the reference's constants for a material. */
MPMG_API int mpmg_default_params(int material, double *mp);

/* Fills cfg with defaults (reference inside bounds, tolerances, device 0). */
MPMG_API int mpmg_config_init(mpmg_config *cfg);

/*
 * Creates a simulation from host arrays of n particles: mass, volume,
 * position, velocity and in-plane stress, the columns of the reference's
 * particle file (src/reader.c:66-99).  The arrays are copied; the caller keeps
 * them.  On success *out holds the context.
 */
MPMG_API int mpmg_create(const mpmg_config *cfg, size_t n, const double *m, const double *v,
                const double *x, const double *y, const double *vx, const double *vy,
                const double *sxx, const double *sxy, const double *syy, mpmg_ctx **out);
MPMG_API int mpmg_destroy(mpmg_ctx *ctx);

/* Advances nsteps time steps (each: USL step + load update), asynchronously
   on the context's stream.  Errors found on the device are reported by the
   next mpmg_synchronize or read-back. */
MPMG_API int mpmg_step(mpmg_ctx *ctx, int nsteps);
MPMG_API int mpmg_synchronize(mpmg_ctx *ctx);

/* Named host read-back / write of one field (particle fields in the caller's
   particle order, node fields in node-number order).  Particle fields: x y v
   v0 m vx vy ax ay bx by sxx sxy syy ux uy exx exy eyy wxy xl yl Txx Txy Tyx
   Tyy Tzz state0..state10.  Node fields: node_m node_mx node_my node_fx
   node_fy node_vx node_vy node_ax node_ay node_gf. */
MPMG_API int mpmg_get_field(mpmg_ctx *ctx, const char *name, double *host_out);
/* Reads count fields at once, each device array behind them downloaded
   once: a whole output frame, as the driver's write_frame
   (src/writer.c:190-201, called from src/main.c:957) reads the particles'
   m v x y x_t y_t sxx sxy syy ux uy state[9] state[10].  host_out[k]
   receives names[k]. */
MPMG_API int mpmg_get_fields(mpmg_ctx *ctx, int count, const char *const *names, double *const *host_out);

/* The driver's output files.  mpmg_write_frame writes one write_frame block
   (src/writer.c:190-201: a "frame t n" line, then write_particle's row per
   particle, src/writer.c:169-186) to fd, formatted on several host threads
   from one batched device read.  mpmg_write_state writes write_state's file
   (src/writer.c:266-380) with every value in %.17g, so that a restart is
   exact; mpmg_read_state reads such a file (and the reference's own, in
   %lg) into a new context whose grid size, spacing and dt come from the
   file and the rest from base (read_state, src/reader.c:123-243, which also
   fails to allocate job->active; here activity is restored with the
   particles).  Color, the deformation gradient and the CPDI corners are
   written as mpm_init leaves them (0, identity, 0). */
MPMG_API int mpmg_write_frame(mpmg_ctx *ctx, FILE *fd, size_t frame, double t);
/* write_element_frame (src/writer.c:205-263): a header line, then per
   element its four corners and the volume-weighted mean stress (sxx, sxy,
   syy) of its active particles, summed in particle order. */
MPMG_API int mpmg_write_element_frame(mpmg_ctx *ctx, FILE *fd, size_t frame, double t);
MPMG_API int mpmg_write_state(mpmg_ctx *ctx, FILE *fd, double t_stop);
MPMG_API int mpmg_read_state(FILE *fd, const mpmg_config *base, mpmg_ctx **out);
MPMG_API int mpmg_set_field(mpmg_ctx *ctx, const char *name, const double *host_in);

/* Element of each particle (-1 outside) and active flags
   (job->in_element / job->active, process.h:145-146). */
MPMG_API int mpmg_get_map(mpmg_ctx *ctx, int *in_element, int *active);
MPMG_API int mpmg_set_map(mpmg_ctx *ctx, const int *in_element, const int *active);

/* The last step's cell sort: sorted keys (element, or num_elements for
   inactive particles), the permutation (sorted position -> particle index)
   and per-element start offsets (num_elements + 1 entries). */
MPMG_API int mpmg_get_sort(mpmg_ctx *ctx, int *sorted_keys, int *perm, int *cell_start);

/* Online tuning of a mixed-form context's tiles and launch shape (no
   counterpart in the reference).  First the tiles, at the default launch
   shape: a batch's P2G tile (256 elements a block staging 1024 particles a
   pass, 128 staging 512, or 512 staging 1024; a single simulation runs the
   fused P2G and grid update) with the G2P tile (256 or 128 particles).  Then,
   with the fastest tiles, the persistent G2P grid (1 up to as many blocks per
   SM as fit) and the steps per replayed CUDA graph (4, 8, 16).  Every
   candidate runs the simulation itself (a warm-up graph, then steps_per_trial
   steps rounded up to whole graphs, timed with CUDA events) and the fastest
   is kept for later steps.  No knob changes any result: the trajectory is the
   untuned one, advanced by steps_advanced steps. */
typedef struct mpmg_tuning {
    int g2p_blocks_per_sm;
    int graph_steps;
    double ms_per_step;          /* of the configuration kept */
    double default_ms_per_step;  /* of the default (default tiles, all G2P blocks that fit, 8 steps per graph) */
    int candidates;
    int steps_advanced;
    int p2g_elements;            /* batched P2G tile kept: elements a block (0 for a single simulation) */
    int p2g_stage;               /* batched P2G tile kept: particles staged a pass */
    int g2p_tile;                /* G2P tile kept: particles a tile */
} mpmg_tuning;
MPMG_API int mpmg_autotune(mpmg_ctx *ctx, int steps_per_trial, mpmg_tuning *best);

MPMG_API int mpmg_get_time(mpmg_ctx *ctx, double *t, int *step_number);
/* Asynchronous read-back of the step record (time, step count, device
   status) for pipelined drivers: mpmg_record_async enqueues the copy of the
   record as it stands after the work issued so far into ring slot
   0..3; mpmg_record_wait waits for that copy and returns what it holds
   (errors as mpmg_get_time).  A driver can issue step k + 1 before waiting
   for step k's record, so the GPU never idles on the host. */
MPMG_API int mpmg_record_async(mpmg_ctx *ctx, int slot);
MPMG_API int mpmg_record_wait(mpmg_ctx *ctx, int slot, double *t, int *step_number);
/* Per-step records written by the step itself (no counterpart in the
   reference): with slots > 0, every step ends with one small kernel that
   copies the step record (time, step count, solver bookkeeping, device
   status) into slot (step - 1) % slots of a ring in mapped pinned host
   memory, so steps can run in CUDA graphs of many steps and the host still
   reads each step's result.  slots = 0 turns it off.
   mpmg_record_ring_wait waits (bounded, about 10 s) for the record of step
   step_number, checks its device status as mpmg_record_wait does, and
   returns its time and step count; it fails with MPMG_ERR_INVALID when that
   slot already holds a later step, or a later step overwrote it while it
   was being read (read within `slots` steps). */
MPMG_API int mpmg_record_ring(mpmg_ctx *ctx, int slots);
MPMG_API int mpmg_record_ring_wait(mpmg_ctx *ctx, long long step_number, double *t, int *step_out);
/* The ring's read protocol on one slot, host memory only (no CUDA call), as
   mpmg_record_ring_wait uses it: a slot is a 16-byte header whose first
   64-bit word is a sequence lock (-1 while the GPU writes the body, then the
   step number), followed by body_bytes of record.  Waits up to timeout_s
   seconds for the sequence to reach step_number (MPMG_ERR_DEVICE when it
   does not), copies the body into out with `copy` (memcpy when NULL) and
   reads the sequence again: MPMG_ERR_INVALID when it was or became anything
   but step_number, i.e. a later step overwrote the slot before or during the
   copy. */
MPMG_API int mpmg_ring_read_slot(const void *slot, size_t body_bytes, long long step_number, void *out,
                                 double timeout_s, void (*copy)(void *, const void *, size_t));
MPMG_API int mpmg_set_time(mpmg_ctx *ctx, double t, int step_number);
MPMG_API int mpmg_sizes(mpmg_ctx *ctx, size_t *num_particles, size_t *num_nodes, size_t *num_elements);

/* Batched ensembles (no counterpart in the reference, which runs one job per
   process: its plugins keep static state).  count independent simulations
   in one context, each with its own configuration: grid size and spacing,
   material parameters (mu_s, ...), boundary conditions (box or square silo,
   e.g. an outlet-width sweep), time step and gravity.  The members share the
   precision (a mixed form), the material kind (isolin or g_local_mu2) and the
   device.  Member k's counts[k] particles follow member k-1's in the
   particle arrays.  mpmg_step advances every member by nsteps of its own
   dt, all members in the same kernel launches (one CUDA graph per step or
   chunk of steps).  Particle and node fields read back concatenated in
   member order (mpmg_batch_member gives each member's offsets and sizes);
   mpmg_get_map reports elements local to each member; mpmg_get_time and
   mpmg_set_time act on member 0 and on all members. */
MPMG_API int mpmg_batch_create(int count, const mpmg_config *cfgs, const size_t *counts, const double *m,
                               const double *v, const double *x, const double *y, const double *vx,
                               const double *vy, const double *sxx, const double *sxy, const double *syy,
                               mpmg_ctx **out);
MPMG_API int mpmg_batch_count(mpmg_ctx *ctx, int *count);
MPMG_API int mpmg_batch_member(mpmg_ctx *ctx, int member, size_t *first_particle, size_t *num_particles,
                               size_t *first_node, size_t *num_nodes, size_t *first_element,
                               size_t *num_elements);
MPMG_API int mpmg_batch_get_time(mpmg_ctx *ctx, int member, double *t, int *step_number);

/* Reverse-mode adjoint of the FP64 step (no counterpart in the reference).
   mpmg_adj_forward_tape advances nsteps ordinary steps from the current
   state, keeping the particle state every checkpoint_every steps.
   mpmg_adj_backward takes the gradient of a loss with respect to the final
   positions (dl_dx, dl_dy, particle order) and returns in dl_dtheta[4] its
   gradient with respect to the material parameters mu_s, mu_2, I0 (the
   g_local_mu2 constants, mpmg_config.mp) and E; each checkpoint segment is
   run forward again with its steps recorded on the device, then reversed by
   hand-written adjoint kernels of the material update, G2P, grid update and
   P2G.  The context is left at the taped run's final state.  The element of
   each particle and the branches of the material law are held fixed within
   a step.  mpmg_adj_state then reads the adjoint of a field of the run's
   initial state: x y vx vy v sxx sxy syy Tzz.  FP64 form, isolin,
   g_local_mu2 or g_nonlocal_mu2 (its fluidity solve reversed by a solve of
   the same symmetric system for the fluidity's adjoint), one simulation. */
MPMG_API int mpmg_adj_forward_tape(mpmg_ctx *ctx, int nsteps, int checkpoint_every);
MPMG_API int mpmg_adj_backward(mpmg_ctx *ctx, const double *dl_dx, const double *dl_dy, double *dl_dtheta);
MPMG_API int mpmg_adj_state(mpmg_ctx *ctx, const char *name, double *host_out);
/* One parameter's gradient from the last mpmg_adj_backward: index 0 mu_s,
   1 mu_2, 2 I0, 3 E (the four dl_dtheta holds), 4 the nonlocal amplitude A
   of g_nonlocal_mu2 (zero for the local materials). */
MPMG_API int mpmg_adj_gradient(mpmg_ctx *ctx, int index, double *out);

/* Runs only the material update on every active particle from the current
   strain rates (the per-particle path of the reference's tests/test_material.c).
   Local materials only. */
MPMG_API int mpmg_material_only(mpmg_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t) for callers that time or order
   work against it. */
MPMG_API int mpmg_get_stream(mpmg_ctx *ctx, void **stream);

/* Per-phase GPU timing with CUDA events on the context's stream.  When
   enabled, mpmg_step records events around each phase; mpmg_phase_times
   returns accumulated milliseconds and launch counts per phase and resets
   them.  Phase names: see mpmg_phase_name. */
MPMG_API int mpmg_enable_phase_timing(mpmg_ctx *ctx, int enable);
MPMG_API int mpmg_phase_count(void);
MPMG_API const char *mpmg_phase_name(int phase);
MPMG_API int mpmg_phase_times(mpmg_ctx *ctx, double *ms, long *launches);

/* Fluidity solve statistics of the last step (nonlocal materials). */
MPMG_API int mpmg_last_solve(mpmg_ctx *ctx, int *iterations, double *rel_residual);

/* Number of kernel launches issued by the library since the context was
   created (or since the last reset). */
MPMG_API int mpmg_launch_count(mpmg_ctx *ctx, long *launches, int reset);

/* FP64 FMA throughput of the given device in FLOP/s (an FMA counts two),
   measured with a short kernel of independent FMA chains (best of three
   timed launches after one warm-up).  No counterpart in the reference: it
   is the compute bound of the plain FP64 form's kernels, which the
   benchmark reports beside their memory bound. */
MPMG_API int mpmg_measure_fp64_rate(int device, double *flops_per_s);

/*
 * Cell sort without any allocation.  No counterpart in the reference: it
 * gives the same element order as the binning every mpmg_step performs (the
 * GPU form of find_filled_elements, libmpm/process_usl.c:677-723), to callers
 * that cannot call cudaMalloc -- hosts whose device memory belongs to their
 * own pool allocator, and the reference's dlopen'd plugins, which own no
 * device memory.
 *
 * d_keys holds n element keys on the device.  A key in [0, num_elements) is
 * an element; num_elements marks a particle outside the grid, and so does any
 * key outside [0, num_elements] (the reference's -1, for instance): those are
 * clamped to num_elements and sort into the run after the last element.
 * Outputs, also device arrays the caller provides: the keys sorted stably
 * (d_sorted_keys, n, with the clamping applied), the permutation from sorted
 * position to particle index (d_perm, n) and the start of every element's
 * run (d_cell_start, num_elements + 1; entry num_elements is where the
 * outside run starts).  The three outputs must not overlap one another; any
 * of them may overlap d_keys, which is read only by the first kernel.  Work
 * is queued on `stream` (a cudaStream_t; NULL for the default stream) and is
 * complete when the stream is.  num_elements must lie in [1, 2^30)
 * (MPMG_ERR_INVALID otherwise).
 *
 * Scratch is a fixed device array inside this library (about 19 MB), held by
 * every GPU that loads it until the process exits; n above
 * MPMG_NOALLOC_MAX_PARTICLES is rejected with MPMG_ERR_SCRATCH_LIMIT.  The
 * first call on a device looks up that array's device address and keeps it
 * for the life of the process, so make the first call on each device before
 * any stream capture, and do not call this entry point on a device after
 * resetting it (cudaDeviceReset) in the same process: the kept address would
 * be stale.  All calls share the array, which keeps the last call's contents:
 * calls that overlap on the GPU race, so serialise them.  The entry point
 * calls no cudaMalloc or cudaFree.
 */
#define MPMG_NOALLOC_MAX_PARTICLES (1u << 20)
MPMG_API int mpmg_sort_cells_noalloc(const int *d_keys, int n, int num_elements, int *d_sorted_keys,
                                     int *d_perm, int *d_cell_start, void *stream);

MPMG_API const char *mpmg_status_string(int status);
/* Text of the last error on this thread (CUDA error text or argument check). */
MPMG_API const char *mpmg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
