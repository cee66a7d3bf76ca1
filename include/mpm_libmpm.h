/*
 * libmpm-compatible interface of mpm_gb300: the entry points and data types
 * the reference driver (src/main.c) and its dlopen'd material and
 * boundary-condition plugins compile against, with the explicit USL step run
 * on the GPU.  A driver built against the reference's libmpm headers links
 * against libmpm_gb300.so instead of libmpm.a.
 *
 * The types reproduce the reference's memory layout field for field, because
 * the driver and the plugins read and write them directly: particle_t
 * (libmpm/particle.h:34-147, 1280 bytes), node_t (libmpm/node.h:11-54,
 * 152 bytes), element_t (libmpm/element.h:29-67, 1504 bytes), job_t
 * (libmpm/process.h:116-213, 800 bytes) and threadtask_t
 * (libmpm/process.h:215-249, 96 bytes) on LP64.  The sizes are checked at
 * compile time in csrc/mpmg_libmpm.cu.
 *
 * Entry points (reference declarations they replace):
 *   mpm_init                          libmpm/process_usl.c:68   (process.h:251)
 *   explicit_mpm_step_usl_threaded    libmpm/process_usl.c:465  (process_usl.h:14)
 *   explicit_mpm_step_musl_threaded   libmpm/process_usl.c:284  (process_usl.h:13)
 *   find_filled_elements              libmpm/process_usl.c:677  (process_usl.h:17)
 *   mpm_cleanup                       libmpm/process_usl.c:974  (process.h:253)
 *   initial_loads, time_varying_loads libmpm/loading.c:21,34
 *   the *_split phase functions       libmpm/process_usl.h:15-22 (below)
 * plus additions that return an int status instead of exiting:
 *   mpm_gpu_attach, mpm_gpu_step, mpm_gpu_sync_host, mpm_gpu_detach, and the
 *   adjoint pair mpm_adj_forward_tape, mpm_adj_backward.
 */
#ifndef MPM_LIBMPM_H
#define MPM_LIBMPM_H

#include <pthread.h>
#include <stddef.h>
#include <stdio.h>
#include <time.h>

#include "mpm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DEPVAR 11
#define NDIM 3
#define NODES_PER_ELEMENT 4
#define NODAL_DOF 3
#define XDOF_IDX 0
#define YDOF_IDX 1

/* Stress/strain tensor indices of a 3x3 row-major tensor. */
#define XX 0
#define XY 1
#define XZ 2
#define YX 3
#define YY 4
#define YZ 5
#define ZX 6
#define ZY 7
#define ZZ 8

typedef struct particle_s {
    double x, y;                  /* position */
    double xl, yl;                /* local coordinates in the element */
    double v;                     /* volume */
    double v0;                    /* initial volume */
    double s[4];                  /* shape function values */
    double m;                     /* mass */
    double x_t, y_t;              /* velocity */
    double x_tt, y_tt;            /* acceleration */
    double bx, by;                /* body force per unit mass */
    double sxx, sxy, syy;         /* in-plane stress */
    double T[NDIM * NDIM];        /* full 3D stress */
    double exx_t, exy_t, eyy_t, wxy_t;   /* strain rate, spin */
    double L[NDIM * NDIM];        /* velocity gradient */
    double Fxx, Fxy, Fyx, Fyy;    /* deformation gradient */
    double ux, uy;                /* displacement */
    double color;
    double state[DEPVAR];         /* material state variables */
    int material;
    double grad_s[4][2];
    int element;
    double real_sxx, real_sxy, real_syy;
    double real_state[DEPVAR];
    double r1_initial[2], r2_initial[2];
    double r1[2], r2[2];
    double corners[4][2];
    double cornersl[4][2];
    double sc[4][4];
    double grad_sc[4][4][2];
    int corner_elements[4];
    void *material_data;
    size_t id;
} particle_t;

typedef struct node_s {
    int num_filled_element_neighbors;
    double mass_filled_element_neighbors;
    double m;
    double x, y;
    double ux, uy;
    double x_t, y_t;
    double x_tt, y_tt;
    double mx_t, my_t;
    double mx_tt, my_tt;
    double fx, fy;
    double rho;
    int velocity_update_flag;
} node_t;

typedef struct element_s {
    int color;
    int color_idx;
    int nodes[NODES_PER_ELEMENT];
    int n;
    double m;
    int filled;
    int neighbors[8];
    double grad_x, grad_y, grad_mag;
    double n_x, n_y, n_theta;
    double v;
    int p_index;
    double p_dist;
    double sxx, sxy, syy;
    double exx_t, exy_t, eyy_t;
    double wxy_t;
    double p;
    double tau;
    double kku_element[NODAL_DOF * NODES_PER_ELEMENT][NODAL_DOF * NODES_PER_ELEMENT];
    double f_element[NODAL_DOF * NODES_PER_ELEMENT];
    double jacobian[2][2];
} element_t;

enum solver_e { IMPLICIT_SOLVER = 0, EXPLICIT_SOLVER_USF, EXPLICIT_SOLVER_USL, NUM_SOLVERS };

typedef struct material_s { double E; double nu; double rho; } material_t;

typedef struct ts_control_s {
    double dt_max, dt_min, dt;
    int automatic_dt;
    int allow_dt_increase;
    int stable_dt_threshold;
} timestep_control_t;

typedef struct im_control_s {
    double du_norm_ratio, q_norm_ratio, du_norm_converged;
    int unstable_iteration_count;
    int stable_step_count;
} implicit_control_t;

typedef struct op_control_s {
    char *directory, *user, *particle_filename, *element_filename, *state_filename, *log_filename;
    char *particle_filename_fullpath, *element_filename_fullpath, *state_filename_fullpath,
        *log_filename_fullpath;
    FILE *particle_fd, *element_fd, *state_fd, *log_fd;
    FILE *info_fd;
    char *job_name, *job_description;
    int job_id;
    char *date;
    int override_directory_with_id;
    int prepend_date;
    int modified_directory;
    double sample_rate_hz;
} output_control_t;

struct job_s;

typedef struct mat_control_s {
    const char *material_filename;
    int use_builtin;
    void (*material_init)(struct job_s *);
    void (*calculate_stress)(struct job_s *);
    void (*calculate_stress_threaded)(void *);
    double *fp64_props;
    int *int_props;
    size_t num_fp64_props;
    size_t num_int_props;
} material_control_t;

typedef struct bc_control_s {
    const char *bc_filename;
    int use_builtin;
    void (*bc_init)(void *);
    int (*bc_validate)(void *);
    void (*bc_time_varying)(void *);
    void (*bc_momentum)(void *);
    void (*bc_force)(void *);
    double *fp64_props;
    int *int_props;
    size_t num_fp64_props;
    size_t num_int_props;
} boundary_control_t;

typedef struct job_s {
    double t, dt, t_stop;
    size_t frame;
    int stepcount;
    size_t num_particles, num_nodes, num_elements, num_colors;
    size_t *color_indices;
    size_t *particle_by_element_color_lengths;
    size_t **particle_by_element_color_lists;
    size_t N;
    double h;
    int use_cpdi;
    struct timespec tic, toc;
    node_t *nodes;
    particle_t *particles;
    element_t *elements;
    int *in_element;
    int *active;
    double *h1, *h2, *h3, *h4;
    double *b11, *b12, *b13, *b14;
    double *b21, *b22, *b23, *b24;
    int *node_u_map, *inv_node_u_map;
    double *u_dirichlet;
    int *u_dirichlet_mask;
    int *node_number_override;
    int vec_len;
    enum solver_e solver;
    timestep_control_t timestep;
    implicit_control_t implicit;
    output_control_t output;
    material_control_t material;
    boundary_control_t boundary;
    int step_number;
    double step_start_time;
    pthread_barrier_t *step_barrier;
    pthread_barrier_t *serialize_barrier;
    size_t num_threads;
    int *update_elementlists;
    int *update_elementlists_flag;
} job_t;

typedef struct s_threadtask {
    size_t id, num_threads;
    size_t gidx_min, gidx_max;
    size_t offset, blocksize;
    size_t n_offset, n_blocksize;
    size_t e_offset, e_blocksize;
    size_t stride;
    job_t *job;
} threadtask_t;

/*
 * Same contract as the reference: copies the particles (the caller keeps its
 * array), builds nodes, elements, colours and the initial element map, and
 * sets the default dt of process_usl.c:261.  No GPU work happens here.
 */
MPMG_API job_t *mpm_init(int N, double h, particle_t *particles, size_t num_particles, double t);

/*
 * Called by every thread of the driver's team with its threadtask_t, as the
 * reference's step is.  The team meets at job->serialize_barrier; one thread
 * runs the whole step on the GPU (attaching on the first call: the material
 * and boundary conditions are chosen by the plugin file's basename, isolin,
 * g_local_mu2, g_nonlocal_mu2, g_nonlocal, dp_ri_mt, g_local_mu2_plane_strain,
 * g_local_mu2_true_2d, g_local_mu2_ext, g_nonlocal_avg, g_nonlocal_bicgstab,
 * g_nonlocalxs71 / box, square_silo) while the rest
 * wait; then job->t advances and, when the driver will write a frame after
 * this step (job->t >= job->frame / sample_rate) or the run ends, the host
 * particle array is refreshed from the GPU.  On a GPU error it prints the
 * reason and exits with the reference's code (EXIT_ERROR_CS_SOL for a failed
 * fluidity solve, EXIT_ERROR_MATERIAL_FILE for an unsupported plugin).
 */
MPMG_API void explicit_mpm_step_usl_threaded(void *task);
/* The MUSL step (second projection of the moved particles' momentum before
   the strain rate); the job's GPU context is created with the scheme of the
   first step entry called. */
MPMG_API void explicit_mpm_step_musl_threaded(void *task);

/* The reference's per-(thread, colour) particle lists (host; the driver calls
   it once before the time loop). */
MPMG_API void find_filled_elements(job_t *job);

/*
 * The phases of the threaded USL step (libmpm/process_usl.h:15-22), with the
 * reference's names, signatures and ranges, on the job's host arrays: each
 * call gathers its range, runs one FP64 kernel on the GPU (the attached
 * context's device, device 0 without one) and writes the results back, in
 * the reference's operation order.  They do not touch an attached GPU
 * context's device state.  Threads may call them concurrently on disjoint
 * ranges; a CUDA failure ends the process (the reference's phases return
 * nothing).
 *   move_grid_split                      process_usl.c:596-625  (process_usl.h:15)
 *   create_particle_to_element_map_threaded  process_usl.c:631-674  (:16)
 *   calculate_shapefunctions_split       process_usl.c:727-760  (:18)
 *   calculate_strainrate_split           process_usl.c:764-808  (:19; the CPDI
 *                                        branch, dead in the reference, ends the
 *                                        process)
 *   map_to_grid_explicit_split           process_usl.c:812-910  (:20; called by
 *                                        every thread of the team like the
 *                                        reference's: the thread with id 0 maps
 *                                        all lists, and all meet at the job's
 *                                        barrier once per colour)
 *   move_particles_explicit_usl_split    process_usl.c:914-957  (:21)
 *   update_particle_densities_split      process_usl.c:961-970  (:22)
 */
MPMG_API void move_grid_split(job_t *job, size_t n_start, size_t n_stop);
MPMG_API void create_particle_to_element_map_threaded(threadtask_t *task);
MPMG_API void calculate_shapefunctions_split(job_t *job, size_t p_start, size_t p_stop);
MPMG_API void calculate_strainrate_split(job_t *job, size_t p_start, size_t p_stop);
MPMG_API void map_to_grid_explicit_split(job_t *job, size_t thread_id);
MPMG_API void move_particles_explicit_usl_split(job_t *job, size_t p_start, size_t p_stop);
MPMG_API void update_particle_densities_split(job_t *job, size_t p_start, size_t p_stop);

MPMG_API void mpm_cleanup(job_t *job);

/* Body forces: 0 before the first step, then the 9.8 m/s^2 ramp over 0.1 s.
   When a GPU context is attached the device applies the same ramp, and the
   host copy of bx, by is refreshed with the particles. */
MPMG_API void initial_loads(job_t *job);
MPMG_API void time_varying_loads(job_t *job);

/* Additions with status returns. */
MPMG_API int mpm_gpu_attach(job_t *job);
MPMG_API int mpm_gpu_step(job_t *job, int nsteps);
MPMG_API int mpm_gpu_sync_host(job_t *job);
MPMG_API int mpm_gpu_detach(job_t *job);

/* The adjoint pair on a job (see mpmg_adj_forward_tape / mpmg_adj_backward in
   mpm_gb300.h): nsteps taped steps from the job's current state (job->t
   advances), then the gradient of a loss on the final positions with respect
   to (mu_s, mu_2, I0, E).  The host particles are not refreshed by either;
   call mpm_gpu_sync_host for them. */
MPMG_API int mpm_adj_forward_tape(job_t *job, int nsteps, int checkpoint_every);
MPMG_API int mpm_adj_backward(job_t *job, const double *dl_dx, const double *dl_dy, double *dl_dtheta);

#ifdef __cplusplus
}
#endif

#endif
