/*
 * Test infrastructure: the oracle.  A plain-C, pthreaded CPU restatement of
 * the reference's explicit USL step (libmpm/process_usl.c:465-970), its
 * material plugins (materialsrc/isolin.c, g_local_mu2.c, g_nonlocal_mu2.c,
 * g_nonlocal.c), its boundary plugins (bcsrc/box.c, square_silo.c) and its
 * loading (libmpm/loading.c).  Only tests/, the smoke check and the CPU
 * baseline of bench.py load it; the product library never does.
 *
 * Differences from the reference, all deliberate:
 *  - The grid may be Nx x Ny nodes (the reference is N x N); the inside test
 *    of the element map uses the bounds xmax, ymax (1.0 in the reference,
 *    process_usl.c:43-44).
 *  - Material constants the reference fixes with #define are runtime
 *    parameters (defaults are the reference values).
 *  - g_nonlocal_mu2's uninitialised lambda (g_nonlocal_mu2.c:154) takes the
 *    value K - 2G/3 of :257.
 *  - The fluidity system is solved by a banded LDL^T (direct) or by
 *    Jacobi-preconditioned CG, in place of CXSparse's LU.
 *  - Gravity may be the reference ramp (loading.c:34-54) or a constant.
 */
#ifndef MPM_ORACLE_H
#define MPM_ORACLE_H

#include <stddef.h>

enum orc_material { ORC_ISOLIN = 0, ORC_G_LOCAL_MU2 = 1, ORC_G_NONLOCAL_MU2 = 2, ORC_G_NONLOCAL = 3,
                    ORC_DP_RI_MT = 4, ORC_G_LOCAL_MU2_PLANE_STRAIN = 5, ORC_G_LOCAL_MU2_TRUE_2D = 6,
                    ORC_G_LOCAL_MU2_EXT = 7, ORC_G_NONLOCAL_AVG = 8, ORC_G_LOCAL_MU2_REVERSE = 9 };
enum orc_bc { ORC_BOX = 0, ORC_SQUARE_SILO = 1 };
enum orc_gravity { ORC_GRAVITY_REFERENCE_RAMP = 0, ORC_GRAVITY_CONSTANT = 1 };
enum orc_solver { ORC_SOLVER_DIRECT = 0, ORC_SOLVER_PCG = 1 };

/* Material parameter slots (mp[]). */
enum orc_mparam {
    ORC_MP_E = 0, ORC_MP_NU, ORC_MP_MU_S, ORC_MP_MU_2, ORC_MP_I0, ORC_MP_GRAINS_RHO,
    ORC_MP_GRAINS_D, ORC_MP_A, ORC_MP_RHO_CRITICAL, ORC_MP_B, ORC_MP_COHESION,
    ORC_MP_COUNT = 16
};

/* Step scheme: update stress last (explicit_mpm_step_usl_threaded,
   process_usl.c:465-592) or the modified form with a second projection of
   the updated particle momentum (explicit_mpm_step_musl_threaded,
   process_usl.c:284-462). */
enum orc_scheme { ORC_USL = 0, ORC_MUSL = 1 };

typedef struct orc_config {
    int Nx, Ny;          /* nodes per grid row / column */
    double h;            /* element edge length */
    double xmax, ymax;   /* element-map inside bounds */
    double dt;
    int material;        /* enum orc_material */
    double mp[ORC_MP_COUNT];
    int bc;              /* enum orc_bc */
    double bcf[4];       /* box: x0, y0, w, h.  silo: hole radius, open time, wall fraction */
    int bci[4];          /* box: friction bits left, bottom, right, top */
    int gravity_mode;    /* enum orc_gravity */
    double gravity;      /* constant mode: body force per unit mass in y */
    int nthreads;
    int solver;          /* enum orc_solver (nonlocal materials) */
    double cg_tol;       /* relative residual for ORC_SOLVER_PCG */
    int cg_maxit;
    int scheme;          /* enum orc_scheme */
} orc_config;

typedef struct orc_sim orc_sim;

/* Fills mp[] with the reference's constants for the material kind. */
void orc_default_params(int material, double *mp);

orc_sim *orc_create(const orc_config *cfg, size_t n, const double *m, const double *v,
                    const double *x, const double *y, const double *vx, const double *vy,
                    const double *sxx, const double *sxy, const double *syy);
void orc_destroy(orc_sim *s);

/* Runs nsteps of the driver loop: USL (or MUSL) step, then the serial tail
   (time_varying_loads).  Returns 0, or a nonzero status on a solver failure. */
int orc_step(orc_sim *s, int nsteps);

/* Runs only the material update on all particles with the current strain
   rates (the per-particle path of tests/test_material.c:173-177). */
int orc_material_only(orc_sim *s);

/* Named field access.  Particle fields: x y xl yl v v0 m vx vy ax ay bx by
   sxx sxy syy ux uy exx exy eyy wxy Txx Txy Tyx Tyy Tzz state0..state10.
   Node fields: node_m node_mx node_my node_fx node_fy node_vx node_vy
   node_ax node_ay.  Returns the element count, or -1 for an unknown name. */
long orc_get_field(orc_sim *s, const char *name, double *out);
long orc_set_field(orc_sim *s, const char *name, const double *in);
void orc_get_map(orc_sim *s, int *in_element, int *active);
void orc_set_map(orc_sim *s, const int *in_element, const int *active);
double orc_time(orc_sim *s);
void orc_set_time(orc_sim *s, double t, int step_number);
size_t orc_num_particles(orc_sim *s);
size_t orc_num_nodes(orc_sim *s);

/* Colour lists as find_filled_elements builds them (process_usl.c:703-720),
   concatenated; lengths[T*4]. */
void orc_get_color_lists(orc_sim *s, size_t *out, size_t *lengths);
/* Element occupancy (filled, n, m) from the last find_filled_elements. */
void orc_get_elements(orc_sim *s, int *filled, int *count, double *mass);

/* Last fluidity solve: iterations (0 for direct) and relative residual. */
int orc_last_solve(orc_sim *s, int *iters, double *resid);

#endif
