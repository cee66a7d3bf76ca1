/*
 * Test infrastructure: the oracle (CPU restatement of the reference's USL
 * step).  See mpm_oracle.h for scope and deliberate differences.  Every
 * phase cites the reference lines it follows; the arithmetic keeps the
 * reference's operation order so that, compiled with -ffp-contract=off, it
 * reproduces the reference bit for bit on the reference's own cases.
 *
 * The thread team mirrors the reference driver: particles, nodes and
 * elements are split into contiguous ranges per thread (src/main.c:747-774),
 * P2G walks per-(thread, colour) particle lists with a barrier per colour
 * (process_usl.c:842-907), and serial sections run on one thread between
 * barriers (process_usl.c:519-567, src/main.c:951-976).
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "banded.h"
#include "mpm_oracle.h"

#define TOL 1e-10       /* process_usl.c:25 */
#define DEPVAR 11       /* particle.h:13 */
#define NCOLORS 4       /* process_usl.c:147 */

/* 3x3 tensor component indices, particle.h:22-31. */
#define XX 0
#define XY 1
#define XZ 2
#define YX 3
#define YY 4
#define YZ 5
#define ZX 6
#define ZY 7
#define ZZ 8

typedef struct orc_task {
    struct orc_sim *s;
    size_t id;
    size_t p0, p1, n0, n1, e0, e1;
    int nsteps;
    int status;
} orc_task;

struct orc_sim {
    orc_config c;
    size_t np, nn, ne;
    size_t Ex, Ey;            /* elements per row / column */
    double t;
    int step_number;
    double step_start_time;
    double G, K, lambda;      /* derived elastic constants (material_init) */

    /* particles */
    double *x, *y, *xl, *yl, *v, *v0, *m, *vx, *vy, *ax, *ay, *bx, *by;
    double *sxx, *sxy, *syy, *ux, *uy, *exx, *exy, *eyy, *wxy;
    double *T;                /* 9 per particle (g_local_mu2) */
    double *state;            /* DEPVAR per particle */
    int *in_element, *active;
    double *h1, *h2, *h3, *h4, *b11, *b12, *b13, *b14, *b21, *b22, *b23, *b24;

    /* nodes */
    double *nx, *ny;
    double *nm, *nmx, *nmy, *nmxx, *nmyy, *nfx, *nfy, *nvx, *nvy, *nax, *nay, *nux, *nuy;
    int *mask;                /* 3 per node: x, y, unused DOF */

    /* elements */
    int *enodes;              /* 4 per element: BL, BR, TR, TL */
    int *ecolor, *ecolor_idx, *efilled, *en;
    double *em;
    size_t color_indices[NCOLORS];

    /* per-(thread, colour) particle lists, find_filled_elements */
    size_t **lists;
    size_t *list_len;
    int *update_flags;

    /* thread team */
    size_t T_threads;
    orc_task *tasks;
    pthread_barrier_t bar;

    /* nonlocal solve */
    double *gf_nodes;
    long *node_map;
    int solve_status;
    int solve_iters;
    double solve_resid;
};

/*---------------------------------------------------------------------------*/
void orc_default_params(int material, double *mp)
{
    for (int i = 0; i < ORC_MP_COUNT; i++) {
        mp[i] = 0.0;
    }
    mp[ORC_MP_E] = 1e6;
    mp[ORC_MP_NU] = 0.3;
    switch (material) {
    case ORC_G_LOCAL_MU2:             /* g_local_mu2.c:30-41 */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_MU_2] = 0.6435;
        mp[ORC_MP_I0] = 0.278 / 1.0;
        mp[ORC_MP_GRAINS_D] = 0.001 * 5;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0f; /* g_local_mu2.c:236 literal */
        break;
    case ORC_G_NONLOCAL_MU2:          /* g_nonlocal_mu2.c:32-47 */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_A] = 0.48;
        mp[ORC_MP_MU_2] = 0.6435;
        mp[ORC_MP_I0] = 0.278;
        mp[ORC_MP_GRAINS_D] = 0.005;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0;
        break;
    case ORC_DP_RI_MT:                /* dp_ri_mt.c:66-76 reads E, nu, mu_s */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0f; /* dp_ri_mt.c:159 literal */
        break;
    case ORC_G_LOCAL_MU2_PLANE_STRAIN: /* g_local_mu2_plane_strain.c:27-38 */
    case ORC_G_LOCAL_MU2_TRUE_2D:      /* g_local_mu2_true_2d.c:27-38 */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_MU_2] = 0.6435;
        mp[ORC_MP_I0] = 0.278 / 1.0;
        mp[ORC_MP_GRAINS_D] = material == ORC_G_LOCAL_MU2_TRUE_2D ? 0.01 * 5 : 0.001 * 5;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0f;
        break;
    case ORC_G_LOCAL_MU2_REVERSE:      /* g_local_mu2_reverse.c:33-53 */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_MU_2] = 0.6435;
        mp[ORC_MP_I0] = 0.278 / 1.0;
        mp[ORC_MP_GRAINS_D] = 0.01 * 5;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0f;
        break;
    case ORC_G_LOCAL_MU2_EXT:          /* g_local_mu2_ext.c:26-45 */
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_A] = 4.8;
        mp[ORC_MP_MU_2] = 0.6435;
        mp[ORC_MP_I0] = 0.278 / 1.0;
        mp[ORC_MP_GRAINS_D] = 0.01 * 5;
        mp[ORC_MP_RHO_CRITICAL] = 1485.0f;
        break;
    case ORC_G_NONLOCAL:              /* g_nonlocal.c:31-48 */
    case ORC_G_NONLOCAL_AVG:          /* g_nonlocal_avg.c: the same constants */
        mp[ORC_MP_E] = 1e8;
        mp[ORC_MP_NU] = 0.3;
        mp[ORC_MP_MU_S] = 0.3819;
        mp[ORC_MP_GRAINS_RHO] = 2450;
        mp[ORC_MP_B] = 0.9377 * 20;
        mp[ORC_MP_A] = 0.48;
        mp[ORC_MP_GRAINS_D] = 0.01 * 5;
        mp[ORC_MP_COHESION] = 1e-2;
        break;
    default:
        break;
    }
}

static double *dalloc(size_t n)
{
    return (double *)calloc(n ? n : 1, sizeof(double));
}

static int *ialloc(size_t n)
{
    return (int *)calloc(n ? n : 1, sizeof(int));
}

/* WHICH_ELEMENT4, process_usl.c:43-44, with the inside bounds as parameters
   and an explicit range check (the reference indexes out of range when
   floor(x/h) rounds up to Nx-1 at x just below 1). */
static int which_element(const orc_sim *s, double xp, double yp)
{
    if (!(xp < s->c.xmax && xp >= 0.0 && yp < s->c.ymax && yp >= 0.0)) {
        return -1;
    }
    double e = floor(xp / s->c.h) + floor(yp / s->c.h) * (double)(s->c.Nx - 1);
    if (!(e >= 0.0) || e >= (double)s->ne) {
        return -1;
    }
    int ix = (int)floor(xp / s->c.h);
    if (ix >= s->c.Nx - 1) {
        return -1;
    }
    return (int)e;
}

static void find_filled_elements(orc_sim *s);

/*---------------------------------------------------------------------------*/
orc_sim *orc_create(const orc_config *cfg, size_t n, const double *m, const double *v,
                    const double *x, const double *y, const double *vx, const double *vy,
                    const double *sxx, const double *sxy, const double *syy)
{
    if (cfg->Nx < 2 || cfg->Ny < 2 || !(cfg->h > 0)) {
        return NULL;
    }
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->c = *cfg;
    if (s->c.nthreads < 1) {
        s->c.nthreads = 1;
    }
    s->np = n;
    s->Ex = (size_t)cfg->Nx - 1;
    s->Ey = (size_t)cfg->Ny - 1;
    s->nn = (size_t)cfg->Nx * (size_t)cfg->Ny;
    s->ne = s->Ex * s->Ey;

    size_t np = n;
#define PA(f) s->f = dalloc(np)
    PA(x); PA(y); PA(xl); PA(yl); PA(v); PA(v0); PA(m); PA(vx); PA(vy); PA(ax); PA(ay);
    PA(bx); PA(by); PA(sxx); PA(sxy); PA(syy); PA(ux); PA(uy); PA(exx); PA(exy); PA(eyy);
    PA(wxy); PA(h1); PA(h2); PA(h3); PA(h4); PA(b11); PA(b12); PA(b13); PA(b14);
    PA(b21); PA(b22); PA(b23); PA(b24);
#undef PA
    s->T = dalloc(9 * np);
    s->state = dalloc(DEPVAR * np);
    s->in_element = ialloc(np);
    s->active = ialloc(np);

    size_t nn = s->nn;
#define NA(f) s->f = dalloc(nn)
    NA(nx); NA(ny); NA(nm); NA(nmx); NA(nmy); NA(nmxx); NA(nmyy); NA(nfx); NA(nfy);
    NA(nvx); NA(nvy); NA(nax); NA(nay); NA(nux); NA(nuy); NA(gf_nodes);
#undef NA
    s->mask = ialloc(3 * nn);
    s->node_map = (long *)calloc(nn ? nn : 1, sizeof(long));

    /* mpm_init particle copy, process_usl.c:88-126 */
    for (size_t i = 0; i < np; i++) {
        s->m[i] = m[i];
        s->v[i] = v[i];
        s->x[i] = x[i];
        s->y[i] = y[i];
        s->vx[i] = vx[i];
        s->vy[i] = vy[i];
        s->sxx[i] = sxx[i];
        s->sxy[i] = sxy[i];
        s->syy[i] = syy[i];
        s->v0[i] = v[i];
    }

    /* node_number_to_coords, element.c:10-19 */
    for (size_t i = 0; i < nn; i++) {
        int ii = (int)(i % (size_t)cfg->Nx);
        int jj = (int)(i / (size_t)cfg->Nx);
        s->nx[i] = ii * cfg->h;
        s->ny[i] = jj * cfg->h;
    }

    /* element connectivity and colour, process_usl.c:136-158 */
    s->enodes = ialloc(4 * s->ne);
    s->ecolor = ialloc(s->ne);
    s->ecolor_idx = ialloc(s->ne);
    s->efilled = ialloc(s->ne);
    s->en = ialloc(s->ne);
    s->em = dalloc(s->ne);
    for (size_t e = 0; e < s->ne; e++) {
        size_t r = e / s->Ex, c = e % s->Ex;
        int n0 = (int)(r * (size_t)cfg->Nx + c);
        s->enodes[4 * e + 0] = n0;
        s->enodes[4 * e + 1] = n0 + 1;
        s->enodes[4 * e + 2] = n0 + 1 + cfg->Nx;
        s->enodes[4 * e + 3] = n0 + cfg->Nx;
        s->ecolor[e] = (int)(2 * (r % 2) + ((c % 2) + 1) - 1);
    }

    /* initial element map, process_usl.c:236-244 */
    for (size_t i = 0; i < np; i++) {
        s->in_element[i] = which_element(s, s->x[i], s->y[i]);
        s->active[i] = (s->in_element[i] < 0) ? 0 : 1;
    }

    /* thread split, src/main.c:747-774 */
    size_t T = (size_t)s->c.nthreads;
    s->T_threads = T;
    s->tasks = (orc_task *)calloc(T, sizeof(orc_task));
    size_t ps = np / T + ((np % T) ? 1 : 0);
    size_t ns = nn / T + ((nn % T) ? 1 : 0);
    size_t es = s->ne / T + ((s->ne % T) ? 1 : 0);
    for (size_t i = 0; i < T; i++) {
        orc_task *t = &s->tasks[i];
        t->s = s;
        t->id = i;
        t->p0 = i * ps < np ? i * ps : np;
        t->p1 = t->p0 + ps < np ? t->p0 + ps : np;
        t->n0 = i * ns < nn ? i * ns : nn;
        t->n1 = t->n0 + ns < nn ? t->n0 + ns : nn;
        t->e0 = i * es < s->ne ? i * es : s->ne;
        t->e1 = t->e0 + es < s->ne ? t->e0 + es : s->ne;
    }
    pthread_barrier_init(&s->bar, NULL, (unsigned)T);
    s->lists = (size_t **)calloc(T * NCOLORS, sizeof(size_t *));
    for (size_t i = 0; i < T * NCOLORS; i++) {
        s->lists[i] = (size_t *)calloc(np ? np : 1, sizeof(size_t));
    }
    s->list_len = (size_t *)calloc(T * NCOLORS, sizeof(size_t));
    s->update_flags = ialloc(T);
    for (size_t i = 0; i < T; i++) {
        s->update_flags[i] = 1;
    }

    /* initial_loads, loading.c:21-30 */
    for (size_t i = 0; i < np; i++) {
        s->bx[i] = 0;
        s->by[i] = 0;
    }
    if (s->c.gravity_mode == ORC_GRAVITY_CONSTANT) {
        for (size_t i = 0; i < np; i++) {
            s->by[i] = s->c.gravity;
        }
    }

    /* material_init */
    double E = s->c.mp[ORC_MP_E], nu = s->c.mp[ORC_MP_NU];
    s->G = E / (2.0 * (1.0 + nu));
    s->K = E / (3.0 * (1.0 - 2 * nu));
    s->lambda = s->K - 2.0 * s->G / 3.0;
    if (s->c.material == ORC_G_NONLOCAL || s->c.material == ORC_G_NONLOCAL_AVG) {
        /* g_nonlocal.c:34-35: G and K from the compile-time EMOD and NUMOD. */
        s->G = (E / (2.0f * (1.0f + nu)));
        s->K = (E / (3.0f * (1.0f - 2 * nu)));
    }
    for (size_t i = 0; i < np; i++) {
        double *st = s->state + DEPVAR * i;
        for (int k = 0; k < DEPVAR; k++) {
            st[k] = 0;
        }
        if (s->c.material == ORC_G_LOCAL_MU2) {
            /* g_local_mu2.c:110-120 */
            double *T9 = s->T + 9 * i;
            T9[XX] = s->sxx[i];
            T9[XY] = s->sxy[i];
            T9[XZ] = 0;
            T9[YX] = s->sxy[i];
            T9[YY] = s->syy[i];
            T9[YZ] = 0;
            T9[ZX] = 0;
            T9[ZY] = 0;
            T9[ZZ] = 0;
        } else if (s->c.material == ORC_G_NONLOCAL_MU2) {
            /* g_nonlocal_mu2.c:78-82 */
            st[0] = ((s->m[i] / s->v[i]) > s->c.mp[ORC_MP_RHO_CRITICAL]) ? 1 : 0;
        }
    }
    /* src/main.c:806-812: the driver builds the element lists once before
       the time loop. */
    find_filled_elements(s);
    s->solve_status = 0;
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (s == NULL) {
        return;
    }
    double **dp[] = {&s->x, &s->y, &s->xl, &s->yl, &s->v, &s->v0, &s->m, &s->vx, &s->vy,
                     &s->ax, &s->ay, &s->bx, &s->by, &s->sxx, &s->sxy, &s->syy, &s->ux,
                     &s->uy, &s->exx, &s->exy, &s->eyy, &s->wxy, &s->T, &s->state,
                     &s->h1, &s->h2, &s->h3, &s->h4, &s->b11, &s->b12, &s->b13, &s->b14,
                     &s->b21, &s->b22, &s->b23, &s->b24, &s->nx, &s->ny, &s->nm, &s->nmx,
                     &s->nmy, &s->nmxx, &s->nmyy, &s->nfx, &s->nfy, &s->nvx, &s->nvy,
                     &s->nax, &s->nay, &s->nux, &s->nuy, &s->em, &s->gf_nodes};
    for (size_t i = 0; i < sizeof(dp) / sizeof(dp[0]); i++) {
        free(*dp[i]);
    }
    free(s->in_element);
    free(s->active);
    free(s->mask);
    free(s->node_map);
    free(s->enodes);
    free(s->ecolor);
    free(s->ecolor_idx);
    free(s->efilled);
    free(s->en);
    for (size_t i = 0; i < s->T_threads * NCOLORS; i++) {
        free(s->lists[i]);
    }
    free(s->lists);
    free(s->list_len);
    free(s->update_flags);
    free(s->tasks);
    pthread_barrier_destroy(&s->bar);
    free(s);
}

/*---------------------------------------------------------------------------*/
/* find_filled_elements, process_usl.c:677-723 */
static void find_filled_elements(orc_sim *s)
{
    for (int c = 0; c < NCOLORS; c++) {
        s->color_indices[c] = 0;
    }
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        int p = s->in_element[i];
        s->efilled[p] = 1;
        s->en[p]++;
        s->em[p] += s->m[i];
    }
    for (size_t e = 0; e < s->ne; e++) {
        if (s->efilled[e]) {
            s->ecolor_idx[e] = (int)s->color_indices[s->ecolor[e]];
            s->color_indices[s->ecolor[e]]++;
        }
    }
    for (size_t i = 0; i < s->T_threads * NCOLORS; i++) {
        s->list_len[i] = 0;
    }
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        int p = s->in_element[i];
        size_t c_idx = (size_t)s->ecolor[p];
        size_t t_idx = (size_t)s->ecolor_idx[p] % s->T_threads;
        size_t tc = t_idx * NCOLORS + c_idx;
        s->lists[tc][s->list_len[tc]++] = i;
    }
}

/* bc_time_varying: box.c:106-167 and square_silo.c:58-91 (node numbering
   override is the identity in both, box.c:171-180, square_silo.c:94-103). */
static void generate_dirichlet_bcs(orc_sim *s)
{
    size_t Nx = (size_t)s->c.Nx, Ny = (size_t)s->c.Ny;
    memset(s->mask, 0, sizeof(int) * 3 * s->nn);
    if (s->c.bc == ORC_BOX) {
        double x0 = s->c.bcf[0], y0 = s->c.bcf[1], w = s->c.bcf[2], hh = s->c.bcf[3];
        /* box.c:92-95: column and row indices of the walls */
        size_t left_col = (size_t)(x0 * (Nx - 1));
        size_t right_col = (size_t)((x0 + w) * (Nx - 1));
        size_t bottom_row = (size_t)(y0 * (Ny - 1));
        size_t top_row = (size_t)((y0 + hh) * (Ny - 1));
        int lf = s->c.bci[0], bf = s->c.bci[1], rf = s->c.bci[2], tf = s->c.bci[3];
        for (size_t n = left_col; n <= right_col; n++) {
            size_t b = n + bottom_row * Nx;
            size_t t = n + top_row * Nx;
            if (bf & 1) s->mask[3 * b + 0] = 1;
            if (bf & 2) s->mask[3 * b + 1] = 1;
            if (tf & 1) s->mask[3 * t + 0] = 1;
            if (tf & 2) s->mask[3 * t + 1] = 1;
        }
        for (size_t n = bottom_row; n <= top_row; n++) {
            size_t l = n * Nx + left_col;
            size_t r = n * Nx + right_col;
            if (lf & 1) s->mask[3 * l + 0] = 1;
            if (lf & 2) s->mask[3 * l + 1] = 1;
            if (rf & 1) s->mask[3 * r + 0] = 1;
            if (rf & 2) s->mask[3 * r + 1] = 1;
        }
    } else {
        double hole_radius = s->c.bcf[0], open_time = s->c.bcf[1];
        size_t wall_col = (size_t)(int)((Nx - 1) * s->c.bcf[2]);   /* square_silo.c:44 */
        for (size_t n = 0; n < Nx; n++) {
            if (s->nx[n] <= hole_radius && s->t > open_time) {
                continue;
            }
            s->mask[3 * n + 0] = 1;
            s->mask[3 * n + 1] = 1;
        }
        for (size_t n = 0; n < Ny; n++) {
            s->mask[3 * (0 + n * Nx) + 0] = 1;
            s->mask[3 * (wall_col + n * Nx) + 0] = 1;
        }
    }
}

/* time_varying_loads, loading.c:34-54 */
static void time_varying_loads(orc_sim *s)
{
    double gravity;
    if (s->c.gravity_mode == ORC_GRAVITY_CONSTANT) {
        gravity = s->c.gravity;
    } else if ((0.1 + s->step_start_time) > s->t) {
        gravity = -9.8 * ((s->t - s->step_start_time) / 0.1);
    } else {
        gravity = -9.8;
    }
    for (size_t i = 0; i < s->np; i++) {
        s->bx[i] = 0;
        s->by[i] = gravity;
    }
}

/*---------------------------------------------------------------------------*/
/* Material kernels. */

static double negative_root(double a, double b, double c)
{
    /* g_local_mu2.c:90-99 */
    double x;
    if (b > 0) {
        x = (-b - sqrt(b * b - 4 * a * c)) / (2 * a);
    } else {
        x = (2 * c) / (-b + sqrt(b * b - 4 * a * c));
    }
    return x;
}

/* isolin calculate_stress_threaded, isolin.c:75-116 */
static void isolin_range(orc_sim *s, size_t p0, size_t p1)
{
    const double G = s->G, lambda = s->lambda, dt = s->c.dt;
    for (size_t i = p0; i < p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double trD = s->exx[i] + s->eyy[i];
        double dsjxx = lambda * trD + 2.0 * G * s->exx[i];
        double dsjxy = 2.0 * G * s->exy[i];
        double dsjyy = lambda * trD + 2.0 * G * s->eyy[i];
        dsjxx += 2 * s->wxy[i] * s->sxy[i];
        dsjxy -= s->wxy[i] * (s->sxx[i] - s->syy[i]);
        dsjyy -= 2 * s->wxy[i] * s->sxy[i];
        s->sxx[i] += dt * dsjxx;
        s->sxy[i] += dt * dsjxy;
        s->syy[i] += dt * dsjyy;
    }
}

/* 3x3 helpers restated from libmpm/tensor.c (operation order kept). */
static void t_mul(double *C, const double *A, const double *B)      /* tensor.c:270-289 */
{
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            C[i * 3 + j] = A[3 * i + 0] * B[3 * 0 + j] + A[3 * i + 1] * B[3 * 1 + j]
                         + A[3 * i + 2] * B[3 * 2 + j];
        }
    }
}

static double t_trace(const double *A)                               /* tensor.c:51-61 */
{
    double tr = 0;
    for (int i = 0; i < 3; i++) {
        tr += A[i * 3 + i];
    }
    return tr;
}

/* g_local_mu2 calculate_stress_threaded, g_local_mu2.c:165-310 */
static void g_local_mu2_range(orc_sim *s, size_t p0, size_t p1)
{
    const double G = s->G, K = s->K, dt = s->c.dt;
    const double *mp = s->c.mp;
    const double lambda = K - 2.0 * G / 3.0;
    for (size_t i = p0; i < p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *T = s->T + 9 * i;
        double *st = s->state + DEPVAR * i;
        double L[9], W[9], D[9], Ttr[9], JS[9], temp[9], T0[9];
        L[XX] = s->exx[i];
        L[XY] = s->exy[i] + s->wxy[i];
        L[XZ] = 0;
        L[YX] = s->exy[i] - s->wxy[i];
        L[YY] = s->eyy[i];
        L[YZ] = 0;
        L[ZX] = 0;
        L[ZY] = 0;
        L[ZZ] = 0;
        for (int a = 0; a < 3; a++) {
            for (int b = 0; b < 3; b++) {
                W[a * 3 + b] = 0.5 * (L[a * 3 + b] - L[b * 3 + a]);   /* tensor.c:370-384 */
                D[a * 3 + b] = 0.5 * (L[a * 3 + b] + L[b * 3 + a]);   /* tensor.c:330-344 */
            }
        }
        memcpy(Ttr, D, sizeof(Ttr));
        double trD = t_trace(D);
        t_mul(JS, W, T);
        t_mul(temp, T, W);
        for (int k = 0; k < 9; k++) {
            temp[k] *= -1.0;
        }
        for (int k = 0; k < 9; k++) {
            JS[k] += temp[k];
        }
        for (int k = 0; k < 9; k++) {
            Ttr[k] *= 2.0 * G;
        }
        Ttr[XX] += lambda * trD;
        Ttr[YY] += lambda * trD;
        Ttr[ZZ] += lambda * trD;
        for (int k = 0; k < 9; k++) {
            Ttr[k] += JS[k];
        }
        for (int k = 0; k < 9; k++) {
            Ttr[k] *= dt;
        }
        for (int k = 0; k < 9; k++) {
            Ttr[k] += T[k];
        }
        /* tensor_decompose3, tensor.c:205-224 */
        double p_tr = t_trace(Ttr) / 3.0;
        memcpy(T0, Ttr, sizeof(T0));
        for (int a = 0; a < 3; a++) {
            T0[a * 3 + a] = T0[a * 3 + a] - p_tr;
        }
        /* tensor_contraction3, tensor.c:422-437 */
        double tau_tr = 0;
        for (int k = 0; k < 9; k++) {
            tau_tr += T0[k] * T0[k];
        }
        tau_tr = sqrt(0.5 * tau_tr);
        p_tr *= -1.0;

        int density_flag = (s->m[i] / s->v[i]) < mp[ORC_MP_RHO_CRITICAL];
        double nup_tau;
        if (density_flag || p_tr <= 0) {
            nup_tau = 0;
            for (int k = 0; k < 9; k++) {
                T[k] = 0;
            }
        } else if (p_tr > 0) {
            double tau_tau, scale_factor;
            double S0 = mp[ORC_MP_MU_S] * p_tr;
            if (tau_tr <= S0) {
                tau_tau = tau_tr;
                scale_factor = 1.0;
            } else {
                double S2 = mp[ORC_MP_MU_2] * p_tr;
                double alpha = G * mp[ORC_MP_I0] * dt * sqrt(p_tr / mp[ORC_MP_GRAINS_RHO])
                               / mp[ORC_MP_GRAINS_D];
                double B = -(S2 + tau_tr + alpha);
                double H = S2 * tau_tr + S0 * alpha;
                tau_tau = negative_root(1.0, B, H);
                scale_factor = (tau_tau / tau_tr);
            }
            nup_tau = ((tau_tr - tau_tau) / G) / dt;
            for (int k = 0; k < 9; k++) {
                T0[k] *= scale_factor;
            }
            memcpy(T, T0, sizeof(T0));
            T[XX] -= p_tr;
            T[YY] -= p_tr;
            T[ZZ] -= p_tr;
        } else {
            nup_tau = 0;
        }
        s->sxx[i] = T[XX];
        s->sxy[i] = T[XY];
        s->syy[i] = T[YY];
        st[9] += nup_tau * dt;
        st[10] = nup_tau;
    }
}

/* The local returns written on the in-plane stress (sxx, sxy, syy):
     dp_ri_mt                  dp_ri_mt.c:99-200                   trial3d, Drucker-Prager
     g_local_mu2_plane_strain  g_local_mu2_plane_strain.c:157-265  trial3d, mu(I), beta
     g_local_mu2_true_2d       g_local_mu2_true_2d.c:157-260       2D trial, mu(I), beta
   trial3d carries szz in state[1] and takes p = -(sxx + syy + szz) / 3, the
   2D trial p = -(sxx + syy) / 2.  beta (state[5]) records -p / (K dt) on the
   dilute branch.  state[9] accumulates the plastic strain, state[10] holds
   its rate. */
static void plane_return_range(orc_sim *s, size_t p0, size_t p1, int trial3d, int mu_i, int with_beta)
{
    const double G = s->G, K = s->K, dt = s->c.dt;
    const double *mp = s->c.mp;
    const double lambda = K - 2.0 * G / 3.0;
    for (size_t i = p0; i < p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double trD = s->exx[i] + s->eyy[i];
        double dsjxx = lambda * trD + 2.0 * G * s->exx[i];
        double dsjxy = 2.0 * G * s->exy[i];
        double dsjyy = lambda * trD + 2.0 * G * s->eyy[i];
        dsjxx += 2 * s->wxy[i] * s->sxy[i];
        dsjxy -= s->wxy[i] * (s->sxx[i] - s->syy[i]);
        dsjyy -= 2 * s->wxy[i] * s->sxy[i];
        double sxx_tr = s->sxx[i] + dt * dsjxx;
        double sxy_tr = s->sxy[i] + dt * dsjxy;
        double syy_tr = s->syy[i] + dt * dsjyy;
        double szz_tr = 0, p_tr, t0zz = 0, tau_tr;
        if (trial3d) {
            szz_tr = st[1] + dt * lambda * trD;
            p_tr = -(sxx_tr + syy_tr + szz_tr) / 3.0;
        } else {
            p_tr = -0.5 * (sxx_tr + syy_tr);
        }
        double t0xx = sxx_tr + p_tr;
        double t0xy = sxy_tr;
        double t0yy = syy_tr + p_tr;
        if (trial3d) {
            t0zz = szz_tr + p_tr;
            tau_tr = sqrt(0.5 * (t0xx * t0xx + 2 * t0xy * t0xy + t0yy * t0yy + t0zz * t0zz));
        } else {
            tau_tr = sqrt(0.5 * (t0xx * t0xx + 2 * t0xy * t0xy + t0yy * t0yy));
        }
        int density_flag = (s->m[i] / s->v[i]) < mp[ORC_MP_RHO_CRITICAL];
        double nup_tau;
        if (density_flag || p_tr <= 0) {
            nup_tau = tau_tr / (G * dt);
            if (with_beta) {
                st[5] = -p_tr / (K * dt);
            }
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
            if (trial3d) {
                st[1] = 0;
            }
        } else if (p_tr > 0) {
            double S0 = mp[ORC_MP_MU_S] * p_tr;
            double tau_tau, scale_factor;
            if (tau_tr <= S0) {
                tau_tau = tau_tr;
                scale_factor = 1.0;
            } else if (mu_i) {
                double S2 = mp[ORC_MP_MU_2] * p_tr;
                double alpha = G * mp[ORC_MP_I0] * dt * sqrt(p_tr / mp[ORC_MP_GRAINS_RHO])
                               / mp[ORC_MP_GRAINS_D];
                double B = -(S2 + tau_tr + alpha);
                double H = S2 * tau_tr + S0 * alpha;
                tau_tau = negative_root(1.0, B, H);
                scale_factor = (tau_tau / tau_tr);
            } else {
                tau_tau = S0;
                scale_factor = tau_tau / tau_tr;
            }
            nup_tau = ((tau_tr - tau_tau) / G) / dt;
            if (with_beta) {
                st[5] = 0;
            }
            s->sxx[i] = scale_factor * t0xx - p_tr;
            s->sxy[i] = scale_factor * t0xy;
            s->syy[i] = scale_factor * t0yy - p_tr;
            if (trial3d) {
                st[1] = scale_factor * t0zz - p_tr;
            }
        } else {
            nup_tau = 0;   /* p_tr is NaN */
        }
        st[9] += nup_tau * dt;
        st[10] = nup_tau;
    }
}

static int plane_return_material(int material, size_t p0, size_t p1, orc_sim *s)
{
    switch (material) {
    case ORC_DP_RI_MT:
        plane_return_range(s, p0, p1, 1, 0, 0);
        return 1;
    case ORC_G_LOCAL_MU2_PLANE_STRAIN:
        plane_return_range(s, p0, p1, 1, 1, 1);
        return 1;
    case ORC_G_LOCAL_MU2_TRUE_2D:
        plane_return_range(s, p0, p1, 0, 1, 1);
        return 1;
    default:
        return 0;
    }
}

/* mu_from_gammadot, g_local_mu2_ext.c:75-95 */
static double mu_from_gammadot(double gammadot, double p, double dsqrtrhos, double mu_s, double mu_2,
                               double inum_0)
{
    double mu;
    if (p <= 0) {
        mu = mu_2;
    } else {
        double inum = dsqrtrhos * gammadot / sqrt(p);
        if (inum <= 0) {
            mu = mu_s;
        } else {
            mu = mu_s + (mu_2 - mu_s) / ((inum_0 / inum) + 1.0);
        }
    }
    return mu;
}

/* g_local_mu2_ext calculate_stress_threaded, g_local_mu2_ext.c:165-368, run
   by every thread of the team.  Three phases separated by team barriers:
   (1) the local fluidity gammadotp / mu_t from the start-of-step pressure
   (state[0] mu_t, state[4] gflocal); (2) per colour, each particle adds
   -v gflocal |grad N_j|^2 to its element's nodes (the team's per-(thread,
   colour) lists, a barrier per colour), then gf = A^2 d^2 mu_t times the
   element average (state[3]) lowers gammadotp where mu_t > mu_s; (3) a
   plane-stress elastic trial with the Jaumann terms, returned to
   mu(gammadotp) (p + c) with c = 1e-2.  Node values live in gf_nodes. */
static void g_local_mu2_ext_thread(orc_task *task)
{
    orc_sim *s = task->s;
    const double *mp = s->c.mp;
    const double E = mp[ORC_MP_E], nu = mp[ORC_MP_NU], G = s->G, K = s->K, dt = s->c.dt;
    const double mu_s = mp[ORC_MP_MU_S], mu_2 = mp[ORC_MP_MU_2], I0 = mp[ORC_MP_I0];
    const double d = mp[ORC_MP_GRAINS_D], Acoef = mp[ORC_MP_A];
    const double dsqrtrhos = d * sqrt(mp[ORC_MP_GRAINS_RHO]);
    const double c = 1e-2;
    double *d2 = s->gf_nodes;

    for (size_t i = task->n0; i < task->n1; i++) {
        d2[i] = 0;
    }
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double p_t = -0.5 * (s->sxx[i] + s->syy[i]);
        if (st[10] == 0) {
            st[4] = 0;
        } else {
            st[0] = mu_from_gammadot(st[10], p_t, dsqrtrhos, mu_s, mu_2, I0);
            st[4] = st[10] / st[0];
        }
    }
    pthread_barrier_wait(&s->bar);

    for (int cc = 0; cc < NCOLORS; cc++) {
        size_t tc = task->id * NCOLORS + (size_t)cc;
        for (size_t k = 0; k < s->list_len[tc]; k++) {
            size_t i = s->lists[tc][k];
            const int *nn = s->enodes + 4 * s->in_element[i];
            double sj[4];
            sj[0] = s->b11[i] * s->b11[i] + s->b21[i] * s->b21[i];
            sj[1] = s->b12[i] * s->b12[i] + s->b22[i] * s->b22[i];
            sj[2] = s->b13[i] * s->b13[i] + s->b23[i] * s->b23[i];
            sj[3] = s->b14[i] * s->b14[i] + s->b24[i] * s->b24[i];
            for (int j = 0; j < 4; j++) {
                d2[nn[j]] += -s->v[i] * s->state[DEPVAR * i + 4] * sj[j];
            }
        }
        pthread_barrier_wait(&s->bar);
    }

    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        const int *nn = s->enodes + 4 * s->in_element[i];
        st[3] = 0;
        for (int j = 0; j < 4; j++) {
            st[3] += 0.25 * d2[nn[j]];
        }
        st[3] = Acoef * Acoef * d * d * st[0] * st[3];
        if (st[0] > mu_s) {
            st[10] = st[10] - (st[3] / fabs(st[0] - mu_s));
        }
        if (st[10] < 0) {
            st[10] = 0;
        }
    }
    pthread_barrier_wait(&s->bar);

    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double p_t = -0.5 * (s->sxx[i] + s->syy[i]);
        double dsjxx = dt * (E / (1 - nu * nu)) * ((s->exx[i]) + nu * (s->eyy[i]));
        double dsjxy = dt * (E / (2 * (1 + nu))) * (s->exy[i]);
        double dsjyy = dt * (E / (1 - nu * nu)) * ((s->eyy[i]) + nu * (s->exx[i]));
        dsjxx -= 2 * dt * s->wxy[i] * s->sxy[i];
        dsjxy += dt * s->wxy[i] * (s->sxx[i] - s->syy[i]);
        dsjyy += 2 * dt * s->wxy[i] * s->sxy[i];
        double sxx_tr = s->sxx[i] + dsjxx;
        double sxy_tr = s->sxy[i] + dsjxy;
        double syy_tr = s->syy[i] + dsjyy;
        double p_tr = -0.5 * (sxx_tr + syy_tr);
        double t0xx = sxx_tr + p_tr;
        double t0xy = sxy_tr;
        double t0yy = syy_tr + p_tr;
        double tau_tr = sqrt(0.5 * (t0xx * t0xx + 2 * t0xy * t0xy + t0yy * t0yy));
        st[0] = mu_from_gammadot(st[10], p_t, dsqrtrhos, mu_s, mu_2, I0);
        double tau_tau = st[0] * (p_tr + c);
        double f = tau_tr - tau_tau;
        int density_flag = (s->m[i] / s->v[i]) < mp[ORC_MP_RHO_CRITICAL];
        double nup_tau;
        if (density_flag) {
            nup_tau = (tau_tr) / (G * dt);
            st[5] = -p_tr / (K * dt);
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
        } else if (f < 0) {
            nup_tau = 0;
            st[5] = 0;
            s->sxx[i] = t0xx - p_tr;
            s->sxy[i] = t0xy;
            s->syy[i] = t0yy - p_tr;
        } else if (f >= 0 && p_tr > -c / st[0]) {
            nup_tau = (tau_tr - tau_tau) / (G * dt);
            st[5] = 0;
            double scale_factor = (tau_tau / tau_tr);
            s->sxx[i] = scale_factor * t0xx - p_tr;
            s->sxy[i] = scale_factor * t0xy;
            s->syy[i] = scale_factor * t0yy - p_tr;
        } else if (p_tr <= -c / st[0]) {
            nup_tau = tau_tr / (G * dt);
            st[5] = ((c / st[0]) - p_tr) / (K * dt);
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
        } else {
            nup_tau = 0;   /* NaN: the reference prints the particle and keeps s */
        }
        st[9] += nup_tau * dt;
        st[10] = nup_tau;
    }
}

/* g_local_mu2_reverse calculate_stress_threaded, g_local_mu2_reverse.c:166-302:
   a rate-dependent return to mu(I) (p + c), c = 0, with mu from the previous
   step's gammadotp and start-of-step pressure, and the Jaumann terms of the
   opposite sign to isolin's.  beta in state[5]. */
static void g_local_mu2_reverse_range(orc_sim *s, size_t p0, size_t p1)
{
    const double G = s->G, K = s->K, dt = s->c.dt;
    const double *mp = s->c.mp;
    const double lambda = K - 2.0 * G / 3.0;
    const double c = 0;
    for (size_t i = p0; i < p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double p_t = -0.5 * (s->sxx[i] + s->syy[i]);
        double trD = s->exx[i] + s->eyy[i];
        double dsjxx = lambda * trD + 2.0 * G * s->exx[i];
        double dsjxy = 2.0 * G * s->exy[i];
        double dsjyy = lambda * trD + 2.0 * G * s->eyy[i];
        dsjxx -= 2 * s->wxy[i] * s->sxy[i];
        dsjxy += s->wxy[i] * (s->sxx[i] - s->syy[i]);
        dsjyy += 2 * s->wxy[i] * s->sxy[i];
        double sxx_tr = s->sxx[i] + dt * dsjxx;
        double sxy_tr = s->sxy[i] + dt * dsjxy;
        double syy_tr = s->syy[i] + dt * dsjyy;
        double p_tr = -0.5 * (sxx_tr + syy_tr);
        double t0xx = sxx_tr + p_tr;
        double t0xy = sxy_tr;
        double t0yy = syy_tr + p_tr;
        double tau_tr = sqrt(0.5 * (t0xx * t0xx + 2 * t0xy * t0xy + t0yy * t0yy));
        double inertial_num = st[10] * mp[ORC_MP_GRAINS_D] * sqrt(mp[ORC_MP_GRAINS_RHO]);
        double mu_t;
        if (p_t <= 0) {
            mu_t = mp[ORC_MP_MU_2];
        } else {
            inertial_num = inertial_num / sqrt(p_t);
            if (inertial_num <= 0) {
                mu_t = mp[ORC_MP_MU_S];
            } else {
                mu_t = mp[ORC_MP_MU_S] + (mp[ORC_MP_MU_2] - mp[ORC_MP_MU_S]) / ((mp[ORC_MP_I0] / inertial_num) + 1.0);
            }
        }
        double tau_tau = mu_t * (p_tr + c);
        double f = tau_tr - tau_tau;
        int density_flag = (s->m[i] / s->v[i]) < mp[ORC_MP_RHO_CRITICAL];
        double nup_tau;
        if (density_flag) {
            nup_tau = (tau_tr) / (G * dt);
            st[5] = -p_tr / (K * dt);
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
        } else if (f < 0) {
            nup_tau = 0;
            st[5] = 0;
            s->sxx[i] = t0xx - p_tr;
            s->sxy[i] = t0xy;
            s->syy[i] = t0yy - p_tr;
        } else if (f >= 0 && p_tr > -c / mu_t) {
            nup_tau = (f / G) / dt;
            st[5] = 0;
            double scale_factor = (tau_tau / tau_tr);
            s->sxx[i] = scale_factor * t0xx - p_tr;
            s->sxy[i] = scale_factor * t0xy;
            s->syy[i] = scale_factor * t0yy - p_tr;
        } else if (p_tr <= -c / mu_t) {
            nup_tau = tau_tr / (G * dt);
            st[5] = ((c / mu_t) - p_tr) / (K * dt);
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
        } else {
            nup_tau = 0;   /* NaN: the reference prints the particle and keeps s */
        }
        st[9] += nup_tau * dt;
        st[10] = nup_tau;
    }
}

/* Trial Jaumann stress shared by g_nonlocal_mu2.c:166-186 and :271-290. */
static void nonlocal_mu2_trial(const orc_sim *s, size_t i, double *p_tr, double *t0xx,
                               double *t0xy, double *t0yy, double *tau_tr)
{
    const double G = s->G, dt = s->c.dt;
    const double lambda = s->K - 2.0 * G / 3.0;
    double trD = s->exx[i] + s->eyy[i];
    double dsjxx = lambda * trD + 2.0 * G * s->exx[i];
    double dsjxy = 2.0 * G * s->exy[i];
    double dsjyy = lambda * trD + 2.0 * G * s->eyy[i];
    dsjxx += 2 * s->wxy[i] * s->sxy[i];
    dsjxy -= s->wxy[i] * (s->sxx[i] - s->syy[i]);
    dsjyy -= 2 * s->wxy[i] * s->sxy[i];
    double sxx_tr = s->sxx[i] + dt * dsjxx;
    double sxy_tr = s->sxy[i] + dt * dsjxy;
    double syy_tr = s->syy[i] + dt * dsjyy;
    *p_tr = -0.5 * (sxx_tr + syy_tr);
    *t0xx = sxx_tr + *p_tr;
    *t0xy = sxy_tr;
    *t0yy = syy_tr + *p_tr;
    *tau_tr = sqrt(0.5 * (*t0xx * *t0xx + 2 * *t0xy * *t0xy + *t0yy * *t0yy));
}

/* calculate_bulk_granular_fluidity, g_nonlocal_mu2.c:238-321 */
static void nonlocal_mu2_bulk(orc_sim *s)
{
    const double G = s->G, dt = s->c.dt;
    const double *mp = s->c.mp;
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double p_tr, t0xx, t0xy, t0yy, tau_tr;
        nonlocal_mu2_trial(s, i, &p_tr, &t0xx, &t0xy, &t0yy, &tau_tr);
        if ((s->m[i] / s->v[i]) < mp[ORC_MP_RHO_CRITICAL] || p_tr < 0) {
            st[0] = 0;
        } else {
            st[0] = 1;
        }
        if (st[0] == 0 || p_tr <= 0) {
            st[5] = 0;
            st[6] = 0;
        } else if (p_tr > 0) {
            double tau_tau, scale_factor;
            double S0 = mp[ORC_MP_MU_S] * p_tr;
            if (tau_tr <= S0) {
                tau_tau = tau_tr;
                scale_factor = 1.0;
            } else {
                double S2 = mp[ORC_MP_MU_2] * p_tr;
                double alpha = G * mp[ORC_MP_I0] * dt * sqrt(p_tr / mp[ORC_MP_GRAINS_RHO])
                               / mp[ORC_MP_GRAINS_D];
                double B = -(S2 + tau_tr + alpha);
                double H = S2 * tau_tr + S0 * alpha;
                tau_tau = negative_root(1.0, B, H);
                scale_factor = (tau_tau / tau_tr);
            }
            st[5] = (p_tr / (G * dt)) * ((1.0 / scale_factor) - 1.0);
            st[6] = fabs((tau_tau / p_tr) - mp[ORC_MP_MU_S])
                    / (mp[ORC_MP_A] * mp[ORC_MP_A] * mp[ORC_MP_GRAINS_D] * mp[ORC_MP_GRAINS_D]);
        } else {
            st[5] = 0;
            st[6] = 0;
        }
    }
}

/* calculate_bulk_granular_fluidity, g_nonlocal.c:306-352 (all particles) */
static void nonlocal_bulk(orc_sim *s)
{
    const double *mp = s->c.mp;
    const double p_cap = 1e-2;
    for (size_t i = 0; i < s->np; i++) {
        double *st = s->state + DEPVAR * i;
        double p_t = -0.5 * (s->sxx[i] + s->syy[i]);
        double sxx_tr0 = s->sxx[i] + p_t;
        double sxy_tr0 = s->sxy[i];
        double syy_tr0 = s->syy[i] + p_t;
        double tau_t = sqrt(0.5 * (sxx_tr0 * sxx_tr0 + 2 * sxy_tr0 * sxy_tr0 + syy_tr0 * syy_tr0));
        if (p_t < p_cap) {
            p_t = p_cap;
        }
        double S0 = p_t * mp[ORC_MP_MU_S];
        st[4] = mp[ORC_MP_B] * mp[ORC_MP_GRAINS_D] * sqrt(p_t * mp[ORC_MP_GRAINS_RHO]);
        st[10] = fabs(tau_t / p_t - mp[ORC_MP_MU_S])
                 / (mp[ORC_MP_GRAINS_D] * mp[ORC_MP_GRAINS_D] * mp[ORC_MP_A] * mp[ORC_MP_A]);
        if (tau_t > S0) {
            st[5] = (p_t / st[4]) * (1 - S0 / tau_t);
        } else {
            st[5] = 0;
        }
    }
}

/*
 * solve_diffusion_part: g_nonlocal_mu2.c:325-578 (dense particles only, plus a
 * 1e-10 diagonal) and g_nonlocal.c:356-592 (all active particles, no shift).
 * Unknowns are nodes with m > tol, numbered in ascending node order.
 */
static int nonlocal_solve(orc_sim *s, int mu2)
{
    const double tol = mu2 ? 0.0 : 1e-10;
    const int gf_local_slot = 5;
    const int xisq_slot = mu2 ? 6 : 10;
    long slda = 0;
    for (size_t i = 0; i < s->nn; i++) {
        s->node_map[i] = -1;
        s->gf_nodes[i] = 0;
    }
    for (size_t i = 0; i < s->nn; i++) {
        if (s->nm[i] > tol) {
            s->node_map[i] = slda++;
        }
    }
    if (slda == 0) {
        return 3;
    }
    long w = (long)s->c.Nx + 1;
    if (w > slda - 1) {
        w = slda - 1 > 0 ? slda - 1 : 0;
    }
    double *f = dalloc((size_t)slda);
    double *band = NULL;
    double *stencil = NULL;         /* PCG: 9 couplings per unknown (3x3 node block) */
    if (s->c.solver == ORC_SOLVER_DIRECT) {
        band = dalloc((size_t)slda * (size_t)(w + 1));
    } else {
        stencil = dalloc((size_t)slda * 9);
    }

    /* RHS, g_nonlocal_mu2.c:418-452 */
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        const double *st = s->state + DEPVAR * i;
        if (mu2 && st[0] == 0) {
            continue;
        }
        int p = s->in_element[i];
        if (p == -1) {
            continue;
        }
        double sv[4] = {s->h1[i], s->h2[i], s->h3[i], s->h4[i]};
        const int *nn = s->enodes + 4 * p;
        for (int ei = 0; ei < 4; ei++) {
            long sgi = s->node_map[nn[ei]];
            if (sgi < 0) {
                continue;
            }
            f[sgi] += (s->v[i]) * st[gf_local_slot] * st[xisq_slot] * sv[ei];
        }
    }

    /* Stiffness, g_nonlocal_mu2.c:455-507; summed per entry in particle order
       like cs_compress + cs_dupl do. */
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        const double *st = s->state + DEPVAR * i;
        if (mu2 && st[0] == 0) {
            continue;
        }
        int p = s->in_element[i];
        if (p == -1) {
            continue;
        }
        double sv[4] = {s->h1[i], s->h2[i], s->h3[i], s->h4[i]};
        double gs[4][2] = {{s->b11[i], s->b21[i]}, {s->b12[i], s->b22[i]},
                           {s->b13[i], s->b23[i]}, {s->b14[i], s->b24[i]}};
        const int *nn = s->enodes + 4 * p;
        double xisq = st[xisq_slot];
        for (int ei = 0; ei < 4; ei++) {
            for (int ej = 0; ej < 4; ej++) {
                long sgi = s->node_map[nn[ei]], sgj = s->node_map[nn[ej]];
                if (sgi < 0 || sgj < 0) {
                    continue;
                }
                double val = s->v[i] * (xisq * sv[ei] * sv[ej]
                                        + (gs[ei][0] * gs[ej][0] + gs[ei][1] * gs[ej][1]));
                if (band != NULL) {
                    if (sgi >= sgj) {
                        band[(size_t)sgi * (size_t)(w + 1) + (size_t)(sgj - sgi + w)] += val;
                    }
                } else {
                    /* neighbour slot from the node offset: dx, dy in {-1,0,1} */
                    int dx = (nn[ej] % s->c.Nx) - (nn[ei] % s->c.Nx);
                    int dy = (nn[ej] / s->c.Nx) - (nn[ei] / s->c.Nx);
                    stencil[(size_t)sgi * 9 + (size_t)((dy + 1) * 3 + (dx + 1))] += val;
                }
            }
        }
    }
    if (mu2) {
        for (long k = 0; k < slda; k++) {
            if (band != NULL) {
                band[(size_t)k * (size_t)(w + 1) + (size_t)w] += 1e-10;
            } else {
                stencil[(size_t)k * 9 + 4] += 1e-10;
            }
        }
    }

    int status = 0;
    if (band != NULL) {
        if (!oracle_band_ldlt_solve(slda, w, band, f)) {
            status = 2;      /* EXIT_ERROR_CS_SOL, exitcodes.h:14 */
        }
        s->solve_iters = 0;
        s->solve_resid = 0;
    } else {
        /* Jacobi-preconditioned CG on the 9-point coupling rows. */
        long *inv = (long *)malloc(sizeof(long) * (size_t)slda);
        for (size_t i = 0; i < s->nn; i++) {
            if (s->node_map[i] >= 0) {
                inv[s->node_map[i]] = (long)i;
            }
        }
        double *xv = dalloc((size_t)slda), *r = dalloc((size_t)slda), *z = dalloc((size_t)slda);
        double *pv = dalloc((size_t)slda), *q = dalloc((size_t)slda);
        double *pn = dalloc(s->nn);
        double bnorm = 0;
        for (long k = 0; k < slda; k++) {
            r[k] = f[k];
            bnorm += f[k] * f[k];
        }
        bnorm = sqrt(bnorm);
        double rz = 0;
        for (long k = 0; k < slda; k++) {
            double d = stencil[(size_t)k * 9 + 4];
            z[k] = r[k] / d;
            pv[k] = z[k];
            rz += r[k] * z[k];
        }
        int it = 0;
        double rn = bnorm;
        if (bnorm > 0) {
            for (it = 0; it < s->c.cg_maxit; it++) {
                for (long k = 0; k < slda; k++) {
                    pn[inv[k]] = pv[k];
                }
                double pq = 0;
                for (long k = 0; k < slda; k++) {
                    long node = inv[k];
                    int ix = (int)(node % s->c.Nx), iy = (int)(node / s->c.Nx);
                    double acc = 0;
                    for (int dy = -1; dy <= 1; dy++) {
                        for (int dx = -1; dx <= 1; dx++) {
                            double a = stencil[(size_t)k * 9 + (size_t)((dy + 1) * 3 + (dx + 1))];
                            if (a != 0.0) {
                                acc += a * pn[(size_t)(iy + dy) * (size_t)s->c.Nx + (size_t)(ix + dx)];
                            }
                        }
                    }
                    q[k] = acc;
                    pq += pv[k] * acc;
                }
                double alpha = rz / pq;
                double rz_new = 0, rr = 0;
                for (long k = 0; k < slda; k++) {
                    xv[k] += alpha * pv[k];
                    r[k] -= alpha * q[k];
                    z[k] = r[k] / stencil[(size_t)k * 9 + 4];
                    rz_new += r[k] * z[k];
                    rr += r[k] * r[k];
                }
                rn = sqrt(rr);
                if (rn <= s->c.cg_tol * bnorm) {
                    it++;
                    break;
                }
                double beta = rz_new / rz;
                rz = rz_new;
                for (long k = 0; k < slda; k++) {
                    pv[k] = z[k] + beta * pv[k];
                }
            }
        }
        for (long k = 0; k < slda; k++) {
            f[k] = xv[k];
        }
        s->solve_iters = it;
        s->solve_resid = bnorm > 0 ? rn / bnorm : 0;
        if (!(s->solve_resid <= s->c.cg_tol) && bnorm > 0) {
            status = 2;
        }
        free(inv); free(xv); free(r); free(z); free(pv); free(q); free(pn);
    }

    /* g_nonlocal_mu2.c:521-564: nodal fluidity, then G2P to the particles. */
    for (size_t i = 0; i < s->nn; i++) {
        if (s->node_map[i] != -1) {
            s->gf_nodes[i] = f[s->node_map[i]];
        }
    }
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        int p = s->in_element[i];
        if (p == -1) {
            continue;
        }
        double sv[4] = {s->h1[i], s->h2[i], s->h3[i], s->h4[i]};
        const int *nn = s->enodes + 4 * p;
        double gf = 0;
        for (int ei = 0; ei < 4; ei++) {
            if (s->c.material == ORC_G_NONLOCAL_AVG) {
                gf += 0.25 * s->gf_nodes[nn[ei]];    /* g_nonlocal_avg.c:575-578 */
            } else {
                gf += s->gf_nodes[nn[ei]] * sv[ei];
            }
        }
        s->state[DEPVAR * i + 3] = gf;
    }
    free(f);
    free(band);
    free(stencil);
    return status;
}

/* calculate_stress, g_nonlocal_mu2.c:126-221 */
static int g_nonlocal_mu2_stress(orc_sim *s)
{
    const double G = s->G, dt = s->c.dt;
    nonlocal_mu2_bulk(s);
    int status = nonlocal_solve(s, 1);
    for (size_t i = 0; i < s->np; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double *st = s->state + DEPVAR * i;
        double p_tr, t0xx, t0xy, t0yy, tau_tr, nup_tau;
        nonlocal_mu2_trial(s, i, &p_tr, &t0xx, &t0xy, &t0yy, &tau_tr);
        if (st[0] == 0 || p_tr <= 0) {
            nup_tau = 0;
            s->sxx[i] = 0;
            s->sxy[i] = 0;
            s->syy[i] = 0;
        } else if (p_tr > 0) {
            double scale_factor = p_tr / (G * dt * st[3] + p_tr);
            double tau_tau = tau_tr * scale_factor;
            nup_tau = ((tau_tr - tau_tau) / G) / dt;
            s->sxx[i] = scale_factor * t0xx - p_tr;
            s->sxy[i] = scale_factor * t0xy;
            s->syy[i] = scale_factor * t0yy - p_tr;
        } else {
            nup_tau = 0;
        }
        st[9] += nup_tau * dt;
        st[10] = nup_tau;
    }
    return status;
}

/* calculate_stress, g_nonlocal.c:103-301 (all particles, explicit update) */
static int g_nonlocal_stress(orc_sim *s)
{
    const double *mp = s->c.mp;
    const double EMOD = mp[ORC_MP_E], NUMOD = mp[ORC_MP_NU], MU_S = mp[ORC_MP_MU_S];
    const double G = s->G, dt = s->c.dt, c = mp[ORC_MP_COHESION];
    nonlocal_bulk(s);
    int status = nonlocal_solve(s, 0);
    for (size_t i = 0; i < s->np; i++) {
        double *st = s->state + DEPVAR * i;
        double gf = st[3];
        double sxx = s->sxx[i], sxy = s->sxy[i], syy = s->syy[i];
        double exx = s->exx[i], exy = s->exy[i], eyy = s->eyy[i], wxy = s->wxy[i];
        double p_t = -0.5 * (sxx + syy);
        double sxx_t0 = sxx + p_t, sxy_t0 = sxy, syy_t0 = syy + p_t;
        double tau_t = sqrt(0.5 * (sxx_t0 * sxx_t0 + 2 * sxy_t0 * sxy_t0 + syy_t0 * syy_t0));

        double dsjxx = dt * (EMOD / (1 - NUMOD * NUMOD)) * ((exx) + NUMOD * (eyy));
        double dsjxy = dt * (EMOD / (2 * (1 + NUMOD))) * (exy);
        double dsjyy = dt * (EMOD / (1 - NUMOD * NUMOD)) * ((eyy) + NUMOD * (exx));
        dsjxx -= 2 * dt * wxy * sxy;
        dsjxy += dt * wxy * (sxx - syy);
        dsjyy += 2 * dt * wxy * sxy;
        double sxx_tr = sxx + dsjxx, syy_tr = syy + dsjyy;
        double p_tr = -0.5 * (sxx_tr + syy_tr);
        if (p_tr < c) {
            s->sxx[i] = 0.5 * c / MU_S;
            s->sxy[i] = 0;
            s->syy[i] = 0.5 * c / MU_S;
            continue;
        }
        /* g_nonlocal.c:170-213 compute a trial flow direction and rate that
           the explicit update below overwrites; they have no effect. */
        p_t = -0.5 * (sxx + syy);
        sxx_t0 = sxx + p_t;
        sxy_t0 = sxy;
        syy_t0 = syy + p_t;
        tau_t = sqrt(0.5 * (sxx_t0 * sxx_t0 + 2 * sxy_t0 * sxy_t0 + syy_t0 * syy_t0));
        double Npxx = sqrt(0.5) * sxx_t0 / tau_t;
        double Npxy = sqrt(0.5) * sxy_t0 / tau_t;
        double Npyy = sqrt(0.5) * syy_t0 / tau_t;
        double dxx0 = 0.5 * (exx - eyy), dxy0 = exy, dyy0 = 0.5 * (eyy - exx);
        double gammadot = sqrt(2 * (dxx0 * dxx0 + 2 * dxy0 * dxy0 + dyy0 * dyy0));
        double nup_tau, dpxx, dpxy, dpyy;
        if (p_t > c && gf > 0) {
            nup_tau = gf * tau_t / p_t;
            if (nup_tau < 0) {
                nup_tau = 0;
            }
            if (nup_tau > gammadot) {
                nup_tau = gammadot;
            }
            dpxx = sqrt(0.5) * (nup_tau) * Npxx;
            dpxy = sqrt(0.5) * (nup_tau) * Npxy;
            dpyy = sqrt(0.5) * (nup_tau) * Npyy;
        } else {
            nup_tau = 0;
            dpxx = 0;
            dpxy = 0;
            dpyy = 0;
        }
        if (s->t == 0) {
            nup_tau = 0;
            dpxx = 0;
            dpxy = 0;
            dpyy = 0;
        }
        dsjxx = dt * (EMOD / (1 - NUMOD * NUMOD)) * ((exx - dpxx) + NUMOD * (eyy - dpyy));
        dsjxy = dt * (EMOD / (2 * (1 + NUMOD))) * (exy - dpxy);
        dsjyy = dt * (EMOD / (1 - NUMOD * NUMOD)) * ((eyy - dpyy) + NUMOD * (exx - dpxx));
        dsjxx -= 2 * dt * wxy * sxy;
        dsjxy += dt * wxy * (sxx - syy);
        dsjyy += 2 * dt * wxy * sxy;
        st[9] += nup_tau * dt;
        s->sxx[i] += dsjxx;
        s->sxy[i] += dsjxy;
        s->syy[i] += dsjyy;
    }
    (void)G;
    return status;
}

/*---------------------------------------------------------------------------*/
/* map_to_grid_explicit_split (process_usl.c:812-910; map.c:85-104): each
   thread adds its (thread, colour) list's particles to the nodes, with a
   barrier after each colour. */
static void p2g_by_colour(orc_task *task)
{
    orc_sim *s = task->s;
    for (int c = 0; c < NCOLORS; c++) {
        size_t tc = task->id * NCOLORS + (size_t)c;
        for (size_t k = 0; k < s->list_len[tc]; k++) {
            size_t i = s->lists[tc][k];
            const int *nn = s->enodes + 4 * s->in_element[i];
            double sv[4] = {s->h1[i], s->h2[i], s->h3[i], s->h4[i]};
            double pdata[7];
            pdata[0] = s->m[i];
            pdata[1] = s->vx[i] * s->m[i];
            pdata[2] = s->vy[i] * s->m[i];
            pdata[3] = s->ax[i] * s->m[i];
            pdata[4] = s->ay[i] * s->m[i];
            pdata[5] = s->bx[i] * s->m[i];
            pdata[6] = s->by[i] * s->m[i];
            double sd[3];
            sd[0] = -s->sxx[i] * s->v[i];
            sd[1] = -s->sxy[i] * s->v[i];
            sd[2] = -s->syy[i] * s->v[i];
            for (int a = 0; a < 4; a++) {
                int nd = nn[a];
                s->nm[nd] += sv[a] * pdata[0];
                s->nmx[nd] += sv[a] * pdata[1];
                s->nmy[nd] += sv[a] * pdata[2];
                s->nmxx[nd] += sv[a] * pdata[3];
                s->nmyy[nd] += sv[a] * pdata[4];
                s->nfx[nd] += sv[a] * pdata[5];
                s->nfy[nd] += sv[a] * pdata[6];
            }
            double d1[4] = {s->b11[i], s->b12[i], s->b13[i], s->b14[i]};
            for (int a = 0; a < 4; a++) {
                s->nfx[nn[a]] += d1[a] * sd[0];
                s->nfy[nn[a]] += d1[a] * sd[1];
            }
            double d2[4] = {s->b21[i], s->b22[i], s->b23[i], s->b24[i]};
            for (int a = 0; a < 4; a++) {
                s->nfx[nn[a]] += d2[a] * sd[1];
                s->nfy[nn[a]] += d2[a] * sd[2];
            }
        }
        pthread_barrier_wait(&s->bar);
    }

}

/* Thread-team phases of explicit_mpm_step_usl_threaded, process_usl.c:465-592. */

static void step_thread(orc_task *task)
{
    orc_sim *s = task->s;
    const size_t Nx = (size_t)s->c.Nx;
    const double h = s->c.h, dt = s->c.dt;

    pthread_barrier_wait(&s->bar);

    /* clear grid, process_usl.c:484-504 */
    for (size_t i = task->n0; i < task->n1; i++) {
        s->nm[i] = 0; s->nmx[i] = 0; s->nmy[i] = 0; s->nmxx[i] = 0; s->nmyy[i] = 0;
        s->nvx[i] = 0; s->nvy[i] = 0; s->nax[i] = 0; s->nay[i] = 0; s->nfx[i] = 0;
        s->nfy[i] = 0; s->nux[i] = 0; s->nuy[i] = 0;
    }
    for (size_t e = task->e0; e < task->e1; e++) {
        s->efilled[e] = 0;
        s->en[e] = 0;
        s->em[e] = 0;
    }

    /* element map, process_usl.c:631-674 */
    int changed = 0;
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        int p = which_element(s, s->x[i], s->y[i]);
        if (p != s->in_element[i]) {
            changed = 1;
        }
        s->in_element[i] = p;
        if (p == -1) {
            s->active[i] = 0;
        }
    }
    s->update_flags[task->id] = changed;

    /* shape functions, process_usl.c:727-760; particle.c:14-30;
       interpolate.c:23-65 */
    const double dxl_dx = 1.0 / h;
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        int p = s->in_element[i];
        int n = s->enodes[4 * p];
        double xl = (s->x[i] - s->nx[n]) / h;
        double sg = copysign(1.0, xl);
        if ((sg * xl) > 1.0f && ((sg * xl) - 1.0f) < TOL) {
            xl = sg;
        }
        double yl = (s->y[i] - s->ny[n]) / h;
        sg = copysign(1.0, yl);
        if ((sg * yl) > 1.0f && ((sg * yl) - 1.0f) < TOL) {
            yl = sg;
        }
        s->h1[i] = (1 - xl) * (1 - yl);
        s->h2[i] = (xl) * (1 - yl);
        s->h3[i] = (xl) * (yl);
        s->h4[i] = (1 - xl) * (yl);
        s->b11[i] = -(1 - yl) * dxl_dx;
        s->b12[i] = (1 - yl) * dxl_dx;
        s->b13[i] = (yl) * dxl_dx;
        s->b14[i] = -(yl) * dxl_dx;
        s->b21[i] = -(1 - xl) * dxl_dx;
        s->b22[i] = -(xl) * dxl_dx;
        s->b23[i] = (xl) * dxl_dx;
        s->b24[i] = (1 - xl) * dxl_dx;
        s->xl[i] = xl;
        s->yl[i] = yl;
    }

    /* serial: time, element lists, BC masks, process_usl.c:519-546 */
    if (pthread_barrier_wait(&s->bar) == PTHREAD_BARRIER_SERIAL_THREAD) {
        s->t += dt;
        int flag = 0;
        for (size_t i = 0; i < s->T_threads; i++) {
            flag += s->update_flags[i];
        }
        if (flag != 0) {
            find_filled_elements(s);
        }
        generate_dirichlet_bcs(s);
    }
    pthread_barrier_wait(&s->bar);

    /* P2G by colour, process_usl.c:812-910; map.c:85-104 */
    p2g_by_colour(task);

    /* serial: bc_momentum, bc_force, process_usl.c:552-567; box.c:183-224 */
    if (pthread_barrier_wait(&s->bar) == PTHREAD_BARRIER_SERIAL_THREAD) {
        for (size_t i = 0; i < s->nn; i++) {
            if (s->mask[3 * i + 0]) s->nmx[i] = 0;
            if (s->mask[3 * i + 1]) s->nmy[i] = 0;
        }
        for (size_t i = 0; i < s->nn; i++) {
            if (s->mask[3 * i + 0]) s->nfx[i] = 0;
            if (s->mask[3 * i + 1]) s->nfy[i] = 0;
        }
    }
    pthread_barrier_wait(&s->bar);

    /* move_grid_split, process_usl.c:596-625 */
    for (size_t i = task->n0; i < task->n1; i++) {
        double m = s->nm[i];
        if (m > TOL) {
            s->nax[i] = s->nfx[i] / m;
            s->nay[i] = s->nfy[i] / m;
            s->nmx[i] += dt * s->nfx[i];
            s->nmy[i] += dt * s->nfy[i];
            s->nvx[i] = s->nmx[i] / m;
            s->nvy[i] = s->nmy[i] / m;
            s->nux[i] = dt * s->nvx[i];
            s->nuy[i] = dt * s->nvy[i];
        } else {
            s->nax[i] = 0;
            s->nay[i] = 0;
            s->nvx[i] = 0;
            s->nvy[i] = 0;
        }
    }
    pthread_barrier_wait(&s->bar);

    /* move_particles_explicit_usl_split, process_usl.c:914-957 */
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        double sv[4] = {s->h1[i], s->h2[i], s->h3[i], s->h4[i]};
        const int *nn = s->enodes + 4 * s->in_element[i];
        s->ax[i] = 0;
        s->ay[i] = 0;
        for (int j = 0; j < 4; j++) {
            double m = s->nm[nn[j]];
            if (m < TOL) {
                continue;
            }
            s->ax[i] += ((sv[j] * s->nfx[nn[j]]) / m);
            s->ay[i] += ((sv[j] * s->nfy[nn[j]]) / m);
        }
        s->vx[i] += dt * s->ax[i];
        s->vy[i] += dt * s->ay[i];
        double dux = 0, duy = 0;
        for (int j = 0; j < 4; j++) {
            double m = s->nm[nn[j]];
            if (m < TOL) {
                continue;
            }
            dux += ((sv[j] * s->nmx[nn[j]]) / m);
            duy += ((sv[j] * s->nmy[nn[j]]) / m);
        }
        dux *= dt;
        duy *= dt;
        s->x[i] += dux;
        s->y[i] += duy;
        s->ux[i] += dux;
        s->uy[i] += duy;
    }

    if (s->c.scheme == ORC_MUSL) {
        /* explicit_mpm_step_musl_threaded, process_usl.c:398-444: clear the
           nodes, map the moved particles' momentum to them again with the
           start-of-step shape functions, take nodal velocities from it.  The
           reference zeroes the constrained momenta (bc_momentum) after the
           velocities are formed, so the constraint does not reach them. */
        pthread_barrier_wait(&s->bar);
        for (size_t i = task->n0; i < task->n1; i++) {
            s->nm[i] = 0; s->nmx[i] = 0; s->nmy[i] = 0; s->nmxx[i] = 0; s->nmyy[i] = 0;
            s->nvx[i] = 0; s->nvy[i] = 0; s->nax[i] = 0; s->nay[i] = 0; s->nfx[i] = 0;
            s->nfy[i] = 0; s->nux[i] = 0; s->nuy[i] = 0;
        }
        pthread_barrier_wait(&s->bar);
        p2g_by_colour(task);
        pthread_barrier_wait(&s->bar);
        for (size_t i = task->n0; i < task->n1; i++) {
            if (s->nm[i] > TOL) {
                s->nvx[i] = s->nmx[i] / s->nm[i];
                s->nvy[i] = s->nmy[i] / s->nm[i];
            } else {
                s->nvx[i] = 0;
                s->nvy[i] = 0;
            }
        }
        if (pthread_barrier_wait(&s->bar) == PTHREAD_BARRIER_SERIAL_THREAD) {
            for (size_t i = 0; i < s->nn; i++) {
                if (s->mask[3 * i + 0]) s->nmx[i] = 0;
                if (s->mask[3 * i + 1]) s->nmy[i] = 0;
            }
        }
        pthread_barrier_wait(&s->bar);
    }

    /* calculate_strainrate_split, process_usl.c:764-808 (non-CPDI branch) */
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        const int *nn = s->enodes + 4 * s->in_element[i];
        s->exx[i] = 0;
        s->exy[i] = 0;
        s->eyy[i] = 0;
        s->wxy[i] = 0;
        double exx = 1.0 * (s->b11[i] * s->nvx[nn[0]] + s->b12[i] * s->nvx[nn[1]]
                            + s->b13[i] * s->nvx[nn[2]] + s->b14[i] * s->nvx[nn[3]]);
        double eyy = 1.0 * (s->b21[i] * s->nvy[nn[0]] + s->b22[i] * s->nvy[nn[1]]
                            + s->b23[i] * s->nvy[nn[2]] + s->b24[i] * s->nvy[nn[3]]);
        double dx_tdy = 1.0 * (s->b21[i] * s->nvx[nn[0]] + s->b22[i] * s->nvx[nn[1]]
                               + s->b23[i] * s->nvx[nn[2]] + s->b24[i] * s->nvx[nn[3]]);
        double dy_tdx = 1.0 * (s->b11[i] * s->nvy[nn[0]] + s->b12[i] * s->nvy[nn[1]]
                               + s->b13[i] * s->nvy[nn[2]] + s->b14[i] * s->nvy[nn[3]]);
        s->exx[i] = exx;
        s->eyy[i] = eyy;
        s->exy[i] = 0.5 * (dx_tdy + dy_tdx);
        s->wxy[i] = 0.5 * (dx_tdy - dy_tdx);
    }

    /* update_particle_densities_split, process_usl.c:961-970 */
    for (size_t i = task->p0; i < task->p1; i++) {
        if (s->active[i] == 0) {
            continue;
        }
        s->v[i] = s->v[i] * exp(dt * (s->exx[i] + s->eyy[i]));
    }

    /* material calculate_stress_threaded, process_usl.c:589 */
    switch (s->c.material) {
    case ORC_ISOLIN:
        isolin_range(s, task->p0, task->p1);
        break;
    case ORC_G_LOCAL_MU2:
        g_local_mu2_range(s, task->p0, task->p1);
        break;
    case ORC_DP_RI_MT:
    case ORC_G_LOCAL_MU2_PLANE_STRAIN:
    case ORC_G_LOCAL_MU2_TRUE_2D:
        plane_return_material(s->c.material, task->p0, task->p1, s);
        break;
    case ORC_G_LOCAL_MU2_EXT:
        g_local_mu2_ext_thread(task);
        break;
    case ORC_G_LOCAL_MU2_REVERSE:
        g_local_mu2_reverse_range(s, task->p0, task->p1);
        break;
    case ORC_G_NONLOCAL_MU2:
        /* g_nonlocal_mu2.c:113-123: thread 0 solves for everyone.  The
           reference has no barrier here, so with more than one thread its
           solve reads particles other threads are still updating (a data
           race: results vary run to run).  The oracle waits for the team,
           which reproduces the reference's single-thread results. */
        pthread_barrier_wait(&s->bar);
        if (task->id == 0) {
            task->status = g_nonlocal_mu2_stress(s);
        }
        break;
    case ORC_G_NONLOCAL:
    case ORC_G_NONLOCAL_AVG:
        pthread_barrier_wait(&s->bar);
        if (task->id == 0) {
            task->status = g_nonlocal_stress(s);
        }
        break;
    default:
        break;
    }
    (void)Nx;
}

static void *team_main(void *arg)
{
    orc_task *task = (orc_task *)arg;
    orc_sim *s = task->s;
    for (int k = 0; k < task->nsteps; k++) {
        step_thread(task);
        /* driver tail, src/main.c:951-976 */
        if (pthread_barrier_wait(&s->bar) == PTHREAD_BARRIER_SERIAL_THREAD) {
            time_varying_loads(s);
        }
    }
    return NULL;
}

int orc_step(orc_sim *s, int nsteps)
{
    size_t T = s->T_threads;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * T);
    for (size_t i = 0; i < T; i++) {
        s->tasks[i].nsteps = nsteps;
        s->tasks[i].status = 0;
    }
    for (size_t i = 0; i + 1 < T; i++) {
        pthread_create(&th[i], NULL, team_main, &s->tasks[i + 1]);
    }
    team_main(&s->tasks[0]);
    for (size_t i = 0; i + 1 < T; i++) {
        pthread_join(th[i], NULL);
    }
    free(th);
    return s->tasks[0].status;
}

int orc_material_only(orc_sim *s)
{
    switch (s->c.material) {
    case ORC_ISOLIN:
        isolin_range(s, 0, s->np);
        return 0;
    case ORC_G_LOCAL_MU2:
        g_local_mu2_range(s, 0, s->np);
        return 0;
    case ORC_DP_RI_MT:
    case ORC_G_LOCAL_MU2_PLANE_STRAIN:
    case ORC_G_LOCAL_MU2_TRUE_2D:
        plane_return_material(s->c.material, 0, s->np, s);
        return 0;
    case ORC_G_LOCAL_MU2_REVERSE:
        g_local_mu2_reverse_range(s, 0, s->np);
        return 0;
    default:
        return 1;
    }
}

/*---------------------------------------------------------------------------*/
static double *field_ptr(orc_sim *s, const char *name, size_t *count, int *stride, int *offset)
{
    *stride = 1;
    *offset = 0;
    *count = s->np;
    struct { const char *n; double *p; } pf[] = {
        {"x", s->x}, {"y", s->y}, {"xl", s->xl}, {"yl", s->yl}, {"v", s->v}, {"v0", s->v0},
        {"m", s->m}, {"vx", s->vx}, {"vy", s->vy}, {"ax", s->ax}, {"ay", s->ay},
        {"bx", s->bx}, {"by", s->by}, {"sxx", s->sxx}, {"sxy", s->sxy}, {"syy", s->syy},
        {"ux", s->ux}, {"uy", s->uy}, {"exx", s->exx}, {"exy", s->exy}, {"eyy", s->eyy},
        {"wxy", s->wxy}};
    for (size_t k = 0; k < sizeof(pf) / sizeof(pf[0]); k++) {
        if (strcmp(name, pf[k].n) == 0) {
            return pf[k].p;
        }
    }
    struct { const char *n; int off; } tf[] = {
        {"Txx", XX}, {"Txy", XY}, {"Tyx", YX}, {"Tyy", YY}, {"Tzz", ZZ}};
    for (size_t k = 0; k < sizeof(tf) / sizeof(tf[0]); k++) {
        if (strcmp(name, tf[k].n) == 0) {
            *stride = 9;
            *offset = tf[k].off;
            return s->T;
        }
    }
    if (strncmp(name, "state", 5) == 0) {
        int k = atoi(name + 5);
        if (k >= 0 && k < DEPVAR) {
            *stride = DEPVAR;
            *offset = k;
            return s->state;
        }
    }
    *count = s->nn;
    struct { const char *n; double *p; } nf[] = {
        {"node_m", s->nm}, {"node_mx", s->nmx}, {"node_my", s->nmy}, {"node_fx", s->nfx},
        {"node_fy", s->nfy}, {"node_vx", s->nvx}, {"node_vy", s->nvy}, {"node_ax", s->nax},
        {"node_ay", s->nay}, {"node_gf", s->gf_nodes}};
    for (size_t k = 0; k < sizeof(nf) / sizeof(nf[0]); k++) {
        if (strcmp(name, nf[k].n) == 0) {
            return nf[k].p;
        }
    }
    return NULL;
}

long orc_get_field(orc_sim *s, const char *name, double *out)
{
    size_t count;
    int stride, offset;
    double *p = field_ptr(s, name, &count, &stride, &offset);
    if (p == NULL) {
        return -1;
    }
    for (size_t i = 0; i < count; i++) {
        out[i] = p[(size_t)stride * i + (size_t)offset];
    }
    return (long)count;
}

long orc_set_field(orc_sim *s, const char *name, const double *in)
{
    size_t count;
    int stride, offset;
    double *p = field_ptr(s, name, &count, &stride, &offset);
    if (p == NULL) {
        return -1;
    }
    for (size_t i = 0; i < count; i++) {
        p[(size_t)stride * i + (size_t)offset] = in[i];
    }
    return (long)count;
}

void orc_get_map(orc_sim *s, int *in_element, int *active)
{
    memcpy(in_element, s->in_element, sizeof(int) * s->np);
    memcpy(active, s->active, sizeof(int) * s->np);
}

void orc_set_map(orc_sim *s, const int *in_element, const int *active)
{
    memcpy(s->in_element, in_element, sizeof(int) * s->np);
    memcpy(s->active, active, sizeof(int) * s->np);
}

double orc_time(orc_sim *s)
{
    return s->t;
}

void orc_set_time(orc_sim *s, double t, int step_number)
{
    s->t = t;
    s->step_number = step_number;
}

size_t orc_num_particles(orc_sim *s)
{
    return s->np;
}

size_t orc_num_nodes(orc_sim *s)
{
    return s->nn;
}

void orc_get_color_lists(orc_sim *s, size_t *out, size_t *lengths)
{
    size_t k = 0;
    for (size_t tc = 0; tc < s->T_threads * NCOLORS; tc++) {
        lengths[tc] = s->list_len[tc];
        for (size_t i = 0; i < s->list_len[tc]; i++) {
            out[k++] = s->lists[tc][i];
        }
    }
}

void orc_get_elements(orc_sim *s, int *filled, int *count, double *mass)
{
    memcpy(filled, s->efilled, sizeof(int) * s->ne);
    memcpy(count, s->en, sizeof(int) * s->ne);
    memcpy(mass, s->em, sizeof(double) * s->ne);
}

int orc_last_solve(orc_sim *s, int *iters, double *resid)
{
    *iters = s->solve_iters;
    *resid = s->solve_resid;
    return s->solve_status;
}
