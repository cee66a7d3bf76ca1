/*
 * Test infrastructure (oracle only): drives the reference's own compiled
 * libmpm (process_usl.c, loading.c, ...) and its dlopen'd material and
 * boundary-condition plugins, so that tests can read the reference's state
 * step by step.  Built by oracle/build.py into oracle/_ref/ from the
 * reference tree; never shipped and never linked into the product library.
 *
 * The set-up follows the reference driver, src/main.c, without libconfuse
 * (absent here):
 *   mpm_init                                 src/main.c:415
 *   dlopen/dlsym of the material plugin      src/main.c:427-456
 *   material and BC properties               src/main.c:458-467, 550-559
 *   dlopen/dlsym of the BC plugin            src/main.c:500-543
 *   job->dt from the configuration           src/main.c:742
 *   task split, barriers, colour lists       src/main.c:747-804
 *   clear elements, find_filled_elements     src/main.c:806-812
 *   initial_loads, material_init             src/main.c:814-815
 *   bc_validate                              src/main.c:820
 * and the time loop follows mpm_run_until (src/main.c:934-982) minus frame
 * output: step, barrier, then the serial tail time_varying_loads.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <dlfcn.h>
#include <pthread.h>

#include "process.h"
#include "process_usl.h"
#include "particle.h"
#include "node.h"
#include "element.h"

/* libmpm/loading.c:21,34 (no header in the reference). */
void initial_loads(job_t *job);
void time_varying_loads(job_t *job);

typedef struct refh_s {
    int musl;        /* 1: explicit_mpm_step_musl_threaded instead of the USL step */
    job_t *job;
    threadtask_t *tasks;
    int nthreads;
    int nsteps;
    void *mat_so;
    void *bc_so;
    FILE *log;
} refh_t;

/* Plugins without calculate_stress_threaded (materialsrc/g_nonlocal.c) are
   refused by the reference driver (src/main.c:449-455).  The harness runs
   them the way g_nonlocal_mu2.c:113-123 runs itself: task 0 calls
   calculate_stress for the whole job. */
static void (*g_serial_stress)(job_t *) = NULL;
static void serial_stress_threaded(void *arg)
{
    threadtask_t *task = (threadtask_t *)arg;
    if (task->id == 0) {
        g_serial_stress(task->job);
    }
}

static void *load_sym(void *so, const char *name, int *err)
{
    dlerror();
    void *p = dlsym(so, name);
    if (dlerror() != NULL) {
        fprintf(stderr, "ref_harness: missing symbol '%s'\n", name);
        *err = 1;
    }
    return p;
}

/*
 * pin: n rows of 9 values (m, v, x, y, x_t, y_t, sxx, sxy, syy), the columns
 * of the reference's particle file (src/reader.c:66-99).
 */
refh_t *refh_create(int N, double h, size_t n, const double *pin,
                    const char *mat_so_path, const double *mprops, size_t nmprops,
                    const char *bc_so_path, const double *bprops, size_t nbprops,
                    const int *biprops, size_t nbiprops, double dt, int nthreads)
{
    int err = 0;
    if (nthreads < 1) {
        nthreads = 1;
    }
    particle_t *p = (particle_t *)calloc(n, sizeof(particle_t));
    for (size_t i = 0; i < n; i++) {
        p[i].m = pin[9 * i + 0];
        p[i].v = pin[9 * i + 1];
        p[i].x = pin[9 * i + 2];
        p[i].y = pin[9 * i + 3];
        p[i].x_t = pin[9 * i + 4];
        p[i].y_t = pin[9 * i + 5];
        p[i].sxx = pin[9 * i + 6];
        p[i].sxy = pin[9 * i + 7];
        p[i].syy = pin[9 * i + 8];
    }

    refh_t *r = (refh_t *)calloc(1, sizeof(refh_t));
    job_t *job = mpm_init(N, h, p, n, 1e30);
    free(p);
    r->job = job;
    r->log = fopen("/dev/null", "w");
    job->output.log_fd = r->log;

    job->material.use_builtin = 0;
    job->material.material_filename = mat_so_path;
    r->mat_so = dlopen(mat_so_path, RTLD_NOW | RTLD_LOCAL);
    if (r->mat_so == NULL) {
        fprintf(stderr, "ref_harness: dlopen(%s): %s\n", mat_so_path, dlerror());
        return NULL;
    }
    *(void **)&job->material.material_init = load_sym(r->mat_so, "material_init", &err);
    *(void **)&job->material.calculate_stress = load_sym(r->mat_so, "calculate_stress", &err);
    dlerror();
    *(void **)&job->material.calculate_stress_threaded = dlsym(r->mat_so, "calculate_stress_threaded");
    if (dlerror() != NULL || job->material.calculate_stress_threaded == NULL) {
        g_serial_stress = job->material.calculate_stress;
        job->material.calculate_stress_threaded = serial_stress_threaded;
    }

    job->material.num_fp64_props = nmprops;
    job->material.num_int_props = 0;
    job->material.fp64_props = (double *)malloc(sizeof(double) * (nmprops + 1));
    job->material.int_props = (int *)malloc(sizeof(int));
    memcpy(job->material.fp64_props, mprops, sizeof(double) * nmprops);

    job->boundary.use_builtin = 0;
    job->boundary.bc_filename = bc_so_path;
    r->bc_so = dlopen(bc_so_path, RTLD_NOW | RTLD_LOCAL);
    if (r->bc_so == NULL) {
        fprintf(stderr, "ref_harness: dlopen(%s): %s\n", bc_so_path, dlerror());
        return NULL;
    }
    *(void **)&job->boundary.bc_init = load_sym(r->bc_so, "bc_init", &err);
    *(void **)&job->boundary.bc_validate = load_sym(r->bc_so, "bc_validate", &err);
    *(void **)&job->boundary.bc_time_varying = load_sym(r->bc_so, "bc_time_varying", &err);
    *(void **)&job->boundary.bc_momentum = load_sym(r->bc_so, "bc_momentum", &err);
    *(void **)&job->boundary.bc_force = load_sym(r->bc_so, "bc_force", &err);
    if (err) {
        return NULL;
    }
    job->boundary.num_fp64_props = nbprops;
    job->boundary.num_int_props = nbiprops;
    job->boundary.fp64_props = (double *)malloc(sizeof(double) * (nbprops + 1));
    job->boundary.int_props = (int *)malloc(sizeof(int) * (nbiprops + 1));
    memcpy(job->boundary.fp64_props, bprops, sizeof(double) * nbprops);
    memcpy(job->boundary.int_props, biprops, sizeof(int) * nbiprops);

    job->dt = dt;

    r->nthreads = nthreads;
    r->tasks = (threadtask_t *)calloc((size_t)nthreads, sizeof(threadtask_t));
    job->step_barrier = (pthread_barrier_t *)malloc(sizeof(pthread_barrier_t));
    job->serialize_barrier = (pthread_barrier_t *)malloc(sizeof(pthread_barrier_t));
    size_t T = (size_t)nthreads;
    size_t psplit = job->num_particles / T + ((job->num_particles % T) ? 1 : 0);
    size_t nsplit = job->num_nodes / T + ((job->num_nodes % T) ? 1 : 0);
    size_t esplit = job->num_elements / T + ((job->num_elements % T) ? 1 : 0);
    for (size_t i = 0; i < T; i++) {
        threadtask_t *t = &r->tasks[i];
        t->id = i;
        t->num_threads = T;
        t->job = job;
        t->offset = i * psplit;
        t->blocksize = (t->offset < job->num_particles)
            ? ((psplit < job->num_particles - t->offset) ? psplit : job->num_particles - t->offset) : 0;
        t->n_offset = i * nsplit;
        t->n_blocksize = (t->n_offset < job->num_nodes)
            ? ((nsplit < job->num_nodes - t->n_offset) ? nsplit : job->num_nodes - t->n_offset) : 0;
        t->e_offset = i * esplit;
        t->e_blocksize = (t->e_offset < job->num_elements)
            ? ((esplit < job->num_elements - t->e_offset) ? esplit : job->num_elements - t->e_offset) : 0;
        t->gidx_max = job->num_particles;
        t->gidx_min = 0;
    }
    job->num_threads = T;
    pthread_barrier_init(job->step_barrier, NULL, (unsigned)T);
    pthread_barrier_init(job->serialize_barrier, NULL, (unsigned)T);

    job->update_elementlists = (int *)malloc(sizeof(int) * T);
    for (size_t i = 0; i < T; i++) {
        job->update_elementlists[i] = 1;
    }
    job->particle_by_element_color_lengths =
        (size_t *)malloc(sizeof(size_t) * job->num_colors * T);
    job->particle_by_element_color_lists =
        (size_t **)malloc(sizeof(size_t *) * job->num_colors * T);
    for (size_t i = 0; i < job->num_colors * T; i++) {
        job->particle_by_element_color_lists[i] =
            (size_t *)malloc(sizeof(size_t) * (job->num_particles + 1));
    }

    for (size_t i = 0; i < job->num_elements; i++) {
        job->elements[i].filled = 0;
        job->elements[i].n = 0;
        job->elements[i].m = 0;
    }
    find_filled_elements(job);
    initial_loads(job);
    job->material.material_init(job);
    if (job->boundary.bc_validate(job) == 0) {
        fprintf(stderr, "ref_harness: bc_validate failed\n");
        return NULL;
    }
    return r;
}

/* The scheme of the team refh_step runs (one team at a time). */
static int g_musl = 0;

static void *run_steps(void *arg)
{
    threadtask_t *task = (threadtask_t *)arg;
    job_t *job = task->job;
    /* refh_step stores the step count in job->stepcount before the team starts. */
    int nsteps = job->stepcount;
    for (int k = 0; k < nsteps; k++) {
        if (g_musl) {
            explicit_mpm_step_musl_threaded(task);
        } else {
            explicit_mpm_step_usl_threaded(task);
        }
        int rc = pthread_barrier_wait(job->serialize_barrier);
        if (rc == PTHREAD_BARRIER_SERIAL_THREAD) {
            time_varying_loads(job);
        }
    }
    return NULL;
}

/* Runs nsteps of the driver's time loop on the harness's thread team. */
void refh_set_scheme(refh_t *r, int musl)
{
    r->musl = musl;
}

int refh_step(refh_t *r, int nsteps)
{
    job_t *job = r->job;
    job->stepcount = nsteps;
    g_musl = r->musl;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)r->nthreads);
    for (int i = 0; i < r->nthreads - 1; i++) {
        pthread_create(&th[i], NULL, run_steps, &r->tasks[i]);
    }
    run_steps(&r->tasks[r->nthreads - 1]);
    for (int i = 0; i < r->nthreads - 1; i++) {
        pthread_join(th[i], NULL);
    }
    free(th);
    job->stepcount = 0;
    return 0;
}

double refh_time(refh_t *r)
{
    return r->job->t;
}

size_t refh_num_particles(refh_t *r)
{
    return r->job->num_particles;
}

/*
 * Particle fields, REFH_PF values per particle:
 *  0 x, 1 y, 2 xl, 3 yl, 4 v, 5 m, 6 x_t, 7 y_t, 8 x_tt, 9 y_tt, 10 bx, 11 by,
 *  12 sxx, 13 sxy, 14 syy, 15 ux, 16 uy, 17 exx_t, 18 exy_t, 19 eyy_t,
 *  20 wxy_t, 21 T_xx, 22 T_xy, 23 T_yx, 24 T_yy, 25 T_zz, 26..36 state[0..10]
 */
#define REFH_PF 37
int refh_particle_fields(void)
{
    return REFH_PF;
}

void refh_get_particles(refh_t *r, double *out, int *in_element, int *active)
{
    job_t *job = r->job;
    for (size_t i = 0; i < job->num_particles; i++) {
        const particle_t *p = &job->particles[i];
        double *o = out + (size_t)REFH_PF * i;
        o[0] = p->x; o[1] = p->y; o[2] = p->xl; o[3] = p->yl;
        o[4] = p->v; o[5] = p->m; o[6] = p->x_t; o[7] = p->y_t;
        o[8] = p->x_tt; o[9] = p->y_tt; o[10] = p->bx; o[11] = p->by;
        o[12] = p->sxx; o[13] = p->sxy; o[14] = p->syy;
        o[15] = p->ux; o[16] = p->uy;
        o[17] = p->exx_t; o[18] = p->exy_t; o[19] = p->eyy_t; o[20] = p->wxy_t;
        o[21] = p->T[XX]; o[22] = p->T[XY]; o[23] = p->T[YX]; o[24] = p->T[YY];
        o[25] = p->T[ZZ];
        for (int k = 0; k < DEPVAR; k++) {
            o[26 + k] = p->state[k];
        }
        in_element[i] = job->in_element[i];
        active[i] = job->active[i];
    }
}

/* Node fields, 9 per node: m, mx_t, my_t, fx, fy, x_t, y_t, x_tt, y_tt. */
void refh_get_nodes(refh_t *r, double *out)
{
    job_t *job = r->job;
    for (size_t i = 0; i < job->num_nodes; i++) {
        const node_t *n = &job->nodes[i];
        double *o = out + 9 * i;
        o[0] = n->m; o[1] = n->mx_t; o[2] = n->my_t; o[3] = n->fx; o[4] = n->fy;
        o[5] = n->x_t; o[6] = n->y_t; o[7] = n->x_tt; o[8] = n->y_tt;
    }
}

/* Element occupancy from find_filled_elements: filled, n per element. */
void refh_get_elements(refh_t *r, int *filled, int *count, double *mass)
{
    job_t *job = r->job;
    for (size_t i = 0; i < job->num_elements; i++) {
        filled[i] = job->elements[i].filled;
        count[i] = job->elements[i].n;
        mass[i] = job->elements[i].m;
    }
}

/*
 * The per-(thread, colour) particle lists built by find_filled_elements
 * (libmpm/process_usl.c:703-720), concatenated in tc order into out (length
 * at least num_particles); lengths[T*4] receives each list's length.
 */
void refh_get_color_lists(refh_t *r, size_t *out, size_t *lengths)
{
    job_t *job = r->job;
    size_t k = 0;
    for (size_t tc = 0; tc < job->num_threads * job->num_colors; tc++) {
        lengths[tc] = job->particle_by_element_color_lengths[tc];
        for (size_t i = 0; i < lengths[tc]; i++) {
            out[k++] = job->particle_by_element_color_lists[tc][i];
        }
    }
}

void refh_destroy(refh_t *r)
{
    if (r == NULL) {
        return;
    }
    job_t *job = r->job;
    for (size_t i = 0; i < job->num_colors * job->num_threads; i++) {
        free(job->particle_by_element_color_lists[i]);
    }
    free(job->particle_by_element_color_lists);
    free(job->particle_by_element_color_lengths);
    free(job->update_elementlists);
    pthread_barrier_destroy(job->step_barrier);
    pthread_barrier_destroy(job->serialize_barrier);
    free(job->step_barrier);
    free(job->serialize_barrier);
    free(job->material.fp64_props);
    free(job->material.int_props);
    free(job->boundary.fp64_props);
    free(job->boundary.int_props);
    mpm_cleanup(job);
    free(job);
    free(r->tasks);
    if (r->log != NULL) {
        fclose(r->log);
    }
    /* Plugins keep static state; leave them loaded for the process. */
    free(r);
}

/* src/writer.c:190-201, :205-263 and :266-380, linked into this harness from
   the reference's own writer.c. */
void write_frame(FILE *fd, size_t frame, double time, job_t *job);
void write_element_frame(FILE *fd, size_t frame, double time, job_t *job);
void write_state(FILE *fd, job_t *job);

/* Writes the job with the reference's writer: what 0 = write_frame, 1 =
   write_element_frame (both with the given frame number and time), 2 =
   write_state.  Returns 0, or 1 when the file cannot be opened. */
int refh_write(refh_t *r, const char *path, int what, size_t frame, double time)
{
    FILE *fd = fopen(path, "w");
    if (fd == NULL) {
        return 1;
    }
    if (what == 0) {
        write_frame(fd, frame, time, r->job);
    } else if (what == 1) {
        write_element_frame(fd, frame, time, r->job);
    } else {
        write_state(fd, r->job);
    }
    fclose(fd);
    return 0;
}
