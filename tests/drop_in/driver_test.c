/*
 * Test driver for the libmpm-compatible entry points (include/mpm_libmpm.h).
 * It drives libmpm_gb300.so the way the reference driver drives libmpm
 * (src/main.c:415-839 and mpm_run_until, :934-982): mpm_init, the material
 * and boundary-condition plugin names and properties, the task split, the
 * barriers and colour lists, find_filled_elements, initial_loads, then a
 * pthread team that calls explicit_mpm_step_usl_threaded followed by the
 * serial tail (frame check, time_varying_loads).  No plugin is loaded: the
 * GPU library runs the material and boundary conditions named by the files.
 *
 * usage: driver_test IN OUT [musl]   (musl: explicit_mpm_step_musl_threaded)
 * IN  (native binary): int32 N, nthreads, nsteps, nmprops, nbprops, nbiprops;
 *     float64 h, dt, sample_rate; char material[64], bc[64];
 *     float64 mprops[nmprops], bprops[nbprops]; int32 biprops[nbiprops];
 *     int64 n; float64 particles[n][9] (m v x y x_t y_t sxx sxy syy)
 * OUT: int64 n; float64 t; int64 frames; then per particle float64
 *     x y x_t y_t sxx sxy syy v ux uy state9 state10, int32 in_element, active
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpm_libmpm.h"

static int g_nsteps;
static long g_frames;
static int g_musl;

static void *run(void *arg)
{
    threadtask_t *task = (threadtask_t *)arg;
    job_t *job = task->job;
    for (int k = 0; k < g_nsteps; k++) {
        if (g_musl) {
            explicit_mpm_step_musl_threaded(task);
        } else {
            explicit_mpm_step_usl_threaded(task);
        }
        if (pthread_barrier_wait(job->serialize_barrier) == PTHREAD_BARRIER_SERIAL_THREAD) {
            job->stepcount++;
            if (job->t >= (job->frame / job->output.sample_rate_hz)) {
                g_frames++;          /* write_frame would read job->particles here */
                job->frame++;
            }
            time_varying_loads(job);
        }
    }
    return NULL;
}

#define READ(ptr, sz, cnt) do { if (fread(ptr, sz, cnt, f) != (size_t)(cnt)) { fprintf(stderr, "short input\n"); return 2; } } while (0)

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    g_musl = argc > 3 && strcmp(argv[3], "musl") == 0;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[6];
    double hd[3];
    static char material[64], bc[64];
    READ(hdr, sizeof(int32_t), 6);
    READ(hd, sizeof(double), 3);
    READ(material, 1, 64);
    READ(bc, 1, 64);
    int N = hdr[0], T = hdr[1];
    g_nsteps = hdr[2];
    double *mprops = malloc(sizeof(double) * (hdr[3] + 1));
    double *bprops = malloc(sizeof(double) * (hdr[4] + 1));
    int *biprops = malloc(sizeof(int) * (hdr[5] + 1));
    READ(mprops, sizeof(double), hdr[3]);
    READ(bprops, sizeof(double), hdr[4]);
    READ(biprops, sizeof(int32_t), hdr[5]);
    int64_t n;
    READ(&n, sizeof(int64_t), 1);
    particle_t *pdata = calloc((size_t)n + 1, sizeof(particle_t));
    for (int64_t i = 0; i < n; i++) {
        double r[9];
        READ(r, sizeof(double), 9);
        pdata[i].m = r[0]; pdata[i].v = r[1]; pdata[i].x = r[2]; pdata[i].y = r[3];
        pdata[i].x_t = r[4]; pdata[i].y_t = r[5]; pdata[i].sxx = r[6]; pdata[i].sxy = r[7]; pdata[i].syy = r[8];
    }
    fclose(f);

    job_t *job = mpm_init(N, hd[0], pdata, (size_t)n, 1e30);          /* src/main.c:415 */
    job->material.use_builtin = 0;                                   /* :416-456 */
    job->material.material_filename = material;
    job->material.num_fp64_props = (size_t)hdr[3];
    job->material.fp64_props = mprops;
    job->boundary.use_builtin = 0;                                   /* :486-559 */
    job->boundary.bc_filename = bc;
    job->boundary.num_fp64_props = (size_t)hdr[4];
    job->boundary.fp64_props = bprops;
    job->boundary.num_int_props = (size_t)hdr[5];
    job->boundary.int_props = biprops;
    job->dt = hd[1];                                                 /* :742 */
    job->output.sample_rate_hz = hd[2];

    threadtask_t *tasks = calloc((size_t)T, sizeof(threadtask_t));  /* :747-774 */
    size_t ps = job->num_particles / T + ((job->num_particles % T) ? 1 : 0);
    for (int i = 0; i < T; i++) {
        tasks[i].id = (size_t)i;
        tasks[i].num_threads = (size_t)T;
        tasks[i].job = job;
        tasks[i].offset = (size_t)i * ps;
        tasks[i].blocksize = tasks[i].offset < job->num_particles
            ? (ps < job->num_particles - tasks[i].offset ? ps : job->num_particles - tasks[i].offset) : 0;
    }
    job->num_threads = (size_t)T;
    job->step_barrier = malloc(sizeof(pthread_barrier_t));
    job->serialize_barrier = malloc(sizeof(pthread_barrier_t));
    pthread_barrier_init(job->step_barrier, NULL, (unsigned)T);
    pthread_barrier_init(job->serialize_barrier, NULL, (unsigned)T);
    job->update_elementlists = malloc(sizeof(int) * T);
    job->particle_by_element_color_lengths = malloc(sizeof(size_t) * 4 * T);   /* :800-804 */
    job->particle_by_element_color_lists = malloc(sizeof(size_t *) * 4 * T);
    for (int i = 0; i < 4 * T; i++) job->particle_by_element_color_lists[i] = malloc(sizeof(size_t) * ((size_t)n + 1));
    find_filled_elements(job);                                       /* :812 */
    initial_loads(job);                                              /* :814 */
    job->frame = 0;

    pthread_t *th = malloc(sizeof(pthread_t) * T);                   /* :832-839 */
    for (int i = 0; i < T - 1; i++) pthread_create(&th[i], NULL, run, &tasks[i]);
    run(&tasks[T - 1]);
    for (int i = 0; i < T - 1; i++) pthread_join(th[i], NULL);

    if (mpm_gpu_sync_host(job) != 0) {
        fprintf(stderr, "sync failed\n");
        return 3;
    }
    FILE *o = fopen(argv[2], "wb");
    fwrite(&n, sizeof(int64_t), 1, o);
    fwrite(&job->t, sizeof(double), 1, o);
    int64_t frames = g_frames;
    fwrite(&frames, sizeof(int64_t), 1, o);
    for (int64_t i = 0; i < n; i++) {
        const particle_t *p = &job->particles[i];
        double r[12] = {p->x, p->y, p->x_t, p->y_t, p->sxx, p->sxy, p->syy, p->v, p->ux, p->uy,
                        p->state[9], p->state[10]};
        fwrite(r, sizeof(double), 12, o);
        int32_t e[2] = {job->in_element[i], job->active[i]};
        fwrite(e, sizeof(int32_t), 2, o);
    }
    fclose(o);
    mpm_cleanup(job);
    return 0;
}
