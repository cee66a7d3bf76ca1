// The phase functions of the reference's threaded USL step
// (libmpm/process_usl.h:15-22), exported with the reference's names and
// signatures: each works on the job's host arrays like the reference's, over
// the same particle, node or thread range, with the arithmetic on the GPU.
// A call gathers its range's inputs into one device buffer, runs one FP64
// kernel, and scatters the results back into job->particles, job->nodes and
// the shape-function arrays.  The kernels follow the reference's operation
// order with correctly rounded operations and no contracted multiply-adds,
// so a phase gives the reference's values.
//
// These calls do not touch a GPU context attached to the job
// (mpm_gpu_attach): the step the context runs keeps its own state on the
// device, and the host arrays these phases read and write are refreshed from
// it only by mpm_gpu_sync_host.  They run on the attached context's device
// (device 0 without one), each on its own stream, so that the driver's
// threads may call them concurrently on disjoint ranges, as the reference's
// step does.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "../../include/mpm_libmpm.h"
#include "mpmg_materials.cuh"

int mpmg_libmpm_job_device(job_t *job);   // mpmg_libmpm.cu

namespace {

constexpr double kTol = 1e-10;   // process_usl.c:25

// A CUDA failure in a void phase function ends the process, as the
// reference's driver does on its own errors.
void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        fprintf(stderr, "mpm_gb300: %s: %s\n", what, cudaGetErrorString(e));
        exit(EXIT_FAILURE);
    }
}

// One call's device buffer and stream: `slices` double arrays of n values.
struct Stage {
    int n = 0, slices = 0;
    std::vector<double> host;
    double *dev = nullptr;
    cudaStream_t stream = nullptr;

    Stage(job_t *job, int n_, int slices_) : n(n_), slices(slices_), host((size_t)n_ * slices_, 0.0)
    {
        check(cudaSetDevice(mpmg_libmpm_job_device(job)), "cudaSetDevice");
        check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        if (n > 0) check(cudaMalloc(&dev, host.size() * sizeof(double)), "cudaMalloc");
    }
    ~Stage()
    {
        if (dev != nullptr) cudaFree(dev);
        if (stream != nullptr) cudaStreamDestroy(stream);
    }
    double *h(int k) { return host.data() + (size_t)k * n; }
    void up() { check(cudaMemcpyAsync(dev, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, stream), "copy to device"); }
    void down()
    {
        check(cudaGetLastError(), "kernel launch");
        check(cudaMemcpyAsync(host.data(), dev, host.size() * sizeof(double), cudaMemcpyDeviceToHost, stream), "copy to host");
        check(cudaStreamSynchronize(stream), "phase kernel");
    }
};

inline int blocks(int n)
{
    return n > 0 ? (n + 255) / 256 : 1;
}

// global_to_local_coords (libmpm/particle.c:14-30): one coordinate.
__device__ __forceinline__ double local_coord(double x, double xr, double h)
{
    double l = __ddiv_rn(__dsub_rn(x, xr), h);
    const double sgn = copysign(1.0, l);
    const double a = sgn * l;
    if (a > 1.0 && __dsub_rn(a, 1.0) < kTol) l = sgn;
    return l;
}

// Slices: in x, y, xn, yn; out xl, yl, h1..h4, b11..b14, b21..b24.
__global__ void shape_kernel(int n, double h, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xl = local_coord(a[i], a[2 * n + i], h);
    const double yl = local_coord(a[n + i], a[3 * n + i], h);
    double *o = a + 4 * (size_t)n;
    o[i] = xl;
    o[n + i] = yl;
    // tent and grad_tent (libmpm/interpolate.c:23-65)
    const double ox = __dsub_rn(1.0, xl), oy = __dsub_rn(1.0, yl);
    o[2 * n + i] = __dmul_rn(ox, oy);
    o[3 * n + i] = __dmul_rn(xl, oy);
    o[4 * n + i] = __dmul_rn(xl, yl);
    o[5 * n + i] = __dmul_rn(ox, yl);
    const double dxl = __ddiv_rn(1.0, h), dyl = __ddiv_rn(1.0, h);
    o[6 * n + i] = __dmul_rn(-oy, dxl);
    o[7 * n + i] = __dmul_rn(oy, dxl);
    o[8 * n + i] = __dmul_rn(yl, dxl);
    o[9 * n + i] = __dmul_rn(-yl, dxl);
    o[10 * n + i] = __dmul_rn(-ox, dyl);
    o[11 * n + i] = __dmul_rn(-xl, dyl);
    o[12 * n + i] = __dmul_rn(xl, dyl);
    o[13 * n + i] = __dmul_rn(ox, dyl);
}

// SMEAR4 (process_usl.c:53-58): ((a1 n1 + a2 n2) + a3 n3) + a4 n4.
__device__ __forceinline__ double smear4(const double *a, const double *v)
{
    double s = __dadd_rn(__dmul_rn(a[0], v[0]), __dmul_rn(a[1], v[1]));
    s = __dadd_rn(s, __dmul_rn(a[2], v[2]));
    return __dadd_rn(s, __dmul_rn(a[3], v[3]));
}

// Slices: in b11..b14, b21..b24, x_t of the 4 nodes, y_t of the 4 nodes;
// out exx_t, exy_t, eyy_t, wxy_t.
__global__ void strainrate_kernel(int n, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double b1[4], b2[4], xt[4], yt[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        b1[k] = a[(size_t)k * n + i];
        b2[k] = a[(size_t)(4 + k) * n + i];
        xt[k] = a[(size_t)(8 + k) * n + i];
        yt[k] = a[(size_t)(12 + k) * n + i];
    }
    const double dxtdy = smear4(b2, xt), dytdx = smear4(b1, yt);
    double *o = a + 16 * (size_t)n;
    o[i] = smear4(b1, xt);
    o[n + i] = __dmul_rn(0.5, __dadd_rn(dxtdy, dytdx));
    o[2 * n + i] = smear4(b2, yt);
    o[3 * n + i] = __dmul_rn(0.5, __dsub_rn(dxtdy, dytdx));
}

// Slices: in m, fx, fy, mx_t, my_t, ux, uy; out x_tt, y_tt, mx_t, my_t, x_t,
// y_t, ux, uy (move_grid_split, process_usl.c:596-625).
__global__ void move_grid_kernel(int n, double dt, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double m = a[i], fx = a[n + i], fy = a[2 * n + i];
    double mx = a[3 * n + i], my = a[4 * n + i], ux = a[5 * n + i], uy = a[6 * n + i];
    double xtt = 0, ytt = 0, xt = 0, yt = 0;
    if (m > kTol) {
        xtt = __ddiv_rn(fx, m);
        ytt = __ddiv_rn(fy, m);
        mx = __dadd_rn(mx, __dmul_rn(dt, fx));
        my = __dadd_rn(my, __dmul_rn(dt, fy));
        xt = __ddiv_rn(mx, m);
        yt = __ddiv_rn(my, m);
        ux = __dmul_rn(dt, xt);
        uy = __dmul_rn(dt, yt);
    }
    double *o = a + 7 * (size_t)n;
    o[i] = xtt;
    o[n + i] = ytt;
    o[2 * n + i] = mx;
    o[3 * n + i] = my;
    o[4 * n + i] = xt;
    o[5 * n + i] = yt;
    o[6 * n + i] = ux;
    o[7 * n + i] = uy;
}

// Slices: in h1..h4; for each of the 4 nodes m, fx, fy, mx_t, my_t (20);
// x_t, y_t, x, y, ux, uy; out x_tt, y_tt, x_t, y_t, x, y, ux, uy
// (move_particles_explicit_usl_split, process_usl.c:914-957).
__global__ void move_particles_kernel(int n, double dt, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto at = [&](int k) { return a[(size_t)k * n + i]; };
    double xtt = 0, ytt = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double s = at(j), m = at(4 + 5 * j);
        if (m < kTol) continue;
        xtt = __dadd_rn(xtt, __ddiv_rn(__dmul_rn(s, at(5 + 5 * j)), m));
        ytt = __dadd_rn(ytt, __ddiv_rn(__dmul_rn(s, at(6 + 5 * j)), m));
    }
    const double xt = __dadd_rn(at(24), __dmul_rn(dt, xtt));
    const double yt = __dadd_rn(at(25), __dmul_rn(dt, ytt));
    double dux = 0, duy = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double s = at(j), m = at(4 + 5 * j);
        if (m < kTol) continue;
        dux = __dadd_rn(dux, __ddiv_rn(__dmul_rn(s, at(7 + 5 * j)), m));
        duy = __dadd_rn(duy, __ddiv_rn(__dmul_rn(s, at(8 + 5 * j)), m));
    }
    dux = __dmul_rn(dux, dt);
    duy = __dmul_rn(duy, dt);
    double *o = a + 30 * (size_t)n;
    o[i] = xtt;
    o[n + i] = ytt;
    o[2 * n + i] = xt;
    o[3 * n + i] = yt;
    o[4 * n + i] = __dadd_rn(at(26), dux);
    o[5 * n + i] = __dadd_rn(at(27), duy);
    o[6 * n + i] = __dadd_rn(at(28), dux);
    o[7 * n + i] = __dadd_rn(at(29), duy);
}

// Slices: in v, exx_t, eyy_t; out v (update_particle_densities_split,
// process_usl.c:961-970).
__global__ void densities_kernel(int n, double dt, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[3 * (size_t)n + i] = __dmul_rn(a[i], mat::exp_small(__dmul_rn(dt, __dadd_rn(a[n + i], a[2 * n + i]))));
}

// Slices: in x, y; out the element (WHICH_ELEMENT4, process_usl.c:43-44,
// as a double).
__global__ void element_map_kernel(int n, double h, double nm1, double *a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = a[n + i];
    double e = -1;
    if (x < 1.0 && x >= 0.0 && y < 1.0 && y >= 0.0)
        e = (double)(int)__dadd_rn(floor(__ddiv_rn(x, h)), __dmul_rn(floor(__ddiv_rn(y, h)), nm1));
    a[2 * (size_t)n + i] = e;
}

// P2G by node (map_to_grid_explicit_split, process_usl.c:812-910, with
// accumulate_p_to_n_ds_list47/42, libmpm/map.c:85-104): node k adds the
// contributions listed for it in entry order (the order the reference's
// colour loop adds them).  Particle slices (np each): h1..h4, b11..b14,
// b21..b24, m, x_t, y_t, x_tt, y_tt, bx, by, sxx, sxy, syy, v.  Node slices
// (nn each, in and out): m, mx_t, my_t, mx_tt, my_tt, fx, fy.  An entry is
// particle * 4 + corner.
__global__ void p2g_nodes_kernel(int nn, int np, const double *__restrict__ pd, double *__restrict__ nd,
                                 const int *__restrict__ start, const long long *__restrict__ entry)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn) return;
    double v[7];
#pragma unroll
    for (int f = 0; f < 7; f++) v[f] = nd[(size_t)f * nn + k];
    auto P = [&](int s, long long p) { return pd[(size_t)s * np + p]; };
    for (int e = start[k]; e < start[k + 1]; e++) {
        const long long p = entry[e] >> 2;
        const int c = (int)(entry[e] & 3);
        const double s = P(c, p), m = P(12, p);
        const double pdata[7] = {m, __dmul_rn(P(13, p), m), __dmul_rn(P(14, p), m), __dmul_rn(P(15, p), m),
                                 __dmul_rn(P(16, p), m), __dmul_rn(P(17, p), m), __dmul_rn(P(18, p), m)};
#pragma unroll
        for (int f = 0; f < 7; f++) v[f] = __dadd_rn(v[f], __dmul_rn(s, pdata[f]));
        const double vol = P(22, p);
        const double sx = __dmul_rn(-P(19, p), vol), sxy = __dmul_rn(-P(20, p), vol), sy = __dmul_rn(-P(21, p), vol);
        const double b1 = P(4 + c, p), b2 = P(8 + c, p);
        v[5] = __dadd_rn(v[5], __dmul_rn(b1, sx));
        v[6] = __dadd_rn(v[6], __dmul_rn(b1, sxy));
        v[5] = __dadd_rn(v[5], __dmul_rn(b2, sxy));
        v[6] = __dadd_rn(v[6], __dmul_rn(b2, sy));
    }
#pragma unroll
    for (int f = 0; f < 7; f++) nd[(size_t)f * nn + k] = v[f];
}

}  // namespace

extern "C" {

void calculate_shapefunctions_split(job_t *job, size_t p_start, size_t p_stop)
{
    std::vector<size_t> idx;
    for (size_t i = p_start; i < p_stop; i++)
        if (job->active[i] != 0) idx.push_back(i);
    Stage S(job, (int)idx.size(), 18);
    for (size_t k = 0; k < idx.size(); k++) {
        const size_t i = idx[k];
        const node_t &nd = job->nodes[job->elements[job->in_element[i]].nodes[0]];
        S.h(0)[k] = job->particles[i].x;
        S.h(1)[k] = job->particles[i].y;
        S.h(2)[k] = nd.x;
        S.h(3)[k] = nd.y;
    }
    if (S.n == 0) return;
    S.up();
    shape_kernel<<<blocks(S.n), 256, 0, S.stream>>>(S.n, job->h, S.dev);
    S.down();
    double *sf[12] = {job->h1, job->h2, job->h3, job->h4, job->b11, job->b12,
                      job->b13, job->b14, job->b21, job->b22, job->b23, job->b24};
    for (size_t k = 0; k < idx.size(); k++) {
        const size_t i = idx[k];
        const double xl = S.h(4)[k], yl = S.h(5)[k];
        for (int q = 0; q < 12; q++) sf[q][i] = S.h(6 + q)[k];
        if (xl < 0.0f || xl > 1.0f || yl < 0.0f || yl > 1.0f)
            fprintf(stderr, "Particle %zu outside of element %zu (%g, %g).\n", i, (size_t)job->in_element[i], xl,
                    yl);
        job->particles[i].xl = xl;
        job->particles[i].yl = yl;
    }
}

void calculate_strainrate_split(job_t *job, size_t p_start, size_t p_stop)
{
    if (job->use_cpdi) {
        // the reference sets use_cpdi = 0 (process_usl.c:264) and nothing
        // fills the corner gradients its CPDI branch reads
        fprintf(stderr, "mpm_gb300: calculate_strainrate_split: the CPDI branch is not supported\n");
        exit(EXIT_FAILURE);
    }
    std::vector<size_t> idx;
    for (size_t i = p_start; i < p_stop; i++)
        if (job->active[i] != 0) idx.push_back(i);
    Stage S(job, (int)idx.size(), 20);
    double *b[8] = {job->b11, job->b12, job->b13, job->b14, job->b21, job->b22, job->b23, job->b24};
    for (size_t k = 0; k < idx.size(); k++) {
        const size_t i = idx[k];
        const int *nn = job->elements[job->in_element[i]].nodes;
        for (int q = 0; q < 8; q++) S.h(q)[k] = b[q][i];
        for (int q = 0; q < 4; q++) {
            S.h(8 + q)[k] = job->nodes[nn[q]].x_t;
            S.h(12 + q)[k] = job->nodes[nn[q]].y_t;
        }
    }
    if (S.n == 0) return;
    S.up();
    strainrate_kernel<<<blocks(S.n), 256, 0, S.stream>>>(S.n, S.dev);
    S.down();
    for (size_t k = 0; k < idx.size(); k++) {
        particle_t &p = job->particles[idx[k]];
        p.exx_t = S.h(16)[k];
        p.exy_t = S.h(17)[k];
        p.eyy_t = S.h(18)[k];
        p.wxy_t = S.h(19)[k];
    }
}

void move_grid_split(job_t *job, size_t n_start, size_t n_stop)
{
    const int n = n_stop > n_start ? (int)(n_stop - n_start) : 0;
    Stage S(job, n, 15);
    for (int k = 0; k < n; k++) {
        const node_t &nd = job->nodes[n_start + k];
        S.h(0)[k] = nd.m;
        S.h(1)[k] = nd.fx;
        S.h(2)[k] = nd.fy;
        S.h(3)[k] = nd.mx_t;
        S.h(4)[k] = nd.my_t;
        S.h(5)[k] = nd.ux;
        S.h(6)[k] = nd.uy;
    }
    if (n == 0) return;
    S.up();
    move_grid_kernel<<<blocks(n), 256, 0, S.stream>>>(n, job->dt, S.dev);
    S.down();
    for (int k = 0; k < n; k++) {
        node_t &nd = job->nodes[n_start + k];
        nd.x_tt = S.h(7)[k];
        nd.y_tt = S.h(8)[k];
        nd.mx_t = S.h(9)[k];
        nd.my_t = S.h(10)[k];
        nd.x_t = S.h(11)[k];
        nd.y_t = S.h(12)[k];
        nd.ux = S.h(13)[k];
        nd.uy = S.h(14)[k];
    }
}

void move_particles_explicit_usl_split(job_t *job, size_t p_start, size_t p_stop)
{
    std::vector<size_t> idx;
    for (size_t i = p_start; i < p_stop; i++)
        if (job->active[i] != 0) idx.push_back(i);
    Stage S(job, (int)idx.size(), 38);
    double *sf[4] = {job->h1, job->h2, job->h3, job->h4};
    for (size_t k = 0; k < idx.size(); k++) {
        const size_t i = idx[k];
        const int *nn = job->elements[job->in_element[i]].nodes;
        for (int j = 0; j < 4; j++) {
            const node_t &nd = job->nodes[nn[j]];
            S.h(j)[k] = sf[j][i];
            S.h(4 + 5 * j)[k] = nd.m;
            S.h(5 + 5 * j)[k] = nd.fx;
            S.h(6 + 5 * j)[k] = nd.fy;
            S.h(7 + 5 * j)[k] = nd.mx_t;
            S.h(8 + 5 * j)[k] = nd.my_t;
        }
        const particle_t &p = job->particles[i];
        S.h(24)[k] = p.x_t;
        S.h(25)[k] = p.y_t;
        S.h(26)[k] = p.x;
        S.h(27)[k] = p.y;
        S.h(28)[k] = p.ux;
        S.h(29)[k] = p.uy;
    }
    if (S.n == 0) return;
    S.up();
    move_particles_kernel<<<blocks(S.n), 256, 0, S.stream>>>(S.n, job->dt, S.dev);
    S.down();
    for (size_t k = 0; k < idx.size(); k++) {
        particle_t &p = job->particles[idx[k]];
        p.x_tt = S.h(30)[k];
        p.y_tt = S.h(31)[k];
        p.x_t = S.h(32)[k];
        p.y_t = S.h(33)[k];
        p.x = S.h(34)[k];
        p.y = S.h(35)[k];
        p.ux = S.h(36)[k];
        p.uy = S.h(37)[k];
    }
}

void update_particle_densities_split(job_t *job, size_t p_start, size_t p_stop)
{
    std::vector<size_t> idx;
    for (size_t i = p_start; i < p_stop; i++)
        if (job->active[i] != 0) idx.push_back(i);
    Stage S(job, (int)idx.size(), 4);
    for (size_t k = 0; k < idx.size(); k++) {
        const particle_t &p = job->particles[idx[k]];
        S.h(0)[k] = p.v;
        S.h(1)[k] = p.exx_t;
        S.h(2)[k] = p.eyy_t;
    }
    if (S.n == 0) return;
    S.up();
    densities_kernel<<<blocks(S.n), 256, 0, S.stream>>>(S.n, job->dt, S.dev);
    S.down();
    for (size_t k = 0; k < idx.size(); k++) job->particles[idx[k]].v = S.h(3)[k];
}

void create_particle_to_element_map_threaded(threadtask_t *task)
{
    job_t *job = task->job;
    const size_t p_start = task->offset, p_stop = task->offset + task->blocksize;
    std::vector<size_t> idx;
    for (size_t i = p_start; i < p_stop; i++)
        if (job->active[i] != 0) idx.push_back(i);
    Stage S(job, (int)idx.size(), 3);
    for (size_t k = 0; k < idx.size(); k++) {
        S.h(0)[k] = job->particles[idx[k]].x;
        S.h(1)[k] = job->particles[idx[k]].y;
    }
    if (S.n > 0) {
        S.up();
        element_map_kernel<<<blocks(S.n), 256, 0, S.stream>>>(S.n, job->h, (double)(job->N - 1), S.dev);
        S.down();
    }
    // the bookkeeping and the log lines of process_usl.c:641-666
    unsigned int changed = 0;
    for (size_t k = 0; k < idx.size(); k++) {
        const size_t i = idx[k];
        const int p = (int)S.h(2)[k];
        if (p != job->in_element[i]) {
            changed = 1;
            if (job->output.log_fd != NULL)
                fprintf(job->output.log_fd, "[%g] Particle %zu @(%g, %g) left element %d, now in element %d.\n",
                        job->t, i, job->particles[i].x, job->particles[i].y, job->in_element[i], p);
        }
        job->in_element[i] = p;
        if (p == -1) {
            if (job->output.log_fd != NULL)
                fprintf(job->output.log_fd, "[%g] Particle %zu outside of grid (%g, %g), marking as inactive.\n",
                        job->t, i, job->particles[i].x, job->particles[i].y);
            job->active[i] = 0;
        }
    }
    job->update_elementlists[task->id] = (int)changed;
}

void map_to_grid_explicit_split(job_t *job, size_t thread_id)
{
    // The calling thread with thread_id 0 maps every thread's lists (the
    // reference's threads each map their own); every caller then meets the
    // others at the job's barrier once per colour, as in the reference, so
    // that all of them return with the nodes complete.
    if (thread_id == 0) {
        const int np = (int)job->num_particles, nn = (int)job->num_nodes;
        // each node's contributions in the order the reference's colour loop
        // adds them: colour, then thread, then list position
        std::vector<int> start((size_t)nn + 1, 0);
        const size_t T = job->num_threads, C = job->num_colors;
        auto for_each = [&](auto &&fn) {
            for (size_t c = 0; c < C; c++)
                for (size_t t = 0; t < T; t++) {
                    const size_t tc = t * C + c;
                    for (size_t q = 0; q < job->particle_by_element_color_lengths[tc]; q++) {
                        const size_t p = job->particle_by_element_color_lists[tc][q];
                        const int *nl = job->elements[job->in_element[p]].nodes;
                        for (int k = 0; k < 4; k++) fn(p, k, nl[k]);
                    }
                }
        };
        for_each([&](size_t, int, int node) { start[(size_t)node + 1]++; });
        for (int k = 0; k < nn; k++) start[(size_t)k + 1] += start[k];
        std::vector<long long> entry((size_t)start[nn]);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for_each([&](size_t p, int k, int node) { entry[(size_t)fill[node]++] = ((long long)p << 2) | k; });

        Stage Pd(job, np, 23), Nd(job, nn, 7);
        double *sf[12] = {job->h1, job->h2, job->h3, job->h4, job->b11, job->b12,
                          job->b13, job->b14, job->b21, job->b22, job->b23, job->b24};
        for (int i = 0; i < np; i++) {
            for (int q = 0; q < 12; q++) Pd.h(q)[i] = sf[q][i];
            const particle_t &p = job->particles[i];
            const double f[11] = {p.m, p.x_t, p.y_t, p.x_tt, p.y_tt, p.bx, p.by, p.sxx, p.sxy, p.syy, p.v};
            for (int q = 0; q < 11; q++) Pd.h(12 + q)[i] = f[q];
        }
        for (int k = 0; k < nn; k++) {
            const node_t &nd = job->nodes[k];
            const double f[7] = {nd.m, nd.mx_t, nd.my_t, nd.mx_tt, nd.my_tt, nd.fx, nd.fy};
            for (int q = 0; q < 7; q++) Nd.h(q)[k] = f[q];
        }
        int *d_start = nullptr;
        long long *d_entry = nullptr;
        check(cudaMalloc(&d_start, start.size() * sizeof(int)), "cudaMalloc");
        check(cudaMalloc(&d_entry, (entry.empty() ? 1 : entry.size()) * sizeof(long long)), "cudaMalloc");
        check(cudaMemcpyAsync(d_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, Nd.stream),
              "copy to device");
        if (!entry.empty())
            check(cudaMemcpyAsync(d_entry, entry.data(), entry.size() * sizeof(long long), cudaMemcpyHostToDevice,
                                  Nd.stream),
                  "copy to device");
        if (np > 0) {
            Pd.up();
            check(cudaStreamSynchronize(Pd.stream), "copy to device");
        }
        if (nn > 0) {
            Nd.up();
            p2g_nodes_kernel<<<blocks(nn), 256, 0, Nd.stream>>>(nn, np, Pd.dev, Nd.dev, d_start, d_entry);
            Nd.down();
        }
        cudaFree(d_start);
        cudaFree(d_entry);
        for (int k = 0; k < nn; k++) {
            node_t &nd = job->nodes[k];
            nd.m = Nd.h(0)[k];
            nd.mx_t = Nd.h(1)[k];
            nd.my_t = Nd.h(2)[k];
            nd.mx_tt = Nd.h(3)[k];
            nd.my_tt = Nd.h(4)[k];
            nd.fx = Nd.h(5)[k];
            nd.fy = Nd.h(6)[k];
        }
    }
    if (job->serialize_barrier != NULL)
        for (size_t c = 0; c < job->num_colors; c++) pthread_barrier_wait(job->serialize_barrier);
}

}  // extern "C"
