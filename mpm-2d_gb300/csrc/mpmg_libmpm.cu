// libmpm-compatible entry points (include/mpm_libmpm.h) over the flat C ABI.
//
// The host-side bookkeeping follows the reference's libmpm so that a driver
// and plugins built against it see the same job_t: mpm_init
// (libmpm/process_usl.c:68-280), find_filled_elements (:677-723),
// mpm_cleanup (:974-1004), initial_loads and time_varying_loads
// (libmpm/loading.c:21-54).  The time step itself runs on the GPU through an
// mpmg_ctx kept in a side table keyed by the job pointer, so job_t keeps the
// reference's layout.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mpm_libmpm.h"

void mpmg_set_error(const char *fmt, ...);   // mpmg_api.cu

static_assert(sizeof(particle_t) == 1280, "particle_t layout (libmpm/particle.h)");
static_assert(sizeof(node_t) == 152, "node_t layout (libmpm/node.h)");
static_assert(sizeof(element_t) == 1504, "element_t layout (libmpm/element.h)");
static_assert(sizeof(job_t) == 800, "job_t layout (libmpm/process.h)");
static_assert(sizeof(threadtask_t) == 96, "threadtask_t layout (libmpm/process.h)");
static_assert(offsetof(particle_t, T) == 160 && offsetof(particle_t, state) == 392, "particle_t offsets");
static_assert(offsetof(job_t, in_element) == 176 && offsetof(job_t, h1) == 192, "job_t offsets");
static_assert(offsetof(job_t, material) == 584 && offsetof(job_t, boundary) == 656, "job_t offsets");

namespace {

// exitcodes.h:12-24 of the reference
enum { EXIT_ERROR_CS_SOL = 0x02, EXIT_ERROR_MATERIAL_FILE = 0x21, EXIT_ERROR_BC_PROPS = 0x22 };

const double kEmodDefault = 1e6;   // libmpm/material.h:12 (the default dt only)

struct GpuJob {
    mpmg_ctx *ctx = nullptr;
    int material = -1;
    int device = 0;                // the context's CUDA device
    double gravity_next = 0.0;     // what time_varying_loads last computed
};

std::mutex g_jobs_mutex;
std::unordered_map<job_t *, GpuJob> g_jobs;

GpuJob *find_job(job_t *job)
{
    std::lock_guard<std::mutex> lock(g_jobs_mutex);
    auto it = g_jobs.find(job);
    return it == g_jobs.end() ? nullptr : &it->second;
}

std::string basename_noext(const char *path)
{
    if (path == nullptr) return "";
    std::string s(path);
    size_t slash = s.find_last_of('/');
    if (slash != std::string::npos) s = s.substr(slash + 1);
    size_t dot = s.find('.');
    if (dot != std::string::npos) s = s.substr(0, dot);
    return s;
}

int material_kind(const char *file)
{
    std::string b = basename_noext(file);
    if (b == "isolin") return MPMG_ISOLIN;
    if (b == "g_local_mu2") return MPMG_G_LOCAL_MU2;
    if (b == "g_nonlocal_mu2") return MPMG_G_NONLOCAL_MU2;
    if (b == "g_nonlocal" || b == "g_nonlocalxs71") return MPMG_G_NONLOCAL;   // xs71: the same code
    if (b == "g_nonlocal_avg" || b == "g_nonlocal_bicgstab") return MPMG_G_NONLOCAL_AVG;
    if (b == "dp_ri_mt") return MPMG_DP_RI_MT;
    if (b == "g_local_mu2_plane_strain") return MPMG_G_LOCAL_MU2_PLANE_STRAIN;
    if (b == "g_local_mu2_true_2d") return MPMG_G_LOCAL_MU2_TRUE_2D;
    if (b == "g_local_mu2_ext") return MPMG_G_LOCAL_MU2_EXT;
    if (b == "g_local_mu2_reverse") return MPMG_G_LOCAL_MU2_REVERSE;
    return -1;
}

int bc_kind(const char *file)
{
    std::string b = basename_noext(file);
    if (b == "box") return MPMG_BOX;
    if (b == "square_silo") return MPMG_SQUARE_SILO;
    return -1;
}

// Slots of particle_t::state each material keeps (the plugins' #define maps).
bool uses_state(int material, int k)
{
    switch (material) {
    case MPMG_G_LOCAL_MU2: return k == 9 || k == 10;
    case MPMG_G_NONLOCAL_MU2: return k == 0 || k == 3 || k == 4 || k == 5 || k == 6 || k == 9 || k == 10;
    case MPMG_G_NONLOCAL:
    case MPMG_G_NONLOCAL_AVG: return k == 3 || k == 4 || k == 5 || k == 9 || k == 10;
    case MPMG_DP_RI_MT: return k == 1 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_PLANE_STRAIN: return k == 1 || k == 5 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_TRUE_2D:
    case MPMG_G_LOCAL_MU2_REVERSE: return k == 5 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_EXT: return k == 0 || k == 3 || k == 4 || k == 5 || k == 9 || k == 10;
    default: return false;
    }
}

double ramp_gravity(const job_t *job)
{
    // loading.c:38-42
    if ((0.1 + job->step_start_time) > job->t) return -9.8 * ((job->t - job->step_start_time) / 0.1);
    return -9.8;
}

void builtin_material_init(job_t *) {}
void builtin_calculate_stress(job_t *) {}

int report(int rc)
{
    if (rc != MPMG_OK) fprintf(stderr, "mpm_gb300: %s (%s)\n", mpmg_status_string(rc), mpmg_last_error());
    return rc;
}

}  // namespace

// CUDA device of the job's attached context, 0 when none is attached (the
// phase functions of csrc/mpmg_split.cu run there).
int mpmg_libmpm_job_device(job_t *job)
{
    GpuJob *gj = find_job(job);
    return gj != nullptr ? gj->device : 0;
}

extern "C" {

job_t *mpm_init(int N, double h, particle_t *particles, size_t num_particles, double t)
{
    job_t *job = (job_t *)calloc(1, sizeof(job_t));
    job->t = 0;
    job->t_stop = t;
    job->frame = 0;
    job->N = (size_t)N;
    job->h = h;
    job->num_nodes = (size_t)N * (size_t)N;
    job->num_particles = num_particles;
    job->num_elements = (size_t)(N - 1) * (size_t)(N - 1);

    job->particles = (particle_t *)calloc(num_particles ? num_particles : 1, sizeof(particle_t));
    memcpy(job->particles, particles, num_particles * sizeof(particle_t));
    for (size_t i = 0; i < num_particles; i++) {
        particle_t *p = &job->particles[i];
        p->real_sxx = p->sxx;
        p->real_sxy = p->sxy;
        p->real_syy = p->syy;
        p->exx_t = p->exy_t = p->eyy_t = p->wxy_t = 0;
        p->Fxx = 1;
        p->Fxy = 0;
        p->Fyx = 0;
        p->Fyy = 1;
        p->ux = p->uy = 0;
        p->material_data = NULL;
        p->id = i;
        p->state[9] = 0;
        p->state[10] = 0;
        memset(p->corners, 0, sizeof(p->corners));
        p->color = 0;
    }

    job->nodes = (node_t *)calloc(job->num_nodes, sizeof(node_t));
    for (size_t i = 0; i < job->num_nodes; i++) {
        int ii = (int)(i % (size_t)N), jj = (int)(i / (size_t)N);
        job->nodes[i].x = ii * h;
        job->nodes[i].y = jj * h;
    }

    const size_t Ne = (size_t)N - 1;
    job->elements = (element_t *)calloc(job->num_elements ? job->num_elements : 1, sizeof(element_t));
    for (size_t e = 0; e < job->num_elements; e++) {
        size_t r = e / Ne, c = e % Ne;
        int n0 = (int)(r * (size_t)N + c);
        element_t *el = &job->elements[e];
        el->nodes[0] = n0;
        el->nodes[1] = n0 + 1;
        el->nodes[2] = n0 + 1 + N;
        el->nodes[3] = n0 + N;
        el->color = (int)(2 * (r % 2) + (c % 2));
        for (int k = 0; k < 8; k++) el->neighbors[k] = -1;
        // process_usl.c:172-197 (row/column indices written as in the reference)
        if (r != Ne) {
            el->neighbors[2] = (int)((c) * Ne + (r + 1));
            if (c != Ne) el->neighbors[1] = (int)((c + 1) * Ne + (r + 1));
            if (c != 0) el->neighbors[3] = (int)((c - 1) * Ne + (r + 1));
        }
        if (r != 0) {
            el->neighbors[6] = (int)((c) * Ne + (r - 1));
            if (c != Ne) el->neighbors[7] = (int)((c + 1) * Ne + (r - 1));
            if (c != 0) el->neighbors[5] = (int)((c - 1) * Ne + (r - 1));
        }
        if (c != Ne) el->neighbors[0] = (int)((c + 1) * Ne + r);
        if (c != 0) el->neighbors[4] = (int)((c - 1) * Ne + r);
    }
    job->num_colors = 4;
    job->color_indices = (size_t *)calloc(job->num_colors, sizeof(size_t));

    size_t np = num_particles ? num_particles : 1;
    job->in_element = (int *)malloc(np * sizeof(int));
    job->active = (int *)malloc(np * sizeof(int));
    double **sf[] = {&job->h1, &job->h2, &job->h3, &job->h4, &job->b11, &job->b12, &job->b13, &job->b14,
                     &job->b21, &job->b22, &job->b23, &job->b24};
    for (double **a : sf) *a = (double *)calloc(np, sizeof(double));
    job->vec_len = NODAL_DOF * (int)job->num_nodes;
    job->u_dirichlet = (double *)calloc((size_t)NODAL_DOF * job->num_nodes, sizeof(double));
    job->u_dirichlet_mask = (int *)calloc((size_t)NODAL_DOF * job->num_nodes, sizeof(int));
    job->node_number_override = (int *)malloc((size_t)job->vec_len * sizeof(int));
    for (int k = 0; k < job->vec_len; k++) job->node_number_override[k] = k;

    // Initial element map (process_usl.c:236-244): WHICH_ELEMENT4 on the unit square.
    for (size_t i = 0; i < num_particles; i++) {
        double x = job->particles[i].x, y = job->particles[i].y;
        int e = -1;
        if (x < 1.0 && x >= 0.0 && y < 1.0 && y >= 0.0) {
            double fx = floor(x / h), fy = floor(y / h);
            if (fx < (double)Ne && fy < (double)Ne) e = (int)(fx + fy * (double)Ne);
        }
        job->in_element[i] = e;
        job->active[i] = (e < 0) ? 0 : 1;
    }
    for (size_t i = 0; i < num_particles; i++) {
        particle_t *p = &job->particles[i];
        p->v0 = p->v;
        p->r1_initial[0] = 0.5 * sqrt(p->v0);
        p->r1_initial[1] = 0;
        p->r2_initial[0] = 0;
        p->r2_initial[1] = 0.5 * sqrt(p->v0);
    }
    // process_usl.c:261
    if (num_particles > 0)
        job->dt = 0.4 * job->h * sqrt(job->particles[0].m / (job->particles[0].v * kEmodDefault));
    job->use_cpdi = 0;
    job->material.num_fp64_props = 0;
    job->material.num_int_props = 0;
    job->material.fp64_props = NULL;
    job->material.int_props = NULL;
    job->material.material_filename = NULL;
    job->material.material_init = builtin_material_init;
    job->material.calculate_stress = builtin_calculate_stress;
    job->step_number = 0;
    job->step_start_time = job->t;
    return job;
}

void find_filled_elements(job_t *job)
{
    for (size_t c = 0; c < job->num_colors; c++) job->color_indices[c] = 0;
    for (size_t i = 0; i < job->num_particles; i++) {
        if (job->active[i] == 0) continue;
        element_t *el = &job->elements[job->in_element[i]];
        el->filled = 1;
        el->n++;
        el->m += job->particles[i].m;
    }
    for (size_t e = 0; e < job->num_elements; e++) {
        element_t *el = &job->elements[e];
        if (el->filled) el->color_idx = (int)job->color_indices[el->color]++;
    }
    if (job->particle_by_element_color_lengths == NULL || job->particle_by_element_color_lists == NULL)
        return;
    size_t T = job->num_threads ? job->num_threads : 1;
    for (size_t k = 0; k < T * job->num_colors; k++) job->particle_by_element_color_lengths[k] = 0;
    for (size_t i = 0; i < job->num_particles; i++) {
        if (job->active[i] == 0) continue;
        const element_t *el = &job->elements[job->in_element[i]];
        size_t tc = ((size_t)el->color_idx % T) * job->num_colors + (size_t)el->color;
        job->particle_by_element_color_lists[tc][job->particle_by_element_color_lengths[tc]++] = i;
    }
}

void initial_loads(job_t *job)
{
    for (size_t i = 0; i < job->num_particles; i++) {
        job->particles[i].bx = 0;
        job->particles[i].by = 0;
        job->particles[i].material = 1;   // M_DRUCKER_PRAGER (material.h:19)
    }
}

void time_varying_loads(job_t *job)
{
    double g = ramp_gravity(job);
    GpuJob *gj = find_job(job);
    if (gj != nullptr && gj->ctx != nullptr) {
        // The device applies the same ramp; the host copy is written when the
        // particles are brought back (mpm_gpu_sync_host).
        gj->gravity_next = g;
        return;
    }
    for (size_t i = 0; i < job->num_particles; i++) {
        job->particles[i].bx = 0;
        job->particles[i].by = g;
    }
}

// The step scheme a job's context is created with: the entry point the
// driver calls decides (explicit_mpm_step_usl_threaded or
// explicit_mpm_step_musl_threaded).
static thread_local int t_attach_scheme = MPMG_SCHEME_USL;

int mpm_gpu_attach(job_t *job)
{
    if (job == nullptr) return MPMG_ERR_INVALID;
    if (find_job(job) != nullptr) return MPMG_OK;
    int mat = material_kind(job->material.material_filename);
    int bc = bc_kind(job->boundary.bc_filename);
    if (mat < 0 || bc < 0) {
        mpmg_set_error("no device implementation of material '%s' / boundary conditions '%s'",
                       job->material.material_filename ? job->material.material_filename : "(builtin)",
                       job->boundary.bc_filename ? job->boundary.bc_filename : "(builtin)");
        return MPMG_ERR_UNSUPPORTED;
    }
    mpmg_config cfg;
    mpmg_config_init(&cfg);
    cfg.scheme = t_attach_scheme;
    cfg.Nx = cfg.Ny = (int)job->N;
    cfg.h = job->h;
    cfg.dt = job->dt;
    cfg.material = mat;
    mpmg_default_params(mat, cfg.mp);
    if (mat != MPMG_G_NONLOCAL && mat != MPMG_G_NONLOCAL_AVG) {
        // E and nu from the configuration (isolin.c:46-51, g_local_mu2.c:131-140);
        // g_nonlocal.c fixes them at compile time.
        if (job->material.num_fp64_props < 2) {
            mpmg_set_error("material needs at least 2 properties (E, nu)");
            return MPMG_ERR_INVALID;
        }
        cfg.mp[MPMG_MP_E] = job->material.fp64_props[0];
        cfg.mp[MPMG_MP_NU] = job->material.fp64_props[1];
    }
    if (mat == MPMG_DP_RI_MT) {
        // dp_ri_mt.c:66-76
        if (job->material.num_fp64_props < 3) {
            mpmg_set_error("dp_ri_mt needs at least 3 properties (E, nu, mu_s)");
            return MPMG_ERR_INVALID;
        }
        cfg.mp[MPMG_MP_MU_S] = job->material.fp64_props[2];
    }
    cfg.bc = bc;
    size_t need_f = (bc == MPMG_BOX) ? 4 : 3, need_i = (bc == MPMG_BOX) ? 4 : 0;
    if (job->boundary.num_fp64_props != need_f || job->boundary.num_int_props < need_i) {
        mpmg_set_error("boundary conditions need %zu float and %zu integer properties", need_f, need_i);
        return MPMG_ERR_INVALID;
    }
    for (size_t k = 0; k < need_f; k++) cfg.bcf[k] = job->boundary.fp64_props[k];
    for (size_t k = 0; k < need_i; k++) cfg.bci[k] = job->boundary.int_props[k];

    size_t n = job->num_particles;
    std::vector<double> f[9];
    for (auto &v : f) v.resize(n ? n : 1);
    for (size_t i = 0; i < n; i++) {
        const particle_t *p = &job->particles[i];
        f[0][i] = p->m; f[1][i] = p->v; f[2][i] = p->x; f[3][i] = p->y; f[4][i] = p->x_t;
        f[5][i] = p->y_t; f[6][i] = p->sxx; f[7][i] = p->sxy; f[8][i] = p->syy;
    }
    mpmg_ctx *ctx = nullptr;
    int rc = mpmg_create(&cfg, n, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(),
                         f[5].data(), f[6].data(), f[7].data(), f[8].data(), &ctx);
    if (rc != MPMG_OK) return rc;
    std::vector<double> tmp(n ? n : 1);
    auto put = [&](const char *name, auto getter) {
        for (size_t i = 0; i < n; i++) tmp[i] = getter(job->particles[i]);
        return mpmg_set_field(ctx, name, tmp.data());
    };
    rc = put("ux", [](const particle_t &p) { return p.ux; });
    if (rc == MPMG_OK) rc = put("uy", [](const particle_t &p) { return p.uy; });
    if (rc == MPMG_OK) rc = put("v0", [](const particle_t &p) { return p.v0; });
    if (rc == MPMG_OK && mat == MPMG_G_LOCAL_MU2) rc = put("Tzz", [](const particle_t &p) { return p.T[ZZ]; });
    for (int k = 0; k < DEPVAR && rc == MPMG_OK; k++) {
        if (!uses_state(mat, k)) continue;
        for (size_t i = 0; i < n; i++) tmp[i] = job->particles[i].state[k];
        char name[16];
        snprintf(name, sizeof(name), "state%d", k);
        rc = mpmg_set_field(ctx, name, tmp.data());
    }
    if (rc == MPMG_OK) rc = mpmg_set_map(ctx, job->in_element, job->active);
    // Before the first step the reference's bodies carry initial_loads' zero;
    // afterwards time_varying_loads' ramp.
    if (rc == MPMG_OK) rc = mpmg_set_time(ctx, job->t, job->t > 0 ? 1 : 0);
    if (rc != MPMG_OK) {
        mpmg_destroy(ctx);
        return rc;
    }
    std::lock_guard<std::mutex> lock(g_jobs_mutex);
    GpuJob &gj = g_jobs[job];
    gj.ctx = ctx;
    gj.material = mat;
    gj.device = cfg.device;
    gj.gravity_next = ramp_gravity(job);
    return MPMG_OK;
}

int mpm_gpu_sync_host(job_t *job)
{
    GpuJob *gj = find_job(job);
    if (gj == nullptr) return MPMG_ERR_INVALID;
    mpmg_ctx *ctx = gj->ctx;
    size_t n = job->num_particles;
    std::vector<double> a(n ? n : 1);
    struct Field { const char *name; size_t off; };
    const Field fields[] = {
        {"x", offsetof(particle_t, x)}, {"y", offsetof(particle_t, y)}, {"v", offsetof(particle_t, v)},
        {"vx", offsetof(particle_t, x_t)}, {"vy", offsetof(particle_t, y_t)},
        {"sxx", offsetof(particle_t, sxx)}, {"sxy", offsetof(particle_t, sxy)},
        {"syy", offsetof(particle_t, syy)}, {"ux", offsetof(particle_t, ux)}, {"uy", offsetof(particle_t, uy)},
        {"by", offsetof(particle_t, by)}};
    for (const Field &f : fields) {
        int rc = mpmg_get_field(ctx, f.name, a.data());
        if (rc != MPMG_OK) return rc;
        for (size_t i = 0; i < n; i++) *(double *)((char *)&job->particles[i] + f.off) = a[i];
    }
    if (gj->material == MPMG_G_LOCAL_MU2) {
        int rc = mpmg_get_field(ctx, "Tzz", a.data());
        if (rc != MPMG_OK) return rc;
        for (size_t i = 0; i < n; i++) {
            particle_t *p = &job->particles[i];
            p->T[XX] = p->sxx;
            p->T[XY] = p->T[YX] = p->sxy;
            p->T[YY] = p->syy;
            p->T[ZZ] = a[i];
        }
    }
    for (int k = 0; k < DEPVAR; k++) {
        if (!uses_state(gj->material, k)) continue;
        char name[16];
        snprintf(name, sizeof(name), "state%d", k);
        int rc = mpmg_get_field(ctx, name, a.data());
        if (rc != MPMG_OK) return rc;
        for (size_t i = 0; i < n; i++) job->particles[i].state[k] = a[i];
    }
    for (size_t i = 0; i < n; i++) job->particles[i].bx = 0;
    int rc = mpmg_get_map(ctx, job->in_element, job->active);
    if (rc != MPMG_OK) return rc;
    std::vector<double> nm(job->num_nodes), nvx(job->num_nodes), nvy(job->num_nodes);
    if ((rc = mpmg_get_field(ctx, "node_m", nm.data())) != MPMG_OK) return rc;
    if ((rc = mpmg_get_field(ctx, "node_vx", nvx.data())) != MPMG_OK) return rc;
    if ((rc = mpmg_get_field(ctx, "node_vy", nvy.data())) != MPMG_OK) return rc;
    for (size_t k = 0; k < job->num_nodes; k++) {
        job->nodes[k].m = nm[k];
        job->nodes[k].x_t = nvx[k];
        job->nodes[k].y_t = nvy[k];
    }
    return MPMG_OK;
}

int mpm_gpu_step(job_t *job, int nsteps)
{
    int rc = mpm_gpu_attach(job);
    if (rc != MPMG_OK) return rc;
    GpuJob *gj = find_job(job);
    rc = mpmg_step(gj->ctx, nsteps);
    if (rc != MPMG_OK) return rc;
    for (int k = 0; k < nsteps; k++) job->t += job->dt;   // process_usl.c:522, step by step
    return mpmg_synchronize(gj->ctx);
}

int mpm_adj_forward_tape(job_t *job, int nsteps, int checkpoint_every)
{
    int rc = mpm_gpu_attach(job);
    if (rc != MPMG_OK) return rc;
    GpuJob *gj = find_job(job);
    rc = mpmg_adj_forward_tape(gj->ctx, nsteps, checkpoint_every);
    if (rc != MPMG_OK) return rc;
    for (int k = 0; k < nsteps; k++) job->t += job->dt;   // process_usl.c:522, step by step
    return MPMG_OK;
}

int mpm_adj_backward(job_t *job, const double *dl_dx, const double *dl_dy, double *dl_dtheta)
{
    GpuJob *gj = find_job(job);
    if (gj == nullptr || gj->ctx == nullptr) {
        mpmg_set_error("job has no taped GPU run (mpm_adj_forward_tape)");
        return MPMG_ERR_INVALID;
    }
    return mpmg_adj_backward(gj->ctx, dl_dx, dl_dy, dl_dtheta);
}

int mpm_gpu_detach(job_t *job)
{
    mpmg_ctx *ctx = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_jobs_mutex);
        auto it = g_jobs.find(job);
        if (it == g_jobs.end()) return MPMG_OK;
        ctx = it->second.ctx;
        g_jobs.erase(it);
    }
    return mpmg_destroy(ctx);
}

static void threaded_step(threadtask_t *task, int scheme)
{
    job_t *job = task->job;
    int serial = (job->serialize_barrier == NULL) ? 1 : (pthread_barrier_wait(job->serialize_barrier) ==
                                                         PTHREAD_BARRIER_SERIAL_THREAD);
    if (serial) {
        t_attach_scheme = scheme;
        int rc = mpm_gpu_step(job, 1);
        t_attach_scheme = MPMG_SCHEME_USL;
        // The driver writes a frame after this step when t reaches the next
        // sample time (src/main.c:955), and the state when the run ends.
        if (rc == MPMG_OK) {
            double rate = job->output.sample_rate_hz;
            bool frame_due = rate > 0 && job->t >= (job->frame / rate);
            if (frame_due || job->t >= job->t_stop) rc = mpm_gpu_sync_host(job);
        }
        if (rc != MPMG_OK) {
            report(rc);
            exit(rc == MPMG_ERR_SOLVER ? EXIT_ERROR_CS_SOL : EXIT_ERROR_MATERIAL_FILE);
        }
    }
    if (job->serialize_barrier != NULL) pthread_barrier_wait(job->serialize_barrier);
}

void explicit_mpm_step_usl_threaded(void *arg)
{
    threaded_step((threadtask_t *)arg, MPMG_SCHEME_USL);
}

void explicit_mpm_step_musl_threaded(void *arg)
{
    threaded_step((threadtask_t *)arg, MPMG_SCHEME_MUSL);
}

void mpm_cleanup(job_t *job)
{
    mpm_gpu_detach(job);
    free(job->nodes);
    free(job->particles);
    free(job->elements);
    free(job->in_element);
    free(job->active);
    double *sf[] = {job->h1, job->h2, job->h3, job->h4, job->b11, job->b12, job->b13, job->b14,
                    job->b21, job->b22, job->b23, job->b24};
    for (double *a : sf) free(a);
    free(job->u_dirichlet);
    free(job->u_dirichlet_mask);
    free(job->node_number_override);
    free(job->color_indices);
}

}  // extern "C"
