#include <algorithm>
// C ABI of the mpm_gb300 library: context lifecycle, host field I/O, stepping,
// timing and error reporting.  See include/mpm_gb300.h for the contract.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <vector>

#include <atomic>
#include <chrono>

#include "mpmg_internal.cuh"

namespace {

void drop_graphs(mpmg_ctx *ctx);   // cached step graphs, recaptured on next use
thread_local char g_last_error[512] = "";

const char *kPhaseNames[PH_COUNT] = {"keys", "sort", "p2g", "grid", "g2p", "fluidity"};

template <typename T>
int dalloc(T **p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        mpmg_set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        return MPMG_ERR_NOMEM;
    }
    return MPMG_OK;
}

int upload(mpmg_ctx *ctx, double *dst, const double *src, size_t n)
{
    if (n == 0) return MPMG_OK;
    MPMG_CHECK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return MPMG_OK;
}

int fill_zero(mpmg_ctx *ctx, void *p, size_t bytes)
{
    if (p == nullptr || bytes == 0) return MPMG_OK;
    MPMG_CHECK(cudaMemsetAsync(p, 0, bytes, ctx->stream));
    return MPMG_OK;
}

// Which state slots each material keeps (the reference's #define maps).
bool material_uses_state(int material, int k)
{
    switch (material) {
    case MPMG_G_LOCAL_MU2:      // g_local_mu2.c:43-53 (gammap, gammadotp)
        return k == 9 || k == 10;
    case MPMG_G_NONLOCAL_MU2:   // g_nonlocal_mu2.c:49-57
        return k == 0 || k == 3 || k == 4 || k == 5 || k == 6 || k == 9 || k == 10;
    case MPMG_G_NONLOCAL:       // g_nonlocal.c:51-61
    case MPMG_G_NONLOCAL_AVG:
        return k == 3 || k == 4 || k == 5 || k == 9 || k == 10;
    case MPMG_DP_RI_MT:         // dp_ri_mt.c:27-29 (szz, gammap, gammadotp)
        return k == 1 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_PLANE_STRAIN:   // g_local_mu2_plane_strain.c:43-51 (szz, beta, gammap, gammadotp)
        return k == 1 || k == 5 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_TRUE_2D:        // g_local_mu2_true_2d.c:43-51 (beta, gammap, gammadotp)
        return k == 5 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_REVERSE:        // g_local_mu2_reverse.c:57-64 (beta, gammap, gammadotp)
        return k == 5 || k == 9 || k == 10;
    case MPMG_G_LOCAL_MU2_EXT:            // g_local_mu2_ext.c:47-57 (mu_t, gf, gflocal, beta, gammap, gammadotp)
        return k == 0 || k == 3 || k == 4 || k == 5 || k == 9 || k == 10;
    default:
        return false;
    }
}

// The step records (one StepParams per simulation, then the status word)
// live in one device block with a pinned host mirror, so a read-back of all
// of them is one copy.
size_t step_record_bytes(const mpmg_ctx *ctx)
{
    return ctx->status_offset + 16;
}

int alloc_step_record(mpmg_ctx *ctx, int count)
{
    ctx->status_offset = ((size_t)count * sizeof(StepParams) + 15) / 16 * 16;
    unsigned char *block = nullptr;
    cudaError_t e = cudaMalloc((void **)&block, step_record_bytes(ctx));
    if (e != cudaSuccess) {
        mpmg_set_error("cudaMalloc of the step record failed: %s", cudaGetErrorString(e));
        return MPMG_ERR_NOMEM;
    }
    ctx->d_params = (StepParams *)block;
    ctx->d_status = (int *)(block + ctx->status_offset);
    e = cudaHostAlloc((void **)&ctx->h_record, step_record_bytes(ctx), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        ctx->h_record = nullptr;
        mpmg_set_error("cudaHostAlloc of the step record failed: %s", cudaGetErrorString(e));
        return MPMG_ERR_NOMEM;
    }
    return MPMG_OK;
}

// The step parameters and the status word of a read-back step record: the
// parameters go to ctx->h_params, device-side errors to their status codes.
int take_record(mpmg_ctx *ctx, const unsigned char *rec)
{
    int st = 0;
    memcpy(&ctx->h_params, rec, sizeof(StepParams));
    memcpy(&st, rec + ctx->status_offset, sizeof(int));
    if (st != 0) {
        // Report each device-side error once; the caller decides whether to go on.
        MPMG_CHECK(cudaMemset(ctx->d_status, 0, sizeof(int)));
    }
    if (st & MPMG_DEV_ERR_SPIN) {
        mpmg_bin_reset(ctx);
        mpmg_set_error("a grid-wide wait (binning scan or fluidity solver) timed out");
        return MPMG_ERR_DEVICE;
    }
    if (st & MPMG_DEV_ERR_BOUNDS) {
        mpmg_set_error("a kernel found an index out of range");
        return MPMG_ERR_DEVICE;
    }
    if (st & MPMG_DEV_ERR_SOLVER) {
        mpmg_set_error("fluidity solve did not reach the relative residual %g in %d iterations",
                       ctx->cfg.solver_tol, ctx->cfg.solver_maxit);
        return MPMG_ERR_SOLVER;
    }
    return MPMG_OK;
}

int sync_status(mpmg_ctx *ctx)
{
    MPMG_CHECK(cudaMemcpyAsync(ctx->h_record, ctx->d_params, step_record_bytes(ctx), cudaMemcpyDeviceToHost,
                               ctx->stream));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    return take_record(ctx, ctx->h_record);
}

struct FieldRef {
    double *ptr;        // device array, or nullptr for an all-zero / computed field
    size_t count;
    int kind;           // 0 device array, 1 zeros, 2 constant by (gravity)
};

int find_field(mpmg_ctx *ctx, const char *name, FieldRef *f, bool for_write)
{
    f->ptr = nullptr;
    f->count = ctx->np;
    f->kind = 0;
    struct { const char *n; double *p; } pf[] = {
        {"x", ctx->x}, {"y", ctx->y}, {"v", ctx->v}, {"v0", ctx->v0}, {"m", ctx->m},
        {"vx", ctx->vx}, {"vy", ctx->vy}, {"sxx", ctx->sxx}, {"sxy", ctx->sxy}, {"syy", ctx->syy},
        {"ux", ctx->ux}, {"uy", ctx->uy}, {"Txx", ctx->sxx}, {"Txy", ctx->sxy}, {"Tyx", ctx->sxy},
        {"Tyy", ctx->syy}, {"ax", ctx->ax}, {"ay", ctx->ay}, {"exx", ctx->exx}, {"exy", ctx->exy},
        {"eyy", ctx->eyy}, {"wxy", ctx->wxy}, {"xl", ctx->xl}, {"yl", ctx->yl}, {"Tzz", ctx->Tzz}};
    for (auto &e : pf) {
        if (strcmp(name, e.n) == 0) {
            if (e.p == nullptr) {
                if (for_write) {
                    mpmg_set_error("field '%s' is not kept by this configuration", name);
                    return MPMG_ERR_UNKNOWN_FIELD;
                }
                f->kind = 1;
            }
            f->ptr = e.p;
            return MPMG_OK;
        }
    }
    if (strcmp(name, "bx") == 0) {
        f->kind = 1;
        return for_write ? MPMG_ERR_UNKNOWN_FIELD : MPMG_OK;
    }
    if (strcmp(name, "by") == 0) {
        f->kind = 2;
        return for_write ? MPMG_ERR_UNKNOWN_FIELD : MPMG_OK;
    }
    if (strncmp(name, "state", 5) == 0 && name[5] != 0) {
        char *end = nullptr;
        long k = strtol(name + 5, &end, 10);
        if (*end == 0 && k >= 0 && k < MPMG_DEPVAR) {
            f->ptr = ctx->state[k];
            if (f->ptr == nullptr) {
                if (for_write) {
                    mpmg_set_error("state slot %ld is not used by this material", k);
                    return MPMG_ERR_UNKNOWN_FIELD;
                }
                f->kind = 1;
            }
            return MPMG_OK;
        }
    }
    f->count = ctx->nn;
    struct { const char *n; double *p; } nf[] = {
        {"node_m", ctx->node_m}, {"node_mx", ctx->node_mx}, {"node_my", ctx->node_my},
        {"node_fx", ctx->node_fx}, {"node_fy", ctx->node_fy}, {"node_vx", ctx->node_vx},
        {"node_vy", ctx->node_vy}, {"node_ax", ctx->node_ax}, {"node_ay", ctx->node_ay},
        {"node_gf", ctx->node_gf}};
    for (auto &e : nf) {
        if (strcmp(name, e.n) == 0) {
            if (e.p == nullptr) {
                if (for_write) {
                    mpmg_set_error("field '%s' is not kept by this configuration", name);
                    return MPMG_ERR_UNKNOWN_FIELD;
                }
                f->kind = 1;
            }
            f->ptr = e.p;
            return MPMG_OK;
        }
    }
    mpmg_set_error("unknown field '%s'", name);
    return MPMG_ERR_UNKNOWN_FIELD;
}

// The body force the reference's time_varying_loads leaves in by after the
// last completed step (loading.c:34-54), or initial_loads before any step.
double current_by(const mpmg_ctx *ctx)
{
    const StepParams &p = ctx->h_params;
    if (ctx->cfg.gravity_mode == MPMG_GRAVITY_CONSTANT) return ctx->cfg.gravity;
    if (p.step_count == 0) return 0.0;
    if ((0.1 + p.step_start_time) > p.t) return -9.8 * ((p.t - p.step_start_time) / 0.1);
    return -9.8;
}

}  // namespace

void mpmg_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int mpmg_cuda_status(cudaError_t e, const char *what)
{
    mpmg_set_error("%s: %s", what, cudaGetErrorString(e));
    return (e == cudaErrorMemoryAllocation) ? MPMG_ERR_NOMEM : MPMG_ERR_CUDA;
}

void mpmg_phase_begin(mpmg_ctx *ctx, int phase)
{
    if (ctx->timing) {
        cudaEventRecord(ctx->ev[2 * phase], ctx->stream);
        ctx->phase_used[phase] = 1;
    }
}

void mpmg_phase_end(mpmg_ctx *ctx, int phase)
{
    if (ctx->timing) cudaEventRecord(ctx->ev[2 * phase + 1], ctx->stream);
}

extern "C" {

const char *mpmg_last_error(void)
{
    return g_last_error;
}

const char *mpmg_status_string(int status)
{
    switch (status) {
    case MPMG_OK: return "ok";
    case MPMG_ERR_SOLVER: return "fluidity solve did not converge";
    case MPMG_ERR_INVALID: return "invalid argument";
    case MPMG_ERR_CUDA: return "CUDA error";
    case MPMG_ERR_NOMEM: return "out of device memory";
    case MPMG_ERR_UNKNOWN_FIELD: return "unknown field";
    case MPMG_ERR_UNSUPPORTED: return "unsupported material or boundary condition";
    case MPMG_ERR_DEVICE: return "device-side error";
    case MPMG_ERR_SCRATCH_LIMIT: return "size exceeds the fixed scratch capacity";
    default: return "unknown status";
    }
}

int mpmg_default_params(int material, double *mp)
{
    if (mp == nullptr) return MPMG_ERR_INVALID;
    for (int i = 0; i < MPMG_MP_COUNT; i++) mp[i] = 0.0;
    mp[MPMG_MP_E] = 1e6;
    mp[MPMG_MP_NU] = 0.3;
    switch (material) {
    case MPMG_ISOLIN:
        return MPMG_OK;
    case MPMG_G_LOCAL_MU2:      // g_local_mu2.c:30-41
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_MU_2] = 0.6435;
        mp[MPMG_MP_I0] = 0.278 / 1.0;
        mp[MPMG_MP_GRAINS_D] = 0.001 * 5;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0f;
        return MPMG_OK;
    case MPMG_G_NONLOCAL_MU2:   // g_nonlocal_mu2.c:32-47
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_A] = 0.48;
        mp[MPMG_MP_MU_2] = 0.6435;
        mp[MPMG_MP_I0] = 0.278;
        mp[MPMG_MP_GRAINS_D] = 0.005;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0;
        return MPMG_OK;
    case MPMG_DP_RI_MT:         // dp_ri_mt.c:66-76 reads E, nu, mu_s from the configuration
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0f;   // dp_ri_mt.c:159 literal
        return MPMG_OK;
    case MPMG_G_LOCAL_MU2_PLANE_STRAIN:   // g_local_mu2_plane_strain.c:27-39 (compile-time there)
    case MPMG_G_LOCAL_MU2_TRUE_2D:        // g_local_mu2_true_2d.c:27-39
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_MU_2] = 0.6435;
        mp[MPMG_MP_I0] = 0.278 / 1.0;
        mp[MPMG_MP_GRAINS_D] = material == MPMG_G_LOCAL_MU2_TRUE_2D ? 0.01 * 5 : 0.001 * 5;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0f;
        return MPMG_OK;
    case MPMG_G_LOCAL_MU2_REVERSE:        // g_local_mu2_reverse.c:33-53 (compile-time there)
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_MU_2] = 0.6435;
        mp[MPMG_MP_I0] = 0.278 / 1.0;
        mp[MPMG_MP_GRAINS_D] = 0.01 * 5;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0f;
        return MPMG_OK;
    case MPMG_G_LOCAL_MU2_EXT:            // g_local_mu2_ext.c:26-45 (compile-time there)
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_A] = 4.8;
        mp[MPMG_MP_MU_2] = 0.6435;
        mp[MPMG_MP_I0] = 0.278 / 1.0;
        mp[MPMG_MP_GRAINS_D] = 0.01 * 5;
        mp[MPMG_MP_RHO_CRITICAL] = 1485.0f;
        return MPMG_OK;
    case MPMG_G_NONLOCAL:       // g_nonlocal.c:31-48 (g_nonlocal_avg.c the same)
    case MPMG_G_NONLOCAL_AVG:
        mp[MPMG_MP_E] = 1e8;
        mp[MPMG_MP_NU] = 0.3;
        mp[MPMG_MP_MU_S] = 0.3819;
        mp[MPMG_MP_GRAINS_RHO] = 2450;
        mp[MPMG_MP_B] = 0.9377 * 20;
        mp[MPMG_MP_A] = 0.48;
        mp[MPMG_MP_GRAINS_D] = 0.01 * 5;
        mp[MPMG_MP_COHESION] = 1e-2;
        return MPMG_OK;
    default:
        mpmg_set_error("unknown material kind %d", material);
        return MPMG_ERR_UNSUPPORTED;
    }
}

int mpmg_config_init(mpmg_config *cfg)
{
    if (cfg == nullptr) return MPMG_ERR_INVALID;
    memset(cfg, 0, sizeof(*cfg));
    cfg->xmax = 1.0;
    cfg->ymax = 1.0;
    cfg->solver_tol = 1e-10;
    cfg->solver_maxit = 20000;
    mpmg_default_params(MPMG_ISOLIN, cfg->mp);
    return MPMG_OK;
}

int mpmg_destroy(mpmg_ctx *ctx)
{
    if (ctx == nullptr) return MPMG_OK;
    cudaSetDevice(ctx->dev);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    double **dp[] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->m, &ctx->v, &ctx->v0, &ctx->sxx,
                     &ctx->sxy, &ctx->syy, &ctx->ux, &ctx->uy, &ctx->Tzz, &ctx->ax, &ctx->ay,
                     &ctx->exx, &ctx->exy, &ctx->eyy, &ctx->wxy, &ctx->xl, &ctx->yl, &ctx->cell_sums,
                     &ctx->node_m, &ctx->node_ax, &ctx->node_ay, &ctx->node_vx, &ctx->node_vy,
                     &ctx->node_mx, &ctx->node_my, &ctx->node_fx, &ctx->node_fy, &ctx->node_gf,
                     &ctx->nl_trial};
    for (double **p : dp) {
        cudaFree(*p);
        *p = nullptr;
    }
    for (int k = 0; k < MPMG_DEPVAR; k++) cudaFree(ctx->state[k]);
    cudaFree(ctx->in_element);
    cudaFree(ctx->active);
    cudaFree(ctx->keys);
    cudaFree(ctx->sorted_keys);
    cudaFree(ctx->perm);
    cudaFree(ctx->cell_start);
    cudaFree(ctx->d_params);      // the step record block (d_status lies inside it)
    if (ctx->h_record) cudaFreeHost(ctx->h_record);
    for (int k = 0; k < MPMG_RECORD_SLOTS; k++) {
        if (ctx->h_ring[k]) cudaFreeHost(ctx->h_ring[k]);
        if (ctx->ring_ev[k]) cudaEventDestroy(ctx->ring_ev[k]);
    }
    if (ctx->rring_h) cudaFreeHost(ctx->rring_h);
    mpmg_bin_free(ctx);
    mpmg_nonlocal_free(ctx);
    mpmg_mixed_free(ctx);
    mpmg_adj_free(ctx);
    if (ctx->batch) {
        cudaFree(ctx->batch->d_members);
        cudaFree(ctx->batch->d_elem_off);
        cudaFree(ctx->batch->d_node_off);
        delete ctx->batch;
        ctx->batch = nullptr;
    }
    drop_graphs(ctx);
    for (int k = 0; k < 2 * PH_COUNT; k++)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MPMG_OK;
}

namespace {

// Checks one simulation's configuration (mpm_init's and the plugins'
// bc_validate checks); n is its particle count.
int validate_config(const mpmg_config *cfg, size_t n)
{
    if (cfg->Nx < 2 || cfg->Ny < 2 || !(cfg->h > 0) || !(cfg->dt > 0) || !(cfg->xmax > 0) ||
        !(cfg->ymax > 0)) {
        mpmg_set_error("grid needs Nx, Ny >= 2 and positive h, dt, xmax, ymax");
        return MPMG_ERR_INVALID;
    }
    if ((double)(cfg->Nx - 1) * (double)(cfg->Ny - 1) >= 2147483647.0 || n >= 2147483647u) {
        mpmg_set_error("grid or particle count exceeds 32-bit indexing");
        return MPMG_ERR_INVALID;
    }
    if (cfg->material < MPMG_ISOLIN || cfg->material > MPMG_G_LOCAL_MU2_REVERSE) {
        mpmg_set_error("unknown material kind %d", cfg->material);
        return MPMG_ERR_UNSUPPORTED;
    }
    if (cfg->bc != MPMG_BOX && cfg->bc != MPMG_SQUARE_SILO) {
        mpmg_set_error("unknown boundary-condition kind %d", cfg->bc);
        return MPMG_ERR_UNSUPPORTED;
    }
    if (cfg->solver_precond != MPMG_PRECOND_MULTIGRID && cfg->solver_precond != MPMG_PRECOND_JACOBI) {
        mpmg_set_error("unknown fluidity preconditioner %d", cfg->solver_precond);
        return MPMG_ERR_INVALID;
    }
    if (cfg->precision < MPMG_PRECISION_FP64 || cfg->precision > MPMG_PRECISION_MIXED_F64NODE) {
        mpmg_set_error("unknown precision %d", cfg->precision);
        return MPMG_ERR_INVALID;
    }
    if (cfg->scheme != MPMG_SCHEME_USL && cfg->scheme != MPMG_SCHEME_MUSL) {
        mpmg_set_error("unknown step scheme %d", cfg->scheme);
        return MPMG_ERR_INVALID;
    }
    if (cfg->scheme == MPMG_SCHEME_MUSL &&
        (cfg->precision != MPMG_PRECISION_FP64 ||
         cfg->material == MPMG_G_NONLOCAL_MU2 || cfg->material == MPMG_G_NONLOCAL ||
         cfg->material == MPMG_G_NONLOCAL_AVG ||
         cfg->material == MPMG_G_LOCAL_MU2_EXT)) {
        mpmg_set_error("the MUSL step runs in the FP64 form for the particle-local materials");
        return MPMG_ERR_UNSUPPORTED;
    }
    if (cfg->bc == MPMG_BOX) {
        // box.c:42-96 bc_validate
        double x0 = cfg->bcf[0], y0 = cfg->bcf[1], w = cfg->bcf[2], hh = cfg->bcf[3];
        if (x0 < 0 || y0 < 0 || x0 > 1.0 || y0 > 1.0 || w < 0 || hh < 0 || x0 + w > 1.0 || y0 + hh > 1.0) {
            mpmg_set_error("box must lie inside the unit fractions of the grid");
            return MPMG_ERR_INVALID;
        }
    }
    return MPMG_OK;
}

int check_device(int device)
{
    int ndev = 0;
    cudaError_t de = cudaGetDeviceCount(&ndev);
    if (de != cudaSuccess || ndev <= device || device < 0) {
        mpmg_set_error("no CUDA device %d available (%s)", device,
                       de != cudaSuccess ? cudaGetErrorString(de) : "device count too small");
        return MPMG_ERR_CUDA;
    }
    return MPMG_OK;
}

}  // namespace

// Device state of the mixed form (one simulation or a batch): FP32 particle
// state lives in ctx->mixed; the context keeps the sort, the step records
// (one per simulation) and the status word.
static int init_mixed_context(mpmg_ctx *ctx, const double *m, const double *v, const double *x, const double *y,
                       const double *vx, const double *vy, const double *sxx, const double *sxy,
                       const double *syy)
{
    const size_t n = ctx->np;
    const int count = ctx->batch ? ctx->batch->count : 1;
    int rc;
    if ((rc = dalloc(&ctx->in_element, n)) != MPMG_OK) return rc;
    if ((rc = dalloc(&ctx->active, n)) != MPMG_OK) return rc;
    if ((rc = dalloc(&ctx->sorted_keys, n)) != MPMG_OK) return rc;
    if ((rc = dalloc(&ctx->perm, n)) != MPMG_OK) return rc;
    if ((rc = dalloc(&ctx->cell_start, ctx->ne + 1)) != MPMG_OK) return rc;
    if (ctx->cfg.store_transients) {
        double **tn[] = {&ctx->node_mx, &ctx->node_my, &ctx->node_fx, &ctx->node_fy};
        for (double **p : tn)
            if ((rc = dalloc(p, ctx->nn)) != MPMG_OK) return rc;
    }
    if ((rc = alloc_step_record(ctx, count)) != MPMG_OK) return rc;
    if ((rc = mpmg_bin_init(ctx)) != MPMG_OK) return rc;
    if ((rc = fill_zero(ctx, ctx->cell_start, (ctx->ne + 1) * sizeof(int))) != MPMG_OK) return rc;
    if ((rc = fill_zero(ctx, ctx->d_status, sizeof(int))) != MPMG_OK) return rc;
    std::vector<StepParams> p0(count);
    for (int k = 0; k < count; k++) {
        const mpmg_config &c = ctx->batch ? ctx->batch->cfg[k] : ctx->cfg;
        p0[k] = StepParams{};
        p0[k].gravity = (c.gravity_mode == MPMG_GRAVITY_CONSTANT) ? c.gravity : 0.0;
    }
    ctx->h_params = p0[0];
    MPMG_CHECK(cudaMemcpyAsync(ctx->d_params, p0.data(), count * sizeof(StepParams), cudaMemcpyHostToDevice,
                               ctx->stream));
    if ((rc = mpmg_mixed_init(ctx, m, v, x, y, vx, vy, sxx, sxy, syy)) != MPMG_OK) return rc;
    return sync_status(ctx);
}

int mpmg_create(const mpmg_config *cfg, size_t n, const double *m, const double *v, const double *x,
                const double *y, const double *vx, const double *vy, const double *sxx,
                const double *sxy, const double *syy, mpmg_ctx **out)
{
    if (out == nullptr || cfg == nullptr) {
        mpmg_set_error("null configuration or output pointer");
        return MPMG_ERR_INVALID;
    }
    *out = nullptr;
    int vrc = validate_config(cfg, n);
    if (vrc != MPMG_OK) return vrc;
    if (n > 0 && (!m || !v || !x || !y || !vx || !vy || !sxx || !sxy || !syy)) {
        mpmg_set_error("null particle array");
        return MPMG_ERR_INVALID;
    }
    vrc = check_device(cfg->device);
    if (vrc != MPMG_OK) return vrc;

    mpmg_ctx *ctx = new (std::nothrow) mpmg_ctx();
    if (ctx == nullptr) return MPMG_ERR_NOMEM;
    ctx->cfg = *cfg;
    if (!(ctx->cfg.solver_tol > 0)) ctx->cfg.solver_tol = 1e-10;
    if (ctx->cfg.solver_maxit <= 0) ctx->cfg.solver_maxit = 20000;
    ctx->dev = cfg->device;
    ctx->np = n;
    ctx->Ex = cfg->Nx - 1;
    ctx->Ey = cfg->Ny - 1;
    ctx->nn = (size_t)cfg->Nx * (size_t)cfg->Ny;
    ctx->ne = (size_t)ctx->Ex * (size_t)ctx->Ey;
    ctx->inv_h = 1.0 / cfg->h;
    int bits = 1;
    while (((size_t)1 << bits) <= ctx->ne) bits++;
    ctx->key_bits = bits;

    // material_init (isolin.c:31-59 / g_local_mu2.c / g_nonlocal_mu2.c / g_nonlocal.c:34-35)
    double E = cfg->mp[MPMG_MP_E], nu = cfg->mp[MPMG_MP_NU];
    ctx->G = E / (2.0 * (1.0 + nu));
    ctx->K = E / (3.0 * (1.0 - 2 * nu));
    ctx->lambda = ctx->K - 2.0 * ctx->G / 3.0;

    int rc;
#define TRY(call)                        \
    do {                                 \
        rc = (call);                     \
        if (rc != MPMG_OK) goto fail;    \
    } while (0)

    if (cudaSetDevice(ctx->dev) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        mpmg_set_error("cannot open CUDA device %d", ctx->dev);
        rc = MPMG_ERR_CUDA;
        goto fail;
    }
    for (int k = 0; k < 2 * PH_COUNT; k++) {
        if (cudaEventCreate(&ctx->ev[k]) != cudaSuccess) {
            rc = MPMG_ERR_CUDA;
            goto fail;
        }
    }
    {
        const bool transients = cfg->store_transients != 0;
        const bool nonlocal = cfg->material == MPMG_G_NONLOCAL_MU2 || cfg->material == MPMG_G_NONLOCAL ||
                              cfg->material == MPMG_G_NONLOCAL_AVG;
        const bool mixed =
            cfg->precision == MPMG_PRECISION_MIXED || cfg->precision == MPMG_PRECISION_MIXED_F64NODE;
        if (mixed && (cfg->material == MPMG_G_NONLOCAL || cfg->material == MPMG_G_NONLOCAL_AVG)) {
            mpmg_set_error("mixed precision supports isolin, g_local_mu2 and g_nonlocal_mu2");
            rc = MPMG_ERR_UNSUPPORTED;
            goto fail;
        }
        if (mixed) {
            TRY(init_mixed_context(ctx, m, v, x, y, vx, vy, sxx, sxy, syy));
            *out = ctx;
            return MPMG_OK;
        }
        double **always[] = {&ctx->x, &ctx->y, &ctx->vx, &ctx->vy, &ctx->m, &ctx->v, &ctx->v0,
                             &ctx->sxx, &ctx->sxy, &ctx->syy, &ctx->ux, &ctx->uy};
        for (double **p : always) TRY(dalloc(p, n));
        if (cfg->material == MPMG_G_LOCAL_MU2) TRY(dalloc(&ctx->Tzz, n));
        for (int k = 0; k < MPMG_DEPVAR; k++)
            if (material_uses_state(cfg->material, k)) TRY(dalloc(&ctx->state[k], n));
        if (transients) {
            TRY(dalloc(&ctx->ax, n));
            TRY(dalloc(&ctx->ay, n));
        }
        // strain rates and start-of-step local coordinates outlive the G2P
        // where a later phase reads them: the nonlocal solve, MUSL's second
        // projection and g_local_mu2_ext's nodal fluidity Laplacian
        const bool keep_rates = transients || nonlocal || cfg->scheme == MPMG_SCHEME_MUSL ||
                                cfg->material == MPMG_G_LOCAL_MU2_EXT;
        if (keep_rates) {
            double **sr[] = {&ctx->exx, &ctx->exy, &ctx->eyy, &ctx->wxy};
            for (double **p : sr) TRY(dalloc(p, n));
            TRY(dalloc(&ctx->xl, n));
            TRY(dalloc(&ctx->yl, n));
        }
        TRY(dalloc(&ctx->in_element, n));
        TRY(dalloc(&ctx->active, n));
        TRY(dalloc(&ctx->keys, n));
        TRY(dalloc(&ctx->sorted_keys, n));
        TRY(dalloc(&ctx->perm, n));
        TRY(dalloc(&ctx->cell_start, ctx->ne + 1));
        TRY(dalloc(&ctx->cell_sums, 20 * ctx->ne));
        double **nodes[] = {&ctx->node_m, &ctx->node_ax, &ctx->node_ay, &ctx->node_vx, &ctx->node_vy,
                            &ctx->node_gf};
        for (double **p : nodes) TRY(dalloc(p, ctx->nn));
        if (transients) {
            double **tn[] = {&ctx->node_mx, &ctx->node_my, &ctx->node_fx, &ctx->node_fy};
            for (double **p : tn) TRY(dalloc(p, ctx->nn));
        }
        TRY(alloc_step_record(ctx, 1));
        TRY(mpmg_bin_init(ctx));
        if (nonlocal) TRY(mpmg_nonlocal_init(ctx));
        if (cfg->material == MPMG_G_NONLOCAL_MU2) TRY(dalloc(&ctx->nl_trial, 5 * n));

        // mpm_init copies (process_usl.c:88-126) and material_init.
        TRY(upload(ctx, ctx->m, m, n));
        TRY(upload(ctx, ctx->v, v, n));
        TRY(upload(ctx, ctx->v0, v, n));
        TRY(upload(ctx, ctx->x, x, n));
        TRY(upload(ctx, ctx->y, y, n));
        TRY(upload(ctx, ctx->vx, vx, n));
        TRY(upload(ctx, ctx->vy, vy, n));
        TRY(upload(ctx, ctx->sxx, sxx, n));
        TRY(upload(ctx, ctx->sxy, sxy, n));
        TRY(upload(ctx, ctx->syy, syy, n));
        TRY(fill_zero(ctx, ctx->ux, n * sizeof(double)));
        TRY(fill_zero(ctx, ctx->uy, n * sizeof(double)));
        TRY(fill_zero(ctx, ctx->Tzz, n * sizeof(double)));
        for (int k = 0; k < MPMG_DEPVAR; k++) TRY(fill_zero(ctx, ctx->state[k], n * sizeof(double)));
        double **zero_p[] = {&ctx->ax, &ctx->ay, &ctx->exx, &ctx->exy, &ctx->eyy, &ctx->wxy, &ctx->xl, &ctx->yl};
        for (double **p : zero_p) TRY(fill_zero(ctx, *p, n * sizeof(double)));
        double **zero_n[] = {&ctx->node_m, &ctx->node_ax, &ctx->node_ay, &ctx->node_vx, &ctx->node_vy,
                             &ctx->node_mx, &ctx->node_my, &ctx->node_fx, &ctx->node_fy, &ctx->node_gf};
        for (double **p : zero_n) TRY(fill_zero(ctx, *p, ctx->nn * sizeof(double)));
        TRY(fill_zero(ctx, ctx->cell_start, (ctx->ne + 1) * sizeof(int)));
        TRY(fill_zero(ctx, ctx->d_status, sizeof(int)));
        StepParams p0 = {};
        ctx->h_params = p0;
        MPMG_CHECK(cudaMemcpyAsync(ctx->d_params, &ctx->h_params, sizeof(StepParams),
                                   cudaMemcpyHostToDevice, ctx->stream));

        // Initial element map (process_usl.c:236-244) on the host copy of x, y.
        int *emap = new (std::nothrow) int[n > 0 ? n : 1];
        int *act = new (std::nothrow) int[n > 0 ? n : 1];
        if (emap == nullptr || act == nullptr) {
            delete[] emap;
            delete[] act;
            rc = MPMG_ERR_NOMEM;
            goto fail;
        }
        for (size_t i = 0; i < n; i++) {
            double xp = x[i], yp = y[i];
            int e = -1;
            if (xp < cfg->xmax && xp >= 0.0 && yp < cfg->ymax && yp >= 0.0) {
                double fx = floor(xp / cfg->h), fy = floor(yp / cfg->h);
                if (fx < (double)ctx->Ex && fy < (double)ctx->Ey) e = (int)(fx + fy * (double)ctx->Ex);
            }
            emap[i] = e;
            act[i] = e < 0 ? 0 : 1;
        }
        cudaError_t ce = cudaMemcpy(ctx->in_element, emap, n * sizeof(int), cudaMemcpyHostToDevice);
        if (ce == cudaSuccess) ce = cudaMemcpy(ctx->active, act, n * sizeof(int), cudaMemcpyHostToDevice);
        delete[] emap;
        delete[] act;
        if (ce != cudaSuccess) {
            rc = mpmg_cuda_status(ce, "initial element map upload");
            goto fail;
        }
        rc = sync_status(ctx);
        if (rc != MPMG_OK) goto fail;
    }
#undef TRY
    *out = ctx;
    return MPMG_OK;
fail:
    mpmg_destroy(ctx);
    return rc;
}

int mpmg_batch_create(int count, const mpmg_config *cfgs, const size_t *counts, const double *m,
                      const double *v, const double *x, const double *y, const double *vx, const double *vy,
                      const double *sxx, const double *sxy, const double *syy, mpmg_ctx **out)
{
    if (out == nullptr || cfgs == nullptr || counts == nullptr || count < 1) {
        mpmg_set_error("batch needs at least one configuration, the particle counts and an output pointer");
        return MPMG_ERR_INVALID;
    }
    *out = nullptr;
    size_t np = 0, ne = 0, nn = 0;
    for (int k = 0; k < count; k++) {
        const mpmg_config &c = cfgs[k];
        int vrc = validate_config(&c, counts[k]);
        if (vrc != MPMG_OK) return vrc;
        if (c.precision != MPMG_PRECISION_MIXED && c.precision != MPMG_PRECISION_MIXED_F64NODE) {
            mpmg_set_error("batch member %d: batches run the mixed-precision form", k);
            return MPMG_ERR_UNSUPPORTED;
        }
        if (c.material != MPMG_ISOLIN && c.material != MPMG_G_LOCAL_MU2 && c.material != MPMG_DP_RI_MT) {
            mpmg_set_error("batch member %d: batches support isolin, g_local_mu2 and dp_ri_mt", k);
            return MPMG_ERR_UNSUPPORTED;
        }
        if (c.precision != cfgs[0].precision || c.material != cfgs[0].material || c.device != cfgs[0].device ||
            c.store_transients != cfgs[0].store_transients) {
            mpmg_set_error("batch member %d: members share the precision, material kind, device and "
                           "transient storage; their grids, parameters, boundaries and time steps may differ",
                           k);
            return MPMG_ERR_INVALID;
        }
        np += counts[k];
        ne += (size_t)(c.Nx - 1) * (size_t)(c.Ny - 1);
        nn += (size_t)c.Nx * (size_t)c.Ny;
    }
    if (np >= 2147483647u || ne >= 2147483647u || nn >= 2147483647u) {
        mpmg_set_error("batch totals exceed 32-bit indexing");
        return MPMG_ERR_INVALID;
    }
    if (np > 0 && (!m || !v || !x || !y || !vx || !vy || !sxx || !sxy || !syy)) {
        mpmg_set_error("null particle array");
        return MPMG_ERR_INVALID;
    }
    int rc = check_device(cfgs[0].device);
    if (rc != MPMG_OK) return rc;

    mpmg_ctx *ctx = new (std::nothrow) mpmg_ctx();
    if (ctx == nullptr) return MPMG_ERR_NOMEM;
    ctx->cfg = cfgs[0];
    ctx->dev = cfgs[0].device;
    ctx->np = np;
    ctx->ne = ne;
    ctx->nn = nn;
    ctx->Ex = cfgs[0].Nx - 1;
    ctx->Ey = cfgs[0].Ny - 1;
    ctx->inv_h = 1.0 / cfgs[0].h;
    int bits = 1;
    while (((size_t)1 << bits) <= ctx->ne) bits++;
    ctx->key_bits = bits;
    {
        const double E = cfgs[0].mp[MPMG_MP_E], nu = cfgs[0].mp[MPMG_MP_NU];
        ctx->G = E / (2.0 * (1.0 + nu));
        ctx->K = E / (3.0 * (1.0 - 2 * nu));
        ctx->lambda = ctx->K - 2.0 * ctx->G / 3.0;
    }
    BatchInfo *b = new (std::nothrow) BatchInfo();
    if (b == nullptr) {
        delete ctx;
        return MPMG_ERR_NOMEM;
    }
    ctx->batch = b;
    b->count = count;
    b->cfg.assign(cfgs, cfgs + count);
    b->poff.assign(count + 1, 0);
    b->eoff.assign(count + 1, 0);
    b->noff.assign(count + 1, 0);
    for (int k = 0; k < count; k++) {
        b->poff[k + 1] = b->poff[k] + counts[k];
        b->eoff[k + 1] = b->eoff[k] + (size_t)(cfgs[k].Nx - 1) * (size_t)(cfgs[k].Ny - 1);
        b->noff[k + 1] = b->noff[k] + (size_t)cfgs[k].Nx * (size_t)cfgs[k].Ny;
    }
    if (cudaSetDevice(ctx->dev) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        mpmg_set_error("cannot open CUDA device %d", ctx->dev);
        rc = MPMG_ERR_CUDA;
        goto fail;
    }
    for (int k = 0; k < 2 * PH_COUNT; k++) {
        if (cudaEventCreate(&ctx->ev[k]) != cudaSuccess) {
            rc = MPMG_ERR_CUDA;
            goto fail;
        }
    }
    rc = init_mixed_context(ctx, m, v, x, y, vx, vy, sxx, sxy, syy);
    if (rc != MPMG_OK) goto fail;
    *out = ctx;
    return MPMG_OK;
fail:
    mpmg_destroy(ctx);
    return rc;
}

int mpmg_batch_count(mpmg_ctx *ctx, int *count)
{
    if (ctx == nullptr || count == nullptr) return MPMG_ERR_INVALID;
    *count = ctx->batch ? ctx->batch->count : 1;
    return MPMG_OK;
}

int mpmg_batch_member(mpmg_ctx *ctx, int member, size_t *first_particle, size_t *num_particles,
                      size_t *first_node, size_t *num_nodes, size_t *first_element, size_t *num_elements)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    const int count = ctx->batch ? ctx->batch->count : 1;
    if (member < 0 || member >= count) {
        mpmg_set_error("member %d outside a batch of %d", member, count);
        return MPMG_ERR_INVALID;
    }
    size_t p0 = 0, p1 = ctx->np, n0 = 0, n1 = ctx->nn, e0 = 0, e1 = ctx->ne;
    if (ctx->batch) {
        const BatchInfo &b = *ctx->batch;
        p0 = b.poff[member], p1 = b.poff[member + 1];
        n0 = b.noff[member], n1 = b.noff[member + 1];
        e0 = b.eoff[member], e1 = b.eoff[member + 1];
    }
    if (first_particle) *first_particle = p0;
    if (num_particles) *num_particles = p1 - p0;
    if (first_node) *first_node = n0;
    if (num_nodes) *num_nodes = n1 - n0;
    if (first_element) *first_element = e0;
    if (num_elements) *num_elements = e1 - e0;
    return MPMG_OK;
}

int mpmg_batch_get_time(mpmg_ctx *ctx, int member, double *t, int *step_number)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    const int count = ctx->batch ? ctx->batch->count : 1;
    if (member < 0 || member >= count) {
        mpmg_set_error("member %d outside a batch of %d", member, count);
        return MPMG_ERR_INVALID;
    }
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    int rc = sync_status(ctx);
    if (rc != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    StepParams p;
    memcpy(&p, ctx->h_record + (size_t)member * sizeof(StepParams), sizeof(StepParams));
    if (t) *t = p.t;
    if (step_number) *step_number = (int)p.step_count;
    return MPMG_OK;
}

}  // extern "C"

namespace {

// The step's own read-back (mpmg_record_ring): one block copies the step
// record (times, step count, solver bookkeeping, device status) into the ring
// slot of the step just completed, in mapped pinned host memory.  The slot's
// first word is a sequence lock: it is set to -1 before the body is written
// and to the step number after it, with system-scope fences between, so that
// a host that reads the step number, copies the body and then reads the same
// step number again has read a body that no later step was writing
// (mpmg_ring_read_slot).  The kernel waits for the step's last kernel
// (programmatic dependent launch) and lets the next step's first kernel start
// its prologue at once.
__global__ void record_ring_kernel(const unsigned char *__restrict__ rec, int bytes,
                                   const StepParams *__restrict__ sp, unsigned char *ring, int slot_bytes,
                                   int slots)
{
    mpmg_pdl_trigger();
    mpmg_pdl_wait();
    const long long step = sp->step_count;
    unsigned char *dst = ring + (size_t)((step - 1 + slots) % slots) * (size_t)slot_bytes;
    if (threadIdx.x == 0) {
        *reinterpret_cast<volatile long long *>(dst) = -1;
        __threadfence_system();
    }
    __syncthreads();
    __threadfence_system();
    for (int i = threadIdx.x * 4; i < bytes; i += blockDim.x * 4)
        *reinterpret_cast<volatile uint32_t *>(dst + 16 + i) = *reinterpret_cast<const uint32_t *>(rec + i);
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) {
        *reinterpret_cast<volatile long long *>(dst) = step;
        __threadfence_system();
    }
}

int launch_one_step(mpmg_ctx *ctx)
{
    int rc = ctx->mixed ? mpmg_mixed_step(ctx) : mpmg_launch_step(ctx);
    if (rc != MPMG_OK || ctx->rring_slots <= 0) return rc;
    MPMG_CHECK(mpmg_launch_pdl(true, record_ring_kernel, dim3(1), dim3(64), 0, ctx->stream,
                               (const unsigned char *)ctx->d_params, (int)step_record_bytes(ctx),
                               (const StepParams *)ctx->d_params, ctx->rring_d, (int)ctx->rring_slot_bytes,
                               ctx->rring_slots));
    ctx->launches += 1;
    return MPMG_OK;
}

int parity(const mpmg_ctx *ctx)
{
    return ctx->mixed ? ctx->mixed->cur : 0;
}

// Captures `steps` consecutive steps (starting at the current buffer parity)
// into an executable graph.  Capturing runs nothing, so the host-side parity
// is put back afterwards.
int capture_steps(mpmg_ctx *ctx, int steps, cudaGraphExec_t *out, long *launches)
{
    const int p0 = parity(ctx);
    const long l0 = ctx->launches;
    MPMG_CHECK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = MPMG_OK;
    for (int k = 0; k < steps && rc == MPMG_OK; k++) rc = launch_one_step(ctx);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (ctx->mixed) ctx->mixed->cur = p0;
    *launches = ctx->launches - l0;
    ctx->launches = l0;
    if (rc != MPMG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return mpmg_cuda_status(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return mpmg_cuda_status(e, "cudaGraphInstantiate");
    return MPMG_OK;
}

// Steps through CUDA graphs: chunks of MPMG_GRAPH_CHUNK steps, then single
// steps.  The nonlocal materials (a cooperative solver launch per step) and
// phase timing run eagerly instead.
bool graphs_apply(const mpmg_ctx *ctx)
{
    const bool nonlocal = ctx->cfg.material == MPMG_G_NONLOCAL_MU2 || ctx->cfg.material == MPMG_G_NONLOCAL ||
                          ctx->cfg.material == MPMG_G_NONLOCAL_AVG;
    return !nonlocal && !ctx->timing;
}

void drop_graphs(mpmg_ctx *ctx)
{
    for (int p = 0; p < 2; p++) {
        if (ctx->graph_chunk[p]) cudaGraphExecDestroy(ctx->graph_chunk[p]);
        if (ctx->graph_single[p]) cudaGraphExecDestroy(ctx->graph_single[p]);
        ctx->graph_chunk[p] = ctx->graph_single[p] = nullptr;
    }
}

int step_with_graphs(mpmg_ctx *ctx, int nsteps)
{
    const int chunk_steps = ctx->graph_steps > 0 ? ctx->graph_steps : MPMG_GRAPH_CHUNK;
    while (nsteps > 0) {
        const int p = parity(ctx);
        const bool chunk = nsteps >= chunk_steps;
        cudaGraphExec_t *g = chunk ? &ctx->graph_chunk[p] : &ctx->graph_single[p];
        long *gl = chunk ? &ctx->graph_chunk_launches[p] : &ctx->graph_single_launches[p];
        if (*g == nullptr) {
            int rc = capture_steps(ctx, chunk ? chunk_steps : 1, g, gl);
            if (rc != MPMG_OK) return rc;
        }
        MPMG_CHECK(cudaGraphLaunch(*g, ctx->stream));
        ctx->launches += *gl;
        const int done = chunk ? chunk_steps : 1;
        if (ctx->mixed && (done & 1)) ctx->mixed->cur ^= 1;
        nsteps -= done;
    }
    return MPMG_OK;
}

}  // namespace

extern "C" {

// Online tuning of the mixed step's tiles and launch shape, on the
// simulation itself.  First the tiles: every batched-P2G tile (elements a
// block, particles staged a pass; batches only, a single simulation runs the
// fused P2G) with every G2P tile, at the default launch shape; then, with
// the fastest tiles, the launch shape: G2P blocks per SM x steps per graph.
// Each candidate runs a warm-up graph and then steps_per_trial steps
// (rounded up to whole graphs) timed with CUDA events.  No knob changes any
// result, so the trajectory is the one an untuned run takes; it advances by
// every trial's steps.
int mpmg_autotune(mpmg_ctx *ctx, int steps_per_trial, mpmg_tuning *best)
{
    if (ctx == nullptr || best == nullptr || steps_per_trial < 1) return MPMG_ERR_INVALID;
    if (ctx->mixed == nullptr || !graphs_apply(ctx)) {
        mpmg_set_error("autotuning applies to the mixed forms stepped through CUDA graphs");
        return MPMG_ERR_UNSUPPORTED;
    }
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    memset(best, 0, sizeof(*best));
    const int chunk_opts[3] = {4, 8, 16};
    const int g2p_tiles[2] = {256, 128};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    MPMG_CHECK(cudaEventCreate(&e0));
    MPMG_CHECK(cudaEventCreate(&e1));
    int rc = MPMG_OK, tried = 0, advanced = 0;
    double default_ms = 0;
    // one timed trial of the current configuration; ms per step in *per
    auto trial_of = [&](int ch, double *per) -> int {
        ctx->graph_steps = ch;
        drop_graphs(ctx);
        const int trial = ((steps_per_trial + ch - 1) / ch) * ch;
        int r = step_with_graphs(ctx, ch);                    // capture and warm up
        if (r != MPMG_OK) return r;
        if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) return MPMG_ERR_CUDA;
        r = step_with_graphs(ctx, trial);
        if (r != MPMG_OK) return r;
        if (cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            return MPMG_ERR_CUDA;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *per = ms / trial;
        advanced += ch + trial;
        tried += 1;
        return MPMG_OK;
    };
    // tiles, at the default launch shape
    const int p2g_n = ctx->batch ? mpmg_mixed_p2g_variants() : 1;
    double best_ms = 1e30;
    int best_pv = 0, best_tile = g2p_tiles[0];
    for (int pv = 0; pv < p2g_n && rc == MPMG_OK; pv++) {
        for (int t = 0; t < 2 && rc == MPMG_OK; t++) {
            rc = mpmg_mixed_set_tiles(ctx, pv, g2p_tiles[t]);
            if (rc != MPMG_OK) break;
            double per = 0;
            rc = trial_of(MPMG_GRAPH_CHUNK, &per);
            if (rc != MPMG_OK) break;
            if (pv == 0 && t == 0) default_ms = per;
            if (per < best_ms) {
                best_ms = per;
                best_pv = pv;
                best_tile = g2p_tiles[t];
            }
        }
    }
    // launch shape, with those tiles
    int best_ps = 0, best_ch = MPMG_GRAPH_CHUNK, last_ps = -1;
    if (rc == MPMG_OK) rc = mpmg_mixed_set_tiles(ctx, best_pv, best_tile);
    const int per_sm_max = ctx->mixed->g2p_per_sm_max;
    best_ps = per_sm_max;
    for (int a = 1; a <= per_sm_max && rc == MPMG_OK; a++) {
        const int ps = mpmg_mixed_set_g2p_per_sm(ctx, a);
        if (ps == last_ps) continue;   // clamped to one already tried
        last_ps = ps;
        for (int b = 0; b < 3 && rc == MPMG_OK; b++) {
            double per = 0;
            rc = trial_of(chunk_opts[b], &per);
            if (rc != MPMG_OK) break;
            if (per < best_ms) {
                best_ms = per;
                best_ps = ps;
                best_ch = chunk_opts[b];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == MPMG_OK) rc = sync_status(ctx);
    if (tried > 0 && rc == MPMG_OK) {
        mpmg_mixed_set_tiles(ctx, best_pv, best_tile);
        mpmg_mixed_set_g2p_per_sm(ctx, best_ps);
        ctx->graph_steps = best_ch;
    } else {
        mpmg_mixed_set_tiles(ctx, 0, g2p_tiles[0]);
        ctx->graph_steps = MPMG_GRAPH_CHUNK;
        best_pv = 0;
        best_tile = g2p_tiles[0];
        best_ps = ctx->mixed->g2p_per_sm_max;
        best_ch = MPMG_GRAPH_CHUNK;
    }
    drop_graphs(ctx);
    best->g2p_blocks_per_sm = best_ps;
    best->graph_steps = best_ch;
    best->ms_per_step = best_ms < 1e30 ? best_ms : 0.0;
    best->default_ms_per_step = default_ms;
    best->candidates = tried;
    best->steps_advanced = advanced;
    if (ctx->batch) mpmg_mixed_p2g_shape(best_pv, &best->p2g_elements, &best->p2g_stage);
    best->g2p_tile = best_tile;
    return rc;
}

int mpmg_step(mpmg_ctx *ctx, int nsteps)
{
    if (ctx == nullptr || nsteps < 0) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    if (graphs_apply(ctx)) return step_with_graphs(ctx, nsteps);
    for (int k = 0; k < nsteps; k++) {
        for (int ph = 0; ph < PH_COUNT; ph++) ctx->phase_used[ph] = 0;
        int rc = launch_one_step(ctx);
        if (rc != MPMG_OK) return rc;
        if (ctx->timing) {
            MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
            for (int ph = 0; ph < PH_COUNT; ph++) {
                if (!ctx->phase_used[ph]) continue;
                float ms = 0;
                MPMG_CHECK(cudaEventElapsedTime(&ms, ctx->ev[2 * ph], ctx->ev[2 * ph + 1]));
                ctx->phase_ms[ph] += ms;
                ctx->phase_launches[ph] += 1;
            }
        }
    }
    return MPMG_OK;
}

int mpmg_synchronize(mpmg_ctx *ctx)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    return sync_status(ctx);
}

int mpmg_get_field(mpmg_ctx *ctx, const char *name, double *host_out)
{
    if (ctx == nullptr || name == nullptr || host_out == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    FieldRef f;
    int rc;
    if (ctx->mixed) {
        rc = sync_status(ctx);
        if (rc != MPMG_OK) return rc;
        rc = mpmg_mixed_get(ctx, name, host_out);
        if (rc != MPMG_ERR_UNKNOWN_FIELD) return rc;
    }
    rc = find_field(ctx, name, &f, false);
    if (rc != MPMG_OK) return rc;
    rc = sync_status(ctx);
    if (rc != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    if (f.kind == 1) {
        for (size_t i = 0; i < f.count; i++) host_out[i] = 0.0;
    } else if (f.kind == 2) {
        double by = current_by(ctx);
        for (size_t i = 0; i < f.count; i++) host_out[i] = by;
    } else if (f.count > 0) {
        MPMG_CHECK(cudaMemcpy(host_out, f.ptr, f.count * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return MPMG_OK;
}

int mpmg_get_fields(mpmg_ctx *ctx, int count, const char *const *names, double *const *host_out)
{
    if (ctx == nullptr || count < 0 || (count > 0 && (names == nullptr || host_out == nullptr)))
        return MPMG_ERR_INVALID;
    for (int k = 0; k < count; k++)
        if (names[k] == nullptr || host_out[k] == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    std::vector<char> done(count > 0 ? count : 1, 0);
    if (ctx->mixed) {
        int rc = sync_status(ctx);
        if (rc != MPMG_OK) return rc;
        bool *flags = new bool[count > 0 ? count : 1];
        rc = mpmg_mixed_get_many(ctx, count, names, host_out, flags);
        for (int k = 0; k < count; k++) done[k] = flags[k];
        delete[] flags;
        if (rc != MPMG_OK) return rc;
    }
    for (int k = 0; k < count; k++) {
        if (done[k]) continue;
        int rc = mpmg_get_field(ctx, names[k], host_out[k]);
        if (rc != MPMG_OK) return rc;
    }
    return MPMG_OK;
}

int mpmg_set_field(mpmg_ctx *ctx, const char *name, const double *host_in)
{
    if (ctx == nullptr || name == nullptr || host_in == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    if (ctx->mixed) return mpmg_mixed_set(ctx, name, host_in);
    FieldRef f;
    int rc = find_field(ctx, name, &f, true);
    if (rc != MPMG_OK) return rc;
    if (f.count > 0)
        MPMG_CHECK(cudaMemcpyAsync(f.ptr, host_in, f.count * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    return MPMG_OK;
}

int mpmg_get_map(mpmg_ctx *ctx, int *in_element, int *active)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    if (ctx->mixed) return mpmg_mixed_get_map(ctx, in_element, active);
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    if (in_element && ctx->np)
        MPMG_CHECK(cudaMemcpy(in_element, ctx->in_element, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
    if (active && ctx->np)
        MPMG_CHECK(cudaMemcpy(active, ctx->active, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
    return MPMG_OK;
}

int mpmg_set_map(mpmg_ctx *ctx, const int *in_element, const int *active)
{
    if (ctx == nullptr || in_element == nullptr || active == nullptr) return MPMG_ERR_INVALID;
    if (ctx->mixed) {
        mpmg_set_error("the mixed-precision form derives the element map from positions");
        return MPMG_ERR_UNSUPPORTED;
    }
    for (size_t i = 0; i < ctx->np; i++) {
        if (active[i] && (in_element[i] < 0 || (size_t)in_element[i] >= ctx->ne)) {
            mpmg_set_error("active particle %zu has element %d outside the grid", i, in_element[i]);
            return MPMG_ERR_INVALID;
        }
    }
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    if (ctx->np) {
        MPMG_CHECK(cudaMemcpy(ctx->in_element, in_element, ctx->np * sizeof(int), cudaMemcpyHostToDevice));
        MPMG_CHECK(cudaMemcpy(ctx->active, active, ctx->np * sizeof(int), cudaMemcpyHostToDevice));
    }
    return MPMG_OK;
}

int mpmg_get_sort(mpmg_ctx *ctx, int *sorted_keys, int *perm, int *cell_start)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    if (sorted_keys && ctx->np) {
        if (ctx->mixed) {
            // The mixed step does not store the sorted keys: they are the keys
            // it sorted (the element array of the buffer before the last
            // step's swap), taken in permutation order.
            std::vector<int> p(ctx->np), k(ctx->np);
            const int *keys = ctx->mixed->cur ? ctx->in_element : ctx->active;
            MPMG_CHECK(cudaMemcpy(p.data(), ctx->perm, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
            MPMG_CHECK(cudaMemcpy(k.data(), keys, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
            for (size_t j = 0; j < ctx->np; j++) sorted_keys[j] = k[p[j]];
        } else {
            MPMG_CHECK(cudaMemcpy(sorted_keys, ctx->sorted_keys, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
        }
    }
    if (perm && ctx->np) {
        MPMG_CHECK(cudaMemcpy(perm, ctx->perm, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
        if (ctx->mixed) {
            // The mixed form's permutation indexes the storage it sorted (the
            // buffer before the last step's swap); report particle indices.
            float4 *rec = new float4[ctx->np];
            cudaError_t e = cudaMemcpy(rec, ctx->mixed->D[1 - ctx->mixed->cur], ctx->np * sizeof(float4),
                                       cudaMemcpyDeviceToHost);
            if (e == cudaSuccess)
                for (size_t k = 0; k < ctx->np; k++) perm[k] = mpmg_float_bits(rec[perm[k]].z);
            delete[] rec;
            if (e != cudaSuccess) return mpmg_cuda_status(e, "mixed permutation read-back");
        }
    }
    if (cell_start)
        MPMG_CHECK(cudaMemcpy(cell_start, ctx->cell_start, (ctx->ne + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    return MPMG_OK;
}

int mpmg_get_time(mpmg_ctx *ctx, double *t, int *step_number)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    int rc = sync_status(ctx);
    if (rc != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    if (t) *t = ctx->h_params.t;
    if (step_number) *step_number = (int)ctx->h_params.step_count;
    return MPMG_OK;
}

int mpmg_record_async(mpmg_ctx *ctx, int slot)
{
    if (ctx == nullptr || slot < 0 || slot >= MPMG_RECORD_SLOTS) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    if (ctx->h_ring[slot] == nullptr) {
        MPMG_CHECK(cudaHostAlloc((void **)&ctx->h_ring[slot], step_record_bytes(ctx), cudaHostAllocDefault));
        MPMG_CHECK(cudaEventCreateWithFlags(&ctx->ring_ev[slot], cudaEventDisableTiming));
    }
    MPMG_CHECK(cudaMemcpyAsync(ctx->h_ring[slot], ctx->d_params, step_record_bytes(ctx), cudaMemcpyDeviceToHost,
                               ctx->stream));
    MPMG_CHECK(cudaEventRecord(ctx->ring_ev[slot], ctx->stream));
    return MPMG_OK;
}

int mpmg_record_ring(mpmg_ctx *ctx, int slots)
{
    if (ctx == nullptr || slots < 0 || slots > (1 << 20)) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    if (ctx->rring_h != nullptr) {
        MPMG_CHECK(cudaFreeHost(ctx->rring_h));
        ctx->rring_h = nullptr;
        ctx->rring_d = nullptr;
    }
    ctx->rring_slots = 0;
    drop_graphs(ctx);          // the captured steps gain or lose the record launch
    if (slots == 0) return MPMG_OK;
    const size_t slot_bytes = (16 + step_record_bytes(ctx) + 15) / 16 * 16;
    MPMG_CHECK(cudaHostAlloc((void **)&ctx->rring_h, slots * slot_bytes, cudaHostAllocMapped));
    memset(ctx->rring_h, 0, slots * slot_bytes);
    MPMG_CHECK(cudaHostGetDevicePointer((void **)&ctx->rring_d, ctx->rring_h, 0));
    ctx->rring_slot_bytes = slot_bytes;
    ctx->rring_slots = slots;
    return MPMG_OK;
}

int mpmg_ring_read_slot(const void *slot_ptr, size_t body_bytes, long long step_number, void *out,
                        double timeout_s, void (*copy)(void *, const void *, size_t))
{
    if (slot_ptr == nullptr || out == nullptr || step_number < 1) return MPMG_ERR_INVALID;
    const unsigned char *slot = static_cast<const unsigned char *>(slot_ptr);
    const volatile long long *seq = reinterpret_cast<const volatile long long *>(slot);
    // bounded wait: the step may still be queued behind others; -1 marks a
    // slot whose body is being written (this step's or a later one's)
    const auto t0 = std::chrono::steady_clock::now();
    long long seen;
    while ((seen = *seq) < step_number) {
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > timeout_s) {
            mpmg_set_error("step %lld's record did not arrive", step_number);
            return MPMG_ERR_DEVICE;
        }
    }
    if (seen != step_number) {
        mpmg_set_error("step %lld's ring slot was overwritten by step %lld before it was read", step_number,
                       seen);
        return MPMG_ERR_INVALID;
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    if (copy != nullptr) copy(out, slot + 16, body_bytes);
    else memcpy(out, slot + 16, body_bytes);
    std::atomic_thread_fence(std::memory_order_acquire);
    seen = *seq;
    if (seen != step_number) {
        mpmg_set_error("step %lld's ring slot was overwritten (sequence %lld) while it was read", step_number,
                       seen);
        return MPMG_ERR_INVALID;
    }
    return MPMG_OK;
}

int mpmg_record_ring_wait(mpmg_ctx *ctx, long long step_number, double *t, int *step_out)
{
    if (ctx == nullptr || ctx->rring_slots <= 0 || step_number < 1) return MPMG_ERR_INVALID;
    const unsigned char *slot =
        ctx->rring_h + (size_t)((step_number - 1) % ctx->rring_slots) * ctx->rring_slot_bytes;
    std::vector<unsigned char> rec(step_record_bytes(ctx));
    int rc = mpmg_ring_read_slot(slot, rec.size(), step_number, rec.data(), 10.0, nullptr);
    if (rc == MPMG_ERR_DEVICE) {
        cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e != cudaSuccess && e != cudaErrorNotReady) return mpmg_cuda_status(e, "record ring");
        return rc;
    }
    if (rc == MPMG_ERR_INVALID) {
        mpmg_set_error("step %lld's ring slot was overwritten (read the ring within %d steps)", step_number,
                       ctx->rring_slots);
        return rc;
    }
    rc = take_record(ctx, rec.data());
    if (rc != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    if (t) *t = ctx->h_params.t;
    if (step_out) *step_out = (int)ctx->h_params.step_count;
    return rc;
}

int mpmg_record_wait(mpmg_ctx *ctx, int slot, double *t, int *step_number)
{
    if (ctx == nullptr || slot < 0 || slot >= MPMG_RECORD_SLOTS || ctx->h_ring[slot] == nullptr)
        return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    MPMG_CHECK(cudaEventSynchronize(ctx->ring_ev[slot]));
    int rc = take_record(ctx, ctx->h_ring[slot]);
    if (rc != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    if (t) *t = ctx->h_params.t;
    if (step_number) *step_number = (int)ctx->h_params.step_count;
    return rc;
}

int mpmg_set_time(mpmg_ctx *ctx, double t, int step_number)
{
    if (ctx == nullptr || step_number < 0) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    const int count = ctx->batch ? ctx->batch->count : 1;
    std::vector<StepParams> p(count);
    MPMG_CHECK(cudaMemcpy(p.data(), ctx->d_params, count * sizeof(StepParams), cudaMemcpyDeviceToHost));
    for (int k = 0; k < count; k++) {
        const mpmg_config &c = ctx->batch ? ctx->batch->cfg[k] : ctx->cfg;
        p[k].t = t;
        p[k].step_count = step_number;
        // body force the next step uses (the FP64 form recomputes it on the device)
        if (c.gravity_mode == MPMG_GRAVITY_CONSTANT) p[k].gravity = c.gravity;
        else if (step_number == 0) p[k].gravity = 0.0;
        else if ((0.1 + p[k].step_start_time) > t) p[k].gravity = -9.8 * ((t - p[k].step_start_time) / 0.1);
        else p[k].gravity = -9.8;
    }
    ctx->h_params = p[0];
    MPMG_CHECK(cudaMemcpy(ctx->d_params, p.data(), count * sizeof(StepParams), cudaMemcpyHostToDevice));
    return MPMG_OK;
}

int mpmg_sizes(mpmg_ctx *ctx, size_t *num_particles, size_t *num_nodes, size_t *num_elements)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    if (num_particles) *num_particles = ctx->np;
    if (num_nodes) *num_nodes = ctx->nn;
    if (num_elements) *num_elements = ctx->ne;
    return MPMG_OK;
}

int mpmg_material_only(mpmg_ctx *ctx)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    if (ctx->cfg.material == MPMG_G_NONLOCAL_MU2 || ctx->cfg.material == MPMG_G_NONLOCAL ||
        ctx->cfg.material == MPMG_G_NONLOCAL_AVG ||
        ctx->cfg.material == MPMG_G_LOCAL_MU2_EXT || ctx->mixed) {
        mpmg_set_error("material-only update is defined for local materials in FP64");
        return MPMG_ERR_UNSUPPORTED;
    }
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    int rc = mpmg_launch_material_only(ctx);
    if (rc != MPMG_OK) return rc;
    return sync_status(ctx);
}

int mpmg_get_stream(mpmg_ctx *ctx, void **stream)
{
    if (ctx == nullptr || stream == nullptr) return MPMG_ERR_INVALID;
    *stream = (void *)ctx->stream;
    return MPMG_OK;
}

int mpmg_enable_phase_timing(mpmg_ctx *ctx, int enable)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    ctx->timing = enable ? 1 : 0;
    for (int k = 0; k < PH_COUNT; k++) {
        ctx->phase_ms[k] = 0;
        ctx->phase_launches[k] = 0;
    }
    return MPMG_OK;
}

int mpmg_phase_count(void)
{
    return PH_COUNT;
}

const char *mpmg_phase_name(int phase)
{
    return (phase >= 0 && phase < PH_COUNT) ? kPhaseNames[phase] : "";
}

int mpmg_phase_times(mpmg_ctx *ctx, double *ms, long *launches)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    for (int k = 0; k < PH_COUNT; k++) {
        if (ms) ms[k] = ctx->phase_ms[k];
        if (launches) launches[k] = ctx->phase_launches[k];
        ctx->phase_ms[k] = 0;
        ctx->phase_launches[k] = 0;
    }
    return MPMG_OK;
}

int mpmg_last_solve(mpmg_ctx *ctx, int *iterations, double *rel_residual)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    int rc = sync_status(ctx);
    if (iterations) *iterations = ctx->h_params.solve_iters;
    if (rel_residual) *rel_residual = ctx->h_params.solve_rel_resid;
    return rc;
}

int mpmg_launch_count(mpmg_ctx *ctx, long *launches, int reset)
{
    if (ctx == nullptr) return MPMG_ERR_INVALID;
    if (launches) *launches = ctx->launches;
    if (reset) ctx->launches = 0;
    return MPMG_OK;
}

}  // extern "C"

namespace {

// Eight independent FMA chains per thread, so that the FP64 pipe, not the
// chains' latency, sets the rate.
__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = (threadIdx.x + c) * 1e-9;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += x[c];
    if (s == 12345.0) out[0] = s;   // never true; keeps the chains live
}

}  // namespace

extern "C" int mpmg_measure_fp64_rate(int device, double *flops_per_s)
{
    if (flops_per_s == nullptr) return MPMG_ERR_INVALID;
    MPMG_CHECK(cudaSetDevice(device));
    int sms = 0;
    MPMG_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    double *out = nullptr;
    MPMG_CHECK(cudaMalloc(&out, sizeof(double)));
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = MPMG_OK;
    cudaError_t err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double best = 0;
    for (int r = 0; r < 4 && err == cudaSuccess; r++) {
        cudaEventRecord(e0, s);
        fp64_fma_probe_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1, s);
        err = cudaEventSynchronize(e1);
        float ms = 0;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
        if (err == cudaSuccess && r > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3));
    }
    if (err != cudaSuccess) rc = mpmg_cuda_status(err, "FP64 rate probe");
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    *flops_per_s = best;
    return rc;
}
