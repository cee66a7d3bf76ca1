// Nonlocal granular fluidity on the GPU (reference: solve_diffusion_part and
// calculate_stress of materialsrc/g_nonlocal_mu2.c:126-578, and the older
// operator variant materialsrc/g_nonlocal.c:103-592).
//
// The reference assembles a sparse matrix from particle quadrature every step
// and factorises it with CXSparse's LU.  Here the same operator
//     K = sum_p v_p [ xi_p^-2 N N^T + grad N grad N^T ]  (+ 1e-10 I for mu2)
// is kept as 10 unique entries of each element's symmetric 4x4 block plus a
// 4-entry right-hand side, summed over the element's particle segment in
// sorted order (one thread per element, fixed order).  The system is solved
// matrix-free by Jacobi-preconditioned CG in one cooperative persistent
// kernel: every node applies its four elements' rows, inner products are
// per-block partial sums reduced in a fixed order (deterministic), and all
// grid-wide waits are bounded.  The unknowns are the nodes with mass above
// the reference's threshold (g_nonlocal_mu2.c:365-381: m > 0; g_nonlocal.c:
// m > 1e-10).  The initial guess is zero, like the reference's direct solve,
// or with mpmg_config.solver_warm_start the previous step's nodal fluidity,
// except on rows that no element touches, whose solution is zero; the
// stopping test is the same relative residual either way.
#include "mpmg_internal.cuh"
#include "mpmg_materials.cuh"

// Level table of the multigrid preconditioner (pcg_mg_kernel), built at
// set-up: level l has Nx x Ny nodes, C of them per block; its node arrays
// start at node g of the global pools and its per-block arrays at float sm
// of a block's shared memory.
constexpr int kMgMaxLevels = 16;

struct MgLevel {
    int Nx, Ny, nn, C;
    int b0;                // first block that owns nodes of the level (blocks b0, b0 + 1, ...
                           // own C nodes each)
    int cx, cy;            // coarsened from the finer level along x, y (level 0: 0)
    int local;             // 1: block 0 holds the whole level (C = nn) in shared memory
    int g;                 // first node of the level in the global pools
    int sm;                // shared memory (floats): spread level: its b, z1, res; held
                           // level: its rows (coef[9][nn], l1inv[nn])
    int smv;               // held level: its b, z1, res, zf (shared memory, floats)
};

struct MgPlan {
    int L, nblocks, total; // levels, blocks, nodes over all levels
    int Lg;                // first level held by block 0 (levels Lg .. L - 1)
    int sm_zf0, sm_vec, sm_fp64;   // shared memory (floats): level 0's own V-cycle
                                   // results; the held levels' vectors (also the
                                   // reduction scratch and the staging area of the
                                   // spread phases); the FP64 region
    MgLevel lv[kMgMaxLevels];
    float *coef;           // [9][total]: 9-point rows, q = 3 (dj + 1) + (di + 1)
    float *rsum;           // [total]: row sums
    float *l1inv;          // [total]: inverse absolute row sums (0: not an unknown)
    unsigned long long *z1, *res, *zf;   // [total] tagged words each
    unsigned int *tag;     // tag counter
};

// Nodes [n0, n0 + cnt) of level lv owned by block b (cnt <= 0: none).
__host__ __device__ inline void mg_own_range(const MgLevel &lv, int b, int &n0, int &cnt)
{
    n0 = (b - lv.b0) * lv.C;
    cnt = b < lv.b0 ? 0 : (lv.nn - n0 < lv.C ? lv.nn - n0 : lv.C);
}

namespace {

constexpr int kSolveThreads = 256;
constexpr long long kSpinLimit = 20000000;   // polls per grid barrier (~1 s)

// Upper-triangle index of (a, b) in the 10-entry symmetric block.
__device__ __forceinline__ int sym_index(int a, int b)
{
    if (a > b) { int t = a; a = b; b = t; }
    // rows: (0,0..3)=0..3, (1,1..3)=4..6, (2,2..3)=7..8, (3,3)=9
    const int row_start[4] = {0, 4, 7, 9};
    return row_start[a] + (b - a);
}

__global__ void nonlocal_bulk_kernel(int n, mat::NonlocalParams np, const double *__restrict__ sxx,
                                     const double *__restrict__ sxy, const double *__restrict__ syy,
                                     double *__restrict__ eta, double *__restrict__ gf_bulk,
                                     double *__restrict__ xisq)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double e, g, xi;
    mat::nonlocal_bulk(np, sxx[i], sxy[i], syy[i], e, g, xi);
    eta[i] = e;
    gf_bulk[i] = g;
    xisq[i] = xi;
}

// Element blocks and right-hand sides (g_nonlocal_mu2.c:418-507): per
// particle, v (xi^-2 s_r s_c + grad s_r . grad s_c) and v gf_local xi^-2 s_r.
// With s = (ox oy, a oy, a b, ox b) (ox = 1 - a, oy = 1 - b), h grad s is
// ((-oy, -ox), (oy, -a), (b, a), (-b, ox)), so every grad s_r . grad s_c h^2
// is a combination of 1, a, a^2, b, b^2: the element sums five moments of v
// (sum v, v a, v a^2, v b, v b^2) and forms the ten gradient entries from
// them once, instead of per particle.  The kernel is bound by the FP64 pipe
// (1/64 of the FP32 rate on GB300); the mass part stays per particle.
__global__ void __launch_bounds__(128) assemble_kernel(
    int ne, int Ex, double inv_h, int dense_only, const int *__restrict__ cell_start,
    const uint32_t *__restrict__ perm, const double *__restrict__ xl, const double *__restrict__ yl,
    const double *__restrict__ v, const double *__restrict__ dense, const double *__restrict__ gfl,
    const double *__restrict__ xisq, double *__restrict__ elem_k, double *__restrict__ elem_f)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int k0 = cell_start[e], k1 = cell_start[e + 1];
    if (k0 == k1) return;
    double K[10], F[4];
#pragma unroll
    for (int k = 0; k < 10; k++) K[k] = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = 0;
    double m0 = 0, ma = 0, maa = 0, mb = 0, mbb = 0;
    for (int k = k0; k < k1; k++) {
        const int i = (int)perm[k];
        if (dense_only && dense[i] == 0) continue;
        const double a = xl[i], b = yl[i];
        const double ox = 1 - a, oy = 1 - b;
        const double s[4] = {ox * oy, a * oy, a * b, ox * b};
        const double vol = v[i], w = vol * xisq[i];
        const double fv = w * gfl[i];
        double ws[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            F[r] = fma(fv, s[r], F[r]);
            ws[r] = w * s[r];
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
#pragma unroll
            for (int c = r; c < 4; c++) K[sym_index(r, c)] = fma(ws[r], s[c], K[sym_index(r, c)]);
        }
        const double va = vol * a, vb = vol * b;
        m0 += vol;
        ma += va;
        mb += vb;
        maa = fma(va, a, maa);
        mbb = fma(vb, b, mbb);
    }
    // sum v grad s_r . grad s_c h^2 from the moments, rows (0,0..3),
    // (1,1..3), (2,2..3), (3,3)
    const double g02 = (maa - ma) + (mbb - mb);
    const double gg[10] = {
        (2 * m0 - 2 * ma + maa) + (mbb - 2 * mb),       // oy^2 + ox^2
        (ma - maa) - (m0 - 2 * mb + mbb),               // ox a - oy^2
        g02,                                            // -oy b - ox a
        (mb - mbb) - (m0 - 2 * ma + maa),               // oy b - ox^2
        (m0 - 2 * mb + mbb) + maa,                      // oy^2 + a^2
        (mb - mbb) - maa,                               // oy b - a^2
        g02,                                            // -oy b - a ox
        mbb + maa,                                      // b^2 + a^2
        (ma - maa) - mbb,                               // ox a - b^2
        mbb + (m0 - 2 * ma + maa)};                     // b^2 + ox^2
    const double ih2 = inv_h * inv_h;
#pragma unroll
    for (int k = 0; k < 10; k++) elem_k[(size_t)k * ne + e] = fma(gg[k], ih2, K[k]);
#pragma unroll
    for (int k = 0; k < 4; k++) elem_f[(size_t)k * ne + e] = F[k];
    (void)Ex;
}

struct SolveArgs {
    int Nx, Ny, Ex, Ey, ne;
    double dof_tol;      // node is an unknown when m > dof_tol
    double shift;        // diagonal shift (1e-10 for g_nonlocal_mu2)
    double tol;          // relative residual
    int maxit;
    const double *node_m;
    const int *cell_start;
    const double *elem_k, *elem_f;
    double *x, *r, *p, *q, *dinv;
    double *w;           // A u of the current residual
    double *u;           // D^-1 r
    double *coef;        // 9-point rows, coef[k * nn + n], k = 3 (dj + 1) + (di + 1)
    double *partials;    // [4][nblocks]
    unsigned int *barrier;
    int *status;
    StepParams *sp;
};

// Block-wide sum of up to three values in a fixed order; result valid in
// thread 0.  One warp adds: lane l sums the values of threads l, l + 32, ...
// then the lanes combine in a shuffle tree.  (GB300 issues FP64 at 1/64 of
// the FP32 rate, so the reduction keeps its FP64 adds to one warp rather
// than a tree in every warp.)
__device__ __forceinline__ void block_sum3(double &a, double &b, double &c)
{
    __shared__ double sh[3][kSolveThreads];
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    sh[2][threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double x = sh[0][lane], y = sh[1][lane], z = sh[2][lane];
#pragma unroll
        for (int k = 1; k < kSolveThreads / 32; k++) {
            x += sh[0][lane + 32 * k];
            y += sh[1][lane + 32 * k];
            z += sh[2][lane + 32 * k];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
            z += __shfl_down_sync(0xffffffffu, z, off);
        }
        a = x;
        b = y;
        c = z;
    }
    __syncthreads();
}

// Sums slot s of the per-block partials in a fixed order; every block gets
// the same value.
__device__ __forceinline__ double grid_total(const double *partials, int slot, int nblocks)
{
    __shared__ double sh[kSolveThreads / 32];
    __shared__ double result;
    double acc = 0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) acc += __ldcg(partials + (size_t)slot * nblocks + k);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) sh[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < kSolveThreads / 32; k++) t += sh[k];
        result = t;
    }
    __syncthreads();
    double out = result;
    __syncthreads();
    return out;
}

// Slots a, b, c of the per-block partials summed in one pass by one warp
// (lane l takes partials l, l + 32, ..., then a shuffle tree): the same fixed
// order in every block, so every block gets the same three values.
__device__ __forceinline__ void grid_total3(const double *partials, int a, int b, int c, int nblocks, double &ta,
                                            double &tb, double &tc)
{
    __shared__ double res[3];
    if (threadIdx.x < 32) {
        double x = 0, y = 0, z = 0;
        for (int k = threadIdx.x; k < nblocks; k += 32) {
            x += __ldcg(partials + (size_t)a * nblocks + k);
            y += __ldcg(partials + (size_t)b * nblocks + k);
            z += __ldcg(partials + (size_t)c * nblocks + k);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
            z += __shfl_down_sync(0xffffffffu, z, off);
        }
        if (threadIdx.x == 0) {
            res[0] = x;
            res[1] = y;
            res[2] = z;
        }
    }
    __syncthreads();
    ta = res[0];
    tb = res[1];
    tc = res[2];
    __syncthreads();
}

// Row of node (i, j) as a 9-point stencil and its right-hand side: the four
// elements around the node (south-west, south-east, north-west, north-east),
// each element's corners in order.  The node is corner a = TR, TL, BR, BL of
// them; corner b of an element lies at offset (bx, by) from its BL node, so
// every stencil index is a compile-time constant.
__device__ __forceinline__ void build_row(const SolveArgs &S, int i, int j, double cf[9], double *rhs)
{
    constexpr int qx[4] = {-1, 0, -1, 0}, qy[4] = {-1, -1, 0, 0};   // element offset of each quadrant
    constexpr int qa[4] = {2, 3, 1, 0};                             // the node's corner in it
    constexpr int bx[4] = {0, 1, 1, 0}, by[4] = {0, 0, 1, 1};       // corner offsets BL BR TR TL
    double f = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ci = i + qx[q], cj = j + qy[q];
        if (ci < 0 || cj < 0 || ci >= S.Ex || cj >= S.Ey) continue;
        const int e = cj * S.Ex + ci;
        if (S.cell_start[e] == S.cell_start[e + 1]) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int di = qx[q] + bx[b], dj = qy[q] + by[b];
            cf[3 * (dj + 1) + (di + 1)] += S.elem_k[(size_t)sym_index(qa[q], b) * S.ne + e];
        }
        f += S.elem_f[(size_t)qa[q] * S.ne + e];
    }
    *rhs = f;
}

// dinv == +0 (not an unknown) tested on the integer pipe: dinv is either a
// positive reciprocal or +0 by construction.
__device__ __forceinline__ bool is_zero(double d)
{
    return __double_as_longlong(d) == 0;
}

// (A v)(n) from the stored 9-point row.  v of the neighbours is written by
// other blocks between grid barriers, so it is read through L2 (__ldcg).
// Missing neighbours (outside the grid) have zero coefficients and are
// skipped by index, so the row costs nine FP64 FMAs and no comparisons on the
// FP64 pipe (GB300 runs FP64 at 1/64 of the FP32 rate).
__device__ __forceinline__ double apply_stencil(const SolveArgs &S, int n, int i, int j, const double *v)
{
    const int nn = S.Nx * S.Ny;
    double acc = 0;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
        if (j + dj < 0 || j + dj >= S.Ny) continue;
#pragma unroll
        for (int di = -1; di <= 1; di++) {
            if (i + di < 0 || i + di >= S.Nx) continue;
            acc = fma(S.coef[(size_t)(3 * (dj + 1) + (di + 1)) * nn + n], __ldcg(v + n + dj * S.Nx + di), acc);
        }
    }
    return acc;
}

// Jacobi-preconditioned conjugate gradients in the Chronopoulos-Gear form
// (Chronopoulos and Gear, 1989): the two inner products of an iteration are
// taken together, so an iteration needs two grid-wide synchronisations (one
// for the new residual, one for the reduction) instead of three.
//   p = u + beta p;  s = w + beta s;  x += alpha p;  r -= alpha s
//   u = D^-1 r;  w = A u;  gamma' = <r, u>;  delta = <w, u>
//   beta = gamma' / gamma;  alpha = gamma' / (delta - beta gamma' / alpha)
__global__ void __launch_bounds__(kSolveThreads, 2) pcg_kernel(SolveArgs S)
{
    const int nn = S.Nx * S.Ny;
    const int nblocks = gridDim.x;
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;

    // Set-up: 9-point rows (with the diagonal shift), unknown mask via dinv,
    // right-hand side in r, warm start in x.
    for (int n = tid; n < nn; n += stride) {
        const int j = n / S.Nx, i = n - j * S.Nx;
        double cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double f = 0;
        const bool dof = S.node_m[n] > S.dof_tol;
        bool coupled = false;
        if (dof) {
            build_row(S, i, j, cf, &f);
#pragma unroll
            for (int q = 0; q < 9; q++) coupled |= (__double_as_longlong(cf[q]) << 1) != 0;
            cf[4] += S.shift;
        }
        if (dof && cf[4] > 0) {
            S.dinv[n] = 1.0 / cf[4];
            S.r[n] = f;
            // a row no element touches holds only the shift and a zero
            // right-hand side: its solution is zero, whatever the start
            if (!coupled) S.x[n] = 0;
        } else {
            S.dinv[n] = 0;
            S.r[n] = 0;
            S.x[n] = 0;
#pragma unroll
            for (int k = 0; k < 9; k++) cf[k] = 0;
        }
#pragma unroll
        for (int k = 0; k < 9; k++) S.coef[(size_t)k * nn + n] = cf[k];
    }
    if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;

    // r = b - A x (x of the neighbours is final since the set-up barrier; r
    // is read only at its own node here)
    double bb = 0, d1 = 0, d2 = 0;
    for (int n = tid; n < nn; n += stride) {
        if (is_zero(S.dinv[n])) continue;
        const int j = n / S.Nx, i = n - j * S.Nx;
        const double b = S.r[n];
        S.r[n] = b - apply_stencil(S, n, i, j, S.x);
        bb += b * b;
    }
    block_sum3(bb, d1, d2);
    if (threadIdx.x == 0) S.partials[2 * nblocks + blockIdx.x] = bb;
    if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;
    bb = grid_total(S.partials, 2, nblocks);
    for (int n = tid; n < nn; n += stride) S.u[n] = S.dinv[n] * S.r[n];
    if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;

    // u = D^-1 r, w = A u, gamma = <r, u>, delta = <w, u>, <r, r>
    double gamma = 0, delta = 0, rr = 0;
    for (int n = tid; n < nn; n += stride) {
        if (is_zero(S.dinv[n])) {
            S.w[n] = 0;
            S.p[n] = 0;
            S.q[n] = 0;
            continue;
        }
        const int j = n / S.Nx, i = n - j * S.Nx;
        const double r = S.r[n], u = S.u[n];
        const double w = apply_stencil(S, n, i, j, S.u);
        S.w[n] = w;
        S.p[n] = 0;      // p, s (in q) start at zero: the first update sets p = u, s = w
        S.q[n] = 0;
        gamma += r * u;
        delta += w * u;
        rr += r * r;
    }
    block_sum3(gamma, delta, rr);
    if (threadIdx.x == 0) {
        S.partials[0 * nblocks + blockIdx.x] = gamma;
        S.partials[1 * nblocks + blockIdx.x] = delta;
        S.partials[3 * nblocks + blockIdx.x] = rr;
    }
    if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;
    grid_total3(S.partials, 0, 1, 3, nblocks, gamma, delta, rr);
    const double target = S.tol * S.tol * bb;

    int it = 0;
    bool converged = (rr <= target);
    if (bb == 0) {
        // No load: the solution is zero (the warm start is discarded).
        for (int n = tid; n < nn; n += stride) S.x[n] = 0;
        rr = 0;
        converged = true;
    }
    double alpha = gamma / delta, beta = 0;
    __shared__ double sh_scalar[2];
    __shared__ int sh_next;
    while (!converged && it < S.maxit) {
        // p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s (own nodes)
        for (int n = tid; n < nn; n += stride) {
            const double dv = S.dinv[n];
            if (is_zero(dv)) continue;
            const double p = fma(beta, S.p[n], S.u[n]);
            const double sv = fma(beta, S.q[n], S.w[n]);
            const double r = fma(-alpha, sv, S.r[n]);
            S.p[n] = p;
            S.q[n] = sv;
            S.x[n] = fma(alpha, p, S.x[n]);
            S.r[n] = r;
            S.u[n] = dv * r;
        }
        if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;
        double gn = 0, dl = 0, rn = 0;
        for (int n = tid; n < nn; n += stride) {
            if (is_zero(S.dinv[n])) continue;
            const int j = n / S.Nx, i = n - j * S.Nx;
            const double r = S.r[n], u = S.u[n];
            const double w = apply_stencil(S, n, i, j, S.u);
            S.w[n] = w;
            gn = fma(r, u, gn);
            dl = fma(w, u, dl);
            rn = fma(r, r, rn);
        }
        block_sum3(gn, dl, rn);
        if (threadIdx.x == 0) {
            S.partials[0 * nblocks + blockIdx.x] = gn;
            S.partials[1 * nblocks + blockIdx.x] = dl;
            S.partials[3 * nblocks + blockIdx.x] = rn;
        }
        if (!mpmg_grid_barrier(S.barrier, nblocks, S.status, kSpinLimit)) return;
        grid_total3(S.partials, 0, 1, 3, nblocks, gn, dl, rr);
        it++;
        // The recurrence's scalars, formed by one thread and shared through
        // shared memory (three FP64 divisions, which every warp would
        // otherwise issue); the next writes come after the next grid barrier.
        if (threadIdx.x == 0) {
            int next = 0;                        // 0: go on, 1: give up, 2: converged
            if (!(rr == rr)) {
                next = 1;                        // NaN
            } else if (rr <= target) {
                next = 2;
            } else {
                const double beta_n = gn / gamma;
                const double eta = dl - beta_n * gn / alpha;
                if (!(eta > 0)) {
                    next = 1;                    // breakdown of the recurrence: report non-convergence
                } else {
                    sh_scalar[0] = beta_n;
                    sh_scalar[1] = gn / eta;
                }
            }
            sh_next = next;
        }
        __syncthreads();
        const int next = sh_next;
        if (next == 1) break;
        if (next == 2) {
            converged = true;
            break;
        }
        beta = sh_scalar[0];
        alpha = sh_scalar[1];
        gamma = gn;
    }
    if (tid == 0) {
        S.sp->solve_iters = it;
        S.sp->solve_converged = converged ? 1 : 0;
        S.sp->solve_rel_resid = (bb > 0) ? sqrt(rr / bb) : 0.0;
        if (!converged) atomicOr(S.status, MPMG_DEV_ERR_SOLVER);
    }
}

// ---------------------------------------------------------------------------
// The same Chronopoulos-Gear PCG with each block's rows and vectors resident
// in shared memory.  Block b owns the contiguous nodes [b C, b C + C) (a few
// grid rows) for the whole solve: their nine-point rows, D^-1, r, p, s, w
// and u stay in shared memory, x stays in global memory (read and written
// once an iteration), and u is also written to global memory so that the
// neighbouring blocks can read the Nx + 1 halo nodes on either side of their
// range.  An iteration is then
//   A  p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = D^-1 r
//      (own nodes, shared memory; u also to global)
//                                  -- wait for the two neighbouring blocks
//   B  halo of u from global (one batched load); w = A u; block partials of
//      <r, u>, <w, u>, <r, r>                                -- grid barrier
//   C  every block sums the partials in one fixed order (one batched load)
//      and forms the scalars.
// Compared with pcg_kernel, whose grid-stride loops read every vector and
// row from L2 with dependent loads in each sweep, the only global reads an
// iteration waits for are the halo and the partials.  The arithmetic and
// the order of every sum are fixed, so the result does not depend on
// timing.  The kernel runs when a block's share of the grid fits in shared
// memory (pcg_tile_fits); pcg_kernel covers the rest.

constexpr int kTileThreads = 512;
constexpr int kTileTrips = 4;   // nodes a thread: a block owns at most kTileTrips * kTileThreads

// Sum of (a, b, c) over the block in a fixed order; the result is returned
// to every thread.  Only warp 0 adds: lane l sums the values of threads l,
// l + 32, ... from shared memory, then the lanes combine in a shuffle tree.
// (GB300 issues FP64 at 1/64 of the FP32 rate, and a shuffle tree in every
// warp would cost as many FP64 adds as the rows of an iteration.)
// scratch holds 3 * blockDim.x + 3 doubles.
__device__ __forceinline__ void tile_sum3(double &a, double &b, double &c, double *scratch)
{
    const int nt = blockDim.x;
    scratch[threadIdx.x] = a;
    scratch[nt + threadIdx.x] = b;
    scratch[2 * nt + threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        // four interleaved partial sums a value (a fixed order) to shorten
        // the chain of dependent FP64 adds
        double x0 = 0, x1 = 0, x2 = 0, x3 = 0, y0 = 0, y1 = 0, y2 = 0, y3 = 0, z0 = 0, z1 = 0, z2 = 0, z3 = 0;
        for (int t = lane; t < nt; t += 128) {
            x0 += scratch[t];
            y0 += scratch[nt + t];
            z0 += scratch[2 * nt + t];
            if (t + 32 < nt) {
                x1 += scratch[t + 32];
                y1 += scratch[nt + t + 32];
                z1 += scratch[2 * nt + t + 32];
            }
            if (t + 64 < nt) {
                x2 += scratch[t + 64];
                y2 += scratch[nt + t + 64];
                z2 += scratch[2 * nt + t + 64];
            }
            if (t + 96 < nt) {
                x3 += scratch[t + 96];
                y3 += scratch[nt + t + 96];
                z3 += scratch[2 * nt + t + 96];
            }
        }
        double x = (x0 + x1) + (x2 + x3), y = (y0 + y1) + (y2 + y3), z = (z0 + z1) + (z2 + z3);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
            z += __shfl_down_sync(0xffffffffu, z, off);
        }
        if (lane == 0) {
            scratch[3 * nt] = x;
            scratch[3 * nt + 1] = y;
            scratch[3 * nt + 2] = z;
        }
    }
    __syncthreads();
    a = scratch[3 * nt];
    b = scratch[3 * nt + 1];
    c = scratch[3 * nt + 2];
    __syncthreads();
}

// Slots (sa, sb, sc) of the per-block partials summed over all blocks in one
// fixed order by warp 0 (lane l takes blocks l, l + 32, ..., then a shuffle
// tree); every block computes the same totals.
__device__ __forceinline__ void tile_totals3(const double *partials, int sa, int sb, int sc, int nblocks,
                                             double &ta, double &tb, double &tc, double *scratch)
{
    const int nt = blockDim.x;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        // all loads first (up to kMaxTotals per lane), then the adds in order
        constexpr int kMaxTotals = 8;
        double va[kMaxTotals], vb[kMaxTotals], vc[kMaxTotals];
#pragma unroll
        for (int q = 0; q < kMaxTotals; q++) {
            const int t = lane + 32 * q;
            const bool in = t < nblocks;
            va[q] = in ? __ldcg(partials + (size_t)sa * nblocks + t) : 0.0;
            vb[q] = in ? __ldcg(partials + (size_t)sb * nblocks + t) : 0.0;
            vc[q] = in ? __ldcg(partials + (size_t)sc * nblocks + t) : 0.0;
        }
        double x = 0, y = 0, z = 0;
#pragma unroll
        for (int q = 0; q < kMaxTotals; q++) {
            x += va[q];
            y += vb[q];
            z += vc[q];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
            z += __shfl_down_sync(0xffffffffu, z, off);
        }
        if (lane == 0) {
            scratch[3 * nt] = x;
            scratch[3 * nt + 1] = y;
            scratch[3 * nt + 2] = z;
        }
    }
    __syncthreads();
    ta = scratch[3 * nt];
    tb = scratch[3 * nt + 1];
    tc = scratch[3 * nt + 2];
    __syncthreads();
}

// Grid barrier on a counter that only grows: episode k of a launch ends
// when the counter reaches k * nblocks (the counter starts at zero at each
// launch).  Thread 0 of each block publishes the block's writes (fence,
// then a fire-and-forget add) and polls with acquire loads; the poll is
// bounded, and a timeout or another block's timeout sets the spin error.
__device__ __forceinline__ bool tile_grid_barrier(unsigned int *counter, unsigned int target, int *status)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
        long long polls = 0;
        for (;;) {
            unsigned int v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(counter) : "memory");
            if ((int)(v - target) >= 0) break;
            if (++polls > kSpinLimit || (*(volatile int *)status & MPMG_DEV_ERR_SPIN) != 0) {
                atomicOr(status, MPMG_DEV_ERR_SPIN);
                break;
            }
        }
    }
    __syncthreads();
    return (*(volatile int *)status & MPMG_DEV_ERR_SPIN) == 0;
}

// Point-to-point wait of phase A -> B: block b publishes that its u of
// iteration `tag` is written (flags[b] = tag, after a fence) and waits until
// its neighbours b - 1 and b + 1, whose ranges its halo reads, have
// published the same tag.  Bounded like the barrier.
__device__ __forceinline__ bool tile_neighbour_wait(unsigned int *flags, unsigned int tag, int *status)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(flags + blockIdx.x), "r"(tag) : "memory");
        long long polls = 0;
        for (int side = -1; side <= 1; side += 2) {
            const int nb = (int)blockIdx.x + side;
            if (nb < 0 || nb >= (int)gridDim.x) continue;
            for (;;) {
                unsigned int v;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(flags + nb) : "memory");
                if ((int)(v - tag) >= 0) break;
                if (++polls > kSpinLimit || (*(volatile int *)status & MPMG_DEV_ERR_SPIN) != 0) {
                    atomicOr(status, MPMG_DEV_ERR_SPIN);
                    break;
                }
            }
        }
    }
    __syncthreads();
    return (*(volatile int *)status & MPMG_DEV_ERR_SPIN) == 0;
}

// (A v) at own node k from the shared-memory rows and the extended vector
// ve (own nodes at ve[k + H], halo below at ve[0, H), above after the own
// nodes).  Missing neighbours are skipped by index.
__device__ __forceinline__ double tile_stencil(const double *coef, int C, int H, int k, int i, int j, int Nx,
                                               int Ny, const double *ve)
{
    double acc = 0;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
        if (j + dj < 0 || j + dj >= Ny) continue;
#pragma unroll
        for (int di = -1; di <= 1; di++) {
            if (i + di < 0 || i + di >= Nx) continue;
            acc = fma(coef[(3 * (dj + 1) + (di + 1)) * C + k], ve[k + H + dj * Nx + di], acc);
        }
    }
    return acc;
}

// Fills the halo of ve (Nx + 1 nodes on either side of [n0, n1)) from the
// global vector g; nodes outside the grid read zero.
__device__ __forceinline__ void tile_halo(const double *g, int n0, int n1, int nn, int H, double *ve)
{
    for (int t = threadIdx.x; t < 2 * H; t += blockDim.x) {
        const int m = t < H ? n0 - H + t : n1 + (t - H);
        ve[m - n0 + H] = (m >= 0 && m < nn) ? __ldcg(g + m) : 0.0;
    }
}

__global__ void __launch_bounds__(kTileThreads, 1) pcg_tile_kernel(SolveArgs S, int C, int warm, unsigned int *flags)
{
    extern __shared__ double sm[];
    const int Nx = S.Nx, Ny = S.Ny, nn = Nx * Ny, H = Nx + 1;
    const int nblocks = gridDim.x;
    const int n0 = blockIdx.x * C;
    const int n1 = min(n0 + C, nn);
    const int cnt = n1 - n0;
    double *coef = sm;                      // 9 C
    double *dinv = coef + 9 * C;            // C each
    double *r = dinv + C, *p = r + C, *s = p + C, *w = s + C;
    double *ve = w + C;                     // C + 2 H: u (or x) with its halo
    double *scratch = ve + C + 2 * H;       // 3 kTileThreads + 3
    __shared__ double sh_scalar[2];
    __shared__ int sh_next;
    unsigned int episode = 0;      // grid barriers passed (S.barrier[0] counts arrivals)

    // Set-up: rows (with the diagonal shift), D^-1 (zero for nodes that are
    // not unknowns), right-hand side in r, the start in x.  A row that no
    // element touches holds only the shift and a zero right-hand side, so
    // its solution is zero: a warm start there is cleared.
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        const int n = n0 + k, j = n / Nx, i = n - j * Nx;
        double cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double f = 0;
        const bool dof = S.node_m[n] > S.dof_tol;
        bool coupled = false;
        if (dof) {
            build_row(S, i, j, cf, &f);
#pragma unroll
            for (int q = 0; q < 9; q++) coupled |= (__double_as_longlong(cf[q]) << 1) != 0;
            cf[4] += S.shift;
        }
        if (dof && cf[4] > 0) {
            dinv[k] = 1.0 / cf[4];
            r[k] = f;
            if (!warm || !coupled) S.x[n] = 0;
        } else {
            dinv[k] = 0;
            r[k] = 0;
            S.x[n] = 0;
#pragma unroll
            for (int q = 0; q < 9; q++) cf[q] = 0;
        }
#pragma unroll
        for (int q = 0; q < 9; q++) coef[q * C + k] = cf[q];
    }
    if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;

    // r = b - A x, <b, b>
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) ve[k + H] = __ldcg(S.x + n0 + k);
    tile_halo(S.x, n0, n1, nn, H, ve);
    __syncthreads();
    double bb = 0, z0 = 0, z1 = 0;
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        const double dv = dinv[k];
        double u = 0;
        if (!is_zero(dv)) {
            const int n = n0 + k, j = n / Nx, i = n - j * Nx;
            const double b = r[k];
            const double rk = b - tile_stencil(coef, C, H, k, i, j, Nx, Ny, ve);
            r[k] = rk;
            bb = fma(b, b, bb);
            u = dv * rk;
        }
        p[k] = 0;      // p, s start at zero: the first update sets p = u, s = w
        s[k] = 0;
        S.u[n0 + k] = u;
    }
    tile_sum3(bb, z0, z1, scratch);
    if (threadIdx.x == 0) S.partials[2 * nblocks + blockIdx.x] = bb;
    if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
    tile_totals3(S.partials, 2, 2, 2, nblocks, bb, z0, z1, scratch);

    // w = A u, gamma = <r, u>, delta = <w, u>, <r, r>
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) ve[k + H] = __ldcg(S.u + n0 + k);
    tile_halo(S.u, n0, n1, nn, H, ve);
    __syncthreads();
    double gamma = 0, delta = 0, rr = 0;
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        double wk = 0;
        if (!is_zero(dinv[k])) {
            const int n = n0 + k, j = n / Nx, i = n - j * Nx;
            const double rk = r[k], u = ve[k + H];
            wk = tile_stencil(coef, C, H, k, i, j, Nx, Ny, ve);
            gamma = fma(rk, u, gamma);
            delta = fma(wk, u, delta);
            rr = fma(rk, rk, rr);
        }
        w[k] = wk;
    }
    tile_sum3(gamma, delta, rr, scratch);
    if (threadIdx.x == 0) {
        S.partials[0 * nblocks + blockIdx.x] = gamma;
        S.partials[1 * nblocks + blockIdx.x] = delta;
        S.partials[3 * nblocks + blockIdx.x] = rr;
    }
    if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
    tile_totals3(S.partials, 0, 1, 3, nblocks, gamma, delta, rr, scratch);
    const double target = S.tol * S.tol * bb;

    int it = 0;
    bool converged = (rr <= target);
    if (bb == 0) {
        // No load: the solution is zero (the warm start is discarded).
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) S.x[n0 + k] = 0;
        rr = 0;
        converged = true;
    }
    double alpha = gamma / delta, beta = 0;
    while (!converged && it < S.maxit) {
        // A: own nodes only; this thread's x values are loaded first (all
        // loads in flight at once; a block owns at most kTileTrips *
        // kTileThreads nodes)
        double xr[kTileTrips];
#pragma unroll
        for (int q = 0; q < kTileTrips; q++) {
            const int k = threadIdx.x + q * kTileThreads;
            xr[q] = k < cnt ? __ldcg(S.x + n0 + k) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kTileTrips; q++) {
            const int k = threadIdx.x + q * kTileThreads;
            if (k >= cnt) break;
            const double dv = dinv[k];
            if (is_zero(dv)) continue;
            const int n = n0 + k;
            const double pk = fma(beta, p[k], ve[k + H]);
            const double sk = fma(beta, s[k], w[k]);
            const double rk = fma(-alpha, sk, r[k]);
            p[k] = pk;
            s[k] = sk;
            r[k] = rk;
            S.x[n] = fma(alpha, pk, xr[q]);
            const double u = dv * rk;
            ve[k + H] = u;
            S.u[n] = u;
        }
        // the halo needs only the neighbours' u of this iteration; they read
        // ours, and nobody rewrites u before the reduction barrier below
        if (!tile_neighbour_wait(flags, (unsigned)it + 1u, S.status)) return;
        // B: halo, w = A u, partials
        tile_halo(S.u, n0, n1, nn, H, ve);
        __syncthreads();
        double gn = 0, dl = 0, rn = 0;
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            if (is_zero(dinv[k])) continue;
            const int n = n0 + k, j = n / Nx, i = n - j * Nx;
            const double rk = r[k], u = ve[k + H];
            const double wk = tile_stencil(coef, C, H, k, i, j, Nx, Ny, ve);
            w[k] = wk;
            gn = fma(rk, u, gn);
            dl = fma(wk, u, dl);
            rn = fma(rk, rk, rn);
        }
        tile_sum3(gn, dl, rn, scratch);
        if (threadIdx.x == 0) {
            S.partials[0 * nblocks + blockIdx.x] = gn;
            S.partials[1 * nblocks + blockIdx.x] = dl;
            S.partials[3 * nblocks + blockIdx.x] = rn;
        }
        if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
        // C: totals and scalars
        tile_totals3(S.partials, 0, 1, 3, nblocks, gn, dl, rr, scratch);
        it++;
        if (threadIdx.x == 0) {
            int next = 0;                        // 0: go on, 1: give up, 2: converged
            if (!(rr == rr)) {
                next = 1;                        // NaN
            } else if (rr <= target) {
                next = 2;
            } else {
                const double beta_n = gn / gamma;
                const double eta = dl - beta_n * gn / alpha;
                if (!(eta > 0)) {
                    next = 1;                    // breakdown of the recurrence: report non-convergence
                } else {
                    sh_scalar[0] = beta_n;
                    sh_scalar[1] = gn / eta;
                }
            }
            sh_next = next;
        }
        __syncthreads();
        const int next = sh_next;
        if (next == 1) break;
        if (next == 2) {
            converged = true;
            break;
        }
        beta = sh_scalar[0];
        alpha = sh_scalar[1];
        gamma = gn;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.sp->solve_iters = it;
        S.sp->solve_converged = converged ? 1 : 0;
        S.sp->solve_rel_resid = (bb > 0) ? sqrt(rr / bb) : 0.0;
        if (!converged) atomicOr(S.status, MPMG_DEV_ERR_SOLVER);
    }
}

// Shared memory of pcg_tile_kernel for C nodes a block on an Nx-wide grid.
inline size_t pcg_tile_smem(int C, int Nx)
{
    return sizeof(double) * ((size_t)15 * C + 2 * (size_t)(Nx + 1) + 3 * kTileThreads + 8);
}

// ---------------------------------------------------------------------------
// Multigrid-preconditioned conjugate gradients (pcg_mg_kernel).
//
// Jacobi-PCG needs O(l / h) iterations on this operator, where l is the size
// of the regions near yield: there the cooperativity length grows, xi^-2
// falls, and the Laplacian part dominates.  On the 513^2 silo it took 30
// iterations a step after 4 steps, 137 after 18 and 809 after 60.  A
// geometric multigrid V-cycle on the node lattice makes the count nearly
// independent of the grid: 6 to 9 iterations on the same systems.
//
// Hierarchy.  Level 0 is the node lattice.  Level l + 1 keeps every second
// node of level l along each direction with more than 3 nodes
// (n -> n / 2 + 1), down to at most 3 x 3 nodes.  Prolongation P is bilinear
// interpolation, restriction is P^T, and the coarse operators are the
// Galerkin products A_{l+1} = P^T A_l P, formed every solve in FP32.  Each
// node keeps its full 9-point row, its row sum s = A 1 and the inverse of
// its absolute row sum.  P reproduces constants, so a coarse row sum is
// P^T s, and a coarse diagonal is set to that row sum minus the row's
// off-diagonal entries.  The near-null space of a Neumann-like operator
// (only the 1e-10 shift and the xi^-2-weighted mass keep it from being
// singular) therefore survives FP32 coarsening.
//
// Preconditioner: one V(1,1) cycle in FP32 on r / |r|.
//   * On each level, one l1-Jacobi step (Baker, Falgout, Kolev and Yang,
//     2011).  D_l1 is each row's absolute sum, so the smoother converges
//     without an eigenvalue estimate.  The step size is the Chebyshev step
//     for the interval [0.3, 1] of D_l1^-1 A.
//   * Then the residual and its restriction.
//   * At the coarsest level, an exact solve: an FP64 inverse formed every
//     solve.
//   * On the way up, prolongation and one post-smoothing step of the same
//     size.
//
// Outer iteration: FP64 CG in the one-reduction form of Chronopoulos and
// Gear.  It uses the Polak-Ribiere beta, which tolerates the rounding of an
// FP32 preconditioner (whose Galerkin rows are symmetric only to rounding):
//   beta  = -alpha <s, u> / gamma_old
//   pi    = delta + 2 beta <s, u> + beta^2 pi_old
//   alpha = gamma / pi
// where u = M r, w = A u, gamma = <r, u>, delta = <w, u>, and s = A p by
// recurrence.  Each iteration needs one grid barrier, for the four inner
// products.
//
// Where the levels live.  A level of more than 2048 nodes is spread over the
// blocks in contiguous node ranges (level 0 over blocks 1 .. n - 1, so that
// block 0 has no level-0 work); the coarser levels are held whole by block
// 0, whose threads meet at block barriers between phases.  All blocks
// restrict into the first held level and block 0 stages it.
//
// Synchronisation between blocks.  Each phase writes its level vector to
// global memory as 64-bit words: an FP32 value plus a 32-bit tag that names
// the V-cycle.  A phase stages the words it needs from other blocks (a halo
// or a band of rows) into shared memory once; if some carry an older tag, a
// lane polls one of them with a pause after each stale answer and, once that
// one is current, the warp loads its stale words again together.  A word is stored with one
// single-copy-atomic 64-bit store, so its value and tag arrive together,
// with no fences or flags.
//   * Each phase vector is written once per V-cycle, and the outer grid
//     barrier separates V-cycles, so no value is overwritten while a reader
//     may still need it.
//   * Each solve reserves its tags (maxit + 2, from a counter in device
//     memory), so it never accepts a word written by an earlier solve.
//   * Polls are bounded, like the barriers.

constexpr int kMgThreads = 512;
constexpr int kMgTrips = 4;            // nodes of a level a thread owns at most
constexpr int kMgLocal = kMgTrips * kMgThreads;   // levels this small are held by block 0
constexpr int kMgCoarse = 9;           // nodes of the coarsest level at most (3 x 3)
// one smoothing step: the Chebyshev step for [0.3, 1], 1 / 0.65
constexpr float kMgOmega = 1.0f / 0.65f;
// polls of one wait before it gives up (a poll is one L2 round trip, about
// a microsecond: a few seconds in all)
constexpr long long kMgPollLimit = 1ll << 22;
// sleep of a waiting warp after a stale answer (ns)
constexpr unsigned kMgNap = 128;

__device__ __forceinline__ unsigned long long mg_ld(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ void mg_st(unsigned long long *p, float x, unsigned tag)
{
    const unsigned long long v = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(x);
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v));
}

// A word that needs no wait: value 0 with the current tag.
__device__ __forceinline__ unsigned long long mg_zero(unsigned tag)
{
    return (unsigned long long)tag << 32;
}

__device__ __forceinline__ float mg_f(unsigned long long v)
{
    return __uint_as_float((unsigned)v);
}

__device__ __forceinline__ bool mg_give_up(long long polls, int *status)
{
    if ((polls & 15) != 0) return false;
    if (polls > kMgPollLimit || (*(volatile int *)status & MPMG_DEV_ERR_SPIN) != 0) {
        atomicOr(status, MPMG_DEV_ERR_SPIN);
        return true;
    }
    return false;
}

// Waits until every word of v carries `tag` (addr(t, q) is the address of
// word q of trip t, for T trips of Q words).  Called by whole warps.  While some lane holds stale
// words, one lane polls one of them and the warp sleeps kMgNap ns after a
// stale answer; once that word is current, every lane loads its stale words
// again together.  A phase so waits a round trip or two after its last
// input is written, while a waiting warp neither floods L2 with polls (which
// slows the stores it waits for) nor takes many issue slots from the warps
// that compute.  Bounded (kMgPollLimit polls, or another block's timeout):
// then the spin error is set and the words read 0.
template <int T, int Q, class Addr>
__device__ __forceinline__ void mg_resolve(unsigned long long (&v)[T][Q], unsigned tag, int *status, Addr addr)
{
    const unsigned lane = threadIdx.x & 31u;
    for (long long polls = 1;; polls++) {
        int ft = -1, fq = 0;
#pragma unroll
        for (int t = T - 1; t >= 0; t--) {
#pragma unroll
            for (int q = Q - 1; q >= 0; q--) {
                if ((unsigned)(v[t][q] >> 32) != tag) {
                    ft = t;
                    fq = q;
                }
            }
        }
        const unsigned stale = __ballot_sync(0xffffffffu, ft >= 0);
        if (stale == 0) return;
        if (mg_give_up(polls, status)) {
#pragma unroll
            for (int t = 0; t < T; t++) {
#pragma unroll
                for (int q = 0; q < Q; q++) v[t][q] = mg_zero(tag);
            }
            return;
        }
        const unsigned leader = __ffs(stale) - 1;
        int fresh = 0;
        if (lane == leader) fresh = (unsigned)(mg_ld(addr(ft, fq)) >> 32) == tag;
        if (!__shfl_sync(0xffffffffu, fresh, leader)) {
            __nanosleep(kMgNap);
            continue;
        }
#pragma unroll
        for (int t = 0; t < T; t++) {
#pragma unroll
            for (int q = 0; q < Q; q++) {
                if ((unsigned)(v[t][q] >> 32) != tag) v[t][q] = mg_ld(addr(t, q));
            }
        }
    }
}

// Copies the words of two node ranges of a level vector (nn nodes), [a0, a1)
// to d0 and [b0, b1) to d1, as floats once they carry `tag`; nodes outside
// the level read 0.  Called by the whole block; ends with a block barrier.
__device__ __forceinline__ void mg_stage(const unsigned long long *w, int nn, int a0, int a1, float *d0, int b0,
                                         int b1, float *d1, unsigned tag, int *status)
{
    constexpr int T = 4;
    const int na = max(a1 - a0, 0), nt = na + max(b1 - b0, 0);
    for (int base = 0; base < nt; base += T * kMgThreads) {
        unsigned long long v[T][1];
#pragma unroll
        for (int t = 0; t < T; t++) {
            const int u = base + threadIdx.x + t * kMgThreads;
            const int m = u < na ? a0 + u : b0 + (u - na);
            v[t][0] = (u < nt && m >= 0 && m < nn) ? mg_ld(w + m) : mg_zero(tag);
        }
        mg_resolve(v, tag, status, [&](int t, int) {
            const int u = base + threadIdx.x + t * kMgThreads;
            return w + (u < na ? a0 + u : b0 + (u - na));
        });
#pragma unroll
        for (int t = 0; t < T; t++) {
            const int u = base + threadIdx.x + t * kMgThreads;
            if (u < na) d0[u] = mg_f(v[t][0]);
            else if (u < nt) d1[u - na] = mg_f(v[t][0]);
        }
    }
    __syncthreads();
}

// Per-level arrays in shared memory (floats).  A level spread over the
// blocks keeps its b, z1, res (C each) at lv.sm; level 0 also keeps its rows
// at float 0 (coef0[9][C0], l1inv0[C0]).  A level held by block 0 keeps its
// rows at lv.sm and b, z1, res, zf (nn each) at lv.smv.
struct MgShared {
    float *b, *z1, *res;
};

__device__ __forceinline__ MgShared mg_shared(float *sm, const MgLevel &lv)
{
    MgShared s;
    s.b = sm + (lv.local ? lv.smv : lv.sm);
    s.z1 = s.b + lv.C;
    s.res = s.z1 + lv.C;
    return s;
}

// Row entry q of own node k (global node n) of level l, and D_l1^-1.
__device__ __forceinline__ float mg_coef(const MgPlan &P, const float *sm, int l, int q, int k, int n)
{
    if (l == 0) return sm[q * P.lv[0].C + k];
    if (P.lv[l].local) return sm[P.lv[l].sm + q * P.lv[l].nn + n];
    return __ldcg(P.coef + (size_t)q * P.total + P.lv[l].g + n);
}

__device__ __forceinline__ float mg_l1inv(const MgPlan &P, const float *sm, int l, int k, int n)
{
    if (l == 0) return sm[9 * P.lv[0].C + k];
    if (P.lv[l].local) return sm[P.lv[l].sm + 9 * P.lv[l].nn + n];
    return __ldcg(P.l1inv + P.lv[l].g + n);
}

// Coarse parents of fine coordinate g along a direction: g even (or the
// direction not coarsened) -> one parent with weight 1; g odd -> the two
// coarse neighbours with weight 1/2.
__device__ __forceinline__ int mg_parents(int g, int coarsened, int &p0, int &p1)
{
    if (!coarsened) {
        p0 = p1 = g;
        return 1;
    }
    p0 = g >> 1;
    p1 = (g + 1) >> 1;
    return (g & 1) ? 2 : 1;
}

// Rows fa .. fb of the finer level F under the coarse nodes [c0, c0 + cnt)
// of level lv (their restriction support).
__host__ __device__ inline void mg_fine_rows(const MgLevel &lv, const MgLevel &F, int c0, int cnt, int &fa, int &fb)
{
    const int cja = c0 / lv.Nx, cjb = (c0 + cnt - 1) / lv.Nx;
    fa = lv.cy ? (2 * cja - 1 > 0 ? 2 * cja - 1 : 0) : cja;
    fb = lv.cy ? (2 * cjb + 1 < F.Ny - 1 ? 2 * cjb + 1 : F.Ny - 1) : cjb;
}

// Rows ya .. yb of the coarser level Cl holding the parents of the nodes
// n0 - H .. n0 + cnt + H of level lv (H = lv.Nx + 1, clipped to the level).
__host__ __device__ inline void mg_parent_rows(const MgLevel &lv, const MgLevel &Cl, int n0, int cnt, int &ya,
                                               int &yb)
{
    const int H = lv.Nx + 1;
    const int lo = n0 - H > 0 ? n0 - H : 0, hi = n0 + cnt + H < lv.nn ? n0 + cnt + H : lv.nn;
    const int ja = lo / lv.Nx, jb = (hi - 1) / lv.Nx;
    ya = Cl.cy ? ja >> 1 : ja;
    yb = Cl.cy ? (jb + 1) >> 1 : jb;
}

// Fine coordinate of support slot s (0, 1, 2) of coarse coordinate c, or -1.
__device__ __forceinline__ int mg_fine_of(int c, int s, int coarsened)
{
    return coarsened ? 2 * c + s - 1 : (s == 1 ? c : -1);
}

// Writes a level's row of node (level offset g + n): entries, row sum,
// D_l1^-1 (a row with no entries is not an unknown: all zero).
// Also into `held` (a held level's shared-memory rows, coef[9][nn] then
// l1inv[nn], at node k of nn) when given.
__device__ __forceinline__ void mg_put_row(const MgPlan &P, int at, float a[9], float rs, float *held = nullptr,
                                           int k = 0, int nn = 0)
{
    float l1 = 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) l1 += fabsf(a[q]);
    const float li = l1 > 0.0f ? 1.0f / l1 : 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const float v = li > 0.0f ? a[q] : 0.0f;
        P.coef[(size_t)q * P.total + at] = v;
        if (held != nullptr) held[q * nn + k] = v;
    }
    P.rsum[at] = rs;
    P.l1inv[at] = li;
    if (held != nullptr) held[9 * nn + k] = li;
}

// Offset of fine coordinate 2c + o (coarsened) or c + o (not) from its first
// coarse parent relative to c, and whether it has a second one at +1.
template <int CO>
__device__ __forceinline__ constexpr int mg_par0(int o)
{
    return CO ? (o >= 0 ? o / 2 : -((1 - o) / 2)) : o;
}

template <int CO>
__device__ __forceinline__ constexpr bool mg_par2(int o)
{
    return CO ? (o & 1) != 0 : false;
}

// Galerkin row of coarse node (ci, cj) of level c from the rows of level
// c - 1: the nine entries of P^T A P, the row sum P^T s, and the diagonal
// set to the row sum minus the off-diagonal entries.  CX, CY: the level is
// coarsened along x, y (every index into the row is then a constant).
template <int CX, int CY>
__device__ void mg_galerkin_row_t(const MgPlan &P, int c, int I, int ci, int cj, float *held)
{
    const MgLevel &F = P.lv[c - 1], &Cl = P.lv[c];
    float acc[9];
#pragma unroll
    for (int q = 0; q < 9; q++) acc[q] = 0.0f;
    float srow = 0.0f;
#pragma unroll
    for (int sy = 0; sy < 3; sy++) {
        if (!CY && sy != 1) continue;
        const int fy = CY ? 2 * cj + sy - 1 : cj;
        // one row of the fine support at a time: its rows loaded together
        float a[3][9], sf[3];
        bool in[3];
#pragma unroll
        for (int sx = 0; sx < 3; sx++) {
            const int fx = CX ? 2 * ci + sx - 1 : ci;
            in[sx] = (CX || sx == 1) && fx >= 0 && fx < F.Nx && fy >= 0 && fy < F.Ny;
            const int fi = in[sx] ? fy * F.Nx + fx : 0;
#pragma unroll
            for (int q = 0; q < 9; q++) a[sx][q] = in[sx] ? __ldcg(P.coef + (size_t)q * P.total + F.g + fi) : 0.0f;
            sf[sx] = in[sx] ? __ldcg(P.rsum + F.g + fi) : 0.0f;
        }
#pragma unroll
        for (int sx = 0; sx < 3; sx++) {
            if (!in[sx]) continue;
            const float wi = (CY ? ((sy == 1) ? 1.0f : 0.5f) : 1.0f) * (CX ? ((sx == 1) ? 1.0f : 0.5f) : 1.0f);
            srow = fmaf(wi, sf[sx], srow);
#pragma unroll
            for (int q = 0; q < 9; q++) {
                // fine neighbour at offset ox, oy from (2 ci, 2 cj) (or (ci, cj));
                // entries towards nodes outside the grid are zero
                const int ox = (CX ? sx - 1 : 0) + q % 3 - 1, oy = (CY ? sy - 1 : 0) + q / 3 - 1;
                const int x0 = mg_par0<CX>(ox) + 1, y0 = mg_par0<CY>(oy) + 1;
                const bool x2 = mg_par2<CX>(ox), y2 = mg_par2<CY>(oy);
                const float v = wi * a[sx][q] * (x2 ? 0.5f : 1.0f) * (y2 ? 0.5f : 1.0f);
                acc[y0 * 3 + x0] += v;
                if (x2) acc[y0 * 3 + x0 + 1] += v;
                if (y2) acc[(y0 + 1) * 3 + x0] += v;
                if (x2 && y2) acc[(y0 + 1) * 3 + x0 + 1] += v;
            }
        }
    }
    acc[4] = srow - (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[5] + acc[6]) + (acc[7] + acc[8])));
    mg_put_row(P, Cl.g + I, acc, srow, held, I, Cl.nn);
}

__device__ __noinline__ void mg_galerkin_row(const MgPlan &P, int c, int I, int ci, int cj, float *held)
{
    const MgLevel &Cl = P.lv[c];
    if (Cl.cx && Cl.cy) mg_galerkin_row_t<1, 1>(P, c, I, ci, cj, held);
    else if (Cl.cx) mg_galerkin_row_t<1, 0>(P, c, I, ci, cj, held);
    else if (Cl.cy) mg_galerkin_row_t<0, 1>(P, c, I, ci, cj, held);
    else mg_galerkin_row_t<0, 0>(P, c, I, ci, cj, held);
}

// Sum of four values over the block in a fixed order, returned to every
// thread (warp 0 adds; scratch holds 4 * blockDim.x + 4 doubles).
__device__ __forceinline__ void mg_sum4(double v[4], double *scratch)
{
    const int nt = blockDim.x;
#pragma unroll
    for (int c = 0; c < 4; c++) scratch[c * nt + threadIdx.x] = v[c];
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double a[4][2];
#pragma unroll
        for (int c = 0; c < 4; c++) a[c][0] = a[c][1] = 0;
        for (int t = lane; t < nt; t += 64) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                a[c][0] += scratch[c * nt + t];
                if (t + 32 < nt) a[c][1] += scratch[c * nt + t + 32];
            }
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            double x = a[c][0] + a[c][1];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
            if (lane == 0) scratch[4 * nt + c] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 4; c++) v[c] = scratch[4 * nt + c];
    __syncthreads();
}

// The four per-block partials summed over all blocks in one fixed order by
// warp 0; every block computes the same totals.
__device__ __forceinline__ void mg_totals4(const double *partials, int nblocks, double v[4], double *scratch,
                                           int slots = 4)
{
    const int nt = blockDim.x;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        constexpr int kMax = 8;     // blocks <= 32 * kMax
        double x[4] = {0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < kMax; q++) {
            const int t = lane + 32 * q;
            if (t < nblocks) {
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (c < slots) x[c] += __ldcg(partials + (size_t)c * nblocks + t);
            }
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) x[c] += __shfl_down_sync(0xffffffffu, x[c], off);
            if (lane == 0) scratch[4 * nt + c] = x[c];
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 4; c++) v[c] = scratch[4 * nt + c];
    __syncthreads();
}

// The phases of a level spread over the blocks.  Block b owns the nodes
// [b C, b C + C) of the level, whose b, z1 and res stay in its shared memory.
// A phase copies the words it needs from other blocks (the halo of Nx + 1
// nodes on either side of the range, or the band of rows a restriction or
// prolongation reads) into the staging area once, then runs its stencil from
// shared memory.  Entries of the rows towards nodes outside the grid are
// zero, so a stencil that wraps around a row end reads a finite value it
// multiplies by zero.

// Residual phase of level l: res = b - A z1, kept in shared memory and
// published.
__device__ __forceinline__ void mg_residual(const MgPlan &P, float *sm, int l, const MgShared &S, unsigned tag,
                                            int *status)
{
    const MgLevel &lv = P.lv[l];
    int n0, cnt;
    mg_own_range(lv, blockIdx.x, n0, cnt);
    if (cnt <= 0) return;
    const int H = lv.Nx + 1;
    float *ze = sm + P.sm_vec;          // z1 at nodes n0 - H .. n0 + cnt + H
    for (int k = threadIdx.x; k < cnt; k += kMgThreads) ze[H + k] = S.z1[k];
    mg_stage(P.z1 + lv.g, lv.nn, n0 - H, n0, ze, n0 + cnt, n0 + cnt + H, ze + H + cnt, tag, status);
    for (int k = threadIdx.x; k < cnt; k += kMgThreads) {
        const int n = n0 + k;
        const float *z = ze + H + k;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) acc = fmaf(mg_coef(P, sm, l, q, k, n), z[(q / 3 - 1) * lv.Nx + (q % 3 - 1)], acc);
        const float r = S.b[k] - acc;
        S.res[k] = r;
        mg_st(P.res + lv.g + n, r, tag);
    }
    __syncthreads();
}

// Restriction to the spread level c from the spread level c - 1: the fine
// residual rows under this block's coarse nodes are staged, then
// b = P^T res and the pre-smoothing step z1 = omega D_l1^-1 b (published).
__device__ __forceinline__ void mg_restrict(const MgPlan &P, float *sm, int c, const MgShared &S, unsigned tag,
                                            int *status)
{
    const MgLevel &F = P.lv[c - 1], &lv = P.lv[c];
    int c0, cnt;
    mg_own_range(lv, blockIdx.x, c0, cnt);
    if (cnt <= 0) return;
    int fa, fb;
    mg_fine_rows(lv, F, c0, cnt, fa, fb);
    float *rf = sm + P.sm_vec;          // fine residual rows fa .. fb
    mg_stage(P.res + F.g, F.nn, fa * F.Nx, (fb + 1) * F.Nx, rf, 0, 0, rf, tag, status);
    for (int k = threadIdx.x; k < cnt; k += kMgThreads) {
        const int I = c0 + k, cj = I / lv.Nx, ci = I - cj * lv.Nx;
        float b = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int fx = mg_fine_of(ci, q % 3, lv.cx), fy = mg_fine_of(cj, q / 3, lv.cy);
            if (fx < 0 || fx >= F.Nx || fy < 0 || fy >= F.Ny) continue;
            const float w = ((q % 3 == 1) ? 1.0f : 0.5f) * ((q / 3 == 1) ? 1.0f : 0.5f);
            b = fmaf(w, rf[(fy - fa) * F.Nx + fx], b);
        }
        S.b[k] = b;
        const float z = kMgOmega * mg_l1inv(P, sm, c, k, I) * b;
        S.z1[k] = z;
        mg_st(P.z1 + lv.g + I, z, tag);
    }
    __syncthreads();
}

// Restriction to the first level held by block 0 (c = Lg) from the spread
// level c - 1, by all blocks: block b forms b = P^T res at the coarse nodes
// [b Ch, b Ch + Ch) (Ch = ceil(nn / blocks)) from the staged fine residual
// rows under them, and publishes it in the held level's z1 words (which a
// held level does not otherwise use).  Block 0 then stages the whole level.
__device__ __forceinline__ void mg_restrict_to_held(const MgPlan &P, float *sm, int c, unsigned tag, int *status)
{
    const MgLevel &F = P.lv[c - 1], &lv = P.lv[c];
    const int Ch = (lv.nn + (int)gridDim.x - 1) / (int)gridDim.x;
    const int c0 = blockIdx.x * Ch, cnt = min(Ch, lv.nn - c0);
    if (cnt <= 0) return;
    int fa, fb;
    mg_fine_rows(lv, F, c0, cnt, fa, fb);
    float *rf = sm + P.sm_vec;          // fine residual rows fa .. fb
    mg_stage(P.res + F.g, F.nn, fa * F.Nx, (fb + 1) * F.Nx, rf, 0, 0, rf, tag, status);
    for (int k = threadIdx.x; k < cnt; k += kMgThreads) {
        const int I = c0 + k, cj = I / lv.Nx, ci = I - cj * lv.Nx;
        float b = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int fx = mg_fine_of(ci, q % 3, lv.cx), fy = mg_fine_of(cj, q / 3, lv.cy);
            if (fx < 0 || fx >= F.Nx || fy < 0 || fy >= F.Ny) continue;
            const float w = ((q % 3 == 1) ? 1.0f : 0.5f) * ((q / 3 == 1) ? 1.0f : 0.5f);
            b = fmaf(w, rf[(fy - fa) * F.Nx + fx], b);
        }
        mg_st(P.z1 + lv.g + I, b, tag);
    }
    __syncthreads();
}

// Prolongation and post-smoothing at the spread level l from the coarse
// solution of level l + 1: with z2 = z1 + P zc and res = b - A z1,
//   z = z2 + omega D_l1^-1 (res - A P zc)   (published; zero off the unknowns)
// The coarse rows holding the parents of the nodes n0 - H .. n0 + cnt + H
// are staged, P zc is formed at those nodes, then the stencil runs.  zown:
// this block's results also into shared memory (level 0), or null.
__device__ __forceinline__ void mg_prolong(const MgPlan &P, float *sm, int l, const MgShared &S, unsigned tag,
                                           int *status, float *zown)
{
    const MgLevel &lv = P.lv[l], &Cl = P.lv[l + 1];
    int n0, cnt;
    mg_own_range(lv, blockIdx.x, n0, cnt);
    if (cnt <= 0) return;
    const int H = lv.Nx + 1, E = cnt + 2 * H;
    int ya, yb;
    mg_parent_rows(lv, Cl, n0, cnt, ya, yb);
    float *pz = sm + P.sm_vec;          // P zc at nodes n0 - H .. n0 + cnt + H
    float *cz = pz + E;                 // coarse rows ya .. yb
    mg_stage(P.zf + Cl.g, Cl.nn, ya * Cl.Nx, (yb + 1) * Cl.Nx, cz, 0, 0, cz, tag, status);
    for (int u = threadIdx.x; u < E; u += kMgThreads) {
        const int m = n0 - H + u;
        float v = 0.0f;
        if (m >= 0 && m < lv.nn) {
            const int j = m / lv.Nx, i = m - j * lv.Nx;
            int px0, px1, py0, py1;
            const int npx = mg_parents(i, Cl.cx, px0, px1);
            const int npy = mg_parents(j, Cl.cy, py0, py1);
            const float *r0 = cz + (py0 - ya) * Cl.Nx, *r1 = cz + (py1 - ya) * Cl.Nx;
            v = r0[px0];
            if (npx == 2) v += r0[px1];
            if (npy == 2) v += r1[px0];
            if (npx == 2 && npy == 2) v += r1[px1];
            v *= ((npx == 2) ? 0.5f : 1.0f) * ((npy == 2) ? 0.5f : 1.0f);
        }
        pz[u] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kMgThreads) {
        const int n = n0 + k;
        const float *p = pz + H + k;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) acc = fmaf(mg_coef(P, sm, l, q, k, n), p[(q / 3 - 1) * lv.Nx + (q % 3 - 1)], acc);
        const float li = mg_l1inv(P, sm, l, k, n);
        const float z = (li == 0.0f) ? 0.0f : S.z1[k] + p[0] + kMgOmega * li * (S.res[k] - acc);
        mg_st(P.zf + lv.g + n, z, tag);
        if (zown != nullptr) zown[k] = z;
    }
    __syncthreads();
}

// Phases of the levels held by block 0: shared memory only, a block barrier
// after each.
struct MgHeld {
    const float *coef, *l1inv;
    float *b, *z1, *res, *zf;
    int Nx, Ny, nn;
};

__device__ __forceinline__ MgHeld mg_held(float *sm, const MgLevel &lv)
{
    MgHeld h;
    h.coef = sm + lv.sm;
    h.l1inv = h.coef + 9 * lv.nn;
    h.b = sm + lv.smv;
    h.z1 = h.b + lv.nn;
    h.res = h.z1 + lv.nn;
    h.zf = h.res + lv.nn;
    h.Nx = lv.Nx;
    h.Ny = lv.Ny;
    h.nn = lv.nn;
    return h;
}

// res = b - A z1 on a held level.
__device__ __forceinline__ void mgh_residual(const MgHeld &H)
{
    for (int n = threadIdx.x; n < H.nn; n += blockDim.x) {
        const int j = n / H.Nx, i = n - j * H.Nx;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int di = q % 3 - 1, dj = q / 3 - 1;
            if (i + di < 0 || i + di >= H.Nx || j + dj < 0 || j + dj >= H.Ny) continue;
            acc = fmaf(H.coef[q * H.nn + n], H.z1[n + dj * H.Nx + di], acc);
        }
        H.res[n] = H.b[n] - acc;
    }
    __syncthreads();
}

// b = P^T res of the finer held level F, then z1 = omega D_l1^-1 b (not at
// the coarsest level).
__device__ __forceinline__ void mgh_restrict(const MgHeld &F, const MgHeld &H, const MgLevel &lv, bool coarsest)
{
    for (int I = threadIdx.x; I < H.nn; I += blockDim.x) {
        const int cj = I / H.Nx, ci = I - cj * H.Nx;
        float b = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int fx = mg_fine_of(ci, q % 3, lv.cx), fy = mg_fine_of(cj, q / 3, lv.cy);
            if (fx < 0 || fx >= F.Nx || fy < 0 || fy >= F.Ny) continue;
            const float w = ((q % 3 == 1) ? 1.0f : 0.5f) * ((q / 3 == 1) ? 1.0f : 0.5f);
            b = fmaf(w, F.res[fy * F.Nx + fx], b);
        }
        H.b[I] = b;
        if (!coarsest) H.z1[I] = kMgOmega * H.l1inv[I] * b;
    }
    __syncthreads();
}

// Prolongation and post-smoothing on a held level from the coarser held
// level C (its zf): z = z1 + P zc + omega D_l1^-1 (res - A P zc).  P zc is
// formed once a node, into b (not needed after the level's residual), then
// the stencil reads it.
__device__ __forceinline__ void mgh_prolong(const MgHeld &H, const MgHeld &Cz, const MgLevel &Cl)
{
    for (int n = threadIdx.x; n < H.nn; n += blockDim.x) {
        const int j = n / H.Nx, i = n - j * H.Nx;
        int px0, px1, py0, py1;
        const int npx = mg_parents(i, Cl.cx, px0, px1);
        const int npy = mg_parents(j, Cl.cy, py0, py1);
        const float *r0 = Cz.zf + py0 * Cz.Nx, *r1 = Cz.zf + py1 * Cz.Nx;
        float pz = r0[px0];
        if (npx == 2) pz += r0[px1];
        if (npy == 2) pz += r1[px0];
        if (npx == 2 && npy == 2) pz += r1[px1];
        H.b[n] = pz * (((npx == 2) ? 0.5f : 1.0f) * ((npy == 2) ? 0.5f : 1.0f));
    }
    __syncthreads();
    for (int n = threadIdx.x; n < H.nn; n += blockDim.x) {
        const int j = n / H.Nx, i = n - j * H.Nx;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int di = q % 3 - 1, dj = q / 3 - 1;
            if (i + di < 0 || i + di >= H.Nx || j + dj < 0 || j + dj >= H.Ny) continue;
            acc = fmaf(H.coef[q * H.nn + n], H.b[n + dj * H.Nx + di], acc);
        }
        const float li = H.l1inv[n];
        H.zf[n] = (li == 0.0f) ? 0.0f : H.z1[n] + H.b[n] + kMgOmega * li * (H.res[n] - acc);
    }
    __syncthreads();
}

// The V-cycle on b0 (already in level 0's b): the result lands in level 0's
// zf words with this tag.  Levels 0 .. Lg - 1 are spread over the blocks;
// block 0 runs levels Lg .. L - 1 in its shared memory and publishes level
// Lg's result for the way up.
template <class Defer>
__device__ void mg_vcycle(const MgPlan &P, float *sm, const double *cinv, unsigned tag, int *status, Defer defer)
{
    const int L = P.L, Lg = P.Lg;
    if (Lg == 0) {
        defer();
        // one block holds every level
        const MgHeld H = mg_held(sm, P.lv[0]);
        for (int n = threadIdx.x; n < H.nn; n += blockDim.x) H.z1[n] = kMgOmega * H.l1inv[n] * H.b[n];
        __syncthreads();
        for (int l = 0; l + 1 < L; l++) {
            const MgHeld Hl = mg_held(sm, P.lv[l]);
            mgh_residual(Hl);
            mgh_restrict(Hl, mg_held(sm, P.lv[l + 1]), P.lv[l + 1], l + 1 == L - 1);
        }
        const MgHeld Hc = mg_held(sm, P.lv[L - 1]);
        if (threadIdx.x < Hc.nn) {
            double z = 0;
            for (int m = 0; m < Hc.nn; m++) z = fma(cinv[threadIdx.x * kMgCoarse + m], (double)Hc.b[m], z);
            Hc.zf[threadIdx.x] = (float)z;
        }
        __syncthreads();
        for (int l = L - 2; l >= 0; l--) mgh_prolong(mg_held(sm, P.lv[l]), mg_held(sm, P.lv[l + 1]), P.lv[l + 1]);
        return;
    }
    {
        // pre-smoothing at level 0
        const MgLevel &lv = P.lv[0];
        const MgShared S = mg_shared(sm, lv);
        int n0, cnt;
        mg_own_range(lv, blockIdx.x, n0, cnt);
        for (int k = threadIdx.x; k < cnt; k += kMgThreads) {
            const float z = kMgOmega * sm[9 * lv.C + k] * S.b[k];
            S.z1[k] = z;
            mg_st(P.z1 + n0 + k, z, tag);
        }
    }
    for (int l = 0; l < Lg; l++) {
        mg_residual(P, sm, l, mg_shared(sm, P.lv[l]), tag, status);
        if (l + 1 < Lg) mg_restrict(P, sm, l + 1, mg_shared(sm, P.lv[l + 1]), tag, status);
    }
    mg_restrict_to_held(P, sm, Lg, tag, status);
    // work that is not on the V-cycle's path, while block 0 runs the held
    // levels (block 0 owns no level-0 nodes, so it has none)
    defer();
    if (blockIdx.x == 0) {
        {
            // the first held level's b from every block, then its
            // pre-smoothing step (not at the coarsest level)
            const MgHeld H = mg_held(sm, P.lv[Lg]);
            mg_stage(P.z1 + P.lv[Lg].g, H.nn, 0, H.nn, H.b, 0, 0, H.b, tag, status);
            if (Lg + 1 < L) {
                for (int n = threadIdx.x; n < H.nn; n += blockDim.x) H.z1[n] = kMgOmega * H.l1inv[n] * H.b[n];
            }
            __syncthreads();
        }
        for (int l = Lg; l + 1 < L; l++) {
            const MgHeld H = mg_held(sm, P.lv[l]);
            mgh_residual(H);
            mgh_restrict(H, mg_held(sm, P.lv[l + 1]), P.lv[l + 1], l + 1 == L - 1);
        }
        {
            // exact solve at the coarsest level
            const MgHeld H = mg_held(sm, P.lv[L - 1]);
            if (threadIdx.x < H.nn) {
                double z = 0;
                for (int m = 0; m < H.nn; m++) z = fma(cinv[threadIdx.x * kMgCoarse + m], (double)H.b[m], z);
                H.zf[threadIdx.x] = (float)z;
            }
            __syncthreads();
        }
        for (int l = L - 2; l >= Lg; l--) mgh_prolong(mg_held(sm, P.lv[l]), mg_held(sm, P.lv[l + 1]), P.lv[l + 1]);
        const MgHeld H = mg_held(sm, P.lv[Lg]);
        for (int n = threadIdx.x; n < H.nn; n += blockDim.x) mg_st(P.zf + P.lv[Lg].g + n, H.zf[n], tag);
        __syncthreads();      // the staging area of the spread phases aliases the held vectors
    }
    for (int l = Lg - 1; l >= 0; l--)
        mg_prolong(P, sm, l, mg_shared(sm, P.lv[l]), tag, status, l == 0 ? sm + P.sm_zf0 : nullptr);
}

// Shared memory of pcg_mg_kernel (the offsets are in the plan): level 0's
// rows, the spread levels' vectors, the held levels' rows, level 0's own
// V-cycle results, the held levels' vectors (at least the reduction
// scratch), then doubles: the outer vectors r and w, the coarsest inverse
// and the elimination matrix.
inline size_t pcg_mg_smem(const MgPlan &P)
{
    const size_t doubles = 2 * (size_t)P.lv[0].C + kMgCoarse * kMgCoarse + 2 * kMgCoarse * kMgCoarse;
    return (size_t)P.sm_fp64 * sizeof(float) + doubles * sizeof(double);
}

__global__ void __launch_bounds__(kMgThreads, 1) pcg_mg_kernel(SolveArgs S, const MgPlan *__restrict__ plan,
                                                                int warm)
{
    extern __shared__ double smd[];
    // the level table, indexed by level below, from global memory into
    // shared memory
    __shared__ MgPlan P;
    for (int e = threadIdx.x; e < (int)(sizeof(MgPlan) / sizeof(int)); e += blockDim.x)
        reinterpret_cast<int *>(&P)[e] = __ldg(reinterpret_cast<const int *>(plan) + e);
    __syncthreads();
    float *sm = reinterpret_cast<float *>(smd);
    const int Nx = S.Nx, Ny = S.Ny, nn = Nx * Ny;
    const int nblocks = gridDim.x;
    const MgLevel &L0 = P.lv[0];
    int n0, cnt;
    mg_own_range(L0, blockIdx.x, n0, cnt);
    float *zf0 = sm + P.sm_zf0;                       // level 0's own V-cycle results
    double *scratch = reinterpret_cast<double *>(sm + P.sm_vec);   // 4 kMgThreads + 4 (between V-cycles)
    double *dv = reinterpret_cast<double *>(sm + P.sm_fp64);
    double *r = dv, *w = r + L0.C;                    // outer residual and A u
    double *cinv = w + L0.C;                          // kMgCoarse^2
    double *gj = cinv + kMgCoarse * kMgCoarse;        // kMgCoarse x 2 kMgCoarse (coarsest inverse)
    __shared__ double sh_scalar[5];
    __shared__ int sh_next;
    unsigned int episode = 0;
    unsigned tag0;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(tag0) : "l"(P.tag));
    double x[kMgTrips], sv[kMgTrips];   // the outer x and s of this thread's nodes (p is in S.p)
    double bbp = 0;                     // this thread's share of <b, b>

    // Level 0: FP64 rows (global, for the outer matvec), right-hand side,
    // start; FP32 rows (global for the Galerkin products, and this block's in
    // shared memory).  Entries towards nodes that are not unknowns are left
    // out of the FP32 rows, whose own rows are zero.
#pragma unroll
    for (int t = 0; t < kMgTrips; t++) {
        const int k = threadIdx.x + t * kMgThreads;
        x[t] = 0;
        sv[t] = 0;
        if (k >= cnt) continue;
        const int n = n0 + k, j = n / Nx, i = n - j * Nx;
        double cf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double f = 0;
        const bool dof = S.node_m[n] > S.dof_tol;
        bool coupled = false;
        if (dof) {
            build_row(S, i, j, cf, &f);
#pragma unroll
            for (int q = 0; q < 9; q++) coupled |= (__double_as_longlong(cf[q]) << 1) != 0;
            cf[4] += S.shift;
        }
        const bool unknown = dof && cf[4] > 0;
        if (unknown) {
            r[k] = f;
            x[t] = (warm && coupled) ? S.x[n] : 0.0;
        } else {
            r[k] = 0;
#pragma unroll
            for (int q = 0; q < 9; q++) cf[q] = 0;
        }
        S.p[n] = 0;
#pragma unroll
        for (int q = 0; q < 9; q++) S.coef[(size_t)q * nn + n] = cf[q];
        S.x[n] = x[t];
        double rsum = 0;
        float a[9];
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int di = q % 3 - 1, dj = q / 3 - 1;
            const bool in = i + di >= 0 && i + di < Nx && j + dj >= 0 && j + dj < Ny;
            const bool nbu = unknown && (q == 4 || (in && S.node_m[n + dj * Nx + di] > S.dof_tol));
            a[q] = nbu ? (float)cf[q] : 0.0f;
            if (nbu) rsum += cf[q];
        }
        mg_put_row(P, n, a, (float)rsum, sm, k, L0.C);
        if (unknown) bbp = fma(f, f, bbp);
    }
    // From a zero start r = b: <b, b> rides on the first grid barrier (a warm
    // start forms r = b - A x and its sums after the set-up instead).
    if (!warm) {
        double part0[4] = {bbp, 0, 0, 0};
        mg_sum4(part0, scratch);
        if (threadIdx.x == 0) S.partials[blockIdx.x] = part0[0];
    }
    if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
    double bb0 = 0;
    if (!warm) {
        double tot[4];
        mg_totals4(S.partials, nblocks, tot, scratch, 1);
        bb0 = tot[0];
    }
    // every block has read the tag counter: reserve this solve's tags
    if (blockIdx.x == 0 && threadIdx.x == 0) *P.tag = tag0 + (unsigned)S.maxit + 2u;

    // Coarse levels: Galerkin rows, one level after another (a grid barrier
    // after each level spread over the blocks, a block barrier after each
    // level held by block 0).
    for (int c = 1; c < P.L; c++) {
        const MgLevel &lv = P.lv[c];
        int c0, ccnt;
        mg_own_range(lv, blockIdx.x, c0, ccnt);
        for (int k = threadIdx.x; k < ccnt; k += kMgThreads) {
            const int I = c0 + k, cj = I / lv.Nx, ci = I - cj * lv.Nx;
            mg_galerkin_row(P, c, I, ci, cj, lv.local ? sm + lv.sm : nullptr);
        }
        if (!lv.local) {
            if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
        } else if (blockIdx.x == 0) {
            __syncthreads();
        }
    }
    // The coarsest level's inverse (block 0): Gauss-Jordan on the matrix of
    // its active nodes, in FP64, with the diagonal from the row sum.  A node
    // whose pivot is not positive is left out (its correction is zero).
    if (blockIdx.x == 0) {
        const MgLevel &lv = P.lv[P.L - 1];
        const int nc = lv.nn, w2 = 2 * kMgCoarse;
        for (int e = threadIdx.x; e < kMgCoarse * w2; e += kMgThreads) gj[e] = 0;
        __syncthreads();
        if (threadIdx.x < nc) {
            const int a = threadIdx.x, j = a / lv.Nx, i = a - j * lv.Nx;
            double off = 0;
#pragma unroll
            for (int q = 0; q < 9; q++) {
                if (q == 4) continue;
                const int di = q % 3 - 1, dj = q / 3 - 1;
                if (i + di < 0 || i + di >= lv.Nx || j + dj < 0 || j + dj >= lv.Ny) continue;
                const double e = (double)__ldcg(P.coef + (size_t)q * P.total + lv.g + a);
                gj[a * w2 + (a + dj * lv.Nx + di)] = e;
                off += e;
            }
            const bool active = __ldcg(P.l1inv + lv.g + a) > 0.0f;
            gj[a * w2 + a] = active ? (double)__ldcg(P.rsum + lv.g + a) - off : 0.0;
            gj[a * w2 + kMgCoarse + a] = 1.0;
        }
        __syncthreads();
        for (int piv = 0; piv < nc; piv++) {
            if (threadIdx.x == 0) {
                const double d = gj[piv * w2 + piv];
                sh_scalar[0] = d > 0 ? 1.0 / d : 0.0;     // one reciprocal a pivot
            }
            __syncthreads();
            const double id = sh_scalar[0];
            // this step's factors, read before the rows change
            const int row = threadIdx.x / w2, col = threadIdx.x % w2;
            const bool mine = threadIdx.x < nc * w2;
            const double fac = mine ? gj[row * w2 + piv] : 0.0;
            const double pv = mine ? gj[piv * w2 + col] : 0.0;
            __syncthreads();
            if (mine) {
                if (id == 0.0) {
                    if (row == piv || col == piv || col == kMgCoarse + piv) gj[row * w2 + col] = 0;
                } else if (row == piv) {
                    gj[row * w2 + col] = pv * id;
                } else {
                    gj[row * w2 + col] -= fac * (pv * id);
                }
            }
            __syncthreads();
        }
        for (int e = threadIdx.x; e < kMgCoarse * kMgCoarse; e += kMgThreads) {
            const int a = e / kMgCoarse, b = e % kMgCoarse;
            cinv[e] = (a < nc && b < nc) ? gj[a * w2 + kMgCoarse + b] : 0.0;
        }
        __syncthreads();
    }

    // warm start: r = b - A x, <b, b>, <r, r> (x of the neighbours is final
    // since the first barrier)
    double part[4] = {0, 0, 0, 0};
    double bb, rr;
    if (!warm) {
        bb = bb0;
        rr = bb0;
    } else {
#pragma unroll
        for (int t = 0; t < kMgTrips; t++) {
            const int k = threadIdx.x + t * kMgThreads;
            if (k >= cnt) continue;
            const int n = n0 + k, j = n / Nx, i = n - j * Nx;
            const double b = r[k];
            double ax = 0;
#pragma unroll
            for (int q = 0; q < 9; q++) {
                const int di = q % 3 - 1, dj = q / 3 - 1;
                if (i + di < 0 || i + di >= Nx || j + dj < 0 || j + dj >= Ny) continue;
                ax = fma(S.coef[(size_t)q * nn + n], __ldcg(S.x + n + dj * Nx + di), ax);
            }
            const double rk = b - ax;
            r[k] = rk;
            part[0] = fma(b, b, part[0]);
            part[1] = fma(rk, rk, part[1]);
        }
        mg_sum4(part, scratch);
        if (threadIdx.x == 0) {
            S.partials[0 * nblocks + blockIdx.x] = part[0];
            S.partials[1 * nblocks + blockIdx.x] = part[1];
            S.partials[2 * nblocks + blockIdx.x] = 0;
            S.partials[3 * nblocks + blockIdx.x] = 0;
        }
        if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
        mg_totals4(S.partials, nblocks, part, scratch);
        bb = part[0];
        rr = part[1];
    }
    const double target = S.tol * S.tol * bb;

    int it = 0;
    bool converged = false, failed = false;
    double alpha = 0, beta = 0, pi = 0, gamma = 0;
    if (bb == 0) {
#pragma unroll
        for (int t = 0; t < kMgTrips; t++) x[t] = 0;     // no load: the solution is zero
        rr = 0;
        converged = true;
    } else if (rr <= target) {
        converged = true;                                 // the start already meets the tolerance
    }
    // |r| and its reciprocal, formed once by thread 0 (GB300 runs FP64 at
    // 1/64 of the FP32 rate)
    if (threadIdx.x == 0 && !converged) {
        sh_scalar[3] = sqrt(rr);
        sh_scalar[4] = 1.0 / sh_scalar[3];
    }
    __syncthreads();
    double sig_u = 0;       // u = sig_u zf0 (the last V-cycle's result)
    for (int v = 0; !converged && !failed; v++) {
        const double sig_prev = sig_u;
        if (v > 0) {
            // s = w + beta s, r -= alpha s (the V-cycle's input); p and x
            // follow inside the V-cycle (defer below)
#pragma unroll
            for (int t = 0; t < kMgTrips; t++) {
                const int k = threadIdx.x + t * kMgThreads;
                if (k >= cnt) continue;
                const double sk = fma(beta, sv[t], w[k]);
                sv[t] = sk;
                r[k] = fma(-alpha, sk, r[k]);
            }
            it++;
        }
        // u = |r| V(r / |r|) (|r| of the last reduction), w = A u, and the
        // inner products
        const double sig = sh_scalar[3], isig = sh_scalar[4];
        sig_u = sig;
        {
            const MgShared Sh = mg_shared(sm, L0);
#pragma unroll
            for (int t = 0; t < kMgTrips; t++) {
                const int k = threadIdx.x + t * kMgThreads;
                if (k < cnt) Sh.b[k] = (float)(r[k] * isig);
            }
        }
        const unsigned tag = tag0 + (unsigned)v;
        // p = u + beta p, x += alpha p, with u = sig_prev zf0 (the last
        // V-cycle's result, in zf0 until level 0's prolongation)
        auto defer = [&]() {
            if (v == 0) return;
#pragma unroll
            for (int t = 0; t < kMgTrips; t++) {
                const int k = threadIdx.x + t * kMgThreads;
                if (k >= cnt) continue;
                const int n = n0 + k;
                const double pk = fma(beta, S.p[n], sig_prev * (double)zf0[k]);
                S.p[n] = pk;
                x[t] = fma(alpha, pk, x[t]);
            }
        };
        mg_vcycle(P, sm, cinv, tag, S.status, defer);
        {
            // the V-cycle's result at this block's nodes and their halo of
            // Nx + 1 nodes on either side: a held level 0's zf, or this
            // block's own results (zf0) and the neighbours' staged words
            const bool held0 = P.Lg == 0;
            const int H = Nx + 1;
            const float *zh = sm + P.lv[0].smv + 3 * P.lv[0].C;
            float *st = sm + P.sm_vec;      // zf at nodes n0 - H .. n0 + cnt + H
            if (!held0 && cnt > 0) {
                for (int k = threadIdx.x; k < cnt; k += kMgThreads) st[H + k] = zf0[k];
                mg_stage(P.zf, nn, n0 - H, n0, st, n0 + cnt, n0 + cnt + H, st + H + cnt, tag, S.status);
            }
            part[0] = part[1] = part[2] = part[3] = 0;
#pragma unroll
            for (int t = 0; t < kMgTrips; t++) {
                const int k = threadIdx.x + t * kMgThreads;
                if (k >= cnt) continue;
                const int n = n0 + k;
                double az = 0;
#pragma unroll
                for (int q = 0; q < 9; q++) {
                    // rows are zero towards nodes outside the grid (a held
                    // level 0 reads no node outside the level)
                    const int d = (q / 3 - 1) * Nx + (q % 3 - 1), m = n + d;
                    const float zq = !held0 ? st[H + k + d] : (m < 0 || m >= nn) ? 0.0f : zh[m];
                    az = fma(S.coef[(size_t)q * nn + n], (double)zq, az);
                }
                const float zo = held0 ? zh[n] : st[H + k];
                const double uk = sig * (double)zo, wk = sig * az, rk = r[k];
                zf0[k] = zo;
                w[k] = wk;
                part[0] = fma(rk, uk, part[0]);
                part[1] = fma(wk, uk, part[1]);
                part[2] = fma(sv[t], uk, part[2]);
                part[3] = fma(rk, rk, part[3]);
            }
        }
        __syncthreads();      // the scratch aliases the held levels' vectors (a held level 0's zf)
        mg_sum4(part, scratch);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) S.partials[c * nblocks + blockIdx.x] = part[c];
        }
        if (!tile_grid_barrier(S.barrier, ++episode * (unsigned)nblocks, S.status)) return;
        mg_totals4(S.partials, nblocks, part, scratch);
        const double gn = part[0], dl = part[1], sg = part[2];
        rr = part[3];
        if (threadIdx.x == 0) {
            int next = 0;                       // 0: go on, 1: give up, 2: converged
            if (!(rr == rr)) {
                next = 1;                       // NaN
            } else if (rr <= target) {
                next = 2;
            } else if (it >= S.maxit) {
                next = 1;
            } else {
                const double bn = (v == 0) ? 0.0 : -alpha * sg / gamma;
                const double pn = dl + 2.0 * bn * sg + bn * bn * pi;
                if (!(pn > 0)) {
                    next = 1;                   // breakdown: report non-convergence
                } else {
                    sh_scalar[0] = bn;
                    sh_scalar[1] = pn;
                    sh_scalar[2] = gn / pn;
                    sh_scalar[3] = sqrt(rr);
                    sh_scalar[4] = 1.0 / sh_scalar[3];
                }
            }
            sh_next = next;
        }
        __syncthreads();
        const int next = sh_next;
        if (next == 1) failed = true;
        if (next == 2) converged = true;
        if (next == 0) {
            beta = sh_scalar[0];
            pi = sh_scalar[1];
            alpha = sh_scalar[2];
            gamma = gn;
        }
        __syncthreads();
    }
#pragma unroll
    for (int t = 0; t < kMgTrips; t++) {
        const int k = threadIdx.x + t * kMgThreads;
        if (k < cnt) S.x[n0 + k] = x[t];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.sp->solve_iters = it;
        S.sp->solve_converged = converged ? 1 : 0;
        S.sp->solve_rel_resid = (bb > 0) ? sqrt(rr / bb) : 0.0;
        if (!converged) atomicOr(S.status, MPMG_DEV_ERR_SOLVER);
    }
}

// Nodal fluidity back to the particles, then the stress update
// (g_nonlocal_mu2.c:545-564 and :160-218; g_nonlocal.c:559-578, :154-298).
// AVG: the element average of the four nodal values instead of the shape
// functions (g_nonlocal_avg.c:575-578). MU2 reads the trial stress the G2P
// kept (trial: p_d, t0xx, t0xy, t0yy, tau, value-major) in place of the
// strain rates.
template <bool MU2, bool AVG>
__global__ void __launch_bounds__(256) fluidity_stress_kernel(
    int n, int Nx, int Ex, mat::Elastic el, mat::NonlocalParams np, const StepParams *__restrict__ sp,
    const int *__restrict__ active, const int *__restrict__ in_element, const double *__restrict__ xl,
    const double *__restrict__ yl, const double *__restrict__ node_gf, const double *__restrict__ exx,
    const double *__restrict__ exy, const double *__restrict__ eyy, const double *__restrict__ wxy,
    const double *__restrict__ trial, double *__restrict__ gf, double *__restrict__ sxx,
    double *__restrict__ sxy, double *__restrict__ syy, double *__restrict__ gammap,
    double *__restrict__ gammadotp)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool act = active[i] != 0;
    double g = 0;
    if (act) {
        const int e = in_element[i];
        const int ci = e % Ex, cj = e / Ex;
        const int n0 = cj * Nx + ci;
        const double a = xl[i], b = yl[i];
        const double ox = 1 - a, oy = 1 - b;
        if (AVG) {
            g += 0.25 * node_gf[n0];
            g += 0.25 * node_gf[n0 + 1];
            g += 0.25 * node_gf[n0 + 1 + Nx];
            g += 0.25 * node_gf[n0 + Nx];
        } else {
            g += node_gf[n0] * (ox * oy);
            g += node_gf[n0 + 1] * (a * oy);
            g += node_gf[n0 + 1 + Nx] * (a * b);
            g += node_gf[n0 + Nx] * (ox * b);
        }
        gf[i] = g;
    }
    if (MU2) {
        if (!act) return;
        const size_t N = (size_t)n;
        const double p_d = trial[i];
        double s0 = 0, s1 = 0, s2 = 0, gp = gammap[i], gdp;
        if (p_d != p_d) {   // NaN trial pressure: the start-of-step stress stays
            s0 = sxx[i];
            s1 = sxy[i];
            s2 = syy[i];
        }
        mat::nonlocal_mu2_stress(el, g, p_d, trial[N + i], trial[2 * N + i], trial[3 * N + i],
                                 trial[4 * N + i], s0, s1, s2, gp, gdp);
        sxx[i] = s0;
        sxy[i] = s1;
        syy[i] = s2;
        gammap[i] = gp;
        gammadotp[i] = gdp;
    } else {
        double s0 = sxx[i], s1 = sxy[i], s2 = syy[i], gp = gammap[i];
        mat::nonlocal_stress(np, el.G, el.dt, sp->t, gf[i], exx[i], exy[i], eyy[i], wxy[i], s0, s1, s2, gp);
        sxx[i] = s0;
        sxy[i] = s1;
        syy[i] = s2;
        gammap[i] = gp;
    }
}

inline int blocks_for(size_t n, int threads)
{
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    return (int)(b > 0 ? b : 1);
}

}  // namespace

int mpmg_nonlocal_init(mpmg_ctx *ctx)
{
    const size_t ne = ctx->ne > 0 ? ctx->ne : 1, nn = ctx->nn;
    MPMG_CHECK(cudaMalloc(&ctx->elem_k, 10 * ne * sizeof(double)));
    MPMG_CHECK(cudaMalloc(&ctx->elem_f, 4 * ne * sizeof(double)));
    double **vecs[] = {&ctx->cg_x, &ctx->cg_r, &ctx->cg_p, &ctx->cg_q, &ctx->cg_dinv, &ctx->cg_w};
    for (double **v : vecs) {
        MPMG_CHECK(cudaMalloc(v, nn * sizeof(double)));
        MPMG_CHECK(cudaMemsetAsync(*v, 0, nn * sizeof(double), ctx->stream));
    }
    MPMG_CHECK(cudaMalloc(&ctx->cg_coef, 9 * nn * sizeof(double)));
    int per_sm = 0, sms = 0;
    MPMG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_kernel, kSolveThreads, 0));
    MPMG_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->dev));
    if (per_sm < 1) {
        mpmg_set_error("fluidity solver kernel cannot be resident");
        return MPMG_ERR_CUDA;
    }
    // One or two blocks per SM: enough to cover the nodes with grid-stride
    // loops while keeping the grid barrier short.
    int want = sms * (per_sm < 2 ? per_sm : 2);
    int need = (int)((nn + kSolveThreads - 1) / kSolveThreads);
    ctx->cg_blocks = want < need ? want : (need > 0 ? need : 1);
    // The tiled kernel: one block per SM, each block's share of the nodes
    // resident in shared memory, where it fits.
    ctx->cg_tile_blocks = 0;
    {
        // at least kTileThreads nodes a block, so that small grids take few
        // blocks (and a short grid barrier)
        int C = (int)((nn + sms - 1) / sms);
        if (C < kTileThreads) C = kTileThreads;
        // a block's halo (Nx + 1 nodes either side) must lie in the two
        // neighbouring blocks, the only ones its point-to-point wait covers
        if (C < ctx->cfg.Nx + 1) C = ctx->cfg.Nx + 1;
        const int blocks = C > 0 ? (int)((nn + C - 1) / C) : 0;
        const size_t smem = pcg_tile_smem(C, ctx->cfg.Nx);
        int optin = 0;
        MPMG_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
        if (blocks > 0 && smem <= (size_t)optin && C <= kTileTrips * kTileThreads && blocks <= 8 * 32) {
            MPMG_CHECK(cudaFuncSetAttribute(pcg_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
            int tile_per_sm = 0;
            MPMG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tile_per_sm, pcg_tile_kernel, kTileThreads,
                                                                     smem));
            if (tile_per_sm >= 1) {
                ctx->cg_tile_blocks = blocks;
                ctx->cg_tile_nodes = C;
                ctx->cg_tile_smem = smem;
            }
        }
    }
    // The multigrid-preconditioned kernel: one block per SM at most, each
    // block's share of every level and its outer vectors in shared memory.
    ctx->mg_host = nullptr;
    ctx->mg_dev = nullptr;
    ctx->mg_rows = nullptr;
    ctx->mg_words = nullptr;
    ctx->mg_tag = nullptr;
    ctx->mg_smem = 0;
    int mg_blocks = 0;
    {
        MgPlan P;
        memset(&P, 0, sizeof(P));
        // a grid whose level 0 fits one block runs on one block
        int nb = nn <= (size_t)kMgLocal ? 1 : (int)((nn + kMgThreads - 1) / kMgThreads);
        if (nb > sms) nb = sms;
        if (nb < 1) nb = 1;
        int Nx = ctx->cfg.Nx, Ny = ctx->cfg.Ny, L = 0, total = 0, cxs = 0, cys = 0;
        bool ok = Nx >= 1 && Ny >= 1;
        while (ok) {
            MgLevel &lv = P.lv[L];
            lv.Nx = Nx;
            lv.Ny = Ny;
            lv.nn = Nx * Ny;
            // on one block every level is held; otherwise level 0 is spread
            // and the coarser levels of at most kMgLocal nodes are held
            lv.local = (nb == 1 || (L > 0 && lv.nn <= kMgLocal)) ? 1 : 0;
            // a spread level 0 is shared by blocks 1 .. nb - 1: block 0, which
            // runs the held levels, then has no level-0 work (the outer
            // iteration's p and x updates of the other blocks run while it
            // holds the V-cycle)
            lv.b0 = (L == 0 && !lv.local) ? 1 : 0;
            lv.C = lv.local ? lv.nn : (lv.nn + (nb - lv.b0) - 1) / (nb - lv.b0);
            lv.cx = cxs;
            lv.cy = cys;
            lv.g = total;
            total += lv.nn;
            L++;
            if (Nx <= 3 && Ny <= 3) break;
            if (L == kMgMaxLevels) ok = false;
            cxs = Nx > 3;
            cys = Ny > 3;
            if (cxs) Nx = Nx / 2 + 1;
            if (cys) Ny = Ny / 2 + 1;
        }
        P.L = L;
        P.nblocks = nb;
        P.total = total;
        P.Lg = L;
        for (int l = L - 1; l >= 0 && P.lv[l].local; l--) P.Lg = l;
        // a hierarchy of one level (at most 3 x 3 nodes) is left to Jacobi
        ok = ok && L >= 2 && P.Lg < L && P.lv[0].C <= kMgTrips * kMgThreads && nb <= 8 * 32 &&
             P.lv[L - 1].nn <= kMgCoarse;
        if (ok) {
            // shared memory offsets (floats)
            int off = 10 * P.lv[0].C;                    // level 0's rows
            for (int l = 0; l < P.Lg; l++) {
                P.lv[l].sm = off;                        // spread levels: b, z1, res
                off += 3 * P.lv[l].C;
            }
            for (int l = P.Lg; l < L; l++) {
                if (l == 0) continue;                    // a held level 0 keeps its rows at 0
                P.lv[l].sm = off;                        // held levels' rows
                off += 10 * P.lv[l].nn;
            }
            P.sm_zf0 = off;
            off += P.lv[0].C;
            off = (off + 1) & ~1;
            P.sm_vec = off;                              // held levels' vectors
            int vec = 0;
            for (int l = P.Lg; l < L; l++) {
                P.lv[l].smv = off + vec;
                vec += 4 * P.lv[l].nn;
            }
            const int scratch = 2 * (4 * kMgThreads + 4);   // the reduction scratch (doubles) aliases them
            // so does the staging area of the spread phases: a level's range
            // and its halo, with the coarse rows of a prolongation, or the
            // fine rows of a restriction
            int ext = 0;
            for (int b = 0; b < nb; b++) {
                for (int l = 0; l < P.Lg; l++) {
                    const MgLevel &lv = P.lv[l];
                    int n0, cnt;
                    mg_own_range(lv, b, n0, cnt);
                    if (cnt <= 0) continue;
                    int ya, yb, fa, fb;
                    mg_parent_rows(lv, P.lv[l + 1], n0, cnt, ya, yb);
                    const int pro = cnt + 2 * (lv.Nx + 1) + (yb - ya + 1) * P.lv[l + 1].Nx;
                    if (pro > ext) ext = pro;
                    if (l >= 1) {
                        mg_fine_rows(lv, P.lv[l - 1], n0, cnt, fa, fb);
                        const int res = (fb - fa + 1) * P.lv[l - 1].Nx;
                        if (res > ext) ext = res;
                    }
                }
                if (P.Lg > 0 && P.Lg < L) {
                    // the restriction to the first held level, by all blocks
                    const MgLevel &lv = P.lv[P.Lg];
                    const int Ch = (lv.nn + nb - 1) / nb, c0 = b * Ch;
                    const int cnt = lv.nn - c0 < Ch ? lv.nn - c0 : Ch;
                    if (cnt > 0) {
                        int fa, fb;
                        mg_fine_rows(lv, P.lv[P.Lg - 1], c0, cnt, fa, fb);
                        const int res = (fb - fa + 1) * P.lv[P.Lg - 1].Nx;
                        if (res > ext) ext = res;
                    }
                }
            }
            int region = vec > scratch ? vec : scratch;
            if (ext > region) region = ext;
            off += region;
            P.sm_fp64 = (off + 1) & ~1;
        }
        const size_t smem = ok ? pcg_mg_smem(P) : 0;
        int optin = 0;
        MPMG_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
        if (ok && smem + sizeof(MgPlan) + 256 <= (size_t)optin) {
            MPMG_CHECK(cudaFuncSetAttribute(pcg_mg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int mg_per_sm = 0;
            MPMG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mg_per_sm, pcg_mg_kernel, kMgThreads, smem));
            if (mg_per_sm >= 1) {
                MPMG_CHECK(cudaMalloc(&ctx->mg_rows, 11 * (size_t)total * sizeof(float)));
                MPMG_CHECK(cudaMalloc(&ctx->mg_words, 3 * (size_t)total * sizeof(unsigned long long)));
                MPMG_CHECK(cudaMemsetAsync(ctx->mg_words, 0, 3 * (size_t)total * sizeof(unsigned long long),
                                           ctx->stream));
                MPMG_CHECK(cudaMalloc(&ctx->mg_tag, sizeof(unsigned int)));
                const unsigned int first_tag = 1;   // the pools start with tag 0
                MPMG_CHECK(cudaMemcpyAsync(ctx->mg_tag, &first_tag, sizeof(first_tag), cudaMemcpyHostToDevice,
                                           ctx->stream));
                P.coef = ctx->mg_rows;
                P.rsum = ctx->mg_rows + 9 * (size_t)total;
                P.l1inv = ctx->mg_rows + 10 * (size_t)total;
                P.z1 = ctx->mg_words;
                P.res = ctx->mg_words + total;
                P.zf = ctx->mg_words + 2 * (size_t)total;
                P.tag = ctx->mg_tag;
                ctx->mg_host = new MgPlan(P);
                MPMG_CHECK(cudaMalloc(&ctx->mg_dev, sizeof(MgPlan)));
                MPMG_CHECK(cudaMemcpyAsync(ctx->mg_dev, ctx->mg_host, sizeof(MgPlan), cudaMemcpyHostToDevice,
                                           ctx->stream));
                MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
                ctx->mg_smem = smem;
                mg_blocks = nb;
            }
        }
    }
    int part_blocks = ctx->cg_blocks > ctx->cg_tile_blocks ? ctx->cg_blocks : ctx->cg_tile_blocks;
    if (mg_blocks > part_blocks) part_blocks = mg_blocks;
    MPMG_CHECK(cudaMalloc(&ctx->cg_partials, 4 * (size_t)part_blocks * sizeof(double)));
    // barrier counter + generation, then one neighbour flag per tiled block
    MPMG_CHECK(cudaMalloc(&ctx->cg_barrier, (2 + (size_t)ctx->cg_tile_blocks) * sizeof(unsigned int)));
    MPMG_CHECK(cudaMemsetAsync(ctx->cg_barrier, 0, 2 * sizeof(unsigned int), ctx->stream));
    return MPMG_OK;
}

void mpmg_nonlocal_free(mpmg_ctx *ctx)
{
    double **ptrs[] = {&ctx->elem_k, &ctx->elem_f, &ctx->cg_x, &ctx->cg_r, &ctx->cg_p, &ctx->cg_q,
                       &ctx->cg_dinv, &ctx->cg_w, &ctx->cg_coef, &ctx->cg_partials};
    for (double **p : ptrs) {
        cudaFree(*p);
        *p = nullptr;
    }
    cudaFree(ctx->cg_barrier);
    ctx->cg_barrier = nullptr;
    cudaFree(ctx->mg_rows);
    cudaFree(ctx->mg_words);
    cudaFree(ctx->mg_tag);
    cudaFree(ctx->mg_dev);
    delete ctx->mg_host;
    ctx->mg_rows = nullptr;
    ctx->mg_words = nullptr;
    ctx->mg_tag = nullptr;
    ctx->mg_dev = nullptr;
    ctx->mg_host = nullptr;
}

// The fluidity system on element blocks elem_k and right-hand sides elem_f
// (the layout assemble_kernel writes), unknowns the nodes with node_m above
// the material's threshold: one cooperative launch of the PCG, the solution
// in x (its previous contents are the initial guess unless zero_start).  The
// forward step solves for the nodal fluidity; the adjoint step solves the
// same symmetric system for the adjoint of the fluidity.
int mpmg_solve_fluidity_system(mpmg_ctx *ctx, const double *elem_k, const double *elem_f, const double *node_m,
                               const int *cell_start, double *x, bool zero_start)
{
    cudaStream_t s = ctx->stream;
    const mpmg_config &c = ctx->cfg;
    const bool mu2 = c.material == MPMG_G_NONLOCAL_MU2;
    SolveArgs S;
    S.Nx = c.Nx;
    S.Ny = c.Ny;
    S.Ex = ctx->Ex;
    S.Ey = ctx->Ey;
    S.ne = (int)ctx->ne;
    S.dof_tol = mu2 ? 0.0 : MPMG_TOL;
    S.shift = mu2 ? 1e-10 : 0.0;
    S.tol = c.solver_tol;
    S.maxit = c.solver_maxit;
    S.node_m = node_m;
    S.cell_start = cell_start;
    S.elem_k = elem_k;
    S.elem_f = elem_f;
    S.x = x;
    S.r = ctx->cg_r;
    S.p = ctx->cg_p;
    S.q = ctx->cg_q;
    S.dinv = ctx->cg_dinv;
    S.w = ctx->cg_w;
    S.u = ctx->cg_x;
    S.coef = ctx->cg_coef;
    S.partials = ctx->cg_partials;
    S.barrier = ctx->cg_barrier;
    S.status = ctx->d_status;
    S.sp = ctx->d_params;
    if (zero_start) MPMG_CHECK(cudaMemsetAsync(x, 0, ctx->nn * sizeof(double), s));
    MPMG_CHECK(cudaMemsetAsync(ctx->cg_barrier, 0, 2 * sizeof(unsigned int), s));
    if (ctx->mg_dev != nullptr && c.solver_precond == MPMG_PRECOND_MULTIGRID) {
        int warm = zero_start ? 0 : 1;
        const MgPlan *plan = ctx->mg_dev;
        void *args[] = {&S, &plan, &warm};
        MPMG_CHECK(cudaLaunchCooperativeKernel((const void *)pcg_mg_kernel, dim3(ctx->mg_host->nblocks),
                                               dim3(kMgThreads), args, ctx->mg_smem, s));
    } else if (ctx->cg_tile_blocks > 0) {
        int C = ctx->cg_tile_nodes, warm = zero_start ? 0 : 1;
        unsigned int *flags = ctx->cg_barrier + 2;
        MPMG_CHECK(cudaMemsetAsync(flags, 0, (size_t)ctx->cg_tile_blocks * sizeof(unsigned int), s));
        void *args[] = {&S, &C, &warm, &flags};
        MPMG_CHECK(cudaLaunchCooperativeKernel((const void *)pcg_tile_kernel, dim3(ctx->cg_tile_blocks),
                                               dim3(kTileThreads), args, ctx->cg_tile_smem, s));
    } else {
        void *args[] = {&S};
        MPMG_CHECK(cudaLaunchCooperativeKernel((const void *)pcg_kernel, dim3(ctx->cg_blocks),
                                               dim3(kSolveThreads), args, 0, s));
    }
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}

// The fluidity solve on the assembled element blocks (ctx->elem_k,
// ctx->elem_f): the nodal fluidity lands in ctx->node_gf.
int mpmg_launch_solve(mpmg_ctx *ctx)
{
    return mpmg_solve_fluidity_system(ctx, ctx->elem_k, ctx->elem_f, ctx->node_m, ctx->cell_start, ctx->node_gf,
                                      !ctx->cfg.solver_warm_start);
}

int mpmg_launch_fluidity(mpmg_ctx *ctx)
{
    cudaStream_t s = ctx->stream;
    const mpmg_config &c = ctx->cfg;
    const bool mu2 = c.material == MPMG_G_NONLOCAL_MU2;
    const int n = (int)ctx->np, ne = (int)ctx->ne;
    mat::NonlocalParams np;
    np.E = c.mp[MPMG_MP_E];
    np.nu = c.mp[MPMG_MP_NU];
    np.mu_s = c.mp[MPMG_MP_MU_S];
    np.grains_rho = c.mp[MPMG_MP_GRAINS_RHO];
    np.B = c.mp[MPMG_MP_B];
    np.A = c.mp[MPMG_MP_A];
    np.grains_d = c.mp[MPMG_MP_GRAINS_D];
    np.cohesion = c.mp[MPMG_MP_COHESION];
    if (!mu2) {
        nonlocal_bulk_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, np, ctx->sxx, ctx->sxy, ctx->syy,
                                                                ctx->state[4], ctx->state[5], ctx->state[10]);
        ctx->launches += 1;
    }
    const double *xisq = mu2 ? ctx->state[6] : ctx->state[10];
    assemble_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(ne, ctx->Ex, ctx->inv_h, mu2 ? 1 : 0, ctx->cell_start,
                                                        ctx->perm, ctx->xl, ctx->yl, ctx->v, ctx->state[0],
                                                        ctx->state[5], xisq, ctx->elem_k, ctx->elem_f);
    ctx->launches += 1;

    int rc = mpmg_launch_solve(ctx);
    if (rc != MPMG_OK) return rc;

    mat::Elastic el;
    el.G = ctx->G;
    el.twoG = 2.0 * ctx->G;
    el.K = ctx->K;
    el.lambda = ctx->lambda;
    el.dt = c.dt;
    el.inv_G = 1.0 / ctx->G;
    el.inv_dt = 1.0 / c.dt;
    el.Gdt = ctx->G * c.dt;
    el.inv_Gdt = 1.0 / el.Gdt;
    if (mu2) {
        fluidity_stress_kernel<true, false><<<blocks_for(n, 256), 256, 0, s>>>(
            n, c.Nx, ctx->Ex, el, np, ctx->d_params, ctx->active, ctx->in_element, ctx->xl, ctx->yl,
            ctx->node_gf, ctx->exx, ctx->exy, ctx->eyy, ctx->wxy, ctx->nl_trial, ctx->state[3], ctx->sxx,
            ctx->sxy, ctx->syy, ctx->state[9], ctx->state[10]);
    } else {
        auto k = c.material == MPMG_G_NONLOCAL_AVG ? fluidity_stress_kernel<false, true>
                                                   : fluidity_stress_kernel<false, false>;
        k<<<blocks_for(n, 256), 256, 0, s>>>(
            n, c.Nx, ctx->Ex, el, np, ctx->d_params, ctx->active, ctx->in_element, ctx->xl, ctx->yl,
            ctx->node_gf, ctx->exx, ctx->exy, ctx->eyy, ctx->wxy, ctx->state[0], ctx->state[3], ctx->sxx,
            ctx->sxy, ctx->syy, ctx->state[9], ctx->state[10]);
    }
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
