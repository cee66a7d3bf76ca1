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

// Element blocks and right-hand sides (g_nonlocal_mu2.c:418-507).
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
    for (int k = k0; k < k1; k++) {
        const int i = (int)perm[k];
        if (dense_only && dense[i] == 0) continue;
        const double a = xl[i], b = yl[i];
        const double ox = 1 - a, oy = 1 - b;
        const double s[4] = {ox * oy, a * oy, a * b, ox * b};
        const double gx[4] = {-oy * inv_h, oy * inv_h, b * inv_h, -b * inv_h};
        const double gy[4] = {-ox * inv_h, -a * inv_h, a * inv_h, ox * inv_h};
        const double vol = v[i], xi = xisq[i];
        const double fv = vol * gfl[i] * xi;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            F[r] += fv * s[r];
#pragma unroll
            for (int c = r; c < 4; c++) {
                K[sym_index(r, c)] += vol * (xi * s[r] * s[c] + (gx[r] * gx[c] + gy[r] * gy[c]));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 10; k++) elem_k[(size_t)k * ne + e] = K[k];
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

// Nodal fluidity back to the particles, then the stress update
// (g_nonlocal_mu2.c:545-564 and :160-218; g_nonlocal.c:559-578, :154-298).
// AVG: the element average of the four nodal values instead of the shape
// functions (g_nonlocal_avg.c:575-578).
template <bool MU2, bool AVG>
__global__ void __launch_bounds__(256) fluidity_stress_kernel(
    int n, int Nx, int Ex, mat::Elastic el, mat::NonlocalParams np, const StepParams *__restrict__ sp,
    const int *__restrict__ active, const int *__restrict__ in_element, const double *__restrict__ xl,
    const double *__restrict__ yl, const double *__restrict__ node_gf, const double *__restrict__ exx,
    const double *__restrict__ exy, const double *__restrict__ eyy, const double *__restrict__ wxy,
    const double *__restrict__ dense, double *__restrict__ gf, double *__restrict__ sxx,
    double *__restrict__ sxy, double *__restrict__ syy, double *__restrict__ gammap,
    double *__restrict__ gammadotp)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool act = active[i] != 0;
    if (act) {
        const int e = in_element[i];
        const int ci = e % Ex, cj = e / Ex;
        const int n0 = cj * Nx + ci;
        const double a = xl[i], b = yl[i];
        const double ox = 1 - a, oy = 1 - b;
        double g = 0;
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
        double s0 = sxx[i], s1 = sxy[i], s2 = syy[i], gp = gammap[i], gdp;
        mat::nonlocal_mu2_stress(el, dense[i], gf[i], exx[i], exy[i], eyy[i], wxy[i], s0, s1, s2, gp, gdp);
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
    const int part_blocks = ctx->cg_blocks > ctx->cg_tile_blocks ? ctx->cg_blocks : ctx->cg_tile_blocks;
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
    if (ctx->cg_tile_blocks > 0) {
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
    el.K = ctx->K;
    el.lambda = ctx->lambda;
    el.dt = c.dt;
    el.inv_G = 1.0 / ctx->G;
    el.inv_dt = 1.0 / c.dt;
    if (mu2) {
        fluidity_stress_kernel<true, false><<<blocks_for(n, 256), 256, 0, s>>>(
            n, c.Nx, ctx->Ex, el, np, ctx->d_params, ctx->active, ctx->in_element, ctx->xl, ctx->yl,
            ctx->node_gf, ctx->exx, ctx->exy, ctx->eyy, ctx->wxy, ctx->state[0], ctx->state[3], ctx->sxx,
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
