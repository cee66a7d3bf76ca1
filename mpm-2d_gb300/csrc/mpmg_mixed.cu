// Mixed-precision explicit USL step (MPMG_PRECISION_MIXED).
//
// Same phases as the FP64 step (mpmg_step.cu), re-laid out for bandwidth:
//   * Particle state is FP32.  Positions are stored as the element index plus
//     FP32 local coordinates xl, yl in [0, 1) (the coordinates the reference's
//     shape functions use, particle.c:14-30), so the shape functions need no
//     subtraction and a position keeps ~1e-7 h of resolution anywhere in the
//     domain.  A particle that leaves the grid (process_usl.c:660-666) keeps
//     its global position in the xl, yl slots and the element sentinel.
//   * The stored element index is the sort key: there is no separate keys
//     pass; the binning (mpmg_bin.cu) sorts storage positions by it.
//   * The G2P runs over stored particles (independent, coalesced loads) and
//     writes each one to its sorted position (the binning's inverse
//     permutation) in the other buffer, so the storage stays in element order
//     from step to step at no extra traffic and the next step's gathers are
//     nearly sequential.
//   * P2G corner sums of an element's particle segment are FP32 (a few
//     particles each); the four elements around a node are summed in
//     float-float (an unevaluated sum of two FP32 values, ~48 bits) for mass
//     and momentum, the momentum update and the division by nodal mass are
//     float-float as well, all on the FP32 pipe, and the node's acceleration
//     and velocity are stored in FP32 for the gathers.
// Time and gravity advance on the device: the G2P's first thread moves t and
// the next step's gravity (loading.c:34-54) once all reads of them are done.
#include <math.h>
#include <string.h>

#include <vector>

#include "mpmg_internal.cuh"

namespace {

struct GeomM {
    int Nx, Ny, Ex, Ey, ne;
    float hf, inv_hf;
    double h;
    float xmaxf, ymaxf;
};

struct BcM {
    int kind;
    int left_col, right_col, bottom_row, top_row, lf, bf, rf, tf;
    double open_time;
    int hole_last_col;     // last column i with i h <= hole radius (square_silo.c)
    int wall_col;
};

struct Buf {
    float4 *A, *B, *C, *D;
};

Buf buf(const MixedState *s, int b)
{
    Buf o;
    o.A = s->A[b];
    o.B = s->B[b];
    o.C = s->C[b];
    o.D = s->D[b];
    return o;
}

struct MatF {
    float G, K, lambda, dt;
    float mu_s, mu_2, I0, grains_rho, grains_d, rho_critical;
};

// isolin (isolin.c:75-116) in FP32.
__device__ __forceinline__ void isolin_f(const MatF &p, float exx, float exy, float eyy, float wxy,
                                         float &sxx, float &sxy, float &syy)
{
    float trD = exx + eyy;
    float twoG = 2.0f * p.G;
    float dsjxx = p.lambda * trD + twoG * exx + 2.0f * wxy * sxy;
    float dsjxy = twoG * exy - wxy * (sxx - syy);
    float dsjyy = p.lambda * trD + twoG * eyy - 2.0f * wxy * sxy;
    sxx += p.dt * dsjxx;
    sxy += p.dt * dsjxy;
    syy += p.dt * dsjyy;
}

// g_local_mu2 (g_local_mu2.c:165-310) in FP32, plane-strain stress
// [[Txx, Txy, 0], [Txy, Tyy, 0], [0, 0, Tzz]].
__device__ __forceinline__ void g_local_mu2_f(const MatF &p, float m, float v, float exx, float exy,
                                              float eyy, float wxy, float &Txx, float &Txy, float &Tyy,
                                              float &Tzz, float &gp, float &gdp)
{
    const float G = p.G, dt = p.dt;
    const float twoG = 2.0f * G;
    const float trD = exx + eyy;
    const float lt = p.lambda * trD;
    // Jaumann terms W T - T W with W_xy = wxy
    const float JSxx = 2.0f * wxy * Txy;
    const float JSxy = wxy * (Tyy - Txx);
    const float JSyy = -2.0f * wxy * Txy;
    const float Txx_tr = (exx * twoG + lt + JSxx) * dt + Txx;
    const float Txy_tr = (exy * twoG + JSxy) * dt + Txy;
    const float Tyy_tr = (eyy * twoG + lt + JSyy) * dt + Tyy;
    const float Tzz_tr = lt * dt + Tzz;
    const float pm = (Txx_tr + Tyy_tr + Tzz_tr) * (1.0f / 3.0f);
    const float T0xx = Txx_tr - pm, T0yy = Tyy_tr - pm, T0zz = Tzz_tr - pm, T0xy = Txy_tr;
    const float tau_tr = sqrtf(0.5f * (T0xx * T0xx + 2.0f * T0xy * T0xy + T0yy * T0yy + T0zz * T0zz));
    const float p_tr = -pm;
    float nup = 0.0f;
    if (m / v < p.rho_critical || p_tr <= 0.0f) {
        Txx = Txy = Tyy = Tzz = 0.0f;
    } else if (p_tr > 0.0f) {
        const float S0 = p.mu_s * p_tr;
        float tau_tau = tau_tr, scale = 1.0f;
        if (tau_tr > S0) {
            const float S2 = p.mu_2 * p_tr;
            const float alpha = G * p.I0 * dt * sqrtf(p_tr / p.grains_rho) / p.grains_d;
            const float B = -(S2 + tau_tr + alpha);
            const float H = S2 * tau_tr + S0 * alpha;
            const float disc = sqrtf(B * B - 4.0f * H);
            tau_tau = (B > 0.0f) ? (-B - disc) * 0.5f : (2.0f * H) / (-B + disc);
            scale = tau_tau / tau_tr;
        }
        nup = (tau_tr - tau_tau) / G / dt;
        Txx = T0xx * scale - p_tr;
        Txy = T0xy * scale;
        Tyy = T0yy * scale - p_tr;
        Tzz = T0zz * scale - p_tr;
    }
    gp += nup * dt;
    gdp = nup;
}

__device__ __forceinline__ void bc_mask_m(const BcM &bc, int i, int j, double t_now, bool &mx, bool &my)
{
    mx = false;
    my = false;
    if (bc.kind == MPMG_BOX) {
        bool on_row = (i >= bc.left_col && i <= bc.right_col);
        bool on_col = (j >= bc.bottom_row && j <= bc.top_row);
        if (on_row && j == bc.bottom_row) { mx |= (bc.bf & 1) != 0; my |= (bc.bf & 2) != 0; }
        if (on_row && j == bc.top_row) { mx |= (bc.tf & 1) != 0; my |= (bc.tf & 2) != 0; }
        if (on_col && i == bc.left_col) { mx |= (bc.lf & 1) != 0; my |= (bc.lf & 2) != 0; }
        if (on_col && i == bc.right_col) { mx |= (bc.rf & 1) != 0; my |= (bc.rf & 2) != 0; }
    } else {
        if (j == 0 && !(i <= bc.hole_last_col && t_now > bc.open_time)) {
            mx = true;
            my = true;
        }
        if (i == 0 || i == bc.wall_col) mx = true;
    }
}

// ---------------------------------------------------------------------------

// P2G: a block takes 256 consecutive elements, one thread each, and works
// through them in passes of whole elements whose particles (a contiguous
// range of the binned order) fit a 1024-particle shared-memory stage.  Each
// pass stages slots and particle records with coalesced, batched loads (the
// slots are close to the identity because the storage is kept in element
// order); then every thread orders its element's stage indices by storage
// position (insertion sort in shared memory: the deterministic,
// launch-order-independent order), writes perm and rank, and sums its
// particles in that order: 4 corners x (m, mvx, mvy, fx, fy) in FP32
// (process_usl.c:491-522 per particle, regrouped per element).  An element
// with more particles than the stage is summed alone from global memory.
constexpr int kP2GThreads = 256;
constexpr int kP2GChunk = 1024;
constexpr int kP2GBatch = 2;        // particles per thread whose loads are in flight together

__device__ __forceinline__ void p2g_accumulate(float (&acc)[4][5], float ih, float grav, float xl, float yl,
                                               float vx, float vy, float m, float vol, float sxx, float sxy,
                                               float syy)
{
    const float ox = 1.0f - xl, oy = 1.0f - yl;
    const float s[4] = {ox * oy, xl * oy, xl * yl, ox * yl};
    const float gx[4] = {-oy * ih, oy * ih, yl * ih, -yl * ih};
    const float gy[4] = {-ox * ih, -xl * ih, xl * ih, ox * ih};
    const float pmx = vx * m, pmy = vy * m, pby = grav * m;
    const float s0 = -sxx * vol, s1 = -sxy * vol, s2 = -syy * vol;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        acc[a][0] += s[a] * m;
        acc[a][1] += s[a] * pmx;
        acc[a][2] += s[a] * pmy;
        acc[a][3] += gx[a] * s0 + gy[a] * s1;
        acc[a][4] += s[a] * pby + gx[a] * s1 + gy[a] * s2;
    }
}

__global__ void __launch_bounds__(kP2GThreads, 4) mx_p2g_kernel(GeomM g, const int *__restrict__ cell_start,
                                                                const uint32_t *__restrict__ slots,
                                                                uint32_t *__restrict__ perm,
                                                                uint32_t *__restrict__ rank, Buf P,
                                                                const StepParams *__restrict__ sp,
                                                                float *__restrict__ cell_sums)
{
    __shared__ float sh[9][kP2GChunk];
    __shared__ uint32_t sh_slot[kP2GChunk];
    __shared__ uint16_t sh_ord[kP2GChunk];
    __shared__ int sh_cs[kP2GThreads + 1];
    const int e0 = blockIdx.x * kP2GThreads;
    const int ne_blk = min(kP2GThreads, g.ne - e0);
    for (int t = threadIdx.x; t <= ne_blk; t += kP2GThreads) sh_cs[t] = cell_start[e0 + t];
    __syncthreads();
    const int me = threadIdx.x;
    const int k0 = me < ne_blk ? sh_cs[me] : 0, k1 = me < ne_blk ? sh_cs[me + 1] : 0;
    const float grav = (float)sp->gravity;
    const float ih = g.inv_hf;
    int ea = 0;
    while (ea < ne_blk) {
        // elements [ea, eb) of this pass: the most whose particles fit the stage
        const int limit = sh_cs[ea] + kP2GChunk;
        int lo = ea + 1, hi = ne_blk;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sh_cs[mid] <= limit) lo = mid;
            else hi = mid - 1;
        }
        const int eb = lo;
        const int base = sh_cs[ea], end = sh_cs[eb];
        const bool mine = me >= ea && me < eb && k1 > k0;
        float acc[4][5];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int f = 0; f < 5; f++) acc[a][f] = 0.0f;
        if (end - base <= kP2GChunk) {
            for (int k = base + (int)threadIdx.x; k < end; k += kP2GBatch * kP2GThreads) {
                uint32_t sl[kP2GBatch];
                float4 a4[kP2GBatch], b4[kP2GBatch];
                float c[kP2GBatch];
#pragma unroll
                for (int u = 0; u < kP2GBatch; u++) {
                    const int kk = k + u * kP2GThreads;
                    sl[u] = kk < end ? slots[kk] : 0u;
                }
#pragma unroll
                for (int u = 0; u < kP2GBatch; u++) {
                    if (k + u * kP2GThreads < end) {
                        a4[u] = P.A[sl[u]];
                        b4[u] = P.B[sl[u]];
                        c[u] = P.C[sl[u]].x;
                    }
                }
#pragma unroll
                for (int u = 0; u < kP2GBatch; u++) {
                    const int j = k + u * kP2GThreads - base;
                    if (j < end - base) {
                        sh_slot[j] = sl[u];
                        sh[0][j] = a4[u].x;
                        sh[1][j] = a4[u].y;
                        sh[2][j] = a4[u].z;
                        sh[3][j] = a4[u].w;
                        sh[4][j] = b4[u].x;
                        sh[5][j] = b4[u].y;
                        sh[6][j] = b4[u].z;
                        sh[7][j] = b4[u].w;
                        sh[8][j] = c[u];
                    }
                }
            }
            __syncthreads();
            if (mine) {
                const int j0 = k0 - base, j1 = k1 - base;
                for (int j = j0; j < j1; j++) {
                    const uint32_t x = sh_slot[j];
                    int t = j - 1;
                    while (t >= j0 && sh_slot[sh_ord[t]] > x) {
                        sh_ord[t + 1] = sh_ord[t];
                        t--;
                    }
                    sh_ord[t + 1] = (uint16_t)j;
                }
                for (int j = j0; j < j1; j++) {
                    const int q = sh_ord[j];
                    const uint32_t i = sh_slot[q];
                    perm[base + j] = i;
                    rank[i] = (uint32_t)(base + j);
                    p2g_accumulate(acc, ih, grav, sh[0][q], sh[1][q], sh[2][q], sh[3][q], sh[4][q], sh[5][q],
                                   sh[6][q], sh[7][q], sh[8][q]);
                }
            }
            __syncthreads();
        } else if (mine) {
            // a single element larger than the stage
            mpmg_order_segment(slots, perm, rank, k0, k1);
            for (int k = k0; k < k1; k++) {
                const uint32_t i = perm[k];
                const float4 a4 = P.A[i], b4 = P.B[i];
                p2g_accumulate(acc, ih, grav, a4.x, a4.y, a4.z, a4.w, b4.x, b4.y, b4.z, b4.w, P.C[i].x);
            }
        }
        if (mine) {
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int f = 0; f < 5; f++) cell_sums[(size_t)(a * 5 + f) * g.ne + e0 + me] = acc[a][f];
        }
        ea = eb;
    }
}

// Double-FP32 ("float-float") helpers: a value is hi + lo with |lo| <= ulp(hi)/2,
// about 48 significant bits, on the FP32 pipe (GB300's FP64 rate is 1/64 of
// its FP32 rate).  TwoSum is Knuth's error-free addition.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float v)
{
    const float s = __fadd_rn(hi, v);
    const float bv = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(v, bv));
    hi = s;
    lo = __fadd_rn(lo, err);
}

__device__ __forceinline__ void ff_norm(float &hi, float &lo)
{
    const float s = __fadd_rn(hi, lo);
    lo = __fsub_rn(lo, __fsub_rn(s, hi));
    hi = s;
}

// (nh + nl) / (dh + dl) rounded to FP32: one Newton correction of the FP32
// quotient with the exact residual nh - q dh (FMA).
__device__ __forceinline__ float ff_div(float nh, float nl, float dh, float dl, float r)
{
    const float q = __fmul_rn(nh, r);
    float res = __fmaf_rn(-q, dh, nh);
    res = __fadd_rn(res, nl);
    res = __fmaf_rn(-q, dl, res);
    return __fmaf_rn(res, r, q);
}

// Grid update, one thread per node: the four elements' corner sums in
// colour order (process_usl.c:524-540), float-float for mass and momentum;
// boundary masks; momentum update and nodal velocity / acceleration
// (process_usl.c:542-566).
__global__ void __launch_bounds__(256) mx_grid_kernel(GeomM g, BcM bc, const int *__restrict__ cell_start,
                                                      const float *__restrict__ cell_sums,
                                                      const StepParams *__restrict__ sp, double dt,
                                                      float dt_hi, float dt_lo, float tol,
                                                      float2 *__restrict__ node_mass, float4 *__restrict__ node4,
                                                      double *__restrict__ node_mx,
                                                      double *__restrict__ node_my, double *__restrict__ node_fx,
                                                      double *__restrict__ node_fy)
{
    const int nn = g.Nx * g.Ny;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int i = n % g.Nx, j = n / g.Nx;
    float mh = 0, ml = 0, xh = 0, xl = 0, yh = 0, yl = 0;
    float fx = 0, fy = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        int e = cj * g.Ex + ci;
        if (cell_start[e] == cell_start[e + 1]) continue;
        int a = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
        const float *cs = cell_sums + (size_t)(a * 5) * g.ne + e;
        ff_add(mh, ml, cs[0]);
        ff_add(xh, xl, cs[(size_t)g.ne]);
        ff_add(yh, yl, cs[(size_t)2 * g.ne]);
        fx += cs[(size_t)3 * g.ne];
        fy += cs[(size_t)4 * g.ne];
    }
    ff_norm(mh, ml);
    bool bx, by;
    bc_mask_m(bc, i, j, sp->t + dt, bx, by);
    if (bx) { xh = 0; xl = 0; fx = 0; }
    if (by) { yh = 0; yl = 0; fy = 0; }
    float4 nd = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mh > tol) {
        // 1/m to ~FP32 accuracy of the float-float mass, then
        // p += dt f with dt = dt_hi + dt_lo and the exact product error.
        float r = __frcp_rn(mh);
        r = __fmaf_rn(r, __fmaf_rn(-ml, r, __fmaf_rn(-mh, r, 1.0f)), r);
        const float px = __fmul_rn(dt_hi, fx), py = __fmul_rn(dt_hi, fy);
        const float ex = __fmaf_rn(dt_lo, fx, __fmaf_rn(dt_hi, fx, -px));
        const float ey = __fmaf_rn(dt_lo, fy, __fmaf_rn(dt_hi, fy, -py));
        ff_add(xh, xl, px);
        xl = __fadd_rn(xl, ex);
        ff_add(yh, yl, py);
        yl = __fadd_rn(yl, ey);
        ff_norm(xh, xl);
        ff_norm(yh, yl);
        nd.x = fx * r;
        nd.y = fy * r;
        nd.z = ff_div(xh, xl, mh, ml, r);
        nd.w = ff_div(yh, yl, mh, ml, r);
    }
    node_mass[n] = make_float2(mh, ml);
    node4[n] = nd;
    if (node_mx != nullptr) {
        node_mx[n] = (double)xh + (double)xl;
        node_my[n] = (double)yh + (double)yl;
        node_fx[n] = fx;
        node_fy[n] = fy;
    }
}

// One thread per stored particle i (coalesced, independent loads); the
// particle is written to its sorted position rank[i] of the other buffer.
template <int MATERIAL>
__global__ void __launch_bounds__(256, 4) mx_g2p_kernel(GeomM g, int n, MatF mp, const uint32_t *__restrict__ rank,
                                                     Buf S, Buf D, const int *__restrict__ cell_src,
                                                     int *__restrict__ cell_dst, const float4 *__restrict__ node4,
                                                     uint32_t *__restrict__ bins, StepParams *sp, double dt,
                                                     int gravity_mode, double gravity_const)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        // Advance t and compute the next step's body force (the driver's
        // time_varying_loads, loading.c:34-54).  No kernel of this step reads
        // them after this point.
        const double t = sp->t + dt;
        sp->t = t;
        sp->step_count += 1;
        double grav;
        if (gravity_mode == MPMG_GRAVITY_CONSTANT) grav = gravity_const;
        else if ((0.1 + sp->step_start_time) > t) grav = -9.8 * ((t - sp->step_start_time) / 0.1);
        else grav = -9.8;
        sp->gravity = grav;
    }
    uint32_t new_key = (uint32_t)g.ne;
    uint32_t dst = 0;
    if (i < n) {
        dst = rank[i];
        const int e = cell_src[i];
        const float4 a4 = S.A[i], b4 = S.B[i], c4 = S.C[i], d4 = S.D[i];
        if (e >= g.ne) {
            // outside the grid: carried along unchanged
            D.A[dst] = a4;
            D.B[dst] = b4;
            D.C[dst] = c4;
            D.D[dst] = d4;
            cell_dst[dst] = g.ne;
        } else {
            const int ci = e % g.Ex, cj = e / g.Ex;
            const int n0 = cj * g.Nx + ci;
            const float ih = g.inv_hf;
            const float xl = a4.x, yl = a4.y;
            const float ox = 1.0f - xl, oy = 1.0f - yl;
            const float s[4] = {ox * oy, xl * oy, xl * yl, ox * yl};
            const float gx[4] = {-oy * ih, oy * ih, yl * ih, -yl * ih};
            const float gy[4] = {-ox * ih, -xl * ih, xl * ih, ox * ih};
            const float4 nq[4] = {node4[n0], node4[n0 + 1], node4[n0 + 1 + g.Nx], node4[n0 + g.Nx]};
            float xtt = 0, ytt = 0, dux = 0, duy = 0, exx = 0, eyy = 0, dxdy = 0, dydx = 0;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                xtt += s[a] * nq[a].x;
                ytt += s[a] * nq[a].y;
                dux += s[a] * nq[a].z;
                duy += s[a] * nq[a].w;
                exx += gx[a] * nq[a].z;
                eyy += gy[a] * nq[a].w;
                dxdy += gy[a] * nq[a].z;
                dydx += gx[a] * nq[a].w;
            }
            const float dtf = mp.dt;
            const float vx = a4.z + dtf * xtt, vy = a4.w + dtf * ytt;
            dux *= dtf;
            duy *= dtf;
            const float exy = 0.5f * (dxdy + dydx), wxy = 0.5f * (dxdy - dydx);
            const float m = b4.x;
            const float vol = b4.y * expf(dtf * (exx + eyy));
            float sxx = b4.z, sxy = b4.w, syy = c4.x, Tzz = c4.w, gp = d4.x, gdp = d4.y;
            if (MATERIAL == MPMG_ISOLIN) {
                isolin_f(mp, exx, exy, eyy, wxy, sxx, sxy, syy);
            } else {
                g_local_mu2_f(mp, m, vol, exx, exy, eyy, wxy, sxx, sxy, syy, Tzz, gp, gdp);
            }

            // New element from the local coordinates (WHICH_ELEMENT4, process_usl.c:43-44).
            float nxl = xl + dux * ih, nyl = yl + duy * ih;
            const float fxl = floorf(nxl), fyl = floorf(nyl);
            const int nci = ci + (int)fxl, ncj = cj + (int)fyl;
            nxl -= fxl;
            nyl -= fyl;
            const float xg = ((float)nci + nxl) * g.hf, yg = ((float)ncj + nyl) * g.hf;
            const bool inside = nci >= 0 && ncj >= 0 && nci < g.Ex && ncj < g.Ey && xg < g.xmaxf &&
                                yg < g.ymaxf && xg >= 0.0f && yg >= 0.0f;
            if (inside) {
                new_key = (uint32_t)(ncj * g.Ex + nci);
            } else {
                nxl = xg;      // global position of a particle that left the grid
                nyl = yg;
            }
            D.A[dst] = make_float4(nxl, nyl, vx, vy);
            D.B[dst] = make_float4(m, vol, sxx, sxy);
            D.C[dst] = make_float4(syy, c4.y + dux, c4.z + duy, Tzz);
            D.D[dst] = make_float4(gp, gdp, d4.z, 0.0f);
            cell_dst[dst] = (int)new_key;
        }
    }
    // the next step's bins, by destination position (the binning's first phase)
    mpmg_bin_count(new_key, i < n, (uint32_t)g.ne, dst >> 5, bins);
}

inline int blocks_for(size_t n, int threads)
{
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    return (int)(b > 0 ? b : 1);
}

GeomM make_geom(const mpmg_ctx *ctx)
{
    GeomM g;
    g.Nx = ctx->cfg.Nx;
    g.Ny = ctx->cfg.Ny;
    g.Ex = ctx->Ex;
    g.Ey = ctx->Ey;
    g.ne = (int)ctx->ne;
    g.h = ctx->cfg.h;
    g.hf = (float)ctx->cfg.h;
    g.inv_hf = (float)ctx->inv_h;
    g.xmaxf = (float)ctx->cfg.xmax;
    g.ymaxf = (float)ctx->cfg.ymax;
    return g;
}

BcM make_bc(const mpmg_ctx *ctx)
{
    BcM b = {};
    const mpmg_config &c = ctx->cfg;
    b.kind = c.bc;
    if (c.bc == MPMG_BOX) {
        b.left_col = (int)(size_t)(c.bcf[0] * (double)(c.Nx - 1));
        b.right_col = (int)(size_t)((c.bcf[0] + c.bcf[2]) * (double)(c.Nx - 1));
        b.bottom_row = (int)(size_t)(c.bcf[1] * (double)(c.Ny - 1));
        b.top_row = (int)(size_t)((c.bcf[1] + c.bcf[3]) * (double)(c.Ny - 1));
        b.lf = c.bci[0];
        b.bf = c.bci[1];
        b.rf = c.bci[2];
        b.tf = c.bci[3];
    } else {
        // the largest i with (i h <= radius), the reference's test, in FP64
        b.hole_last_col = -1;
        for (int i = 0; i < c.Nx && ((double)i * c.h) <= c.bcf[0]; i++) b.hole_last_col = i;
        b.open_time = c.bcf[1];
        b.wall_col = (int)((double)(c.Nx - 1) * c.bcf[2]);
    }
    return b;
}

MatF make_mat(const mpmg_ctx *ctx)
{
    MatF p;
    const mpmg_config &c = ctx->cfg;
    p.G = (float)ctx->G;
    p.K = (float)ctx->K;
    p.lambda = (float)(ctx->K - 2.0 * ctx->G / 3.0);
    p.dt = (float)c.dt;
    p.mu_s = (float)c.mp[MPMG_MP_MU_S];
    p.mu_2 = (float)c.mp[MPMG_MP_MU_2];
    p.I0 = (float)c.mp[MPMG_MP_I0];
    p.grains_rho = (float)c.mp[MPMG_MP_GRAINS_RHO];
    p.grains_d = (float)c.mp[MPMG_MP_GRAINS_D];
    p.rho_critical = (float)c.mp[MPMG_MP_RHO_CRITICAL];
    if (c.material == MPMG_ISOLIN) p.lambda = (float)ctx->lambda;
    return p;
}

template <typename T>
int dalloc(T **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return mpmg_cuda_status(e, "cudaMalloc (mixed state)");
    }
    return MPMG_OK;
}

// Cell and local coordinates of a host position (FP64, as WHICH_ELEMENT4).
void locate(const mpmg_ctx *ctx, double x, double y, int *cell, float *xl, float *yl)
{
    const mpmg_config &c = ctx->cfg;
    if (x < c.xmax && x >= 0.0 && y < c.ymax && y >= 0.0) {
        double fx = floor(x / c.h), fy = floor(y / c.h);
        if (fx < (double)ctx->Ex && fy < (double)ctx->Ey) {
            *cell = (int)(fx + fy * (double)ctx->Ex);
            double lx = (x - fx * c.h) / c.h, ly = (y - fy * c.h) / c.h;
            float fxl = (float)lx, fyl = (float)ly;
            if (fxl >= 1.0f) fxl = nextafterf(1.0f, 0.0f);
            if (fyl >= 1.0f) fyl = nextafterf(1.0f, 0.0f);
            *xl = fxl;
            *yl = fyl;
            return;
        }
    }
    *cell = (int)ctx->ne;
    *xl = (float)x;
    *yl = (float)y;
}

}  // namespace

int mpmg_mixed_init(mpmg_ctx *ctx, const double *m, const double *v, const double *x, const double *y,
                    const double *vx, const double *vy, const double *sxx, const double *sxy, const double *syy)
{
    if (ctx->cfg.material != MPMG_ISOLIN && ctx->cfg.material != MPMG_G_LOCAL_MU2) {
        mpmg_set_error("mixed precision supports isolin and g_local_mu2");
        return MPMG_ERR_UNSUPPORTED;
    }
    MixedState *s = new MixedState();
    memset(s, 0, sizeof(*s));
    ctx->mixed = s;
    const size_t n = ctx->np;
    int rc;
    for (int b = 0; b < 2; b++) {
        float4 **f[] = {&s->A[b], &s->B[b], &s->C[b], &s->D[b]};
        for (float4 **p : f)
            if ((rc = dalloc(p, n)) != MPMG_OK) return rc;
    }
    if ((rc = dalloc(&s->cell_sums, 20 * ctx->ne)) != MPMG_OK) return rc;
    if ((rc = dalloc(&s->node4, ctx->nn)) != MPMG_OK) return rc;
    if ((rc = dalloc(&s->node_mass, ctx->nn)) != MPMG_OK) return rc;
    MPMG_CHECK(cudaMemset(s->node_mass, 0, ctx->nn * sizeof(float2)));

    // host staging: element, local coordinates, records
    std::vector<float4> ha(n ? n : 1), hb(n ? n : 1), hc(n ? n : 1), hd(n ? n : 1);
    std::vector<int> cell(n ? n : 1);
    for (size_t i = 0; i < n; i++) {
        float xl, yl;
        locate(ctx, x[i], y[i], &cell[i], &xl, &yl);
        ha[i] = make_float4(xl, yl, (float)vx[i], (float)vy[i]);
        hb[i] = make_float4((float)m[i], (float)v[i], (float)sxx[i], (float)sxy[i]);
        hc[i] = make_float4((float)syy[i], 0.0f, 0.0f, 0.0f);
        hd[i] = make_float4(0.0f, 0.0f, mpmg_bits_float((int)i), 0.0f);
    }
    cudaError_t e = cudaSuccess;
    if (n > 0) {
        e = cudaMemcpy(s->A[0], ha.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->B[0], hb.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->C[0], hc.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->D[0], hd.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        // element index of the stored particles of buffer 0 (see cell_array)
        if (e == cudaSuccess) e = cudaMemcpy(ctx->in_element, cell.data(), n * sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return mpmg_cuda_status(e, "mixed state upload");
    s->cur = 0;
    // the first step's element counts; every G2P counts the next step's
    return mpmg_bin_count(ctx, (const uint32_t *)ctx->in_element);
}

void mpmg_mixed_free(mpmg_ctx *ctx)
{
    MixedState *s = ctx->mixed;
    if (s == nullptr) return;
    for (int b = 0; b < 2; b++) {
        cudaFree(s->A[b]);
        cudaFree(s->B[b]);
        cudaFree(s->C[b]);
        cudaFree(s->D[b]);
    }
    cudaFree(s->cell_sums);
    cudaFree(s->node4);
    cudaFree(s->node_mass);
    delete s;
    ctx->mixed = nullptr;
}

// Element index array of buffer b (buffer 0 uses ctx->in_element, buffer 1
// ctx->active: in the mixed form those two int arrays hold the stored
// particles' elements).
static int *cell_array(mpmg_ctx *ctx, int b)
{
    return b == 0 ? ctx->in_element : ctx->active;
}

int mpmg_mixed_step(mpmg_ctx *ctx)
{
    MixedState *s = ctx->mixed;
    cudaStream_t st = ctx->stream;
    const mpmg_config &c = ctx->cfg;
    const GeomM g = make_geom(ctx);
    const int n = (int)ctx->np;
    const int cur = s->cur, nxt = 1 - cur;
    const float dt_hi = (float)c.dt, dt_lo = (float)(c.dt - (double)dt_hi);

    mpmg_phase_begin(ctx, PH_SORT);
    int rc = mpmg_bin_scan_scatter(ctx, (const uint32_t *)cell_array(ctx, cur), nullptr);
    if (rc != MPMG_OK) return rc;
    mpmg_phase_end(ctx, PH_SORT);

    Buf S = buf(s, cur), D = buf(s, nxt);
    mpmg_phase_begin(ctx, PH_P2G);
    mx_p2g_kernel<<<blocks_for(ctx->ne, kP2GThreads), kP2GThreads, 0, st>>>(
        g, ctx->cell_start, ctx->bin.slots, ctx->perm, ctx->bin.rank, S, ctx->d_params, s->cell_sums);
    mpmg_phase_end(ctx, PH_P2G);

    mpmg_phase_begin(ctx, PH_GRID);
    mx_grid_kernel<<<blocks_for(ctx->nn, 256), 256, 0, st>>>(
        g, make_bc(ctx), ctx->cell_start, s->cell_sums, ctx->d_params, c.dt, dt_hi, dt_lo, (float)MPMG_TOL,
        s->node_mass, s->node4, ctx->node_mx, ctx->node_my, ctx->node_fx, ctx->node_fy);
    mpmg_phase_end(ctx, PH_GRID);

    mpmg_phase_begin(ctx, PH_G2P);
    const MatF mp = make_mat(ctx);
    if (c.material == MPMG_ISOLIN) {
        mx_g2p_kernel<MPMG_ISOLIN><<<blocks_for(n, 256), 256, 0, st>>>(
            g, n, mp, ctx->bin.rank, S, D, cell_array(ctx, cur), cell_array(ctx, nxt), s->node4, ctx->bin.counts,
            ctx->d_params, c.dt, c.gravity_mode, c.gravity);
    } else {
        mx_g2p_kernel<MPMG_G_LOCAL_MU2><<<blocks_for(n, 256), 256, 0, st>>>(
            g, n, mp, ctx->bin.rank, S, D, cell_array(ctx, cur), cell_array(ctx, nxt), s->node4, ctx->bin.counts,
            ctx->d_params, c.dt, c.gravity_mode, c.gravity);
    }
    mpmg_phase_end(ctx, PH_G2P);
    ctx->launches += 3;
    s->cur = nxt;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}

// ---------------------------------------------------------------------------
// Host read-back.

namespace {

int download4(mpmg_ctx *ctx, const float4 *d, std::vector<float4> &h)
{
    h.resize(ctx->np ? ctx->np : 1);
    if (ctx->np == 0) return MPMG_OK;
    MPMG_CHECK(cudaMemcpy(h.data(), d, ctx->np * sizeof(float4), cudaMemcpyDeviceToHost));
    return MPMG_OK;
}

int download_i(mpmg_ctx *ctx, const int *d, std::vector<int> &h)
{
    h.resize(ctx->np ? ctx->np : 1);
    if (ctx->np == 0) return MPMG_OK;
    MPMG_CHECK(cudaMemcpy(h.data(), d, ctx->np * sizeof(int), cudaMemcpyDeviceToHost));
    return MPMG_OK;
}

int pids(mpmg_ctx *ctx, std::vector<int> &pid)
{
    std::vector<float4> d;
    int rc = download4(ctx, ctx->mixed->D[ctx->mixed->cur], d);
    if (rc != MPMG_OK) return rc;
    pid.resize(d.size());
    for (size_t k = 0; k < ctx->np; k++) pid[k] = mpmg_float_bits(d[k].z);
    return MPMG_OK;
}

// Record and component of each writable particle field.
bool field_slot(const char *name, int *rec, int *comp)
{
    struct { const char *n; int r, c; } f[] = {
        {"vx", 0, 2}, {"vy", 0, 3}, {"m", 1, 0}, {"v", 1, 1}, {"sxx", 1, 2}, {"sxy", 1, 3}, {"Txx", 1, 2},
        {"Txy", 1, 3}, {"Tyx", 1, 3}, {"syy", 2, 0}, {"Tyy", 2, 0}, {"ux", 2, 1}, {"uy", 2, 2}, {"Tzz", 2, 3},
        {"state9", 3, 0}, {"state10", 3, 1}};
    for (auto &e : f) {
        if (strcmp(name, e.n) == 0) {
            *rec = e.r;
            *comp = e.c;
            return true;
        }
    }
    return false;
}

float4 *record(MixedState *s, int b, int rec)
{
    return rec == 0 ? s->A[b] : rec == 1 ? s->B[b] : rec == 2 ? s->C[b] : s->D[b];
}

float get_comp(const float4 &v, int c)
{
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

void set_comp(float4 &v, int c, float x)
{
    if (c == 0) v.x = x;
    else if (c == 1) v.y = x;
    else if (c == 2) v.z = x;
    else v.w = x;
}

}  // namespace

int mpmg_mixed_get_map(mpmg_ctx *ctx, int *in_element, int *active)
{
    MixedState *s = ctx->mixed;
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    std::vector<int> cell, pid;
    int rc;
    if ((rc = download_i(ctx, cell_array(ctx, s->cur), cell)) != MPMG_OK) return rc;
    if ((rc = pids(ctx, pid)) != MPMG_OK) return rc;
    for (size_t k = 0; k < ctx->np; k++) {
        int e = cell[k] < (int)ctx->ne ? cell[k] : -1;
        if (in_element) in_element[pid[k]] = e;
        if (active) active[pid[k]] = e >= 0 ? 1 : 0;
    }
    return MPMG_OK;
}

int mpmg_mixed_get(mpmg_ctx *ctx, const char *name, double *out)
{
    MixedState *s = ctx->mixed;
    const int b = s->cur;
    const size_t n = ctx->np;
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    int rc;
    if (strncmp(name, "node_", 5) == 0) {
        int comp = -1;
        if (strcmp(name, "node_ax") == 0) comp = 0;
        else if (strcmp(name, "node_ay") == 0) comp = 1;
        else if (strcmp(name, "node_vx") == 0) comp = 2;
        else if (strcmp(name, "node_vy") == 0) comp = 3;
        if (strcmp(name, "node_m") == 0) {
            std::vector<float2> h(ctx->nn);
            MPMG_CHECK(cudaMemcpy(h.data(), s->node_mass, ctx->nn * sizeof(float2), cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < ctx->nn; k++) out[k] = (double)h[k].x + (double)h[k].y;
            return MPMG_OK;
        }
        if (comp < 0) return MPMG_ERR_UNKNOWN_FIELD;   // FP64 node arrays: the common path
        std::vector<float4> h(ctx->nn);
        MPMG_CHECK(cudaMemcpy(h.data(), s->node4, ctx->nn * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < ctx->nn; k++) out[k] = get_comp(h[k], comp);
        return MPMG_OK;
    }
    std::vector<int> pid, cell;
    if ((rc = pids(ctx, pid)) != MPMG_OK) return rc;
    if (strcmp(name, "x") == 0 || strcmp(name, "y") == 0) {
        const bool isx = name[0] == 'x';
        std::vector<float4> a;
        if ((rc = download_i(ctx, cell_array(ctx, b), cell)) != MPMG_OK) return rc;
        if ((rc = download4(ctx, s->A[b], a)) != MPMG_OK) return rc;
        for (size_t k = 0; k < n; k++) {
            const double local = isx ? a[k].x : a[k].y;
            if (cell[k] < (int)ctx->ne) {
                int c = isx ? cell[k] % ctx->Ex : cell[k] / ctx->Ex;
                out[pid[k]] = ((double)c + local) * ctx->cfg.h;
            } else {
                out[pid[k]] = local;
            }
        }
        return MPMG_OK;
    }
    int rec, comp;
    if (!field_slot(name, &rec, &comp)) return MPMG_ERR_UNKNOWN_FIELD;
    std::vector<float4> a;
    if ((rc = download4(ctx, record(s, b, rec), a)) != MPMG_OK) return rc;
    for (size_t k = 0; k < n; k++) out[pid[k]] = (double)get_comp(a[k], comp);
    return MPMG_OK;
}

int mpmg_mixed_set(mpmg_ctx *ctx, const char *name, const double *in)
{
    MixedState *s = ctx->mixed;
    const int b = s->cur;
    const size_t n = ctx->np;
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    int rec, comp;
    if (!field_slot(name, &rec, &comp)) {
        mpmg_set_error("field '%s' cannot be written in the mixed-precision form", name);
        return MPMG_ERR_UNKNOWN_FIELD;
    }
    std::vector<int> pid;
    std::vector<float4> a;
    int rc;
    if ((rc = pids(ctx, pid)) != MPMG_OK) return rc;
    if ((rc = download4(ctx, record(s, b, rec), a)) != MPMG_OK) return rc;
    for (size_t k = 0; k < n; k++) set_comp(a[k], comp, (float)in[pid[k]]);
    if (n) MPMG_CHECK(cudaMemcpy(record(s, b, rec), a.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    return MPMG_OK;
}
