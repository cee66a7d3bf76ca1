// Mixed-precision explicit USL step (MPMG_PRECISION_MIXED and
// MPMG_PRECISION_MIXED_F64NODE).
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
//     float-float as well, all on the FP32 pipe (MPMG_PRECISION_MIXED_F64NODE:
//     in FP64), and the node's acceleration and velocity are stored in FP32
//     for the gathers.
// Time and gravity advance on the device: the G2P's first thread moves t and
// the next step's gravity (loading.c:34-54) once all reads of them are done.
#include <math.h>
#include <string.h>

#include <vector>

#include "mpmg_internal.cuh"

namespace {

struct GeomM {
    int Nx, Ny, Ex, Ey, ne;
    MpmgDiv div_Ex, div_Nx;
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
    // constant factors of the g_local_mu2 update, formed in FP64 on the host
    float inv_grains_rho;  // 1 / grains_rho
    float alpha_coef;      // G I0 dt / grains_d
    float inv_G_dt;        // 1 / (G dt)
    float inv_A2d2;        // 1 / (A^2 d^2), the nonlocal cooperativity scale (g_nonlocal_mu2)
};

// isolin (isolin.c:75-116) in FP32.  Every rounding is spelled out (explicit
// FMAs), so each instantiation of the G2P (single simulation or batch)
// evaluates the law to the same bits; left to the compiler, a sum of two
// products can be contracted either way round.
__device__ __forceinline__ void isolin_f(const MatF &p, float exx, float exy, float eyy, float wxy,
                                         float &sxx, float &sxy, float &syy)
{
    const float trD = __fadd_rn(exx, eyy);
    const float twoG = 2.0f * p.G, twoW = 2.0f * wxy;
    const float dsjxx = __fmaf_rn(twoW, sxy, __fmaf_rn(p.lambda, trD, __fmul_rn(twoG, exx)));
    const float dsjxy = __fmaf_rn(-wxy, __fsub_rn(sxx, syy), __fmul_rn(twoG, exy));
    const float dsjyy = __fmaf_rn(-twoW, sxy, __fmaf_rn(p.lambda, trD, __fmul_rn(twoG, eyy)));
    sxx = __fmaf_rn(p.dt, dsjxx, sxx);
    sxy = __fmaf_rn(p.dt, dsjxy, sxy);
    syy = __fmaf_rn(p.dt, dsjyy, syy);
}

// dp_ri_mt (dp_ri_mt.c:99-200) in FP32; szz travels where g_local_mu2 keeps
// Tzz.
__device__ __forceinline__ void dp_ri_mt_f(const MatF &p, float m, float v, float exx, float exy,
                                           float eyy, float wxy, float &sxx, float &sxy, float &syy,
                                           float &szz, float &gp, float &gdp)
{
    const float twoG = 2.0f * p.G, dt = p.dt, twoW = 2.0f * wxy;
    const float trD = __fadd_rn(exx, eyy);
    const float lt = __fmul_rn(p.lambda, trD);
    const float sxx_tr = __fmaf_rn(dt, __fmaf_rn(twoW, sxy, __fmaf_rn(twoG, exx, lt)), sxx);
    const float sxy_tr = __fmaf_rn(dt, __fmaf_rn(-wxy, __fsub_rn(sxx, syy), __fmul_rn(twoG, exy)), sxy);
    const float syy_tr = __fmaf_rn(dt, __fmaf_rn(-twoW, sxy, __fmaf_rn(twoG, eyy, lt)), syy);
    const float szz_tr = __fmaf_rn(dt, lt, szz);
    const float p_tr = __fmul_rn(-__fadd_rn(__fadd_rn(sxx_tr, syy_tr), szz_tr), 1.0f / 3.0f);
    const float t0xx = __fadd_rn(sxx_tr, p_tr), t0xy = sxy_tr, t0yy = __fadd_rn(syy_tr, p_tr);
    const float t0zz = __fadd_rn(szz_tr, p_tr);
    float q = __fmul_rn(t0xx, t0xx);
    q = __fmaf_rn(2.0f * t0xy, t0xy, q);
    q = __fmaf_rn(t0yy, t0yy, q);
    q = __fmaf_rn(t0zz, t0zz, q);
    const float tau_tr = sqrtf(0.5f * q);
    float nup = 0.0f;
    if (m < __fmul_rn(p.rho_critical, v) || p_tr <= 0.0f) {
        nup = __fmul_rn(tau_tr, p.inv_G_dt);
        sxx = sxy = syy = szz = 0.0f;
    } else if (p_tr > 0.0f) {
        const float S0 = __fmul_rn(p.mu_s, p_tr);
        float tau_tau = tau_tr, scale = 1.0f;
        if (tau_tr > S0) {
            tau_tau = S0;
            scale = __fdividef(S0, tau_tr);
        }
        nup = __fmul_rn(__fsub_rn(tau_tr, tau_tau), p.inv_G_dt);
        sxx = __fmaf_rn(scale, t0xx, -p_tr);
        sxy = __fmul_rn(scale, t0xy);
        syy = __fmaf_rn(scale, t0yy, -p_tr);
        szz = __fmaf_rn(scale, t0zz, -p_tr);
    }
    gp = __fmaf_rn(nup, dt, gp);
    gdp = nup;
}

// g_local_mu2 (g_local_mu2.c:165-310) in FP32, plane-strain stress
// [[Txx, Txy, 0], [Txy, Tyy, 0], [0, 0, Tzz]].
__device__ __forceinline__ void g_local_mu2_f(const MatF &p, float m, float v, float exx, float exy,
                                              float eyy, float wxy, float &Txx, float &Txy, float &Tyy,
                                              float &Tzz, float &gp, float &gdp)
{
    const float G = p.G, dt = p.dt;
    const float twoG = 2.0f * G;
    const float trD = __fadd_rn(exx, eyy);
    const float lt = __fmul_rn(p.lambda, trD);
    // Jaumann terms W T - T W with W_xy = wxy
    const float JSxx = __fmul_rn(2.0f * wxy, Txy);
    const float JSxy = __fmul_rn(wxy, __fsub_rn(Tyy, Txx));
    const float JSyy = -JSxx;
    const float Txx_tr = __fmaf_rn(__fadd_rn(__fmaf_rn(exx, twoG, lt), JSxx), dt, Txx);
    const float Txy_tr = __fmaf_rn(__fmaf_rn(exy, twoG, JSxy), dt, Txy);
    const float Tyy_tr = __fmaf_rn(__fadd_rn(__fmaf_rn(eyy, twoG, lt), JSyy), dt, Tyy);
    const float Tzz_tr = __fmaf_rn(lt, dt, Tzz);
    const float pm = __fmul_rn(__fadd_rn(__fadd_rn(Txx_tr, Tyy_tr), Tzz_tr), 1.0f / 3.0f);
    const float T0xx = __fsub_rn(Txx_tr, pm), T0yy = __fsub_rn(Tyy_tr, pm), T0zz = __fsub_rn(Tzz_tr, pm);
    const float T0xy = Txy_tr;
    float q = __fmul_rn(T0xx, T0xx);
    q = __fmaf_rn(2.0f * T0xy, T0xy, q);
    q = __fmaf_rn(T0yy, T0yy, q);
    q = __fmaf_rn(T0zz, T0zz, q);
    const float tau_tr = sqrtf(0.5f * q);
    const float p_tr = -pm;
    float nup = 0.0f;
    // m / v < rho_critical with v > 0; the divisions of the reference become
    // products with the host-formed reciprocals, and the two that remain use
    // the fast FP32 divide (about 2 ulp), all well inside the mixed form's
    // FP32 rounding budget.  Every rounding is spelled out, as in isolin_f.
    if (m < __fmul_rn(p.rho_critical, v) || p_tr <= 0.0f) {
        Txx = Txy = Tyy = Tzz = 0.0f;
    } else if (p_tr > 0.0f) {
        const float S0 = __fmul_rn(p.mu_s, p_tr);
        float tau_tau = tau_tr, scale = 1.0f;
        if (tau_tr > S0) {
            const float S2 = __fmul_rn(p.mu_2, p_tr);
            const float alpha = __fmul_rn(p.alpha_coef, sqrtf(__fmul_rn(p_tr, p.inv_grains_rho)));
            const float B = -__fadd_rn(__fadd_rn(S2, tau_tr), alpha);
            const float H = __fmaf_rn(S2, tau_tr, __fmul_rn(S0, alpha));
            const float disc = sqrtf(__fmaf_rn(B, B, -4.0f * H));
            tau_tau = (B > 0.0f) ? __fmul_rn(__fsub_rn(-B, disc), 0.5f) : __fdividef(2.0f * H, __fadd_rn(-B, disc));
            scale = __fdividef(tau_tau, tau_tr);
        }
        nup = __fmul_rn(__fsub_rn(tau_tr, tau_tau), p.inv_G_dt);
        Txx = __fmaf_rn(T0xx, scale, -p_tr);
        Txy = __fmul_rn(T0xy, scale);
        Tyy = __fmaf_rn(T0yy, scale, -p_tr);
        Tzz = __fmaf_rn(T0zz, scale, -p_tr);
    }
    gp = __fmaf_rn(nup, dt, gp);
    gdp = nup;
}

// g_nonlocal_mu2 on the FP32 state: the 2D trial Jaumann stress
// (g_nonlocal_mu2.c:166-186, with lambda = K - 2G/3 where the reference
// leaves it uninitialised), the bulk fluidity of
// calculate_bulk_granular_fluidity (:238-321) and the stress update once the
// nodal fluidity is known (:160-218).  These evaluate in FP64 (about sixty
// FP64 operations per particle, small beside the fluidity solve): the local
// fluidity p / (G dt) (1 / scale - 1) cancels near yield, and in FP32 that
// cancellation biased the flow (an 8 % faster silo discharge than the FP64
// form; within the FP64 form's own round-off spread once evaluated in FP64).
__device__ __forceinline__ void nonlocal_mu2_trial_f(const MatF &p, float exx, float exy, float eyy, float wxy,
                                                     float sxx, float sxy, float syy, float &p_tr, float &t0xx,
                                                     float &t0xy, float &t0yy, float &tau_tr)
{
    const double twoG = 2.0 * (double)p.G, trD = (double)exx + eyy, dt = p.dt, lam = p.lambda;
    const double w2s = 2.0 * (double)wxy * sxy;
    const double sxx_tr = sxx + dt * (lam * trD + twoG * exx + w2s);
    const double sxy_tr = sxy + dt * (twoG * exy - (double)wxy * ((double)sxx - syy));
    const double syy_tr = syy + dt * (lam * trD + twoG * eyy - w2s);
    const double pt = -0.5 * (sxx_tr + syy_tr);
    const double a = sxx_tr + pt, b = sxy_tr, c = syy_tr + pt;
    p_tr = (float)pt; t0xx = (float)a; t0xy = (float)b; t0yy = (float)c;
    tau_tr = (float)sqrt(0.5 * (a * a + 2.0 * b * b + c * c));
}

__device__ __forceinline__ void nonlocal_mu2_bulk_f(const MatF &p, float m, float v, float p_tr, float tau_tr,
                                                    float &dense, float &gf_local, float &xisq_inv)
{
    dense = (m < p.rho_critical * v || p_tr < 0.0f) ? 0.0f : 1.0f;
    gf_local = 0.0f;
    xisq_inv = 0.0f;
    if (dense != 0.0f && p_tr > 0.0f) {
        const double pr = p_tr, tau = tau_tr;
        const double S0 = (double)p.mu_s * pr;
        double tau_tau = tau;
        if (tau > S0) {
            const double S2 = (double)p.mu_2 * pr;
            const double alpha = (double)p.alpha_coef * sqrt(pr * (double)p.inv_grains_rho);
            const double B = -(S2 + tau + alpha);
            const double H = S2 * tau + S0 * alpha;
            const double disc = sqrt(B * B - 4.0 * H);
            tau_tau = (B > 0.0) ? (-B - disc) * 0.5 : (2.0 * H) / (-B + disc);
            // (1 / scale - 1) with scale = tau_tau / tau, as one quotient
            gf_local = (float)(pr * (double)p.inv_G_dt * ((tau - tau_tau) / tau_tau));
        }
        xisq_inv = (float)(fabs(tau_tau / pr - (double)p.mu_s) * (double)p.inv_A2d2);
    }
}

// p_d: the trial pressure where the particle is dense, 0 where it is not.
__device__ __forceinline__ void nonlocal_mu2_stress_f(const MatF &p, float gf, float p_d, float t0xx, float t0xy,
                                                      float t0yy, float tau_tr, float &sxx, float &sxy, float &syy,
                                                      float &gp, float &gdp)
{
    const float p_tr = p_d;
    float nup = 0.0f;
    if (!(p_tr > 0.0f)) {
        sxx = sxy = syy = 0.0f;
    } else {
        const double scale = (double)p_tr / ((double)p.G * p.dt * gf + p_tr);
        nup = (float)((tau_tr - tau_tr * scale) * (double)p.inv_G_dt);
        sxx = (float)(scale * t0xx - p_tr);
        sxy = (float)(scale * t0xy);
        syy = (float)(scale * t0yy - p_tr);
    }
    gp += nup * p.dt;
    gdp = nup;
}

// Per-particle values the nonlocal step keeps from the G2P to the assembly
// and the stress update after the fluidity solve, indexed by stored position:
// T = {p_d, t0xx, t0xy, t0yy}, the trial stress of g_nonlocal_mu2.c:166-186
// with the dense flag folded into the pressure (p_d = p_tr where dense, 0
// where not); F = {tau_tr, gf_local, xisq_inv, v_d}, v_d the updated volume
// where dense and 0 where not.
struct NLOut {
    float4 *T, *F;
};

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

// One simulation's constants.  A single simulation passes its own as a kernel
// parameter; a batch (several simulations concatenated in one context) keeps
// a device table of them and looks an element's or node's member up in the
// first-index tables.
struct MemberM {
    GeomM g;
    BcM bc;
    MatF mat;
    double dt;
    float dt_hi, dt_lo;    // dt = dt_hi + dt_lo (float-float)
    int gravity_mode;
    double gravity_const;
    int e0, nd0;           // first global element and node of the member
};

struct BatchView {
    const MemberM *m;
    const int *elem_off;   // first global element of each member, then the total
    const int *node_off;   // first global node of each member, then the total
    int count;
};

// The member holding global index x: the largest k with off[k] <= x.
__device__ __forceinline__ int find_member(const int *__restrict__ off, int count, int x)
{
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------

// P2G of a batch (a single simulation runs mx_p2g_grid_kernel, which sums
// the same way over element tiles and finishes the nodes itself): a block
// takes 256 consecutive elements, one thread each, and works
// through them in passes of whole elements whose particles (a contiguous
// range of the binned order) fit a 1024-particle shared-memory stage.  Each
// pass loads the range's slots (coalesced) and copies the particle records
// they point to into shared memory with asynchronous copies (cp.async; the
// slots are close to the identity because the storage is kept in element
// order, so the copies are nearly sequential); then every thread orders its
// element's stage indices by storage position (insertion sort in shared
// memory: the deterministic, launch-order-independent order), writes perm
// and rank, and sums its particles in that order: 4 corners x (m, mvx, mvy,
// fx, fy) in FP32 (process_usl.c:491-522 per particle, regrouped per
// element).  An element with more particles than the stage is summed alone
// from global memory.
//
// The stage is padded: with about four particles an element, the threads of
// a warp read entries about four apart, which in an unpadded array land on
// the same few banks (16-byte records 64 bytes apart, 4-byte words 16 bytes
// apart).  One pad record after every 8 records, one pad word after every 32
// words and two pad halves after every 64 halves spread them over all banks.
//
// The batched kernel's tile (elements per block = threads, particles staged
// per pass) is a template: mpmg_autotune picks one of kP2GVariants at run
// time.  The fused single-simulation kernel stages 4 entries a thread.
constexpr int kP2GPer = 4;   // stage entries per thread of the fused kernel

__device__ __forceinline__ int pad16b(int j) { return j + (j >> 3); }
__device__ __forceinline__ int pad4b(int j) { return j + (j >> 5); }
__device__ __forceinline__ int pad2b(int j) { return j + ((j >> 6) << 1); }

// (elements a block, staged particles) of the batched P2G; variant 0 is the
// default
constexpr int kP2GVariants = 3;
constexpr int kP2GElems[kP2GVariants] = {256, 128, 512};
constexpr int kP2GStage[kP2GVariants] = {1024, 512, 1024};

__device__ __forceinline__ void p2g_accumulate(float (&acc)[4][5], float ih, float grav, float4 a4, float4 b4,
                                               float syy)
{
    const float xl = a4.x, yl = a4.y, m = b4.x, vol = b4.y;
    const float ox = 1.0f - xl, oy = 1.0f - yl;
    const float s[4] = {ox * oy, xl * oy, xl * yl, ox * yl};
    const float gx[4] = {-oy * ih, oy * ih, yl * ih, -yl * ih};
    const float gy[4] = {-ox * ih, -xl * ih, xl * ih, ox * ih};
    const float pmx = a4.z * m, pmy = a4.w * m, pby = grav * m;
    const float s0 = -b4.z * vol, s1 = -b4.w * vol, s2 = -syy * vol;
    // every rounding spelled out, so that the batched and the fused kernels
    // (separate inlined copies) sum to the same bits
#pragma unroll
    for (int a = 0; a < 4; a++) {
        acc[a][0] = __fmaf_rn(s[a], m, acc[a][0]);
        acc[a][1] = __fmaf_rn(s[a], pmx, acc[a][1]);
        acc[a][2] = __fmaf_rn(s[a], pmy, acc[a][2]);
        acc[a][3] = __fadd_rn(acc[a][3], __fmaf_rn(gy[a], s1, __fmul_rn(gx[a], s0)));
        acc[a][4] = __fadd_rn(acc[a][4], __fmaf_rn(gy[a], s2, __fmaf_rn(gx[a], s1, __fmul_rn(s[a], pby))));
    }
}

template <int kP2GThreads, int kP2GChunk, bool BATCH>
__global__ void __launch_bounds__(kP2GThreads, 1024 / kP2GThreads) mx_p2g_kernel(
    const __grid_constant__ MemberM m0, BatchView bv, int ne_total, const int *__restrict__ cell_start,
    const uint32_t *__restrict__ slots, uint32_t *__restrict__ perm, uint32_t *__restrict__ rank, Buf P,
    const StepParams *__restrict__ sp, float *__restrict__ cell_sums)
{
    constexpr int kP2GPer = kP2GChunk / kP2GThreads;   // stage entries per thread
    constexpr int kP2GChunk16 = kP2GChunk + kP2GChunk / 8;
    constexpr int kP2GChunk4 = kP2GChunk + kP2GChunk / 32;
    constexpr int kP2GChunk2 = kP2GChunk + kP2GChunk / 32;
    __shared__ float4 sh_a[kP2GChunk16];
    __shared__ float4 sh_b[kP2GChunk16];
    __shared__ float sh_syy[kP2GChunk4];
    __shared__ uint32_t sh_slot[kP2GChunk4];
    __shared__ uint16_t sh_ord[kP2GChunk2];
    __shared__ int sh_cs[kP2GThreads + 1];
    const int e0 = blockIdx.x * kP2GThreads;
    const int ne_blk = min(kP2GThreads, ne_total - e0);
    // element offsets come from the scan, two kernels back; the slots from
    // the scatter, the kernel just before
    for (int t = threadIdx.x; t <= ne_blk; t += kP2GThreads) sh_cs[t] = cell_start[e0 + t];
    mpmg_pdl_wait();
    __syncthreads();
    const int me = threadIdx.x;
    const int k0 = me < ne_blk ? sh_cs[me] : 0, k1 = me < ne_blk ? sh_cs[me + 1] : 0;
    float grav, ih;
    if (BATCH) {
        const int k = find_member(bv.elem_off, bv.count, min(e0 + me, ne_total - 1));
        grav = (float)sp[k].gravity;
        ih = bv.m[k].g.inv_hf;
    } else {
        grav = (float)sp->gravity;
        ih = m0.g.inv_hf;
    }
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
            uint32_t sl[kP2GPer];
#pragma unroll
            for (int u = 0; u < kP2GPer; u++) {
                const int k = base + (int)threadIdx.x + u * kP2GThreads;
                sl[u] = k < end ? slots[k] : 0u;
            }
#pragma unroll
            for (int u = 0; u < kP2GPer; u++) {
                const int j = (int)threadIdx.x + u * kP2GThreads;
                if (base + j < end) {
                    sh_slot[pad4b(j)] = sl[u];
                    mpmg_cp_async16(&sh_a[pad16b(j)], P.A + sl[u]);
                    mpmg_cp_async16(&sh_b[pad16b(j)], P.B + sl[u]);
                    mpmg_cp_async4(&sh_syy[pad4b(j)], &P.C[sl[u]].x);
                }
            }
            mpmg_cp_async_wait_all();
            __syncthreads();
            if (mine) {
                const int j0 = k0 - base, j1 = k1 - base;
                for (int j = j0; j < j1; j++) {
                    const uint32_t x = sh_slot[pad4b(j)];
                    int t = j - 1;
                    while (t >= j0 && sh_slot[pad4b(sh_ord[pad2b(t)])] > x) {
                        sh_ord[pad2b(t + 1)] = sh_ord[pad2b(t)];
                        t--;
                    }
                    sh_ord[pad2b(t + 1)] = (uint16_t)j;
                }
                for (int j = j0; j < j1; j++) {
                    const int q = sh_ord[pad2b(j)];
                    const uint32_t i = sh_slot[pad4b(q)];
                    perm[base + j] = i;
                    rank[i] = (uint32_t)(base + j);
                    p2g_accumulate(acc, ih, grav, sh_a[pad16b(q)], sh_b[pad16b(q)], sh_syy[pad4b(q)]);
                }
            }
            __syncthreads();
        } else if (mine) {
            // a single element larger than the stage
            mpmg_order_segment(slots, perm, rank, k0, k1);
            for (int k = k0; k < k1; k++) {
                const uint32_t i = perm[k];
                p2g_accumulate(acc, ih, grav, P.A[i], P.B[i], P.C[i].x);
            }
        }
        if (mine) {
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int f = 0; f < 5; f++) cell_sums[(size_t)(a * 5 + f) * ne_total + e0 + me] = acc[a][f];
        }
        ea = eb;
    }
    mpmg_pdl_trigger();
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

// One node of the grid update: the four elements' corner sums in colour
// order (process_usl.c:524-540), float-float for mass and momentum; boundary
// masks; momentum update and nodal velocity / acceleration
// (process_usl.c:542-566).  cs + off[c] is the node's corner mass sum in
// colour element c (off[c] < 0 when that element is absent or holds no
// particle); the corner's other four sums follow at stride fs.
template <bool F64NODE, typename Off>
__device__ __forceinline__ void node_finish(const MemberM &M, double t_next, float tol, int i, int j, int n,
                                            const float *__restrict__ cs, const Off (&off)[4], Off fs,
                                            float2 *__restrict__ node_mass, float4 *__restrict__ node4,
                                            double *__restrict__ node_mx, double *__restrict__ node_my,
                                            double *__restrict__ node_fx, double *__restrict__ node_fy,
                                            double *__restrict__ node_m64)
{
    const double dt = M.dt;
    const float dt_hi = M.dt_hi, dt_lo = M.dt_lo;
    float mh = 0, ml = 0, xh = 0, xl = 0, yh = 0, yl = 0;
    float fx = 0, fy = 0;
    double m64 = 0, mx64 = 0, my64 = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        if (off[c] < 0) continue;
        const float *p = cs + off[c];
        if (F64NODE) {
            m64 += (double)p[0];
            mx64 += (double)p[fs];
            my64 += (double)p[2 * fs];
        } else {
            ff_add(mh, ml, p[0]);
            ff_add(xh, xl, p[fs]);
            ff_add(yh, yl, p[2 * fs]);
        }
        fx += p[3 * fs];
        fy += p[4 * fs];
    }
    bool bx, by;
    bc_mask_m(M.bc, i, j, t_next, bx, by);
    if (F64NODE) {
        if (bx) { mx64 = 0; fx = 0; }
        if (by) { my64 = 0; fy = 0; }
        float4 nd = make_float4(0.f, 0.f, 0.f, 0.f);
        if (m64 > (double)MPMG_TOL) {
            // FP64 momentum update and division (1 / m: the FP32 reciprocal
            // refined by one Newton step, ~2^-46 relative)
            double r = (double)__frcp_rn((float)m64);
            r = fma(r, fma(-m64, r, 1.0), r);
            mx64 += dt * (double)fx;
            my64 += dt * (double)fy;
            const float rf = (float)r;
            nd.x = fx * rf;
            nd.y = fy * rf;
            nd.z = (float)(mx64 * r);
            nd.w = (float)(my64 * r);
        }
        const float mhi = (float)m64;
        node_mass[n] = make_float2(mhi, (float)(m64 - (double)mhi));
        if (node_m64 != nullptr) node_m64[n] = m64;
        node4[n] = nd;
        if (node_mx != nullptr) {
            node_mx[n] = mx64;
            node_my[n] = my64;
            node_fx[n] = fx;
            node_fy[n] = fy;
        }
        return;
    }
    ff_norm(mh, ml);
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
    if (node_m64 != nullptr) node_m64[n] = (double)mh + (double)ml;
    node4[n] = nd;
    if (node_mx != nullptr) {
        node_mx[n] = (double)xh + (double)xl;
        node_my[n] = (double)yh + (double)yl;
        node_fx[n] = fx;
        node_fy[n] = fy;
    }
}

// Grid update of a batch, one thread per node, from the corner sums
// mx_p2g_kernel left in global memory.
template <bool F64NODE, bool BATCH>
__global__ void __launch_bounds__(256) mx_grid_kernel(const __grid_constant__ MemberM m0, BatchView bv, int ne_total,
                                                      int nn_total, const int *__restrict__ cell_start,
                                                      const float *__restrict__ cell_sums,
                                                      const StepParams *__restrict__ sp, float tol,
                                                      float2 *__restrict__ node_mass, float4 *__restrict__ node4,
                                                      double *__restrict__ node_mx,
                                                      double *__restrict__ node_my, double *__restrict__ node_fx,
                                                      double *__restrict__ node_fy, double *__restrict__ node_m64)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn_total) return;
    const int k = BATCH ? find_member(bv.node_off, bv.count, n) : 0;
    const MemberM &M = BATCH ? bv.m[k] : m0;
    const GeomM &g = M.g;
    const int ln = n - M.nd0;
    const int j = (int)mpmg_div((uint32_t)ln, g.div_Nx), i = ln - j * g.Nx;
    // the four elements in colour order, where they hold particles
    // (cell_start is from the scan, three kernels back)
    long long off[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        const int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        off[c] = -1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        const int e = M.e0 + cj * g.Ex + ci;
        const int a = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
        if (cell_start[e] != cell_start[e + 1]) off[c] = (long long)(a * 5) * ne_total + e;
    }
    const double t_next = sp[k].t + M.dt;
    mpmg_pdl_wait();        // the corner sums come from the P2G just before
    mpmg_pdl_trigger();
    node_finish<F64NODE>(M, t_next, tol, i, j, n, cell_sums, off, (long long)ne_total, node_mass, node4, node_mx,
                         node_my, node_fx, node_fy, node_m64);
}

// P2G and grid update in one kernel, for a single simulation.  A block takes
// a TX x TY tile of elements, one thread each, sums them exactly as
// mx_p2g_kernel does (the same staging, order and arithmetic), leaves the 20
// corner sums in shared memory and finishes the (TX - 1) x (TY - 1) nodes
// whose four elements all lie in the tile exactly as mx_grid_kernel does.
// Neighbouring tiles share one column or row of elements, which both sum to
// the same values; perm and rank of an element are written by the one tile
// where it is not in the first column or row.  An element with more
// particles than the stage is ordered in global memory: by its owner in
// perm, by the other tiles in a scratch copy of their own (one per kind of
// overlap).  The corner sums never reach global memory and the grid update
// needs no launch.
template <int TX, int TY>
struct FusedTile {
    static constexpr int threads = TX * TY;
    static constexpr int chunk = 4 * threads;                  // staged particles a pass
    static constexpr int c16 = chunk + chunk / 8, c4 = chunk + chunk / 32, c2 = chunk + chunk / 32;
    static constexpr int sum_stride = threads + 1;             // corner-sum row in shared memory
    static constexpr int rows_per_warp = 32 / TX;
    static constexpr size_t smem = sizeof(float4) * 2 * c16 + sizeof(float) * 2 * c4 + sizeof(uint16_t) * c2;
    static_assert(TX * (32 / TX) == 32 && rows_per_warp <= 2 && threads % 32 == 0, "a warp stages one or two whole tile rows");
    static_assert(sizeof(float) * 20 * sum_stride <= smem, "the corner sums overlay the stage");
};
constexpr int kFusedTX = 16, kFusedTY = 16;
using FusedT = FusedTile<kFusedTX, kFusedTY>;

template <bool F64NODE, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, 1024 / (TX * TY)) mx_p2g_grid_kernel(
    const __grid_constant__ MemberM M, int np, int tiles_x, const int *__restrict__ cell_start,
    const uint32_t *__restrict__ slots, uint32_t *__restrict__ perm, uint32_t *__restrict__ rank,
    uint32_t *__restrict__ halo_perm, Buf P, const StepParams *__restrict__ sp, float tol,
    float2 *__restrict__ node_mass, float4 *__restrict__ node4, double *__restrict__ node_mx,
    double *__restrict__ node_my, double *__restrict__ node_fx, double *__restrict__ node_fy,
    double *__restrict__ node_m64)
{
    using T = FusedTile<TX, TY>;
    constexpr int NT = T::threads, CH = T::chunk, SS = T::sum_stride;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int sh_off[NT + 1];     // stage offsets of the tile's elements
    __shared__ int sh_gs[TY];          // storage position of each tile row's first particle
    __shared__ int sh_wsum[NT / 32];
    float4 *sh_a = reinterpret_cast<float4 *>(smem);
    float4 *sh_b = sh_a + T::c16;
    float *sh_syy = reinterpret_cast<float *>(sh_b + T::c16);
    uint32_t *sh_slot = reinterpret_cast<uint32_t *>(sh_syy + T::c4);
    uint16_t *sh_ord = reinterpret_cast<uint16_t *>(sh_slot + T::c4);
    float *sh_sum = reinterpret_cast<float *>(smem);

    const int me = threadIdx.x, lane = me & 31, warp = me >> 5;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int lx = me % TX, ly = me / TX;
    const int ei = tx * (TX - 1) - 1 + lx, ej = ty * (TY - 1) - 1 + ly;
    const bool exists = ei >= 0 && ej >= 0 && ei < M.g.Ex && ej < M.g.Ey;
    const bool owner = lx > 0 && ly > 0;
    // element offsets come from the scan, two kernels back
    int k0 = 0, k1 = 0;
    if (exists) {
        const int e = ej * M.g.Ex + ei;
        k0 = cell_start[e];
        k1 = cell_start[e + 1];
    }
    const int cnt = k1 - k0;
    // stage offsets: exclusive prefix of the counts in tile order
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) sh_wsum[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; w++) wbase += sh_wsum[w];
    sh_off[me] = wbase + incl - cnt;
    if (me == NT - 1) sh_off[NT] = wbase + incl;
    // a row's elements are consecutive, so its particles are one storage run
    if (exists && (lx == 0 || ei == 0)) sh_gs[ly] = k0;
    // the slots come from the scatter, the kernel just before
    mpmg_pdl_wait();
    __syncthreads();
    const float grav = (float)sp->gravity, ih = M.g.inv_hf;
    float acc[4][5];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int f = 0; f < 5; f++) acc[a][f] = 0.0f;
    int ea = 0;
    while (ea < NT) {
        // elements [ea, eb) of this pass: the most whose particles fit the
        // stage (usually all the rest)
        const int limit = sh_off[ea] + CH;
        int lo = sh_off[NT] <= limit ? NT : ea + 1, hi = NT;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sh_off[mid] <= limit) lo = mid;
            else hi = mid - 1;
        }
        const int eb = lo;
        const int base = sh_off[ea], end = sh_off[eb];
        const bool mine = me >= ea && me < eb && cnt > 0;
        if (end - base <= CH) {
            // each warp stages its tile rows' share of the pass (one or two
            // storage runs), four loads in flight a lane
            int s0 = 0, n0 = 0, g0 = 0, s1 = 0, n1 = 0, g1 = 0;
            {
                const int r = warp * T::rows_per_warp;
                s0 = max(sh_off[r * TX], base);
                n0 = max(min(sh_off[r * TX + TX], end) - s0, 0);
                if (n0 > 0) g0 = sh_gs[r] - sh_off[r * TX];
                if (T::rows_per_warp == 2) {
                    s1 = max(sh_off[(r + 1) * TX], base);
                    n1 = max(min(sh_off[(r + 1) * TX + TX], end) - s1, 0);
                    if (n1 > 0) g1 = sh_gs[r + 1] - sh_off[(r + 1) * TX];
                }
            }
            for (int v0 = 0; v0 < n0 + n1; v0 += 32 * kP2GPer) {
                uint32_t sl[kP2GPer];
                int q[kP2GPer];
#pragma unroll
                for (int u = 0; u < kP2GPer; u++) {
                    const int v = v0 + lane + 32 * u;
                    q[u] = -1;
                    sl[u] = 0u;
                    if (v < n0) {
                        q[u] = s0 + v - base;
                        sl[u] = slots[g0 + s0 + v];
                    } else if (v < n0 + n1) {
                        q[u] = s1 + (v - n0) - base;
                        sl[u] = slots[g1 + s1 + (v - n0)];
                    }
                }
#pragma unroll
                for (int u = 0; u < kP2GPer; u++) {
                    if (q[u] < 0) continue;
                    sh_slot[pad4b(q[u])] = sl[u];
                    mpmg_cp_async16(&sh_a[pad16b(q[u])], P.A + sl[u]);
                    mpmg_cp_async16(&sh_b[pad16b(q[u])], P.B + sl[u]);
                    mpmg_cp_async4(&sh_syy[pad4b(q[u])], &P.C[sl[u]].x);
                }
            }
            mpmg_cp_async_wait_all();
            __syncthreads();
            if (mine) {
                const int j0 = sh_off[me] - base, j1 = j0 + cnt;
                for (int j = j0; j < j1; j++) {
                    const uint32_t x = sh_slot[pad4b(j)];
                    int t = j - 1;
                    while (t >= j0 && sh_slot[pad4b(sh_ord[pad2b(t)])] > x) {
                        sh_ord[pad2b(t + 1)] = sh_ord[pad2b(t)];
                        t--;
                    }
                    sh_ord[pad2b(t + 1)] = (uint16_t)j;
                }
                for (int j = j0; j < j1; j++) {
                    const int q = sh_ord[pad2b(j)];
                    const uint32_t i = sh_slot[pad4b(q)];
                    if (owner) {
                        perm[k0 + (j - j0)] = i;
                        rank[i] = (uint32_t)(k0 + (j - j0));
                    }
                    p2g_accumulate(acc, ih, grav, sh_a[pad16b(q)], sh_b[pad16b(q)], sh_syy[pad4b(q)]);
                }
            }
            __syncthreads();
        } else if (mine) {
            // a single element larger than the stage
            uint32_t *order = perm;
            if (!owner) order = halo_perm + (size_t)(lx == 0 ? (ly == 0 ? 2 : 0) : 1) * (size_t)np;
            mpmg_order_segment(slots, order, owner ? rank : nullptr, k0, k1);
            for (int k = k0; k < k1; k++) {
                const uint32_t i = order[k];
                p2g_accumulate(acc, ih, grav, P.A[i], P.B[i], P.C[i].x);
            }
        }
        ea = eb;
    }
    // the stage is free: the corner sums take its place
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int f = 0; f < 5; f++) sh_sum[(a * 5 + f) * SS + me] = acc[a][f];
    __syncthreads();
    if (me < (TX - 1) * (TY - 1)) {
        const int i = tx * (TX - 1) + me % (TX - 1), j = ty * (TY - 1) + me / (TX - 1);
        if (i < M.g.Nx && j < M.g.Ny) {
            // the node's elements lie in the tile (local column and row
            // nx or nx + 1, ny or ny + 1); one outside the grid has no
            // particles, so the count test alone skips it
            const int nx = me % (TX - 1), ny = me / (TX - 1);
            int off[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int dx = ((i & 1) == (c & 1)) ? 1 : 0;
                const int dy = ((j & 1) == (c >> 1)) ? 1 : 0;
                const int le = (ny + dy) * TX + nx + dx;
                const int a = dx ? (dy ? 0 : 3) : (dy ? 1 : 2);
                off[c] = sh_off[le + 1] != sh_off[le] ? (a * 5) * SS + le : -1;
            }
            node_finish<F64NODE>(M, sp->t + M.dt, tol, i, j, j * M.g.Nx + i, sh_sum, off, SS, node_mass, node4,
                                 node_mx, node_my, node_fx, node_fy, node_m64);
        }
    }
    mpmg_pdl_trigger();
}

// G2P of one particle read from the stored position i (element e of member
// M, local to it), written to position dst of the other buffer: velocity and displacement from the
// nodal accelerations and velocities (process_usl.c:568-611), strain rate
// and vorticity (process_usl.c:613-640), volume (process_usl.c:642-650), the
// material's stress update, and the new element (process_usl.c:660-666).
// Returns the new global element key (sentinel outside the grid).
template <int MATERIAL>
__device__ __forceinline__ uint32_t g2p_particle(const MemberM &M, uint32_t sentinel,
                                                 const float4 *__restrict__ node4, int e, float4 a4, float4 b4,
                                                 float4 c4, float4 d4, uint32_t dst, Buf D,
                                                 int *__restrict__ cell_dst, int src, NLOut nl)
{
    const GeomM &g = M.g;
    const MatF &mp = M.mat;
    const int cj = (int)mpmg_div((uint32_t)e, g.div_Ex), ci = e - cj * g.Ex;
    const int n0 = M.nd0 + cj * g.Nx + ci;
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
    } else if (MATERIAL == MPMG_G_LOCAL_MU2) {
        g_local_mu2_f(mp, m, vol, exx, exy, eyy, wxy, sxx, sxy, syy, Tzz, gp, gdp);
    } else if (MATERIAL == MPMG_DP_RI_MT) {
        dp_ri_mt_f(mp, m, vol, exx, exy, eyy, wxy, sxx, sxy, syy, Tzz, gp, gdp);
    } else {
        // g_nonlocal_mu2: bulk fluidity now; the stress waits for the solve
        float p_tr, t0xx, t0xy, t0yy, tau_tr, dense, gfl, xisq;
        nonlocal_mu2_trial_f(mp, exx, exy, eyy, wxy, sxx, sxy, syy, p_tr, t0xx, t0xy, t0yy, tau_tr);
        nonlocal_mu2_bulk_f(mp, m, vol, p_tr, tau_tr, dense, gfl, xisq);
        const bool d = dense != 0.0f;
        nl.T[src] = make_float4(d ? p_tr : 0.0f, t0xx, t0xy, t0yy);
        nl.F[src] = make_float4(tau_tr, gfl, xisq, d ? vol : 0.0f);
    }

    // New element from the local coordinates (WHICH_ELEMENT4, process_usl.c:43-44).
    float nxl = xl + dux * ih, nyl = yl + duy * ih;
    const float fxl = floorf(nxl), fyl = floorf(nyl);
    const int nci = ci + (int)fxl, ncj = cj + (int)fyl;
    nxl -= fxl;
    nyl -= fyl;
    const float xg = ((float)nci + nxl) * g.hf, yg = ((float)ncj + nyl) * g.hf;
    const bool inside = nci >= 0 && ncj >= 0 && nci < g.Ex && ncj < g.Ey && xg < g.xmaxf && yg < g.ymaxf &&
                        xg >= 0.0f && yg >= 0.0f;
    uint32_t new_key = sentinel;
    if (inside) {
        new_key = (uint32_t)(M.e0 + ncj * g.Ex + nci);
    } else {
        nxl = xg;      // global position of a particle that left the grid
        nyl = yg;
    }
    D.A[dst] = make_float4(nxl, nyl, vx, vy);
    D.B[dst] = make_float4(m, vol, sxx, sxy);
    D.C[dst] = make_float4(syy, c4.y + dux, c4.z + duy, Tzz);
    D.D[dst] = make_float4(gp, gdp, d4.z, d4.w);
    cell_dst[dst] = (int)new_key;
    return new_key;
}

// The G2P streams the stored particles through shared memory with bulk
// asynchronous copies (TMA): a persistent block of 256 threads takes tiles of
// 256 consecutive stored particles (records A-D, element, destination rank:
// 18 KB) round-robin, keeps kG2PStages tiles in flight on one mbarrier each,
// and one thread per particle computes from the staged copy.  The writes go
// to the sorted position rank[i] of the other buffer (the storage stays in
// element order from step to step).  The last, partial tile is read directly.
// Every wait is bounded: on a timeout the kernel sets MPMG_DEV_ERR_SPIN,
// waits (bounded) for its own copies still in flight, and returns.
// The tile (256 by default, or 128: mpmg_autotune's choice) is a template.
constexpr int kG2PStages = 3;
constexpr long long kG2PWaitLimit = 1ll << 22;

template <int TILE>
struct G2PStage {
    float4 A[TILE], B[TILE], C[TILE], D[TILE];
    int src[TILE];
    uint32_t rank[TILE];
};
template <int TILE>
constexpr size_t g2p_smem_bytes()
{
    return sizeof(G2PStage<TILE>) * kG2PStages;
}
static_assert(sizeof(G2PStage<128>) % 16 == 0 && sizeof(G2PStage<256>) % 16 == 0,
              "stage arrays must stay 16-byte aligned");
constexpr int kG2PTiles = 2;
constexpr int kG2PTileSizes[kG2PTiles] = {256, 128};

template <int MATERIAL, bool BATCH, int kG2PTile>
__global__ void __launch_bounds__(kG2PTile, 768 / kG2PTile) mx_g2p_kernel(
    const __grid_constant__ MemberM m0, BatchView bv, int ne_total, int n, const uint32_t *__restrict__ rank,
    Buf S, Buf D, const int *__restrict__ cell_src, int *__restrict__ cell_dst, const float4 *__restrict__ node4,
    uint32_t *__restrict__ bins, StepParams *sp, int *status, NLOut nl)
{
    using G2PStage = ::G2PStage<kG2PTile>;
    constexpr uint32_t kG2PStageBytes = (uint32_t)sizeof(G2PStage);
    extern __shared__ __align__(128) unsigned char g2p_smem[];
    G2PStage *stage = reinterpret_cast<G2PStage *>(g2p_smem);
    __shared__ __align__(8) uint64_t full[kG2PStages];
    __shared__ int abort_s;
    const int tid = threadIdx.x;
    const int num_tiles = (n + kG2PTile - 1) / kG2PTile;
    uint32_t inflight = 0;      // thread 0: stages with a copy outstanding
    if (tid == 0) {
        for (int k = 0; k < kG2PStages; k++) mpmg_mbar_init(&full[k], 1);
        mpmg_mbar_init_fence();
        abort_s = 0;
    }
    __syncthreads();
    auto issue = [&](int tile, int k) {
        const size_t base = (size_t)tile * kG2PTile;
        mpmg_mbar_expect_tx(&full[k], kG2PStageBytes);
        mpmg_bulk_g2s(stage[k].A, S.A + base, kG2PTile * 16, &full[k]);
        mpmg_bulk_g2s(stage[k].B, S.B + base, kG2PTile * 16, &full[k]);
        mpmg_bulk_g2s(stage[k].C, S.C + base, kG2PTile * 16, &full[k]);
        mpmg_bulk_g2s(stage[k].D, S.D + base, kG2PTile * 16, &full[k]);
        mpmg_bulk_g2s(stage[k].src, cell_src + base, kG2PTile * 4, &full[k]);
        mpmg_bulk_g2s(stage[k].rank, rank + base, kG2PTile * 4, &full[k]);
        inflight |= 1u << k;
    };
    if (tid == 0) {
        for (int k = 0; k < kG2PStages; k++) {
            const int tile = blockIdx.x + k * gridDim.x;
            if (tile < num_tiles && (tile + 1) * kG2PTile <= n) issue(tile, k);
        }
    }
    // The stored records and elements come from the previous step's G2P and
    // the ranks from this step's P2G, two kernels back: the first copies are
    // in flight before the wait.  The nodal values come from the grid
    // update just before.
    mpmg_pdl_wait();
    if (blockIdx.x == 0) {
        // Advance t and compute the next step's body force (the driver's
        // time_varying_loads, loading.c:34-54), one thread per member.  No
        // kernel of this step reads them after this point.
        for (int k = tid; k < (BATCH ? bv.count : 1); k += kG2PTile) {
            const MemberM &M = BATCH ? bv.m[k] : m0;
            StepParams *p = sp + k;
            const double t = p->t + M.dt;
            p->t = t;
            p->step_count += 1;
            double grav;
            if (M.gravity_mode == MPMG_GRAVITY_CONSTANT) grav = M.gravity_const;
            else if ((0.1 + p->step_start_time) > t) grav = -9.8 * ((t - p->step_start_time) / 0.1);
            else grav = -9.8;
            p->gravity = grav;
        }
    }
    uint32_t parity = 0;        // per stage: phase to wait for
    int k = 0;
    for (int tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
        const int base = tile * kG2PTile;
        const int i = base + tid;
        const bool full_tile = base + kG2PTile <= n;
        bool have = i < n;
        float4 a4, b4, c4, d4;
        int e = 0;
        uint32_t dst = 0;
        if (full_tile) {
            if (mpmg_mbar_wait(&full[k], (parity >> k) & 1u, kG2PWaitLimit)) {
                a4 = stage[k].A[tid];
                b4 = stage[k].B[tid];
                c4 = stage[k].C[tid];
                d4 = stage[k].D[tid];
                e = stage[k].src[tid];
                dst = stage[k].rank[tid];
                if (tid == 0) inflight &= ~(1u << k);
                parity ^= 1u << k;
            } else {
                atomicOr(status, MPMG_DEV_ERR_SPIN);
                abort_s = 1;
                have = false;
            }
        } else if (have) {
            a4 = S.A[i];
            b4 = S.B[i];
            c4 = S.C[i];
            d4 = S.D[i];
            e = cell_src[i];
            dst = rank[i];
        }
        const uint32_t sentinel = (uint32_t)ne_total;
        uint32_t new_key = sentinel;
        if (have) {
            if (e >= ne_total) {
                // outside the grid: carried along unchanged
                D.A[dst] = a4;
                D.B[dst] = b4;
                D.C[dst] = c4;
                D.D[dst] = d4;
                cell_dst[dst] = ne_total;
            } else {
                const int mk = BATCH ? find_member(bv.elem_off, bv.count, e) : 0;
                const MemberM &M = BATCH ? bv.m[mk] : m0;
                new_key = g2p_particle<MATERIAL>(M, sentinel, node4, e - M.e0, a4, b4, c4, d4, dst, D, cell_dst,
                                                 i, nl);
            }
        }
        // the next step's bins, by destination position (the binning's first phase)
        mpmg_bin_count(new_key, have, sentinel, dst >> 5, bins);
        __syncthreads();        // every thread is done with stage k
        if (abort_s) {
            if (tid == 0)
                for (int q = 0; q < kG2PStages; q++)
                    if (inflight & (1u << q)) mpmg_mbar_wait(&full[q], (parity >> q) & 1u, kG2PWaitLimit);
            return;
        }
        if (tid == 0 && full_tile) {
            const int next = tile + kG2PStages * gridDim.x;
            if (next < num_tiles && (next + 1) * kG2PTile <= n) {
                mpmg_fence_proxy_async();
                issue(next, k);
            }
        }
        k = (k + 1 == kG2PStages) ? 0 : k + 1;
    }
    mpmg_pdl_trigger();
}

// g_nonlocal_mu2 element blocks and right-hand sides (g_nonlocal_mu2.c:418-507)
// from the stored particles of this step's binned order: start-of-step shape
// functions (the local coordinates still in S.A), updated volume, dense flag,
// local fluidity and cooperativity from the G2P.  FP32 sums of an element's
// few particles, stored in FP64 for the solver.
__device__ __forceinline__ int sym_index_m(int a, int b)
{
    if (a > b) {
        const int t = a;
        a = b;
        b = t;
    }
    const int row_start[4] = {0, 4, 7, 9};
    return row_start[a] + (b - a);
}

__global__ void __launch_bounds__(128) mx_assemble_kernel(int ne, float inv_h, const int *__restrict__ cell_start,
                                                          const uint32_t *__restrict__ perm,
                                                          const float4 *__restrict__ SA, NLOut nl,
                                                          double *__restrict__ elem_k, double *__restrict__ elem_f)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int k0 = cell_start[e], k1 = cell_start[e + 1];
    if (k0 == k1) return;
    float K[10], F[4];
#pragma unroll
    for (int k = 0; k < 10; k++) K[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = 0.0f;
    for (int k = k0; k < k1; k++) {
        const uint32_t i = perm[k];
        const float4 f4 = nl.F[i];
        if (f4.w == 0.0f) continue;      // not dense
        const float4 a4 = SA[i];
        const float a = a4.x, b = a4.y, ox = 1.0f - a, oy = 1.0f - b;
        const float sf[4] = {ox * oy, a * oy, a * b, ox * b};
        const float gx[4] = {-oy * inv_h, oy * inv_h, b * inv_h, -b * inv_h};
        const float gy[4] = {-ox * inv_h, -a * inv_h, a * inv_h, ox * inv_h};
        const float vol = f4.w, xi = f4.z, fv = vol * f4.y * xi;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            F[r] += fv * sf[r];
#pragma unroll
            for (int c = r; c < 4; c++) K[sym_index_m(r, c)] += vol * (xi * sf[r] * sf[c] + (gx[r] * gx[c] + gy[r] * gy[c]));
        }
    }
#pragma unroll
    for (int k = 0; k < 10; k++) elem_k[(size_t)k * ne + e] = (double)K[k];
#pragma unroll
    for (int k = 0; k < 4; k++) elem_f[(size_t)k * ne + e] = (double)F[k];
}

// After the solve: the nodal fluidity at each particle's start-of-step
// position (g_nonlocal_mu2.c:545-564) and the stress update (:160-218),
// written over the record the G2P put at the particle's new position.
__global__ void __launch_bounds__(256) mx_fluidity_stress_kernel(GeomM g, MatF mp, int n, Buf S, Buf D,
                                                                 const uint32_t *__restrict__ rank,
                                                                 const int *__restrict__ cell_src,
                                                                 const double *__restrict__ node_gf, NLOut nl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = cell_src[i];
    if (e >= g.ne) return;
    const uint32_t dst = rank[i];
    const int cj = (int)mpmg_div((uint32_t)e, g.div_Ex), ci = e - cj * g.Ex;
    const int n0 = cj * g.Nx + ci;
    const float4 a4 = S.A[i];
    const float gp0 = S.D[i].x;
    const float a = a4.x, b = a4.y, ox = 1.0f - a, oy = 1.0f - b;
    const float gf = (float)node_gf[n0] * (ox * oy) + (float)node_gf[n0 + 1] * (a * oy) +
                     (float)node_gf[n0 + 1 + g.Nx] * (a * b) + (float)node_gf[n0 + g.Nx] * (ox * b);
    const float4 t4 = nl.T[i];
    const float tau_tr = nl.F[i].x;
    float sxx, sxy, syy, gp = gp0, gdp;
    nonlocal_mu2_stress_f(mp, gf, t4.x, t4.y, t4.z, t4.w, tau_tr, sxx, sxy, syy, gp, gdp);
    float *Bd = reinterpret_cast<float *>(D.B + dst);
    float *Cd = reinterpret_cast<float *>(D.C + dst);
    float *Dd = reinterpret_cast<float *>(D.D + dst);
    Bd[2] = sxx;
    Bd[3] = sxy;
    Cd[0] = syy;
    Dd[0] = gp;
    Dd[1] = gdp;
    Dd[3] = gf;
}

inline int blocks_for(size_t n, int threads)
{
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    return (int)(b > 0 ? b : 1);
}

GeomM make_geom(const mpmg_config &c)
{
    GeomM g;
    g.Nx = c.Nx;
    g.Ny = c.Ny;
    g.Ex = c.Nx - 1;
    g.Ey = c.Ny - 1;
    g.ne = g.Ex * g.Ey;
    g.div_Ex = mpmg_div_init((uint32_t)(g.Ex > 0 ? g.Ex : 1));
    g.div_Nx = mpmg_div_init((uint32_t)(c.Nx > 0 ? c.Nx : 1));
    g.h = c.h;
    g.hf = (float)c.h;
    g.inv_hf = (float)(1.0 / c.h);
    g.xmaxf = (float)c.xmax;
    g.ymaxf = (float)c.ymax;
    return g;
}

BcM make_bc(const mpmg_config &c)
{
    BcM b = {};
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

// material_init (isolin.c:31-59, g_local_mu2.c:126-160) in FP32 form.
MatF make_mat(const mpmg_config &c)
{
    MatF p;
    const double E = c.mp[MPMG_MP_E], nu = c.mp[MPMG_MP_NU];
    const double G = E / (2.0 * (1.0 + nu));
    const double K = E / (3.0 * (1.0 - 2 * nu));
    p.G = (float)G;
    p.K = (float)K;
    p.lambda = (float)(K - 2.0 * G / 3.0);
    p.dt = (float)c.dt;
    p.mu_s = (float)c.mp[MPMG_MP_MU_S];
    p.mu_2 = (float)c.mp[MPMG_MP_MU_2];
    p.I0 = (float)c.mp[MPMG_MP_I0];
    p.grains_rho = (float)c.mp[MPMG_MP_GRAINS_RHO];
    p.grains_d = (float)c.mp[MPMG_MP_GRAINS_D];
    p.rho_critical = (float)c.mp[MPMG_MP_RHO_CRITICAL];
    const double rho = c.mp[MPMG_MP_GRAINS_RHO], d = c.mp[MPMG_MP_GRAINS_D];
    p.inv_grains_rho = rho != 0.0 ? (float)(1.0 / rho) : 0.0f;
    p.alpha_coef = d != 0.0 ? (float)(G * c.mp[MPMG_MP_I0] * c.dt / d) : 0.0f;
    p.inv_G_dt = (G * c.dt) != 0.0 ? (float)(1.0 / (G * c.dt)) : 0.0f;
    const double A = c.mp[MPMG_MP_A];
    p.inv_A2d2 = (A * A * d * d) != 0.0 ? (float)(1.0 / (A * A * d * d)) : 0.0f;
    return p;
}

MemberM make_member(const mpmg_config &c, size_t e0, size_t nd0)
{
    MemberM M;
    M.g = make_geom(c);
    M.bc = make_bc(c);
    M.mat = make_mat(c);
    M.dt = c.dt;
    M.dt_hi = (float)c.dt;
    M.dt_lo = (float)(c.dt - (double)M.dt_hi);
    M.gravity_mode = c.gravity_mode;
    M.gravity_const = c.gravity;
    M.e0 = (int)e0;
    M.nd0 = (int)nd0;
    return M;
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

// Geometry of one simulation for placing its particles.
struct PlaceGeom {
    double h, xmax, ymax;
    int Ex, Ey, e0;
};

// The initial records of particle i from the caller's FP64 arrays (staged on
// the device, array k at in[k]): the element and local coordinates of
// WHICH_ELEMENT4 (process_usl.c:43-44; the particle.c:14-30 coordinates,
// held below 1 in FP32), -1 outside the grid, where xl, yl keep the
// position.  The FP64 operations are the _rn intrinsics, so the keys are
// the same whatever the host compiler would have fused.
__global__ void __launch_bounds__(256) mx_place_kernel(int n, const double *const *in, PlaceGeom single,
                                                       const PlaceGeom *__restrict__ members,
                                                       const int *__restrict__ poff, int count, int ne_total,
                                                       Buf P, int *__restrict__ cell)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PlaceGeom g = members ? members[find_member(poff, count, i)] : single;
    const double m = in[0][i], v = in[1][i], x = in[2][i], y = in[3][i], vx = in[4][i], vy = in[5][i];
    const double sxx = in[6][i], sxy = in[7][i], syy = in[8][i];
    int local = -1;
    float xl = (float)x, yl = (float)y;
    if (x < g.xmax && x >= 0.0 && y < g.ymax && y >= 0.0) {
        const double fx = floor(__ddiv_rn(x, g.h)), fy = floor(__ddiv_rn(y, g.h));
        if (fx < (double)g.Ex && fy < (double)g.Ey) {
            local = (int)__dadd_rn(fx, __dmul_rn(fy, (double)g.Ex));
            const double lx = __ddiv_rn(__dsub_rn(x, __dmul_rn(fx, g.h)), g.h);
            const double ly = __ddiv_rn(__dsub_rn(y, __dmul_rn(fy, g.h)), g.h);
            xl = __double2float_rn(lx);
            yl = __double2float_rn(ly);
            if (xl >= 1.0f) xl = __int_as_float(0x3f7fffff);   // the float just below 1
            if (yl >= 1.0f) yl = __int_as_float(0x3f7fffff);
        }
    }
    cell[i] = local < 0 ? ne_total : g.e0 + local;
    P.A[i] = make_float4(xl, yl, (float)vx, (float)vy);
    P.B[i] = make_float4((float)m, (float)v, (float)sxx, (float)sxy);
    P.C[i] = make_float4((float)syy, 0.0f, 0.0f, 0.0f);
    P.D[i] = make_float4(0.0f, 0.0f, __int_as_float(i), 0.0f);
}

using G2PKernel = void (*)(MemberM, BatchView, int, int, const uint32_t *, Buf, Buf, const int *, int *,
                          const float4 *, uint32_t *, StepParams *, int *, NLOut);

template <int TILE>
G2PKernel g2p_variant_t(int material, bool batch)
{
    if (material == MPMG_ISOLIN)
        return batch ? mx_g2p_kernel<MPMG_ISOLIN, true, TILE> : mx_g2p_kernel<MPMG_ISOLIN, false, TILE>;
    if (material == MPMG_G_NONLOCAL_MU2) return mx_g2p_kernel<MPMG_G_NONLOCAL_MU2, false, TILE>;
    if (material == MPMG_DP_RI_MT)
        return batch ? mx_g2p_kernel<MPMG_DP_RI_MT, true, TILE> : mx_g2p_kernel<MPMG_DP_RI_MT, false, TILE>;
    return batch ? mx_g2p_kernel<MPMG_G_LOCAL_MU2, true, TILE> : mx_g2p_kernel<MPMG_G_LOCAL_MU2, false, TILE>;
}

// The G2P kernel of a material and tile (one of kG2PTileSizes).
G2PKernel g2p_variant(int material, bool batch, int tile)
{
    return tile == 128 ? g2p_variant_t<128>(material, batch) : g2p_variant_t<256>(material, batch);
}

size_t g2p_smem_size(int tile)
{
    return tile == 128 ? g2p_smem_bytes<128>() : g2p_smem_bytes<256>();
}

using P2GKernel = void (*)(MemberM, BatchView, int, const int *, const uint32_t *, uint32_t *, uint32_t *, Buf,
                          const StepParams *, float *);

// The batched P2G of variant v (kP2GElems[v] elements a block).
P2GKernel p2g_variant(int v)
{
    if (v == 1) return mx_p2g_kernel<kP2GElems[1], kP2GStage[1], true>;
    if (v == 2) return mx_p2g_kernel<kP2GElems[2], kP2GStage[2], true>;
    return mx_p2g_kernel<kP2GElems[0], kP2GStage[0], true>;
}

}  // namespace

int mpmg_mixed_init(mpmg_ctx *ctx, const double *m, const double *v, const double *x, const double *y,
                    const double *vx, const double *vy, const double *sxx, const double *sxy, const double *syy)
{
    const int mat = ctx->cfg.material;
    if (mat != MPMG_ISOLIN && mat != MPMG_G_LOCAL_MU2 && mat != MPMG_DP_RI_MT &&
        !(mat == MPMG_G_NONLOCAL_MU2 && ctx->batch == nullptr)) {
        mpmg_set_error("mixed precision supports isolin, g_local_mu2, dp_ri_mt and (outside batches) g_nonlocal_mu2");
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
    if (ctx->batch != nullptr) {
        if ((rc = dalloc(&s->cell_sums, 20 * ctx->ne)) != MPMG_OK) return rc;
    } else if ((rc = dalloc(&s->halo_perm, 3 * n)) != MPMG_OK) {
        return rc;
    }
    if ((rc = dalloc(&s->node4, ctx->nn)) != MPMG_OK) return rc;
    if ((rc = dalloc(&s->node_mass, ctx->nn)) != MPMG_OK) return rc;
    if ((rc = dalloc(&s->export_buf, n)) != MPMG_OK) return rc;
    if (mat == MPMG_G_NONLOCAL_MU2) {
        // the fluidity solve: FP64 nodal mass (unknown mask), nodal fluidity,
        // element blocks and Krylov vectors, and the per-particle G2P values
        if ((rc = dalloc(&s->nl_T, n)) != MPMG_OK) return rc;
        if ((rc = dalloc(&s->nl_F, n)) != MPMG_OK) return rc;
        if ((rc = dalloc(&ctx->node_m, ctx->nn)) != MPMG_OK) return rc;
        if ((rc = dalloc(&ctx->node_gf, ctx->nn)) != MPMG_OK) return rc;
        MPMG_CHECK(cudaMemset(ctx->node_gf, 0, ctx->nn * sizeof(double)));
        if ((rc = mpmg_nonlocal_init(ctx)) != MPMG_OK) return rc;
    }
    MPMG_CHECK(cudaMemset(s->node_mass, 0, ctx->nn * sizeof(float2)));

    // members: one, or the batch's (their constants and first-index tables)
    BatchInfo *bt = ctx->batch;
    const int count = bt ? bt->count : 1;
    if (bt) {
        std::vector<MemberM> hm(count);
        std::vector<int> eo(count + 1), no(count + 1);
        for (int k = 0; k < count; k++) hm[k] = make_member(bt->cfg[k], bt->eoff[k], bt->noff[k]);
        for (int k = 0; k <= count; k++) {
            eo[k] = (int)bt->eoff[k];
            no[k] = (int)bt->noff[k];
        }
        MemberM *dm = nullptr;
        if ((rc = dalloc(&dm, count)) != MPMG_OK) return rc;
        bt->d_members = dm;
        if ((rc = dalloc(&bt->d_elem_off, count + 1)) != MPMG_OK) return rc;
        if ((rc = dalloc(&bt->d_node_off, count + 1)) != MPMG_OK) return rc;
        MPMG_CHECK(cudaMemcpy(dm, hm.data(), count * sizeof(MemberM), cudaMemcpyHostToDevice));
        MPMG_CHECK(cudaMemcpy(bt->d_elem_off, eo.data(), (count + 1) * sizeof(int), cudaMemcpyHostToDevice));
        MPMG_CHECK(cudaMemcpy(bt->d_node_off, no.data(), (count + 1) * sizeof(int), cudaMemcpyHostToDevice));
    }

    // The caller's FP64 arrays go to the device as they are, into buffer 1's
    // records and the export buffer (64 + 8 bytes a particle: the nine
    // arrays), and a kernel places the particles and builds buffer 0's
    // records and elements.
    if (n > 0) {
        double *stage[9];
        float4 *const spare[4] = {s->A[1], s->B[1], s->C[1], s->D[1]};
        for (int k = 0; k < 8; k++) stage[k] = reinterpret_cast<double *>(spare[k / 2]) + (k % 2) * n;
        stage[8] = s->export_buf;
        const double *src[9] = {m, v, x, y, vx, vy, sxx, sxy, syy};
        for (int k = 0; k < 9; k++)
            MPMG_CHECK(cudaMemcpyAsync(stage[k], src[k], n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        // scratch freed on every way out
        struct Scratch {
            double **stage = nullptr;
            PlaceGeom *geo = nullptr;
            int *poff = nullptr;
            ~Scratch()
            {
                cudaFree(stage);
                cudaFree(geo);
                cudaFree(poff);
            }
        } sc;
        if ((rc = dalloc(&sc.stage, 9)) != MPMG_OK) return rc;
        MPMG_CHECK(cudaMemcpyAsync(sc.stage, stage, sizeof(stage), cudaMemcpyHostToDevice, ctx->stream));
        const mpmg_config &c0 = bt ? bt->cfg[0] : ctx->cfg;
        const PlaceGeom single{c0.h, c0.xmax, c0.ymax, c0.Nx - 1, c0.Ny - 1, 0};
        std::vector<PlaceGeom> hg;
        std::vector<int> hp;
        if (bt) {
            hg.resize(count);
            hp.resize(count + 1);
            for (int k = 0; k < count; k++) {
                const mpmg_config &ck = bt->cfg[k];
                hg[k] = PlaceGeom{ck.h, ck.xmax, ck.ymax, ck.Nx - 1, ck.Ny - 1, (int)bt->eoff[k]};
            }
            for (int k = 0; k <= count; k++) hp[k] = (int)bt->poff[k];
            if ((rc = dalloc(&sc.geo, count)) != MPMG_OK) return rc;
            if ((rc = dalloc(&sc.poff, count + 1)) != MPMG_OK) return rc;
            MPMG_CHECK(cudaMemcpyAsync(sc.geo, hg.data(), count * sizeof(PlaceGeom), cudaMemcpyHostToDevice,
                                       ctx->stream));
            MPMG_CHECK(cudaMemcpyAsync(sc.poff, hp.data(), (count + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                       ctx->stream));
        }
        mx_place_kernel<<<blocks_for(n, 256), 256, 0, ctx->stream>>>((int)n, sc.stage, single, sc.geo, sc.poff, count,
                                                                    (int)ctx->ne, buf(s, 0), ctx->in_element);
        ctx->launches += 1;
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return mpmg_cuda_status(e, "mixed state upload");
    }
    s->cur = 0;
    // persistent G2P grid: as many blocks as fit on the device at once, at
    // most one per tile
    int sms = 0;
    MPMG_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->dev));
    for (int t = 0; t < kG2PTiles; t++) {
        const int tile = kG2PTileSizes[t];
        MPMG_CHECK(cudaFuncSetAttribute(g2p_variant(ctx->cfg.material, bt != nullptr, tile),
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g2p_smem_size(tile)));
    }
    MPMG_CHECK(cudaFuncSetAttribute(mx_p2g_grid_kernel<false, kFusedTX, kFusedTY>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FusedT::smem));
    MPMG_CHECK(cudaFuncSetAttribute(mx_p2g_grid_kernel<true, kFusedTX, kFusedTY>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FusedT::smem));
    s->sms = sms > 0 ? sms : 1;
    s->p2g_variant = 0;
    rc = mpmg_mixed_set_tiles(ctx, 0, kG2PTileSizes[0]);
    if (rc != MPMG_OK) return rc;
    // the first step's element counts; every G2P counts the next step's
    return mpmg_bin_count(ctx, (const uint32_t *)ctx->in_element);
}

// Persistent G2P grid of per_sm blocks per SM (clamped to what fits), at
// most one block per tile.  Which block takes which tile does not change any
// particle's result.
int mpmg_mixed_set_g2p_per_sm(mpmg_ctx *ctx, int per_sm)
{
    MixedState *s = ctx->mixed;
    if (per_sm < 1) per_sm = 1;
    if (per_sm > s->g2p_per_sm_max) per_sm = s->g2p_per_sm_max;
    const size_t tiles = (ctx->np + s->g2p_tile - 1) / s->g2p_tile;
    size_t blocks = (size_t)s->sms * (size_t)per_sm;
    if (blocks > tiles) blocks = tiles;
    s->g2p_blocks = (int)(blocks > 0 ? blocks : 1);
    return per_sm;
}

// The tiles of the mixed step: the batched P2G's variant (elements a block
// and staged particles, kP2GElems / kP2GStage; single simulations run the
// fused kernel and ignore it) and the G2P tile (kG2PTileSizes).  The G2P
// grid goes back to all the blocks of the new tile that fit.  Tiles change
// which block handles which elements or particles, never a result.
int mpmg_mixed_set_tiles(mpmg_ctx *ctx, int p2g_variant, int g2p_tile)
{
    MixedState *s = ctx->mixed;
    if (s == nullptr || p2g_variant < 0 || p2g_variant >= kP2GVariants || (g2p_tile != 256 && g2p_tile != 128))
        return MPMG_ERR_INVALID;
    int per_sm = 0;
    MPMG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, g2p_variant(ctx->cfg.material, ctx->batch != nullptr, g2p_tile), g2p_tile, g2p_smem_size(g2p_tile)));
    s->p2g_variant = p2g_variant;
    s->g2p_tile = g2p_tile;
    s->g2p_per_sm_max = per_sm > 0 ? per_sm : 1;
    mpmg_mixed_set_g2p_per_sm(ctx, s->g2p_per_sm_max);
    return MPMG_OK;
}

int mpmg_mixed_p2g_variants()
{
    return kP2GVariants;
}

void mpmg_mixed_p2g_shape(int v, int *elements, int *stage)
{
    *elements = kP2GElems[v];
    *stage = kP2GStage[v];
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
    cudaFree(s->halo_perm);
    cudaFree(s->node4);
    cudaFree(s->node_mass);
    cudaFree(s->export_buf);
    cudaFree(s->nl_T);
    cudaFree(s->nl_F);
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

// The batch view of a context (a single simulation: one member, no tables).
static BatchView batch_view(const mpmg_ctx *ctx)
{
    BatchView bv = {nullptr, nullptr, nullptr, 1};
    if (ctx->batch) {
        bv.m = (const MemberM *)ctx->batch->d_members;
        bv.elem_off = ctx->batch->d_elem_off;
        bv.node_off = ctx->batch->d_node_off;
        bv.count = ctx->batch->count;
    }
    return bv;
}

int mpmg_mixed_step(mpmg_ctx *ctx)
{
    MixedState *s = ctx->mixed;
    cudaStream_t st = ctx->stream;
    const mpmg_config &c = ctx->cfg;
    const bool batch = ctx->batch != nullptr;
    const MemberM m0 = make_member(batch ? ctx->batch->cfg[0] : c, 0, 0);
    const BatchView bv = batch_view(ctx);
    const int n = (int)ctx->np, ne = (int)ctx->ne, nn = (int)ctx->nn;
    const int cur = s->cur, nxt = 1 - cur;

    mpmg_phase_begin(ctx, PH_SORT);
    int rc = mpmg_bin_scan_scatter(ctx, (const uint32_t *)cell_array(ctx, cur), nullptr, true);
    if (rc != MPMG_OK) return rc;
    mpmg_phase_end(ctx, PH_SORT);

    Buf S = buf(s, cur), D = buf(s, nxt);
    const bool f64 = c.precision == MPMG_PRECISION_MIXED_F64NODE;
    const bool nonlocal = c.material == MPMG_G_NONLOCAL_MU2;
    double *node_m64 = nonlocal ? ctx->node_m : (double *)nullptr;
    if (!batch) {
        // P2G and grid update fused over element tiles
        mpmg_phase_begin(ctx, PH_P2G);
        const int tiles_x = (m0.g.Nx + kFusedTX - 2) / (kFusedTX - 1);
        const int tiles_y = (m0.g.Ny + kFusedTY - 2) / (kFusedTY - 1);
        MPMG_CHECK(mpmg_launch_pdl(true, f64 ? mx_p2g_grid_kernel<true, kFusedTX, kFusedTY>
                                             : mx_p2g_grid_kernel<false, kFusedTX, kFusedTY>,
                                   dim3(tiles_x * tiles_y), dim3(FusedT::threads), FusedT::smem, st, m0, n,
                                   tiles_x, (const int *)ctx->cell_start, (const uint32_t *)ctx->bin.slots,
                                   ctx->perm, ctx->bin.rank, s->halo_perm, S, (const StepParams *)ctx->d_params,
                                   (float)MPMG_TOL, s->node_mass, s->node4, ctx->node_mx, ctx->node_my,
                                   ctx->node_fx, ctx->node_fy, node_m64));
        mpmg_phase_end(ctx, PH_P2G);
    } else {
        mpmg_phase_begin(ctx, PH_P2G);
        const int pe = kP2GElems[s->p2g_variant];
        MPMG_CHECK(mpmg_launch_pdl(true, p2g_variant(s->p2g_variant), dim3(blocks_for(ctx->ne, pe)), dim3(pe), 0,
                                   st, m0, bv, ne, (const int *)ctx->cell_start,
                                   (const uint32_t *)ctx->bin.slots, ctx->perm, ctx->bin.rank, S,
                                   (const StepParams *)ctx->d_params, s->cell_sums));
        mpmg_phase_end(ctx, PH_P2G);

        mpmg_phase_begin(ctx, PH_GRID);
        MPMG_CHECK(mpmg_launch_pdl(true, f64 ? mx_grid_kernel<true, true> : mx_grid_kernel<false, true>,
                                   dim3(blocks_for(ctx->nn, 256)), dim3(256), 0, st, m0, bv, ne, nn,
                                   (const int *)ctx->cell_start, (const float *)s->cell_sums,
                                   (const StepParams *)ctx->d_params, (float)MPMG_TOL, s->node_mass, s->node4,
                                   ctx->node_mx, ctx->node_my, ctx->node_fx, ctx->node_fy, node_m64));
        mpmg_phase_end(ctx, PH_GRID);
    }

    mpmg_phase_begin(ctx, PH_G2P);
    MPMG_CHECK(mpmg_launch_pdl(true, g2p_variant(c.material, batch, s->g2p_tile), dim3(s->g2p_blocks),
                               dim3(s->g2p_tile), g2p_smem_size(s->g2p_tile), st, m0, bv, ne, n, (const uint32_t *)ctx->bin.rank, S, D,
                               (const int *)cell_array(ctx, cur), cell_array(ctx, nxt), (const float4 *)s->node4,
                               ctx->bin.counts, ctx->d_params, ctx->d_status, NLOut{s->nl_T, s->nl_F}));
    mpmg_phase_end(ctx, PH_G2P);
    ctx->launches += batch ? 3 : 2;
    if (nonlocal) {
        // the fluidity solve (FP64 Krylov) and the stress update
        mpmg_phase_begin(ctx, PH_FLUIDITY);
        mx_assemble_kernel<<<blocks_for(ctx->ne, 128), 128, 0, st>>>(
            ne, m0.g.inv_hf, ctx->cell_start, ctx->perm, S.A, NLOut{s->nl_T, s->nl_F}, ctx->elem_k, ctx->elem_f);
        rc = mpmg_launch_solve(ctx);
        if (rc != MPMG_OK) return rc;
        mx_fluidity_stress_kernel<<<blocks_for(n, 256), 256, 0, st>>>(m0.g, m0.mat, n, S, D, ctx->bin.rank,
                                                                      cell_array(ctx, cur), ctx->node_gf,
                                                                      NLOut{s->nl_T, s->nl_F});
        mpmg_phase_end(ctx, PH_FLUIDITY);
        ctx->launches += 2;
    }
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
bool field_slot(int material, const char *name, int *rec, int *comp)
{
    if (material == MPMG_DP_RI_MT && strcmp(name, "state1") == 0) {
        *rec = 2;    // szz (dp_ri_mt.c:27) sits in the Tzz slot
        *comp = 3;
        return true;
    }
    struct { const char *n; int r, c; } f[] = {
        {"vx", 0, 2}, {"vy", 0, 3}, {"m", 1, 0}, {"v", 1, 1}, {"sxx", 1, 2}, {"sxy", 1, 3}, {"Txx", 1, 2},
        {"Txy", 1, 3}, {"Tyx", 1, 3}, {"syy", 2, 0}, {"Tyy", 2, 0}, {"ux", 2, 1}, {"uy", 2, 2}, {"Tzz", 2, 3},
        {"state9", 3, 0}, {"state10", 3, 1}, {"state3", 3, 3}};
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
    const BatchInfo *bt = ctx->batch;
    for (size_t k = 0; k < ctx->np; k++) {
        int e = cell[k] < (int)ctx->ne ? cell[k] : -1;
        if (e >= 0 && bt) {
            // element local to the particle's member
            const size_t ge = (size_t)e;
            int lo = 0, hi = bt->count - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (bt->eoff[mid] <= ge) lo = mid;
                else hi = mid - 1;
            }
            e = (int)(ge - bt->eoff[lo]);
        }
        if (in_element) in_element[pid[k]] = e;
        if (active) active[pid[k]] = e >= 0 ? 1 : 0;
    }
    return MPMG_OK;
}

namespace {

// One particle field of the stored records in the caller's particle order,
// widened to FP64 (the particle index travels in D.z).  Positions are the
// element's corner plus the local coordinate, times h, as the host
// read-back computes them; a particle outside the grid holds its position.
__global__ void mx_export_kernel(int n, const float4 *__restrict__ rec, int comp, const float4 *__restrict__ drec,
                                 const int *__restrict__ cell, int xy, const __grid_constant__ MemberM m0,
                                 BatchView bv, int ne, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int pid = __float_as_int(drec[i].z);
    const float4 r = rec[i];
    const float v = comp == 0 ? r.x : comp == 1 ? r.y : comp == 2 ? r.z : r.w;
    double o = (double)v;
    if (xy != 0) {
        const int c = cell[i];
        if (c < ne) {
            const MemberM &M = bv.count > 1 ? bv.m[find_member(bv.elem_off, bv.count, c)] : m0;
            const int lc = c - M.e0;
            const int cj = (int)mpmg_div((uint32_t)lc, M.g.div_Ex), ci = lc - cj * M.g.Ex;
            o = ((double)(xy == 1 ? ci : cj) + (double)v) * M.g.h;
        }
    }
    out[pid] = o;
}

int frame_get(mpmg_ctx *ctx, const char *name, double *out)
{
    MixedState *s = ctx->mixed;
    const int b = s->cur;
    const size_t n = ctx->np;
    if (strncmp(name, "node_", 5) == 0) {
        if (strcmp(name, "node_m") == 0) {
            std::vector<float2> h(ctx->nn);
            MPMG_CHECK(cudaMemcpy(h.data(), s->node_mass, ctx->nn * sizeof(float2), cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < ctx->nn; k++) out[k] = (double)h[k].x + (double)h[k].y;
            return MPMG_OK;
        }
        int comp = -1;
        if (strcmp(name, "node_ax") == 0) comp = 0;
        else if (strcmp(name, "node_ay") == 0) comp = 1;
        else if (strcmp(name, "node_vx") == 0) comp = 2;
        else if (strcmp(name, "node_vy") == 0) comp = 3;
        if (comp < 0) return MPMG_ERR_UNKNOWN_FIELD;   // FP64 node arrays: the common path
        std::vector<float4> h(ctx->nn);
        MPMG_CHECK(cudaMemcpy(h.data(), s->node4, ctx->nn * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < ctx->nn; k++) out[k] = get_comp(h[k], comp);
        return MPMG_OK;
    }
    int rec = 0, comp = 0, xy = 0;
    if (strcmp(name, "x") == 0) xy = 1;
    else if (strcmp(name, "y") == 0) { xy = 2; comp = 1; }
    else if (!field_slot(ctx->cfg.material, name, &rec, &comp)) return MPMG_ERR_UNKNOWN_FIELD;
    if (n == 0) return MPMG_OK;
    const MemberM m0 = make_member(ctx->batch ? ctx->batch->cfg[0] : ctx->cfg, 0, 0);
    mx_export_kernel<<<blocks_for(n, 256), 256, 0, ctx->stream>>>((int)n, record(s, b, rec), comp, s->D[b],
                                                                   cell_array(ctx, b), xy, m0, batch_view(ctx),
                                                                   (int)ctx->ne, s->export_buf);
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    MPMG_CHECK(cudaMemcpyAsync(out, s->export_buf, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    return MPMG_OK;
}

}  // namespace

int mpmg_mixed_get(mpmg_ctx *ctx, const char *name, double *out)
{
    return frame_get(ctx, name, out);
}

// Several fields; done[k] is set for every field read here (the others are
// not held by the mixed state).
int mpmg_mixed_get_many(mpmg_ctx *ctx, int count, const char *const *names, double *const *out, bool *done)
{
    for (int k = 0; k < count; k++) {
        done[k] = false;
        const int rc = frame_get(ctx, names[k], out[k]);
        if (rc == MPMG_OK) done[k] = true;
        else if (rc != MPMG_ERR_UNKNOWN_FIELD) return rc;
    }
    return MPMG_OK;
}

int mpmg_mixed_set(mpmg_ctx *ctx, const char *name, const double *in)
{
    MixedState *s = ctx->mixed;
    const int b = s->cur;
    const size_t n = ctx->np;
    MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
    int rec, comp;
    if (!field_slot(ctx->cfg.material, name, &rec, &comp)) {
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
