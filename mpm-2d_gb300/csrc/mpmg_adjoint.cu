// Reverse-mode adjoint of the FP64 explicit USL step (no counterpart in the
// reference, which has no derivatives): gradients of a loss on the final
// particle positions with respect to the material parameters, through every
// step of a trajectory.
//
// Forward (mpmg_adj_forward_tape): the ordinary FP64 step, with the particle
// state saved every K steps (checkpoints).  Backward (mpmg_adj_backward):
// segment by segment from the last, the forward steps of the segment are run
// again from its checkpoint with each step's inputs recorded on the device
// (particle state at the step start, elements and activity after the keys
// phase, the binned order, the nodal mass, acceleration and velocity, the
// step's time and gravity), then the segment's steps are reversed one by one:
//
//   adj_g2p    per particle: the material update (isolin or g_local_mu2),
//              volume, strain rate, velocity and position gathers, and the
//              start-of-step shape functions, reversed; writes the particle's
//              share of the adjoint nodal velocity and acceleration, and the
//              parameter adjoint (block partial sums)
//   adj_cells  per element: those shares summed over the element's particles
//              in the binned order (fixed order, no atomics)
//   adj_grid   per node: the four elements' sums in colour order, the
//              boundary masks and the nodal update (v = p/m, a = f/m,
//              p += dt f) reversed -> adjoint nodal momentum, force and mass
//   adj_p2g    per particle: the P2G of mass, momentum and internal force
//              reversed (a gather from the four nodes)
//   theta      the step's block partials added, in block order, to the
//              parameter adjoint
//
// The element of each particle is held fixed within a step (the map from
// positions to elements is piecewise constant), and the branches of the
// material law (elastic / plastic / stress-free) are those the forward step
// took.  Everything is FP64 and deterministic.
#include <math.h>
#include <string.h>

#include <vector>

#include "mpmg_fp64_common.cuh"
#include "mpmg_internal.cuh"
#include "mpmg_materials.cuh"

namespace {

using fp64::BcParams;
using fp64::GridGeom;
using fp64::ShapeFns;

constexpr int kAdjThreads = 256;
constexpr int kStateFields = 9;     // x y vx vy v sxx sxy syy Tzz
constexpr int kNodeFields = 5;      // m ax ay vx vy

// Parameter adjoint slots (mpmg_adj_backward's dtheta).
enum { TH_MU_S = 0, TH_MU_2 = 1, TH_I0 = 2, TH_E = 3, TH_COUNT = 4, TH_A = 4, TH_ALL = 5 };

struct MatParams {
    double G, K, lambda, dt, nu;
    double mu_s, mu_2, I0, grains_rho, grains_d, rho_critical;
    double A;               // nonlocal amplitude (g_nonlocal_mu2)
};

// ---------------------------------------------------------------------------
// Material laws reversed.  Inputs: the start-of-step stress T, the strain
// rate and spin (exx, exy, eyy, wxy), mass and updated volume; Tb the
// adjoint of the updated stress.  Outputs: the adjoint of T (overwrites Tb),
// of the strain rate and spin, and the parameter adjoint in terms of G, K
// (folded into E by the caller), mu_s, mu_2 and I0.

struct MatAdj {
    double exx, exy, eyy, wxy;
    double G, K, lambda, mu_s, mu_2, I0, A;
};

// isolin.c:75-116: s' = s + dt (lambda trD I + 2G D + W s - s W).
__device__ void isolin_adj(const MatParams &p, double exx, double exy, double eyy, double wxy, double sxx,
                           double sxy, double syy, double Tb[4], MatAdj &a)
{
    const double dt = p.dt, trD = exx + eyy;
    const double bxx = Tb[0], bxy = Tb[1], byy = Tb[2];
    a.exx += dt * (p.lambda * (bxx + byy) + 2.0 * p.G * bxx);
    a.eyy += dt * (p.lambda * (bxx + byy) + 2.0 * p.G * byy);
    a.exy += dt * 2.0 * p.G * bxy;
    a.wxy += dt * (2.0 * sxy * bxx - (sxx - syy) * bxy - 2.0 * sxy * byy);
    a.lambda += dt * trD * (bxx + byy);
    a.G += dt * 2.0 * (exx * bxx + exy * bxy + eyy * byy);
    Tb[0] = bxx - dt * wxy * bxy;
    Tb[2] = byy + dt * wxy * bxy;
    Tb[1] = bxy + dt * 2.0 * wxy * (bxx - byy);
    Tb[3] = 0.0;
}

// g_local_mu2.c:165-310 (plane strain, T = [[Txx, Txy, 0], [Txy, Tyy, 0],
// [0, 0, Tzz]]): trial Jaumann stress, deviatoric split, mu(I) return map.
__device__ void g_local_mu2_adj(const MatParams &p, double m, double v, double exx, double exy, double eyy,
                                double wxy, double Txx, double Txy, double Tyy, double Tzz, double Tb[4],
                                MatAdj &a)
{
    const double G = p.G, dt = p.dt, lambda = p.lambda;
    const double trD = exx + eyy;
    const double lt = lambda * trD;
    const double Ttr_xx = (2.0 * G * exx + lt + 2.0 * wxy * Txy) * dt + Txx;
    const double Ttr_xy = (2.0 * G * exy + wxy * (Tyy - Txx)) * dt + Txy;
    const double Ttr_yy = (2.0 * G * eyy + lt - 2.0 * wxy * Txy) * dt + Tyy;
    const double Ttr_zz = lt * dt + Tzz;
    const double pm = (Ttr_xx + Ttr_yy + Ttr_zz) / 3.0;
    const double T0xx = Ttr_xx - pm, T0yy = Ttr_yy - pm, T0zz = Ttr_zz - pm, T0xy = Ttr_xy;
    const double tt = T0xx * T0xx + 2.0 * T0xy * T0xy + T0yy * T0yy + T0zz * T0zz;
    const double tau = sqrt(0.5 * tt);
    const double pr = -pm;

    // adjoint of the trial stress
    double bxx = 0, bxy = 0, byy = 0, bzz = 0;
    if (m / v < p.rho_critical || !(pr > 0)) {
        // stress-free (or undefined) branch: T' = 0 does not depend on anything
    } else {
        const double S0 = p.mu_s * pr;
        if (tau <= S0) {
            // elastic: T' = T0 - p I = T_trial
            bxx = Tb[0];
            bxy = Tb[1];
            byy = Tb[2];
            bzz = Tb[3];
        } else {
            const double S2 = p.mu_2 * pr;
            const double sq = sqrt(pr / p.grains_rho);
            const double ca = G * p.I0 * dt / p.grains_d;
            const double alpha = ca * sq;
            const double B = -(S2 + tau + alpha);
            const double H = S2 * tau + S0 * alpha;
            const double disc = sqrt(B * B - 4.0 * H);
            double taup, dB, dH;     // tau' and its partial derivatives
            if (B > 0) {
                taup = 0.5 * (-B - disc);
                dB = 0.5 * (-1.0 - B / disc);
                dH = 1.0 / disc;
            } else {
                const double q = -B + disc;
                taup = 2.0 * H / q;
                const double dqB = -1.0 + B / disc, dqH = -2.0 / disc;
                dB = -2.0 * H / (q * q) * dqB;
                dH = 2.0 / q - 2.0 * H / (q * q) * dqH;
            }
            const double s = taup / tau;
            // T'_ii = T0_ii s + pm (ii = xx, yy, zz), T'_xy = T0xy s
            const double sb = Tb[0] * T0xx + Tb[1] * T0xy + Tb[2] * T0yy + Tb[3] * T0zz;
            double b0xx = Tb[0] * s, b0xy = Tb[1] * s, b0yy = Tb[2] * s, b0zz = Tb[3] * s;
            double pmb = Tb[0] + Tb[2] + Tb[3];
            const double taupb = sb / tau;
            double taub = -sb * taup / (tau * tau);
            const double Bb = taupb * dB, Hb = taupb * dH;
            // H = S2 tau + S0 alpha; B = -(S2 + tau + alpha)
            double S2b = Hb * tau - Bb;
            taub += Hb * S2 - Bb;
            double S0b = Hb * alpha;
            const double alphab = Hb * S0 - Bb;
            // alpha = ca sqrt(p / rho_g), ca = G I0 dt / d
            double prb = alphab * ca * 0.5 / (sq * p.grains_rho);
            const double cab = alphab * sq;
            a.G += cab * p.I0 * dt / p.grains_d;
            a.I0 += cab * G * dt / p.grains_d;
            a.mu_2 += S2b * pr;
            prb += S2b * p.mu_2;
            a.mu_s += S0b * pr;
            prb += S0b * p.mu_s;
            pmb -= prb;
            // tau = sqrt(tt / 2), tt = T0xx^2 + 2 T0xy^2 + T0yy^2 + T0zz^2
            const double ttb = taub / (4.0 * tau);
            b0xx += 2.0 * T0xx * ttb;
            b0xy += 4.0 * T0xy * ttb;
            b0yy += 2.0 * T0yy * ttb;
            b0zz += 2.0 * T0zz * ttb;
            // T0_ii = Ttr_ii - pm, pm = (Ttr_xx + Ttr_yy + Ttr_zz) / 3
            pmb -= b0xx + b0yy + b0zz;
            bxx = b0xx + pmb / 3.0;
            byy = b0yy + pmb / 3.0;
            bzz = b0zz + pmb / 3.0;
            bxy = b0xy;
        }
    }
    // trial stress reversed
    const double trb = bxx + byy + bzz;
    a.exx += dt * (2.0 * G * bxx + lambda * trb);
    a.eyy += dt * (2.0 * G * byy + lambda * trb);
    a.exy += dt * 2.0 * G * bxy;
    a.wxy += dt * (2.0 * Txy * bxx + (Tyy - Txx) * bxy - 2.0 * Txy * byy);
    a.G += dt * 2.0 * (exx * bxx + exy * bxy + eyy * byy);
    a.lambda += dt * trD * trb;
    Tb[0] = bxx - dt * wxy * bxy;
    Tb[1] = bxy + dt * 2.0 * wxy * (bxx - byy);
    Tb[2] = byy + dt * wxy * bxy;
    Tb[3] = bzz;
}

// Upper-triangle index of (a, b), a <= b, in an element's 10-entry symmetric
// block (the layout of the fluidity assembly).
__device__ __forceinline__ int sym10(int a, int b)
{
    const int row_start[4] = {0, 4, 7, 9};
    return row_start[a] + (b - a);
}

// g_nonlocal_mu2 reversed for one particle: the stress update after the
// fluidity solve (g_nonlocal_mu2.c:160-218), the bulk fluidity
// (calculate_bulk_granular_fluidity, :238-321) and the particle's share of
// the assembled system (:418-507: K_ab += v (xi^-2 N_a N_b + grad N_a .
// grad N_b), f_a += v gf_local xi^-2 N_a over dense particles).  gf is the
// fluidity interpolated at the particle; kb and fb are the adjoints of its
// element's block and right-hand side.  Returns, besides Tb and a as
// g_local_mu2_adj does, the adjoint of the updated volume (vb) and adds the
// adjoints of the shape values and gradients to sb, gxb, gyb.  (The
// adjoint of gf itself is formed by adj_nl_pre_kernel.)
__device__ void g_nonlocal_mu2_adj(const MatParams &p, double m, double v, double exx, double exy, double eyy,
                                   double wxy, double Txx, double Txy, double Tyy, const ShapeFns &f, double gf,
                                   const double kb[10], const double fb[4], double Tb[4], MatAdj &a, double &vb,
                                   double sb[4], double gxb[4], double gyb[4])
{
    const double G = p.G, dt = p.dt, lambda = p.K - 2.0 * G / 3.0;
    const double trD = exx + eyy;
    const double sxx_tr = Txx + dt * (lambda * trD + 2.0 * G * exx + 2.0 * wxy * Txy);
    const double sxy_tr = Txy + dt * (2.0 * G * exy - wxy * (Txx - Tyy));
    const double syy_tr = Tyy + dt * (lambda * trD + 2.0 * G * eyy - 2.0 * wxy * Txy);
    const double pr = -0.5 * (sxx_tr + syy_tr);
    const double t0xx = sxx_tr + pr, t0xy = sxy_tr, t0yy = syy_tr + pr;
    const double tau = sqrt(0.5 * (t0xx * t0xx + 2.0 * t0xy * t0xy + t0yy * t0yy));
    const bool dense = !(m / v < p.rho_critical || pr < 0);
    double t0xxb = 0, t0xyb = 0, t0yyb = 0, prb = 0, taub = 0;
    vb = 0;
    if (dense && pr > 0) {
        // stress update: s = pr / (G dt gf + pr), T' = s t0 - pr I
        const double den = G * dt * gf + pr;
        const double sc = pr / den;
        const double sbar = Tb[0] * t0xx + Tb[1] * t0xy + Tb[2] * t0yy;
        t0xxb += sc * Tb[0];
        t0xyb += sc * Tb[1];
        t0yyb += sc * Tb[2];
        prb -= Tb[0] + Tb[2];
        prb += sbar * (G * dt * gf) / (den * den);
        a.G -= sbar * pr * dt * gf / (den * den);

        // bulk fluidity: tau' from the mu(I) return (tau itself below yield)
        const double S0 = p.mu_s * pr;
        const bool plastic = tau > S0;
        double taup = tau, dB = 0, dH = 0, S2 = 0, alpha = 0, sq = 0, ca = 0;
        if (plastic) {
            S2 = p.mu_2 * pr;
            sq = sqrt(pr / p.grains_rho);
            ca = G * p.I0 * dt / p.grains_d;
            alpha = ca * sq;
            const double B = -(S2 + tau + alpha);
            const double H = S2 * tau + S0 * alpha;
            const double disc = sqrt(B * B - 4.0 * H);
            if (B > 0) {
                taup = 0.5 * (-B - disc);
                dB = 0.5 * (-1.0 - B / disc);
                dH = 1.0 / disc;
            } else {
                const double q = -B + disc;
                taup = 2.0 * H / q;
                const double dqB = -1.0 + B / disc, dqH = -2.0 / disc;
                dB = -2.0 * H / (q * q) * dqB;
                dH = 2.0 / q - 2.0 * H / (q * q) * dqH;
            }
        }
        const double gfl = plastic ? pr / (G * dt) * (tau / taup - 1.0) : 0.0;
        const double D = p.A * p.A * p.grains_d * p.grains_d;
        const double r = taup / pr - p.mu_s;
        const double xisq = fabs(r) / D;

        // the particle's share of the element block and right-hand side
        double xisqb = 0, gflb = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
#pragma unroll
            for (int j = i; j < 4; j++) {
                const double k = kb[sym10(i, j)];
                vb += k * (xisq * f.s[i] * f.s[j] + f.gx[i] * f.gx[j] + f.gy[i] * f.gy[j]);
                xisqb += k * v * f.s[i] * f.s[j];
                sb[i] += k * v * xisq * f.s[j];
                sb[j] += k * v * xisq * f.s[i];
                gxb[i] += k * v * f.gx[j];
                gxb[j] += k * v * f.gx[i];
                gyb[i] += k * v * f.gy[j];
                gyb[j] += k * v * f.gy[i];
            }
            vb += fb[i] * gfl * xisq * f.s[i];
            gflb += fb[i] * v * xisq * f.s[i];
            xisqb += fb[i] * v * gfl * f.s[i];
            sb[i] += fb[i] * v * gfl * xisq;
        }
        // xi^-2 = |tau' / pr - mu_s| / (A^2 d^2)
        const double rb = xisqb * (r >= 0 ? 1.0 : -1.0) / D;
        a.A -= xisqb * 2.0 * xisq / p.A;
        double taupb = rb / pr;
        prb -= rb * taup / (pr * pr);
        a.mu_s -= rb;
        if (plastic) {
            // gf_local = pr / (G dt) (tau / tau' - 1)
            const double c = pr / (G * dt);
            prb += gflb * (tau / taup - 1.0) / (G * dt);
            a.G -= gflb * gfl / G;
            taub += gflb * c / taup;
            taupb -= gflb * c * tau / (taup * taup);
            // the return's root reversed (as in g_local_mu2_adj)
            const double Bb = taupb * dB, Hb = taupb * dH;
            const double S2b = Hb * tau - Bb;
            taub += Hb * S2 - Bb;
            const double S0b = Hb * alpha;
            const double alphab = Hb * S0 - Bb;
            prb += alphab * ca * 0.5 / (sq * p.grains_rho);
            const double cab = alphab * sq;
            a.G += cab * p.I0 * dt / p.grains_d;
            a.I0 += cab * G * dt / p.grains_d;
            a.mu_2 += S2b * pr;
            prb += S2b * p.mu_2;
            a.mu_s += S0b * pr;
            prb += S0b * p.mu_s;
        } else {
            taub += taupb;
        }
    }
    // tau = sqrt((t0xx^2 + 2 t0xy^2 + t0yy^2) / 2)
    if (tau > 0) {
        t0xxb += taub * t0xx / (2.0 * tau);
        t0xyb += taub * t0xy / tau;
        t0yyb += taub * t0yy / (2.0 * tau);
    }
    // t0 = T_trial + pr I (xx, yy), pr = -(T_trial,xx + T_trial,yy) / 2
    const double P = prb + t0xxb + t0yyb;
    const double bxx = t0xxb - 0.5 * P, byy = t0yyb - 0.5 * P, bxy = t0xyb;
    // the trial Jaumann stress reversed, lambda = K - 2G/3
    a.exx += dt * (lambda * (bxx + byy) + 2.0 * G * bxx);
    a.eyy += dt * (lambda * (bxx + byy) + 2.0 * G * byy);
    a.exy += dt * 2.0 * G * bxy;
    a.wxy += dt * (2.0 * Txy * bxx - (Txx - Tyy) * bxy - 2.0 * Txy * byy);
    a.lambda += dt * trD * (bxx + byy);
    a.G += dt * 2.0 * (exx * bxx + exy * bxy + eyy * byy);
    Tb[0] = bxx - dt * wxy * bxy;
    Tb[2] = byy + dt * wxy * bxy;
    Tb[1] = bxy + dt * 2.0 * wxy * (bxx - byy);
}

// Mixed second derivative of the shape functions, d2 N_a / dx dy (tent
// products): +1, -1, +1, -1 over h^2 for BL, BR, TR, TL.
__device__ __forceinline__ double shape_xy(int a, double inv_h)
{
    return ((a & 1) ? -1.0 : 1.0) * inv_h * inv_h;
}

struct AdjStep {
    GridGeom g;
    BcParams bc;
    MatParams mp;
    int material;
    int n, ne, nn;
    double dt;
    // recorded forward inputs of the step
    const double *state;        // kStateFields x n, start of step
    const double *mass;         // n (constant)
    const int *elem;            // n
    const int *active;          // n
    const uint32_t *perm;       // n
    const int *cell_start;      // ne + 1
    const double *nodes;        // kNodeFields x nn
    const StepParams *params;   // after the step (t used by the BCs, the step's gravity)
    // adjoints
    const double *adj_in;       // kStateFields x n, of the state after the step
    double *adj_out;            // kStateFields x n, of the state at the step start
    double *contrib;            // 16 x n: per particle and corner (Ux, Uy, Ax, Ay) adjoint shares
    double *cell_adj;           // 16 x ne, value-major
    double *node_adj;           // 5 x nn: pb_x, pb_y, fb_x, fb_y, mb
    double *theta_part;         // per adj_g2p block: TH_COUNT + (G, K, lambda) partials
    // g_nonlocal_mu2
    const double *gf_nodes;     // nn: the step's nodal fluidity (solution of the solve)
    double *gfb;                // n: adjoint of the fluidity interpolated at each particle
    double *rhs;                // 4 x ne: its gather to the nodes, as element corner sums
    const double *lam;          // nn: adjoint of the nodal fluidity (the adjoint solve)
};

constexpr int kThetaSlots = 7;   // mu_s mu_2 I0 (direct) G K lambda, E folded later; A (nonlocal)

__global__ void __launch_bounds__(kAdjThreads) adj_g2p_kernel(AdjStep S)
{
    __shared__ double red[kAdjThreads / 32][kThetaSlots];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double th[kThetaSlots] = {0, 0, 0, 0, 0, 0, 0};
    if (i < S.n) {
        const size_t n = (size_t)S.n;
        double in[kStateFields];
#pragma unroll
        for (int f = 0; f < kStateFields; f++) in[f] = S.adj_in[f * n + i];
        const int e = S.elem[i];
        if (!S.active[i] || e < 0) {
            // inactive: the state is carried unchanged
#pragma unroll
            for (int f = 0; f < kStateFields; f++) S.adj_out[f * n + i] = in[f];
#pragma unroll
            for (int k = 0; k < 16; k++) S.contrib[k * n + i] = 0.0;
        } else {
            const GridGeom &g = S.g;
            const double x = S.state[0 * n + i], y = S.state[1 * n + i];
            const double V = S.state[4 * n + i];
            const double Txx = S.state[5 * n + i], Txy = S.state[6 * n + i], Tyy = S.state[7 * n + i],
                         Tzz = S.state[8 * n + i];
            const int ci = e % g.Ex, cj = e / g.Ex;
            const int n0 = cj * g.Nx + ci;
            const int nd[4] = {n0, n0 + 1, n0 + 1 + g.Nx, n0 + g.Nx};
            const double xl = (x - ci * g.h) * g.inv_h, yl = (y - cj * g.h) * g.inv_h;
            const ShapeFns f = fp64::shape(xl, yl, g.inv_h);
            const size_t nn = (size_t)S.nn;
            double ax[4], ay[4], ux[4], uy[4];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                ax[a] = S.nodes[1 * nn + nd[a]];
                ay[a] = S.nodes[2 * nn + nd[a]];
                ux[a] = S.nodes[3 * nn + nd[a]];
                uy[a] = S.nodes[4 * nn + nd[a]];
            }
            double exx = 0, eyy = 0, dxdy = 0, dydx = 0;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                exx += f.gx[a] * ux[a];
                eyy += f.gy[a] * uy[a];
                dxdy += f.gy[a] * ux[a];
                dydx += f.gx[a] * uy[a];
            }
            const double dt = S.dt;
            const double exy = 0.5 * (dxdy + dydx), wxy = 0.5 * (dxdy - dydx);
            const double ex = mat::exp_small(dt * (exx + eyy));
            const double Vn = V * ex;

            // material
            double Tb[4] = {in[5], in[6], in[7], in[8]};
            MatAdj ma = {};
            double vnl = 0, snl[4] = {0, 0, 0, 0}, gxnl[4] = {0, 0, 0, 0}, gynl[4] = {0, 0, 0, 0};
            if (S.material == MPMG_ISOLIN) {
                isolin_adj(S.mp, exx, exy, eyy, wxy, Txx, Txy, Tyy, Tb, ma);
                Tb[3] = in[8];      // isolin leaves Tzz alone
            } else if (S.material == MPMG_G_NONLOCAL_MU2) {
                // the element's nodal fluidity g and its adjoint lam: the block's
                // adjoint is -(lam g^T) symmetrised, the right-hand side's lam
                double gn[4], ln[4], gf = 0;
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    gn[a] = S.gf_nodes[nd[a]];
                    ln[a] = S.lam[nd[a]];
                    gf += gn[a] * f.s[a];
                }
                double kb[10], fb[4];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    fb[a] = ln[a];
#pragma unroll
                    for (int b = a; b < 4; b++)
                        kb[sym10(a, b)] = a == b ? -ln[a] * gn[a] : -(ln[a] * gn[b] + ln[b] * gn[a]);
                }
                g_nonlocal_mu2_adj(S.mp, S.mass[i], Vn, exx, exy, eyy, wxy, Txx, Txy, Tyy, f, gf, kb, fb, Tb, ma,
                                   vnl, snl, gxnl, gynl);
                // the fluidity gather gf = sum N_a g_a, shape values reversed
                const double gfb = S.gfb[i];
#pragma unroll
                for (int a = 0; a < 4; a++) snl[a] += gfb * gn[a];
                Tb[3] = in[8];      // plane stress state: Tzz is carried
            } else {
                g_local_mu2_adj(S.mp, S.mass[i], Vn, exx, exy, eyy, wxy, Txx, Txy, Tyy, Tzz, Tb, ma);
            }
            // volume V' = V exp(dt trD) (the nonlocal assembly also reads V')
            const double vnb = in[4] + vnl;
            const double Vb = vnb * ex;
            const double trb = vnb * Vn * dt;
            const double exxb = ma.exx + trb, eyyb = ma.eyy + trb;
            const double dxdyb = 0.5 * (ma.exy + ma.wxy), dydxb = 0.5 * (ma.exy - ma.wxy);
            // gathers
            double sb[4], gxb[4], gyb[4];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const double uxb = exxb * f.gx[a] + dxdyb * f.gy[a] + dt * f.s[a] * in[0];
                const double uyb = eyyb * f.gy[a] + dydxb * f.gx[a] + dt * f.s[a] * in[1];
                const double axb = dt * f.s[a] * in[2];
                const double ayb = dt * f.s[a] * in[3];
                S.contrib[(a * 4 + 0) * n + i] = uxb;
                S.contrib[(a * 4 + 1) * n + i] = uyb;
                S.contrib[(a * 4 + 2) * n + i] = axb;
                S.contrib[(a * 4 + 3) * n + i] = ayb;
                sb[a] = dt * (ux[a] * in[0] + uy[a] * in[1] + ax[a] * in[2] + ay[a] * in[3]) + snl[a];
                gxb[a] = exxb * ux[a] + dydxb * uy[a] + gxnl[a];
                gyb[a] = eyyb * uy[a] + dxdyb * ux[a] + gynl[a];
            }
            double xb = in[0], yb = in[1];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const double hxy = shape_xy(a, g.inv_h);
                xb += sb[a] * f.gx[a] + gyb[a] * hxy;
                yb += sb[a] * f.gy[a] + gxb[a] * hxy;
            }
            S.adj_out[0 * n + i] = xb;
            S.adj_out[1 * n + i] = yb;
            S.adj_out[2 * n + i] = in[2];
            S.adj_out[3 * n + i] = in[3];
            S.adj_out[4 * n + i] = Vb;
            S.adj_out[5 * n + i] = Tb[0];
            S.adj_out[6 * n + i] = Tb[1];
            S.adj_out[7 * n + i] = Tb[2];
            S.adj_out[8 * n + i] = Tb[3];
            th[0] = ma.mu_s;
            th[1] = ma.mu_2;
            th[2] = ma.I0;
            th[3] = ma.G;
            th[4] = ma.K;
            th[5] = ma.lambda;
            th[6] = ma.A;
        }
    }
    // block partials of the parameter adjoint (fixed tree order)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kThetaSlots; k++) {
        double v = th[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[w][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kThetaSlots) {
        double v = 0;
        for (int q = 0; q < kAdjThreads / 32; q++) v += red[q][threadIdx.x];
        S.theta_part[(size_t)blockIdx.x * kThetaSlots + threadIdx.x] = v;
    }
}

// g_nonlocal_mu2, before adj_g2p: per particle, the adjoint of the fluidity
// interpolated at it, through the stress update s = pr / (G dt gf + pr),
// T' = s t0 - pr I (g_nonlocal_mu2.c:160-218).
__global__ void __launch_bounds__(kAdjThreads) adj_nl_pre_kernel(AdjStep S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int e = S.elem[i];
    double gfb = 0;
    if (S.active[i] && e >= 0) {
        const GridGeom &g = S.g;
        const size_t n = (size_t)S.n, nn = (size_t)S.nn;
        const double x = S.state[0 * n + i], y = S.state[1 * n + i], V = S.state[4 * n + i];
        const double Txx = S.state[5 * n + i], Txy = S.state[6 * n + i], Tyy = S.state[7 * n + i];
        const int ci = e % g.Ex, cj = e / g.Ex;
        const int n0 = cj * g.Nx + ci;
        const int nd[4] = {n0, n0 + 1, n0 + 1 + g.Nx, n0 + g.Nx};
        const double xl = (x - ci * g.h) * g.inv_h, yl = (y - cj * g.h) * g.inv_h;
        const ShapeFns f = fp64::shape(xl, yl, g.inv_h);
        double exx = 0, eyy = 0, dxdy = 0, dydx = 0, gf = 0;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const double ux = S.nodes[3 * nn + nd[a]], uy = S.nodes[4 * nn + nd[a]];
            exx += f.gx[a] * ux;
            eyy += f.gy[a] * uy;
            dxdy += f.gy[a] * ux;
            dydx += f.gx[a] * uy;
            gf += S.gf_nodes[nd[a]] * f.s[a];
        }
        const MatParams &p = S.mp;
        const double dt = S.dt, G = p.G, lambda = p.K - 2.0 * G / 3.0;
        const double exy = 0.5 * (dxdy + dydx), wxy = 0.5 * (dxdy - dydx);
        const double Vn = V * mat::exp_small(dt * (exx + eyy));
        const double trD = exx + eyy;
        const double sxx_tr = Txx + dt * (lambda * trD + 2.0 * G * exx + 2.0 * wxy * Txy);
        const double sxy_tr = Txy + dt * (2.0 * G * exy - wxy * (Txx - Tyy));
        const double syy_tr = Tyy + dt * (lambda * trD + 2.0 * G * eyy - 2.0 * wxy * Txy);
        const double pr = -0.5 * (sxx_tr + syy_tr);
        const bool dense = !(S.mass[i] / Vn < p.rho_critical || pr < 0);
        if (dense && pr > 0) {
            const double den = G * dt * gf + pr;
            const double sbar = S.adj_in[5 * n + i] * (sxx_tr + pr) + S.adj_in[6 * n + i] * sxy_tr +
                                S.adj_in[7 * n + i] * (syy_tr + pr);
            gfb = -sbar * pr * G * dt / (den * den);
        }
    }
    S.gfb[i] = gfb;
}

// g_nonlocal_mu2: per element, the gather gf_p = sum N_a g_a reversed as
// corner sums N_a gfb_p over the element's particles in the binned order
// (the right-hand-side layout of the assembly, so that the solver sums the
// corners to the nodes).
__global__ void __launch_bounds__(128) adj_nl_rhs_kernel(AdjStep S)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= S.ne) return;
    const GridGeom &g = S.g;
    const size_t n = (size_t)S.n;
    const int ci = e % g.Ex, cj = e / g.Ex;
    double F[4] = {0, 0, 0, 0};
    for (int k = S.cell_start[e]; k < S.cell_start[e + 1]; k++) {
        const int i = (int)S.perm[k];
        const double xl = (S.state[0 * n + i] - ci * g.h) * g.inv_h, yl = (S.state[1 * n + i] - cj * g.h) * g.inv_h;
        const ShapeFns f = fp64::shape(xl, yl, g.inv_h);
        const double gfb = S.gfb[i];
#pragma unroll
        for (int a = 0; a < 4; a++) F[a] += f.s[a] * gfb;
    }
#pragma unroll
    for (int a = 0; a < 4; a++) S.rhs[(size_t)a * S.ne + e] = F[a];
}

// Per element: the corner shares of its particles, in the binned order.
__global__ void __launch_bounds__(128) adj_cells_kernel(AdjStep S)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= S.ne) return;
    const int k0 = S.cell_start[e], k1 = S.cell_start[e + 1];
    double acc[16];
#pragma unroll
    for (int k = 0; k < 16; k++) acc[k] = 0.0;
    const size_t n = (size_t)S.n;
    for (int k = k0; k < k1; k++) {
        const int i = (int)S.perm[k];
#pragma unroll
        for (int q = 0; q < 16; q++) acc[q] += S.contrib[q * n + i];
    }
#pragma unroll
    for (int q = 0; q < 16; q++) S.cell_adj[(size_t)q * S.ne + e] = acc[q];
}

// Per node: the nodal update reversed (grid_kernel of mpmg_step.cu).
__global__ void __launch_bounds__(256) adj_grid_kernel(AdjStep S)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= S.nn) return;
    const GridGeom &g = S.g;
    const int i = n % g.Nx, j = n / g.Nx;
    double ub[4] = {0, 0, 0, 0};     // Ux, Uy, Ax, Ay adjoints
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        const int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        const int e = cj * g.Ex + ci;
        if (S.cell_start[e] == S.cell_start[e + 1]) continue;
        const int corner = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
#pragma unroll
        for (int q = 0; q < 4; q++) ub[q] += S.cell_adj[(size_t)(corner * 4 + q) * S.ne + e];
    }
    const size_t nn = (size_t)S.nn;
    const double m = S.nodes[n];
    double pbx = 0, pby = 0, fbx = 0, fby = 0, mb = 0;
    if (m > MPMG_TOL) {
        bool bx, by;
        fp64::bc_mask(S.bc, g, i, j, S.params->t, bx, by);
        const double ax = S.nodes[1 * nn + n], ay = S.nodes[2 * nn + n];
        const double ux = S.nodes[3 * nn + n], uy = S.nodes[4 * nn + n];
        // U = (P + dt F) / m, A = F / m on unmasked components
        if (!bx) {
            pbx = ub[0] / m;
            fbx = (ub[2] + S.dt * ub[0]) / m;
            mb -= (ub[0] * ux + ub[2] * ax) / m;
        }
        if (!by) {
            pby = ub[1] / m;
            fby = (ub[3] + S.dt * ub[1]) / m;
            mb -= (ub[1] * uy + ub[3] * ay) / m;
        }
    }
    S.node_adj[0 * nn + n] = pbx;
    S.node_adj[1 * nn + n] = pby;
    S.node_adj[2 * nn + n] = fbx;
    S.node_adj[3 * nn + n] = fby;
    S.node_adj[4 * nn + n] = mb;
}

// Per particle: P2G (p2g_cells_kernel of mpmg_step.cu) reversed.
__global__ void __launch_bounds__(kAdjThreads) adj_p2g_kernel(AdjStep S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int e = S.elem[i];
    if (!S.active[i] || e < 0) return;
    const GridGeom &g = S.g;
    const size_t n = (size_t)S.n, nn = (size_t)S.nn;
    const double x = S.state[0 * n + i], y = S.state[1 * n + i];
    const double vx = S.state[2 * n + i], vy = S.state[3 * n + i];
    const double V = S.state[4 * n + i];
    const double Txx = S.state[5 * n + i], Txy = S.state[6 * n + i], Tyy = S.state[7 * n + i];
    const double mp = S.mass[i];
    const double grav = S.params->gravity;
    const int ci = e % g.Ex, cj = e / g.Ex;
    const int n0 = cj * g.Nx + ci;
    const int nd[4] = {n0, n0 + 1, n0 + 1 + g.Nx, n0 + g.Nx};
    const double xl = (x - ci * g.h) * g.inv_h, yl = (y - cj * g.h) * g.inv_h;
    const ShapeFns f = fp64::shape(xl, yl, g.inv_h);
    double vxb = 0, vyb = 0, Vb = 0, Txxb = 0, Txyb = 0, Tyyb = 0, xb = 0, yb = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const double pbx = S.node_adj[0 * nn + nd[a]], pby = S.node_adj[1 * nn + nd[a]];
        const double fbx = S.node_adj[2 * nn + nd[a]], fby = S.node_adj[3 * nn + nd[a]];
        const double mb = S.node_adj[4 * nn + nd[a]];
        // m_a += N m; P_a += N m v; F_a += N m b - V T grad N (b = (0, g))
        const double sb = mb * mp + mp * (vx * pbx + vy * pby) + mp * grav * fby;
        vxb += f.s[a] * mp * pbx;
        vyb += f.s[a] * mp * pby;
        const double tgx = Txx * f.gx[a] + Txy * f.gy[a], tgy = Txy * f.gx[a] + Tyy * f.gy[a];
        Vb -= fbx * tgx + fby * tgy;
        Txxb -= V * fbx * f.gx[a];
        Txyb -= V * (fbx * f.gy[a] + fby * f.gx[a]);
        Tyyb -= V * fby * f.gy[a];
        const double gxb = -V * (fbx * Txx + fby * Txy), gyb = -V * (fbx * Txy + fby * Tyy);
        const double hxy = shape_xy(a, g.inv_h);
        xb += sb * f.gx[a] + gyb * hxy;
        yb += sb * f.gy[a] + gxb * hxy;
    }
    S.adj_out[0 * n + i] += xb;
    S.adj_out[1 * n + i] += yb;
    S.adj_out[2 * n + i] += vxb;
    S.adj_out[3 * n + i] += vyb;
    S.adj_out[4 * n + i] += Vb;
    S.adj_out[5 * n + i] += Txxb;
    S.adj_out[6 * n + i] += Txyb;
    S.adj_out[7 * n + i] += Tyyb;
}

// The step's block partials added in block order (one thread per slot).
__global__ void adj_theta_kernel(const double *__restrict__ part, int blocks, double *__restrict__ acc)
{
    const int k = threadIdx.x;
    if (k >= kThetaSlots) return;
    double v = acc[k];
    for (int b = 0; b < blocks; b++) v += part[(size_t)b * kThetaSlots + k];
    acc[k] = v;
}

// Copies the step-start particle state into a tape slot (one launch).
__global__ void save_state_kernel(int n, const double *x, const double *y, const double *vx, const double *vy,
                                  const double *v, const double *sxx, const double *sxy, const double *syy,
                                  const double *Tzz, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    out[0 * N + i] = x[i];
    out[1 * N + i] = y[i];
    out[2 * N + i] = vx[i];
    out[3 * N + i] = vy[i];
    out[4 * N + i] = v[i];
    out[5 * N + i] = sxx[i];
    out[6 * N + i] = sxy[i];
    out[7 * N + i] = syy[i];
    out[8 * N + i] = Tzz ? Tzz[i] : 0.0;
}

__global__ void load_state_kernel(int n, const double *__restrict__ in, double *x, double *y, double *vx,
                                  double *vy, double *v, double *sxx, double *sxy, double *syy, double *Tzz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    x[i] = in[0 * N + i];
    y[i] = in[1 * N + i];
    vx[i] = in[2 * N + i];
    vy[i] = in[3 * N + i];
    v[i] = in[4 * N + i];
    sxx[i] = in[5 * N + i];
    sxy[i] = in[6 * N + i];
    syy[i] = in[7 * N + i];
    if (Tzz) Tzz[i] = in[8 * N + i];
}

// Records the step's outputs the reverse pass needs: elements and activity
// after the keys phase, the binned order, the nodal fields, the step record.
__global__ void save_step_kernel(int n, int ne, int nn, const int *in_element, const int *active,
                                 const uint32_t *perm, const int *cell_start, const double *node_m,
                                 const double *node_ax, const double *node_ay, const double *node_vx,
                                 const double *node_vy, const StepParams *sp, int *__restrict__ elem_out,
                                 int *__restrict__ active_out, uint32_t *__restrict__ perm_out,
                                 int *__restrict__ cs_out, double *__restrict__ nodes_out,
                                 StepParams *__restrict__ sp_out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) *sp_out = *sp;
    if (k < n) {
        elem_out[k] = active[k] ? in_element[k] : -1;
        active_out[k] = active[k];
        perm_out[k] = perm[k];
    }
    if (k <= ne) cs_out[k] = cell_start[k];
    if (k < nn) {
        const size_t N = (size_t)nn;
        nodes_out[0 * N + k] = node_m[k];
        nodes_out[1 * N + k] = node_ax[k];
        nodes_out[2 * N + k] = node_ay[k];
        nodes_out[3 * N + k] = node_vx[k];
        nodes_out[4 * N + k] = node_vy[k];
    }
}

inline int blocks_for(size_t n, int threads)
{
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    return (int)(b > 0 ? b : 1);
}

template <typename T>
int dalloc(T **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return mpmg_cuda_status(e, "cudaMalloc (adjoint tape)");
    }
    return MPMG_OK;
}

}  // namespace

// Tape of a forward run (checkpoints) and the scratch of the reverse pass.
struct AdjTape {
    int K = 0;                      // checkpoint interval
    int nsteps = 0;                 // steps of the taped run
    int nck = 0;                    // checkpoints (steps 0, K, 2K, ... < nsteps)
    double *ck_state = nullptr;     // nck x kStateFields x n
    int *ck_active = nullptr;       // nck x n
    int *ck_elem = nullptr;         // nck x n (in_element)
    StepParams *ck_params = nullptr;   // nck (device)
    double *final_state = nullptr;  // kStateFields x n, the state after the run
    int *final_active = nullptr, *final_elem = nullptr;
    StepParams *final_params = nullptr;
    // one segment of recorded steps
    double *seg_state = nullptr;    // K x kStateFields x n
    int *seg_elem = nullptr, *seg_active = nullptr;   // K x n
    uint32_t *seg_perm = nullptr;   // K x n
    int *seg_cs = nullptr;          // K x (ne + 1)
    double *seg_nodes = nullptr;    // K x kNodeFields x nn
    StepParams *seg_params = nullptr;   // K
    // g_nonlocal_mu2: each recorded step's nodal fluidity and element blocks
    double *seg_gf = nullptr;       // K x nn
    double *seg_ek = nullptr;       // K x 10 x ne
    // reverse pass
    double *adj[2] = {nullptr, nullptr};   // kStateFields x n
    double *contrib = nullptr, *cell_adj = nullptr, *node_adj = nullptr;
    double *theta_part = nullptr, *theta_acc = nullptr;
    double *gfb = nullptr, *rhs = nullptr, *lam = nullptr;   // g_nonlocal_mu2
    double grad[TH_ALL] = {0, 0, 0, 0, 0};   // the last backward pass's parameter gradient
    int cur = 0;                    // adj[cur] holds the latest adjoint state
};

void mpmg_adj_free(mpmg_ctx *ctx)
{
    AdjTape *t = ctx->adj;
    if (t == nullptr) return;
    void *ptrs[] = {t->ck_state, t->ck_active, t->ck_elem, t->ck_params, t->final_state, t->final_active,
                    t->final_elem, t->final_params, t->seg_state, t->seg_elem, t->seg_active, t->seg_perm,
                    t->seg_cs, t->seg_nodes, t->seg_params, t->adj[0], t->adj[1], t->contrib, t->cell_adj,
                    t->node_adj, t->theta_part, t->theta_acc, t->seg_gf, t->seg_ek, t->gfb, t->rhs, t->lam};
    for (void *p : ptrs) cudaFree(p);
    delete t;
    ctx->adj = nullptr;
}

namespace {

int save_state(mpmg_ctx *ctx, double *out)
{
    const int n = (int)ctx->np;
    if (n == 0) return MPMG_OK;
    save_state_kernel<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, ctx->x, ctx->y, ctx->vx, ctx->vy, ctx->v,
                                                                    ctx->sxx, ctx->sxy, ctx->syy, ctx->Tzz, out);
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}

int load_state(mpmg_ctx *ctx, const double *in, const int *active, const int *elem, const StepParams *params)
{
    const int n = (int)ctx->np;
    cudaStream_t s = ctx->stream;
    if (n > 0) {
        load_state_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, in, ctx->x, ctx->y, ctx->vx, ctx->vy, ctx->v,
                                                            ctx->sxx, ctx->sxy, ctx->syy, ctx->Tzz);
        ctx->launches += 1;
        MPMG_CHECK(cudaMemcpyAsync(ctx->active, active, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
        MPMG_CHECK(cudaMemcpyAsync(ctx->in_element, elem, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    MPMG_CHECK(cudaMemcpyAsync(ctx->d_params, params, sizeof(StepParams), cudaMemcpyDeviceToDevice, s));
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}

int snapshot(mpmg_ctx *ctx, double *state, int *active, int *elem, StepParams *params)
{
    int rc = save_state(ctx, state);
    if (rc != MPMG_OK) return rc;
    cudaStream_t s = ctx->stream;
    const size_t n = ctx->np;
    if (n > 0) {
        MPMG_CHECK(cudaMemcpyAsync(active, ctx->active, n * sizeof(int), cudaMemcpyDeviceToDevice, s));
        MPMG_CHECK(cudaMemcpyAsync(elem, ctx->in_element, n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    MPMG_CHECK(cudaMemcpyAsync(params, ctx->d_params, sizeof(StepParams), cudaMemcpyDeviceToDevice, s));
    return MPMG_OK;
}

MatParams make_params(const mpmg_ctx *ctx)
{
    MatParams p;
    const mpmg_config &c = ctx->cfg;
    p.G = ctx->G;
    p.K = ctx->K;
    p.lambda = ctx->lambda;
    p.dt = c.dt;
    p.nu = c.mp[MPMG_MP_NU];
    p.mu_s = c.mp[MPMG_MP_MU_S];
    p.mu_2 = c.mp[MPMG_MP_MU_2];
    p.I0 = c.mp[MPMG_MP_I0];
    p.grains_rho = c.mp[MPMG_MP_GRAINS_RHO];
    p.grains_d = c.mp[MPMG_MP_GRAINS_D];
    p.rho_critical = c.mp[MPMG_MP_RHO_CRITICAL];
    p.A = c.mp[MPMG_MP_A];
    return p;
}

int check_adjoint_ctx(const mpmg_ctx *ctx)
{
    if (ctx->mixed || ctx->batch) {
        mpmg_set_error("the adjoint runs on the FP64 form of a single simulation");
        return MPMG_ERR_UNSUPPORTED;
    }
    if (ctx->cfg.material != MPMG_ISOLIN && ctx->cfg.material != MPMG_G_LOCAL_MU2 &&
        ctx->cfg.material != MPMG_G_NONLOCAL_MU2) {
        mpmg_set_error("the adjoint supports isolin, g_local_mu2 and g_nonlocal_mu2");
        return MPMG_ERR_UNSUPPORTED;
    }
    return MPMG_OK;
}

}  // namespace

extern "C" {

int mpmg_adj_forward_tape(mpmg_ctx *ctx, int nsteps, int checkpoint_every)
{
    if (ctx == nullptr || nsteps < 1 || checkpoint_every < 1) return MPMG_ERR_INVALID;
    int rc = check_adjoint_ctx(ctx);
    if (rc != MPMG_OK) return rc;
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    mpmg_adj_free(ctx);
    AdjTape *t = new (std::nothrow) AdjTape();
    if (t == nullptr) return MPMG_ERR_NOMEM;
    ctx->adj = t;
    const size_t n = ctx->np, ne = ctx->ne, nn = ctx->nn;
    const int K = checkpoint_every < nsteps ? checkpoint_every : nsteps;
    t->K = K;
    t->nsteps = nsteps;
    t->nck = (nsteps + K - 1) / K;
    const size_t nck = (size_t)t->nck;
    if ((rc = dalloc(&t->ck_state, nck * kStateFields * n)) != MPMG_OK ||
        (rc = dalloc(&t->ck_active, nck * n)) != MPMG_OK || (rc = dalloc(&t->ck_elem, nck * n)) != MPMG_OK ||
        (rc = dalloc(&t->ck_params, nck)) != MPMG_OK || (rc = dalloc(&t->final_state, kStateFields * n)) != MPMG_OK ||
        (rc = dalloc(&t->final_active, n)) != MPMG_OK || (rc = dalloc(&t->final_elem, n)) != MPMG_OK ||
        (rc = dalloc(&t->final_params, 1)) != MPMG_OK ||
        (rc = dalloc(&t->seg_state, (size_t)K * kStateFields * n)) != MPMG_OK ||
        (rc = dalloc(&t->seg_elem, (size_t)K * n)) != MPMG_OK ||
        (rc = dalloc(&t->seg_active, (size_t)K * n)) != MPMG_OK ||
        (rc = dalloc(&t->seg_perm, (size_t)K * n)) != MPMG_OK ||
        (rc = dalloc(&t->seg_cs, (size_t)K * (ne + 1))) != MPMG_OK ||
        (rc = dalloc(&t->seg_nodes, (size_t)K * kNodeFields * nn)) != MPMG_OK ||
        (rc = dalloc(&t->seg_params, (size_t)K)) != MPMG_OK ||
        (rc = dalloc(&t->adj[0], kStateFields * n)) != MPMG_OK ||
        (rc = dalloc(&t->adj[1], kStateFields * n)) != MPMG_OK || (rc = dalloc(&t->contrib, 16 * n)) != MPMG_OK ||
        (rc = dalloc(&t->cell_adj, 16 * ne)) != MPMG_OK || (rc = dalloc(&t->node_adj, 5 * nn)) != MPMG_OK ||
        (rc = dalloc(&t->theta_part, (size_t)blocks_for(n, kAdjThreads) * kThetaSlots)) != MPMG_OK ||
        (rc = dalloc(&t->theta_acc, kThetaSlots)) != MPMG_OK) {
        mpmg_adj_free(ctx);
        return rc;
    }
    if (ctx->cfg.material == MPMG_G_NONLOCAL_MU2 &&
        ((rc = dalloc(&t->seg_gf, (size_t)K * nn)) != MPMG_OK ||
         (rc = dalloc(&t->seg_ek, (size_t)K * 10 * ne)) != MPMG_OK || (rc = dalloc(&t->gfb, n)) != MPMG_OK ||
         (rc = dalloc(&t->rhs, 4 * ne)) != MPMG_OK || (rc = dalloc(&t->lam, nn)) != MPMG_OK)) {
        mpmg_adj_free(ctx);
        return rc;
    }
    // The forward run: checkpoint, then K ordinary steps (CUDA graphs).
    for (int c = 0; c < t->nck; c++) {
        rc = snapshot(ctx, t->ck_state + (size_t)c * kStateFields * n, t->ck_active + (size_t)c * n,
                      t->ck_elem + (size_t)c * n, t->ck_params + c);
        if (rc != MPMG_OK) return rc;
        const int steps = (c + 1) * K <= nsteps ? K : nsteps - c * K;
        rc = mpmg_step(ctx, steps);
        if (rc != MPMG_OK) return rc;
    }
    rc = snapshot(ctx, t->final_state, t->final_active, t->final_elem, t->final_params);
    if (rc != MPMG_OK) return rc;
    return mpmg_synchronize(ctx);
}

int mpmg_adj_backward(mpmg_ctx *ctx, const double *dl_dx, const double *dl_dy, double *dl_dtheta)
{
    if (ctx == nullptr || dl_dx == nullptr || dl_dy == nullptr || dl_dtheta == nullptr) return MPMG_ERR_INVALID;
    AdjTape *t = ctx->adj;
    if (t == nullptr) {
        mpmg_set_error("no taped forward run (mpmg_adj_forward_tape)");
        return MPMG_ERR_INVALID;
    }
    MPMG_CHECK(cudaSetDevice(ctx->dev));
    cudaStream_t s = ctx->stream;
    const size_t n = ctx->np, ne = ctx->ne, nn = ctx->nn;
    // adjoint of the final state: the loss gradient with respect to x and y
    t->cur = 0;
    MPMG_CHECK(cudaMemsetAsync(t->adj[0], 0, kStateFields * n * sizeof(double), s));
    if (n > 0) {
        MPMG_CHECK(cudaMemcpyAsync(t->adj[0], dl_dx, n * sizeof(double), cudaMemcpyHostToDevice, s));
        MPMG_CHECK(cudaMemcpyAsync(t->adj[0] + n, dl_dy, n * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    MPMG_CHECK(cudaMemsetAsync(t->theta_acc, 0, kThetaSlots * sizeof(double), s));

    AdjStep S = {};
    S.g = fp64::make_geom(ctx);
    S.bc = fp64::make_bc(ctx);
    S.mp = make_params(ctx);
    S.material = ctx->cfg.material;
    S.n = (int)n;
    S.ne = (int)ne;
    S.nn = (int)nn;
    S.dt = ctx->cfg.dt;
    S.mass = ctx->m;
    S.contrib = t->contrib;
    S.cell_adj = t->cell_adj;
    S.node_adj = t->node_adj;
    S.theta_part = t->theta_part;
    S.gfb = t->gfb;
    S.rhs = t->rhs;
    S.lam = t->lam;
    const bool nonlocal = ctx->cfg.material == MPMG_G_NONLOCAL_MU2;
    const int pblocks = blocks_for(n, kAdjThreads);
    int rc;
    for (int c = t->nck - 1; c >= 0; c--) {
        const int len = (c + 1) * t->K <= t->nsteps ? t->K : t->nsteps - c * t->K;
        // run the segment again from its checkpoint, recording each step
        rc = load_state(ctx, t->ck_state + (size_t)c * kStateFields * n, t->ck_active + (size_t)c * n,
                        t->ck_elem + (size_t)c * n, t->ck_params + c);
        if (rc != MPMG_OK) return rc;
        for (int k = 0; k < len; k++) {
            if ((rc = save_state(ctx, t->seg_state + (size_t)k * kStateFields * n)) != MPMG_OK) return rc;
            if ((rc = mpmg_launch_step(ctx)) != MPMG_OK) return rc;
            const int m = (int)(n > ne + 1 ? (n > nn ? n : nn) : (ne + 1 > nn ? ne + 1 : nn));
            save_step_kernel<<<blocks_for(m, 256), 256, 0, s>>>(
                (int)n, (int)ne, (int)nn, ctx->in_element, ctx->active, ctx->perm, ctx->cell_start, ctx->node_m,
                ctx->node_ax, ctx->node_ay, ctx->node_vx, ctx->node_vy, ctx->d_params, t->seg_elem + (size_t)k * n,
                t->seg_active + (size_t)k * n, t->seg_perm + (size_t)k * n, t->seg_cs + (size_t)k * (ne + 1),
                t->seg_nodes + (size_t)k * kNodeFields * nn, t->seg_params + k);
            ctx->launches += 1;
            if (nonlocal) {
                MPMG_CHECK(cudaMemcpyAsync(t->seg_gf + (size_t)k * nn, ctx->node_gf, nn * sizeof(double),
                                           cudaMemcpyDeviceToDevice, s));
                MPMG_CHECK(cudaMemcpyAsync(t->seg_ek + (size_t)k * 10 * ne, ctx->elem_k, 10 * ne * sizeof(double),
                                           cudaMemcpyDeviceToDevice, s));
            }
        }
        // reverse the segment's steps
        for (int k = len - 1; k >= 0; k--) {
            S.state = t->seg_state + (size_t)k * kStateFields * n;
            S.elem = t->seg_elem + (size_t)k * n;
            S.active = t->seg_active + (size_t)k * n;
            S.perm = t->seg_perm + (size_t)k * n;
            S.cell_start = t->seg_cs + (size_t)k * (ne + 1);
            S.nodes = t->seg_nodes + (size_t)k * kNodeFields * nn;
            S.params = t->seg_params + k;
            S.adj_in = t->adj[t->cur];
            S.adj_out = t->adj[1 - t->cur];
            if (n > 0 && nonlocal) {
                // the fluidity's adjoint: gathered to the nodes, then the same
                // symmetric system solved for it (zero start, same tolerance)
                S.gf_nodes = t->seg_gf + (size_t)k * nn;
                adj_nl_pre_kernel<<<pblocks, kAdjThreads, 0, s>>>(S);
                adj_nl_rhs_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(S);
                ctx->launches += 2;
                MPMG_CHECK(cudaGetLastError());
                rc = mpmg_solve_fluidity_system(ctx, t->seg_ek + (size_t)k * 10 * ne, t->rhs, S.nodes, S.cell_start,
                                                t->lam, true);
                if (rc != MPMG_OK) return rc;
            }
            if (n > 0) {
                adj_g2p_kernel<<<pblocks, kAdjThreads, 0, s>>>(S);
                adj_cells_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(S);
                adj_grid_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(S);
                adj_p2g_kernel<<<pblocks, kAdjThreads, 0, s>>>(S);
                adj_theta_kernel<<<1, 32, 0, s>>>(t->theta_part, pblocks, t->theta_acc);
                ctx->launches += 5;
            }
            MPMG_CHECK(cudaGetLastError());
            t->cur = 1 - t->cur;
        }
    }
    // the run's final state again, so that stepping can go on
    if ((rc = load_state(ctx, t->final_state, t->final_active, t->final_elem, t->final_params)) != MPMG_OK)
        return rc;
    double th[kThetaSlots];
    MPMG_CHECK(cudaMemcpyAsync(th, t->theta_acc, sizeof(th), cudaMemcpyDeviceToHost, s));
    MPMG_CHECK(cudaStreamSynchronize(s));
    // fold the elastic constants into E: G = E / (2 (1 + nu)), K = E / (3 (1 - 2 nu)),
    // lambda = K - 2 G / 3
    const double nu = ctx->cfg.mp[MPMG_MP_NU];
    const double dG = 1.0 / (2.0 * (1.0 + nu)), dK = 1.0 / (3.0 * (1.0 - 2.0 * nu));
    t->grad[TH_MU_S] = th[0];
    t->grad[TH_MU_2] = th[1];
    t->grad[TH_I0] = th[2];
    t->grad[TH_E] = th[3] * dG + th[4] * dK + th[5] * (dK - 2.0 / 3.0 * dG);
    t->grad[TH_A] = th[6];
    for (int k = 0; k < TH_COUNT; k++) dl_dtheta[k] = t->grad[k];
    return mpmg_synchronize(ctx);
}

// One parameter's gradient from the last mpmg_adj_backward: 0 mu_s, 1 mu_2,
// 2 I0, 3 E, 4 the nonlocal amplitude A (zero for the local materials).
int mpmg_adj_gradient(mpmg_ctx *ctx, int index, double *out)
{
    if (ctx == nullptr || out == nullptr || index < 0 || index >= TH_ALL) return MPMG_ERR_INVALID;
    if (ctx->adj == nullptr) return MPMG_ERR_INVALID;
    *out = ctx->adj->grad[index];
    return MPMG_OK;
}

// Adjoint of one field of the taped run's initial state (after
// mpmg_adj_backward): x y vx vy v sxx sxy syy Tzz, in particle order.
int mpmg_adj_state(mpmg_ctx *ctx, const char *name, double *host_out)
{
    if (ctx == nullptr || name == nullptr || host_out == nullptr) return MPMG_ERR_INVALID;
    if (ctx->adj == nullptr) return MPMG_ERR_INVALID;
    static const char *names[kStateFields] = {"x", "y", "vx", "vy", "v", "sxx", "sxy", "syy", "Tzz"};
    for (int f = 0; f < kStateFields; f++) {
        if (strcmp(name, names[f]) == 0) {
            MPMG_CHECK(cudaSetDevice(ctx->dev));
            MPMG_CHECK(cudaStreamSynchronize(ctx->stream));
            if (ctx->np)
                MPMG_CHECK(cudaMemcpy(host_out, ctx->adj->adj[ctx->adj->cur] + (size_t)f * ctx->np,
                                      ctx->np * sizeof(double), cudaMemcpyDeviceToHost));
            return MPMG_OK;
        }
    }
    return MPMG_ERR_UNKNOWN_FIELD;
}

}  // extern "C"
