// The explicit USL step on the GPU (reference: explicit_mpm_step_usl_threaded,
// libmpm/process_usl.c:465-592, plus the driver's time_varying_loads tail,
// src/main.c:975 and libmpm/loading.c:34-54).
//
//   keys      element of every particle (WHICH_ELEMENT4, :43-44 and :631-674);
//             advances t and the gravity scalar in the device StepParams
//   bin       stable counting sort of (element, particle) -> per-element
//             particle segments (find_filled_elements, :677-723; mpmg_bin.cu)
//   p2g       one thread per element sums its particles' contributions to
//             its four corners (map_to_grid_explicit_split, :812-910)
//   grid      one thread per node adds the four adjacent elements' corner
//             sums in colour order 0..3, applies the box / square-silo
//             conditions and the nodal update (bc_momentum, bc_force,
//             move_grid_split :596-625)
//   g2p       one thread per particle: velocity and position update, strain
//             rate, volume and the material law (move_particles :914-957,
//             calculate_strainrate :764-808, update_densities :961-970,
//             calculate_stress_threaded)
//
// Shape functions (tent / grad_tent, interpolate.c:23-65) are recomputed in
// registers from the start-of-step position wherever they are needed.  No
// floating-point atomics are used; every sum has a fixed order.
#include "mpmg_fp64_common.cuh"
#include "mpmg_internal.cuh"
#include "mpmg_materials.cuh"

namespace {

using fp64::BcParams;
using fp64::GridGeom;
using fp64::ShapeFns;
using fp64::bc_mask;
using fp64::make_bc;
using fp64::make_geom;
using fp64::shape;

// ---------------------------------------------------------------------------
// keys

__global__ void __launch_bounds__(256) keys_kernel(GridGeom g, float inv_hf, int n, const double *__restrict__ x,
                                                   const double *__restrict__ y, int *__restrict__ in_element,
                                                   int *__restrict__ active, uint32_t *__restrict__ keys,
                                                   uint32_t sentinel, uint32_t *__restrict__ bins, StepParams *sp,
                                                   double dt, int gravity_mode, double gravity_const)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // time_varying_loads (loading.c:34-54) of the previous step's tail, or
        // initial_loads (loading.c:21-30) before the first step; then t += dt
        // (process_usl.c:522).
        double t = sp->t;
        double grav;
        if (gravity_mode == MPMG_GRAVITY_CONSTANT) {
            grav = gravity_const;
        } else if (sp->step_count == 0) {
            grav = 0.0;
        } else if ((0.1 + sp->step_start_time) > t) {
            grav = -9.8 * ((t - sp->step_start_time) / 0.1);
        } else {
            grav = -9.8;
        }
        sp->gravity = grav;
        sp->t = t + dt;
        sp->step_count += 1;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t key = sentinel;
    if (i < n) {
        if (active[i]) {
            int e = mpmg_which_element_fast(x[i], y[i], g.h, g.inv_h, inv_hf, g.xmax, g.ymax,
                                            __double_as_longlong(g.xmax), __double_as_longlong(g.ymax), g.Ex,
                                            g.Ey);
            in_element[i] = e;
            if (e < 0) {
                active[i] = 0;   // process_usl.c:660-666: outside the grid for good
            } else {
                key = (uint32_t)e;
            }
        }
        keys[i] = key;
    }
    mpmg_bin_count(key, i < n, sentinel, (uint32_t)i >> 5, bins);
}

// ---------------------------------------------------------------------------
// p2g: per-element corner sums over the element's particle segment.
//
// The corner weights are bilinear in the local coordinates (x, y):
// N = {(1-x)(1-y), x(1-y), xy, (1-x)y}, dN/dx h = {-(1-y), 1-y, y, -y},
// dN/dy h = {-(1-x), -x, x, 1-x}.  So the element's four corner sums of a
// particle quantity q follow from four moments, A = sum q, X = sum x q,
// Y = sum y q, Z = sum xy q:  corners A - X - Y + Z, X - Z, Z, Y - Z; and the
// eight internal-force sums from seven moments of the stress terms.  The
// particle loop then costs 29 FP64 operations instead of about 60 (GB300
// issues FP64 at 1/64 of the FP32 rate, and this loop is bound by it); the
// body force (m g per corner), the 1/h of the gradients and the corners are
// formed once per element.  The roundings differ from per-corner sums by a
// few ulps of the element's totals.

__global__ void __launch_bounds__(128) p2g_cells_kernel(
    GridGeom g, int ne, const int *__restrict__ cell_start, const uint32_t *__restrict__ slots,
    uint32_t *__restrict__ perm,
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ m,
    const double *__restrict__ vx, const double *__restrict__ vy, const double *__restrict__ v,
    const double *__restrict__ sxx, const double *__restrict__ sxy, const double *__restrict__ syy,
    const StepParams *__restrict__ sp, double *__restrict__ cell_sums)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int k0 = cell_start[e], k1 = cell_start[e + 1];
    if (k0 == k1) return;
    mpmg_order_segment(slots, perm, nullptr, k0, k1);   // ascending particle index, as the reference's lists
    const int ci = e % g.Ex, cj = e / g.Ex;
    const double cx = ci, cy = cj;   // the element's column and row (element.c:10-19)
    // moments [A, X, Y, Z] of m, m vx, m vy; stress-term moments
    double mm[4] = {0, 0, 0, 0}, mx[4] = {0, 0, 0, 0}, my[4] = {0, 0, 0, 0};
    double P0 = 0, Py0 = 0, P1 = 0, Px1 = 0, Py1 = 0, P2 = 0, Px2 = 0;
    for (int k = k0; k < k1; k++) {
        const int i = (int)perm[k];
        const double xl = mpmg_local_coord_fma(x[i], cx, g.inv_h);
        const double yl = mpmg_local_coord_fma(y[i], cy, g.inv_h);
        const double xy = xl * yl;
        const double pm = m[i];
        const double pmx = vx[i] * pm, pmy = vy[i] * pm;
        const double vol = v[i];
        const double s0 = -sxx[i] * vol, s1 = -sxy[i] * vol, s2 = -syy[i] * vol;
        mm[0] += pm;
        mm[1] = fma(xl, pm, mm[1]);
        mm[2] = fma(yl, pm, mm[2]);
        mm[3] = fma(xy, pm, mm[3]);
        mx[0] += pmx;
        mx[1] = fma(xl, pmx, mx[1]);
        mx[2] = fma(yl, pmx, mx[2]);
        mx[3] = fma(xy, pmx, mx[3]);
        my[0] += pmy;
        my[1] = fma(xl, pmy, my[1]);
        my[2] = fma(yl, pmy, my[2]);
        my[3] = fma(xy, pmy, my[3]);
        P0 += s0;
        Py0 = fma(yl, s0, Py0);
        P1 += s1;
        Px1 = fma(xl, s1, Px1);
        Py1 = fma(yl, s1, Py1);
        P2 += s2;
        Px2 = fma(xl, s2, Px2);
    }
    // corners BL, BR, TR, TL (process_usl.c:140-143)
    double cm[4], cmx[4], cmy[4];
    cm[0] = (mm[0] - mm[1]) - (mm[2] - mm[3]);
    cm[1] = mm[1] - mm[3];
    cm[2] = mm[3];
    cm[3] = mm[2] - mm[3];
    cmx[0] = (mx[0] - mx[1]) - (mx[2] - mx[3]);
    cmx[1] = mx[1] - mx[3];
    cmx[2] = mx[3];
    cmx[3] = mx[2] - mx[3];
    cmy[0] = (my[0] - my[1]) - (my[2] - my[3]);
    cmy[1] = my[1] - my[3];
    cmy[2] = my[3];
    cmy[3] = my[2] - my[3];
    const double ih = g.inv_h;
    const double a0 = P0 - Py0, a1 = P1 - Px1, b1 = P1 - Py1, b2 = P2 - Px2;
    double cfx[4], cfy[4];
    cfx[0] = -(a0 + a1) * ih;
    cfx[1] = (a0 - Px1) * ih;
    cfx[2] = (Py0 + Px1) * ih;
    cfx[3] = (a1 - Py0) * ih;
    // body force bx is zero (loading.c:48); by = g acts on each corner's mass
    const double grav = sp->gravity;
    cfy[0] = fma(grav, cm[0], -(b1 + b2) * ih);
    cfy[1] = fma(grav, cm[1], (b1 - Px2) * ih);
    cfy[2] = fma(grav, cm[2], (Py1 + Px2) * ih);
    cfy[3] = fma(grav, cm[3], (b2 - Py1) * ih);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        cell_sums[(size_t)(c * 5 + 0) * ne + e] = cm[c];
        cell_sums[(size_t)(c * 5 + 1) * ne + e] = cmx[c];
        cell_sums[(size_t)(c * 5 + 2) * ne + e] = cmy[c];
        cell_sums[(size_t)(c * 5 + 3) * ne + e] = cfx[c];
        cell_sums[(size_t)(c * 5 + 4) * ne + e] = cfy[c];
    }
}

// ---------------------------------------------------------------------------
// grid: finish P2G per node, boundary conditions, nodal update.

__global__ void __launch_bounds__(256) grid_kernel(
    GridGeom g, BcParams bc, int ne, const int *__restrict__ cell_start,
    const double *__restrict__ cell_sums, const StepParams *__restrict__ sp, double dt,
    double *__restrict__ node_m, double *__restrict__ node_ax, double *__restrict__ node_ay,
    double *__restrict__ node_vx, double *__restrict__ node_vy, double *__restrict__ node_mx,
    double *__restrict__ node_my, double *__restrict__ node_fx, double *__restrict__ node_fy)
{
    const int nn = g.Nx * g.Ny;
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int i = n % g.Nx, j = n / g.Nx;
    double sum[5] = {0, 0, 0, 0, 0};
    // Colour c = 2 * (row % 2) + (col % 2) (process_usl.c:158); the four
    // elements around a node have the four colours, summed in order 0..3.
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        int e = cj * g.Ex + ci;
        if (cell_start[e] == cell_start[e + 1]) continue;
        int corner = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
#pragma unroll
        for (int f = 0; f < 5; f++) sum[f] += cell_sums[(size_t)(corner * 5 + f) * ne + e];
    }
    double m = sum[0], mx = sum[1], my = sum[2], fx = sum[3], fy = sum[4];
    bool bx, by;
    bc_mask(bc, g, i, j, sp->t, bx, by);
    if (bx) { mx = 0; fx = 0; }
    if (by) { my = 0; fy = 0; }
    double ax = 0, ay = 0, vxn = 0, vyn = 0;
    if (m > MPMG_TOL) {
        // one division: the four quotients by m differ from IEEE division
        // by at most an ulp
        const double inv_m = 1.0 / m;
        ax = fx * inv_m;
        ay = fy * inv_m;
        mx += dt * fx;
        my += dt * fy;
        vxn = mx * inv_m;
        vyn = my * inv_m;
    }
    node_m[n] = m;
    node_ax[n] = ax;
    node_ay[n] = ay;
    node_vx[n] = vxn;
    node_vy[n] = vyn;
    if (node_mx != nullptr) {
        node_mx[n] = mx;
        node_my[n] = my;
        node_fx[n] = fx;
        node_fy[n] = fy;
    }
}

// ---------------------------------------------------------------------------
// g2p + material

struct G2PArgs {
    GridGeom g;
    int n;
    double dt;
    mat::Elastic el;
    mat::Mu2Params mu2;
    mat::NonlocalParams nl;
    const int *in_element;
    const int *active;
    const double *node_ax, *node_ay, *node_vx, *node_vy;
    double *x, *y, *vx, *vy, *ux, *uy, *v, *m;
    double *sxx, *sxy, *syy, *Tzz;
    double *st0, *st1, *st3, *st4, *st5, *st6, *st9, *st10;
    double *ax, *ay, *exx, *exy, *eyy, *wxy, *xl_out, *yl_out;
    // g_nonlocal_mu2: the trial stress the stress update reads after the
    // fluidity solve, 5 per particle, value-major (p_d, t0xx, t0xy, t0yy, tau)
    double *trial;
};

// G2P phases.  USL (process_usl.c:465-592) runs them all in one pass; MUSL
// (process_usl.c:284-462) runs the move first, maps the moved particles'
// momentum to the nodes again (p2g_momentum_kernel, node_velocity_kernel),
// then the strain phase with the nodal velocities of that second projection.
enum { G2P_FULL = 0, G2P_MOVE = 1, G2P_STRAIN = 2 };

// The in-plane local returns on particle i (mat::plane_return): szz in
// state[1] (dp_ri_mt.c:27, g_local_mu2_plane_strain.c:43), beta in state[5],
// gammap in state[9], gammadotp in state[10].
template <int MATERIAL>
__device__ __forceinline__ void plane_return_particle(const G2PArgs &A, int i, double vol, double exx,
                                                      double exy, double eyy, double wxy)
{
    constexpr bool trial3d = MATERIAL != MPMG_G_LOCAL_MU2_TRUE_2D;
    constexpr bool mu_i = MATERIAL != MPMG_DP_RI_MT;
    constexpr bool beta = MATERIAL != MPMG_DP_RI_MT;
    const mat::ReturnParams rp = {A.mu2.mu_s, A.mu2.mu_2, A.mu2.I0, A.mu2.grains_rho, A.mu2.grains_d,
                                  A.mu2.rho_critical};
    double sxx = A.sxx[i], sxy = A.sxy[i], syy = A.syy[i];
    double szz = trial3d ? A.st1[i] : 0.0, b = beta ? A.st5[i] : 0.0;
    double gp = A.st9[i], gdp;
    mat::plane_return<trial3d, mu_i, beta>(A.el, rp, A.m[i], vol, exx, exy, eyy, wxy, sxx, sxy, syy, szz, b,
                                           gp, gdp);
    A.sxx[i] = sxx;
    A.sxy[i] = sxy;
    A.syy[i] = syy;
    if (trial3d) A.st1[i] = szz;
    if (beta) A.st5[i] = b;
    A.st9[i] = gp;
    A.st10[i] = gdp;
}

// g_local_mu2_reverse on particle i: beta in state[5], gammap in state[9],
// gammadotp in state[10] (g_local_mu2_reverse.c:57-64).
__device__ __forceinline__ void reverse_particle(const G2PArgs &A, int i, double vol, double exx, double exy,
                                                 double eyy, double wxy)
{
    double sxx = A.sxx[i], sxy = A.sxy[i], syy = A.syy[i], b = A.st5[i], gp = A.st9[i], gdp = A.st10[i];
    mat::g_local_mu2_reverse(A.el, A.mu2, A.m[i], vol, exx, exy, eyy, wxy, sxx, sxy, syy, b, gp, gdp);
    A.sxx[i] = sxx;
    A.sxy[i] = sxy;
    A.syy[i] = syy;
    A.st5[i] = b;
    A.st9[i] = gp;
    A.st10[i] = gdp;
}

template <int MATERIAL, int PHASE>
__global__ void __launch_bounds__(256) g2p_kernel(G2PArgs A)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || !A.active[i]) return;
    const GridGeom &g = A.g;
    const int e = A.in_element[i];
    const int ci = e % g.Ex, cj = e / g.Ex;
    const int n0 = cj * g.Nx + ci;
    const int nd[4] = {n0, n0 + 1, n0 + 1 + g.Nx, n0 + g.Nx};
    double xl, yl;
    if (PHASE == G2P_STRAIN) {
        // the start-of-step local coordinates the move phase kept
        xl = A.xl_out[i];
        yl = A.yl_out[i];
    } else {
        xl = mpmg_local_coord_fma(A.x[i], (double)ci, g.inv_h);
        yl = mpmg_local_coord_fma(A.y[i], (double)cj, g.inv_h);
    }
    const ShapeFns f = shape(xl, yl, g.inv_h);
    const double dt = A.dt;

    double nvx[4], nvy[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        nvx[a] = A.node_vx[nd[a]];
        nvy[a] = A.node_vy[nd[a]];
    }
    if (PHASE != G2P_STRAIN) {
        // move_particles_explicit_usl_split (process_usl.c:914-957); light
        // nodes (m <= 1e-10) carry zero acceleration and velocity.
        double xtt = 0, ytt = 0, dux = 0, duy = 0;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            xtt += f.s[a] * A.node_ax[nd[a]];
            ytt += f.s[a] * A.node_ay[nd[a]];
            dux += f.s[a] * nvx[a];
            duy += f.s[a] * nvy[a];
        }
        A.vx[i] += dt * xtt;
        A.vy[i] += dt * ytt;
        dux *= dt;
        duy *= dt;
        A.x[i] += dux;
        A.y[i] += duy;
        A.ux[i] += dux;
        A.uy[i] += duy;
        if (A.ax != nullptr) {
            A.ax[i] = xtt;
            A.ay[i] = ytt;
        }
        if (A.xl_out != nullptr) {
            A.xl_out[i] = xl;
            A.yl_out[i] = yl;
        }
        if (PHASE == G2P_MOVE) return;
    }
    // calculate_strainrate_split (process_usl.c:796-803): the sums of
    // grad N_a v_a, with h grad N = ((-oy, -ox), (oy, -a), (b, a), (-b, ox))
    // (a, b the local coordinates), grouped by node differences and scaled
    // by 1 / h once (the same sums in fewer FP64 operations, the pipe that
    // bounds this kernel)
    const double ox = 1 - xl, oy = 1 - yl;
    const double sxv = fma(oy, nvx[1] - nvx[0], yl * (nvx[2] - nvx[3]));   // h sum gx vx
    const double syv = fma(oy, nvy[1] - nvy[0], yl * (nvy[2] - nvy[3]));   // h sum gx vy
    const double txv = fma(ox, nvx[3] - nvx[0], xl * (nvx[2] - nvx[1]));   // h sum gy vx
    const double tyv = fma(ox, nvy[3] - nvy[0], xl * (nvy[2] - nvy[1]));   // h sum gy vy
    const double exx = sxv * g.inv_h, eyy = tyv * g.inv_h;
    const double half_inv_h = 0.5 * g.inv_h;
    const double exy = half_inv_h * (txv + syv);
    const double wxy = half_inv_h * (txv - syv);
    // update_particle_densities_split (process_usl.c:961-970)
    double vol = A.v[i] * mat::exp_small(dt * (exx + eyy));
    A.v[i] = vol;
    if (A.exx != nullptr) {
        A.exx[i] = exx;
        A.exy[i] = exy;
        A.eyy[i] = eyy;
        A.wxy[i] = wxy;
    }

    if (MATERIAL == MPMG_ISOLIN) {
        double sxx = A.sxx[i], sxy = A.sxy[i], syy = A.syy[i];
        mat::isolin(A.el, exx, exy, eyy, wxy, sxx, sxy, syy);
        A.sxx[i] = sxx;
        A.sxy[i] = sxy;
        A.syy[i] = syy;
    } else if (MATERIAL == MPMG_G_LOCAL_MU2) {
        double Txx = A.sxx[i], Txy = A.sxy[i], Tyy = A.syy[i], Tzz = A.Tzz[i];
        double gp = A.st9[i], gdp;
        mat::g_local_mu2(A.el, A.mu2, A.m[i], vol, exx, exy, eyy, wxy, Txx, Txy, Tyy, Tzz, gp, gdp);
        A.sxx[i] = Txx;
        A.sxy[i] = Txy;
        A.syy[i] = Tyy;
        A.Tzz[i] = Tzz;
        A.st9[i] = gp;
        A.st10[i] = gdp;
    } else if (MATERIAL == MPMG_DP_RI_MT || MATERIAL == MPMG_G_LOCAL_MU2_PLANE_STRAIN ||
               MATERIAL == MPMG_G_LOCAL_MU2_TRUE_2D) {
        plane_return_particle<MATERIAL>(A, i, vol, exx, exy, eyy, wxy);
    } else if (MATERIAL == MPMG_G_LOCAL_MU2_REVERSE) {
        reverse_particle(A, i, vol, exx, exy, eyy, wxy);
    } else if (MATERIAL == MPMG_G_LOCAL_MU2_EXT) {
        // first phase only; the stress waits for the nodal Laplacian
        double mu_t = A.st0[i], gfl;
        mat::ext_local_fluidity(A.mu2, A.sxx[i], A.syy[i], A.st10[i], mu_t, gfl);
        A.st0[i] = mu_t;
        A.st4[i] = gfl;
    } else if (MATERIAL == MPMG_G_NONLOCAL_MU2) {
        double p_tr, t0xx, t0xy, t0yy, tau_tr, dense, gfl, xisq;
        mat::nonlocal_mu2_trial(A.el, exx, exy, eyy, wxy, A.sxx[i], A.sxy[i], A.syy[i], p_tr, t0xx, t0xy,
                                t0yy, tau_tr);
        mat::nonlocal_mu2_bulk(A.el, A.mu2, A.m[i], vol, p_tr, tau_tr, dense, gfl, xisq);
        A.st0[i] = dense;
        A.st5[i] = gfl;
        A.st6[i] = xisq;
        const size_t n = (size_t)A.n;
        A.trial[i] = dense != 0 ? p_tr : 0.0;
        A.trial[n + i] = t0xx;
        A.trial[2 * n + i] = t0xy;
        A.trial[3 * n + i] = t0yy;
        A.trial[4 * n + i] = tau_tr;
    }
    // MPMG_G_NONLOCAL computes its bulk fluidity over every particle in the
    // fluidity phase (g_nonlocal.c:306-352).
}

// g_local_mu2_ext's second phase (g_local_mu2_ext.c:232-265): per element,
// each particle's -v gflocal |grad N_j|^2 summed per corner in the binned
// order of the step, with the start-of-step shape-function gradients.
__global__ void __launch_bounds__(128) ext_cells_kernel(
    int ne, double inv_h, const int *__restrict__ cell_start, const uint32_t *__restrict__ perm,
    const double *__restrict__ xl, const double *__restrict__ yl, const double *__restrict__ v,
    const double *__restrict__ gflocal, double *__restrict__ cell_sums)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int k0 = cell_start[e], k1 = cell_start[e + 1];
    double acc[4] = {0, 0, 0, 0};
    for (int k = k0; k < k1; k++) {
        const int i = (int)perm[k];
        const ShapeFns f = shape(xl[i], yl[i], inv_h);
        const double q = mat::mul(-v[i], gflocal[i]);
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const double sj = mat::add(mat::mul(f.gx[a], f.gx[a]), mat::mul(f.gy[a], f.gy[a]));
            acc[a] = mat::add(acc[a], mat::mul(q, sj));
        }
    }
#pragma unroll
    for (int a = 0; a < 4; a++) cell_sums[(size_t)a * ne + e] = acc[a];
}

// The nodal sums of ext_cells_kernel's corners in colour order.
__global__ void __launch_bounds__(256) ext_nodes_kernel(GridGeom g, int ne, const double *__restrict__ cell_sums,
                                                        double *__restrict__ d2)
{
    const int nn = g.Nx * g.Ny;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int i = n % g.Nx, j = n / g.Nx;
    double sum = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        const int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        const int e = cj * g.Ex + ci;
        const int corner = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
        sum = mat::add(sum, cell_sums[(size_t)corner * ne + e]);
    }
    d2[n] = sum;
}

// g_local_mu2_ext's gf and gammadotp correction (g_local_mu2_ext.c:268-290)
// and the stress (mat::ext_stress).
__global__ void __launch_bounds__(256) ext_stress_kernel(G2PArgs A, const double *__restrict__ d2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || !A.active[i]) return;
    const GridGeom &g = A.g;
    const int e = A.in_element[i];
    const int ci = e % g.Ex, cj = e / g.Ex;
    const int n0 = cj * g.Nx + ci;
    const int nd[4] = {n0, n0 + 1, n0 + 1 + g.Nx, n0 + g.Nx};
    double gf = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) gf = mat::add(gf, mat::mul(0.25, d2[nd[a]]));
    double mu_t = A.st0[i], gdp = A.st10[i];
    const double Ad = A.mu2.A, d = A.mu2.grains_d;
    gf = mat::mul(mat::mul(mat::mul(mat::mul(mat::mul(Ad, Ad), d), d), mu_t), gf);
    if (mu_t > A.mu2.mu_s) gdp = mat::sub(gdp, mat::dvd(gf, fabs(mat::sub(mu_t, A.mu2.mu_s))));
    if (gdp < 0) gdp = 0;
    A.st3[i] = gf;
    double sxx = A.sxx[i], sxy = A.sxy[i], syy = A.syy[i], beta = A.st5[i], gp = A.st9[i];
    mat::ext_stress(A.el, A.mu2, A.nl.E, A.nl.nu, A.m[i], A.v[i], A.exx[i], A.exy[i], A.eyy[i], A.wxy[i], sxx, sxy,
                    syy, mu_t, beta, gp, gdp);
    A.sxx[i] = sxx;
    A.sxy[i] = sxy;
    A.syy[i] = syy;
    A.st0[i] = mu_t;
    A.st5[i] = beta;
    A.st9[i] = gp;
    A.st10[i] = gdp;
}

// MUSL's second projection (process_usl.c:424-431): per element, the moved
// particles' mass and momentum with their start-of-step shape functions, in
// the binned order of the step (perm is already ordered by the P2G).
__global__ void __launch_bounds__(128) p2g_momentum_kernel(
    int ne, double inv_h, const int *__restrict__ cell_start, const uint32_t *__restrict__ perm,
    const double *__restrict__ xl, const double *__restrict__ yl, const double *__restrict__ m,
    const double *__restrict__ vx, const double *__restrict__ vy, double *__restrict__ cell_sums)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int k0 = cell_start[e], k1 = cell_start[e + 1];
    if (k0 == k1) return;
    double acc[4][3];
#pragma unroll
    for (int a = 0; a < 4; a++) acc[a][0] = acc[a][1] = acc[a][2] = 0.0;
    for (int k = k0; k < k1; k++) {
        const int i = (int)perm[k];
        const ShapeFns f = shape(xl[i], yl[i], inv_h);
        const double pm = m[i], pmx = vx[i] * pm, pmy = vy[i] * pm;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            acc[a][0] += f.s[a] * pm;
            acc[a][1] += f.s[a] * pmx;
            acc[a][2] += f.s[a] * pmy;
        }
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int q = 0; q < 3; q++) cell_sums[(size_t)(a * 3 + q) * ne + e] = acc[a][q];
}

// MUSL nodal velocities of the second projection (process_usl.c:433-447):
// v = p / m where m > 1e-10, else 0.  The reference zeroes the constrained
// momenta only after forming v, so the boundary conditions do not reach v;
// the zeroed momenta are what it keeps in the nodes (node_mx, node_my).
__global__ void __launch_bounds__(256) node_velocity_kernel(
    GridGeom g, BcParams bc, int ne, const int *__restrict__ cell_start, const double *__restrict__ cell_sums,
    const StepParams *__restrict__ sp, double *__restrict__ node_m, double *__restrict__ node_vx,
    double *__restrict__ node_vy, double *__restrict__ node_mx, double *__restrict__ node_my)
{
    const int nn = g.Nx * g.Ny;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int i = n % g.Nx, j = n / g.Nx;
    double sum[3] = {0, 0, 0};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int ci = ((i & 1) == (c & 1)) ? i : i - 1;
        const int cj = ((j & 1) == (c >> 1)) ? j : j - 1;
        if (ci < 0 || cj < 0 || ci >= g.Ex || cj >= g.Ey) continue;
        const int e = cj * g.Ex + ci;
        if (cell_start[e] == cell_start[e + 1]) continue;
        const int corner = (ci == i) ? ((cj == j) ? 0 : 3) : ((cj == j) ? 1 : 2);
#pragma unroll
        for (int q = 0; q < 3; q++) sum[q] += cell_sums[(size_t)(corner * 3 + q) * ne + e];
    }
    const double m = sum[0];
    double vxn = 0, vyn = 0;
    if (m > MPMG_TOL) {
        vxn = sum[1] / m;
        vyn = sum[2] / m;
    }
    node_m[n] = m;
    node_vx[n] = vxn;
    node_vy[n] = vyn;
    if (node_mx != nullptr) {
        bool bx, by;
        bc_mask(bc, g, i, j, sp->t, bx, by);
        node_mx[n] = bx ? 0.0 : sum[1];
        node_my[n] = by ? 0.0 : sum[2];
    }
}

__global__ void material_only_kernel(G2PArgs A, int material)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || !A.active[i]) return;
    double exx = A.exx[i], exy = A.exy[i], eyy = A.eyy[i], wxy = A.wxy[i];
    if (material == MPMG_ISOLIN) {
        double sxx = A.sxx[i], sxy = A.sxy[i], syy = A.syy[i];
        mat::isolin(A.el, exx, exy, eyy, wxy, sxx, sxy, syy);
        A.sxx[i] = sxx;
        A.sxy[i] = sxy;
        A.syy[i] = syy;
    } else if (material == MPMG_DP_RI_MT) {
        plane_return_particle<MPMG_DP_RI_MT>(A, i, A.v[i], exx, exy, eyy, wxy);
    } else if (material == MPMG_G_LOCAL_MU2_PLANE_STRAIN) {
        plane_return_particle<MPMG_G_LOCAL_MU2_PLANE_STRAIN>(A, i, A.v[i], exx, exy, eyy, wxy);
    } else if (material == MPMG_G_LOCAL_MU2_TRUE_2D) {
        plane_return_particle<MPMG_G_LOCAL_MU2_TRUE_2D>(A, i, A.v[i], exx, exy, eyy, wxy);
    } else if (material == MPMG_G_LOCAL_MU2_REVERSE) {
        reverse_particle(A, i, A.v[i], exx, exy, eyy, wxy);
    } else {
        double Txx = A.sxx[i], Txy = A.sxy[i], Tyy = A.syy[i], Tzz = A.Tzz[i];
        double gp = A.st9[i], gdp;
        mat::g_local_mu2(A.el, A.mu2, A.m[i], A.v[i], exx, exy, eyy, wxy, Txx, Txy, Tyy, Tzz, gp, gdp);
        A.sxx[i] = Txx;
        A.sxy[i] = Txy;
        A.syy[i] = Tyy;
        A.Tzz[i] = Tzz;
        A.st9[i] = gp;
        A.st10[i] = gdp;
    }
}

G2PArgs make_g2p_args(mpmg_ctx *ctx)
{
    G2PArgs A;
    const mpmg_config &c = ctx->cfg;
    A.g = make_geom(ctx);
    A.n = (int)ctx->np;
    A.dt = c.dt;
    A.el.G = ctx->G;
    A.el.twoG = 2.0 * ctx->G;
    A.el.K = ctx->K;
    A.el.lambda = ctx->lambda;
    A.el.dt = c.dt;
    A.el.inv_G = 1.0 / ctx->G;
    A.el.inv_dt = 1.0 / c.dt;
    A.el.Gdt = ctx->G * c.dt;
    A.el.inv_Gdt = 1.0 / A.el.Gdt;
    A.mu2.mu_s = c.mp[MPMG_MP_MU_S];
    A.mu2.mu_2 = c.mp[MPMG_MP_MU_2];
    A.mu2.I0 = c.mp[MPMG_MP_I0];
    A.mu2.grains_rho = c.mp[MPMG_MP_GRAINS_RHO];
    A.mu2.grains_d = c.mp[MPMG_MP_GRAINS_D];
    A.mu2.rho_critical = c.mp[MPMG_MP_RHO_CRITICAL];
    A.mu2.A = c.mp[MPMG_MP_A];
    A.mu2.inv_grains_rho = 1.0 / A.mu2.grains_rho;
    A.mu2.inv_grains_d = 1.0 / A.mu2.grains_d;
    A.mu2.rho_lo = A.mu2.rho_critical * (1.0 - 0x1p-47);
    A.mu2.rho_hi = A.mu2.rho_critical * (1.0 + 0x1p-47);
    A.mu2.AAdd = ((A.mu2.A * A.mu2.A) * A.mu2.grains_d) * A.mu2.grains_d;
    A.mu2.inv_AAdd = 1.0 / A.mu2.AAdd;
    A.mu2.alpha_c = (((ctx->G * A.mu2.I0) * c.dt) / A.mu2.grains_d) / sqrt(A.mu2.grains_rho);
    A.mu2.GI0dt = (ctx->G * A.mu2.I0) * c.dt;
    A.nl.E = c.mp[MPMG_MP_E];
    A.nl.nu = c.mp[MPMG_MP_NU];
    A.nl.mu_s = c.mp[MPMG_MP_MU_S];
    A.nl.grains_rho = c.mp[MPMG_MP_GRAINS_RHO];
    A.nl.B = c.mp[MPMG_MP_B];
    A.nl.A = c.mp[MPMG_MP_A];
    A.nl.grains_d = c.mp[MPMG_MP_GRAINS_D];
    A.nl.cohesion = c.mp[MPMG_MP_COHESION];
    A.in_element = ctx->in_element;
    A.active = ctx->active;
    A.node_ax = ctx->node_ax;
    A.node_ay = ctx->node_ay;
    A.node_vx = ctx->node_vx;
    A.node_vy = ctx->node_vy;
    A.x = ctx->x; A.y = ctx->y; A.vx = ctx->vx; A.vy = ctx->vy; A.ux = ctx->ux; A.uy = ctx->uy;
    A.v = ctx->v; A.m = ctx->m;
    A.sxx = ctx->sxx; A.sxy = ctx->sxy; A.syy = ctx->syy; A.Tzz = ctx->Tzz;
    A.st0 = ctx->state[0]; A.st1 = ctx->state[1]; A.st3 = ctx->state[3]; A.st4 = ctx->state[4]; A.st5 = ctx->state[5];
    A.st6 = ctx->state[6]; A.st9 = ctx->state[9]; A.st10 = ctx->state[10];
    A.ax = ctx->ax; A.ay = ctx->ay;
    A.exx = ctx->exx; A.exy = ctx->exy; A.eyy = ctx->eyy; A.wxy = ctx->wxy;
    A.xl_out = ctx->xl; A.yl_out = ctx->yl;
    A.trial = ctx->nl_trial;
    return A;
}

inline int blocks_for(size_t n, int threads)
{
    size_t b = (n + (size_t)threads - 1) / (size_t)threads;
    return (int)(b > 0 ? b : 1);
}

}  // namespace

int mpmg_launch_step(mpmg_ctx *ctx)
{
    cudaStream_t s = ctx->stream;
    const mpmg_config &c = ctx->cfg;
    const GridGeom g = make_geom(ctx);
    const int n = (int)ctx->np;
    const int ne = (int)ctx->ne;
    const int nn = (int)ctx->nn;

    mpmg_phase_begin(ctx, PH_KEYS);
    keys_kernel<<<blocks_for(n, 256), 256, 0, s>>>(g, (float)ctx->inv_h, n, ctx->x, ctx->y, ctx->in_element,
                                                   ctx->active,
                                                   ctx->keys, (uint32_t)ne, ctx->bin.counts, ctx->d_params,
                                                   c.dt, c.gravity_mode, c.gravity);
    ctx->launches += 1;
    mpmg_phase_end(ctx, PH_KEYS);

    mpmg_phase_begin(ctx, PH_SORT);
    int rc = mpmg_bin_scan_scatter(ctx, ctx->keys, ctx->sorted_keys);
    if (rc != MPMG_OK) return rc;
    mpmg_phase_end(ctx, PH_SORT);

    mpmg_phase_begin(ctx, PH_P2G);
    p2g_cells_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(
        g, ne, ctx->cell_start, ctx->bin.slots, ctx->perm, ctx->x, ctx->y, ctx->m, ctx->vx, ctx->vy, ctx->v, ctx->sxx,
        ctx->sxy, ctx->syy, ctx->d_params, ctx->cell_sums);
    ctx->launches += 1;
    mpmg_phase_end(ctx, PH_P2G);

    mpmg_phase_begin(ctx, PH_GRID);
    grid_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(
        g, make_bc(ctx), ne, ctx->cell_start, ctx->cell_sums, ctx->d_params, c.dt, ctx->node_m,
        ctx->node_ax, ctx->node_ay, ctx->node_vx, ctx->node_vy, ctx->node_mx, ctx->node_my,
        ctx->node_fx, ctx->node_fy);
    ctx->launches += 1;
    mpmg_phase_end(ctx, PH_GRID);

    mpmg_phase_begin(ctx, PH_G2P);
    G2PArgs A = make_g2p_args(ctx);
    if (c.scheme == MPMG_SCHEME_MUSL) {
        // move, second projection of the moved momentum, then strain
        // the move phase does not depend on the material
        g2p_kernel<MPMG_ISOLIN, G2P_MOVE><<<blocks_for(n, 256), 256, 0, s>>>(A);
        p2g_momentum_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(ne, ctx->inv_h, ctx->cell_start, ctx->perm, ctx->xl,
                                                                ctx->yl, ctx->m, ctx->vx, ctx->vy, ctx->cell_sums);
        node_velocity_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(g, make_bc(ctx), ne, ctx->cell_start,
                                                                 ctx->cell_sums, ctx->d_params, ctx->node_m,
                                                                 ctx->node_vx, ctx->node_vy, ctx->node_mx,
                                                                 ctx->node_my);
        switch (c.material) {
        case MPMG_ISOLIN: g2p_kernel<MPMG_ISOLIN, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A); break;
        case MPMG_DP_RI_MT: g2p_kernel<MPMG_DP_RI_MT, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A); break;
        case MPMG_G_LOCAL_MU2_PLANE_STRAIN:
            g2p_kernel<MPMG_G_LOCAL_MU2_PLANE_STRAIN, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_TRUE_2D:
            g2p_kernel<MPMG_G_LOCAL_MU2_TRUE_2D, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_REVERSE:
            g2p_kernel<MPMG_G_LOCAL_MU2_REVERSE, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        default: g2p_kernel<MPMG_G_LOCAL_MU2, G2P_STRAIN><<<blocks_for(n, 256), 256, 0, s>>>(A); break;
        }
        ctx->launches += 4;
    } else {
        switch (c.material) {
        case MPMG_ISOLIN:
            g2p_kernel<MPMG_ISOLIN, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2:
            g2p_kernel<MPMG_G_LOCAL_MU2, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_DP_RI_MT:
            g2p_kernel<MPMG_DP_RI_MT, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_PLANE_STRAIN:
            g2p_kernel<MPMG_G_LOCAL_MU2_PLANE_STRAIN, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_TRUE_2D:
            g2p_kernel<MPMG_G_LOCAL_MU2_TRUE_2D, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_REVERSE:
            g2p_kernel<MPMG_G_LOCAL_MU2_REVERSE, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        case MPMG_G_LOCAL_MU2_EXT:
            g2p_kernel<MPMG_G_LOCAL_MU2_EXT, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            ext_cells_kernel<<<blocks_for(ne, 128), 128, 0, s>>>(ne, ctx->inv_h, ctx->cell_start, ctx->perm, ctx->xl,
                                                                ctx->yl, ctx->v, ctx->state[4], ctx->cell_sums);
            ext_nodes_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(g, ne, ctx->cell_sums, ctx->node_gf);
            ext_stress_kernel<<<blocks_for(n, 256), 256, 0, s>>>(A, ctx->node_gf);
            ctx->launches += 3;
            break;
        case MPMG_G_NONLOCAL_MU2:
            g2p_kernel<MPMG_G_NONLOCAL_MU2, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        default:
            g2p_kernel<MPMG_G_NONLOCAL, G2P_FULL><<<blocks_for(n, 256), 256, 0, s>>>(A);
            break;
        }
        ctx->launches += 1;
    }
    mpmg_phase_end(ctx, PH_G2P);
    MPMG_CHECK(cudaGetLastError());

    if (c.material == MPMG_G_NONLOCAL_MU2 || c.material == MPMG_G_NONLOCAL || c.material == MPMG_G_NONLOCAL_AVG) {
        mpmg_phase_begin(ctx, PH_FLUIDITY);
        rc = mpmg_launch_fluidity(ctx);
        if (rc != MPMG_OK) return rc;
        mpmg_phase_end(ctx, PH_FLUIDITY);
    }
    return MPMG_OK;
}

int mpmg_launch_material_only(mpmg_ctx *ctx)
{
    G2PArgs A = make_g2p_args(ctx);
    if (A.exx == nullptr) {
        mpmg_set_error("material-only update needs store_transients (strain-rate inputs)");
        return MPMG_ERR_INVALID;
    }
    material_only_kernel<<<blocks_for(ctx->np, 256), 256, 0, ctx->stream>>>(A, ctx->cfg.material);
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
