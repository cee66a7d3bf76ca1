// Per-particle constitutive updates as device functions.  Each follows its
// reference plugin line by line; products, sums and quotients use the _rn
// intrinsics so that nvcc cannot fuse them into multiply-adds, which keeps
// the results bit-identical to the reference compiled without contraction.
#pragma once

#include "mpmg_internal.cuh"

namespace mat {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dadd_rn(a, -b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// a / b where the divisor b is fixed for the run and y = RN(1 / b) was
// formed once on the host.  Markstein's correction q' = RN(q + r y), with the
// residual r = a - b q exact through an FMA, is applied twice from q = RN(a y):
// the first brings q within one ulp of a / b, and from there the second
// returns the correctly rounded quotient (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990).  Five FP64 operations in place of a full division; the
// result equals dvd(a, b) for normal operands and quotients (a zero quotient
// comes out +0, and non-finite operands are not carried through).
__device__ __forceinline__ double dvd_known(double a, double b, double y)
{
    double q = __dmul_rn(a, y);
    double r = __fma_rn(-b, q, a);
    q = __fma_rn(r, y, q);
    r = __fma_rn(-b, q, a);
    return __fma_rn(r, y, q);
}

constexpr double kThird = 1.0 / 3.0;   // RN(1/3), the reciprocal of the divisor 3.0

struct Elastic {
    double G, K, lambda, dt;
    double twoG;            // 2 G, exact
    double inv_G, inv_dt;   // RN(1/G), RN(1/dt)
    double Gdt, inv_Gdt;    // RN(G dt), RN(1 / RN(G dt))
};

// exp(x) for the volume update v <- v exp(dt tr D), whose argument is tiny at
// any stable time step: where |x| < 2^-9 the degree-5 Taylor polynomial about
// 0 in Horner form (truncation below x^6 / 720 < 2^-63, under a tenth of an
// ulp of the result, so the result lies within about half an ulp of e^x);
// elsewhere exp().
__device__ __forceinline__ double exp_small(double x)
{
    if ((__double2hiint(x) & 0x7fffffff) < 0x3f600000) {
        double p = __fma_rn(x, 1.0 / 120.0, 1.0 / 24.0);
        p = __fma_rn(p, x, 1.0 / 6.0);
        p = __fma_rn(p, x, 0.5);
        p = __fma_rn(p, x, 1.0);
        return __fma_rn(p, x, 1.0);
    }
    return exp(x);
}

// isolin calculate_stress_threaded, materialsrc/isolin.c:75-116.
__device__ __forceinline__ void isolin(const Elastic &el, double exx, double exy, double eyy,
                                       double wxy, double &sxx, double &sxy, double &syy)
{
    const double twoG = el.twoG;
    double trD = add(exx, eyy);
    double dsjxx = add(mul(el.lambda, trD), mul(twoG, exx));
    double dsjxy = mul(twoG, exy);
    double dsjyy = add(mul(el.lambda, trD), mul(twoG, eyy));
    double w2s = mul(mul(2.0, wxy), sxy);
    dsjxx = add(dsjxx, w2s);
    dsjxy = sub(dsjxy, mul(wxy, sub(sxx, syy)));
    dsjyy = sub(dsjyy, w2s);
    sxx = add(sxx, mul(el.dt, dsjxx));
    sxy = add(sxy, mul(el.dt, dsjxy));
    syy = add(syy, mul(el.dt, dsjyy));
}

// negative_root, g_local_mu2.c:90-99 (also g_nonlocal_mu2.c:226-235).
__device__ __forceinline__ double negative_root(double a, double b, double c)
{
    double disc = __dsqrt_rn(sub(mul(b, b), mul(mul(4.0, a), c)));
    if (b > 0) return dvd(sub(-b, disc), mul(2.0, a));
    return dvd(mul(2.0, c), add(-b, disc));
}

struct Mu2Params {
    double mu_s, mu_2, I0, grains_rho, grains_d, rho_critical, A;
    double inv_grains_rho, inv_grains_d;   // RN(1/grains_rho), RN(1/grains_d)
    double rho_lo, rho_hi;                 // RN(rho_critical (1 - 2^-47)), RN(rho_critical (1 + 2^-47))
    double AAdd, inv_AAdd;                 // RN(RN(RN(A A) d) d) and its reciprocal
    double alpha_c;                        // G I0 dt / (grains_d sqrt(grains_rho))
    double GI0dt;                          // RN(RN(G I0) dt), formed on the host
};

// RN(m / v) < rho_critical, decided as the reference's division and compare
// decide it, without the division for most particles.  For normal v > 0 and
// rho_lo, rho_hi as above: m < RN(v rho_lo) implies
// m / v < rho_critical (1 - 2^-48), hence RN(m / v) < rho_critical; and
// m > RN(v rho_hi) implies m / v > rho_critical (1 + 2^-48), hence
// RN(m / v) > rho_critical (the roundings add at most 3 2^-53 relative, and
// the doubles within 2^-48 of rho_critical are further than an ulp from it).
// Only m inside the bracket, and any v that is not a normal positive number
// above 2^-959 (or a NaN), takes the division.
__device__ __forceinline__ bool below_density(double m, double v, const Mu2Params &mp)
{
    if (__double_as_longlong(v) > 0x0400000000000000LL && __double_as_longlong(v) < 0x7ff0000000000000LL) {
        if (m < __dmul_rn(v, mp.rho_lo)) return true;
        if (m > __dmul_rn(v, mp.rho_hi)) return false;
    }
    return __ddiv_rn(m, v) < mp.rho_critical;
}

// g_local_mu2 calculate_stress_threaded, g_local_mu2.c:165-310, written for
// the plane-strain stress it keeps: T = [[Txx, Txy, 0], [Txy, Tyy, 0],
// [0, 0, Tzz]] (the z-shear components stay zero and T stays symmetric
// because L has no z entries).  The expressions are the tensor.c sums with
// their zero terms removed, in the same order.
__device__ __forceinline__ void g_local_mu2(const Elastic &el, const Mu2Params &mp, double m,
                                            double v, double exx, double exy, double eyy,
                                            double wxy, double &Txx, double &Txy, double &Tyy,
                                            double &Tzz, double &gammap, double &gammadotp)
{
    const double G = el.G, dt = el.dt;
    const double lambda = el.lambda;   // K - 2 G / 3, formed on the host with the same roundings
    // L (:191-199), W = skw(L), D = sym(L) (tensor.c:330-384)
    // Exact shortcuts, bit for bit the reference's values for finite
    // operands below DBL_MAX / 2: 0.5 (x + x) is x; W T - T W has xx entry
    // RN(W Txy) + RN(W Txy), an exact doubling, and yy entry its negative;
    // 0 * 2G is +0.
    double Lxy = add(exy, wxy), Lyx = sub(exy, wxy);
    double Wxy = mul(0.5, sub(Lxy, Lyx));
    double Dxx = exx;
    double Dxy = mul(0.5, add(Lxy, Lyx));
    double Dyy = eyy;
    double trD = add(Dxx, Dyy);
    // Jaumann term JS = W T - T W (:209-212)
    const double wt = mul(Wxy, Txy);
    double JSxx = add(wt, wt);
    double JSxy = add(mul(Wxy, Tyy), -mul(Txx, Wxy));
    double JSyy = -JSxx;
    // trial stress (:215-222)
    const double twoG = el.twoG;
    double lt = mul(lambda, trD);
    double Txx_tr = add(mul(add(add(mul(Dxx, twoG), lt), JSxx), dt), Txx);
    double Txy_tr = add(mul(add(mul(Dxy, twoG), JSxy), dt), Txy);
    double Tyy_tr = add(mul(add(add(mul(Dyy, twoG), lt), JSyy), dt), Tyy);
    double Tzz_tr = add(mul(add(0.0, lt), dt), Tzz);
    // decompose and contract (:225-228; tensor.c:205-224, :422-437)
    double p_tr = dvd_known(add(add(Txx_tr, Tyy_tr), Tzz_tr), 3.0, kThird);
    double T0xx = sub(Txx_tr, p_tr), T0xy = Txy_tr, T0yy = sub(Tyy_tr, p_tr), T0zz = sub(Tzz_tr, p_tr);
    double tt = add(add(add(add(mul(T0xx, T0xx), mul(T0xy, T0xy)), mul(T0xy, T0xy)), mul(T0yy, T0yy)),
                    mul(T0zz, T0zz));
    double tau_tr = __dsqrt_rn(mul(0.5, tt));
    p_tr = -p_tr;

    const bool density_flag = below_density(m, v, mp);
    double nup_tau;
    if (density_flag || p_tr <= 0) {
        nup_tau = 0;
        Txx = 0; Txy = 0; Tyy = 0; Tzz = 0;
    } else if (p_tr > 0) {
        double S0 = mul(mp.mu_s, p_tr);
        if (tau_tr <= S0 && isfinite(tau_tr)) {
            // tau_tau = tau_tr, scale factor 1: (tau_tr - tau_tau) / G / dt
            // is +0 and T0 * 1 is T0 exactly, so neither is formed
            nup_tau = 0;
            Txx = sub(T0xx, p_tr);
            Txy = T0xy;
            Tyy = sub(T0yy, p_tr);
            Tzz = sub(T0zz, p_tr);
        } else {
            double tau_tau, scale_factor;
            if (tau_tr <= S0) {
                tau_tau = tau_tr;
                scale_factor = 1.0;
            } else {
                double S2 = mul(mp.mu_2, p_tr);
                double alpha = dvd_known(mul(mp.GI0dt,
                                             __dsqrt_rn(dvd_known(p_tr, mp.grains_rho, mp.inv_grains_rho))),
                                         mp.grains_d, mp.inv_grains_d);
                double B = -add(add(S2, tau_tr), alpha);
                double H = add(mul(S2, tau_tr), mul(S0, alpha));
                tau_tau = negative_root(1.0, B, H);
                scale_factor = dvd(tau_tau, tau_tr);
            }
            nup_tau = dvd_known(dvd_known(sub(tau_tr, tau_tau), G, el.inv_G), dt, el.inv_dt);
            Txx = sub(mul(T0xx, scale_factor), p_tr);
            Txy = mul(T0xy, scale_factor);
            Tyy = sub(mul(T0yy, scale_factor), p_tr);
            Tzz = sub(mul(T0zz, scale_factor), p_tr);
        }
    } else {
        nup_tau = 0;   // NaN pressure: the reference prints 'u' and keeps T
    }
    gammap = add(gammap, mul(nup_tau, dt));
    gammadotp = nup_tau;
}

// The plane-stress-form local returns that share one structure:
//   dp_ri_mt                  dp_ri_mt.c:99-200                  3D trial, Drucker-Prager return
//   g_local_mu2_plane_strain  g_local_mu2_plane_strain.c:157-265 3D trial, mu(I) return, beta
//   g_local_mu2_true_2d       g_local_mu2_true_2d.c:157-260      2D trial, mu(I) return, beta
// A 3D trial carries the out-of-plane stress szz (state[1]) and takes
// p = -(sxx + syy + szz) / 3; the 2D trial takes p = -(sxx + syy) / 2.  The
// Drucker-Prager return caps tau at mu_s p; the mu(I) return takes the
// negative root of g_local_mu2's quadratic.  Dilute particles (m / v below
// the literal 1485.0f) and particles in tension drop their stress and record
// the whole trial shear as plastic flow, and the beta variants record
// -p / (K dt) in state[5].  state[9] accumulates the plastic strain and
// state[10] holds its rate.
struct ReturnParams {
    double mu_s, mu_2, I0, grains_rho, grains_d, rho_critical;
};

template <bool TRIAL3D, bool MU_I, bool BETA>
__device__ __forceinline__ void plane_return(const Elastic &el, const ReturnParams &rp, double m, double v,
                                             double exx, double exy, double eyy, double wxy, double &sxx,
                                             double &sxy, double &syy, double &szz, double &beta,
                                             double &gammap, double &gammadotp)
{
    const double G = el.G, K = el.K, dt = el.dt;
    const double lambda = el.lambda;   // K - 2 G / 3, formed on the host with the same roundings
    const double twoG = el.twoG;
    double trD = add(exx, eyy);
    double dsjxx = add(mul(lambda, trD), mul(twoG, exx));
    double dsjxy = mul(twoG, exy);
    double dsjyy = add(mul(lambda, trD), mul(twoG, eyy));
    double w2s = mul(mul(2.0, wxy), sxy);
    dsjxx = add(dsjxx, w2s);
    dsjxy = sub(dsjxy, mul(wxy, sub(sxx, syy)));
    dsjyy = sub(dsjyy, w2s);
    double sxx_tr = add(sxx, mul(dt, dsjxx));
    double sxy_tr = add(sxy, mul(dt, dsjxy));
    double syy_tr = add(syy, mul(dt, dsjyy));
    double p_tr, t0zz = 0, szz_tr = 0;
    if (TRIAL3D) {
        szz_tr = add(szz, mul(mul(dt, lambda), trD));
        p_tr = dvd(-add(add(sxx_tr, syy_tr), szz_tr), 3.0);
    } else {
        p_tr = mul(-0.5, add(sxx_tr, syy_tr));
    }
    double t0xx = add(sxx_tr, p_tr), t0xy = sxy_tr, t0yy = add(syy_tr, p_tr);
    double tt = add(add(mul(t0xx, t0xx), mul(mul(2.0, t0xy), t0xy)), mul(t0yy, t0yy));
    if (TRIAL3D) {
        t0zz = add(szz_tr, p_tr);
        tt = add(tt, mul(t0zz, t0zz));
    }
    double tau_tr = __dsqrt_rn(mul(0.5, tt));

    const bool density_flag = dvd(m, v) < rp.rho_critical;
    double nup_tau;
    if (density_flag || p_tr <= 0) {
        nup_tau = dvd(tau_tr, mul(G, dt));
        if (BETA) beta = dvd(-p_tr, mul(K, dt));
        sxx = 0; sxy = 0; syy = 0;
        if (TRIAL3D) szz = 0;
    } else if (p_tr > 0) {
        double S0 = mul(rp.mu_s, p_tr);
        double tau_tau, scale_factor;
        if (tau_tr <= S0) {
            tau_tau = tau_tr;
            scale_factor = 1.0;
        } else if (MU_I) {
            double S2 = mul(rp.mu_2, p_tr);
            double alpha = dvd(mul(mul(mul(G, rp.I0), dt), __dsqrt_rn(dvd(p_tr, rp.grains_rho))), rp.grains_d);
            double B = -add(add(S2, tau_tr), alpha);
            double H = add(mul(S2, tau_tr), mul(S0, alpha));
            tau_tau = negative_root(1.0, B, H);
            scale_factor = dvd(tau_tau, tau_tr);
        } else {
            tau_tau = S0;
            scale_factor = dvd(tau_tau, tau_tr);
        }
        nup_tau = dvd(dvd(sub(tau_tr, tau_tau), G), dt);
        if (BETA) beta = 0;
        sxx = sub(mul(scale_factor, t0xx), p_tr);
        sxy = mul(scale_factor, t0xy);
        syy = sub(mul(scale_factor, t0yy), p_tr);
        if (TRIAL3D) szz = sub(mul(scale_factor, t0zz), p_tr);
    } else {
        nup_tau = 0;   // NaN pressure: the reference prints 'u' and keeps s
    }
    gammap = add(gammap, mul(nup_tau, dt));
    gammadotp = nup_tau;
}

// g_local_mu2_reverse calculate_stress_threaded, g_local_mu2_reverse.c:166-302:
// a rate-dependent return to mu(I) (p + c), c = 0, with mu from the previous
// step's gammadotp and the start-of-step pressure, and Jaumann terms of the
// opposite sign to isolin's.  beta in state[5].
__device__ __forceinline__ void g_local_mu2_reverse(const Elastic &el, const Mu2Params &mp, double m, double v,
                                                    double exx, double exy, double eyy, double wxy, double &sxx,
                                                    double &sxy, double &syy, double &beta, double &gammap,
                                                    double &gammadotp)
{
    const double G = el.G, K = el.K, dt = el.dt, c = 0;
    const double lambda = sub(K, dvd(mul(2.0, G), 3.0));
    const double twoG = el.twoG;
    double p_t = mul(-0.5, add(sxx, syy));
    double trD = add(exx, eyy);
    double dsjxx = add(mul(lambda, trD), mul(twoG, exx));
    double dsjxy = mul(twoG, exy);
    double dsjyy = add(mul(lambda, trD), mul(twoG, eyy));
    double w2s = mul(mul(2.0, wxy), sxy);
    dsjxx = sub(dsjxx, w2s);
    dsjxy = add(dsjxy, mul(wxy, sub(sxx, syy)));
    dsjyy = add(dsjyy, w2s);
    double sxx_tr = add(sxx, mul(dt, dsjxx));
    double sxy_tr = add(sxy, mul(dt, dsjxy));
    double syy_tr = add(syy, mul(dt, dsjyy));
    double p_tr = mul(-0.5, add(sxx_tr, syy_tr));
    double t0xx = add(sxx_tr, p_tr), t0xy = sxy_tr, t0yy = add(syy_tr, p_tr);
    double tau_tr = __dsqrt_rn(mul(0.5, add(add(mul(t0xx, t0xx), mul(mul(2.0, t0xy), t0xy)), mul(t0yy, t0yy))));
    double inum = mul(mul(gammadotp, mp.grains_d), __dsqrt_rn(mp.grains_rho));
    double mu_t;
    if (p_t <= 0) {
        mu_t = mp.mu_2;
    } else {
        inum = dvd(inum, __dsqrt_rn(p_t));
        if (inum <= 0) mu_t = mp.mu_s;
        else mu_t = add(mp.mu_s, dvd(sub(mp.mu_2, mp.mu_s), add(dvd(mp.I0, inum), 1.0)));
    }
    double tau_tau = mul(mu_t, add(p_tr, c));
    double f = sub(tau_tr, tau_tau);
    const bool density_flag = dvd(m, v) < mp.rho_critical;
    const double pmin = dvd(-c, mu_t);
    double nup_tau;
    if (density_flag) {
        nup_tau = dvd(tau_tr, mul(G, dt));
        beta = dvd(-p_tr, mul(K, dt));
        sxx = 0; sxy = 0; syy = 0;
    } else if (f < 0) {
        nup_tau = 0;
        beta = 0;
        sxx = sub(t0xx, p_tr);
        sxy = t0xy;
        syy = sub(t0yy, p_tr);
    } else if (f >= 0 && p_tr > pmin) {
        nup_tau = dvd(dvd(f, G), dt);
        beta = 0;
        double scale_factor = dvd(tau_tau, tau_tr);
        sxx = sub(mul(scale_factor, t0xx), p_tr);
        sxy = mul(scale_factor, t0xy);
        syy = sub(mul(scale_factor, t0yy), p_tr);
    } else if (p_tr <= pmin) {
        nup_tau = dvd(tau_tr, mul(G, dt));
        beta = dvd(sub(dvd(c, mu_t), p_tr), mul(K, dt));
        sxx = 0; sxy = 0; syy = 0;
    } else {
        nup_tau = 0;   // NaN: the reference prints the particle and keeps s
    }
    gammap = add(gammap, mul(nup_tau, dt));
    gammadotp = nup_tau;
}

// mu_from_gammadot, g_local_mu2_ext.c:75-95.
__device__ __forceinline__ double mu_from_gammadot(double gammadot, double p, double dsqrtrhos, double mu_s,
                                                   double mu_2, double inum_0)
{
    if (p <= 0) return mu_2;
    double inum = dvd(mul(dsqrtrhos, gammadot), __dsqrt_rn(p));
    if (inum <= 0) return mu_s;
    return add(mu_s, dvd(sub(mu_2, mu_s), add(dvd(inum_0, inum), 1.0)));
}

// g_local_mu2_ext, first phase (g_local_mu2_ext.c:214-230): the local
// fluidity gammadotp / mu_t from the start-of-step pressure.  mu_t keeps its
// previous value where gammadotp is 0.
__device__ __forceinline__ void ext_local_fluidity(const Mu2Params &mp, double sxx, double syy, double gammadotp,
                                                   double &mu_t, double &gflocal)
{
    double p_t = mul(-0.5, add(sxx, syy));
    if (gammadotp == 0) {
        gflocal = 0;
    } else {
        mu_t = mu_from_gammadot(gammadotp, p_t, mul(mp.grains_d, __dsqrt_rn(mp.grains_rho)), mp.mu_s, mp.mu_2,
                                mp.I0);
        gflocal = dvd(gammadotp, mu_t);
    }
}

// g_local_mu2_ext, third phase (g_local_mu2_ext.c:292-368): plane-stress
// elastic trial with the Jaumann terms, returned to mu(gammadotp) (p + c)
// with c = 1e-2.
__device__ __forceinline__ void ext_stress(const Elastic &el, const Mu2Params &mp, double E, double nu, double m,
                                           double v, double exx, double exy, double eyy, double wxy, double &sxx,
                                           double &sxy, double &syy, double &mu_t, double &beta, double &gammap,
                                           double &gammadotp)
{
    const double G = el.G, K = el.K, dt = el.dt, c = 1e-2;
    double p_t = mul(-0.5, add(sxx, syy));
    const double Ep = dvd(E, sub(1.0, mul(nu, nu)));
    const double Gp = dvd(E, mul(2.0, add(1.0, nu)));
    double dsjxx = mul(mul(dt, Ep), add(exx, mul(nu, eyy)));
    double dsjxy = mul(mul(dt, Gp), exy);
    double dsjyy = mul(mul(dt, Ep), add(eyy, mul(nu, exx)));
    double w2 = mul(mul(mul(2.0, dt), wxy), sxy);
    dsjxx = sub(dsjxx, w2);
    dsjxy = add(dsjxy, mul(mul(dt, wxy), sub(sxx, syy)));
    dsjyy = add(dsjyy, w2);
    double sxx_tr = add(sxx, dsjxx), sxy_tr = add(sxy, dsjxy), syy_tr = add(syy, dsjyy);
    double p_tr = mul(-0.5, add(sxx_tr, syy_tr));
    double t0xx = add(sxx_tr, p_tr), t0xy = sxy_tr, t0yy = add(syy_tr, p_tr);
    double tau_tr = __dsqrt_rn(mul(0.5, add(add(mul(t0xx, t0xx), mul(mul(2.0, t0xy), t0xy)), mul(t0yy, t0yy))));
    mu_t = mu_from_gammadot(gammadotp, p_t, mul(mp.grains_d, __dsqrt_rn(mp.grains_rho)), mp.mu_s, mp.mu_2, mp.I0);
    double tau_tau = mul(mu_t, add(p_tr, c));
    double f = sub(tau_tr, tau_tau);
    const bool density_flag = dvd(m, v) < mp.rho_critical;
    const double pmin = dvd(-c, mu_t);   // -c / mu_t, the reference's -c/mu_t
    double nup_tau;
    if (density_flag) {
        nup_tau = dvd(tau_tr, mul(G, dt));
        beta = dvd(-p_tr, mul(K, dt));
        sxx = 0; sxy = 0; syy = 0;
    } else if (f < 0) {
        nup_tau = 0;
        beta = 0;
        sxx = sub(t0xx, p_tr);
        sxy = t0xy;
        syy = sub(t0yy, p_tr);
    } else if (f >= 0 && p_tr > pmin) {
        nup_tau = dvd(sub(tau_tr, tau_tau), mul(G, dt));
        beta = 0;
        double scale_factor = dvd(tau_tau, tau_tr);
        sxx = sub(mul(scale_factor, t0xx), p_tr);
        sxy = mul(scale_factor, t0xy);
        syy = sub(mul(scale_factor, t0yy), p_tr);
    } else if (p_tr <= pmin) {
        nup_tau = dvd(tau_tr, mul(G, dt));
        beta = dvd(sub(dvd(c, mu_t), p_tr), mul(K, dt));
        sxx = 0; sxy = 0; syy = 0;
    } else {
        nup_tau = 0;   // NaN: the reference prints the particle and keeps s
    }
    gammap = add(gammap, mul(nup_tau, dt));
    gammadotp = nup_tau;
}

// Trial Jaumann stress of g_nonlocal_mu2.c:166-186 (and :271-290), with
// lambda = K - 2G/3 (the reference leaves it uninitialised at :154).
__device__ __forceinline__ void nonlocal_mu2_trial(const Elastic &el, double exx, double exy,
                                                   double eyy, double wxy, double sxx, double sxy,
                                                   double syy, double &p_tr, double &t0xx,
                                                   double &t0xy, double &t0yy, double &tau_tr)
{
    const double dt = el.dt;
    const double lambda = el.lambda;   // sub(K, dvd(mul(2, G), 3)), formed on the host with the same roundings
    const double twoG = el.twoG;
    double trD = add(exx, eyy);
    double dsjxx = add(mul(lambda, trD), mul(twoG, exx));
    double dsjxy = mul(twoG, exy);
    double dsjyy = add(mul(lambda, trD), mul(twoG, eyy));
    double w2s = mul(mul(2.0, wxy), sxy);
    dsjxx = add(dsjxx, w2s);
    dsjxy = sub(dsjxy, mul(wxy, sub(sxx, syy)));
    dsjyy = sub(dsjyy, w2s);
    double sxx_tr = add(sxx, mul(dt, dsjxx));
    double sxy_tr = add(sxy, mul(dt, dsjxy));
    double syy_tr = add(syy, mul(dt, dsjyy));
    p_tr = mul(-0.5, add(sxx_tr, syy_tr));
    t0xx = add(sxx_tr, p_tr);
    t0xy = sxy_tr;
    t0yy = add(syy_tr, p_tr);
    tau_tr = __dsqrt_rn(mul(0.5, add(add(mul(t0xx, t0xx), mul(mul(2.0, t0xy), t0xy)), mul(t0yy, t0yy))));
}

// calculate_bulk_granular_fluidity, g_nonlocal_mu2.c:238-321, for one
// particle, from its trial pressure and shear stress (nonlocal_mu2_trial):
// dense flag, local fluidity and the inverse squared cooperativity length.
// The dense flag and the branches are the reference's decisions on the same
// values.  The flowing branch is the same algebra in fewer FP64 operations
// (these values feed the iterative fluidity solve, not a bit-exact output):
//   alpha    = G I0 dt sqrt(p / rho) / d  = alpha_c sqrt(p)
//   tau_tau  = the negative root of t^2 - B t + H, B = S2 + tau + alpha > 0,
//              as 2 H / (B + sqrt(B^2 - 4 H)) (negative_root's b < 0 branch)
//   gf_local = (p / (G dt)) (tau / tau_tau - 1) = p (tau - tau_tau) / (G dt tau_tau)
// and below yield (scale factor 1) gf_local is +0.
__device__ __forceinline__ void nonlocal_mu2_bulk(const Elastic &el, const Mu2Params &mp, double m,
                                                  double v, double p_tr, double tau_tr, double &dense,
                                                  double &gf_local, double &xisq_inv)
{
    dense = (below_density(m, v, mp) || p_tr < 0) ? 0.0 : 1.0;
    if (dense == 0 || p_tr <= 0) {
        gf_local = 0;
        xisq_inv = 0;
    } else if (p_tr > 0) {
        double tau_tau;
        double S0 = mul(mp.mu_s, p_tr);
        if (tau_tr <= S0) {
            tau_tau = tau_tr;
            gf_local = 0;
        } else {
            double S2 = mul(mp.mu_2, p_tr);
            double alpha = mul(mp.alpha_c, __dsqrt_rn(p_tr));
            double B = add(add(S2, tau_tr), alpha);
            double H = add(mul(S2, tau_tr), mul(S0, alpha));
            tau_tau = dvd(add(H, H), add(B, __dsqrt_rn(sub(mul(B, B), mul(4.0, H)))));
            gf_local = dvd(mul(p_tr, sub(tau_tr, tau_tau)), mul(el.Gdt, tau_tau));
        }
        xisq_inv = dvd_known(fabs(sub(dvd(tau_tau, p_tr), mp.mu_s)), mp.AAdd, mp.inv_AAdd);
    } else {
        gf_local = 0;
        xisq_inv = 0;
    }
}

// Stress update after the fluidity solve, g_nonlocal_mu2.c:160-218. The
// reference forms the trial stress again at :166-186 from the same strain
// rates and start-of-step stress as the bulk pass; the G2P keeps that trial
// instead, with the dense flag folded into the pressure (p_d = p_tr where the
// particle is dense, 0 where it is not), so `dense == 0 || p_tr <= 0` reads
// `p_d <= 0`. sxx, sxy, syy hold the start-of-step stress, which a NaN trial
// pressure keeps (neither branch of the reference is taken).
__device__ __forceinline__ void nonlocal_mu2_stress(const Elastic &el, double gf, double p_d,
                                                    double t0xx, double t0xy, double t0yy,
                                                    double tau_tr, double &sxx, double &sxy,
                                                    double &syy, double &gammap, double &gammadotp)
{
    const double dt = el.dt;
    const double p_tr = p_d;
    double nup_tau;
    if (p_tr <= 0) {
        nup_tau = 0;
        sxx = 0; sxy = 0; syy = 0;
    } else if (p_tr > 0) {
        double scale_factor = dvd(p_tr, add(mul(el.Gdt, gf), p_tr));
        double tau_tau = mul(tau_tr, scale_factor);
        // ((tau - tau_tau) / G) / dt as one quotient by G dt (the fluidity
        // comes from an iterative solve, so this value is not bit-exact
        // with the reference's anyway)
        nup_tau = dvd_known(sub(tau_tr, tau_tau), el.Gdt, el.inv_Gdt);
        sxx = sub(mul(scale_factor, t0xx), p_tr);
        sxy = mul(scale_factor, t0xy);
        syy = sub(mul(scale_factor, t0yy), p_tr);
    } else {
        nup_tau = 0;
    }
    gammap = add(gammap, mul(nup_tau, dt));
    gammadotp = nup_tau;
}

struct NonlocalParams {
    double E, nu, mu_s, grains_rho, B, A, grains_d, cohesion;
};

// calculate_bulk_granular_fluidity, g_nonlocal.c:306-352, for one particle
// (the reference applies it to every particle, active or not).
__device__ __forceinline__ void nonlocal_bulk(const NonlocalParams &np, double sxx, double sxy,
                                              double syy, double &eta, double &gf_bulk,
                                              double &xisq_inv)
{
    const double p_cap = 1e-2;
    double p_t = mul(-0.5, add(sxx, syy));
    double a = add(sxx, p_t), b = sxy, c = add(syy, p_t);
    double tau_t = __dsqrt_rn(mul(0.5, add(add(mul(a, a), mul(mul(2.0, b), b)), mul(c, c))));
    if (p_t < p_cap) p_t = p_cap;
    double S0 = mul(p_t, np.mu_s);
    eta = mul(mul(np.B, np.grains_d), __dsqrt_rn(mul(p_t, np.grains_rho)));
    xisq_inv = dvd(fabs(sub(dvd(tau_t, p_t), np.mu_s)),
                   mul(mul(mul(np.grains_d, np.grains_d), np.A), np.A));
    gf_bulk = (tau_t > S0) ? mul(dvd(p_t, eta), sub(1.0, dvd(S0, tau_t))) : 0.0;
}

// Explicit stress update of g_nonlocal.c:154-298 (every particle).
__device__ __forceinline__ void nonlocal_stress(const NonlocalParams &np, double G, double dt,
                                                double t, double gf, double exx, double exy,
                                                double eyy, double wxy, double &sxx, double &sxy,
                                                double &syy, double &gammap)
{
    const double EMOD = np.E, NUMOD = np.nu, c = np.cohesion;
    const double cA = dvd(EMOD, sub(1.0, mul(NUMOD, NUMOD)));
    const double cB = dvd(EMOD, mul(2.0, add(1.0, NUMOD)));
    double p_t = mul(-0.5, add(sxx, syy));
    double a = add(sxx, p_t), b = sxy, cc = add(syy, p_t);
    double tau_t;
    double dsjxx = mul(mul(dt, cA), add(exx, mul(NUMOD, eyy)));
    double dsjxy = mul(mul(dt, cB), exy);
    double dsjyy = mul(mul(dt, cA), add(eyy, mul(NUMOD, exx)));
    double jw = mul(mul(mul(2.0, dt), wxy), sxy);
    dsjxx = sub(dsjxx, jw);
    dsjxy = add(dsjxy, mul(mul(dt, wxy), sub(sxx, syy)));
    dsjyy = add(dsjyy, jw);
    double p_tr = mul(-0.5, add(add(sxx, dsjxx), add(syy, dsjyy)));
    if (p_tr < c) {
        sxx = dvd(mul(0.5, c), np.mu_s);
        sxy = 0;
        syy = dvd(mul(0.5, c), np.mu_s);
        return;
    }
    tau_t = __dsqrt_rn(mul(0.5, add(add(mul(a, a), mul(mul(2.0, b), b)), mul(cc, cc))));
    const double r = __dsqrt_rn(0.5);
    double Npxx = dvd(mul(r, a), tau_t);
    double Npxy = dvd(mul(r, b), tau_t);
    double Npyy = dvd(mul(r, cc), tau_t);
    double dxx0 = mul(0.5, sub(exx, eyy)), dxy0 = exy, dyy0 = mul(0.5, sub(eyy, exx));
    double gammadot = __dsqrt_rn(mul(2.0, add(add(mul(dxx0, dxx0), mul(mul(2.0, dxy0), dxy0)),
                                              mul(dyy0, dyy0))));
    double nup_tau, dpxx, dpxy, dpyy;
    if (p_t > c && gf > 0) {
        nup_tau = dvd(mul(gf, tau_t), p_t);
        if (nup_tau < 0) nup_tau = 0;
        if (nup_tau > gammadot) nup_tau = gammadot;
        dpxx = mul(mul(r, nup_tau), Npxx);
        dpxy = mul(mul(r, nup_tau), Npxy);
        dpyy = mul(mul(r, nup_tau), Npyy);
    } else {
        nup_tau = 0; dpxx = 0; dpxy = 0; dpyy = 0;
    }
    if (t == 0) {
        nup_tau = 0; dpxx = 0; dpxy = 0; dpyy = 0;
    }
    double exx_e = sub(exx, dpxx), eyy_e = sub(eyy, dpyy);
    dsjxx = mul(mul(dt, cA), add(exx_e, mul(NUMOD, eyy_e)));
    dsjxy = mul(mul(dt, cB), sub(exy, dpxy));
    dsjyy = mul(mul(dt, cA), add(eyy_e, mul(NUMOD, exx_e)));
    dsjxx = sub(dsjxx, jw);
    dsjxy = add(dsjxy, mul(mul(dt, wxy), sub(sxx, syy)));
    dsjyy = add(dsjyy, jw);
    gammap = add(gammap, mul(nup_tau, dt));
    sxx = add(sxx, dsjxx);
    sxy = add(sxy, dsjxy);
    syy = add(syy, dsjyy);
    (void)G;
}

}  // namespace mat
