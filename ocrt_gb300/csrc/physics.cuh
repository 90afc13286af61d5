// physics.cuh — device restatements of the reference's scalar physics:
// Bodhaine Rayleigh depth, US62 / exponential altitude mapping, generalized
// spherical function recurrences, Fresnel and Cox-Munk Mueller kernels.
// All FP64 unless templated; the Cox-Munk kernel is templated so the azimuth
// grid can run in FP32 while the single direct-glint evaluation runs in FP64.
#pragma once
#include "common.cuh"

// ---- Rayleigh optical depth, Bodhaine et al. 1999 (rt_rayleigh.c:46-238) ----
__host__ __device__ inline double gravity_wgs84(double lat_deg, double z_m)
{
    const double lat = lat_deg * OCRT_PI / 180.0;
    const double s1 = sin(lat) * sin(lat);
    const double s2 = sin(2.0 * lat) * sin(2.0 * lat);
    return 9.780327 * (1.0 + 0.0053024 * s1 - 0.0000058 * s2) - 3.086e-6 * z_m;
}

__host__ __device__ inline double bodhaine_tau(double wl_nm, double p_hpa)
{
    const double co2 = 360.0, um = wl_nm / 1000.0, inv2 = 1.0 / (um * um);
    const double fn2 = 1.034 + 3.17e-4 * inv2;
    const double fo2 = 1.096 + 1.385e-3 * inv2 + 1.448e-4 * inv2 * inv2;
    const double xc = co2 / 1.0e4;
    const double king = (78.084 * fn2 + 20.946 * fo2 + 0.934 + xc * 1.15) /
                        (78.084 + 20.946 + 0.934 + xc);
    const double n300 = (8060.51 + 2480990.0 / (132.274 - inv2) + 17455.7 / (39.32957 - inv2)) * 1.0e-8;
    const double nm1 = n300 * (1.0 + 0.54 * (co2 * 1.0e-6 - 0.0003));
    const double nn = (1.0 + nm1) * (1.0 + nm1);
    const double avo = 6.0221367e23;
    const double ns = (avo / 22.4141) * (273.15 / 288.15) * 1.0e-3;
    const double wl_cm = wl_nm * 1.0e-7, wl4 = wl_cm * wl_cm * wl_cm * wl_cm;
    const double sigma = 24.0 * OCRT_PI * OCRT_PI * OCRT_PI * (nn - 1.0) * (nn - 1.0) /
                         (wl4 * ns * ns * (nn + 2.0) * (nn + 2.0)) * king;
    const double ma = 15.0556 * (co2 * 1.0e-6) + 28.9595;
    return sigma * (p_hpa * 1000.0) * avo / (ma * 100.0 * gravity_wgs84(45.0, 5517.56));
}

// ---- altitude mapping (rt_molecular_profile.c:9-105, rt_atm.c:44-51) ----
__device__ inline double us62_pressure(double z)
{
    const double Z[8] = {0.0, 11.0, 20.0, 32.0, 47.0, 51.0, 71.0, 84.852};
    const double P[8] = {101325.0, 22632.1, 5474.89, 868.019, 110.906, 66.9389, 3.95642, 0.3734};
    if (z <= Z[0]) return P[0];
    if (z >= Z[7]) return P[7];
    int lo = 0, hi = 7;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (z < Z[mid]) hi = mid; else lo = mid;
    }
    const double t = (z - Z[lo]) / (Z[hi] - Z[lo]);
    const double a = log(P[lo]), b = log(P[hi]);
    return exp(a + t * (b - a));
}

__device__ inline double clamp01d(double x) { return x <= 0.0 ? 0.0 : (x >= 1.0 ? 1.0 : x); }

__device__ inline double us62_raw(double z)
{
    if (z <= 0.0) return 1.0;
    const double g0 = gravity_wgs84(45.0, 0.0);
    if (z >= 84.852) return clamp01d((0.3734 / gravity_wgs84(45.0, 84852.0)) / (101325.0 / g0));
    return clamp01d((us62_pressure(z) / gravity_wgs84(45.0, z * 1000.0)) / (101325.0 / g0));
}

__device__ inline double us62_grid_above(double z)
{
    if (z <= 0.0) return 1.0;
    if (z >= 84.852) return 0.0;
    const double ft = us62_raw(84.852);
    return clamp01d((us62_raw(z) - ft) / (1.0 - ft));
}

__device__ inline double exp_above(double z, double ztop, double h)
{
    if (z <= 0.0) return 1.0;
    if (z >= ztop) return 0.0;
    const double et = exp(-ztop / h);
    return (exp(-z / h) - et) / (1.0 - et);
}

__device__ inline double ray_above(double z, int profile, double h)
{
    return profile == 1 ? exp_above(z, OCRT_ZTOP_KM, h) : us62_grid_above(z);
}

// The same column fractions with their altitude-independent parts evaluated
// once per thread (the table logarithms, the 45-degree gravity term, the US62
// fraction at 84.852 km, exp(-ztop / h)), for the 64-step level bisection.
struct AboveEval {
    int prof;
    double rh, ah, et_r, et_a;
    double lp[8], a45, q0, ft;
};

__device__ inline double above_g45(const AboveEval &E, double z_m) { return E.a45 - 3.086e-6 * z_m; }

__device__ inline void above_init(AboveEval &E, int prof, double ray_h, double aer_h)
{
    const double P[8] = {101325.0, 22632.1, 5474.89, 868.019, 110.906, 66.9389, 3.95642, 0.3734};
    E.prof = prof; E.rh = ray_h; E.ah = aer_h;
    E.et_r = exp(-OCRT_ZTOP_KM / ray_h);
    E.et_a = exp(-OCRT_ZTOP_KM / aer_h);
    for (int i = 0; i < 8; ++i) E.lp[i] = log(P[i]);
    const double lat = 45.0 * OCRT_PI / 180.0;
    const double s1 = sin(lat) * sin(lat), s2 = sin(2.0 * lat) * sin(2.0 * lat);
    E.a45 = 9.780327 * (1.0 + 0.0053024 * s1 - 0.0000058 * s2);
    E.q0 = 101325.0 / above_g45(E, 0.0);
    E.ft = clamp01d((0.3734 / above_g45(E, 84852.0)) / E.q0);     // us62_raw(84.852)
}

__device__ inline double above_exp(double z, double h, double et)
{
    if (z <= 0.0) return 1.0;
    if (z >= OCRT_ZTOP_KM) return 0.0;
    return (exp(-z / h) - et) / (1.0 - et);
}

__device__ inline double above_ray(const AboveEval &E, double z)
{
    if (E.prof == 1) return above_exp(z, E.rh, E.et_r);
    if (z <= 0.0) return 1.0;
    if (z >= 84.852) return 0.0;
    const double Z[8] = {0.0, 11.0, 20.0, 32.0, 47.0, 51.0, 71.0, 84.852};
    int lo = 0, hi = 7;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (z < Z[mid]) hi = mid; else lo = mid;
    }
    const double t = (z - Z[lo]) / (Z[hi] - Z[lo]);
    const double a = E.lp[lo], b = E.lp[hi];
    const double raw = clamp01d((exp(a + t * (b - a)) / above_g45(E, z * 1000.0)) / E.q0);
    return clamp01d((raw - E.ft) / (1.0 - E.ft));
}

// ---- generalized spherical functions (rt_angular_basis.c:19-124) ----
__host__ __device__ inline double gsf_diag_norm(int m)
{
    double v = 1.0;
    for (int i = 1; i <= m; ++i) v *= sqrt((double)(i + m) / (double)i) * 0.5;
    return v;
}

// The x-independent coefficients of the step l -> l + 1 (l >= max(2, m)):
// c = {f, b, sc, dc, cc} of the scalar and spin-2 three-term recurrences.
__host__ __device__ inline void gsf_step_coefs(int l, int m, double *c)
{
    c[0] = (2.0 * l + 1.0) / sqrt((double)(l + m + 1) * (double)(l - m + 1));
    c[1] = sqrt((double)(l + m) * (double)(l - m)) / (2.0 * l + 1.0);
    c[2] = (double)(l + 1) * (double)(2 * l + 1) /
           sqrt((double)(l + 3) * (double)(l - 1) * (double)(l + m + 1) * (double)(l - m + 1));
    c[3] = sqrt((double)(l + 2) * (double)(l - 2) * (double)(l + m) * (double)(l - m)) /
           ((double)l * (double)(2 * l + 1));
    c[4] = 2.0 * (double)m / ((double)l * (double)(l + 1));
}

// Runs the scalar and spin-2 recurrences for one direction cosine x and
// hands every degree l = 0..L to sink(l, P, R, T).  ctab, when given, holds
// gsf_step_coefs(l, m) at ctab[5 l] (k_gsf_coefs), so the steps need no
// square root or division.
template <class Sink>
__device__ inline void gsf_recur(int L, int m, double x, Sink sink, const double *ctab = nullptr)
{
    double p0 = 0, p1 = 0, r0 = 0, r1 = 0, t0 = 0, t1 = 0;   // degree l-1 and l
    // degrees below the start are zero
    const int l0 = m < 2 ? 2 : m;
    for (int l = 0; l < l0 - 1 && l <= L; ++l) {
        double P = 0.0;
        if (m == 0) P = (l == 0) ? 1.0 : x;
        else if (m == 1 && l == 1) P = sqrt(0.5 * (1.0 - x * x));
        sink(l, P, 0.0, 0.0);
    }
    // seed values at degrees l0-1 and l0
    if (m == 0) {
        p0 = x; p1 = 0.5 * (3.0 * x * x - 1.0);
        r0 = 0.0; r1 = 3.0 * (1.0 - x * x) / (2.0 * sqrt(6.0));
        t0 = 0.0; t1 = 0.0;
    } else if (m == 1) {
        p0 = sqrt(0.5 * (1.0 - x * x)); p1 = x * p0 * sqrt(3.0);
        const double s = sqrt(1.0 - x * x);
        r0 = 0.0; r1 = -x * s * 0.5;
        t0 = 0.0; t1 = -s * 0.5;
    } else {
        const double dn = gsf_diag_norm(m);
        p0 = 0.0; p1 = dn * pow(1.0 - x * x, 0.5 * (double)m);
        const double sn = dn * sqrt((double)m / (double)(m + 1)) * sqrt((double)(m - 1) / (double)(m + 2));
        const double env = pow(1.0 - x * x, 0.5 * (double)m - 1.0);
        r0 = 0.0; r1 = sn * (1.0 + x * x) * env;
        t0 = 0.0; t1 = sn * 2.0 * x * env;
    }
    if (l0 - 1 <= L) sink(l0 - 1, p0, r0, t0);
    if (l0 <= L) sink(l0, p1, r1, t1);
    for (int l = l0; l < L; ++l) {
        double k[5];
        if (ctab) {
#pragma unroll
            for (int q = 0; q < 5; ++q) k[q] = ctab[5 * l + q];
        } else {
            gsf_step_coefs(l, m, k);
        }
        const double f = k[0], b = k[1], sc = k[2], dc = k[3], cc = k[4];
        const double p2 = f * (x * p1 - b * p0);
        const double r2 = sc * (x * r1 - cc * t1 - dc * r0);
        const double t2 = sc * (x * t1 - cc * r1 - dc * t0);
        p0 = p1; p1 = p2; r0 = r1; r1 = r2; t0 = t1; t1 = t2;
        sink(l + 1, p2, r2, t2);
    }
}

// ---- Fresnel reflection Mueller (shared/surface.c:385-420) ----
template <typename T>
__device__ inline void fresnel_R(T mu_i, T nw, int qconv, T *M)
{
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = T(0);
    const T st2 = (T(1) / nw) * (T(1) / nw) * fmax(T(0), T(1) - mu_i * mu_i);
    if (st2 >= T(1)) { M[0] = M[4] = M[8] = T(1); return; }
    const T mt = sqrt(T(1) - st2);
    const T rs = (mu_i - nw * mt) / (mu_i + nw * mt);
    const T rp = (nw * mu_i - mt) / (nw * mu_i + mt);
    const T Rs = rs * rs, Rp = rp * rp;
    const T q = qconv == 1 ? T(0.5) * (Rp - Rs) : T(0.5) * (Rs - Rp);
    M[0] = T(0.5) * (Rs + Rp); M[1] = q; M[3] = q; M[4] = T(0.5) * (Rs + Rp); M[8] = rs * rp;
}

// Water-side reflection Mueller at incidence mu_i from the water (n_w -> 1),
// identity beyond the critical angle (shared/surface.c:385-422 with n1 = n_w).
template <typename T>
__device__ inline void fresnel_R_water(T mu_i, T nw, int qconv, T *M)
{
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = T(0);
    const T st2 = nw * nw * fmax(T(0), T(1) - mu_i * mu_i);
    if (st2 >= T(1)) { M[0] = M[4] = M[8] = T(1); return; }
    const T mt = sqrt(T(1) - st2);
    const T rs = (nw * mu_i - mt) / (nw * mu_i + mt);
    const T rp = (mu_i - nw * mt) / (mu_i + nw * mt);
    const T Rs = rs * rs, Rp = rp * rp;
    const T q = qconv == 1 ? T(0.5) * (Rp - Rs) : T(0.5) * (Rs - Rp);
    M[0] = T(0.5) * (Rs + Rp); M[1] = q; M[3] = q; M[4] = T(0.5) * (Rs + Rp); M[8] = rs * rp;
}

__host__ __device__ inline double slope_variance(double ws, int sigma_type)
{
    if (sigma_type == 1) return 0.003 + 0.00512 * fmax(0.01, ws);
    const double s = 0.0731 * sqrt(fmax(0.0, ws));
    return fmax(s * s, 1e-10);
}

// d(slope variance)/d(wind speed) of slope_variance (0 where a floor is active).
__host__ __device__ inline double slope_variance_dw(double ws, int sigma_type)
{
    if (sigma_type == 1) return ws > 0.01 ? 0.00512 : 0.0;
    const double s2 = 0.0731 * 0.0731 * fmax(0.0, ws);
    return s2 > 1e-10 ? 0.0731 * 0.0731 : 0.0;
}

// Sancer shadowing term of one direction (shared/surface.c:578-598), FP64.
__device__ inline double sancer_lambda(double mu, double slen)
{
    if (!(mu < 1.0 - 1e-10)) return 0.0;
    const double s = sqrt(fmax(1e-20, 1.0 - mu * mu));
    const double nu = (mu / s) / slen;
    if (nu > 20.0) return 0.0;
    return 0.5 * (exp(-nu * nu) / (nu * sqrt(OCRT_PI)) - erfc(nu));
}

// d lambda / d s2 of sancer_lambda with slen = sqrt(s2): lambda depends on
// nu = mu / (sqrt(1 - mu^2) slen) only, dlambda/dnu = -exp(-nu^2) / (2 sqrt(pi) nu^2)
// and dnu/ds2 = -nu / (2 s2), so dlambda/ds2 = exp(-nu^2) / (4 sqrt(pi) nu s2).
__device__ inline double sancer_lambda_ds2(double mu, double slen)
{
    if (!(mu < 1.0 - 1e-10)) return 0.0;
    const double s = sqrt(fmax(1e-20, 1.0 - mu * mu));
    const double nu = (mu / s) / slen;
    if (nu > 20.0) return 0.0;
    return exp(-nu * nu) / (4.0 * sqrt(OCRT_PI) * nu * slen * slen);
}

// Cox-Munk + Fresnel reflection Mueller R(mu_out, mu_in_dn, phi)
// (shared/surface.c:514-619).  sig2 = slope variance, lam = lam_i + lam_v.
// shalf2 = sin^2(phi/2).  The facet-incidence cosine and the facet tilt are
// evaluated in the cancellation-free form
//   4 cos^2(omega) = (mu_o + mu_i)^2 + B,  tan^2(beta) = B / (mu_o + mu_i)^2,
//   B = (s_o - s_i)^2 + 4 s_o s_i sin^2(phi/2),
// algebraically identical to cos(omega) = sqrt((1 - cosTheta)/2) and
// tan^2(beta) = (1 - cos^2 beta)/cos^2 beta of the reference; near the specular
// peak the reference form loses ~eps/sigma^2 in FP32.
// water_side: the internal reflection of an upward beam at the underside of
// the surface (shared/surface.c:1136-1238): the same facet geometry, slope
// density and shadowing, with the water-to-air facet Fresnel matrix.
template <typename T>
__device__ inline void coxmunk_R(T mu_out, T mu_in_dn, T cphi, T sphi, T shalf2, T sig2, T lam,
                                 T nw, int qconv, T *R, T *tb2_out = nullptr, bool water_side = false)
{
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = T(0);
    const T mi = -mu_in_dn;
    const T s1 = sqrt(fmax(T(0), T(1) - mu_out * mu_out));
    const T s2 = sqrt(fmax(T(0), T(1) - mi * mi));
    T cT = mu_out * mi + s1 * s2 * cphi;
    cT = cT > T(1) ? T(1) : (cT < T(-1) ? T(-1) : cT);
    const T mu_sum = mu_out + mu_in_dn;
    const T A2 = mu_sum * mu_sum;
    const T Bt = (s1 - s2) * (s1 - s2) + T(4) * s1 * s2 * shalf2;
    const T cw = T(0.5) * sqrt(A2 + Bt);
    if (cw <= T(1e-6)) return;
    const T cb = mu_sum / (T(2) * cw);
    if (cb <= T(1e-6)) return;
    const T sT = sqrt(fmax(T(0), T(1) - cT * cT));
    const T den = fmax(T(1e-12), sT);
    const T pole = T(1e-8);
    T c1, si1, c2, si2;
    if (s2 <= pole) { c1 = -copysign(T(1), mi) * cphi; si1 = sphi; }
    else {
        c1 = (mu_out - mi * cT) / (den * fmax(T(1e-12), s2));
        si1 = s1 * sphi / den;
        const T nn = sqrt(c1 * c1 + si1 * si1);
        if (nn < T(1e-12)) { c1 = T(1); si1 = T(0); } else { c1 /= nn; si1 /= nn; }
    }
    if (s1 <= pole) { c2 = -copysign(T(1), mu_out) * cphi; si2 = sphi; }
    else {
        c2 = (mi - mu_out * cT) / (den * fmax(T(1e-12), s1));
        si2 = s2 * sphi / den;
        const T nn = sqrt(c2 * c2 + si2 * si2);
        if (nn < T(1e-12)) { c2 = T(1); si2 = T(0); } else { c2 /= nn; si2 /= nn; }
    }
    T MF[9];
    if (water_side) fresnel_R_water<T>(cw, nw, qconv, MF);
    else fresnel_R<T>(cw, nw, qconv, MF);
    const T cb2 = cb * cb;
    const T tb2 = Bt / A2;
    if (tb2_out) *tb2_out = tb2;
    const T Ps = (T(1) / (T(OCRT_PI) * sig2)) * exp(-tb2 / sig2);
    const T brdf = (Ps / (T(1) + lam)) / (T(4) * mu_in_dn * mu_out * cb2 * cb2);
    // R = L2 * MF * L1 * brdf with L(c,s) = [[1,0,0],[0,c2,-s2],[0,s2,c2]]
    const T a1 = c1 * c1 - si1 * si1, b1 = T(2) * c1 * si1;
    const T a2 = c2 * c2 - si2 * si2, b2 = T(2) * c2 * si2;
    // MF * L1 (MF = [[f0,f1,0],[f1,f0,0],[0,0,f8]])
    const T f0 = MF[0], f1 = MF[1], f8 = MF[8];
    const T A00 = f0, A01 = f1 * a1, A02 = -f1 * b1;
    const T A10 = f1, A11 = f0 * a1, A12 = -f0 * b1;
    const T A20 = T(0), A21 = f8 * b1, A22 = f8 * a1;
    R[0] = A00 * brdf; R[1] = A01 * brdf; R[2] = A02 * brdf;
    R[3] = (a2 * A10 - b2 * A20) * brdf; R[4] = (a2 * A11 - b2 * A21) * brdf; R[5] = (a2 * A12 - b2 * A22) * brdf;
    R[6] = (b2 * A10 + a2 * A20) * brdf; R[7] = (b2 * A11 + a2 * A21) * brdf; R[8] = (b2 * A12 + a2 * A22) * brdf;
}

// Direct sunglint reflectance (shared/surface.c:1813-1907), FP64.
__device__ inline void sunglint(const PixDev &d, double mu_v, double phi_v, double tau, double *g)
{
    const double mu0 = d.mu0;
    const double trans = exp(-tau / mu0) * exp(-tau / mu_v);
    if (d.wind < 1e-6) {
        const double fov = 0.5 * OCRT_PI / 180.0;
        const double s0 = sqrt(fmax(0.0, 1.0 - mu0 * mu0));
        const double smu = fov * fmax(s0, 1e-3), sph = fov;
        double de = phi_v;
        while (de > OCRT_PI) de -= 2.0 * OCRT_PI;
        while (de < -OCRT_PI) de += 2.0 * OCRT_PI;
        const double dm = mu_v - mu0;
        const double ex = -0.5 * (dm * dm / (smu * smu) + de * de / (sph * sph));
        if (ex < -50.0) { g[0] = g[1] = g[2] = 0.0; return; }
        double MF[9];
        fresnel_R<double>(mu0, d.n_water, d.q_conv, MF);
        const double den = fmax(2.0 * mu0 * s0 * mu0 * mu_v, 1e-12);
        const double r = 4.0 * OCRT_PI * trans / den * exp(ex);
        g[0] = MF[0] * r; g[1] = MF[3] * r; g[2] = MF[6] * r;
        return;
    }
    const double s2v = slope_variance(d.wind, d.sigma_type);
    const double lam = sancer_lambda(mu0, sqrt(s2v)) + sancer_lambda(mu_v, sqrt(s2v));
    double R[9];
    const double sh = sin(0.5 * phi_v);
    coxmunk_R<double>(mu_v, mu0, cos(phi_v), sin(phi_v), sh * sh, s2v, lam, d.n_water, d.q_conv, R);
    g[0] = OCRT_PI * R[0] * trans; g[1] = OCRT_PI * R[3] * trans; g[2] = OCRT_PI * R[6] * trans;
}
