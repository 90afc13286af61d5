/*
 * ocean.c — FP64 restatement of the coupled atmosphere-ocean solve
 * (rt_solve_case_ocean, rt_solver.c:3468-6660, default path: rough
 * interface, diffuse-top skylight coupling, no IPSS).
 *
 * TEST INFRASTRUCTURE ONLY: part of the oracle (included by ocrt_oracle.c),
 * never linked by the product.  Paths are relative to code/OCRT_C/src/.
 *
 * Pieces:
 *   interface optics      shared/surface.c:57-454, 648-764, 1136-1238,
 *                         1476-1568 (internal reflection R_ww, air->water
 *                         T_aw, water->air T_wa, slope-integrated T_aw)
 *   Fourier kernels       shared/surface.c:1263-1402, 1583-1812
 *   coupling maps         rt_air_water_coupling.c:102-179, 244-311, 598-737
 *   in-water SOS          rt_water_rt.c:3549-7578 (build_inwater_atm
 *                         :2104-2236, diffuse-top primary :681-913,
 *                         intrefl_rough order loop rt_solver.c:2734-2921)
 *   orchestration         rt_solver.c:3468-6660
 */

/* ---------------------------------------------------------------------
 * Interface optics
 * ------------------------------------------------------------------- */
#define POLE_EPS 1.0e-8                  /* shared/surface.c:55 */

/* Snell + Fresnel amplitudes from medium n1 into n2 (surface.c:385-405). */
static int fresnel_amp(double mu_i, double n1, double n2, double *mu_t, double *rs, double *rp)
{
    const double st2 = (n1 / n2) * (n1 / n2) * fmax(0.0, 1.0 - mu_i * mu_i);
    if (st2 >= 1.0) { *mu_t = 0.0; *rs = *rp = 0.0; return 1; }
    *mu_t = sqrt(1.0 - st2);
    *rs = (n1 * mu_i - n2 * *mu_t) / (n1 * mu_i + n2 * *mu_t);
    *rp = (n2 * mu_i - n1 * *mu_t) / (n2 * mu_i + n1 * *mu_t);
    return 0;
}

/* Reflection Mueller (identity on total internal reflection), surface.c:408-422. */
static void fresnel_R_gen(double mu_i, double n1, double n2, int qc, double *M)
{
    double mt, rs, rp;
    for (int i = 0; i < 9; ++i) M[i] = 0.0;
    if (fresnel_amp(mu_i, n1, n2, &mt, &rs, &rp)) { M[0] = M[4] = M[8] = 1.0; return; }
    const double Rs = rs * rs, Rp = rp * rp;
    const double q = qc == 1 ? 0.5 * (Rp - Rs) : 0.5 * (Rs - Rp);
    M[0] = M[4] = 0.5 * (Rs + Rp); M[1] = M[3] = q; M[8] = rs * rp;
}

/* Radiance transmission Mueller (zero on TIR), surface.c:424-453. */
static void fresnel_T_rad(double mu_i, double n1, double n2, int qc, double *M)
{
    double mt, rs, rp;
    for (int i = 0; i < 9; ++i) M[i] = 0.0;
    if (fresnel_amp(mu_i, n1, n2, &mt, &rs, &rp)) return;
    const double ts = 1.0 + rs, tp = (n1 / n2) * (1.0 + rp);
    const double rf = (n2 * n2) / (n1 * n1) * (n2 * mt) / (n1 * mu_i);
    const double Ts = rf * ts * ts, Tp = rf * tp * tp;
    const double q = qc == 1 ? 0.5 * (Tp - Ts) : 0.5 * (Ts - Tp);
    M[0] = M[4] = 0.5 * (Ts + Tp); M[1] = M[3] = q; M[8] = rf * ts * tp;
}

/* Sancer shadowing term lambda(mu) for slope std sqrt(s2v). */
static double sancer_lam(double mu, double sl)
{
    if (!(mu < 1.0 - 1e-10)) return 0.0;
    const double s = sqrt(fmax(1e-20, 1.0 - mu * mu));
    const double nu = (mu / s) / sl;
    return nu <= 20.0 ? 0.5 * (exp(-nu * nu) / (nu * sqrt(PI)) - erfc(nu)) : 0.0;
}

/* Meridian-plane rotation cosines/sines with the pole limits of
 * surface.c:547-572 (incoming cosine mu_a with sine sa, outgoing mu_b, sb). */
static void rot_pair(double mu_a, double sa, double mu_b, double sb, double cT, double cphi, double sphi,
                     double *c1, double *s1, double *c2, double *s2)
{
    const double sT = sqrt(fmax(0.0, 1.0 - cT * cT)), den = fmax(1e-12, sT);
    if (sa <= POLE_EPS) { *c1 = -copysign(1.0, mu_a) * cphi; *s1 = sphi; }
    else {
        double c = (mu_b - mu_a * cT) / (den * fmax(1e-12, sa)), s = sb * sphi / den;
        const double r = sqrt(c * c + s * s);
        if (r < 1e-12) { c = 1.0; s = 0.0; } else { c /= r; s /= r; }
        *c1 = c; *s1 = s;
    }
    if (sb <= POLE_EPS) { *c2 = -copysign(1.0, mu_b) * cphi; *s2 = sphi; }
    else {
        double c = (mu_a - mu_b * cT) / (den * fmax(1e-12, sb)), s = sa * sphi / den;
        const double r = sqrt(c * c + s * s);
        if (r < 1e-12) { c = 1.0; s = 0.0; } else { c /= r; s /= r; }
        *c2 = c; *s2 = s;
    }
}

/* out = L2 . M . L1 * scale */
static void rotate_mueller(const double *M, double c1, double s1, double c2, double s2, double scale, double *out)
{
    double L1[9], L2[9], A[9], B[9];
    rot_L(c1, s1, L1);
    rot_L(c2, s2, L2);
    mul3(M, L1, A);
    mul3(L2, A, B);
    for (int i = 0; i < 9; ++i) out[i] = B[i] * scale;
}

/* Water-side internal reflection of an upward beam mu_in into the downward
 * direction mu_out (shared/surface.c:1136-1238). */
static void R_ww_mueller(double mu_out, double mu_in_dn, double cphi, double sphi,
                         double ws, int st, double nw, int qc, double *R)
{
    for (int i = 0; i < 9; ++i) R[i] = 0.0;
    const double s2v = slope_variance(ws, st);
    const double mi = -mu_in_dn;
    const double s1 = sqrt(fmax(0.0, 1.0 - mu_out * mu_out));
    const double s2 = sqrt(fmax(0.0, 1.0 - mi * mi));
    double cT = mu_out * mi + s1 * s2 * cphi;
    cT = cT > 1.0 ? 1.0 : (cT < -1.0 ? -1.0 : cT);
    const double cw = sqrt(fmax(0.0, 0.5 * (1.0 - cT)));
    if (cw <= 1e-6) return;
    const double cb = (mu_out + mu_in_dn) / (2.0 * cw);
    if (cb <= 1e-6) return;
    double c1, si1, c2, si2;
    rot_pair(mi, s2, mu_out, s1, cT, cphi, sphi, &c1, &si1, &c2, &si2);
    double MF[9];
    fresnel_R_gen(cw, nw, 1.0, qc, MF);
    const double cb2 = cb * cb, tb2 = (1.0 - cb2) / fmax(cb2, 1e-8);
    const double P = (1.0 / (PI * s2v)) * exp(-tb2 / s2v);
    const double sl = sqrt(s2v);
    const double S = 1.0 / (1.0 + sancer_lam(mu_in_dn, sl) + sancer_lam(mu_out, sl));
    rotate_mueller(MF, c1, si1, c2, si2, (P * S) / (4.0 * mu_in_dn * mu_out * cb2 * cb2), R);
}

/* Air -> water facet transmission, incident air mu_i, refracted water mu_o
 * (shared/surface.c:80-119 geometry, 1476-1568 Mueller). */
static void T_aw_mueller(double mu_i, double mu_o, double cphi, double sphi,
                         double ws, int st, double n, int qc, double *T)
{
    for (int i = 0; i < 9; ++i) T[i] = 0.0;
    const double s2v = slope_variance(ws, st);
    if (s2v <= 1e-10 || mu_i <= 1e-9 || mu_o <= 1e-9) return;
    const double si = sqrt(fmax(0.0, 1.0 - mu_i * mu_i)), so = sqrt(fmax(0.0, 1.0 - mu_o * mu_o));
    const double ix = si, iz = mu_i, ox = so * cphi, oy = so * sphi, oz = -mu_o;
    double hx = -(ix + n * ox), hy = -(n * oy), hz = -(iz + n * oz);
    const double hn = sqrt(hx * hx + hy * hy + hz * hz);
    if (hn < 1e-12) return;
    hx /= hn; hy /= hn; hz /= hn;
    if (hz < 0.0) { hx = -hx; hy = -hy; hz = -hz; }
    const double ih = ix * hx + iz * hz, oh = ox * hx + oy * hy + oz * hz;
    if (ih <= 0.0 || hz <= 1e-9) return;
    const double tan2 = (1.0 - hz * hz) / (hz * hz);
    const double D = exp(-tan2 / s2v) / (PI * s2v * hz * hz * hz * hz);
    double den = ih + n * oh;
    den *= den;
    const double sti = sqrt(fmax(0.0, 1.0 - ih * ih)), stt = sti / n;
    double Ts = 0.0, Tp = 0.0;
    if (stt < 1.0) {
        const double ctt = sqrt(fmax(0.0, 1.0 - stt * stt));
        const double rs = (ih - n * ctt) / (ih + n * ctt), rp = (n * ih - ctt) / (n * ih + ctt);
        Ts = 1.0 - rs * rs; Tp = 1.0 - rp * rp;
    }
    if (den < 1e-12) return;
    const double common = (fabs(ih) * fabs(oh)) / (mu_i * mu_o) * (n * n * D) / den;
    const double fs = common * Ts, fp = common * Tp, fsp = common * sqrt(fmax(0.0, Ts * Tp));
    double MT[9] = {0};
    const double q = qc == 1 ? 0.5 * (fp - fs) : 0.5 * (fs - fp);
    MT[0] = MT[4] = 0.5 * (fs + fp); MT[1] = MT[3] = q; MT[8] = fsp;
    /* rotations on photon propagation directions: both cosines negative,
     * azimuth shifted by pi (surface.c:1517-1524) */
    const double cr = -cphi, sr = -sphi, mis = -mu_i, mos = -mu_o;
    double cP = mis * mos + si * so * cr;
    cP = cP > 1.0 ? 1.0 : (cP < -1.0 ? -1.0 : cP);
    double c1, s1, c2, s2;
    rot_pair(mis, si, mos, so, cP, cr, sr, &c1, &s1, &c2, &s2);
    rotate_mueller(MT, c1, s1, c2, s2, 1.0, T);
}

/* Water -> air facet transmission, air outgoing mu2, water upwelling mu1
 * (shared/surface.c:648-764). */
static void T_wa_mueller(double mu2, double mu1, double cphi, double sphi,
                         double ws, int st, double n, int qc, double *T)
{
    for (int i = 0; i < 9; ++i) T[i] = 0.0;
    if (mu1 <= 1e-9 || mu2 <= 1e-9) return;
    const double s2v = slope_variance(ws, st);
    const double s1 = sqrt(fmax(0.0, 1.0 - mu1 * mu1)), s2 = sqrt(fmax(0.0, 1.0 - mu2 * mu2));
    double cP = mu1 * mu2 + s1 * s2 * cphi;
    cP = cP > 1.0 ? 1.0 : (cP < -1.0 ? -1.0 : cP);
    const double Nsq = n * n + 1.0 - 2.0 * n * cP;
    if (Nsq <= 1e-12) return;
    const double Nm = sqrt(Nsq);
    const double cb = (n * mu1 - mu2) / Nm, cw = (n - cP) / Nm;
    if (cb <= 1e-6 || cw <= 1e-6) return;
    double maf, rs, rp;
    if (fresnel_amp(cw, n, 1.0, &maf, &rs, &rp)) return;
    const double ts = 1.0 + rs, tp = n * (1.0 + rp);
    const double cb2 = cb * cb, tb2 = (1.0 - cb2) / fmax(cb2, 1e-8);
    const double P = (1.0 / (PI * s2v)) * exp(-tb2 / s2v);
    const double sl = sqrt(s2v);
    const double S = 1.0 / (1.0 + sancer_lam(mu1, sl) + sancer_lam(mu2, sl));
    const double common = (maf * maf) / (n * mu1 * mu2 * Nsq) * (P / (cb2 * cb2)) * S;
    const double fs = common * ts * ts, fp = common * tp * tp, fsp = common * ts * tp;
    double MT[9] = {0};
    const double q = qc == 1 ? 0.5 * (fp - fs) : 0.5 * (fs - fp);
    MT[0] = MT[4] = 0.5 * (fs + fp); MT[1] = MT[3] = q; MT[8] = fsp;
    double c1, si1, c2, si2;
    rot_pair(mu1, s1, mu2, s2, cP, cphi, sphi, &c1, &si1, &c2, &si2);
    rotate_mueller(MT, c1, si1, c2, si2, 1.0, T);
}

/* Slope-integrated air -> water irradiance transmittance, 101 x 101
 * trapezoid over +-6 sigma (shared/surface.c:144-179). */
static double T_aw_direct(double mu, double nw, double ws, int st)
{
    if (mu <= 1e-9) return 0.0;
    const double s2v = slope_variance(ws, st), ss = sqrt(fmax(0.0, 1.0 - mu * mu));
    if (s2v <= 1e-10) {
        const double stt = ss / nw, ctt = sqrt(fmax(0.0, 1.0 - stt * stt));
        const double rs = (mu - nw * ctt) / (mu + nw * ctt), rp = (nw * mu - ctt) / (nw * mu + ctt);
        return 1.0 - 0.5 * (rs * rs + rp * rp);
    }
    const double sg = sqrt(s2v), L = 6.0 * sg;
    const int N = 101;
    const double dz = 2.0 * L / (double)(N - 1);
    double acc = 0.0;
    for (int i = 0; i < N; ++i) {
        const double zx = -L + i * dz, wx = (i == 0 || i == N - 1) ? 0.5 : 1.0;
        const double proj = mu + zx * ss;
        if (proj <= 0.0) continue;
        for (int j = 0; j < N; ++j) {
            const double zy = -L + j * dz, wy = (j == 0 || j == N - 1) ? 0.5 : 1.0;
            const double r2 = zx * zx + zy * zy;
            const double cti = proj / sqrt(1.0 + r2);
            const double stt = sqrt(fmax(0.0, 1.0 - cti * cti)) / nw, ctt = sqrt(fmax(0.0, 1.0 - stt * stt));
            const double rs = (cti - nw * ctt) / (cti + nw * ctt), rp = (nw * cti - ctt) / (nw * cti + ctt);
            acc += wx * wy * (1.0 / (PI * s2v)) * exp(-r2 / s2v) * proj * (1.0 - 0.5 * (rs * rs + rp * rp));
        }
    }
    double t = acc * dz * dz / mu;
    return t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
}

/* All-mode azimuthal Fourier projection of an interface Mueller kernel on
 * the midpoint phi rule (surface.c:1263-1402, 1583-1812); kind 0 = R_ww,
 * 1 = T_aw (mu_o water, mu_i air), 2 = T_wa (mu_o air, mu_i water).  T_aw and
 * T_wa fold the incoming-U column sign for m > 0 (surface.c:1680-1684,
 * 1722-1729); R_ww does not.  out[m][o][i][9]. */
static void iface_fourier(int kind, const double *mu_o, int no, const double *mu_i, int ni, int M, int nphi,
                          double ws, int st, double nw, int qc, double *out)
{
    static const int cos_entry[9] = {1, 1, 0, 1, 1, 0, 0, 0, 1};
    const double dphi = 2.0 * PI / (double)nphi;
    double *cs = malloc(sizeof(double) * (size_t)nphi * (M + 1) * 2);
    for (int p = 0; p < nphi; ++p) {
        const double phi = (p + 0.5) * dphi;
        for (int m = 0; m <= M; ++m) {
            cs[((size_t)p * (M + 1) + m) * 2] = cos(m * phi);
            cs[((size_t)p * (M + 1) + m) * 2 + 1] = sin(m * phi);
        }
    }
    const size_t slab = (size_t)no * ni * 9;
    memset(out, 0, sizeof(double) * slab * (M + 1));
    for (int o = 0; o < no; ++o)
        for (int i = 0; i < ni; ++i) {
            for (int p = 0; p < nphi; ++p) {
                const double phi = (p + 0.5) * dphi;
                double R[9];
                if (kind == 0) R_ww_mueller(mu_o[o], mu_i[i], cos(phi), sin(phi), ws, st, nw, qc, R);
                else if (kind == 1) T_aw_mueller(mu_i[i], mu_o[o], cos(phi), sin(phi), ws, st, nw, qc, R);
                else T_wa_mueller(mu_o[o], mu_i[i], cos(phi), sin(phi), ws, st, nw, qc, R);
                for (int m = 0; m <= M; ++m) {
                    double *d = out + (size_t)m * slab + ((size_t)o * ni + i) * 9;
                    const double cw = cs[((size_t)p * (M + 1) + m) * 2], sw = cs[((size_t)p * (M + 1) + m) * 2 + 1];
                    for (int e = 0; e < 9; ++e) d[e] += R[e] * (cos_entry[e] ? cw : sw);
                }
            }
            for (int m = 0; m <= M; ++m) {
                const double norm = m == 0 ? 1.0 / (2.0 * PI) : 1.0 / PI;
                double *d = out + (size_t)m * slab + ((size_t)o * ni + i) * 9;
                for (int e = 0; e < 9; ++e) d[e] *= dphi * norm;
                if (kind != 0 && m > 0) { d[2] = -d[2]; d[5] = -d[5]; }
            }
        }
    free(cs);
}

/* Linear interpolation on the sorted, deduplicated copy of an unsorted node
 * set, extrapolating from the end pairs (rt_air_water_coupling.c:102-179). */
static double interp_unsorted(const double *mu, const double *v, int n, double x)
{
    if (n < 2) return n == 1 ? v[0] : 0.0;
    int ord[300];
    double ms[300], vs[300];
    for (int a = 0; a < n; ++a) ord[a] = a;
    for (int a = 1; a < n; ++a) {
        const int k = ord[a];
        int b = a - 1;
        while (b >= 0 && mu[ord[b]] > mu[k]) { ord[b + 1] = ord[b]; --b; }
        ord[b + 1] = k;
    }
    int w = 0;
    for (int a = 0; a < n; ++a) {
        if (w > 0 && fabs(mu[ord[a]] - ms[w - 1]) < 1e-12) continue;
        ms[w] = mu[ord[a]]; vs[w] = v[ord[a]]; ++w;
    }
    if (w < 2) return w == 1 ? vs[0] : 0.0;
    int hi = 1;
    while (hi < w && ms[hi] < x) hi++;
    int lo = hi - 1;
    if (hi >= w) { hi = w - 1; lo = w - 2; }
    const double t = (x - ms[lo]) / (ms[hi] - ms[lo]);
    return (1.0 - t) * vs[lo] + t * vs[hi];
}

/* Rough water -> air coupling of the upwelling 0- field into air directions
 * (rt_air_water_coupling.c:598-737): per air direction a composite water-mu
 * grid (1024-point trapezoid window of +-0.3 around the reverse-Snell
 * direction plus Gauss-Legendre 96 outside it), T_wa rows on 128 azimuths. */
static void couple_water_to_air(const double *Iw, const double *Qw, const double *Uw, const double *mu_w, int nw,
                                int M, double n, int qc, double ws, int st, const double *mu_a, int na,
                                double *Ia, double *Qa, double *Ua)
{
    enum { NWIN = 1024, NGLO = 96 };
    const double WHALF = 0.30;
    const int NTOT = NWIN + NGLO, nphi = 128;
    double xg[NGLO], wg[NGLO];
    ocrt_oracle_gauss(NGLO, xg, wg);
    double *xi = malloc(sizeof(double) * NTOT * 2), *wi = xi + NTOT;
    double *Tm = malloc(sizeof(double) * (size_t)(M + 1) * NTOT * 9);
    for (int ja = 0; ja < na; ++ja) {
        const double mua = mu_a[ja];
        if (!(mua > 0.0) || mua > 1.0) {
            for (int m = 0; m <= M; ++m) Ia[(size_t)m * na + ja] = Qa[(size_t)m * na + ja] = Ua[(size_t)m * na + ja] = 0.0;
            continue;
        }
        const double mws = sqrt(fmax(0.0, 1.0 - (1.0 - mua * mua) / (n * n)));
        double lo = mws - WHALF, hi = mws + WHALF;
        if (lo < 1e-6) lo = 1e-6;
        if (hi > 1.0 - 1e-9) hi = 1.0 - 1e-9;
        const double h = (hi - lo) / (double)(NWIN - 1);
        for (int i = 0; i < NWIN; ++i) { xi[i] = lo + h * (double)i; wi[i] = ((i == 0 || i == NWIN - 1) ? 0.5 : 1.0) * h; }
        for (int i = 0; i < NGLO; ++i) { xi[NWIN + i] = xg[i]; wi[NWIN + i] = (xg[i] > lo && xg[i] < hi) ? 0.0 : wg[i]; }
        iface_fourier(2, &mua, 1, xi, NTOT, M, nphi, ws, st, n, qc, Tm);
        for (int m = 0; m <= M; ++m) {
            const double az = m == 0 ? 2.0 * PI : PI;
            const double *T0 = Tm + (size_t)m * NTOT * 9;
            double sI = 0.0, sQ = 0.0, sU = 0.0;
            for (int i = 0; i < NTOT; ++i) {
                if (wi[i] == 0.0) continue;
                const double wj = az * xi[i] * wi[i];
                const double *T = T0 + (size_t)i * 9;
                const double vI = interp_unsorted(mu_w, Iw + (size_t)m * nw, nw, xi[i]);
                const double vQ = interp_unsorted(mu_w, Qw + (size_t)m * nw, nw, xi[i]);
                const double vU = interp_unsorted(mu_w, Uw + (size_t)m * nw, nw, xi[i]);
                sI += wj * (T[0] * vI + T[1] * vQ + T[2] * vU);
                sQ += wj * (T[3] * vI + T[4] * vQ + T[5] * vU);
                sU += wj * (T[6] * vI + T[7] * vQ + T[8] * vU);
            }
            Ia[(size_t)m * na + ja] = sI; Qa[(size_t)m * na + ja] = sQ; Ua[(size_t)m * na + ja] = sU;
        }
    }
    free(Tm); free(xi);
}

/* ---------------------------------------------------------------------
 * In-water successive orders (rt_water_rt.c:3549-7578, default path)
 * ------------------------------------------------------------------- */
#define DEPOL_WATER 0.039                 /* rt_water_rt.c:2121 */

typedef struct {
    /* inputs */
    double mu_sa, mu_va, raa;             /* air-side sun / view cosines, relative azimuth (deg) */
    double nw, F_sun, ws;
    int st, qc;
    const ocrt_ocean *oc;
    const double *top_I, *top_Q, *top_U;  /* [m][ntop] skylight transmitted into the water, F_sun-scaled */
    const double *top_mu;
    int ntop, top_mmax;
    /* outputs */
    double I_view[3], I_air[3], Ed, Eu, Ed_lvl1, Kd, Ku, tau_lvl1, z_lvl1, mu_sw, tau_max, z_max;
    int nt, n_ring, orders, conv, m_filled;
    double mu_ring[MAX_RING], w_ring[MAX_RING];
    double *up_I, *up_Q, *up_U;           /* [m][n_ring] upwelling at 0-, times F_sun / pi */
} water_t;

static double snell_down(double mu_air, double n)
{
    const double s2 = fmax(0.0, 1.0 - mu_air * mu_air) / (n * n);
    return s2 >= 1.0 ? 0.0 : sqrt(1.0 - s2);
}

/* Transport with a top boundary radiance on the downward columns and a
 * black bottom (rt_solver_integrate_bcs with a top BC, rt_layer_transport.c:107-208). */
static int transport_top(const ctx_t *c, const double *J, const double *top, double *I)
{
    const int n = c->n, nt = c->md.nt;
    for (int k = 0; k <= nt; ++k) F(I, c, k, 0) = NAN;
    for (int j = -n; j <= n; ++j) {
        if (j == 0) continue;
        const double *T = c->Tr + (size_t)RIDX(n, j) * nt;
        const double *A = c->Ca + (size_t)RIDX(n, j) * nt;
        const double *B = c->Cb + (size_t)RIDX(n, j) * nt;
        if (j > 0) {
            double run = 0.0;
            F(I, c, nt, j) = run;
            for (int k = nt - 1; k >= 0; --k) {
                const double jo = F(J, c, k, j), ji = F(J, c, k + 1, j);
                if (!isfinite(jo) || !isfinite(ji)) return -2;
                run = T[k] * run + A[k] * jo + B[k] * ji;
                F(I, c, k, j) = run;
            }
        } else {
            double run = top ? top[-j - 1] : 0.0;
            F(I, c, 0, j) = run;
            for (int k = 1; k <= nt; ++k) {
                const double jo = F(J, c, k, j), ji = F(J, c, k - 1, j);
                if (!isfinite(jo) || !isfinite(ji)) return -2;
                run = T[k - 1] * run + A[k - 1] * jo + B[k - 1] * ji;
                F(I, c, k, j) = run;
            }
        }
    }
    return 0;
}

/* Direct refracted beam with incident polarisation (1, q, 0)
 * (rt_primary_source.c:17-198 with beam_q). */
static void primary_beam_q(const ctx_t *c, const mode_t_ *md, const ocrt_aerosol *par, double bq,
                           double *JI, double *JQ, double *JU)
{
    const int n = c->n, nt = c->md.nt, m = md->m, L = md->L, nd = 2 * n + 1;
    const int mol = m <= 2;
    const double b0 = m == 0 ? c->beta0 : 0.0;
    const double p0 = md->xpl[RIDX(n, 0)], r0 = md->xrl[RIDX(n, 0)];
    double qi[2 * MAX_RING + 1], qq[2 * MAX_RING + 1], qu[2 * MAX_RING + 1];
    for (int j = -n; j <= n; ++j) {
        double a = 0.0, b = 0.0, u = 0.0;
        if (par && bq != 0.0)
            for (int l = m; l <= L && l <= par->L_max; ++l) {
                const double pj = md->P[(size_t)l * nd + RIDX(n, j)];
                const double rj = md->R[(size_t)l * nd + RIDX(n, j)], tj = md->T[(size_t)l * nd + RIDX(n, j)];
                const double rr0 = md->R[(size_t)l * nd + RIDX(n, 0)], t0 = md->T[(size_t)l * nd + RIDX(n, 0)];
                a += pj * rr0 * par->gamma[l];
                b += t0 * tj * par->zeta[l] + rr0 * rj * par->alpha[l];
                u += tj * rr0 * par->alpha[l] + rj * t0 * par->zeta[l];
            }
        qi[RIDX(n, j)] = a; qq[RIDX(n, j)] = b; qu[RIDX(n, j)] = u;
    }
    for (int k = 0; k <= nt; ++k) {
        const double beam = c->md.ch[k], x = c->md.xdel[k], y = c->md.ydel[k];
        for (int j = -n; j <= n; ++j) {
            const double pj = md->xpl[RIDX(n, j)];
            const double mi = b0 + c->beta2 * pj * p0;
            const double mq = mol ? c->gamma2 * md->xrl[RIDX(n, j)] * p0 : 0.0;
            const double mu = mol ? c->gamma2 * md->xtl[RIDX(n, j)] * p0 : 0.0;
            double vi = beam * (x * TAB(md->pfm, n, 0, j) + y * mi);
            double vq = beam * (x * TAB(md->gr, n, 0, j) + y * mq);
            double vu = -beam * (x * TAB(md->gt, n, 0, j) + y * mu);
            if (bq != 0.0) {
                vi += beam * bq * (x * qi[RIDX(n, j)] + y * (mol ? c->gamma2 * pj * r0 : 0.0));
                vq += beam * bq * (x * qq[RIDX(n, j)] + y * (mol ? c->alpha2 * md->xrl[RIDX(n, j)] * r0 : 0.0));
                vu += -beam * bq * (x * qu[RIDX(n, j)] + y * (mol ? c->alpha2 * md->xtl[RIDX(n, j)] * r0 : 0.0));
            }
            F(JI, c, k, j) = vi; F(JQ, c, k, j) = vq; F(JU, c, k, j) = vu;
        }
        F(JI, c, k, 0) = F(JQ, c, k, 0) = F(JU, c, k, 0) = NAN;
    }
}

/* First-scatter source of the transmitted skylight entering through the top:
 * every downward ring column c carries A = 2 w_c S(mu_c) attenuated by
 * exp(-h/mu_c)/2, scattered by the per-mode phase tables (table kernel) and
 * the molecular terms (rt_water_rt.c:681-913). */
static void primary_diffuse_top(const ctx_t *c, const mode_t_ *md, const water_t *W,
                                double *JI, double *JQ, double *JU)
{
    const int n = c->n, nt = c->md.nt, m = md->m;
    const int mol = m <= 2;
    const double b0m = m == 0 ? c->beta0 : 0.0, b2 = c->beta2, g2 = c->gamma2, a2 = c->alpha2;
    const double *eI = W->top_I + (size_t)m * W->ntop, *eQ = W->top_Q + (size_t)m * W->ntop,
                 *eU = W->top_U + (size_t)m * W->ntop;
    const double *xp = md->xpl + n, *xr = md->xrl + n, *xt = md->xtl + n;
    for (int cc = 1; cc <= n; ++cc) {
        const double muc = c->rm[RIDX(n, cc)], wc = c->gb[RIDX(n, cc)];
        double AI = 0.0, AQ = 0.0, AU = 0.0;
        int hit = 0;
        for (int e = 0; e < W->ntop; ++e)
            if (fabs(W->top_mu[e] - muc) < 1e-12) {
                AI = 2.0 * wc * eI[e]; AQ = 2.0 * wc * eQ[e]; AU = 2.0 * wc * eU[e]; hit = 1;
                break;
            }
        if (!hit || (AI == 0.0 && AQ == 0.0 && AU == 0.0)) {
            if (W->ntop >= 2) {
                int lo = 0;
                while (lo + 1 < W->ntop - 1 && W->top_mu[lo + 1] <= muc) ++lo;
                const double m0 = W->top_mu[lo], m1 = W->top_mu[lo + 1];
                double t = (m1 != m0) ? (muc - m0) / (m1 - m0) : 0.0;
                t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
                AI = 2.0 * wc * ((1.0 - t) * eI[lo] + t * eI[lo + 1]);
                AQ = 2.0 * wc * ((1.0 - t) * eQ[lo] + t * eQ[lo + 1]);
                AU = 2.0 * wc * ((1.0 - t) * eU[lo] + t * eU[lo + 1]);
            }
            if (AI == 0.0 && AQ == 0.0 && AU == 0.0) continue;
        }
        for (int j = -n; j <= n; ++j) {
            if (j == 0) continue;
            double sI, sQ, sU, qI, qQ, qU, uI, uQ, uU;
            if (j > 0) {
                sI = TAB(md->pfm, n, cc, -j); sQ = TAB(md->gr, n, cc, -j); sU = -TAB(md->gt, n, cc, -j);
                qI = TAB(md->gr, n, j, -cc); qQ = TAB(md->arr, n, cc, -j); qU = TAB(md->art, n, j, -cc);
                uI = -TAB(md->gt, n, j, -cc); uQ = TAB(md->art, n, cc, -j); uU = -TAB(md->att, n, cc, -j);
            } else {
                sI = TAB(md->pfm, n, cc, -j); sQ = TAB(md->gr, n, cc, -j); sU = -TAB(md->gt, n, cc, -j);
                qI = TAB(md->gr, n, -j, cc); qQ = TAB(md->arr, n, cc, -j); qU = -TAB(md->art, n, -j, cc);
                uI = TAB(md->gt, n, -j, cc); uQ = TAB(md->art, n, cc, -j); uU = -TAB(md->att, n, cc, -j);
            }
            const double xc = xp[-cc], rc = xr[-cc], tc = xt[-cc];
            const double raI = b0m + b2 * xp[j] * xc;
            const double raQ = mol ? g2 * xr[j] * xc : 0.0, raU = mol ? g2 * xt[j] * xc : 0.0;
            const double rqI = mol ? g2 * xp[j] * rc : 0.0, rqQ = mol ? a2 * xr[j] * rc : 0.0;
            const double rqU = mol ? a2 * xt[j] * rc : 0.0;
            const double ruI = mol ? -g2 * xp[j] * tc : 0.0, ruQ = mol ? -a2 * xr[j] * tc : 0.0;
            const double ruU = mol ? -a2 * xt[j] * tc : 0.0;
            for (int k = 0; k <= nt; ++k) {
                const double ch = 0.5 * exp(-c->md.h[k] / muc), xd = c->md.xdel[k], yd = c->md.ydel[k];
                F(JI, c, k, j) += ch * (AI * (xd * sI + yd * raI) + AQ * (xd * qI + yd * rqI) + AU * (xd * uI + yd * ruI));
                F(JQ, c, k, j) += ch * (AI * (xd * sQ + yd * raQ) + AQ * (xd * qQ + yd * rqQ) + AU * (xd * uQ + yd * ruQ));
                F(JU, c, k, j) += -ch * (AI * (xd * sU + yd * raU) + AQ * (xd * qU + yd * rqU) + AU * (xd * uU + yd * ruU));
            }
        }
    }
}

/* Monotone cubic (Fritsch-Carlson) on the upward 0- nodes, as the water view
 * extraction's off-node branch (rt_water_rt.c:914-1046). */
static double pchip_nodes(const double *mu, const double *y, int n, double x);

static int water_solve(water_t *W)
{
    const ocrt_ocean *oc = W->oc;
    const double nw = W->nw;
    const double mu_sw = snell_down(W->mu_sa, nw), mu_vw = snell_down(W->mu_va, nw);
    W->mu_sw = mu_sw;
    if (!(mu_sw > 0.0) || !(mu_vw > 0.0)) return -1;
    /* optical budget (rt_water_rt.c:4405-4440) */
    const double bp = oc->b_particle > 0.0 ? oc->b_particle : 0.0;
    const double b_rt = oc->b_water + bp, ext = oc->a_total + b_rt;
    if (!(ext > 0.0)) return -1;
    const double om_w = oc->b_water / ext, om_p = bp / ext;
    ocrt_aerosol par_s, *par = NULL;
    memset(&par_s, 0, sizeof(par_s));      /* moment path: no value-kernel table */
    if (bp > 0.0 && oc->beta) {
        par_s.tau_a = 0.0; par_s.ssa_a = 1.0; par_s.L_max = oc->L_particle;
        par_s.beta = oc->beta; par_s.gamma = oc->gamma; par_s.alpha = oc->alpha; par_s.zeta = oc->zeta;
        par = &par_s;
    }
    /* depth policy (rt_water_rt.c:5119-5180) or the caller's depth */
    double tau_max;
    int nt;
    if (oc->depth_m > 0.0) {
        tau_max = ext * oc->depth_m;
    } else {
        double gp = 0.0;
        if (par && par->L_max >= 1) { gp = par->beta[1] / 3.0; gp = gp > 0.999 ? 0.999 : (gp < -0.999 ? -0.999 : gp); }
        const double sb = bp + oc->b_water;
        double ge = sb > 0.0 ? bp * gp / sb : 0.0;
        ge = ge > 0.999 ? 0.999 : (ge < -0.999 ? -0.999 : ge);
        double z_req = (oc->tau_base > 0.0 ? oc->tau_base : 20.0) / ext;
        const double te = oc->a_total + b_rt * fmax(0.0, 1.0 - ge);
        if (te > 0.0) { const double ztr = -log(1.0e-8) / te; if (ztr > z_req) z_req = ztr; }
        tau_max = ext * z_req;
    }
    /* layers: Delta tau <= 0.05 (layer_dtau_target), the caller's count a floor
     * under the depth policy and exact for a fixed depth (rt_water_rt.c:5174-5179) */
    nt = (int)ceil(tau_max / 0.05);
    if (oc->n_layers_water > 0 && (oc->depth_m > 0.0 || oc->n_layers_water > nt)) nt = oc->n_layers_water;
    if (nt < 1) nt = 1;
    W->tau_max = tau_max; W->z_max = tau_max / ext; W->nt = nt;

    /* ring: Gauss nodes plus zero-weight view, nadir and sun directions
     * (rt_water_rt.c:5236-5298) */
    const int Nw = oc->n_mu_water;
    double mu_r[MAX_RING], w_r[MAX_RING];
    int nr = Nw;
    if (Nw < 2 || Nw > MAX_RING - 5) return -1;
    ocrt_oracle_gauss(Nw, mu_r, w_r);
    if (oc->view_as_node) ring_insert(mu_r, w_r, &nr, mu_vw);
    ring_insert(mu_r, w_r, &nr, 1.0);
    ring_insert(mu_r, w_r, &nr, mu_sw);
    ring_insert(mu_r, w_r, &nr, W->mu_sa);
    const int n = nr, nd = 2 * n + 1;
    W->n_ring = n;
    for (int j = 0; j < n; ++j) { W->mu_ring[j] = mu_r[j]; W->w_ring[j] = w_r[j]; }

    ctx_t *c = calloc(1, sizeof(ctx_t));
    if (!c) return -3;
    c->n = n; c->mu0 = mu_sw; c->mu_view = mu_vw;
    c->rm[RIDX(n, 0)] = -mu_sw; c->gb[RIDX(n, 0)] = 0.0;
    for (int j = 1; j <= n; ++j) {
        c->rm[RIDX(n, j)] = mu_r[j - 1]; c->rm[RIDX(n, -j)] = -mu_r[j - 1];
        c->gb[RIDX(n, j)] = c->gb[RIDX(n, -j)] = w_r[j - 1];
    }
    const double Aw = 2.0 * (1.0 - DEPOL_WATER) / (2.0 + DEPOL_WATER);
    c->beta0 = 1.0; c->beta2 = 0.5 * Aw; c->gamma2 = -Aw * sqrt(1.5); c->alpha2 = 3.0 * Aw;
    /* homogeneous medium (build_inwater_atm, rt_water_rt.c:2163-2176) */
    medium_t *md = &c->md;
    md->nt = nt; md->tau_total = tau_max;
    md->h = calloc(nt + 1, sizeof(double)); md->ch = calloc(nt + 1, sizeof(double));
    md->xdel = calloc(nt + 1, sizeof(double)); md->ydel = calloc(nt + 1, sizeof(double));
    md->z = calloc(nt + 1, sizeof(double));
    for (int k = 0; k <= nt; ++k) {
        md->h[k] = (double)k * tau_max / (double)nt;
        md->ch[k] = 0.5 * exp(-md->h[k] / mu_sw);
        md->xdel[k] = par ? om_p : 0.0; md->ydel[k] = om_w;
    }
    int rc = transport_prepare(c);
    /* incident-beam polarisation from the flat Fresnel transmission (rt_water_rt.c:5627-5641) */
    double MT[9];
    fresnel_T_rad(W->mu_sa, 1.0, nw, W->qc, MT);
    const double bq = MT[0] != 0.0 ? MT[3] / MT[0] : 0.0;
    const int Lp = par ? par->L_max : 0;
    const int Lws = Lp >= 2 ? Lp : 2;
    const int Mw = oc->m_max_water;
    const int m_loop = Mw < Lws ? Mw : Lws;
    int nphi_ww = 2 * Mw + 16;
    if (nphi_ww < 128) nphi_ww = 128;
    if (nphi_ww < 176) nphi_ww = 176;
    mode_t_ mdm;
    if (!rc) rc = mode_alloc(&mdm, n, Lws);
    const size_t cnt = (size_t)(nt + 1) * nd;
    double *buf = rc ? NULL : calloc(cnt * 15, sizeof(double));
    double *Kw = rc ? NULL : malloc(sizeof(double) * (size_t)(m_loop + 1) * n * n * 9);
    if (!rc && (!buf || !Kw)) rc = -3;
    double *mu_pos = mu_r;
    if (!rc) iface_fourier(0, mu_pos, n, mu_pos, n, m_loop, nphi_ww, W->ws, W->st, nw, W->qc, Kw);
    double Iv[3][MAX_M1] = {{0}}, Ipos0[MAX_RING] = {0}, Ineg0[MAX_RING] = {0}, lvl1[2 * MAX_RING + 1] = {0};
    W->up_I = calloc((size_t)(Mw + 1) * n * 3, sizeof(double));
    W->up_Q = W->up_I + (size_t)(Mw + 1) * n; W->up_U = W->up_Q + (size_t)(Mw + 1) * n;
    int max_orders = 0, all_conv = 1, streak = 0;
    double amp_max = 0.0;
    for (int m = 0; m <= m_loop && !rc; ++m) {
        double *Js[3] = {buf, buf + cnt, buf + 2 * cnt}, *Pr[3] = {buf + 3 * cnt, buf + 4 * cnt, buf + 5 * cnt};
        double *Tt[3] = {buf + 6 * cnt, buf + 7 * cnt, buf + 8 * cnt};
        double *Ip[3] = {buf + 9 * cnt, buf + 10 * cnt, buf + 11 * cnt};
        double *Ic[3] = {buf + 12 * cnt, buf + 13 * cnt, buf + 14 * cnt};
        mode_build(&mdm, m, c->rm, par);
        primary_beam_q(c, &mdm, par, bq, Js[0], Js[1], Js[2]);
        if (W->top_I && m <= W->top_mmax) primary_diffuse_top(c, &mdm, W, Js[0], Js[1], Js[2]);
        for (int s = 0; s < 3 && !rc; ++s) if (transport_top(c, Js[s], NULL, Pr[s])) rc = -2;
        if (rc) break;
        for (int s = 0; s < 3; ++s) { memcpy(Tt[s], Pr[s], cnt * sizeof(double)); memcpy(Ip[s], Pr[s], cnt * sizeof(double)); }
        /* order loop with the internal reflection of the previous order's
         * upwelling at the surface as the top boundary (rt_solver.c:2734-2921) */
        const double *K = Kw + (size_t)m * n * n * 9;
        int orders = 1, conv = 0;
        if (oc->max_orders_water == 1) conv = 1;
        for (int it = 2; it <= oc->max_orders_water && !rc; ++it) {
            if ((rc = ms_source(c, &mdm, Ip[0], Ip[1], Ip[2], Js[0], Js[1], Js[2]))) break;
            double tb[3][MAX_RING];
            const double az = m == 0 ? 2.0 * PI : PI;
            for (int jp = 1; jp <= n; ++jp) {
                double aI = 0.0, aQ = 0.0, aU = 0.0;
                for (int kp = 1; kp <= n; ++kp) {
                    const double iu = F(Ip[0], c, 0, kp), qu = F(Ip[1], c, 0, kp), uu = F(Ip[2], c, 0, kp);
                    const double *R = K + ((size_t)(jp - 1) * n + (kp - 1)) * 9;
                    const double wk = az * c->rm[RIDX(n, kp)] * c->gb[RIDX(n, kp)];
                    aI += wk * (R[0] * iu + R[1] * qu + R[2] * uu);
                    aQ += wk * (R[3] * iu + R[4] * qu + R[5] * uu);
                    aU += wk * (R[6] * iu + R[7] * qu + R[8] * uu);
                }
                tb[0][jp - 1] = aI; tb[1][jp - 1] = aQ; tb[2][jp - 1] = aU;
            }
            for (int s = 0; s < 3 && !rc; ++s) if (transport_top(c, Js[s], tb[s], Ic[s])) rc = -2;
            if (rc) break;
            for (int s = 0; s < 3; ++s)
                for (int k = 0; k <= nt; ++k)
                    for (int j = -n; j <= n; ++j) if (j) F(Tt[s], c, k, j) += F(Ic[s], c, k, j);
            orders = it;
            double mi = 0.0, mt = 0.0;
            for (int s = 0; s < 3; ++s) {
                const double a = sup_norm(c, Ic[s]), b = sup_norm(c, Tt[s]);
                if (a > mi) mi = a;
                if (b > mt) mt = b;
            }
            const double resid = mt > 0.0 ? mi / mt : 0.0;
            if (resid < oc->tolerance_water) { conv = 1; break; }
            /* the order just computed becomes the previous one */
            for (int s = 0; s < 3; ++s) { double *t = Ip[s]; Ip[s] = Ic[s]; Ic[s] = t; }
        }
        if (rc) break;
        if (orders > max_orders) max_orders = orders;
        if (!conv) all_conv = 0;
        /* view sample at 0- (rt_water_rt.c:6081-6138) */
        int jx = 0;
        for (int jp = 1; jp <= n; ++jp) if (fabs(mu_r[jp - 1] - mu_vw) < 1e-13) { jx = jp; break; }
        double up[3][MAX_RING];
        for (int s = 0; s < 3; ++s) for (int jp = 1; jp <= n; ++jp) up[s][jp - 1] = F(Tt[s], c, 0, jp);
        for (int s = 0; s < 3; ++s) {
            if (jx) Iv[s][m] = up[s][jx - 1];
            else if (n >= 4 && mu_vw > mu_r[0] && mu_vw < mu_r[n - 1]) Iv[s][m] = pchip_nodes(mu_r, up[s], n, mu_vw);
            else Iv[s][m] = interp_pos(mu_r, up[s], n, mu_vw);
        }
        /* mode early exit for m >= 3 (rt_water_rt.c:6148-6169) */
        double amp = fabs(Iv[0][m]);
        if (fabs(Iv[1][m]) > amp) amp = fabs(Iv[1][m]);
        if (fabs(Iv[2][m]) > amp) amp = fabs(Iv[2][m]);
        if (amp > amp_max) amp_max = amp;
        if (m >= 3 && amp_max > 0.0) {
            streak = amp < oc->tolerance_water * amp_max ? streak + 1 : 0;
            if (streak >= 2) break;
        }
        const double fsc = W->F_sun / PI;
        for (int jp = 1; jp <= n; ++jp) {
            W->up_I[(size_t)m * n + jp - 1] = up[0][jp - 1] * fsc;
            W->up_Q[(size_t)m * n + jp - 1] = up[1][jp - 1] * fsc;
            W->up_U[(size_t)m * n + jp - 1] = up[2][jp - 1] * fsc;
        }
        if (m == 0) {
            for (int jp = 1; jp <= n; ++jp) { Ipos0[jp - 1] = F(Tt[0], c, 0, jp); Ineg0[jp - 1] = F(Tt[0], c, 0, -jp); }
            for (int j = -n; j <= n; ++j) lvl1[RIDX(n, j)] = F(Tt[0], c, 1, j);
        }
    }
    if (!rc) {
        const double fsc = W->F_sun / PI;
        const double dphi = W->raa * PI / 180.0;
        W->I_view[0] = recon_cos(Iv[0], Mw, dphi) * fsc;
        W->I_view[1] = recon_cos(Iv[1], Mw, dphi) * fsc;
        W->I_view[2] = recon_sin(Iv[2], Mw, dphi) * fsc;
        double Edd = 0.0, Eud = 0.0, Ed1 = 0.0, Eu1 = 0.0;
        for (int jp = 1; jp <= n; ++jp) {
            const double mw = mu_r[jp - 1] * w_r[jp - 1];
            Eud += Ipos0[jp - 1] * mw; Edd += Ineg0[jp - 1] * mw;
            Ed1 += lvl1[RIDX(n, -jp)] * mw; Eu1 += lvl1[RIDX(n, jp)] * mw;
        }
        W->Ed = W->F_sun * mu_sw + 2.0 * PI * Edd * fsc;
        W->Eu = 2.0 * PI * Eud * fsc;
        W->tau_lvl1 = tau_max / (double)nt;
        W->z_lvl1 = W->tau_lvl1 / ext;
        W->Ed_lvl1 = W->F_sun * mu_sw * exp(-W->tau_lvl1 / mu_sw) + 2.0 * PI * Ed1 * fsc;
        const double Eu_l1 = 2.0 * PI * Eu1 * fsc;
        W->Kd = (W->Ed_lvl1 > 0.0 && W->Ed > 0.0) ? -log(W->Ed_lvl1 / W->Ed) / fmax(W->z_lvl1, 1e-12) : 0.0;
        W->Ku = (Eu_l1 > 0.0 && W->Eu > 0.0) ? -log(Eu_l1 / W->Eu) / fmax(W->z_lvl1, 1e-12) : 0.0;
        /* water-leaving radiance at the view (rt_water_rt.c:7225-7256):
         * the coupling operator at the single air view direction */
        double *Ia = calloc((size_t)(m_loop + 1) * 3, sizeof(double));
        double *node = calloc((size_t)(m_loop + 1) * n * 3, sizeof(double));
        for (int m = 0; m <= m_loop; ++m)
            for (int j = 0; j < n; ++j)
                for (int s = 0; s < 3; ++s)
                    node[((size_t)s * (m_loop + 1) + m) * n + j] =
                        (s == 0 ? W->up_I : (s == 1 ? W->up_Q : W->up_U))[(size_t)m * n + j] / fsc;
        couple_water_to_air(node, node + (size_t)(m_loop + 1) * n, node + 2 * (size_t)(m_loop + 1) * n, mu_r, n,
                            m_loop, nw, W->qc, W->ws, W->st, &W->mu_va, 1, Ia, Ia + (m_loop + 1),
                            Ia + 2 * (m_loop + 1));
        double Ivw[3][MAX_M1] = {{0}};
        for (int m = 0; m <= m_loop; ++m) {
            Ivw[0][m] = Ia[m]; Ivw[1][m] = Ia[(m_loop + 1) + m]; Ivw[2][m] = Ia[2 * (m_loop + 1) + m];
        }
        W->I_air[0] = recon_cos(Ivw[0], m_loop, dphi) * fsc;
        W->I_air[1] = recon_cos(Ivw[1], m_loop, dphi) * fsc;
        W->I_air[2] = recon_sin(Ivw[2], m_loop, dphi) * fsc;
        free(Ia); free(node);
        W->orders = max_orders; W->conv = all_conv; W->m_filled = Mw;
    }
    free(buf); free(Kw);
    mode_free(&mdm);
    free(c->Tr); free(c->Ca); free(c->Cb);
    medium_free(&c->md);
    free(c);
    return rc;
}

/* PCHIP with Fritsch-Carlson / Butland derivatives on ascending nodes. */
static double pchip_nodes(const double *mu, const double *y, int n, double x)
{
    return pchip_pos(mu, y, n, x);
}

/* ---------------------------------------------------------------------
 * Orchestration (rt_solver.c:3468-6660)
 * ------------------------------------------------------------------- */
void ocrt_oracle_ocean_default(ocrt_ocean *oc)
{
    memset(oc, 0, sizeof(*oc));
    oc->n_mu_water = 48; oc->m_max_water = 2; oc->max_orders_water = 20; oc->tolerance_water = 1e-7;
    oc->tau_base = 20.0; oc->view_as_node = 1;
}

int ocrt_oracle_solve_ocean(const ocrt_case *cs, const ocrt_opts *op, const ocrt_aerosol *aer_in,
                            const ocrt_ocean *oc, ocrt_result *out, ocrt_ocean_result *wo)
{
    if (!cs || !op || !oc || !out || !wo) return -1;
    if (cs->surface != OCRT_SURFACE_OCEAN) return -1;
    if (op->pssa) return -5;
    if (!(cs->wind_speed > 0.0)) return -5;
    if (!(oc->a_total >= 0.0) || !(oc->b_water >= 0.0) || oc->n_mu_water < 2 || oc->m_max_water < 0 ||
        oc->max_orders_water < 1 || !(oc->tolerance_water > 0.0)) return -1;
    if (oc->b_particle > 0.0 && (!oc->beta || !oc->gamma || !oc->alpha || !oc->zeta || oc->L_particle < 1)) return -1;
    memset(out, 0, sizeof(*out));
    memset(wo, 0, sizeof(*wo));
    const ocrt_aerosol *aer = (aer_in && aer_in->tau_a > 0.0) ? aer_in : NULL;
    const double nw = cs->n_water > 0.0 ? cs->n_water : 1.34;
    const double F_toa = PI, mu0 = cos(cs->sza_deg * PI / 180.0), mu_v = cos(cs->vza_deg * PI / 180.0);
    const int M = op->fourier_m_max;
    /* column depth for the direct beam (rt_solver.c:3740-3770) */
    double tau_r = 0.0;
    if (cs->pressure_hpa > 0.0)
        tau_r = op->tau_r_source == OCRT_TAU_R_FROM_INPUT ? cs->tau_r_input
                                                          : ocrt_oracle_tau_rayleigh(cs->wavelength_nm, cs->pressure_hpa);
    double tau_atm = tau_r + (aer ? aer->tau_a : 0.0);
    if (op->gas) { double tg = 0.0; ocrt_oracle_gas_tau(op->gas, cs->wavelength_nm, NULL, &tg); tau_atm += tg; }
    const double T_dir = (mu0 > 0.0 && tau_atm > 0.0) ? exp(-tau_atm / mu0) : 1.0;
    const double F_boa = F_toa * T_dir;
    if (!(tau_atm > 0.0)) return -1;

    /* pass 1: atmosphere over the rough surface with the BOA export */
    ocrt_case ca = *cs;
    ca.surface = OCRT_SURFACE_BLACK_FRESNEL_OCEAN;
    ca.n_water = nw;
    ocrt_opts oa = *op;
    oa.n_mu = oc->n_mu_water;
    atm_hooks_t hk;
    memset(&hk, 0, sizeof(hk));
    const size_t nb = (size_t)(M + 1) * (oc->n_mu_water + 1);
    double *boa = calloc(nb * 3, sizeof(double));
    hk.boa_I = boa; hk.boa_Q = boa + nb; hk.boa_U = boa + 2 * nb;
    ocrt_result r1;
    g_atm_hooks = &hk;
    int rc = solve_impl(&ca, &oa, aer, NULL, NULL, &r1, NULL);
    g_atm_hooks = NULL;
    if (rc) { free(boa); return rc; }
    const int na = hk.n;
    double mu_a[MAX_RING], w_a[MAX_RING];
    memcpy(mu_a, hk.mu, sizeof(double) * na); memcpy(w_a, hk.w, sizeof(double) * na);
    const double *bI = hk.boa_I, *bQ = hk.boa_Q, *bU = hk.boa_U;   /* [m][na] */

    /* skylight into the water: T_aw on 128 azimuths from the atmosphere ring
     * to the water Gauss grid, odd modes to the water's azimuth base
     * (rt_solver.c:4109-4225; rt_air_water_coupling.c:244-311) */
    const int Nw = oc->n_mu_water;
    double mug[MAX_RING], wg[MAX_RING];
    ocrt_oracle_gauss(Nw, mug, wg);
    double *Tk = malloc(sizeof(double) * (size_t)(M + 1) * Nw * na * 9);
    iface_fourier(1, mug, Nw, mu_a, na, M, 128, cs->wind_speed, cs->sigma_type, nw, cs->q_convention, Tk);
    double *dt = calloc((size_t)(M + 1) * Nw * 3, sizeof(double));
    double *dI = dt, *dQ = dt + (size_t)(M + 1) * Nw, *dU = dt + 2 * (size_t)(M + 1) * Nw;
    for (int m = 0; m <= M; ++m) {
        const double az = m == 0 ? 2.0 * PI : PI;
        for (int iw = 0; iw < Nw; ++iw) {
            double sI = 0.0, sQ = 0.0, sU = 0.0;
            for (int ja = 0; ja < na; ++ja) {
                const double wj = az * mu_a[ja] * w_a[ja];
                if (wj == 0.0) continue;
                const double *T = Tk + (((size_t)m * Nw + iw) * na + ja) * 9;
                const double a = bI[(size_t)m * na + ja], b = bQ[(size_t)m * na + ja], u = bU[(size_t)m * na + ja];
                sI += wj * (T[0] * a + T[1] * b + T[2] * u);
                sQ += wj * (T[3] * a + T[4] * b + T[5] * u);
                sU += wj * (T[6] * a + T[7] * b + T[8] * u);
            }
            const double sg = (m & 1) ? -1.0 : 1.0;
            dI[(size_t)m * Nw + iw] = sg * sI; dQ[(size_t)m * Nw + iw] = sg * sQ; dU[(size_t)m * Nw + iw] = sg * sU;
        }
    }
    free(Tk);
    /* diffuse irradiances at the surface (rt_solver.c:4258-4357) */
    double Ed_sky_w = 0.0, Ed_sky_a = 0.0;
    for (int j = 0; j < na; ++j) {
        const double muL = w_a[j] * mu_a[j] * bI[j];
        Ed_sky_w += muL * T_aw_direct(mu_a[j], nw, cs->wind_speed, cs->sigma_type);
        Ed_sky_a += muL;
    }
    Ed_sky_w *= 2.0 * PI * (F_toa / PI);
    Ed_sky_a *= 2.0 * PI * (F_toa / PI);
    /* refracted direct beam (rt_solver.c:4603-4646) */
    const double mu_sw = snell_down(mu0, nw);
    double Taw = T_aw_direct(mu0, nw, cs->wind_speed, cs->sigma_type);
    Taw = Taw < 0.0 ? 0.0 : (Taw > 1.0 ? 1.0 : Taw);
    const double F_w = F_boa * mu0 * Taw / mu_sw;
    const double dts = F_toa / F_w;
    for (size_t z = 0; z < (size_t)(M + 1) * Nw * 3; ++z) dt[z] *= dts;

    /* pass 2: the water column */
    water_t W;
    memset(&W, 0, sizeof(W));
    W.mu_sa = mu0; W.mu_va = mu_v; W.raa = cs->raa_deg; W.nw = nw; W.F_sun = F_w; W.ws = cs->wind_speed;
    W.st = cs->sigma_type; W.qc = cs->q_convention; W.oc = oc;
    W.top_I = dI; W.top_Q = dQ; W.top_U = dU; W.top_mu = mug; W.ntop = Nw; W.top_mmax = M;
    rc = water_solve(&W);
    if (rc) { free(boa); free(dt); free(W.up_I); return rc; }

    /* water-leaving radiance on the atmosphere ring (rt_solver.c:5071-5122) */
    const int msrc = M < W.m_filled ? M : W.m_filled;
    double *wl = calloc((size_t)(M + 1) * na * 3, sizeof(double));
    {
        const int mf = W.m_filled;
        double *Iu = W.up_I, *Qu = W.up_Q, *Uu = W.up_U;
        double *tmp = calloc((size_t)(msrc + 1) * na * 3, sizeof(double));
        /* the water field is stored [m][n_ring] for modes 0..mf; pass modes 0..msrc */
        (void)mf;
        couple_water_to_air(Iu, Qu, Uu, W.mu_ring, W.n_ring, msrc, nw, cs->q_convention, cs->wind_speed,
                            cs->sigma_type, mu_a, na, tmp, tmp + (size_t)(msrc + 1) * na, tmp + 2 * (size_t)(msrc + 1) * na);
        for (int s = 0; s < 3; ++s)
            memcpy(wl + (size_t)s * (M + 1) * na, tmp + (size_t)s * (msrc + 1) * na, sizeof(double) * (msrc + 1) * na);
        free(tmp);
    }
    /* pass 3: atmosphere driven by the water-leaving bottom source */
    memset(&hk, 0, sizeof(hk));
    hk.bottom_only = 1;
    hk.ext_I = wl; hk.ext_Q = wl + (size_t)(M + 1) * na; hk.ext_U = wl + 2 * (size_t)(M + 1) * na;
    hk.ext_mmax = M;
    ocrt_result r3;
    g_atm_hooks = &hk;
    rc = solve_impl(&ca, &oa, aer, NULL, NULL, &r3, NULL);
    g_atm_hooks = NULL;
    free(wl);
    if (rc) { free(boa); free(dt); free(W.up_I); return rc; }

    /* assembly (rt_solver.c:6314-6647) */
    const double rho_f = PI / (F_toa * mu0);
    out->I_TOA = r1.I_TOA + r3.I_TOA; out->Q_TOA = r1.Q_TOA + r3.Q_TOA; out->U_TOA = r1.U_TOA + r3.U_TOA;
    wo->rho_atm_I = r1.I_TOA / mu0; wo->rho_atm_Q = r1.Q_TOA / mu0; wo->rho_atm_U = r1.U_TOA / mu0;
    wo->rho_water_I = r3.I_TOA * rho_f; wo->rho_water_Q = r3.Q_TOA * rho_f; wo->rho_water_U = r3.U_TOA * rho_f;
    out->rho_I = wo->rho_atm_I + wo->rho_water_I;
    out->rho_Q = wo->rho_atm_Q + wo->rho_water_Q;
    out->rho_U = wo->rho_atm_U + wo->rho_water_U;
    out->tau_R_total = r1.tau_R_total;
    out->kappa_ipss = 1.0;
    out->T_dir_dn = T_dir;
    out->T_diff_dn_hemi = r1.T_diff_dn_hemi;
    out->T_total_dn_hemi = out->T_dir_dn + out->T_diff_dn_hemi;
    out->T_diff_dn_dir = r1.T_diff_dn_dir;
    out->T_dir_up_view = exp(-tau_atm / (mu_v > 0.0 ? mu_v : 1.0));
    out->n_orders_used = W.orders;
    out->converged = W.conv;
    out->order_modes = r1.order_modes + r3.order_modes;
    {
        const double phi_v = (cs->raa_deg - 180.0) * PI / 180.0, mvg = cs->vza_deg > 0.0 ? mu_v : 1.0;
        double g[3];
        sunglint_rho(mvg, phi_v, mu0, cs->wind_speed, cs->sigma_type, nw, tau_atm, cs->q_convention, g);
        out->rho_glint_direct_I = g[0]; out->rho_glint_direct_Q = g[1]; out->rho_glint_direct_U = -g[2];
        out->T_sg_up_dir = g[0] * mu0;
    }
    wo->Lu_0minus_I = W.I_view[0]; wo->Lu_0minus_Q = W.I_view[1]; wo->Lu_0minus_U = W.I_view[2];
    wo->Lu_0plus_I = W.I_air[0]; wo->Lu_0plus_Q = W.I_air[1]; wo->Lu_0plus_U = W.I_air[2];
    wo->Ed_0minus = W.Ed + Ed_sky_w;
    wo->Eu_0minus = W.Eu;
    wo->Ed_0plus = F_boa * mu0 + Ed_sky_a;
    wo->Ed_0minus_direct = F_w * mu_sw;
    wo->Ed_0plus_direct = F_boa * mu0;
    wo->Rrs_0plus_I = W.I_air[0] / wo->Ed_0plus; wo->Rrs_0plus_Q = W.I_air[1] / wo->Ed_0plus;
    wo->Rrs_0plus_U = W.I_air[2] / wo->Ed_0plus;
    wo->rrs_0minus_I = W.I_view[0] / wo->Ed_0minus; wo->rrs_0minus_Q = W.I_view[1] / wo->Ed_0minus;
    wo->rrs_0minus_U = W.I_view[2] / wo->Ed_0minus;
    /* Kd with the unscattered skylight re-added (rt_solver.c:3419-3466) */
    wo->Kd_0minus = W.Kd;
    {
        double q0 = 0.0, q1 = 0.0;
        for (int c = 0; c < Nw; ++c) {
            const double I0 = dI[c];
            if (!(mug[c] > 0.0) || !(wg[c] > 0.0) || !isfinite(I0)) continue;
            q0 += I0 * mug[c] * wg[c];
            q1 += I0 * mug[c] * wg[c] * exp(-W.tau_lvl1 / mug[c]);
        }
        if (q0 > 0.0 && q1 > 0.0 && W.Ed_lvl1 > 0.0 && W.tau_lvl1 > 0.0 && W.z_lvl1 > 0.0) {
            const double sc = 2.0 * PI * (F_w / PI);
            const double E0 = W.Ed + sc * q0, E1 = W.Ed_lvl1 + sc * q1;
            if (E0 > 0.0 && E1 > 0.0) {
                const double kd = -log(E1 / E0) / W.z_lvl1;
                if (isfinite(kd)) wo->Kd_0minus = kd;
            }
        }
    }
    wo->Ku_0minus = W.Ku;
    wo->tau_water = W.tau_max; wo->depth_water_m = W.z_max;
    wo->n_layers_water = W.nt; wo->n_ring_water = W.n_ring;
    wo->orders_water = W.orders; wo->converged_water = W.conv;
    free(boa); free(dt); free(W.up_I);
    return 0;
}
