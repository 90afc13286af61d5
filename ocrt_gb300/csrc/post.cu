// post.cu — per-pixel finalisation in FP64.
//
//   k_ipss      IPSS spherical single-scatter correction kappa and the
//               ray-traced direct-beam slant depth (rt_ipss.c:24-644), one block
//               per pixel, one thread per line-of-sight quadrature node.
//   k_finalize  Fourier reconstruction (rt_fourier.c:9-33), rho = X/mu0, kappa,
//               direct sunglint (shared/surface.c:1813-1907) and the
//               transmittance diagnostics (rt_solver.c:1100-1275).
#include "kernels.cuh"
#include "physics.cuh"

#define IPSS_RE 6371.0

// Slant optical depth from rB toward the sun; +inf when the ray meets the
// ground (shadow).  Per-shell path lengths are taken in closed form: with
// tau' = t + b and p^2 = |rB|^2 - b^2, shell j holds |tau'| in [A_j, A_j+1],
// A = sqrt(max(0, R^2 - p^2)), intersected with tau' > b.  This is the
// reference's sorted-crossing sum (rt_ipss.c:233-318) regrouped by shell.
__device__ double ipss_tau_sun(const double *he, const double *beta, int nl, double mu0, const double *rB)
{
    const double sn = sqrt(fmax(0.0, 1.0 - mu0 * mu0));
    const double un = sqrt(sn * sn + mu0 * mu0);
    const double ux = -sn / un, uz = mu0 / un;
    const double b = rB[0] * ux + rB[2] * uz;
    const double c0 = rB[0] * rB[0] + rB[1] * rB[1] + rB[2] * rB[2];
    const double dg = b * b - (c0 - IPSS_RE * IPSS_RE);
    if (dg >= 0.0) {
        const double sq = sqrt(dg);
        if (-b - sq > 1e-9 || -b + sq > 1e-9) return INFINITY;
    }
    const double p2 = c0 - b * b;
    double tau = 0.0;
    double Rlo = IPSS_RE + he[0];
    double Alo = sqrt(fmax(0.0, Rlo * Rlo - p2));
    for (int j = 0; j < nl; ++j) {
        const double Rhi = IPSS_RE + he[j + 1];
        const double d2 = Rhi * Rhi - p2;
        if (d2 > 0.0) {
            const double Ahi = sqrt(d2);
            // branch tau' in [Alo, Ahi] with tau' > b
            double len = 0.0;
            const double a1 = fmax(Alo, b);
            if (Ahi > a1) len += Ahi - a1;
            // branch tau' in [-Ahi, -Alo] with tau' > b
            const double a2 = fmax(-Ahi, b);
            if (-Alo > a2) len += -Alo - a2;
            tau += len * beta[j];
            Alo = Ahi;
        } else {
            Alo = 0.0;
        }
    }
    return tau;
}

// IPSS for one view direction (vza_deg, raa_deg) of pixel d by the whole
// block; thread 0 writes *kappa and, when tau_dir is non-null, the direct-beam
// slant depth to the surface.
__device__ void ipss_block(const PixDev &d, double vza_deg, double raa_deg, const double *h, const double *z,
                           const double *xd, const double *yd, const double *tabs, const double *mb,
                           const double *vk_th, const double *vk_p11, double *kappa,
                           double *tau_dir)
{
    extern __shared__ double sm[];
    const int nl = d.nt;
    double *he = sm;                    // [nl+1] ascending edges
    double *beta = he + nl + 1;         // [nl]
    double *wsrc = beta + nl;           // [nl]
    double *above = wsrc + nl;          // [nl+1]
    double *lt = above + nl + 1;        // [nl+1] line-of-sight crossings (ascending s)
    double *ltau = lt + nl + 1;         // [nl+1]
    int *llay = (int *)(ltau + nl + 1); // [nl+1]
    __shared__ double red[32];
    __shared__ int have_aer;
    const long long lo = d.lev_off;
    if (threadIdx.x == 0) have_aer = 0;
    __syncthreads();
    for (int k = threadIdx.x; k <= nl; k += blockDim.x) he[k] = z[lo + nl - k];
    __syncthreads();
    for (int j = threadIdx.x; j < nl; j += blockDim.x) {
        const int k = nl - 1 - j;
        const double dz = he[j + 1] - he[j];
        const double dtau = h[lo + k + 1] - h[lo + k];
        beta[j] = (dz > 0.0 && dtau > 0.0) ? dtau / dz : 0.0;
        if (xd[lo + k + 1] > 0.0) have_aer = 1;
    }
    __syncthreads();
    const double tv = vza_deg * OCRT_PI / 180.0, fp = (180.0 - raa_deg) * OCRT_PI / 180.0;
    const int use_w = have_aer && d.mom_off >= 0 && d.tau_a > 0.0;
    double PR = 1.0, PA = 1.0;
    if (use_w) {
        const double sn = sqrt(fmax(0.0, 1.0 - d.mu0 * d.mu0));
        const double ct = sn * sin(tv) * cos(fp) - d.mu0 * cos(tv);
        PR = 1.0 + (1.0 - OCRT_DEPOL) / (2.0 + OCRT_DEPOL) * 0.5 * (3.0 * ct * ct - 1.0);
        if (d.vk_n > 1 && vk_th) {
            // the value kernel's table, linear in the angle (rt_ipss.c:131-146)
            const double *th = vk_th + d.vk_off, *pv = vk_p11 + d.vk_off;
            const int n = d.vk_n;
            const double t = acos(fmax(-1.0, fmin(1.0, ct))) * 180.0 / OCRT_PI;
            if (t <= th[0]) {
                PA = pv[0];
            } else if (t >= th[n - 1]) {
                PA = pv[n - 1];
            } else {
                int lo = 0, hi = n - 1;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (th[mid] <= t) lo = mid; else hi = mid;
                }
                PA = pv[lo] + (t - th[lo]) / (th[hi] - th[lo]) * (pv[hi] - pv[lo]);
            }
        } else {
            double p0 = 1.0, p1 = ct, s = mb[d.mom_off];
            if (d.L_aer >= 1) s += mb[d.mom_off + 1] * p1;
            for (int l = 2; l <= d.L_aer; ++l) {
                const double p2 = ((2.0 * l - 1.0) * ct * p1 - (l - 1.0) * p0) / l;
                s += mb[d.mom_off + l] * p2; p0 = p1; p1 = p2;
            }
            PA = s > 0.0 ? s : 0.0;
        }
    }
    for (int j = threadIdx.x; j < nl; j += blockDim.x) {
        const int k = nl - 1 - j;
        if (use_w) {
            const double wr = yd[lo + k + 1] > 0.0 ? yd[lo + k + 1] : 0.0;
            const double wa = xd[lo + k + 1] > 0.0 ? xd[lo + k + 1] : 0.0;
            wsrc[j] = wr * PR + wa * PA;
        } else if (tabs && d.gas) {
            // the layer's scattering fraction of its extinction (rt_ipss.c:64-70)
            const double dtau = h[lo + k + 1] - h[lo + k];
            const double ta = fmin(fmax(tabs[lo + k], 0.0), dtau);
            wsrc[j] = dtau > 0.0 ? (dtau - ta) / dtau : 0.0;
        } else {
            wsrc[j] = beta[j] > 0.0 ? 1.0 : 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        above[nl] = 0.0;
        for (int j = nl - 1; j >= 0; --j) above[j] = above[j + 1] + beta[j] * (he[j + 1] - he[j]);
    }
    // line of sight, pixel anchored (rt_ipss.c:495-521): radius decreases
    // monotonically from the TOA crossing to the pixel, one crossing per shell
    const double u0 = sin(tv) * cos(fp), u1 = sin(tv) * sin(fp), u2 = cos(tv);
    const double H = he[nl], Rt = IPSS_RE + H;
    const double bq = IPSS_RE * u2;
    const double disc = bq * bq + Rt * Rt - IPSS_RE * IPSS_RE;
    const double smax = -bq + sqrt(disc);
    const double rA[3] = {smax * u0, smax * u1, IPSS_RE + smax * u2};
    const double bl = -(rA[0] * u0 + rA[1] * u1 + rA[2] * u2);
    const double c0l = rA[0] * rA[0] + rA[1] * rA[1] + rA[2] * rA[2];
    // crossing i (0 = TOA at s = 0, nl = pixel at s = smax) for shell index nl - i
    for (int i = threadIdx.x; i <= nl; i += blockDim.x) {
        if (i == 0) lt[i] = 0.0;
        else if (i == nl) lt[i] = smax;
        else {
            const double R = IPSS_RE + he[nl - i];
            lt[i] = -bl - sqrt(bl * bl - (c0l - R * R));
        }
        llay[i] = nl - 1 - i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tau = 0.0;
        for (int i = 0; i < nl; ++i) {
            ltau[i] = tau;
            tau += (lt[i + 1] - lt[i]) * beta[llay[i]];
        }
    }
    __syncthreads();
    const double xq = 1.0 / sqrt(3.0);
    double Iss = 0.0;
    for (int q = threadIdx.x; q < 2 * nl; q += blockDim.x) {
        const int i = q >> 1;
        const int j = llay[i];
        if (!(beta[j] > 0.0)) continue;
        const double sa = lt[i], sb = lt[i + 1];
        const double half = 0.5 * (sb - sa), mid = 0.5 * (sa + sb);
        const double sq = mid + half * ((q & 1) ? xq : -xq);
        const double rB[3] = {rA[0] - sq * u0, rA[1] - sq * u1, rA[2] - sq * u2};
        const double hB = sqrt(rB[0] * rB[0] + rB[1] * rB[1] + rB[2] * rB[2]) - IPSS_RE;
        if (hB < 0.0 || hB > H) continue;
        const double tview = ltau[i] + (sq - sa) * beta[j];
        const double tsun = ipss_tau_sun(he, beta, nl, d.mu0, rB);
        if (!isfinite(tsun)) continue;
        Iss += half * beta[j] * wsrc[j] * exp(-tview - tsun);
    }
    for (int o = 16; o > 0; o >>= 1) Iss += __shfl_xor_sync(0xffffffffu, Iss, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = Iss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
        const double mv = cos(tv);
        double Ipp = 0.0;
        if (mv > 0.0) {
            const double C = 1.0 / mv + 1.0 / d.mu0;
            for (int jj = 0; jj < nl; ++jj) {
                if (!(beta[jj] > 0.0)) continue;
                Ipp += wsrc[jj] / (mv * C) * (exp(-C * above[jj + 1]) - exp(-C * above[jj]));
            }
        }
        *kappa = (!(Ipp > 1.0e-300) || !isfinite(tot)) ? 1.0 : tot / Ipp;
        if (tau_dir) {
            const double r0[3] = {0.0, 0.0, IPSS_RE};
            const double td = ipss_tau_sun(he, beta, nl, d.mu0, r0);
            *tau_dir = isfinite(td) ? td : -1.0;
        }
    }
}

__global__ void k_ipss(const PixDev *px, int P, const double *h, const double *z,
                       const double *xd, const double *yd, const double *tabs,
                       const double *mb, const double *vk_th, const double *vk_p11, double *kappa, double *tau_dir)
{
    const int p = blockIdx.x;
    if (p >= P) return;
    const PixDev &d = px[p];
    if (!d.pssa) {
        if (threadIdx.x == 0) { kappa[p] = 1.0; tau_dir[p] = -1.0; }
        return;
    }
    ipss_block(d, d.vza_deg, d.raa_deg, h, z, xd, yd, tabs, mb, vk_th, vk_p11, &kappa[p], &tau_dir[p]);
}

// IPSS kappa at every (vza, raa) of each pixel's LUT grid: block (point, pixel).
__global__ void k_ipss_lut(const PixDev *px, int P, const double *h, const double *z, const double *xd,
                           const double *yd, const double *tabs, const double *mb, const double *vk_th,
                           const double *vk_p11, const double *lut_vza, const double *lut_raa, double *lut_kappa)
{
    const int p = blockIdx.y;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int npts = d.lut_nv * d.lut_nr;
    for (int pt = blockIdx.x; pt < npts; pt += gridDim.x) {
        double *kout = &lut_kappa[d.lut_oo + pt];
        if (!d.pssa) {
            if (threadIdx.x == 0) *kout = 1.0;
            continue;
        }
        const int iv = pt / d.lut_nr, ir = pt - iv * d.lut_nr;
        ipss_block(d, lut_vza[d.lut_vo + iv], lut_raa[d.lut_ro + ir], h, z, xd, yd, tabs, mb, vk_th, vk_p11, kout,
                   nullptr);
        __syncthreads();
    }
}


__global__ void k_finalize(const PixDev *px, int P, const TaskState *state, const TaskOut *tout,
                           const double *gmu, const double *gw, const double *h,
                           const double *kappa, const double *tau_dir, ocrt_result *res)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const PixDev &d = px[p];
    const int M = d.M;
    const double phi = d.raa_deg * OCRT_PI / 180.0 + OCRT_PI;
    double I = 0, Q = 0, U = 0, Dn = 0;
    int max_orders = 0, conv = 1, om = 0;
    for (int m = 0; m <= M; ++m) {
        const TaskOut &o = tout[d.task0 + m];
        const TaskState &st = state[d.task0 + m];
        const double cm = m == 0 ? 1.0 : 2.0 * cos((double)m * phi);
        const double sm = m == 0 ? 0.0 : 2.0 * sin((double)m * phi);
        I += cm * o.vI; Q += cm * o.vQ; U += sm * o.vU;
        Dn += cm * o.dn_view;
        if (st.orders > max_orders) max_orders = st.orders;
        if (!st.converged) conv = 0;
        om += st.orders;
    }
    ocrt_result r;
    memset(&r, 0, sizeof(r));
    const double mu0 = d.mu0, tau = d.tau_total;
    r.I_TOA = I; r.Q_TOA = Q; r.U_TOA = U;
    r.rho_I = I / mu0; r.rho_Q = Q / mu0; r.rho_U = U / mu0;
    r.tau_R_total = d.tau_r;
    r.kappa_ipss = 1.0;
    const double td = d.pssa ? tau_dir[p] : -1.0;
    if (d.pssa) {
        const double k = kappa[p];
        r.kappa_ipss = k;
        r.rho_I *= k; r.rho_Q *= k; r.rho_U *= k;
        r.I_TOA *= k; r.Q_TOA *= k; r.U_TOA *= k;
    }
    if (d.surface == 2) {
        const double phi_v = (d.raa_deg - 180.0) * OCRT_PI / 180.0;
        const double mv = d.vza_deg > 0.0 ? d.mu_view : 1.0;
        double g[3];
        sunglint(d, mv, phi_v, tau, g);
        if (td >= 0.0) {
            const double cg = exp(-(td - tau / mu0));
            g[0] *= cg; g[1] *= cg; g[2] *= cg;
        }
        if (!d.decouple) { r.rho_I += g[0]; r.rho_Q += g[1]; r.rho_U += -g[2]; }
        if (d.wind > 0.0) {
            r.T_sg_up_dir = g[0] * mu0;
            r.rho_glint_direct_I = g[0]; r.rho_glint_direct_Q = g[1]; r.rho_glint_direct_U = g[2];
        }
    }
    r.n_orders_used = max_orders;
    r.converged = conv;
    r.order_modes = om;
    r.T_dir_dn = td >= 0.0 ? exp(-td) : exp(-tau / mu0);
    r.T_diff_dn_hemi = 2.0 * OCRT_PI * tout[d.task0].fdn / (OCRT_PI * mu0);
    r.T_total_dn_hemi = r.T_dir_dn + r.T_diff_dn_hemi;
    r.T_diff_dn_dir = 2.0 * OCRT_PI * d.mu_view * Dn / (OCRT_PI * mu0);
    r.T_total_up_dir = r.rho_I * mu0;
    r.T_dir_up_view = exp(-tau / (d.mu_view > 0.0 ? d.mu_view : 1.0));
    res[p] = r;
}
