// mie.cu — aerosol models from .mie tables (host code, FP64).
//
//   ocrt_gb_mie_read      read_mie_file                 shared/mie_io.c:174-327
//   ocrt_gb_mie_prepare   rt_aerosol_runtime_prepare    rt_aerosol_runtime.c:13-285
//     spectral AOD / SSA  linterp                       shared/numerics.c:55-67
//     phase in wavelength pchip_interp                  shared/numerics.c:71-131
//     truncation          rt_aerosol_loglin_truncate    rt_aerosol.c:403-552
//     moments             rt_aerosol_compute_vector_legendre  rt_aerosol.c:119-213, 649-774
//                         rt_phase_spin2_m0 / _complete_spherical / _normalize_vector
//                                                       rt_phase_moments.c:6-94
//
// The preparation runs once per (model, wavelength) on the host, as in the
// reference; its outputs are the moment expansion the SOS engine takes and
// the angle-space phase table its value kernel integrates on the device.
// Interpolation and quadrature follow the reference's steps (the published
// Fritsch-Carlson PCHIP, trapezoid rules on a PCHIP-densified angle grid, the
// Legendre and spin-2 recurrences) so that the moments agree with it to
// rounding.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/ocrt_gb300.h"

int ocrt_internal_fail(int rc, const char *msg);

struct ocrt_mie {
    int n_ang = 0, n_wl = 0, n_pw = 0;
    std::vector<double> wl;        // [n_wl] um, spectral grid
    std::vector<double> pwl;       // [n_pw] um, phase grid
    std::vector<double> ang;       // [n_ang] degrees, file order
    std::vector<double> spec;      // [n_wl][6]
    std::vector<double> P11, P12, P33;   // [n_ang][n_pw]
};

struct ocrt_mie_aerosol {
    std::vector<double> beta, gamma, alpha, zeta;
    std::vector<double> theta, p11, p12, p33;
};

namespace {

constexpr double kPi = 3.14159265358979323846;

bool numeric_start(const char *s)
{
    while (*s && std::isspace((unsigned char)*s)) ++s;
    return *s && (std::isdigit((unsigned char)*s) || *s == '-' || *s == '+' || *s == '.');
}

// Leading numbers of a line (at most max_count); stops at the first token
// that does not start like a number.
int leading_numbers(const char *s, double *out, int max_count)
{
    int n = 0;
    while (*s && n < max_count) {
        while (*s && std::isspace((unsigned char)*s)) ++s;
        if (!*s || !(std::isdigit((unsigned char)*s) || *s == '-' || *s == '+' || *s == '.')) break;
        char *end = nullptr;
        const double v = std::strtod(s, &end);
        if (end == s) break;
        out[n++] = v;
        s = end;
    }
    return n;
}

// Linear interpolation on ascending x, clamped to the end values.
double lin_interp(const double *x, const double *y, int n, double xq)
{
    if (n == 0) return 0.0;
    if (n == 1 || xq <= x[0]) return y[0];
    if (xq >= x[n - 1]) return y[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] <= xq) lo = mid; else hi = mid;
    }
    const double t = (xq - x[lo]) / (x[hi] - x[lo]);
    return y[lo] + t * (y[hi] - y[lo]);
}

// Fritsch-Carlson slopes: weighted harmonic mean of the neighbouring secants
// inside, the shape-preserving three-point formula at the ends.
double edge_slope(double h0, double h1, double d0, double d1)
{
    const double m = ((2.0 * h0 + h1) * d0 - h0 * d1) / (h0 + h1);
    if (m * d0 <= 0.0) return 0.0;
    if (d0 * d1 <= 0.0 && std::fabs(m) > 3.0 * std::fabs(d0)) return 3.0 * d0;
    return m;
}

double inner_slope(double hm, double hp, double dm, double dp)
{
    if (dm * dp <= 0.0) return 0.0;
    const double w1 = 2.0 * hp + hm, w2 = hp + 2.0 * hm;
    return (w1 + w2) / (w1 / dm + w2 / dp);
}

double node_slope(const double *x, const double *y, int n, int k)
{
    if (n == 2) return (y[1] - y[0]) / (x[1] - x[0]);
    if (k == 0) return edge_slope(x[1] - x[0], x[2] - x[1], (y[1] - y[0]) / (x[1] - x[0]), (y[2] - y[1]) / (x[2] - x[1]));
    if (k == n - 1)
        return edge_slope(x[n - 1] - x[n - 2], x[n - 2] - x[n - 3], (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]),
                          (y[n - 2] - y[n - 3]) / (x[n - 2] - x[n - 3]));
    const double dm = (y[k] - y[k - 1]) / (x[k] - x[k - 1]), dp = (y[k + 1] - y[k]) / (x[k + 1] - x[k]);
    if (dm == 0.0 || dp == 0.0) return 0.0;
    return inner_slope(x[k] - x[k - 1], x[k + 1] - x[k], dm, dp);
}

double hermite(double ylo, double yhi, double mlo, double mhi, double h, double t)
{
    const double t2 = t * t, t3 = t2 * t;
    return (2.0 * t3 - 3.0 * t2 + 1.0) * ylo + (t3 - 2.0 * t2 + t) * h * mlo + (-2.0 * t3 + 3.0 * t2) * yhi +
           (t3 - t2) * h * mhi;
}

// One PCHIP value (slopes of the bracketing nodes only), clamped outside.
double pchip_point(const double *x, const double *y, int n, double xq)
{
    if (n <= 0) return 0.0;
    if (n == 1 || xq <= x[0]) return y[0];
    if (xq >= x[n - 1]) return y[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] <= xq) lo = mid; else hi = mid;
    }
    const double h = x[hi] - x[lo];
    if (!(h > 0.0)) return lin_interp(x, y, n, xq);
    return hermite(y[lo], y[hi], node_slope(x, y, n, lo), node_slope(x, y, n, hi), h, (xq - x[lo]) / h);
}

// PCHIP through a whole table, evaluated many times (extrapolates with the
// end cubics).
struct Pchip {
    std::vector<double> x, y, m;
    bool build(const double *xs, const double *ys, int n)
    {
        if (n < 3) return false;
        x.assign(xs, xs + n);
        y.assign(ys, ys + n);
        m.assign(n, 0.0);
        std::vector<double> d(n - 1), h(n - 1);
        for (int k = 0; k < n - 1; ++k) {
            h[k] = x[k + 1] - x[k];
            d[k] = (y[k + 1] - y[k]) / h[k];
        }
        for (int k = 1; k < n - 1; ++k) m[k] = inner_slope(h[k - 1], h[k], d[k - 1], d[k]);
        m[0] = edge_slope(h[0], h[1], d[0], d[1]);
        m[n - 1] = edge_slope(h[n - 2], h[n - 3], d[n - 2], d[n - 3]);
        return true;
    }
    double operator()(double xq) const
    {
        const int n = (int)x.size();
        int lo = 0, hi = n - 1;
        if (xq <= x[0]) { lo = 0; hi = 1; }
        else if (xq >= x[n - 1]) { lo = n - 2; hi = n - 1; }
        else {
            while (hi - lo > 1) {
                const int mid = (lo + hi) / 2;
                if (x[mid] <= xq) lo = mid; else hi = mid;
            }
        }
        const double h = x[hi] - x[lo];
        return hermite(y[lo], y[hi], m[lo], m[hi], h, (xq - x[lo]) / h);
    }
};

bool full_range(const double *th, int n)
{
    if (!th || n < 2) return false;
    double lo = th[0], hi = th[0];
    for (int i = 1; i < n; ++i) { lo = std::min(lo, th[i]); hi = std::max(hi, th[i]); }
    return lo <= 0.5 && hi >= 179.5;
}

// Table in ascending angle (reversed when given descending, then a stable
// insertion pass for anything left out of order).
void ascending(const double *th, const double *p, int n, std::vector<double> &ts, std::vector<double> &ps)
{
    bool asc = true;
    for (int i = 1; i < n; ++i) if (th[i] < th[i - 1]) { asc = false; break; }
    ts.resize(n);
    ps.resize(n);
    for (int i = 0; i < n; ++i) {
        ts[i] = asc ? th[i] : th[n - 1 - i];
        ps[i] = asc ? p[i] : p[n - 1 - i];
    }
    if (asc) return;
    for (int i = 1; i < n; ++i) {
        if (ts[i] < ts[i - 1]) {
            const double t = ts[i], v = ps[i];
            int j = i - 1;
            while (j >= 0 && ts[j] > t) { ts[j + 1] = ts[j]; ps[j + 1] = ps[j]; --j; }
            ts[j + 1] = t; ps[j + 1] = v;
        }
    }
}

// chi_l = (2l + 1) / 2 int P(mu) P_l(mu) dmu for l < n_max: P densified by
// PCHIP in angle onto `fine` uniform angles over 0..180 degrees, trapezoid
// in mu, Legendre polynomials by their three-term recurrence.
bool legendre_moments(const double *P, const double *th, int n, int n_max, int fine, double *chi)
{
    if (!full_range(th, n)) return false;
    std::vector<double> ts, ps;
    ascending(th, P, n, ts, ps);
    Pchip f;
    if (!f.build(ts.data(), ps.data(), n)) return false;
    std::vector<double> mu(fine), pf(fine), pl(fine, 1.0), plm(fine, 0.0);
    for (int i = 0; i < fine; ++i) {
        const double t = 180.0 * (fine - 1 - i) / (double)(fine - 1);
        mu[i] = std::cos(t * kPi / 180.0);
        pf[i] = f(t);
    }
    for (int l = 0; l < n_max; ++l) {
        double sum = 0.0, prev = pf[0] * pl[0];
        for (int i = 1; i < fine; ++i) {
            const double cur = pf[i] * pl[i];
            sum += 0.5 * (mu[i] - mu[i - 1]) * (cur + prev);
            prev = cur;
        }
        chi[l] = (2.0 * l + 1.0) * 0.5 * sum;
        if (l + 1 < n_max) {
            for (int i = 0; i < fine; ++i) {
                const double nx = ((2.0 * l + 1.0) * mu[i] * pl[i] - (double)l * plm[i]) / (double)(l + 1);
                plm[i] = pl[i];
                pl[i] = nx;
            }
        }
    }
    return true;
}

// Generalised spherical function P^l_{0,2}(mu) for l = 0 .. L (zero below 2).
void spin2_m0(int L, double mu, double *out)
{
    out[0] = 0.0;
    if (L == 0) return;
    out[1] = 0.0;
    if (L == 1) return;
    out[2] = 3.0 * (1.0 - mu * mu) / (2.0 * std::sqrt(6.0));
    for (int l = 2; l < L; ++l) {
        const double a = (2.0 * l + 1.0) / std::sqrt((double)(l - 1) * (l + 3));
        const double b = std::sqrt((double)(l - 2) * (l + 2)) / (2.0 * l + 1.0);
        out[l + 1] = a * (mu * out[l] - b * out[l - 1]);
    }
}

// gamma_l = (2l + 1) / 2 int P12 P^l_{0,2} dmu on the densified grid of the
// tabulated angle range; per-node trapezoid weights (half spans in mu).
bool spin2_moments(const double *P12, const double *th, int n, int L, int fine, double *gam)
{
    std::vector<double> ts, ps;
    bool asc = true;
    for (int i = 1; i < n; ++i) if (th[i] < th[i - 1]) { asc = false; break; }
    ts.resize(n); ps.resize(n);
    for (int i = 0; i < n; ++i) { ts[i] = asc ? th[i] : th[n - 1 - i]; ps[i] = asc ? P12[i] : P12[n - 1 - i]; }
    Pchip f;
    if (!f.build(ts.data(), ps.data(), n)) return false;
    std::vector<double> mu(fine), val(fine), pol(L + 1);
    const double dt = (ts[n - 1] - ts[0]) / (fine - 1);
    for (int i = 0; i < fine; ++i) {
        const double t = ts[0] + i * dt;
        const int j = fine - 1 - i;
        mu[j] = std::cos(t * kPi / 180.0);
        val[j] = f(t);
    }
    for (int l = 0; l <= L; ++l) gam[l] = 0.0;
    for (int i = 0; i < fine; ++i) {
        spin2_m0(L, mu[i], pol.data());
        const double w = i == 0 ? (mu[1] - mu[0]) * 0.5
                       : i == fine - 1 ? (mu[fine - 1] - mu[fine - 2]) * 0.5
                                       : (mu[i + 1] - mu[i - 1]) * 0.5;
        for (int l = 0; l <= L; ++l) gam[l] += val[i] * pol[l] * w;
    }
    for (int l = 0; l <= L; ++l) gam[l] *= (2.0 * l + 1.0) * 0.5;
    return true;
}

// alpha, zeta (the two diagonal spin-2 families) from the Legendre moments
// of P11 (= P22) and P33: the closed sums over lower orders of rt_phase_moments.c:24-73.
void complete_spherical(int L, const double *b11, const double *b22, const double *d33, double *alpha,
                        double *zeta)
{
    for (int l = 0; l <= L; ++l) { alpha[l] = 0.0; zeta[l] = 0.0; }
    for (int l = 2; l <= L; ++l) {
        const double e = (double)l;
        const double lower = e * (e - 1.0) / ((e + 1.0) * (e + 2.0));
        const double coup = 4.0 * (2.0 * e + 1.0) / (e * (e - 1.0) * (e + 1.0) * (e + 2.0));
        const double base = (e - 1.0) * (e - 1.0);
        double sb = 0.0, sd = 0.0, ob = 0.0, od = 0.0;
        for (int k = l - 1; k >= 0; --k) {
            const int gap = l - k;
            const double w = base - 1.5 * (double)(gap - 1) * (double)(l + k);
            if ((gap & 1) == 0) { sb += w * b11[k]; sd += w * d33[k]; }
            else { ob += w * b22[k]; od += w * d33[k]; }
        }
        zeta[l] = lower * d33[l] - coup * (sd - ob);
        alpha[l] = lower * b11[l] - coup * (sb - od);
    }
}

// Real-angle log10-linear forward-peak truncation: below theta2 = acos(mu2)
// P11 follows the log10-linear continuation through its values at theta1 =
// acos(mu1) and theta2 (both linearly interpolated), P12 and P33 take the
// same ratio; A = 2 (1 - beta_0 of the truncated P11), no truncation when
// A < threshold or the anchors are unusable.
void loglin_truncate(const double *P11, const double *P12, const double *P33, const double *th, int n, double mu1,
                     double mu2, double thresh, double *o11, double *o12, double *o33, double *A_out)
{
    auto copy = [&]() {
        for (int i = 0; i < n; ++i) { o11[i] = P11[i]; o12[i] = P12[i]; o33[i] = P33[i]; }
        *A_out = 0.0;
    };
    bool asc = true;
    for (int i = 1; i < n; ++i) if (th[i] < th[i - 1]) { asc = false; break; }
    std::vector<double> ts(n), p(n);
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) {
        const int j = asc ? i : n - 1 - i;
        ts[i] = th[j]; p[i] = P11[j]; idx[i] = j;
    }
    const double t1 = std::acos(mu1) * 180.0 / kPi, t2 = std::acos(mu2) * 180.0 / kPi;
    int k1 = 0, k2 = 0;
    while (k1 < n && ts[k1] < t1) ++k1;
    while (k2 < n && ts[k2] < t2) ++k2;
    if (k1 >= n || k1 == 0 || k2 >= n || k2 == 0 || k1 <= k2 + 1) { copy(); return; }
    const double a1 = (t1 - ts[k1 - 1]) / (ts[k1] - ts[k1 - 1]);
    const double a2 = (t2 - ts[k2 - 1]) / (ts[k2] - ts[k2 - 1]);
    const double p1 = (1.0 - a1) * p[k1 - 1] + a1 * p[k1];
    const double p2 = (1.0 - a2) * p[k2 - 1] + a2 * p[k2];
    if (p1 <= 0.0 || p2 <= 0.0) { copy(); return; }
    const double r1 = t1 * kPi / 180.0, r2 = t2 * kPi / 180.0;
    const double slope = (std::log10(p2) - std::log10(p1)) / (r2 - r1);
    const double x2 = std::log10(p2);
    std::vector<double> pt(n);
    for (int i = 0; i < n; ++i)
        pt[i] = i < k2 ? std::pow(10.0, x2 + slope * (ts[i] * kPi / 180.0 - r2)) : p[i];
    double chi0 = 0.0;
    if (!legendre_moments(pt.data(), ts.data(), n, 1, 3601, &chi0)) { copy(); return; }
    const double A = 2.0 * (1.0 - chi0);
    if (A < thresh) { copy(); return; }
    for (int i = 0; i < n; ++i) {
        const int o = idx[i];
        const double ratio = p[i] > 0.0 ? pt[i] / p[i] : 1.0;
        o11[o] = pt[i];
        o12[o] = P12[o] * ratio;
        o33[o] = P33[o] * ratio;
    }
    *A_out = A;
}

bool read_lines(const char *path, std::vector<std::string> &lines)
{
    std::ifstream f(path);
    if (!f) return false;
    std::string s;
    while (std::getline(f, s)) {
        while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
        lines.push_back(s);
    }
    return true;
}

bool covers(const std::vector<double> &g, double x)
{
    if (g.size() < 2 || !std::isfinite(x)) return false;
    double lo = g.front(), hi = g.back();
    if (lo > hi) std::swap(lo, hi);
    return x >= lo - 1.0e-12 && x <= hi + 1.0e-12;
}

} // namespace

extern "C" {

void ocrt_mie_opts_default(ocrt_mie_opts *o)
{
    if (!o) return;
    o->L_max = 80;
    o->use_loglin_trunc = 1;
    o->loglin_mu1 = 0.8;
    o->loglin_mu2 = 0.94;
    o->loglin_threshold = 0.1;
    o->use_value_kernel = 1;
}

int ocrt_gb_mie_read(const char *path, ocrt_mie **out)
{
    if (!path || !out) return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: null argument");
    *out = nullptr;
    std::vector<std::string> raw;
    if (!read_lines(path, raw)) return ocrt_internal_fail(OCRT_ERR_ARGS, (std::string("mie: cannot open ") + path).c_str());
    auto m = new ocrt_mie();
    auto bad = [&](const char *why) {
        delete m;
        return ocrt_internal_fail(OCRT_ERR_ARGS, (std::string("mie: ") + path + ": " + why).c_str());
    };
    // angle count: the first line that starts like a number
    size_t p = 0;
    for (; p < raw.size(); ++p)
        if (!raw[p].empty() && numeric_start(raw[p].c_str())) { m->n_ang = std::atoi(raw[p].c_str()); ++p; break; }
    if (m->n_ang <= 0) return bad("no angle count");
    std::vector<std::string> L(raw.begin() + p, raw.end());
    size_t i = 0;
    while (i < L.size() && L[i].empty()) ++i;
    while (i < L.size() && numeric_start(L[i].c_str())) ++i;
    while (i < L.size() && !numeric_start(L[i].c_str())) ++i;
    const size_t s0 = i;
    while (i < L.size() && numeric_start(L[i].c_str())) ++i;
    m->n_wl = (int)(i - s0);
    if (m->n_wl <= 0) return bad("no spectral rows");
    // separate phase grid: a TETA line before the first phase row
    std::vector<double> teta(1024);
    m->n_pw = m->n_wl;
    bool have_teta = false;
    for (size_t j = i; j < L.size(); ++j) {
        const char *s = L[j].c_str();
        while (*s == ' ' || *s == '\t') ++s;
        if (std::strncmp(s, "TETA", 4) == 0) {
            const int nt = leading_numbers(s + 4, teta.data(), 1024);
            if (nt > 0) { m->n_pw = nt; have_teta = true; }
            break;
        }
        if (numeric_start(s)) break;
    }
    m->wl.resize(m->n_wl);
    m->spec.resize((size_t)m->n_wl * 6);
    for (int l = 0; l < m->n_wl; ++l) {
        double row[8];
        if (leading_numbers(L[s0 + l].c_str(), row, 7) < 7) return bad("short spectral row");
        m->wl[l] = row[0];
        for (int c = 0; c < 6; ++c) m->spec[(size_t)l * 6 + c] = row[c + 1];
    }
    m->pwl.resize(m->n_pw);
    for (int l = 0; l < m->n_pw; ++l) m->pwl[l] = have_teta ? teta[l] : m->wl[l];
    m->ang.resize(m->n_ang);
    std::vector<double> *blocks[3] = {&m->P11, &m->P12, &m->P33};
    for (auto *b : blocks) b->assign((size_t)m->n_ang * m->n_pw, 0.0);
    std::vector<double> row(m->n_pw + 1);
    int found = 0;
    while (i < L.size() && found < 3) {
        while (i < L.size() && leading_numbers(L[i].c_str(), row.data(), m->n_pw + 1) != m->n_pw + 1) ++i;
        if (i >= L.size()) break;
        int rows = 0;
        for (int k = 0; k < m->n_ang && i + k < L.size(); ++k) {
            if (leading_numbers(L[i + k].c_str(), row.data(), m->n_pw + 1) < m->n_pw + 1) break;
            if (found == 0) m->ang[k] = row[0];
            for (int l = 0; l < m->n_pw; ++l) (*blocks[found])[(size_t)k * m->n_pw + l] = row[l + 1];
            ++rows;
        }
        if (rows != m->n_ang) break;
        i += m->n_ang;
        ++found;
    }
    if (found < 3) return bad("expected three phase blocks (P11, P12, P33)");
    *out = m;
    return OCRT_OK;
}

void ocrt_gb_mie_free(ocrt_mie *m) { delete m; }

int ocrt_gb_mie_shape(const ocrt_mie *m, int *n_ang, int *n_wl, int *n_phase_wl)
{
    if (!m) return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: null model");
    if (n_ang) *n_ang = m->n_ang;
    if (n_wl) *n_wl = m->n_wl;
    if (n_phase_wl) *n_phase_wl = m->n_pw;
    return OCRT_OK;
}

int ocrt_gb_mie_prepare(const ocrt_mie *m, double wavelength_nm, double aod_ref, double aod_ref_nm,
                        const ocrt_mie_opts *opts, ocrt_mie_aerosol **out, ocrt_aerosol *aer, ocrt_mie_diag *diag)
{
    if (!m || !out || !aer) return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: null argument");
    *out = nullptr;
    ocrt_mie_opts o;
    if (opts) o = *opts; else ocrt_mie_opts_default(&o);
    const double wl = wavelength_nm / 1000.0, wref = aod_ref_nm / 1000.0;
    if (!(aod_ref > 0.0) || !(aod_ref_nm > 0.0) || o.L_max < 2)
        return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: aod_ref and aod_ref_nm must be > 0, L_max >= 2");
    if (!covers(m->wl, wl) || !covers(m->pwl, wl) || !covers(m->wl, wref))
        return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: wavelength outside the table's spectral or phase grid");
    if (!full_range(m->ang.data(), m->n_ang))
        return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: the phase table must span 0..180 degrees");
    const int na = m->n_ang, nw = m->n_wl, np = m->n_pw;
    std::vector<double> col(std::max(nw, np));
    // AOD carried from the reference wavelength by the normalised extinction
    for (int k = 0; k < nw; ++k) col[k] = m->spec[(size_t)k * 6 + 0];
    const double ext_t = lin_interp(m->wl.data(), col.data(), nw, wl);
    const double ext_r = lin_interp(m->wl.data(), col.data(), nw, wref);
    if (!(ext_t > 0.0 && ext_r > 0.0)) return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: non-positive extinction");
    const double ratio = ext_t / ext_r, aod = aod_ref * ratio;
    for (int k = 0; k < nw; ++k) col[k] = m->spec[(size_t)k * 6 + 2];
    const double ssa = lin_interp(m->wl.data(), col.data(), nw, wl);
    // phase elements at the wavelength: PCHIP over the phase grid
    std::vector<double> e[3];
    const std::vector<double> *src[3] = {&m->P11, &m->P12, &m->P33};
    for (int b = 0; b < 3; ++b) {
        e[b].resize(na);
        for (int a = 0; a < na; ++a) {
            for (int k = 0; k < np; ++k) col[k] = (*src[b])[(size_t)a * np + k];
            e[b][a] = pchip_point(m->pwl.data(), col.data(), np, wl);
        }
    }
    double A = 0.0;
    if (o.use_loglin_trunc) {
        std::vector<double> t[3] = {std::vector<double>(na), std::vector<double>(na), std::vector<double>(na)};
        loglin_truncate(e[0].data(), e[1].data(), e[2].data(), m->ang.data(), na,
                        o.loglin_mu1 > 0.0 ? o.loglin_mu1 : 0.8, o.loglin_mu2 > 0.0 ? o.loglin_mu2 : 0.94,
                        o.loglin_threshold > 0.0 ? o.loglin_threshold : 0.1, t[0].data(), t[1].data(),
                        t[2].data(), &A);
        for (int b = 0; b < 3; ++b) e[b].swap(t[b]);
    }
    double tau_eff = aod, ssa_eff = ssa;
    if (o.use_loglin_trunc && A > 0.0) {
        tau_eff = aod * (1.0 - 0.5 * ssa * A);
        ssa_eff = (1.0 - 0.5 * A) * ssa / (1.0 - 0.5 * ssa * A);
    }
    auto h = new ocrt_mie_aerosol();
    const int L = o.L_max;
    h->beta.assign(L + 1, 0.0); h->gamma.assign(L + 1, 0.0);
    h->alpha.assign(L + 1, 0.0); h->zeta.assign(L + 1, 0.0);
    std::vector<double> d33(L + 1, 0.0);
    const double *th = m->ang.data();
    bool ok = legendre_moments(e[0].data(), th, na, L + 1, 4096, h->beta.data()) &&
              spin2_moments(e[1].data(), th, na, L, 4096, h->gamma.data()) &&
              legendre_moments(e[2].data(), th, na, L + 1, 4096, d33.data());
    if (ok) {
        complete_spherical(L, h->beta.data(), h->beta.data(), d33.data(), h->alpha.data(), h->zeta.data());
        const double nb = h->beta[0];
        ok = nb != 0.0 && std::isfinite(nb);
        if (ok)
            for (int l = 0; l <= L; ++l) { h->alpha[l] /= nb; h->beta[l] /= nb; h->gamma[l] /= nb; h->zeta[l] /= nb; }
    }
    // the phase table for the value kernel, normalised by (1/2) int P11 dmu on
    // the same 4096-point densification, ascending in angle
    double chi0 = 0.0;
    if (ok && legendre_moments(e[0].data(), th, na, 1, 4096, &chi0) && chi0 != 0.0)
        for (int b = 0; b < 3; ++b) for (int a = 0; a < na; ++a) e[b][a] /= chi0;
    if (!ok) {
        delete h;
        return ocrt_internal_fail(OCRT_ERR_ARGS, "mie: moment expansion failed");
    }
    const bool desc = na >= 2 && th[0] > th[na - 1];
    h->theta.resize(na); h->p11.resize(na); h->p12.resize(na); h->p33.resize(na);
    for (int a = 0; a < na; ++a) {
        const int s = desc ? na - 1 - a : a;
        h->theta[a] = th[s]; h->p11[a] = e[0][s]; h->p12[a] = e[1][s]; h->p33[a] = e[2][s];
    }
    std::memset(aer, 0, sizeof(*aer));
    aer->tau_a = tau_eff;
    aer->ssa_a = ssa_eff;
    aer->L_max = L;
    aer->beta = h->beta.data(); aer->gamma = h->gamma.data();
    aer->alpha = h->alpha.data(); aer->zeta = h->zeta.data();
    aer->use_value_kernel = o.use_value_kernel ? 1 : 0;
    aer->n_ang_phase = na;
    aer->theta_phase = h->theta.data();
    aer->P11_phase = h->p11.data(); aer->P12_phase = h->p12.data(); aer->P33_phase = h->p33.data();
    if (diag) {
        diag->aod_ref = aod_ref; diag->aod_ref_nm = aod_ref_nm;
        diag->aod_target = aod; diag->extinction_ratio = ratio;
        diag->ssa_raw = ssa; diag->trunc_A = A;
        diag->tau_a_eff = tau_eff; diag->ssa_a_eff = ssa_eff;
    }
    *out = h;
    return OCRT_OK;
}

void ocrt_gb_mie_aerosol_free(ocrt_mie_aerosol *a) { delete a; }

} // extern "C"
