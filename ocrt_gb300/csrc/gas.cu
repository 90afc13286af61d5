// gas.cu — trace-gas absorption: table loading (host), column depths (host)
// and the per-layer absorption step of the level grid (device).
//
//   ocrt_gb_gas_create   rt_absorption_init      rt_absorption.c:486-533
//                        rt_afgl_load            rt_absorption.c:48-175
//                        rt_xsec_load            rt_absorption.c:192-333
//   ocrt_gb_gas_tau      rt_absorption_tau_*     rt_absorption.c:556-600
//   k_gas_apply          rt_atm_apply_gas_absorption  rt_atm.c:437-548
//
// k_gas_apply runs once per solve right after the level grid is built (one
// block per pixel): every thread takes solver layers, evaluates the six gas
// columns and cross sections at the layer's altitude band, then the block
// rescales the scattering fractions by dtau_old / dtau_new, and thread 0
// rebuilds the optical-depth prefix in the reference's summation order.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "gas.cuh"

int ocrt_internal_fail(int rc, const char *msg);

namespace {

const char *const kGas[OCRT_NGAS] = {"h2o", "o3", "o2", "co2", "no2", "ch4"};
const char *const kAfgl[7] = {"usstd76", "tropical", "mlsumm", "mlwint", "sasumm", "sawint", "userdef"};

bool read_lines(const std::string &path, std::vector<std::string> &lines)
{
    std::ifstream f(path);
    if (!f) return false;
    std::string l;
    while (std::getline(f, l)) lines.push_back(l);
    return true;
}

// Data lines: not a '#' comment, not empty (rt_absorption.c:68-72).
bool data_line(const std::string &l) { return !l.empty() && l[0] != '#' && l[0] != '\r'; }

struct Afgl {
    std::vector<double> z, ntot, mr[OCRT_NGAS];
};

// z P T n_total and six mixing ratios in ppmv per level.
int load_afgl(const std::string &path, Afgl &a)
{
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) return OCRT_ERR_ARGS;
    for (const std::string &l : lines) {
        if (!data_line(l)) continue;
        double v[10];
        if (std::sscanf(l.c_str(), "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &v[0], &v[1], &v[2], &v[3], &v[4],
                        &v[5], &v[6], &v[7], &v[8], &v[9]) != 10) {
            if (l.find_first_not_of(" \t\r") == std::string::npos) continue;
            return OCRT_ERR_ARGS;
        }
        a.z.push_back(v[0]);
        a.ntot.push_back(v[3]);
        for (int q = 0; q < OCRT_NGAS; ++q) a.mr[q].push_back(v[4 + q]);
    }
    return a.z.size() >= 2 ? OCRT_OK : OCRT_ERR_ARGS;
}

struct Xsec {
    bool avail = false;
    int nlay = 1;
    std::vector<double> wl, sig;
};

// Layered table ("n_layers" header tag): a wavelength row, then one sigma row
// per table level; otherwise (wavelength, sigma) rows.  An unreadable or
// malformed table, or one whose grid is not increasing or does not cover
// 330-1100 nm (rt_spectral_contract.h), leaves the gas out.
void load_xsec(const std::string &path, Xsec &x)
{
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) return;
    int nlay = 1;
    for (const std::string &l : lines) {
        if (l.empty() || l[0] != '#') continue;
        const size_t p = l.find("n_layers");
        if (p != std::string::npos) {
            std::sscanf(l.c_str() + p, "n_layers = %d", &nlay);
            if (nlay < 1) nlay = 1;
        }
    }
    x.nlay = nlay;
    if (nlay == 1) {
        for (const std::string &l : lines) {
            if (!data_line(l)) continue;
            double a, b;
            if (std::sscanf(l.c_str(), "%lf %lf", &a, &b) != 2) continue;
            x.wl.push_back(a);
            x.sig.push_back(b);
        }
    } else {
        int row = -1;
        for (const std::string &l : lines) {
            if (!data_line(l)) continue;
            const char *p = l.c_str();
            char *e = nullptr;
            if (row < 0) {
                for (;;) {
                    const double v = std::strtod(p, &e);
                    if (e == p) break;
                    x.wl.push_back(v);
                    p = e;
                }
                if (x.wl.size() < 2) return;
                x.sig.assign((size_t)nlay * x.wl.size(), 0.0);
                row = 0;
            } else if (row < nlay) {
                for (size_t i = 0; i < x.wl.size(); ++i) {
                    const double v = std::strtod(p, &e);
                    if (e == p) break;
                    x.sig[(size_t)row * x.wl.size() + i] = v;
                    p = e;
                }
                ++row;
            }
        }
        if (row < 0) { x.wl.clear(); x.sig.clear(); return; }
    }
    const size_t n = x.wl.size();
    if (n < 2) return;
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(x.wl[i]) || (i > 0 && !(x.wl[i] > x.wl[i - 1]))) return;
    if (!(x.wl[0] <= 330.0 + 1e-9 && x.wl[n - 1] >= 1100.0 - 1e-9)) return;
    x.avail = true;
}

}  // namespace

__global__ void k_gas_apply(PixDev *px, int P, double *h, double *ch, double *xd, double *yd, const double *z,
                            double *tabs)
{
    const int p = blockIdx.x;
    if (p >= P) return;
    PixDev &d = px[p];
    if (!d.gas) return;
    const GasDev &G = *d.gas;
    const int nt = d.nt;
    const long long lo = d.lev_off;
    for (int k = threadIdx.x; k < nt; k += blockDim.x)
        tabs[lo + k] = gas_layer_depth(G, z[lo + k], z[lo + k + 1], d.wavelength_nm);
    __syncthreads();
    // scattering fractions of the layer below level k, against the old depths
    for (int k = 1 + threadIdx.x; k <= nt; k += blockDim.x) {
        const double dold = h[lo + k] - h[lo + k - 1], dnew = dold + tabs[lo + k - 1];
        if (dnew > 0.0 && dold > 0.0) {
            xd[lo + k] = xd[lo + k] * dold / dnew;
            yd[lo + k] = yd[lo + k] * dold / dnew;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double cum = 0.0;
        for (int k = 0; k <= nt; ++k) {
            h[lo + k] = h[lo + k] + cum;
            if (k < nt) cum += tabs[lo + k];
        }
        d.tau_total = h[lo + nt];
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= nt; k += blockDim.x) ch[lo + k] = 0.5 * exp(-h[lo + k] / d.mu0);
}

extern "C" {

int ocrt_gb_gas_create(const char *afgl_dir, const char *xsec_dir, int profile, const double *column_override,
                       ocrt_gas **out)
{
    if (!out) return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: null output handle");
    *out = nullptr;
    if (!afgl_dir || !xsec_dir) return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: null data directory");
    if (profile < OCRT_AFGL_USSTD76 || profile > OCRT_AFGL_USERDEF)
        return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: AFGL profile outside 0..6");
    Afgl a;
    const std::string ap = std::string(afgl_dir) + "/afgl_" + kAfgl[profile] + ".dat";
    if (load_afgl(ap, a)) return ocrt_internal_fail(OCRT_ERR_ARGS, ("gas: cannot read AFGL profile " + ap).c_str());
    Xsec xs[OCRT_NGAS];
    const int nlev = (int)a.z.size();
    for (int q = 0; q < OCRT_NGAS; ++q) {
        load_xsec(std::string(xsec_dir) + "/xsec_" + kGas[q] + ".dat", xs[q]);
        // table level i is placed at AFGL level i
        if (xs[q].avail && xs[q].nlay > nlev)
            return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: cross-section table has more levels than the AFGL profile");
    }
    // one host buffer and one device buffer: z | nd[6] | per gas (wl | sig)
    size_t tot = (size_t)nlev * (1 + OCRT_NGAS);
    for (int q = 0; q < OCRT_NGAS; ++q) tot += xs[q].wl.size() + xs[q].sig.size();
    ocrt_gas *g = new ocrt_gas();
    g->hbuf = (double *)std::malloc(sizeof(double) * tot);
    if (!g->hbuf) { delete g; return ocrt_internal_fail(OCRT_ERR_ALLOC, "gas: host allocation"); }
    GasDev &H = g->host;
    std::memset(&H, 0, sizeof(H));
    double *w = g->hbuf;
    H.nlev = nlev;
    std::memcpy(w, a.z.data(), sizeof(double) * nlev);
    H.z = w; w += nlev;
    H.nd = w;
    for (int q = 0; q < OCRT_NGAS; ++q)
        for (int i = 0; i < nlev; ++i) *w++ = a.mr[q][i] * 1e-6 * a.ntot[i];
    for (int q = 0; q < OCRT_NGAS; ++q) {
        const double *n = H.nd + (size_t)q * nlev;
        double col = 0.0;                  // trapezoids on the AFGL grid (rt_absorption.c:160-172)
        for (int i = 0; i + 1 < nlev; ++i) col += 0.5 * (n[i] + n[i + 1]) * ((a.z[i + 1] - a.z[i]) * 1.0e5);
        H.col_default[q] = col;
        if (column_override && column_override[q] >= 0.0) {
            H.col_eff[q] = column_override[q];
            H.overridden[q] = 1;
        } else {
            H.col_eff[q] = col;
        }
        H.avail[q] = xs[q].avail;
        H.nwl[q] = (int)xs[q].wl.size();
        H.nlay[q] = xs[q].nlay;
        std::memcpy(w, xs[q].wl.data(), sizeof(double) * xs[q].wl.size());
        H.wl[q] = w; w += xs[q].wl.size();
        std::memcpy(w, xs[q].sig.data(), sizeof(double) * xs[q].sig.size());
        H.sig[q] = w; w += xs[q].sig.size();
    }
    // device mirror: same offsets, pointers rebased
    if (cudaMalloc(&g->dbuf, sizeof(double) * tot + sizeof(GasDev) + 256) != cudaSuccess) {
        std::free(g->hbuf);
        delete g;
        return ocrt_internal_fail(OCRT_ERR_ALLOC, "gas: device allocation");
    }
    double *db = (double *)g->dbuf;
    auto rebase = [&](const double *hp) { return hp ? db + (hp - g->hbuf) : nullptr; };
    GasDev D = H;
    D.z = rebase(H.z);
    D.nd = rebase(H.nd);
    for (int q = 0; q < OCRT_NGAS; ++q) { D.wl[q] = rebase(H.wl[q]); D.sig[q] = rebase(H.sig[q]); }
    g->dev = (GasDev *)((char *)g->dbuf + ((sizeof(double) * tot + 255) & ~(size_t)255));
    if (cudaMemcpy(db, g->hbuf, sizeof(double) * tot, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->dev, &D, sizeof(GasDev), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(g->dbuf);
        std::free(g->hbuf);
        delete g;
        return ocrt_internal_fail(OCRT_ERR_DEVICE, "gas: upload failed");
    }
    *out = g;
    return OCRT_OK;
}

void ocrt_gb_gas_destroy(ocrt_gas *g)
{
    if (!g) return;
    cudaFree(g->dbuf);
    std::free(g->hbuf);
    delete g;
}

int ocrt_gb_gas_tau(const ocrt_gas *g, double wavelength_nm, double *tau_per_gas, double *tau_total)
{
    if (!g) return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: null handle");
    const GasDev &G = g->host;
    double tot = 0.0;
    for (int q = 0; q < OCRT_NGAS; ++q) {
        double tau = 0.0;
        if (G.avail[q] && G.nlev >= 2) {
            const double nd = G.col_default[q];
            const bool ov = G.overridden[q] && nd > 0.0;
            const double scale = ov ? G.col_eff[q] / nd : 1.0;
            for (int i = 0; i + 1 < G.nlev; ++i) {
                const double z_lo = G.z[i], z_hi = G.z[i + 1];
                double N = gas_column(G, q, z_lo, z_hi);
                if (ov) N *= scale;
                tau += gas_sigma(G, q, 0.5 * (z_lo + z_hi), wavelength_nm) * N;
            }
        }
        if (tau_per_gas) tau_per_gas[q] = tau;
        tot += tau;
    }
    if (tau_total) *tau_total = tot;
    return OCRT_OK;
}

int ocrt_gb_gas_columns(const ocrt_gas *g, double *column_eff, double *column_default, int *overridden)
{
    if (!g) return ocrt_internal_fail(OCRT_ERR_ARGS, "gas: null handle");
    for (int q = 0; q < OCRT_NGAS; ++q) {
        if (column_eff) column_eff[q] = g->host.col_eff[q];
        if (column_default) column_default[q] = g->host.col_default[q];
        if (overridden) overridden[q] = g->host.overridden[q];
    }
    return OCRT_OK;
}

}  // extern "C"
