/*
 * ref_driver.c — thin adapter from this repository's C-ABI structs
 * (include/ocrt_gb300.h) to the reference solver's public API
 * (code/OCRT_C/src/rt_solver.h:84-121), linked against the reference sources
 * compiled by oracle/Makefile into oracle/_ref/libocrt_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY: used here to pin the oracle and to generate the
 * golden fixtures under tests/golden/.  Nothing in the product links it.
 *
 * For OCRT_PROFILE_EXPONENTIAL the reference has no option; this driver
 * composes the reference's own pieces the way its IPSS gate does
 * (tests/test_ipss_gates.c:44-57): the plane-parallel solve with pssa off,
 * then rt_ipss_kappa / rt_ipss_tau_dir_dn_boa on an atmosphere whose level
 * altitudes follow the exponential profile.
 */
#include <math.h>
#include <string.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rt_solver.h"
#include "rt_atm.h"
#include "rt_ipss.h"
#include "rt_raa_convention.h"
#include "shared/surface.h"
#include "rt_absorption.h"
#include "rt_aerosol_runtime.h"
#include "shared/mie_io.h"
#include "../include/ocrt_gb300.h"

#define OCRT_PI_ 3.14159265358979323846

static double exp_frac(double z, double h)
{
    if (z <= 0.0) return 1.0;
    if (z >= 100.0) return 0.0;
    const double et = exp(-100.0 / h);
    return (exp(-z / h) - et) / (1.0 - et);
}

static void fill(const ocrt_case *c, const ocrt_opts *o, rt_case_t *cs, rt_options_t *op)
{
    memset(cs, 0, sizeof(*cs));
    cs->sza_deg = c->sza_deg; cs->vza_deg = c->vza_deg; cs->raa_deg = c->raa_deg;
    cs->wavelength_nm = c->wavelength_nm;
    cs->surface = (rt_surface_kind_t)c->surface;
    cs->pressure_hpa = c->pressure_hpa;
    cs->rayleigh_on = c->pressure_hpa > 0.0;
    cs->tau_R_input = c->tau_r_input;
    cs->n_water = c->n_water; cs->wind_speed = c->wind_speed;
    cs->sigma_type = c->sigma_type; cs->q_convention = c->q_convention;
    cs->decouple_sunglint = c->decouple_sunglint;
    cs->F_sun = OCRT_PI_;
    *op = rt_options_default();
    op->n_mu = o->n_mu; op->n_layers = o->n_layers; op->fourier_m_max = o->fourier_m_max;
    op->sos.max_iterations = o->max_orders; op->sos.tolerance = o->tolerance;
    op->tau_r_source = (rt_tau_r_source_t)o->tau_r_source;
    op->pssa = o->pssa; op->view_as_node = o->view_as_node; op->aer_h_km = o->aer_h_km;
    /* for this driver ocrt_opts.gas holds the reference's own rt_absorption_t */
    op->abs_state = (const void *)o->gas;
}

/* Gas absorption state made by the reference's rt_absorption_init
 * (rt_absorption.c:486); the handle is an rt_absorption_t. */
int ocrt_ref_gas_create(const char *afgl_dir, const char *xsec_dir, int profile,
                        const double *override, ocrt_gas **out)
{
    if (!out) return -1;
    *out = NULL;
    rt_absorption_t *st = calloc(1, sizeof(*st));
    if (!st) return -3;
    double ov[RT_N_GAS];
    for (int g = 0; g < RT_N_GAS; ++g) ov[g] = override ? override[g] : -1.0;
    const int rc = rt_absorption_init(afgl_dir, xsec_dir, (rt_afgl_profile_t)profile, ov, st);
    if (rc < 0 || rc > 0) { rt_absorption_free(st); free(st); return rc ? rc : -1; }
    *out = (ocrt_gas *)st;
    return 0;
}

void ocrt_ref_gas_destroy(ocrt_gas *g)
{
    if (!g) return;
    rt_absorption_free((rt_absorption_t *)g);
    free(g);
}

int ocrt_ref_gas_tau(const ocrt_gas *g, double wl, double *per_gas, double *total)
{
    if (!g) return -1;
    const rt_absorption_t *st = (const rt_absorption_t *)g;
    for (int k = 0; k < RT_N_GAS; ++k)
        if (per_gas) per_gas[k] = rt_absorption_tau_per_gas(st, k, wl);
    if (total) *total = rt_absorption_tau_total(st, wl);
    return 0;
}

int ocrt_ref_gas_columns(const ocrt_gas *g, double *eff, double *def, int *ov)
{
    if (!g) return -1;
    const rt_absorption_t *st = (const rt_absorption_t *)g;
    for (int k = 0; k < RT_N_GAS; ++k) {
        if (eff) eff[k] = st->column_eff[k];
        if (def) def[k] = st->atm.column_default[k];
        if (ov) ov[k] = st->column_overridden[k];
    }
    return 0;
}

int ocrt_ref_solve_case(const ocrt_case *c, const ocrt_opts *o, const ocrt_aerosol *a,
                        ocrt_result *out, ocrt_diag *diag)
{
    rt_case_t cs; rt_options_t op;
    fill(c, o, &cs, &op);
    const int exp_profile = o->rayleigh_profile == OCRT_PROFILE_EXPONENTIAL;
    if (exp_profile) op.pssa = 0;
    double vI[33], vQ[33], vU[33];
    op.toa_view_per_m_I = vI; op.toa_view_per_m_Q = vQ; op.toa_view_per_m_U = vU;
    rt_aerosol_input_t ai;
    memset(&ai, 0, sizeof(ai));
    rt_result_t r;
    int rc;
    if (a && a->tau_a > 0.0) {
        ai.tau_a = a->tau_a; ai.ssa_a = a->ssa_a; ai.L_max = a->L_max;
        ai.betal_aer = a->beta; ai.gammal_aer = a->gamma;
        ai.alphal_aer = a->alpha; ai.zetal_aer = a->zeta;
        ai.use_value_kernel = a->use_value_kernel;
        ai.n_ang_phase = a->n_ang_phase;
        ai.theta_phase = a->theta_phase;
        ai.P11_phase = a->P11_phase; ai.P12_phase = a->P12_phase; ai.P33_phase = a->P33_phase;
        rc = rt_solve_case_pol_aerosol(&cs, &op, &ai, &r);
    } else {
        rc = rt_solve_case_pol(&cs, &op, &r);
    }
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->rho_I = r.rho_I; out->rho_Q = r.rho_Q; out->rho_U = r.rho_U;
    out->I_TOA = r.I_TOA; out->Q_TOA = r.Q_TOA; out->U_TOA = r.U_TOA;
    out->tau_R_total = r.tau_R_total;
    out->n_orders_used = r.n_orders_used; out->converged = r.converged;
    out->kappa_ipss = 1.0;
    for (int m = 0; m <= o->fourier_m_max; ++m) out->order_modes += r.sos_orders_per_m[m];
    out->T_dir_dn = r.T_dir_dn; out->T_diff_dn_hemi = r.T_diff_dn_hemi;
    out->T_total_dn_hemi = r.T_total_dn_hemi; out->T_diff_dn_dir = r.T_diff_dn_dir;
    out->T_total_up_dir = r.T_total_up_dir; out->T_sg_up_dir = r.T_sg_up_dir;
    out->T_dir_up_view = r.T_dir_up_view;
    out->rho_glint_direct_I = r.rho_glint_direct_I;
    out->rho_glint_direct_Q = r.rho_glint_direct_Q;
    out->rho_glint_direct_U = r.rho_glint_direct_U;
    if (diag) {
        for (int m = 0; m <= o->fourier_m_max; ++m) {
            if (diag->orders_per_m) diag->orders_per_m[m] = r.sos_orders_per_m[m];
            if (diag->residual_per_m) diag->residual_per_m[m] = r.sos_residual_per_m[m];
            if (diag->view_I_m) diag->view_I_m[m] = vI[m];
            if (diag->view_Q_m) diag->view_Q_m[m] = vQ[m];
            if (diag->view_U_m) diag->view_U_m[m] = vU[m];
        }
    }
    if (!(exp_profile && o->pssa)) return 0;

    /* IPSS on an exponential altitude profile (Rayleigh only). */
    if (a && a->tau_a > 0.0) return -5;
    const int nt = o->n_layers;
    rt_atm_t atm;
    memset(&atm, 0, sizeof(atm));
    if (rt_atm_alloc(&atm, nt, o->n_mu) != 0) return -3;
    const double mu0 = cos(c->sza_deg * OCRT_PI_ / 180.0);
    if (rt_atm_build_rayleigh(&atm, r.tau_R_total, 0.0279, mu0, RT_RAYLEIGH_MODEL_BODHAINE_1999)) {
        rt_atm_free(&atm); return -1;
    }
    for (int k = 1; k <= nt; ++k) {
        const double f = atm.h[k] / atm.tau_total;
        double zk;
        if (f >= 1.0) zk = 0.0;
        else {
            double lo = 0.0, hi = 100.0;
            for (int it = 0; it < 64; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (exp_frac(mid, o->rayleigh_h_km) > f) lo = mid; else hi = mid;
            }
            zk = 0.5 * (lo + hi);
        }
        atm.z_km_level[k] = zk;
    }
    atm.z_km_level[0] = 100.0;
    rt_ipss_t G;
    memset(&G, 0, sizeof(G));
    if (rt_ipss_init_from_atm(&G, &atm, RT_IPSS_EARTH_RADIUS_KM) != 0) { rt_atm_free(&atm); return -1; }
    const double tau_dir = rt_ipss_tau_dir_dn_boa(&G);
    double kappa = 1.0; int guard = 0;
    rt_ipss_kappa(&G, c->vza_deg, c->raa_deg, &kappa, NULL, NULL, &guard);
    const double tau_t = atm.h[nt];
    rt_ipss_free(&G);
    rt_atm_free(&atm);
    /* undo the plane-parallel glint, scale the diffuse path, redo the glint
     * with the ray-traced slant factor (rt_solver.c:1117-1181) */
    double gI = 0, gQ = 0, gU = 0;
    if (c->surface == OCRT_SURFACE_BLACK_FRESNEL_OCEAN && !c->decouple_sunglint) {
        const double phi_v = rt_raa_to_surface_view_phi(c->raa_deg);
        const double mu_v = c->vza_deg > 0 ? cos(c->vza_deg * OCRT_PI_ / 180.0) : 1.0;
        double g[3];
        surface_direct_sunglint_rho(mu_v, phi_v, mu0, 0.0, c->wind_speed, c->sigma_type,
                                    c->n_water, tau_t, c->q_convention, g);
        gI = g[0]; gQ = g[1]; gU = -g[2];
    }
    const double base_I = out->rho_I - gI, base_Q = out->rho_Q - gQ, base_U = out->rho_U - gU;
    const double cg = tau_dir >= 0.0 ? exp(-(tau_dir - tau_t / mu0)) : 1.0;
    out->kappa_ipss = kappa;
    out->rho_I = base_I * kappa + gI * cg;
    out->rho_Q = base_Q * kappa + gQ * cg;
    out->rho_U = base_U * kappa + gU * cg;
    out->I_TOA *= kappa; out->Q_TOA *= kappa; out->U_TOA *= kappa;
    out->rho_glint_direct_I *= cg; out->rho_glint_direct_Q *= cg; out->rho_glint_direct_U *= cg;
    out->T_sg_up_dir *= cg;
    if (tau_dir >= 0.0) {
        out->T_dir_dn = exp(-tau_dir);
        out->T_total_dn_hemi = out->T_dir_dn + out->T_diff_dn_hemi;
    }
    out->T_total_up_dir = out->rho_I * mu0;
    return 0;
}

/* OpenMP pixel loop over the reference solve, for the CPU baseline. */
int ocrt_ref_solve_batch(int n, const ocrt_case *cases, const ocrt_opts *opts, int opts_per_case,
                         const ocrt_aerosol *aer, int aer_per_case, ocrt_result *out, int n_threads)
{
    int rc_all = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; ++i) {
        const ocrt_opts *o = opts_per_case ? opts + i : opts;
        const ocrt_aerosol *a = aer ? (aer_per_case ? aer + i : aer) : NULL;
        const int rc = ocrt_ref_solve_case(cases + i, o, a, out + i, NULL);
        if (rc) {
#pragma omp critical
            rc_all = rc;
        }
    }
    return rc_all;
}

/* Angle-grid LUT through the reference's own rt_solve_case_pol_lut
 * (rt_solver.h:207-210); US62 profile only. */
int ocrt_ref_solve_case_lut(const ocrt_case *c, const ocrt_opts *o, const ocrt_aerosol *a,
                            ocrt_result *out, ocrt_lut *lut)
{
    if (o->rayleigh_profile == OCRT_PROFILE_EXPONENTIAL) return -5;
    rt_case_t cs; rt_options_t op;
    fill(c, o, &cs, &op);
    rt_lut_grid_out_t L;
    memset(&L, 0, sizeof(L));
    L.n_vza = lut->n_vza; L.vza_deg = lut->vza_deg;
    L.n_raa = lut->n_raa; L.raa_deg = lut->raa_deg;
    L.rho_I = lut->rho_I; L.rho_Q = lut->rho_Q; L.rho_U = lut->rho_U;
    L.T_diff_dn_dir = lut->T_diff_dn_dir; L.T_sg_up_dir = lut->T_sg_up_dir; L.T_total_up_dir = lut->T_total_up_dir;
    L.view_m_max = -1;
    rt_aerosol_input_t ai;
    memset(&ai, 0, sizeof(ai));
    rt_result_t r;
    int rc;
    if (a && a->tau_a > 0.0) {
        ai.tau_a = a->tau_a; ai.ssa_a = a->ssa_a; ai.L_max = a->L_max;
        ai.betal_aer = a->beta; ai.gammal_aer = a->gamma;
        ai.alphal_aer = a->alpha; ai.zetal_aer = a->zeta;
        ai.use_value_kernel = 0;
        rc = rt_solve_case_pol_lut(&cs, &op, &ai, &r, &L);
    } else {
        rc = rt_solve_case_pol_lut(&cs, &op, NULL, &r, &L);
    }
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->rho_I = r.rho_I; out->rho_Q = r.rho_Q; out->rho_U = r.rho_U;
    out->n_orders_used = r.n_orders_used; out->converged = r.converged;
    lut->T_dir_dn = L.T_dir_dn; lut->T_diff_dn_hemi = L.T_diff_dn_hemi;
    return 0;
}

/* The reference's .mie pipeline (read_mie_file + rt_aerosol_runtime_prepare
 * with the CLI's log-linear truncation options, main.c:3646-3670); outputs
 * copied into the caller's arrays: scal = {tau_a, ssa_a, A, ssa_raw,
 * aod_target, extinction_ratio, n_ang}, moments [L_max + 1], phase table
 * [n_ang] (cap entries at most). */
int ocrt_ref_mie_prepare(const char *path, double wl_nm, double aod_ref, double aod_ref_nm, int L_max,
                         int use_loglin, int use_value_kernel, double *scal, double *beta, double *gamma,
                         double *alpha, double *zeta, double *theta, double *p11, double *p12, double *p33,
                         int cap)
{
    mie_data_t mie;
    memset(&mie, 0, sizeof(mie));
    if (read_mie_file(path, &mie) != 0) return -1;
    rt_aerosol_runtime_options_t ro;
    memset(&ro, 0, sizeof(ro));
    ro.aer_L_max = L_max;
    ro.use_loglin_trunc = use_loglin;
    ro.loglin_mu1 = 0.8; ro.loglin_mu2 = 0.94; ro.loglin_threshold = 0.1;
    ro.use_value_kernel = use_value_kernel;
    rt_aerosol_input_t aer;
    rt_aerosol_runtime_diag_t dg;
    memset(&dg, 0, sizeof(dg));
    const int rc = rt_aerosol_runtime_prepare(&mie, wl_nm, aod_ref, aod_ref_nm, &ro, &aer, &dg);
    mie_data_free(&mie);
    if (rc) return -2;
    scal[0] = aer.tau_a; scal[1] = aer.ssa_a; scal[2] = dg.f_fwd; scal[3] = dg.ssa_raw;
    scal[4] = dg.aod_target; scal[5] = dg.extinction_ratio; scal[6] = aer.n_ang_phase;
    for (int l = 0; l <= L_max; ++l) {
        beta[l] = aer.betal_aer[l]; gamma[l] = aer.gammal_aer[l];
        alpha[l] = aer.alphal_aer[l]; zeta[l] = aer.zetal_aer[l];
    }
    const int n = aer.n_ang_phase < cap ? aer.n_ang_phase : cap;
    for (int i = 0; i < n; ++i) {
        theta[i] = aer.theta_phase[i]; p11[i] = aer.P11_phase[i];
        p12[i] = aer.P12_phase[i]; p33[i] = aer.P33_phase[i];
    }
    rt_aerosol_runtime_free(&aer);
    return 0;
}
