/*
 * ocrt — command-line front end of the GB300 SOS solve path.
 *
 * Mirrors the solve-path options of the reference CLI (code/OCRT_C/src/main.c:
 * --sza/--vza/--raa/--wavelength/--surface/--wind-speed/--n-water main.c:1994-2040,
 * --pssa/--decouple-sunglint/--sigma-type/--q-convention main.c:2548-2610,
 * --pressure/--rayleigh/--n-mu/--n-layers/--sos-max-orders/--sos-tolerance/--m-max
 * main.c:2759-2850, --lut-vza-step/--lut-raa-step/--lut-vza-max main.c:2697-2710)
 * with the same gates: the convergence knobs (--n-mu, --sos-max-orders,
 * --sos-tolerance, --sigma-type, --q-convention, and --n-layers without
 * aerosol) keep their validated defaults unless OCRT_ADVANCED=1.
 *
 * Modes (main.c:3486-3530): --vza and --raa together select the single
 * geometry mode, which prints one line in the format of rt_io_print_single
 * (rt_io.c:450-531, non-ocean branch); otherwise the angle-grid LUT mode runs
 * one SOS and writes the CSV of main.c:3857-3884 (stdout or --lut-output).
 * --batch FILE solves every row of a CSV (header sza,vza,raa,wavelength and
 * optional wind,aod) in one device pass and prints one line per row.
 *
 * Aerosol from a .mie model (main.c:2603-2640, 3279-3345, 3646-3686):
 * --mie PATH with --aod-555 TAU or --aod-865 TAU (or --aod TAU at
 * --aod-ref-wavelength NM, default 555) gives the reference's protocol: the
 * AOD carried to the case wavelength by the model's extinction ratio, the
 * log10-linear forward-peak truncation, moments to --aer-l-max (default 80),
 * the value kernel for the intensity phase table, Fourier modes 0..16 when
 * --m-max is not given.  Without --mie an aerosol enters as the synthetic
 * expansion of the moment API (rt_solver.h:94-114): --aod TAU (at the case
 * wavelength), --aer-hg-g G (Henyey-Greenstein beta_l = (2l+1) g^l),
 * --aer-ssa W, --aer-l-max L, with gamma_2 and alpha_2 at 0.3 x the
 * Rayleigh-form values.  When an aerosol is on and --n-layers is not given,
 * 400 layers are used (main.c:3342-3345).
 *
 * Gas absorption is on by default, as in the reference (main.c:1950-1960):
 * the AFGL atmosphere (--atm-profile, default usstd76) and the six
 * cross-section tables are read from inputs/afgl_atm and inputs/xsec under
 * the working directory (the reference's fixed paths), or under
 * $OCRT_GB_INPUTS when that is set.  --gas-column-h2o G (g/cm^2, alias
 * --pwv-g-cm), --gas-column-o3 DU, --gas-column-no2 DU, --gas-column-o2 N,
 * --gas-column-co2 N, --gas-column-ch4 N (molecules/cm^2) rescale a gas's
 * column (main.c:2720-2745); all six at 0 give the gas-free result.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ocrt_gb300.h"

#define DEPOL 0.0279

static int advanced_on(void)
{
    const char *e = getenv("OCRT_ADVANCED");
    return e && *e && strcmp(e, "0") != 0;
}

static int usage(void)
{
    fprintf(stderr,
            "usage: ocrt --surface black|flat|black_fresnel_ocean [--sza D] [--vza D --raa D] [--wavelength NM]\n"
            "            [--wind-speed MS] [--n-water N] [--pressure HPA | --rayleigh on|off | --tau-r TAU]\n"
            "            [--mie PATH --aod-555 TAU|--aod-865 TAU|--aod TAU [--aod-ref-wavelength NM]]\n"
            "            [--aod TAU --aer-hg-g G --aer-ssa W --aer-l-max L --aer-h-km H] [--pssa]\n"
            "            [--decouple-sunglint] [--n-layers K] [--m-max M] [--n-mu N] [--sos-max-orders K]\n"
            "            [--sos-tolerance T] [--lut-vza-step D --lut-raa-step D --lut-vza-max D --lut-output F]\n"
            "            [--batch FILE.csv] [--atm-profile usstd76|tropical|mlsumm|mlwint|sasumm|sawint|userdef]\n"
            "            [--gas-column-h2o G | --pwv-g-cm G] [--gas-column-o3 DU] [--gas-column-no2 DU]\n"
            "            [--gas-column-o2 N] [--gas-column-co2 N] [--gas-column-ch4 N]\n");
    return 2;
}

static double need_d(int argc, char **argv, int *i)
{
    if (*i + 1 >= argc) { fprintf(stderr, "error: %s needs a value\n", argv[*i]); exit(2); }
    char *end = NULL;
    const double v = strtod(argv[++*i], &end);
    if (!end || *end) { fprintf(stderr, "error: bad number '%s' for %s\n", argv[*i], argv[*i - 1]); exit(2); }
    return v;
}

static const char *need_s(int argc, char **argv, int *i)
{
    if (*i + 1 >= argc) { fprintf(stderr, "error: %s needs a value\n", argv[*i]); exit(2); }
    return argv[++*i];
}

/* synthetic aerosol expansion (HG beta, Rayleigh-form gamma_2/alpha_2 x 0.3) */
typedef struct { double *b, *g, *a, *z; } moments_t;

static void hg_moments(double g, int L, moments_t *m)
{
    m->b = calloc(L + 1, sizeof(double)); m->g = calloc(L + 1, sizeof(double));
    m->a = calloc(L + 1, sizeof(double)); m->z = calloc(L + 1, sizeof(double));
    for (int l = 0; l <= L; ++l) m->b[l] = (2.0 * l + 1.0) * pow(g, l);
    const double A = 2.0 * (1.0 - DEPOL) / (2.0 + DEPOL);
    if (L >= 2) { m->g[2] = 0.3 * (-A * sqrt(1.5)); m->a[2] = 0.3 * 3.0 * A; }
}

/* the aerosol's AOD as the output line reports it: at the reference
 * wavelength, that wavelength, at the band, and their ratio */
typedef struct { double ref, ref_nm, band, ratio; } aod_line_t;

static void print_single(const ocrt_case *c, const ocrt_result *r, aod_line_t a)
{
    /* rt_io_print_single, non-ocean branch: quantities this path does not
     * produce (the water signal and the upward diffuse view transmittance)
     * are printed as 0 with T_up_rt_valid = 0. */
    printf("%.10e %.10e %.10e  "
           "TOA_rho_I=%.10e TOA_rho_Q=%.10e TOA_rho_U=%.10e "
           "TOA_rho_glint_direct_I=%.10e TOA_rho_glint_direct_Q=%.10e TOA_rho_glint_direct_U=%.10e "
           "T_dir_dn=%.10e T_diff_dn_hemi=%.10e T_total_dn_hemi=%.10e T_diff_dn_dir=%.10e "
           "T_dir_up_view=%.10e T_diff_up_view=%.10e T_total_up_view=%.10e TOA_water_signal_I=%.10e T_up_rt_valid=%d "
           "diag_sunglint_up_flux_ratio=%.10e diag_TOA_up_flux_ratio=%.10e "
           "AOD_ref=%.10e AOD_ref_nm=%.3f AOD_band=%.10e AOD_ext_ratio=%.10e "
           "tau_R=%.10e sza=%.3f vza=%.3f raa=%.3f wl=%.3f orders=%d conv=%d\n",
           r->rho_I, r->rho_Q, r->rho_U, r->rho_I, r->rho_Q, r->rho_U,
           r->rho_glint_direct_I, r->rho_glint_direct_Q, r->rho_glint_direct_U,
           r->T_dir_dn, r->T_diff_dn_hemi, r->T_total_dn_hemi, r->T_diff_dn_dir,
           r->T_dir_up_view, 0.0, 0.0, 0.0, 0,
           r->T_sg_up_dir, r->T_total_up_dir,
           a.ref, a.ref_nm, a.band, a.ratio,
           r->tau_R_total, c->sza_deg, c->vza_deg, c->raa_deg, c->wavelength_nm, r->n_orders_used, r->converged);
}

static int col_of(char **names, int n, const char *key)
{
    for (int i = 0; i < n; ++i) if (!strcmp(names[i], key)) return i;
    return -1;
}

static int run_batch(const char *path, const ocrt_case *base, const ocrt_opts *o, const ocrt_aerosol *aer_base,
                     double hg_g, double ssa, int L)
{
    FILE *fp = fopen(path, "r");
    if (!fp) { fprintf(stderr, "error: cannot open %s\n", path); return 1; }
    char line[4096];
    if (!fgets(line, sizeof line, fp)) { fclose(fp); fprintf(stderr, "error: empty batch file\n"); return 1; }
    char namebuf[64][32];
    char *names[64]; int nn = 0;
    for (char *t = strtok(line, ",\r\n"); t && nn < 64; t = strtok(NULL, ",\r\n")) {
        snprintf(namebuf[nn], sizeof namebuf[nn], "%s", t);
        names[nn] = namebuf[nn];
        ++nn;
    }
    const int isza = col_of(names, nn, "sza"), ivza = col_of(names, nn, "vza"), iraa = col_of(names, nn, "raa");
    const int iwl = col_of(names, nn, "wavelength"), iwind = col_of(names, nn, "wind"), iaod = col_of(names, nn, "aod");
    if (isza < 0 || ivza < 0 || iraa < 0 || iwl < 0) {
        fclose(fp); fprintf(stderr, "error: batch header needs sza,vza,raa,wavelength\n"); return 1;
    }
    int cap = 1024, n = 0;
    ocrt_case *cs = malloc(sizeof(ocrt_case) * cap);
    ocrt_aerosol *as = malloc(sizeof(ocrt_aerosol) * cap);
    moments_t mom = {0};
    if (L >= 2) hg_moments(hg_g, L, &mom);
    while (fgets(line, sizeof line, fp)) {
        double v[64]; int nv = 0;
        for (char *t = strtok(line, ",\r\n"); t && nv < 64; t = strtok(NULL, ",\r\n")) v[nv++] = atof(t);
        if (nv < nn) continue;
        if (n == cap) { cap *= 2; cs = realloc(cs, sizeof(ocrt_case) * cap); as = realloc(as, sizeof(ocrt_aerosol) * cap); }
        cs[n] = *base;
        cs[n].sza_deg = v[isza]; cs[n].vza_deg = v[ivza]; cs[n].raa_deg = v[iraa]; cs[n].wavelength_nm = v[iwl];
        if (iwind >= 0) cs[n].wind_speed = v[iwind];
        const double aod = iaod >= 0 ? v[iaod] : (aer_base ? aer_base->tau_a : 0.0);
        ocrt_aerosol a = {aod, ssa, L, mom.b, mom.g, mom.a, mom.z};
        as[n] = a;
        ++n;
    }
    fclose(fp);
    ocrt_result *res = calloc(n > 0 ? n : 1, sizeof(ocrt_result));
    const int any_aer = L >= 2;
    const int rc = ocrt_gb_solve_batch(n, cs, o, 0, any_aer ? as : NULL, any_aer ? 1 : 0, res, NULL);
    if (rc) { fprintf(stderr, "error: ocrt_gb_solve_batch rc=%d: %s\n", rc, ocrt_gb_last_error()); return 1; }
    for (int i = 0; i < n; ++i) {
        const double ta = any_aer ? as[i].tau_a : 0.0;
        const aod_line_t al = {ta, cs[i].wavelength_nm, ta, ta > 0.0 ? 1.0 : 0.0};
        print_single(&cs[i], &res[i], al);
    }
    free(cs); free(as); free(res);
    return 0;
}

int main(int argc, char **argv)
{
    ocrt_case c; ocrt_case_default(&c);
    ocrt_opts o; ocrt_opts_default(&o);
    int have_surface = 0, have_vza = 0, have_raa = 0, have_nl = 0, have_lut = 0;
    double aod = 0.0, hg_g = 0.7, ssa = 0.95, aod_ref_nm = 555.0;
    int L = 120, have_L = 0, have_m = 0;
    const char *mie_path = NULL;
    double vstep = 2.5, rstep = 2.5, vmax = 85.0;
    const char *lut_out = NULL, *batch = NULL;
    static const char *const profiles[7] = {"usstd76", "tropical", "mlsumm", "mlwint", "sasumm", "sawint", "userdef"};
    static const char *const gas_names[OCRT_N_GAS] = {"h2o", "o3", "o2", "co2", "no2", "ch4"};
    int atm_profile = OCRT_AFGL_USSTD76;
    double gas_col[OCRT_N_GAS] = {-1.0, -1.0, -1.0, -1.0, -1.0, -1.0};
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (!strcmp(a, "--help") || !strcmp(a, "-h")) return usage();
        else if (!strcmp(a, "--sza")) c.sza_deg = need_d(argc, argv, &i);
        else if (!strcmp(a, "--vza")) { c.vza_deg = need_d(argc, argv, &i); have_vza = 1; }
        else if (!strcmp(a, "--raa")) { c.raa_deg = need_d(argc, argv, &i); have_raa = 1; }
        else if (!strcmp(a, "--wavelength")) c.wavelength_nm = need_d(argc, argv, &i);
        else if (!strcmp(a, "--surface")) {
            const char *s = need_s(argc, argv, &i);
            if (!strcmp(s, "black")) c.surface = OCRT_SURFACE_BLACK;
            else if (!strcmp(s, "flat")) c.surface = OCRT_SURFACE_FLAT;
            else if (!strcmp(s, "black_fresnel_ocean") || !strcmp(s, "black-fresnel-ocean"))
                c.surface = OCRT_SURFACE_BLACK_FRESNEL_OCEAN;
            else if (!strcmp(s, "coxmunk")) {
                fprintf(stderr, "warning: --surface coxmunk is deprecated; use --surface black_fresnel_ocean.\n");
                c.surface = OCRT_SURFACE_BLACK_FRESNEL_OCEAN;
            } else if (!strcmp(s, "lambert")) {
                fprintf(stderr, "error: --surface lambert not implemented (boundary condition not coded).\n");
                return 2;
            } else if (!strcmp(s, "ocean")) {
                fprintf(stderr, "error: --surface ocean (coupled in-water solve) is not on this solve path.\n");
                return 2;
            } else { fprintf(stderr, "error: unknown surface '%s'\n", s); return 2; }
            have_surface = 1;
        }
        else if (!strcmp(a, "--wind-speed")) c.wind_speed = need_d(argc, argv, &i);
        else if (!strcmp(a, "--n-water")) c.n_water = need_d(argc, argv, &i);
        else if (!strcmp(a, "--sigma-type")) {
            c.sigma_type = (int)need_d(argc, argv, &i);
            if (c.sigma_type != 1 && !advanced_on()) {
                fprintf(stderr, "error: --sigma-type %d differs from the default 1 (requires OCRT_ADVANCED=1)\n",
                        c.sigma_type);
                return 2;
            }
        }
        else if (!strcmp(a, "--q-convention")) {
            c.q_convention = (int)need_d(argc, argv, &i);
            if (c.q_convention != 1 && !advanced_on()) {
                fprintf(stderr, "error: --q-convention %d differs from the default 1 (requires OCRT_ADVANCED=1)\n",
                        c.q_convention);
                return 2;
            }
        }
        else if (!strcmp(a, "--pssa")) o.pssa = 1;
        else if (!strcmp(a, "--decouple-sunglint")) c.decouple_sunglint = 1;
        else if (!strcmp(a, "--pressure") || !strcmp(a, "--surface-pressure")) c.pressure_hpa = need_d(argc, argv, &i);
        else if (!strcmp(a, "--no-rayleigh")) c.pressure_hpa = 0.0;
        else if (!strcmp(a, "--rayleigh")) {
            const char *v = need_s(argc, argv, &i);
            if (!strcmp(v, "off")) c.pressure_hpa = 0.0;
            else if (!strcmp(v, "on")) { if (c.pressure_hpa <= 0.0) c.pressure_hpa = 1013.25; }
            else { fprintf(stderr, "error: --rayleigh must be on|off\n"); return 2; }
        }
        else if (!strcmp(a, "--tau-r")) { c.tau_r_input = need_d(argc, argv, &i); o.tau_r_source = OCRT_TAU_R_FROM_INPUT; }
        else if (!strcmp(a, "--aod")) aod = need_d(argc, argv, &i);
        else if (!strcmp(a, "--aod-555")) { aod = need_d(argc, argv, &i); aod_ref_nm = 555.0; }
        else if (!strcmp(a, "--aod-865")) { aod = need_d(argc, argv, &i); aod_ref_nm = 865.0; }
        else if (!strcmp(a, "--aod-ref-wavelength")) aod_ref_nm = need_d(argc, argv, &i);
        else if (!strcmp(a, "--aod-band")) {
            fprintf(stderr, "error: --aod-band was removed because band-specific AOD breaks spectral consistency; "
                            "use --aod-555 or --aod-865\n");
            return 2;
        }
        else if (!strcmp(a, "--mie")) mie_path = need_s(argc, argv, &i);
        else if (!strcmp(a, "--aer-hg-g")) hg_g = need_d(argc, argv, &i);
        else if (!strcmp(a, "--aer-ssa")) ssa = need_d(argc, argv, &i);
        else if (!strcmp(a, "--aer-l-max")) { L = (int)need_d(argc, argv, &i); have_L = 1; }
        else if (!strcmp(a, "--aer-h-km")) o.aer_h_km = need_d(argc, argv, &i);
        else if (!strcmp(a, "--aer")) {
            fprintf(stderr, "error: --aer %s: name the aerosol model file with --mie PATH (.mie)\n",
                    need_s(argc, argv, &i));
            return 2;
        }
        else if (!strcmp(a, "--n-mu")) {
            o.n_mu = (int)need_d(argc, argv, &i);
            if (o.n_mu != 24 && !advanced_on()) {
                fprintf(stderr, "error: --n-mu %d differs from the validated default 24 (requires OCRT_ADVANCED=1)\n",
                        o.n_mu);
                return 2;
            }
        }
        else if (!strcmp(a, "--n-layers")) { o.n_layers = (int)need_d(argc, argv, &i); have_nl = 1; }
        else if (!strcmp(a, "--m-max")) { o.fourier_m_max = (int)need_d(argc, argv, &i); have_m = 1; }
        else if (!strcmp(a, "--sos-max-orders") || !strcmp(a, "--max-orders")) {
            o.max_orders = (int)need_d(argc, argv, &i);
            if (o.max_orders != 20 && !advanced_on()) {
                fprintf(stderr, "error: %s %d differs from the validated default 20 (requires OCRT_ADVANCED=1)\n",
                        a, o.max_orders);
                return 2;
            }
        }
        else if (!strcmp(a, "--sos-tolerance")) {
            o.tolerance = need_d(argc, argv, &i);
            if (o.tolerance != 1e-7 && !advanced_on()) {
                fprintf(stderr, "error: --sos-tolerance %g differs from the validated default 1e-7 "
                                "(requires OCRT_ADVANCED=1)\n", o.tolerance);
                return 2;
            }
        }
        else if (!strcmp(a, "--lut-vza-step") || !strcmp(a, "--vza-gap")) { vstep = need_d(argc, argv, &i); have_lut = 1; }
        else if (!strcmp(a, "--lut-raa-step") || !strcmp(a, "--raa-gap")) { rstep = need_d(argc, argv, &i); have_lut = 1; }
        else if (!strcmp(a, "--lut-vza-max")) vmax = need_d(argc, argv, &i);
        else if (!strcmp(a, "--lut-output")) lut_out = need_s(argc, argv, &i);
        else if (!strcmp(a, "--output-full-grid")) have_lut = 1;
        else if (!strcmp(a, "--batch")) batch = need_s(argc, argv, &i);
        else if (!strcmp(a, "--atm-profile") || !strcmp(a, "--gas-profile")) {
            const char *v = need_s(argc, argv, &i);
            atm_profile = -1;
            for (int k = 0; k < 7; ++k) if (!strcmp(v, profiles[k])) atm_profile = k;
            if (atm_profile < 0) {
                fprintf(stderr, "error: --atm-profile must be one of "
                                "usstd76|tropical|mlsumm|mlwint|sasumm|sawint|userdef\n");
                return 2;
            }
        }
        else if (!strcmp(a, "--gas-column-h2o") || !strcmp(a, "--pwv-g-cm"))
            gas_col[OCRT_GAS_H2O] = need_d(argc, argv, &i) * 6.02214076e23 / 18.01528;
        else if (!strcmp(a, "--gas-column-o3")) gas_col[OCRT_GAS_O3] = need_d(argc, argv, &i) * 2.6868e16;
        else if (!strcmp(a, "--gas-column-no2")) gas_col[OCRT_GAS_NO2] = need_d(argc, argv, &i) * 2.6868e16;
        else if (!strcmp(a, "--gas-column-o2")) gas_col[OCRT_GAS_O2] = need_d(argc, argv, &i);
        else if (!strcmp(a, "--gas-column-co2")) gas_col[OCRT_GAS_CO2] = need_d(argc, argv, &i);
        else if (!strcmp(a, "--gas-column-ch4")) gas_col[OCRT_GAS_CH4] = need_d(argc, argv, &i);
        else { fprintf(stderr, "error: unknown option '%s'\n", a); return usage(); }
    }
    if (!have_surface) {
        fprintf(stderr, "error: --surface is required (black | flat | black_fresnel_ocean)\n");
        return 2;
    }
    if (have_vza != have_raa) {
        fprintf(stderr, "error: single-geometry mode requires BOTH --vza and --raa "
                        "(got only one); omit both for LUT grid mode\n");
        return 2;
    }
    const int single = have_vza && have_raa;
    if (single && have_lut) {
        fprintf(stderr, "error: conflicting mode flags: single geometry (--vza/--raa) vs LUT grid. Pick one.\n");
        return 2;
    }
    if (mie_path && !(aod > 0.0)) {
        fprintf(stderr, "error: aerosol options require --aod-555/--aod-865 > 0 "
                        "(aerosol is disabled at the default --aod-555 0)\n");
        return 2;
    }
    const int aer_on = aod > 0.0;
    if (aer_on && !have_nl) o.n_layers = 400;
    if (mie_path && !have_m) o.fourier_m_max = 16;      /* main.c:3286-3293 */
    if (mie_path && !have_L) L = 80;                   /* main.c:3297-3302 */
    if (!aer_on && have_nl && o.n_layers != 40 && !advanced_on()) {
        fprintf(stderr, "error: --n-layers %d differs from the validated default 40 (requires OCRT_ADVANCED=1)\n",
                o.n_layers);
        return 2;
    }
    if (ocrt_gb_init(0) != OCRT_OK) { fprintf(stderr, "error: %s\n", ocrt_gb_last_error()); return 1; }
    {   /* gas absorption state (main.c:3592-3613) */
        const char *root = getenv("OCRT_GB_INPUTS");
        char afgl_dir[1024], xsec_dir[1024];
        snprintf(afgl_dir, sizeof afgl_dir, "%s/afgl_atm", root && *root ? root : "inputs");
        snprintf(xsec_dir, sizeof xsec_dir, "%s/xsec", root && *root ? root : "inputs");
        ocrt_gas *gas = NULL;
        const int grc = ocrt_gb_gas_create(afgl_dir, xsec_dir, atm_profile, gas_col, &gas);
        if (grc) {
            fprintf(stderr, "error: gas absorption setup failed rc=%d: %s\n", grc, ocrt_gb_last_error());
            return 1;
        }
        o.gas = gas;
        double per[OCRT_N_GAS], tot = 0.0, eff[OCRT_N_GAS];
        int ovr[OCRT_N_GAS];
        ocrt_gb_gas_tau(gas, c.wavelength_nm, per, &tot);
        ocrt_gb_gas_columns(gas, eff, NULL, ovr);
        fprintf(stderr, "rt_absorption (SOS-integrated): \u03bb=%.1fnm \u03c4_abs_col=%.4e\n", c.wavelength_nm, tot);
        for (int g = 0; g < OCRT_N_GAS; ++g)
            fprintf(stderr, "  %s: column=%.3e mol/cm\u00b2%s  \u03c4_abs_col=%.4e\n", gas_names[g], eff[g],
                    ovr[g] ? " (overridden)" : "", per[g]);
    }
    moments_t mom = {0};
    ocrt_aerosol aer;
    memset(&aer, 0, sizeof aer);
    aod_line_t al = {aod, c.wavelength_nm, aod, aer_on ? 1.0 : 0.0};
    ocrt_mie *model = NULL;
    ocrt_mie_aerosol *prep = NULL;
    if (aer_on && mie_path) {
        ocrt_mie_opts mo;
        ocrt_mie_opts_default(&mo);
        mo.L_max = L;
        ocrt_mie_diag md;
        if (ocrt_gb_mie_read(mie_path, &model) ||
            ocrt_gb_mie_prepare(model, c.wavelength_nm, aod, aod_ref_nm, &mo, &prep, &aer, &md)) {
            fprintf(stderr, "error: %s\n", ocrt_gb_last_error());
            return 1;
        }
        al.ref = aod; al.ref_nm = aod_ref_nm; al.band = md.aod_target; al.ratio = md.extinction_ratio;
    } else if (aer_on) {
        if (L < 2) { fprintf(stderr, "error: --aer-l-max must be >= 2\n"); return 2; }
        hg_moments(hg_g, L, &mom);
        aer.tau_a = aod; aer.ssa_a = ssa; aer.L_max = L;
        aer.beta = mom.b; aer.gamma = mom.g; aer.alpha = mom.a; aer.zeta = mom.z;
    }
    if (batch && mie_path) {
        fprintf(stderr, "error: --batch takes the synthetic aerosol expansion (--aod with --aer-hg-g), not --mie\n");
        return 2;
    }
    if (batch) return run_batch(batch, &c, &o, aer_on ? &aer : NULL, hg_g, ssa, aer_on ? L : 0);
    ocrt_result r;
    if (single) {
        const int rc = ocrt_gb_solve_case(&c, &o, aer_on ? &aer : NULL, &r, NULL);
        if (rc) { fprintf(stderr, "error: solve rc=%d: %s\n", rc, ocrt_gb_last_error()); return 1; }
        print_single(&c, &r, al);
        return 0;
    }
    /* LUT grid mode (main.c:3790-3884); the base solve uses vza = raa = 0 */
    if (vstep <= 0 || rstep <= 0 || vmax <= 0 || vmax >= 90.0) {
        fprintf(stderr, "error: invalid LUT grid step/max\n");
        return 2;
    }
    c.vza_deg = 0.0; c.raa_deg = 0.0;
    const int nv = (int)(vmax / vstep) + 1, nr = (int)(360.0 / rstep);
    double *vz = malloc(sizeof(double) * nv), *ra = malloc(sizeof(double) * nr);
    for (int i = 0; i < nv; ++i) vz[i] = i * vstep;
    for (int i = 0; i < nr; ++i) ra[i] = i * rstep;
    const size_t np = (size_t)nv * nr;
    ocrt_lut lut;
    memset(&lut, 0, sizeof lut);
    lut.n_vza = nv; lut.vza_deg = vz; lut.n_raa = nr; lut.raa_deg = ra;
    lut.rho_I = calloc(np, sizeof(double)); lut.rho_Q = calloc(np, sizeof(double)); lut.rho_U = calloc(np, sizeof(double));
    lut.T_diff_dn_dir = calloc(np, sizeof(double)); lut.T_sg_up_dir = calloc(np, sizeof(double));
    lut.T_total_up_dir = calloc(np, sizeof(double));
    const int rc = ocrt_gb_solve_case_lut(&c, &o, aer_on ? &aer : NULL, &r, &lut);
    if (rc) { fprintf(stderr, "error: LUT solve rc=%d: %s\n", rc, ocrt_gb_last_error()); return 1; }
    FILE *fp = lut_out ? fopen(lut_out, "w") : stdout;
    if (!fp) { fprintf(stderr, "error: cannot open LUT output '%s'\n", lut_out); return 1; }
    fprintf(fp, "sza_deg,wavelength_nm,vza_deg,raa_deg,rho_I,rho_Q,rho_U,direct_transmittance,"
                "irradiance_transmittance,diffuse_dn_hemi,diffuse_dn_dir,sunglint_up_flux_ratio_diag,"
                "toa_up_flux_ratio_diag\n");
    const double T_irr = lut.T_dir_dn + lut.T_diff_dn_hemi;
    for (int iv = 0; iv < nv; ++iv)
        for (int ir = 0; ir < nr; ++ir) {
            const size_t k = (size_t)iv * nr + ir;
            fprintf(fp, "%.6f,%.3f,%.6f,%.6f,%.10e,%.10e,%.10e,%.10e,%.10e,%.10e,%.10e,%.10e,%.10e\n",
                    c.sza_deg, c.wavelength_nm, vz[iv], ra[ir], lut.rho_I[k], lut.rho_Q[k], lut.rho_U[k],
                    lut.T_dir_dn, T_irr, lut.T_diff_dn_hemi, lut.T_diff_dn_dir[k], lut.T_sg_up_dir[k],
                    lut.T_total_up_dir[k]);
        }
    if (lut_out) fclose(fp);
    fprintf(stderr, "ocrt: emitted %d x %d = %zu directions to %s\n", nv, nr, np, lut_out ? lut_out : "stdout");
    return 0;
}
