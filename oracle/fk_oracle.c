/*
 * fk_oracle.c -- CPU restatement of the reference's GPP and FF loop nests.
 *
 * TEST INFRASTRUCTURE ONLY (see fk_oracle.h).  Nothing in the CUDA library
 * links or calls this file.
 *
 * Per-term arithmetic follows the reference expression by expression (the
 * same products in the same association, complex multiply as (ac-bd, ad+bc),
 * no fused multiply-add: build with -ffp-contract=off).  The only liberty
 * taken is the ORDER of the outer reductions: the reference sums per-thread
 * partials whose order depends on OpenMP's dynamic schedule, so the oracle
 * stores one partial per (n1, my_igp) and adds them in a fixed order with
 * Neumaier compensation.  Results are therefore independent of thread count
 * and at least as accurate as any schedule of the reference.
 */
#include "fk_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cx;

static inline cx cx_make(double re, double im) { cx r; r.re = re; r.im = im; return r; }
static inline cx cx_ld(const double* p, long i) { return cx_make(p[2 * i], p[2 * i + 1]); }
static inline cx cx_mul(cx a, cx b) { return cx_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cx_conj(cx a) { return cx_make(a.re, -a.im); }
static inline cx cx_add(cx a, cx b) { return cx_make(a.re + b.re, a.im + b.im); }
static inline cx cx_sub(cx a, cx b) { return cx_make(a.re - b.re, a.im - b.im); }
static inline cx cx_scale(cx a, double s) { return cx_make(a.re * s, a.im * s); }
static inline double cx_norm2(cx a) { return a.re * a.re + a.im * a.im; }

/* Neumaier compensated accumulator (deterministic, order-fixed). */
typedef struct { double s, c; } ksum;
static inline void ks_add(ksum* k, double x) {
    double t = k->s + x;
    if (fabs(k->s) >= fabs(x)) k->c += (k->s - t) + x;
    else k->c += (x - t) + k->s;
    k->s = t;
}
static inline double ks_val(const ksum* k) { return k->s + k->c; }
typedef struct { ksum re, im; } kcx;
static inline void kc_add(kcx* k, cx v) { ks_add(&k->re, v.re); ks_add(&k->im, v.im); }
static inline cx kc_val(const kcx* k) { return cx_make(ks_val(&k->re), ks_val(&k->im)); }
static const kcx KCX_ZERO = {{0.0, 0.0}, {0.0, 0.0}};

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ------------------------------------------------------------------ GPP */

/* Column map igp(my_igp), BGW-Kernels/gppKer.cpp:322-328.  -1 = skipped. */
static int gpp_igp(int my_igp, int nc, const int* inv_igp_index,
                   const int* indinv, int indinv_len) {
    int indigp = inv_igp_index[my_igp];
    int igp;
    if (indigp == nc) igp = nc - 1;
    else if (indigp < 0 || indigp >= indinv_len) return -1;
    else igp = indinv[indigp];
    if (igp >= nc || igp < 0) return -1;
    return igp;
}

/* ssxt_scht_solver, BGW-Kernels/gppKer.cpp:19-65.  ieps_s is the I_eps value
 * the caller passes as I_eps_array_igp_myIgp.  physics != 0: the Fortran
 * form of the same block, gppkernel.deslippe.09.30.2014.f90:288-320 (branch-A
 * cden = wxt**2 - wtilde2, and the sexcut test with wxt < 0). */
static inline void gpp_solver(double wxt, cx wtilde, cx wtilde2, cx Omega2,
                              cx matngmatmgp, cx ieps_s, cx* ssxa, cx* scha, int physics) {
    const double to1 = 1e-6;
    const double limitone = 1.0 / (to1 * 4.0);
    const double limittwo = 0.5 * 0.5;
    cx sch, ssx;
    cx wdiff = cx_make(wxt - wtilde.re, -wtilde.im);
    cx cden = wdiff;
    double rden = 1 / cx_norm2(cden);
    cx delw = cx_scale(cx_mul(wtilde, cx_conj(cden)), rden);
    double delwr = cx_norm2(delw);
    double wdiffr = cx_norm2(wdiff);
    if ((wdiffr > limittwo) && (delwr < limitone)) {
        sch = cx_mul(delw, ieps_s);
        if (physics) {
            /* cden = wxt**2 - wtilde2; rden = 1/(cden*conj(cden)); ssx = Omega2*conj(cden)*rden */
            cx cd = cx_make(wxt * wxt - wtilde2.re, 0.0 - wtilde2.im);
            double rd = 1.0 / cx_norm2(cd);
            ssx = cx_scale(cx_mul(Omega2, cx_conj(cd)), rd);
        } else {
            double w2 = wxt * wxt;               /* pow(wxt,2) */
            double rd = 1.00 / (w2 * w2);        /* real(cden*conj(cden)) */
            /* Omega2 * conj(cden) with cden = (w2, 0) */
            cx t = cx_make(Omega2.re * w2 - Omega2.im * (-0.0), Omega2.re * (-0.0) + Omega2.im * w2);
            ssx = cx_scale(t, rd);
        }
    } else if (delwr > to1) {
        sch = cx_make(0.0, 0.0);
        cx c = cx_mul(cx_scale(wtilde2, 4.00), cx_make(delw.re + 0.50, delw.im));
        double rd = 1.00 / cx_norm2(c);
        cx negO = cx_make(-Omega2.re, -Omega2.im);
        ssx = cx_mul(cx_scale(cx_mul(negO, cx_conj(c)), rd), delw);
    } else {
        sch = cx_make(0.0, 0.0);
        ssx = cx_make(0.0, 0.0);
    }
    /* the C++ sexcut test (:60-61) requires abs(wxt) < 0 and never fires; the
     * Fortran one (:319-320) zeroes ssx when wxt < 0 and |ssx| > sexcut*|I_eps| */
    if (physics && wxt < 0.0 && hypot(ssx.re, ssx.im) > 4.0 * hypot(ieps_s.re, ieps_s.im))
        ssx = cx_make(0.0, 0.0);
    *ssxa = cx_mul(matngmatmgp, ssx);
    *scha = cx_mul(matngmatmgp, sch);
}

/* std::complex division and magnitude as the textbook forms: a*conj(b)/|b|^2
 * and hypot(re, im) (the reference's libstdc++ results agree to ~1 ulp). */
static inline cx cx_div(cx a, cx b) {
    const double n = b.re * b.re + b.im * b.im;
    return cx_make((a.re * b.re + a.im * b.im) / n, (a.im * b.re - a.re * b.im) / n);
}
static inline double cx_abs(cx a) { return hypot(a.re, a.im); }

/* gppsum == 1, one (n1, my_igp): gppKerSeq.cpp's flagOCC_solver (:90-139) for
 * occupied bands, else its driver's block loop (:430-447) over
 * noflagOCC_solver (:206-242).  igmax = igp.  sch_array/ssx_array as the
 * driver accumulates them (before the vcoul weight). */
static void gpp_half_sum(int occ_band, int n1, int igp, int nc, const double* aqsm, const double* aqsn,
                         const double* erow, const double* wrow, const double* wx, cx sch_array[3],
                         cx ssx_array[3]) {
    const double to1 = 1e-6, gamma = 0.5;
    const double limitone = 1.0 / (to1 * 4.0), limittwo = 0.5 * 0.5;
    const int igmax = igp;
    const cx aqm = cx_ld(aqsm, (long)n1 * nc + igp);
    const cx mygpvar1 = cx_conj(aqm), mygpvar2 = aqm;
    const double* mrow = aqsm + 2L * n1 * nc;
    const double* nrow = aqsn + 2L * n1 * nc;
    if (occ_band) {
        for (int iw = 0; iw < 3; ++iw) {
            const double wxt = wx[iw];
            cx ssxt = {0, 0}, scht = {0, 0}, matngpmatmg = {0, 0};
            for (int ig = 0; ig < igmax; ++ig) {
                const cx wt = cx_ld(wrow, ig), eps = cx_ld(erow, ig);
                const cx wt2 = cx_mul(wt, wt);
                const cx Omega2 = cx_mul(wt2, eps);
                if (cx_abs(Omega2) < to1) break;
                const cx matngmatmgp = cx_mul(cx_ld(nrow, ig), mygpvar1);
                if (ig != igp) matngpmatmg = cx_mul(cx_conj(cx_ld(mrow, ig)), mygpvar2);
                const cx halfinvwtilde = cx_div(cx_make(0.5, 0.0), wt);
                const cx wmw = cx_make(wxt - wt.re, -wt.im);
                const cx delw = cx_mul(wmw, halfinvwtilde);
                const double ad = cx_abs(delw), delw2 = ad * ad;
                cx sch, ssx;
                if (cx_abs(wmw) < gamma || delw2 < to1) {
                    sch = cx_make(0.0, 0.0);
                    if (cx_abs(wt) > to1)
                        ssx = cx_div(cx_make(-Omega2.re, -Omega2.im),
                                     cx_mul(cx_scale(wt2, 4.0), cx_make(1.0 + delw.re, delw.im)));
                    else
                        ssx = cx_make(0.0, 0.0);
                } else {
                    sch = cx_div(cx_mul(wt, eps), wmw);
                    ssx = cx_div(Omega2, cx_make(wxt * wxt - wt2.re, -wt2.im));
                }
                /* the sexcut test (:119-120) requires abs(wxt) < 0 and never fires */
                cx ssxa, scha;
                if (ig != igp - 1) {
                    ssxa = cx_add(cx_mul(matngmatmgp, ssx), cx_mul(matngpmatmg, cx_conj(ssx)));
                    scha = cx_add(cx_mul(matngmatmgp, sch), cx_mul(matngpmatmg, cx_conj(sch)));
                } else {
                    ssxa = cx_mul(matngmatmgp, ssx);
                    scha = cx_mul(matngmatmgp, sch);
                }
                ssxt = cx_add(ssxt, ssxa);
                scht = cx_add(scht, scha);
            }
            ssx_array[iw] = cx_add(ssx_array[iw], ssxt);
            sch_array[iw] = cx_add(sch_array[iw], cx_scale(scht, 0.5));
        }
        return;
    }
    const int igblk = 512;
    for (int igbeg = 0; igbeg < igmax; igbeg += igblk) {
        const int igend = igbeg + igblk - 1 < igmax ? igbeg + igblk - 1 : igmax;
        for (int iw = 0; iw < 3; ++iw) {
            const double wxt = wx[iw];
            cx scht = {0, 0};
            const int top = igend < igmax - 1 ? igend : igmax - 1;
            /* the interior range (:210): both terms of the pair */
            for (int ig = igbeg; ig < top; ++ig) {
                const cx wt = cx_ld(wrow, ig);
                const cx matngmatmgp = cx_mul(cx_ld(nrow, ig), mygpvar1);
                const cx wdiff = cx_make(wxt - wt.re, -wt.im);
                const cx delw = cx_div(wt, wdiff);
                const double delw2 = cx_norm2(delw), wdiffr = cx_norm2(wdiff);
                const double mult = (fabs(wdiffr) < limittwo || delw2 > limitone) ? 1.0 : 0.0;
                const cx sch = cx_scale(cx_mul(delw, cx_ld(erow, ig)), mult);
                const cx scha = cx_add(cx_mul(matngmatmgp, sch),
                                       cx_mul(cx_mul(cx_conj(cx_ld(mrow, ig)), mygpvar2), cx_conj(sch)));
                scht = cx_add(scht, scha);
            }
            /* the diagonal ig = igmax (:225-240), reached only when igend == igmax-1 */
            if (igend == igmax - 1) {
                const int ig = igmax;
                const cx wt = cx_ld(wrow, ig);
                const cx matngmatmgp = cx_mul(cx_ld(nrow, ig), mygpvar1);
                const cx wdiff = cx_make(wxt - wt.re, -wt.im);
                const cx delw = cx_div(wt, wdiff);
                const double delw2 = cx_norm2(delw), wdiffr = cx_norm2(wdiff);
                const double mult = (fabs(wdiffr) < limittwo || delw2 > limitone) ? 1.0 : 0.0;
                const cx sch = cx_scale(cx_mul(delw, cx_ld(erow, ig)), mult);
                scht = cx_add(scht, cx_mul(matngmatmgp, sch));
            }
            sch_array[iw] = cx_add(sch_array[iw], cx_scale(scht, 0.5));
        }
    }
}

int orc_gpp(int nb, int nv, int nc, int ng,
            const double* aqsm, const double* aqsn,
            const double* I_eps, const double* wtilde, const double* vcoul,
            const int* inv_igp_index, const int* indinv, int indinv_len,
            const double* wx, unsigned flags, int nthreads,
            double* achtemp, double* asxtemp, double* acht_n1_loc,
            double* achstemp, double* sch_out, double* ssx_out) {
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb) return -1;
    const int quirk = (flags & ORC_GPP_ROOT_QUIRKS) != 0;
    const int physics = (flags & ORC_GPP_PHYSICS) != 0;
    if (quirk && (long)(ng - 1) * ng + nc > (long)ng * nc) return -1;
    if (physics && (flags & (ORC_GPP_ROOT_QUIRKS | ORC_GPP_HALF_SUM))) return -1;
    set_threads(nthreads);
    const double limitone = 1.0 / (1e-6 * 4.0);
    const double limittwo = 0.5 * 0.5;
    const int igblk = quirk ? nc : 512; /* gppKer.cpp sums the whole ig range at once */
    const int nvb = nv;

    int* igpmap = (int*)malloc(sizeof(int) * (size_t)ng);
    cx* sch = (cx*)calloc((size_t)nb * ng * 3, sizeof(cx));
    cx* ssx = (cx*)calloc((size_t)(nvb > 0 ? nvb : 1) * ng * 3, sizeof(cx));
    cx* stat = (cx*)calloc((size_t)nb * ng, sizeof(cx));
    if (!igpmap || !sch || !ssx || !stat) { free(igpmap); free(sch); free(ssx); free(stat); return -2; }
    for (int i = 0; i < ng; ++i) igpmap[i] = gpp_igp(i, nc, inv_igp_index, indinv, indinv_len);

    for (int n1 = 0; n1 < nb; ++n1) {
        const int flag_occ = n1 < nv;
#pragma omp parallel for schedule(dynamic)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            if (igp < 0) continue;
            cx sch_array[3] = {{0, 0}, {0, 0}, {0, 0}};
            cx ssx_array[3] = {{0, 0}, {0, 0}, {0, 0}};
            const double* wrow = wtilde + 2L * my_igp * nc;
            const double* erow = I_eps + 2L * my_igp * nc;
            const double* nrow = aqsn + 2L * n1 * nc;
            const cx aqm = cx_ld(aqsm, (long)n1 * nc + igp);
            if (flags & ORC_GPP_HALF_SUM) {
                gpp_half_sum(flag_occ, n1, igp, nc, aqsm, aqsn, erow, wrow, wx, sch_array, ssx_array);
            } else if (flag_occ) {
                /* flagOCC_solver, BGW-Kernels/gppKer.cpp:130-159 */
                for (int iw = 0; iw < 3; ++iw) {
                    cx ssxt = {0, 0}, scht = {0, 0};
                    const double wxt = wx[iw];
                    for (int ig = 0; ig < nc; ++ig) {
                        cx wt = cx_ld(wrow, ig);
                        cx wt2 = cx_mul(wt, wt);
                        cx Omega2 = cx_mul(wt2, cx_ld(erow, ig));
                        cx mygpvar1 = cx_conj(aqm);
                        cx matngmatmgp = cx_mul(cx_ld(nrow, ig), mygpvar1);
                        cx ieps_s = quirk ? cx_ld(I_eps, (long)my_igp * ng + ig) : cx_ld(erow, ig);
                        cx ssxa, scha;
                        gpp_solver(wxt, wt, wt2, Omega2, matngmatmgp, ieps_s, &ssxa, &scha, physics);
                        ssxt = cx_add(ssxt, ssxa);
                        scht = cx_add(scht, scha);
                    }
                    ssx_array[iw] = cx_add(ssx_array[iw], ssxt);
                    sch_array[iw] = cx_add(sch_array[iw], cx_scale(scht, 0.5));
                }
            } else {
                /* cache-blocked noflag block, BGW-Kernels/gppKer.cpp:349-413 */
                const cx mygpvar1 = cx_conj(aqm);
                for (int igbeg = 0; igbeg < nc; igbeg += igblk) {
                    const int igend = igbeg + igblk < nc ? igbeg + igblk : nc;
                    for (int iw = 0; iw < 3; ++iw) {
                        cx scht = {0, 0};
                        const double wxt = wx[iw];
                        for (int ig = igbeg; ig < igend; ++ig) {
                            cx wt = cx_ld(wrow, ig);
                            cx wdiff = cx_make(wxt - wt.re, -wt.im);
                            cx cden = wdiff;
                            double rden = cx_norm2(cden);
                            rden = 1 / rden;
                            cx delw = cx_scale(cx_mul(wt, cx_conj(cden)), rden);
                            double delwr = cx_norm2(delw);
                            double wdiffr = cx_norm2(wdiff);
                            cx scha = cx_mul(cx_mul(cx_mul(mygpvar1, cx_ld(nrow, ig)), delw), cx_ld(erow, ig));
                            if (quirk || ((wdiffr > limittwo) && (delwr < limitone)))
                                scht = cx_add(scht, scha);
                        }
                        sch_array[iw] = cx_add(sch_array[iw], cx_scale(scht, 0.5));
                    }
                }
            }
            cx* so = sch + ((size_t)n1 * ng + my_igp) * 3;
            for (int iw = 0; iw < 3; ++iw) so[iw] = sch_array[iw];
            if (flag_occ) {
                cx* xo = ssx + ((size_t)n1 * ng + my_igp) * 3;
                for (int iw = 0; iw < 3; ++iw) xo[iw] = ssx_array[iw];
            }
            if (flags & ORC_GPP_ACHSTEMP) {
                /* static CH remainder, gppkernel.deslippe.09.30.2014.f90:213-228 */
                cx schstemp = {0, 0};
                for (int ig = 0; ig < nc; ++ig)
                    schstemp = cx_sub(schstemp, cx_mul(cx_mul(cx_ld(nrow, ig), cx_ld(erow, ig)), cx_conj(aqm)));
                stat[(size_t)n1 * ng + my_igp] = cx_scale(cx_scale(schstemp, vcoul[igp]), 0.5);
            }
        }
    }

    /* accumulation into the outputs, BGW-Kernels/gppKer.cpp:416-439 */
    kcx acc[3] = {KCX_ZERO, KCX_ZERO, KCX_ZERO};
    kcx asx[3] = {KCX_ZERO, KCX_ZERO, KCX_ZERO};
    kcx st = KCX_ZERO;
    /* asxtemp += ssx*occ*vcoul (BGW-Kernels/gppKer.cpp:419); the Fortran subtracts it (f90:393) */
    const double occ = physics ? -1.0 : 1.0;
    for (int n1 = 0; n1 < nb; ++n1) {
        kcx n1loc = KCX_ZERO;
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            if (igp < 0) continue;
            const cx* so = sch + ((size_t)n1 * ng + my_igp) * 3;
            for (int iw = 0; iw < 3; ++iw) kc_add(&acc[iw], cx_scale(so[iw], vcoul[igp]));
            kc_add(&n1loc, cx_scale(so[2], vcoul[igp]));
            if (n1 < nv) {
                const cx* xo = ssx + ((size_t)n1 * ng + my_igp) * 3;
                for (int iw = 0; iw < 3; ++iw) kc_add(&asx[iw], cx_scale(cx_scale(xo[iw], occ), vcoul[igp]));
            }
            if (flags & ORC_GPP_ACHSTEMP) kc_add(&st, stat[(size_t)n1 * ng + my_igp]);
        }
        if (acht_n1_loc) { cx v = kc_val(&n1loc); acht_n1_loc[2 * n1] = v.re; acht_n1_loc[2 * n1 + 1] = v.im; }
    }
    for (int iw = 0; iw < 3; ++iw) {
        cx a = kc_val(&acc[iw]), x = kc_val(&asx[iw]);
        achtemp[2 * iw] = a.re; achtemp[2 * iw + 1] = a.im;
        asxtemp[2 * iw] = x.re; asxtemp[2 * iw + 1] = x.im;
    }
    if (achstemp) { cx v = kc_val(&st); achstemp[0] = v.re; achstemp[1] = v.im; }
    if (sch_out) memcpy(sch_out, sch, sizeof(cx) * (size_t)nb * ng * 3);
    if (ssx_out && nv > 0) memcpy(ssx_out, ssx, sizeof(cx) * (size_t)nv * ng * 3);
    free(igpmap); free(sch); free(ssx); free(stat);
    return 0;
}

/* ------------------------------------------------------ real-valued GPP */

/* ssxt_scht_solver of gppKer_real.cpp:17-63 (the sexcut test at :58-59 needs
 * abs(wxt) < 0 and never fires); returns ssx and sch before the
 * matngmatmgp factor. */
static inline void gpp_real_solver(double wxt, double wtilde, double wtilde2, double Omega2, double ieps,
                                   double* ssx, double* sch) {
    const double to1 = 1e-6;
    const double limitone = 1.0 / (to1 * 4.0), limittwo = 0.5 * 0.5;
    const double wdiff = wxt - wtilde;
    double cden = wdiff;
    double rden = 1 / (cden * cden);
    const double delw = wtilde * cden * rden;
    const double delwr = delw * delw, wdiffr = wdiff * wdiff;
    if ((wdiffr > limittwo) && (delwr < limitone)) {
        *sch = delw * ieps;
        cden = wxt * wxt; /* pow(wxt,2) */
        rden = 1.00 / (cden * cden);
        *ssx = Omega2 * cden * rden;
    } else if (delwr > to1) {
        *sch = 0.0;
        cden = 4.00 * wtilde2 * (delw + 0.50);
        rden = 1.00 / (cden * cden);
        *ssx = -Omega2 * cden * rden * delw;
    } else {
        *sch = 0.0;
        *ssx = 0.0;
    }
}

int orc_gpp_real(int nb, int nv, int nc, int ng,
                 const double* aqsm, const double* aqsn,
                 const double* I_eps, const double* wtilde, const double* vcoul,
                 const int* inv_igp_index, const int* indinv, int indinv_len,
                 const double* wx, unsigned flags, int nthreads,
                 double* achtemp, double* asxtemp, double* acht_n1_loc,
                 double* sch_out, double* ssx_out) {
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb) return -1;
    set_threads(nthreads);
    const double limitone = 1.0 / (1e-6 * 4.0), limittwo = 0.5 * 0.5;
    const int zero_masked = (flags & ORC_GPP_REAL_ZERO_MASKED) != 0;
    int* igpmap = (int*)malloc(sizeof(int) * (size_t)ng);
    double* sch = (double*)calloc((size_t)nb * ng * 3, sizeof(double));
    double* ssx = (double*)calloc((size_t)(nv > 0 ? nv : 1) * ng * 3, sizeof(double));
    if (!igpmap || !sch || !ssx) { free(igpmap); free(sch); free(ssx); return -2; }
    for (int i = 0; i < ng; ++i) igpmap[i] = gpp_igp(i, nc, inv_igp_index, indinv, indinv_len);

    for (int n1 = 0; n1 < nb; ++n1) {
        const int flag_occ = n1 < nv;
#pragma omp parallel for schedule(dynamic)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            if (igp < 0) continue;
            const double* erow = I_eps + (size_t)my_igp * nc;
            const double* wrow = wtilde + (size_t)my_igp * nc;
            const double* nrow = aqsn + (size_t)n1 * nc;
            const double mygpvar1 = aqsm[(size_t)n1 * nc + igp];
            double sch_array[3] = {0, 0, 0}, ssx_array[3] = {0, 0, 0};
            if (flag_occ) {
                /* flagOCC_solver, gppKer_real.cpp:124-153 */
                for (int iw = 0; iw < 3; ++iw) {
                    const double wxt = wx[iw];
                    double ssxt = 0.0, scht = 0.0;
                    for (int ig = 0; ig < nc; ++ig) {
                        const double w = wrow[ig];
                        const double w2 = w * w; /* std::pow(wtilde, 2) */
                        const double Omega2 = w2 * erow[ig];
                        const double matngmatmgp = nrow[ig] * mygpvar1;
                        double x, h;
                        gpp_real_solver(wxt, w, w2, Omega2, erow[ig], &x, &h);
                        ssxt += matngmatmgp * x;
                        scht += matngmatmgp * h;
                    }
                    ssx_array[iw] += ssxt;
                    sch_array[iw] += 0.5 * scht;
                }
            } else {
                /* the reference program's block loop, gppKer_real.cpp:341-383: scha persists
                 * over blocks and frequencies of this (n1, my_igp) */
                const int igblk = 512;
                double scha[512];
                memset(scha, 0, sizeof scha);
                for (int igbeg = 0, nblk = 0; igbeg < nc; igbeg += igblk, ++nblk) {
                    const int igend = igblk < nc - igblk * nblk ? igblk : nc - igblk * nblk;
                    for (int iw = 0; iw < 3; ++iw) {
                        const double wxt = wx[iw];
                        double scht = 0.0;
                        for (int ig = 0; ig < igend; ++ig) {
                            const int g = ig + nblk * igblk;
                            const double wdiff = wxt - wrow[g];
                            const double cden = wdiff;
                            double rden = cden * cden;
                            rden = 1 / rden;
                            const double delw = wrow[g] * cden * rden;
                            const double delwr = delw * delw, wdiffr = wdiff * wdiff;
                            if ((wdiffr > limittwo) && (delwr < limitone))
                                scha[ig] = mygpvar1 * nrow[g] * delw * erow[g];
                            else if (zero_masked)
                                scha[ig] = 0.0;
                        }
                        for (int ig = 0; ig < igend; ++ig) scht += scha[ig];
                        sch_array[iw] += 0.5 * scht;
                    }
                }
            }
            double* so = sch + ((size_t)n1 * ng + my_igp) * 3;
            for (int iw = 0; iw < 3; ++iw) so[iw] = sch_array[iw];
            if (flag_occ) {
                double* xo = ssx + ((size_t)n1 * ng + my_igp) * 3;
                for (int iw = 0; iw < 3; ++iw) xo[iw] = ssx_array[iw];
            }
        }
    }

    /* accumulation into the outputs, gppKer_real.cpp:385-412 */
    ksum acc[3] = {{0, 0}, {0, 0}, {0, 0}}, asx[3] = {{0, 0}, {0, 0}, {0, 0}};
    const double occ = 1.0;
    for (int n1 = 0; n1 < nb; ++n1) {
        ksum n1loc = {0, 0};
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            if (igp < 0) continue;
            const double* so = sch + ((size_t)n1 * ng + my_igp) * 3;
            for (int iw = 0; iw < 3; ++iw) ks_add(&acc[iw], so[iw] * vcoul[igp]);
            ks_add(&n1loc, so[2] * vcoul[igp]);
            if (n1 < nv) {
                const double* xo = ssx + ((size_t)n1 * ng + my_igp) * 3;
                for (int iw = 0; iw < 3; ++iw) ks_add(&asx[iw], xo[iw] * occ * vcoul[igp]);
            }
        }
        if (acht_n1_loc) acht_n1_loc[n1] = ks_val(&n1loc);
    }
    for (int iw = 0; iw < 3; ++iw) {
        achtemp[iw] = ks_val(&acc[iw]);
        asxtemp[iw] = ks_val(&asx[iw]);
    }
    if (sch_out) memcpy(sch_out, sch, sizeof(double) * (size_t)nb * ng * 3);
    if (ssx_out && nv > 0) memcpy(ssx_out, ssx, sizeof(double) * (size_t)nv * ng * 3);
    free(igpmap); free(sch); free(ssx);
    return 0;
}

/* ------------------------------------------------------------------- FF */

void orc_ff_compute_fact(double wx, int nFreq, const double* dFreqGrid,
                         double* fact1, double* fact2, int* ifreq,
                         int loop, int flag_occ) {
    /* FFKer_cori/ffKernel.cpp:30-78, including its quirks: a loop-1 bracket
     * of [grid0, grid1] (ifreq 0) is remapped to the last interval, and the
     * loop-2 "ifreq == -1" test never fires. */
    if (loop == 1 && wx > 0.00) {
        for (int ijk = 0; ijk < nFreq - 1; ++ijk)
            if (wx > dFreqGrid[ijk] && wx < dFreqGrid[ijk + 1]) *ifreq = ijk;
        if (*ifreq == 0) *ifreq = nFreq - 2;
        *fact1 = (dFreqGrid[*ifreq + 1] - wx) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
        *fact2 = (wx - dFreqGrid[*ifreq]) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
    } else if (loop == 1) {
        for (int ijk = 0; ijk < nFreq - 1; ++ijk)
            if (-wx > dFreqGrid[ijk] && -wx < dFreqGrid[ijk + 1]) *ifreq = ijk;
        if (*ifreq == 0) *ifreq = nFreq - 2;
        *fact1 = (dFreqGrid[*ifreq + 1] + wx) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
        *fact2 = (-dFreqGrid[*ifreq] - wx) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
    }
    if (loop == 2 && wx > 0.00) {
        for (int ijk = 0; ijk < nFreq - 1; ++ijk)
            if (wx > dFreqGrid[ijk] && wx < dFreqGrid[ijk + 1]) *ifreq = ijk;
        if (*ifreq == -1) *ifreq = nFreq - 2;
        *fact1 = -0.5 * (dFreqGrid[*ifreq + 1] - wx) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
        *fact2 = -0.5 * (wx - dFreqGrid[*ifreq]) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
    } else if (loop == 2 && flag_occ) {
        wx = -wx;
        *ifreq = 0;
        for (int ijk = 0; ijk < nFreq - 1; ++ijk)
            if (wx > dFreqGrid[ijk] && wx < dFreqGrid[ijk + 1]) *ifreq = ijk;
        if (*ifreq == 0) *ifreq = nFreq - 2;
        *fact1 = (dFreqGrid[*ifreq + 1] - wx) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
        *fact2 = (wx - dFreqGrid[*ifreq]) / (dFreqGrid[*ifreq + 1] - dFreqGrid[*ifreq]);
    }
}

/* GPUComplex_divide(a, b), FFKer_cori/Complex.h:201-211 */
static inline cx ff_cdiv(cx a, cx b) {
    cx bc = cx_conj(b);
    cx num = cx_mul(a, bc);
    cx den = cx_mul(b, bc);
    return cx_make(num.re / den.re, num.im / den.re);
}

int orc_ff(int nb, int nv, int nc, int ng, int nfreq, int ne,
           const double* aqsm, const double* aqsn,
           const double* I_epsR, const double* I_epsA, const double* vcoul,
           const int* inv_igp_index, const int* indinv,
           const double* ekq, const double* dFreqGrid, const double* dFreqBrd,
           const double* pref, double pref_zb,
           double freqevalmin, double freqevalstep, double occ,
           unsigned flags, int nthreads,
           double* achsDtemp_o, double* asxDtemp_o, double* achDtemp_o,
           double* achDtemp_cor_o, double* ach2Dtemp_o, double* schDt_o) {
    if (nb <= 0 || nc <= 0 || ng <= 0 || nfreq < 2 || ne <= 0 || nv < 0 || nv > nb || ng > nc) return -1;
    set_threads(nthreads);
    const long plane = (long)ng * nc;
    int* igpmap = (int*)malloc(sizeof(int) * (size_t)ng);
    cx* part = (cx*)calloc((size_t)nb * ng, sizeof(cx));
    cx* schDt = (cx*)calloc((size_t)nb * nfreq, sizeof(cx));
    if (!igpmap || !part || !schDt) { free(igpmap); free(part); free(schDt); return -2; }
    for (int i = 0; i < ng; ++i) {
        int g = indinv[inv_igp_index[i]];
        if (g < 0 || g >= nc) { free(igpmap); free(part); free(schDt); return -1; }
        igpmap[i] = g;
    }

    /* achsDtemp_Kernel, FFKer_cori/ffKernel.cpp:107-131 */
#pragma omp parallel for collapse(2) schedule(static)
    for (int n1 = 0; n1 < nb; ++n1)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            const cx cm = cx_conj(cx_ld(aqsm, (long)n1 * nc + igp));
            const double* er = I_epsR + 2 * (1 * plane + (long)my_igp * nc);
            cx s = {0, 0};
            for (int ig = 0; ig < nc; ++ig)
                s = cx_sub(s, cx_mul(cx_mul(cx_ld(aqsn, (long)n1 * nc + ig), cm), cx_ld(er, ig)));
            part[(size_t)n1 * ng + my_igp] = cx_scale(s, vcoul[igp] * 0.5);
        }
    {
        kcx a = KCX_ZERO;
        for (size_t i = 0; i < (size_t)nb * ng; ++i) kc_add(&a, part[i]);
        cx v = kc_val(&a);
        achsDtemp_o[0] = v.re; achsDtemp_o[1] = v.im;
    }

    /* asxDtemp_Kernel + ssxDittt_kernel, FFKer_cori/ffKernel.cpp:80-104,133-153.
     * wx does not depend on iw (:140), so every iw receives the same sum. */
    kcx* asx = (kcx*)malloc(sizeof(kcx) * (size_t)ne);
    for (int iw = 0; iw < ne; ++iw) asx[iw] = KCX_ZERO;
    for (int n1 = 0; n1 < nv; ++n1) {
        const double wx = freqevalmin - ekq[n1] + freqevalstep;
        double fact1 = 0.00, fact2 = 0.00;
        int ifreq = 0;
        orc_ff_compute_fact(wx, nfreq, dFreqGrid, &fact1, &fact2, &ifreq, 1, 0);
#pragma omp parallel for schedule(static)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpmap[my_igp];
            const cx cm = cx_conj(cx_ld(aqsm, (long)n1 * nc + igp));
            const double* e0 = I_epsR + 2 * ((long)ifreq * plane + (long)my_igp * nc);
            const double* e1 = I_epsR + 2 * ((long)(ifreq + 1) * plane + (long)my_igp * nc);
            cx s = {0, 0};
            for (int ig = 0; ig < nc; ++ig) {
                cx ssxDit = cx_add(cx_scale(cx_ld(e0, ig), fact1), cx_scale(cx_ld(e1, ig), fact2));
                s = cx_add(s, cx_scale(cx_mul(cx_ld(aqsn, (long)n1 * nc + ig), cx_mul(cm, ssxDit)), vcoul[igp]));
            }
            part[my_igp] = s;
        }
        kcx t = KCX_ZERO;
        for (int my_igp = 0; my_igp < ng; ++my_igp) kc_add(&t, part[my_igp]);
        cx v = cx_scale(kc_val(&t), occ);
        for (int iw = 0; iw < ne; ++iw) kc_add(&asx[iw], v);
    }

    /* schDt_matrix: zero in the reference C++ (ffKernel.cpp:421-422), or the
     * band x G x G' contraction of ffkernel.deslippe.best.f90.back1:402-418 */
    if (flags & ORC_FF_SCHDT_GEMM) {
        cx* tz = (cx*)calloc((size_t)nb * nfreq * ng, sizeof(cx));
#pragma omp parallel for collapse(3) schedule(static)
        for (int n1 = 0; n1 < nb; ++n1)
            for (int f = 0; f < nfreq; ++f)
                for (int my_igp = 0; my_igp < ng; ++my_igp) {
                    const double* er = I_epsR + 2 * ((long)f * plane + (long)my_igp * nc);
                    cx s = {0, 0};
                    for (int ig = 0; ig < nc; ++ig)
                        s = cx_add(s, cx_mul(cx_ld(er, ig), cx_ld(aqsn, (long)n1 * nc + ig)));
                    tz[((size_t)n1 * nfreq + f) * ng + my_igp] = s;
                }
        for (int n1 = 0; n1 < nb; ++n1)
            for (int f = 0; f < nfreq; ++f) {
                kcx a = KCX_ZERO;
                for (int my_igp = 0; my_igp < ng; ++my_igp)
                    kc_add(&a, cx_mul(tz[((size_t)n1 * nfreq + f) * ng + my_igp],
                                      cx_conj(cx_ld(aqsm, (long)n1 * nc + igpmap[my_igp]))));
                schDt[(size_t)n1 * nfreq + f] = kc_val(&a);
            }
        free(tz);
    }
    if (schDt_o) memcpy(schDt_o, schDt, sizeof(cx) * (size_t)nb * nfreq);

    /* achDtemp_Kernel + calculate_schDt_lin3, FFKer_cori/ffKernel.cpp:10-28,
     * 155-210, in sequential (n1, ifreq, iw) order.  The reference runs the
     * (n1, ifreq) loop under collapse(2) with shared sch2Di/schDi_cor arrays;
     * the sequential order is the race-free reading of it. */
    const int physics = (flags & ORC_FF_PHYSICS) != 0;
    const double fminI = physics ? freqevalmin : (double)(int)freqevalmin;
    const double fstepI = physics ? freqevalstep : (double)(int)freqevalstep;
    kcx* achd = (kcx*)malloc(sizeof(kcx) * (size_t)ne);
    cx* sch2Di = (cx*)calloc((size_t)ne, sizeof(cx));
    cx* schDi_cor = (cx*)calloc((size_t)ne, sizeof(cx));
    for (int iw = 0; iw < ne; ++iw) achd[iw] = KCX_ZERO;
    const cx pref_zb_compl = cx_make(0.00, pref_zb);
    for (int n1 = 0; n1 < nb; ++n1) {
        const int flag_occ = n1 < nv;
        for (int ifreq = 0; ifreq < nfreq; ++ifreq) {
            const cx schDtv = schDt[(size_t)n1 * nfreq + ifreq];
            const double cedifft_zb = dFreqGrid[ifreq];
            const cx brd = cx_ld(dFreqBrd, ifreq);
            const cx cedifft_coh = cx_make(cedifft_zb - brd.re, 0.00 - brd.im);
            if (ifreq != 0) {
                const double right = cedifft_zb, left = dFreqGrid[ifreq - 1];
                const cx L = schDt[(size_t)n1 * nfreq + ifreq - 1];
                /* operator+ and operator- of GPUComplex update their left
                 * operand (FFKer_cori/Complex.h:48-60): (R+L)*0.5 is the average
                 * and the "difference" is ((R+L)-L). */
                const cx RL = cx_add(schDtv, L);
                const cx schDt_avg = cx_scale(RL, 0.5);
                const cx schDt_lin = cx_sub(RL, L);
                const double dd = right - left;
                const cx schDt_lin2 = cx_make(schDt_lin.re / dd, schDt_lin.im / dd);
                for (int iw = 0; iw < ne; ++iw) {
                    sch2Di[iw] = cx_make(0.0, 0.0);
                    const double ew = fminI - ekq[n1] + (double)(iw - 1) * fstepI;
                    double intfact = (ew - right) / (ew - left);
                    if (intfact < 0.0001) intfact = 0.0001;
                    if (intfact > 10000) intfact = 10000;
                    intfact = -log(intfact);
                    sch2Di[iw] = cx_sub(sch2Di[iw], cx_scale(cx_mul(pref_zb_compl, schDt_avg), intfact));
                    cx lin3;
                    if (flag_occ) {
                        double i2 = fabs((ew + right) / (ew + left));
                        if (i2 < 0.0001) i2 = 0.0001;
                        if (i2 > 10000) i2 = 10000;
                        i2 = log(i2);
                        const double ewn = -fminI - ekq[n1] + (double)(iw - 1) * fstepI;
                        lin3 = cx_scale(cx_add(L, schDt_lin2), (ewn - left) * i2);
                    } else {
                        lin3 = cx_scale(cx_add(L, schDt_lin2), (ew - left) * intfact);
                    }
                    lin3 = cx_add(schDt_lin, lin3);
                    schDi_cor[iw] = cx_sub(schDi_cor[iw], cx_mul(pref_zb_compl, lin3));
                }
            }
            for (int iw = 0; iw < ne; ++iw) {
                const double wx = freqevalmin - ekq[n1] + (iw - 1) * freqevalstep;
                const cx tmp = cx_make(0.00, pref[ifreq]);
                const cx den = cx_make(wx - cedifft_coh.re, 0 - cedifft_coh.im);
                const cx schDi = cx_sub(cx_make(0.0, 0.0), ff_cdiv(cx_mul(tmp, schDtv), den));
                kc_add(&achd[iw], schDi);
            }
        }
    }

    /* achDtemp_cor_Kernel + schDttt_corKernel1/2, FFKer_cori/ffKernel.cpp:212-300 */
    kcx* cor = (kcx*)malloc(sizeof(kcx) * (size_t)ne);
    kcx* a2 = (kcx*)malloc(sizeof(kcx) * (size_t)ne);
    for (int iw = 0; iw < ne; ++iw) { cor[iw] = KCX_ZERO; a2[iw] = KCX_ZERO; }
    for (int n1 = 0; n1 < nb; ++n1) {
        const int flag_occ = n1 < nv;
        const double wx = freqevalmin - ekq[n1] + freqevalstep;
        double fact1 = 0.00, fact2 = 0.00;
        int ifreq = 0;
        orc_ff_compute_fact(wx, nfreq, dFreqGrid, &fact1, &fact2, &ifreq, 2, flag_occ);
        int kind = 0;
        if (wx > 0) { if (!flag_occ) kind = 1; }
        else if (flag_occ) kind = 2;
        cx val = {0, 0};
        if (kind) {
#pragma omp parallel for schedule(static)
            for (int my_igp = 0; my_igp < ng; ++my_igp) {
                const int igp = igpmap[my_igp];
                const cx cm = cx_conj(cx_ld(aqsm, (long)n1 * nc + igp));
                const long o0 = (long)ifreq * plane + (long)my_igp * nc;
                const long o1 = (long)(ifreq + 1) * plane + (long)my_igp * nc;
                cx s = {0, 0};
                for (int ig = 0; ig < nc; ++ig) {
                    cx d0 = cx_sub(cx_ld(I_epsR, o0 + ig), cx_ld(I_epsA, o0 + ig));
                    cx d1 = cx_sub(cx_ld(I_epsR, o1 + ig), cx_ld(I_epsA, o1 + ig));
                    cx sch2Dt = cx_add(cx_scale(d0, fact1), cx_scale(d1, fact2));
                    if (kind == 2) sch2Dt = cx_scale(sch2Dt, -0.5);
                    s = cx_add(s, cx_scale(cx_mul(cx_mul(cx_ld(aqsn, (long)n1 * nc + ig), cm), sch2Dt), vcoul[igp]));
                }
                part[my_igp] = s;
            }
            kcx t = KCX_ZERO;
            for (int my_igp = 0; my_igp < ng; ++my_igp) kc_add(&t, part[my_igp]);
            val = kc_val(&t);
        }
        for (int iw = 0; iw < ne; ++iw) {
            kc_add(&cor[iw], val);
            kc_add(&a2[iw], sch2Di[iw]);
        }
    }

    const int split = (flags & ORC_FF_SPLIT_ACHD) != 0;
    for (int iw = 0; iw < ne; ++iw) {
        cx x = kc_val(&asx[iw]);
        cx d = kc_val(&achd[iw]);
        if (!split) x = cx_add(x, d);  /* achDtemp_Kernel writes asxDtemp (:495) */
        asxDtemp_o[2 * iw] = x.re; asxDtemp_o[2 * iw + 1] = x.im;
        if (achDtemp_o) { achDtemp_o[2 * iw] = split ? d.re : 0.0; achDtemp_o[2 * iw + 1] = split ? d.im : 0.0; }
        cx c = kc_val(&cor[iw]);
        achDtemp_cor_o[2 * iw] = c.re; achDtemp_cor_o[2 * iw + 1] = c.im;
        if (ach2Dtemp_o) { cx v = kc_val(&a2[iw]); ach2Dtemp_o[2 * iw] = v.re; ach2Dtemp_o[2 * iw + 1] = v.im; }
    }
    free(asx); free(achd); free(sch2Di); free(schDi_cor); free(cor); free(a2);
    free(igpmap); free(part); free(schDt);
    return 0;
}
