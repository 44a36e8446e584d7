/*
 * fk_oracle.h -- CPU oracle for the GPP and FF self-energy hot paths.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, on the host, the loop
 * nests of the reference mini-apps so that the CUDA library can be checked
 * against them.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product path never does.
 *
 * Parity pin: the restatement is checked against golden vectors printed by
 * the unmodified reference drivers (BGW-Kernels/gppKer.cpp, gppKer.cpp,
 * FFKer_cori/ffKernel.cpp) and against per-(n1, igp, iw) values returned by
 * the reference's own solver functions (BGW-Kernels/gppKer.cpp:19-159,
 * gppKerSeq.cpp:193-261, FFKer_cori/ffKernel.cpp:30-300) called on seeded
 * random inputs (oracle/ref_harness.cpp, tests/golden/).
 *
 * Complex arrays are interleaved (re, im) doubles, row-major, exactly as the
 * reference lays them out:
 *   aqsmtemp/aqsntemp [number_bands][ncouls]
 *   I_eps/wtilde      [ngpown][ncouls]
 *   I_epsR/I_epsA     [nFreq][ngpown][ncouls]
 */
#ifndef FK_ORACLE_H
#define FK_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* GPP flags */
#define ORC_GPP_ROOT_QUIRKS 0x1u  /* gppKer.cpp (repo root): no noflag mask
                                     (gppKer.cpp:336), flagOCC sch uses
                                     I_eps[my_igp*ngpown+ig] (gppKer.cpp:139) */
#define ORC_GPP_ACHSTEMP    0x2u  /* compute the static-CH remainder achstemp
                                     as in gppkernel.deslippe.09.30.2014.f90:195-229 */
#define ORC_GPP_PHYSICS     0x8u  /* the Fortran source of the kernel
                                     (gppkernel.deslippe.09.30.2014.f90) where it
                                     differs from the C++: branch-A ssx with
                                     cden = wx**2 - wtilde**2 (:302-305), the sexcut
                                     test applied when wx < 0 (:319-320), and asxtemp
                                     subtracted (:393).  Parity unpinned: no Fortran
                                     compiler was available to run the source. */
#define ORC_GPP_HALF_SUM    0x4u  /* gppsum == 1 of gppKerSeq.cpp: the sum over ig
                                     runs below igp with the conjugate pair term
                                     (flagOCC_solver :90-139, noflagOCC_solver
                                     :206-242, driver blocking :430-447) */

/*
 * GPP self-energy sum, BGW-Kernels/gppKer.cpp:303-439.
 * wx[3] are the three evaluation frequencies (BGW-Kernels/gppKer.cpp:310-314).
 * indinv has indinv_len entries; an inv_igp_index entry equal to ncouls maps
 * to igp = ncouls-1 without reading indinv (BGW-Kernels/gppKer.cpp:322-325).
 * Outputs (complex): achtemp[3], asxtemp[3], acht_n1_loc[nb] (nullable),
 * achstemp[1] (nullable), sch_out[nb][ng][3] (nullable; per-(n1,my_igp)
 * sch_array before the vcoul weight), ssx_out[nv][ng][3] (nullable).
 * nthreads <= 0 uses the OpenMP default.  Returns 0, or -1 on bad sizes.
 */
int orc_gpp(int nb, int nv, int nc, int ng,
            const double* aqsm, const double* aqsn,
            const double* I_eps, const double* wtilde, const double* vcoul,
            const int* inv_igp_index, const int* indinv, int indinv_len,
            const double* wx, unsigned flags, int nthreads,
            double* achtemp, double* asxtemp, double* acht_n1_loc,
            double* achstemp, double* sch_out, double* ssx_out);

/* Real-valued GPP flags */
#define ORC_GPP_REAL_ZERO_MASKED 0x10u /* a masked noflag term contributes 0 (the
                                          commented-out else of gppKer_real.cpp:372-373)
                                          instead of the value left in scha[ig] */

/*
 * Real-valued GPP, gppKer_real.cpp:297-396: the loop nest of the GPP sum on
 * double arrays (aqsmtemp/aqsntemp [nb][ncouls], I_eps/wtilde [ngpown][ncouls]).
 * Occupied bands: flagOCC_solver (:124-153) over ssxt_scht_solver (:17-63).
 * Other bands: the reference program's 512-wide blocks (:341-383), where a masked term
 * leaves scha[ig] as it was (the value of the last unmasked term at that
 * block offset, for the same (n1, my_igp), or 0) and every block sum adds all
 * of scha[0 .. igend).  Outputs (real): achtemp[3], asxtemp[3],
 * acht_n1_loc[nb] (nullable), sch_out[nb][ng][3], ssx_out[nv][ng][3]
 * (nullable; per-(n1, my_igp) sch_array / ssx_array before the vcoul weight).
 */
int orc_gpp_real(int nb, int nv, int nc, int ng,
                 const double* aqsm, const double* aqsn,
                 const double* I_eps, const double* wtilde, const double* vcoul,
                 const int* inv_igp_index, const int* indinv, int indinv_len,
                 const double* wx, unsigned flags, int nthreads,
                 double* achtemp, double* asxtemp, double* acht_n1_loc,
                 double* sch_out, double* ssx_out);

/* FF flags */
#define ORC_FF_SCHDT_GEMM  0x1u  /* schDt_matrix from the band x G x G' contraction
                                    (ffkernel.deslippe.best.f90.back1:402-418);
                                    otherwise zero as in FFKer_cori/ffKernel.cpp:421-422 */
#define ORC_FF_PHYSICS     0x2u  /* calculate_schDt_lin3 takes freqevalmin and
                                    freqevalstep as doubles; the reference C++
                                    truncates them to int (ffKernel.cpp:10) */
#define ORC_FF_SPLIT_ACHD  0x4u  /* achDtemp_Kernel writes its own output; the
                                    reference main passes asxDtemp (ffKernel.cpp:495) */

/*
 * FF full-frequency kernels, FFKer_cori/ffKernel.cpp:10-300 in the order main
 * calls them (:480-503).  Outputs (complex): achsDtemp[1], asxDtemp[ne],
 * achDtemp[ne], achDtemp_cor[ne], ach2Dtemp[ne], schDt_matrix[nb][nfreq]
 * (all nullable except achsDtemp/asxDtemp/achDtemp_cor).
 */
int orc_ff(int nb, int nv, int nc, int ng, int nfreq, int ne,
           const double* aqsm, const double* aqsn,
           const double* I_epsR, const double* I_epsA, const double* vcoul,
           const int* inv_igp_index, const int* indinv,
           const double* ekq, const double* dFreqGrid, const double* dFreqBrd,
           const double* pref, double pref_zb,
           double freqevalmin, double freqevalstep, double occ,
           unsigned flags, int nthreads,
           double* achsDtemp, double* asxDtemp, double* achDtemp,
           double* achDtemp_cor, double* ach2Dtemp, double* schDt_matrix);

/* compute_fact, FFKer_cori/ffKernel.cpp:30-78 (exposed for unit tests). */
void orc_ff_compute_fact(double wx, int nfreq, const double* dFreqGrid,
                         double* fact1, double* fact2, int* ifreq,
                         int loop, int flag_occ);

#ifdef __cplusplus
}
#endif
#endif
