// ref_harness_gpp.cpp -- drives the reference's own GPP solver functions on
// caller-supplied inputs (TEST INFRASTRUCTURE ONLY; built by oracle/Makefile
// into oracle/_ref/ when the reference sources are present).
//
// The reference drivers fill their arrays with constants inside main(), so
// their solver functions are the only way to run reference code on seeded
// random inputs.  This harness links, unmodified, the object code of
//   BGW-Kernels/gppKer.cpp  (flagOCC_solver, :130-159, which calls
//                            ssxt_scht_solver, :19-65)
//   gppKerSeq.cpp           (noflagOCC_solver, :193-261, gppsum = 0 branch,
//                            the function form of BGW-Kernels/gppKer.cpp:387-413)
// with their main() renamed by the build, and reports, per (n1, my_igp, iw),
// the sch_array / ssx_array values the reference main accumulates
// (BGW-Kernels/gppKer.cpp:337-413) before the vcoul weight.
//
// With a seventh argument 1 it runs gppKerSeq.cpp's gppsum == 1 mode instead:
// its own flagOCC_solver (:90-139) for occupied bands and its driver's block
// loop (:430-447) over noflagOCC_solver, igmax = igp.
//
// usage: ref_harness_gpp nb nv nc ng in.bin out.bin [gppsum]
//   in.bin : aqsm[nb*nc] aqsn[nb*nc] I_eps[ng*nc] wtilde[ng*nc] (complex128)
//            wx[3] (float64) igp[ng] (int32; the resolved column index)
//   out.bin: sch[nb][ng][3] ssx[nv][ng][3] (complex128)
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

typedef std::complex<double> cd;

void flagOCC_solver(double wxt, cd* wtilde_array_tmp, int my_igp, int n1, cd* aqsmtemp_arr, cd* aqsntemp_arr,
                    cd* I_eps_array_tmp, cd& ssxt, cd& scht, int igmax, int ncouls, int igp, int number_bands,
                    int ngpown);
void noflagOCC_solver(int igbeg, int igend, int igblk, double wxt, cd** wtilde_array, int my_igp, int n1,
                      cd** aqsmtemp, cd** aqsntemp, cd** I_eps_array, int gppsum, cd& ssxt, cd& scht, int igmax,
                      int ncouls, int igp);
void fk_ref_seq_flagOCC_solver(double wxt, cd** wtilde_array, int my_igp, int n1, cd** aqsmtemp, cd** aqsntemp,
                               cd** I_eps_array, int gppsum, cd& ssxt, cd& scht, int igmax, int ncouls, int igp);

int main(int argc, char** argv) {
    if (argc != 7 && argc != 8) {
        std::fprintf(stderr, "usage: %s nb nv nc ng in.bin out.bin [gppsum]\n", argv[0]);
        return 2;
    }
    const int gppsum = argc == 8 ? std::atoi(argv[7]) : 0;
    const int nb = std::atoi(argv[1]), nv = std::atoi(argv[2]), nc = std::atoi(argv[3]), ng = std::atoi(argv[4]);
    std::vector<cd> aqsm((size_t)nb * nc), aqsn((size_t)nb * nc), eps((size_t)ng * nc), wt((size_t)ng * nc);
    double wx[3];
    std::vector<int> igpv(ng);
    FILE* f = std::fopen(argv[5], "rb");
    if (!f) return 3;
    size_t ok = std::fread(aqsm.data(), sizeof(cd), aqsm.size(), f) + std::fread(aqsn.data(), sizeof(cd), aqsn.size(), f) +
                std::fread(eps.data(), sizeof(cd), eps.size(), f) + std::fread(wt.data(), sizeof(cd), wt.size(), f) +
                std::fread(wx, sizeof(double), 3, f) + std::fread(igpv.data(), sizeof(int), ng, f);
    std::fclose(f);
    if (ok != aqsm.size() * 2 + eps.size() * 2 + 3 + (size_t)ng) return 4;

    // gppKerSeq.cpp lays its arrays out transposed, as pointer tables
    // (aqsntemp[ig][n1], I_eps_array[ig][my_igp], wtilde_array[ig][my_igp]).
    std::vector<cd> aqsmT((size_t)nb * nc), aqsnT((size_t)nb * nc), epsT((size_t)ng * nc), wtT((size_t)ng * nc);
    for (int n = 0; n < nb; ++n)
        for (int g = 0; g < nc; ++g) {
            aqsmT[(size_t)g * nb + n] = aqsm[(size_t)n * nc + g];
            aqsnT[(size_t)g * nb + n] = aqsn[(size_t)n * nc + g];
        }
    for (int p = 0; p < ng; ++p)
        for (int g = 0; g < nc; ++g) {
            epsT[(size_t)g * ng + p] = eps[(size_t)p * nc + g];
            wtT[(size_t)g * ng + p] = wt[(size_t)p * nc + g];
        }
    std::vector<cd*> pm(nc), pn(nc), pe(nc), pw(nc);
    for (int g = 0; g < nc; ++g) {
        pm[g] = &aqsmT[(size_t)g * nb];
        pn[g] = &aqsnT[(size_t)g * nb];
        pe[g] = &epsT[(size_t)g * ng];
        pw[g] = &wtT[(size_t)g * ng];
    }

    std::vector<cd> sch((size_t)nb * ng * 3), ssx((size_t)(nv > 0 ? nv : 1) * ng * 3);
    for (int n1 = 0; n1 < nb; ++n1)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpv[my_igp];
            if (igp < 0) continue;
            cd sch_array[3], ssx_array[3];
            if (gppsum == 1) {
                const int igmax = igp;
                for (int iw = 0; iw < 3; ++iw) {
                    if (n1 < nv) {
                        cd scht(0, 0), ssxt(0, 0);
                        fk_ref_seq_flagOCC_solver(wx[iw], pw.data(), my_igp, n1, pm.data(), pn.data(), pe.data(), 1,
                                                  ssxt, scht, igmax, nc, igp);
                        ssx_array[iw] += ssxt;
                        sch_array[iw] += 0.5 * scht;
                    }
                }
                if (n1 >= nv)
                    for (int igbeg = 0; igbeg < igmax; igbeg += 512) {
                        const int igend = igbeg + 511 < igmax ? igbeg + 511 : igmax;
                        for (int iw = 0; iw < 3; ++iw) {
                            cd scht(0, 0), ssxt(0, 0);
                            noflagOCC_solver(igbeg, igend, 512, wx[iw], pw.data(), my_igp, n1, pm.data(), pn.data(),
                                             pe.data(), 1, ssxt, scht, igmax, nc, igp);
                            sch_array[iw] += 0.5 * scht;
                        }
                    }
            } else if (n1 < nv) {
                for (int iw = 0; iw < 3; ++iw) {
                    cd scht(0, 0), ssxt(0, 0);
                    flagOCC_solver(wx[iw], wt.data(), my_igp, n1, aqsm.data(), aqsn.data(), eps.data(), ssxt, scht,
                                   nc, nc, igp, nb, ng);
                    ssx_array[iw] += ssxt;
                    sch_array[iw] += 0.5 * scht;
                }
            } else {
                const int igblk = 512;
                for (int igbeg = 0; igbeg < nc; igbeg += igblk) {
                    const int igend = igbeg + igblk < nc ? igbeg + igblk : nc;
                    for (int iw = 0; iw < 3; ++iw) {
                        cd scht(0, 0), ssxt(0, 0);
                        noflagOCC_solver(igbeg, igend, igblk, wx[iw], pw.data(), my_igp, n1, pm.data(), pn.data(),
                                         pe.data(), 0, ssxt, scht, nc, nc, igp);
                        sch_array[iw] += 0.5 * scht;
                    }
                }
            }
            for (int iw = 0; iw < 3; ++iw) {
                sch[((size_t)n1 * ng + my_igp) * 3 + iw] = sch_array[iw];
                if (n1 < nv) ssx[((size_t)n1 * ng + my_igp) * 3 + iw] = ssx_array[iw];
            }
        }
    FILE* o = std::fopen(argv[6], "wb");
    if (!o) return 5;
    std::fwrite(sch.data(), sizeof(cd), sch.size(), o);
    if (nv > 0) std::fwrite(ssx.data(), sizeof(cd), (size_t)nv * ng * 3, o);
    std::fclose(o);
    return 0;
}
