// ref_harness_ff.cpp -- drives the reference's own FF kernels on
// caller-supplied inputs (TEST INFRASTRUCTURE ONLY; built by oracle/Makefile
// into oracle/_ref/ when the reference sources are present).
//
// Links, unmodified, the object code of FFKer_cori/ffKernel.cpp (its main()
// renamed by the build) and calls its kernels in the order its main does
// (FFKer_cori/ffKernel.cpp:480-503), including main's wiring of asxDtemp as
// achDtemp_Kernel's output (:495).  Run it with OMP_NUM_THREADS=1: the
// reference's achDtemp_Kernel shares scratch arrays across its collapse(2)
// threads.
//
// usage: ref_harness_ff nb nv nc ng nfreq ne in.bin out.bin
//   in.bin : aqsm[nb*nc] aqsn[nb*nc] I_epsR[nfreq*ng*nc] I_epsA[nfreq*ng*nc]
//            dFreqBrd[nfreq] schDt[nb*nfreq] (complex128)
//            vcoul[nc] ekq[nb] dFreqGrid[nfreq] pref[nfreq]
//            pref_zb freqevalmin freqevalstep occ (float64)
//            inv_igp_index[ng] indinv[nc] (int32)
//   out.bin: achsDtemp asxDtemp[ne] achDtemp_cor[ne] ach2Dtemp[ne] (complex128)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Complex.h"

void achsDtemp_Kernel(int number_bands, int ngpown, int ncouls, int* inv_igp_index, int* indinv, GPUComplex* aqsntemp,
                      GPUComplex* aqsmtemp, GPUComplex* I_epsR_array, double* vcoul, GPUComplex& achsDtemp);
void asxDtemp_Kernel(int nvband, int nfreqeval, int ncouls, int ngpown, int numThreads, int nFreq, double freqevalmin,
                     double freqevalstep, double occ, double* ekq, double* dFreqGrid, int* inv_igp_index, int* indinv,
                     GPUComplex* aqsmtemp, GPUComplex* aqsntemp, double* vcoul, GPUComplex* I_epsR_array,
                     GPUComplex* ssxDittt, GPUComplex* asxDtemp);
void achDtemp_Kernel(int number_bands, int nvband, int nfreqeval, int ncouls, int ngpown, int nFreq,
                     double freqevalmin, double freqevalstep, double* ekq, double pref_zb, double* pref,
                     double* dFreqGrid, GPUComplex* dFreqBrd, GPUComplex* schDt_matrix, GPUComplex* schDi,
                     GPUComplex* schDi_cor, GPUComplex* sch2Di, GPUComplex* achDtemp);
void achDtemp_cor_Kernel(int number_bands, int nvband, int nfreqeval, int ncouls, int ngpown, int nFreq,
                         double freqevalmin, double freqevalstep, double* ekq, double* dFreqGrid, int* inv_igp_index,
                         int* indinv, GPUComplex* aqsmtemp, GPUComplex* aqsntemp, double* vcoul,
                         GPUComplex* I_epsR_array, GPUComplex* I_epsA_array, GPUComplex* schDi_cor,
                         GPUComplex* schDi_corb, GPUComplex* sch2Di, GPUComplex* ach2Dtemp, GPUComplex* achDtemp_cor,
                         GPUComplex* achDtemp_corb);

template <class T>
static bool rd(FILE* f, std::vector<T>& v) { return std::fread(v.data(), sizeof(T), v.size(), f) == v.size(); }

int main(int argc, char** argv) {
    if (argc != 9) { std::fprintf(stderr, "usage: %s nb nv nc ng nfreq ne in.bin out.bin\n", argv[0]); return 2; }
    const int nb = std::atoi(argv[1]), nv = std::atoi(argv[2]), nc = std::atoi(argv[3]), ng = std::atoi(argv[4]);
    const int nfreq = std::atoi(argv[5]), ne = std::atoi(argv[6]);
    const size_t plane = (size_t)nfreq * ng * nc;
    std::vector<GPUComplex> aqsm((size_t)nb * nc), aqsn((size_t)nb * nc), epsR(plane), epsA(plane), brd(nfreq),
        schDt((size_t)nb * nfreq);
    std::vector<double> vcoul(nc), ekq(nb), grid(nfreq), pref(nfreq), sc(4);
    std::vector<int> inv(ng), indinv(nc);
    FILE* f = std::fopen(argv[7], "rb");
    if (!f) return 3;
    bool ok = rd(f, aqsm) && rd(f, aqsn) && rd(f, epsR) && rd(f, epsA) && rd(f, brd) && rd(f, schDt) && rd(f, vcoul) &&
              rd(f, ekq) && rd(f, grid) && rd(f, pref) && rd(f, sc) && rd(f, inv) && rd(f, indinv);
    std::fclose(f);
    if (!ok) return 4;
    const double pref_zb = sc[0], fmin = sc[1], fstep = sc[2], occ = sc[3];

    std::vector<GPUComplex> schDi(ne), schDi_cor(ne), schDi_corb(ne), sch2Di(ne), asxDtemp(ne), ach2Dtemp(ne),
        achDtemp_cor(ne), achDtemp_corb(ne), ssxDittt(1);
    GPUComplex achsDtemp;
    achsDtemp_Kernel(nb, ng, nc, inv.data(), indinv.data(), aqsn.data(), aqsm.data(), epsR.data(), vcoul.data(),
                     achsDtemp);
    asxDtemp_Kernel(nv, ne, nc, ng, 1, nfreq, fmin, fstep, occ, ekq.data(), grid.data(), inv.data(), indinv.data(),
                    aqsm.data(), aqsn.data(), vcoul.data(), epsR.data(), ssxDittt.data(), asxDtemp.data());
    achDtemp_Kernel(nb, nv, ne, nc, ng, nfreq, fmin, fstep, ekq.data(), pref_zb, pref.data(), grid.data(), brd.data(),
                    schDt.data(), schDi.data(), schDi_cor.data(), sch2Di.data(), asxDtemp.data());
    achDtemp_cor_Kernel(nb, nv, ne, nc, ng, nfreq, fmin, fstep, ekq.data(), grid.data(), inv.data(), indinv.data(),
                        aqsm.data(), aqsn.data(), vcoul.data(), epsR.data(), epsA.data(), schDi_cor.data(),
                        schDi_corb.data(), sch2Di.data(), ach2Dtemp.data(), achDtemp_cor.data(), achDtemp_corb.data());
    FILE* o = std::fopen(argv[8], "wb");
    if (!o) return 5;
    std::fwrite(&achsDtemp, sizeof(GPUComplex), 1, o);
    std::fwrite(asxDtemp.data(), sizeof(GPUComplex), ne, o);
    std::fwrite(achDtemp_cor.data(), sizeof(GPUComplex), ne, o);
    std::fwrite(ach2Dtemp.data(), sizeof(GPUComplex), ne, o);
    std::fclose(o);
    return 0;
}
