// ref_harness_gpp_real.cpp -- drives the reference's own real-valued
// flagOCC_solver (gppKer_real.cpp:124-153, which calls ssxt_scht_solver
// :17-63) on caller-supplied inputs (TEST INFRASTRUCTURE ONLY; built by
// oracle/Makefile into oracle/_ref/ when the reference sources are present).
//
// gppKer_real.cpp fills its arrays with constants inside main(), and its
// noflag block loop (:341-383) is part of main(), so the occupied-band solver
// is the one piece of its code that runs on seeded inputs.  The object code
// is linked unmodified with main() renamed by the build.  Reported per
// (n1 < nv, my_igp, iw): the sch_array / ssx_array values main() accumulates
// (:325-334) before the vcoul weight.
//
// usage: ref_harness_gpp_real nb nv nc ng in.bin out.bin
//   in.bin : aqsm[nb*nc] aqsn[nb*nc] I_eps[ng*nc] wtilde[ng*nc] (float64)
//            wx[3] (float64) igp[ng] (int32; the resolved column index)
//   out.bin: sch[nv][ng][3] ssx[nv][ng][3] (float64)
#include <cstdio>
#include <cstdlib>
#include <vector>

void flagOCC_solver(double wxt, double* wtilde_array_tmp, int my_igp, int n1, double* aqsmtemp_arr,
                    double* aqsntemp_arr, double* I_eps_array_tmp, double& ssxt, double& scht, int ncouls, int igp,
                    int number_bands, int ngpown);

int main(int argc, char** argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s nb nv nc ng in.bin out.bin\n", argv[0]);
        return 2;
    }
    const int nb = std::atoi(argv[1]), nv = std::atoi(argv[2]), nc = std::atoi(argv[3]), ng = std::atoi(argv[4]);
    std::vector<double> aqsm((size_t)nb * nc), aqsn((size_t)nb * nc), eps((size_t)ng * nc), wt((size_t)ng * nc);
    double wx[3];
    std::vector<int> igpv(ng);
    FILE* f = std::fopen(argv[5], "rb");
    if (!f) return 3;
    size_t ok = std::fread(aqsm.data(), sizeof(double), aqsm.size(), f) +
                std::fread(aqsn.data(), sizeof(double), aqsn.size(), f) +
                std::fread(eps.data(), sizeof(double), eps.size(), f) +
                std::fread(wt.data(), sizeof(double), wt.size(), f) + std::fread(wx, sizeof(double), 3, f) +
                std::fread(igpv.data(), sizeof(int), ng, f);
    std::fclose(f);
    if (ok != aqsm.size() * 2 + eps.size() * 2 + 3 + (size_t)ng) return 4;

    std::vector<double> sch((size_t)nv * ng * 3, 0.0), ssx((size_t)nv * ng * 3, 0.0);
    for (int n1 = 0; n1 < nv; ++n1)
        for (int my_igp = 0; my_igp < ng; ++my_igp) {
            const int igp = igpv[my_igp];
            if (igp < 0) continue;
            for (int iw = 0; iw < 3; ++iw) {
                double ssxt = 0.0, scht = 0.0;
                flagOCC_solver(wx[iw], wt.data(), my_igp, n1, aqsm.data(), aqsn.data(), eps.data(), ssxt, scht, nc,
                               igp, nb, ng);
                ssx[((size_t)n1 * ng + my_igp) * 3 + iw] += ssxt;
                sch[((size_t)n1 * ng + my_igp) * 3 + iw] += 0.5 * scht;
            }
        }
    FILE* o = std::fopen(argv[6], "wb");
    if (!o) return 5;
    std::fwrite(sch.data(), sizeof(double), sch.size(), o);
    std::fwrite(ssx.data(), sizeof(double), ssx.size(), o);
    std::fclose(o);
    return 0;
}
