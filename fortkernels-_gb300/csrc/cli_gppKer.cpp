// cli_gppKer.cpp -- drop-in replacement for the gppKer driver.
//
// Same command line and output lines as BGW-Kernels/gppKer.cpp:161-449:
//   gppKer <number_bands> <number_valence_bands> <number_plane_waves> <nodes_per_mpi_group>
//          [--precision=fp64|mixed] [--quirks] [--achstemp] [--device=N]
// and, with a fifth number, those of gppKerSeq.cpp:263-500:
//   gppKer <number_bands> <number_valence_bands> <number_plane_waves> <nodes_per_mpi_group> <gppsum>
// where gppsum = 1 is its half sum (FK_GPP_HALF_SUM).  gppsum = 0 of that
// driver drops ig = 511 mod 512 from every block (its igend is one short,
// gppKerSeq.cpp:459) and is refused rather than reproduced.
// The arrays are built exactly as that main() builds them (constant 0.5+0.5i
// fills, inv_igp_index[i] = (i+1)*ncouls/ngpown, indinv = identity, wx =
// e_lk - e_n1kq + dw*(iw-1)); the sum itself runs on the GPU through fk_gpp.
// --quirks selects the repo-root gppKer.cpp semantics (FK_GPP_ROOT_QUIRKS).
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <vector>

#include "fk_abi.h"

int main(int argc, char** argv) {
    int pos[5], npos = 0;
    fk_precision prec = FK_FP64;
    unsigned flags = 0;
    int device = 0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strncmp(argv[i], "--precision=", 12)) prec = !std::strcmp(argv[i] + 12, "mixed") ? FK_MIXED : FK_FP64;
        else if (!std::strcmp(argv[i], "--quirks")) flags |= FK_GPP_ROOT_QUIRKS;
        else if (!std::strcmp(argv[i], "--achstemp")) flags |= FK_GPP_ACHSTEMP;
        else if (!std::strncmp(argv[i], "--device=", 9)) device = std::atoi(argv[i] + 9);
        else if (npos < 5) pos[npos++] = std::atoi(argv[i]);
    }
    const bool seq = npos == 5;
    if (seq && pos[4] != 1) {
        std::fprintf(stderr, "gppsum = %d: only gppsum = 1 (the half sum) is provided; the full sum is the "
                             "four-argument form\n", pos[4]);
        return 1;
    }
    if (seq) flags |= FK_GPP_HALF_SUM;
    if (npos != 4 && !seq) {
        std::cout << "The correct form of input is : " << std::endl;
        std::cout << " ./a.out <number_bands> <number_valence_bands> <number_plane_waves> <nodes_per_mpi_group> "
                  << std::endl;
        return 0;
    }
    const int number_bands = pos[0], nvband = pos[1], ncouls = pos[2], nodes_per_group = pos[3];
    const int npes = 1;
    const int ngpown = ncouls / (nodes_per_group * npes);
    const double e_lk = 10, dw = 1, to1 = 1e-6, gamma = 0.5, sexcut = 4.0;
    const double limitone = 1.0 / (to1 * 4.0), limittwo = std::pow(0.5, 2), e_n1kq = 6.0;
    const int nstart = 0, nend = 3;

    fk_ctx_t ctx = nullptr;
    fk_status st = fk_create(device, &ctx);
    if (st != FK_OK) {
        std::fprintf(stderr, "fk_create: %s\n", fk_strerror(st));
        return 1;
    }
    std::cout << "Device = CUDA device " << device << " (" << fk_version() << ")" << std::endl;
    std::cout << "number_bands = " << number_bands << "\t nvband = " << nvband << "\t ncouls = " << ncouls
              << "\t nodes_per_group  = " << nodes_per_group;
    if (seq) std::cout << "\t gppsum = " << pos[4];
    std::cout << "\t ngpown = " << ngpown << "\t nend = " << nend
              << "\t nstart = " << nstart << "\t gamma = " << gamma << "\t sexcut = " << sexcut
              << "\t limitone = " << limitone << "\t limittwo = " << limittwo << std::endl;

    const std::complex<double> expr(0.5, 0.5);
    std::vector<std::complex<double>> aqsm((size_t)number_bands * ncouls, expr), aqsn(aqsm),
        eps((size_t)ngpown * ncouls, expr), wt(eps);
    std::vector<double> vcoul(ncouls, 1.0);
    std::vector<int> inv(ngpown), indinv(ncouls);
    for (int ig = 0; ig < ngpown; ++ig) inv[ig] = (ig + 1) * ncouls / ngpown;
    for (int ig = 0; ig < ncouls; ++ig) indinv[ig] = ig;
    double wx[3];
    for (int iw = nstart; iw < nend; ++iw) {
        wx[iw] = e_lk - e_n1kq + dw * ((iw + 1) - 2);
        if (std::abs(wx[iw]) < to1) wx[iw] = to1;
    }
    std::cout << "Size of wtilde_array = " << (ncouls * ngpown * 2.0 * 8) / std::pow(1024, 2) << " Mbytes" << std::endl;
    std::cout << "Size of aqsntemp = " << (ncouls * number_bands * 2.0 * 8) / std::pow(1024, 2) << " Mbytes"
              << std::endl;
    std::cout << "Size of I_eps_array array = " << (ncouls * ngpown * 2.0 * 8) / std::pow(1024, 2) << " Mbytes"
              << std::endl;

    fk_c128 achtemp[3], asxtemp[3], achstemp;
    std::vector<fk_c128> n1loc(number_bands);
    auto t0 = std::chrono::high_resolution_clock::now();
    st = fk_gpp(ctx, number_bands, nvband, ncouls, ngpown, (const fk_c128*)aqsm.data(), (const fk_c128*)aqsn.data(),
                (const fk_c128*)eps.data(), (const fk_c128*)wt.data(), vcoul.data(), inv.data(), indinv.data(), wx,
                prec, flags, achtemp, asxtemp, n1loc.data(), (flags & FK_GPP_ACHSTEMP) ? &achstemp : nullptr);
    std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
    if (st != FK_OK) {
        std::fprintf(stderr, "fk_gpp: %s: %s\n", fk_strerror(st), fk_last_error(ctx));
        fk_destroy(ctx);
        return 1;
    }
    if (flags & FK_GPP_ACHSTEMP) std::cout << "achstemp = " << std::complex<double>(achstemp.re, achstemp.im) << std::endl;
    for (int iw = nstart; iw < nend; ++iw)
        std::cout << "achtemp[" << iw << "] = " << std::setprecision(15)
                  << std::complex<double>(achtemp[iw].re, achtemp[iw].im) << std::endl;
    std::cout << "********** Chrono Time Taken **********= " << el.count() << " secs" << std::endl;
    fk_destroy(ctx);
    return 0;
}
