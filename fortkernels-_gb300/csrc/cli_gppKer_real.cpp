// cli_gppKer_real.cpp -- drop-in replacement for the real-valued gppKer driver.
//
// Same command line and output lines as gppKer_real.cpp:155-418:
//   gppKer_real <number_bands> <number_valence_bands> <number_plane_waves> <nodes_per_mpi_group>
//               [--precision=fp64|mixed] [--zero-masked] [--device=N]
// The arrays are built as that main() builds them (every array 0.5, vcoul = 1,
// inv_igp_index[i] = (i+1)*ncouls/ngpown, indinv = identity, wx = e_lk -
// e_n1kq + dw*(iw-1)); the sum runs on the GPU through fk_gpp_real.
// --zero-masked counts a masked noflag term as 0 (FK_GPP_REAL_ZERO_MASKED).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <vector>

#include "fk_abi.h"

int main(int argc, char** argv) {
    int pos[4], npos = 0;
    fk_precision prec = FK_FP64;
    unsigned flags = 0;
    int device = 0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strncmp(argv[i], "--precision=", 12)) prec = !std::strcmp(argv[i] + 12, "mixed") ? FK_MIXED : FK_FP64;
        else if (!std::strcmp(argv[i], "--zero-masked")) flags |= FK_GPP_REAL_ZERO_MASKED;
        else if (!std::strncmp(argv[i], "--device=", 9)) device = std::atoi(argv[i] + 9);
        else if (npos < 4) pos[npos++] = std::atoi(argv[i]);
    }
    if (npos != 4) {
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
              << "\t nodes_per_group  = " << nodes_per_group << "\t ngpown = " << ngpown << "\t nend = " << nend
              << "\t nstart = " << nstart << "\t gamma = " << gamma << "\t sexcut = " << sexcut
              << "\t limitone = " << limitone << "\t limittwo = " << limittwo << std::endl;
    std::cout << "Size of wtilde_array = " << (ncouls * ngpown * 2.0 * 8) / std::pow(1024, 2) << " Mbytes" << std::endl;
    std::cout << "Size of aqsntemp = " << (ncouls * number_bands * 2.0 * 8) / std::pow(1024, 2) << " Mbytes"
              << std::endl;
    std::cout << "Size of I_eps_array array = " << (ncouls * ngpown * 2.0 * 8) / std::pow(1024, 2) << " Mbytes"
              << std::endl;

    std::vector<double> aqsm((size_t)number_bands * ncouls, 0.5), aqsn(aqsm), eps((size_t)ngpown * ncouls, 0.5),
        wt(eps), vcoul(ncouls, 1.0);
    std::vector<int> inv(ngpown), indinv(ncouls);
    for (int ig = 0; ig < ngpown; ++ig) inv[ig] = (ig + 1) * ncouls / ngpown;
    for (int ig = 0; ig < ncouls; ++ig) indinv[ig] = ig;
    double wx[3];
    for (int iw = nstart; iw < nend; ++iw) {
        wx[iw] = e_lk - e_n1kq + dw * ((iw + 1) - 2);
        if (std::abs(wx[iw]) < to1) wx[iw] = to1;
    }
    double achtemp[3], asxtemp[3];
    std::vector<double> n1loc(number_bands);
    auto t0 = std::chrono::high_resolution_clock::now();
    st = fk_gpp_real(ctx, number_bands, nvband, ncouls, ngpown, aqsm.data(), aqsn.data(), eps.data(), wt.data(),
                     vcoul.data(), inv.data(), indinv.data(), wx, prec, flags, achtemp, asxtemp, n1loc.data());
    std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
    if (st != FK_OK) {
        std::fprintf(stderr, "fk_gpp_real: %s: %s\n", fk_strerror(st), fk_last_error(ctx));
        fk_destroy(ctx);
        return 1;
    }
    for (int iw = nstart; iw < nend; ++iw)
        std::cout << "achtemp[" << iw << "] = " << std::setprecision(15) << achtemp[iw] << std::endl;
    std::cout << "********** Chrono Time Taken **********= " << el.count() << " secs" << std::endl;
    fk_destroy(ctx);
    return 0;
}
