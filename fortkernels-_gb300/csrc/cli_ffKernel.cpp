// cli_ffKernel.cpp -- drop-in replacement for the ffKernel driver.
//
// Same command line and result lines as FFKer_cori/ffKernel.cpp:302-543:
//   ffKernel number_bands nvband ncouls ngpown nFreq nfreqeval
//            [--precision=fp64|mixed] [--schdt] [--physics] [--device=N]
// Inputs are built as that main() builds them (:398-456); the kernels run on
// the GPU through fk_ff.  --schdt fills schDt_matrix from the band x G x G'
// contraction (ffkernel.deslippe.best.f90.back1:402-418) instead of zero.
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include "fk_abi.h"

int main(int argc, char** argv) {
    int pos[6], npos = 0, device = 0;
    fk_precision prec = FK_FP64;
    unsigned flags = 0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strncmp(argv[i], "--precision=", 12)) prec = !std::strcmp(argv[i] + 12, "mixed") ? FK_MIXED : FK_FP64;
        else if (!std::strcmp(argv[i], "--schdt")) flags |= FK_FF_SCHDT_GEMM;
        else if (!std::strcmp(argv[i], "--physics")) flags |= FK_FF_PHYSICS;
        else if (!std::strncmp(argv[i], "--device=", 9)) device = std::atoi(argv[i] + 9);
        else if (npos < 6) pos[npos++] = std::atoi(argv[i]);
    }
    if (npos != 6) {
        std::cout << "Incorrect Parameters!!! The correct form is " << std::endl;
        std::cout << "./a.out number_bands nvband ncouls ngpown nFreq nfreqeval " << std::endl;
        return 0;
    }
    const int number_bands = pos[0], nvband = pos[1], ncouls = pos[2], ngpown = pos[3], nFreq = pos[4],
              nfreqeval = pos[5];
    if (ngpown > ncouls) {
        std::cout << "Incorrect Parameters!!! ngpown cannot be greater than ncouls. The correct form is " << std::endl;
        std::cout << "./a.out number_bands nvband ncouls ngpown nFreq nfreqeval " << std::endl;
        return 0;
    }
    std::cout << "Device = CUDA device " << device << " (" << fk_version() << ")"
              << "\n number_bands = " << number_bands << "\n nvband = " << nvband << "\n ncouls = " << ncouls
              << "\n ngpown = " << ngpown << "\n nFreq = " << nFreq << "\n nfreqeval = " << nfreqeval << std::endl;

    const std::complex<double> expr(0.5, 0.5), expR(0.5, 0.5), expA(0.5, -0.5), exprP1(0.5, 0.1);
    const double pref_zb = 0.5 / 3.14, freqevalmin = 0.00, freqevalstep = 0.50, occ = 1.00;
    std::vector<int> inv(ngpown), indinv(ncouls);
    std::vector<double> vcoul(ncouls, 1.0), ekq(number_bands), grid(nFreq), pref(nFreq);
    std::vector<std::complex<double>> aqsn((size_t)number_bands * ncouls, expr), aqsm(aqsn),
        epsR((size_t)nFreq * ngpown * ncouls, expR), epsA((size_t)nFreq * ngpown * ncouls, expA),
        brd(nFreq, exprP1);
    for (int i = 0; i < ngpown; ++i) inv[i] = i;
    for (int i = 0; i < ncouls; ++i) indinv[i] = i;
    double dw = -10;
    for (int i = 0; i < number_bands; ++i) {
        ekq[i] = dw;
        dw += 1.00;
    }
    dw = 0.00;
    for (int i = 0; i < nFreq; ++i) {
        grid[i] = dw;
        dw += 2.00;
    }
    for (int i = 0; i < nFreq; ++i) pref[i] = i < nFreq - 1 ? (grid[i + 1] - grid[i]) / 3.14 : pref[i - 1];
    pref[0] *= 0.5;
    pref[nFreq - 1] *= 0.5;

    fk_ctx_t ctx = nullptr;
    fk_status st = fk_create(device, &ctx);
    if (st != FK_OK) {
        std::fprintf(stderr, "fk_create: %s\n", fk_strerror(st));
        return 1;
    }
    fk_c128 achsDtemp;
    std::vector<fk_c128> asxDtemp(nfreqeval), achDtemp_cor(nfreqeval);
    std::cout << "starting Kernels" << std::endl;
    auto t0 = std::chrono::high_resolution_clock::now();
    st = fk_ff(ctx, number_bands, nvband, ncouls, ngpown, nFreq, nfreqeval, (const fk_c128*)aqsm.data(),
               (const fk_c128*)aqsn.data(), (const fk_c128*)epsR.data(), (const fk_c128*)epsA.data(), vcoul.data(),
               inv.data(), indinv.data(), ekq.data(), grid.data(), (const fk_c128*)brd.data(), pref.data(), pref_zb,
               freqevalmin, freqevalstep, occ, prec, flags, &achsDtemp, asxDtemp.data(), nullptr,
               achDtemp_cor.data(), nullptr, nullptr);
    std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
    if (st != FK_OK) {
        std::fprintf(stderr, "fk_ff: %s: %s\n", fk_strerror(st), fk_last_error(ctx));
        fk_destroy(ctx);
        return 1;
    }
    std::cout << "achsDtemp = ";
    std::printf("( %f, %f) \n", achsDtemp.re, achsDtemp.im);
    std::cout << "asxDtemp = ";
    std::printf("( %f, %f) \n", asxDtemp[0].re, asxDtemp[0].im);
    std::cout << "achDtemp_cor = ";
    std::printf("( %f, %f) \n", achDtemp_cor[0].re, achDtemp_cor[0].im);
    std::cout << "********** Total Kernel Time **********= " << el.count() << " secs" << std::endl;
    fk_destroy(ctx);
    return 0;
}
