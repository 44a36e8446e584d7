// fk_static.cu -- fk_gpp_static: the FP64 GPP sum of fk_gpp with every
// intermediate held in one fixed device array compiled into the library, for
// callers that must not allocate device memory (their GPU memory is owned by
// another allocator, or they cannot take the device-wide synchronisation of
// cudaMalloc/cudaFree).  The kernels and their order are those of fk_gpp's
// FP64 path (gpp_run); only where the scratch comes from differs.
#include <cuda_runtime.h>

#include <mutex>

#include "fk_internal.h"

namespace {

// All intermediates of one call: branch-resolved factors, chunk and slice
// partial sums, per-band rows and the output block.  Module data of this
// translation unit: the CUDA runtime reserves it on a GPU when it loads the
// module there.  Under lazy module loading (the default since CUDA 12.2) that
// happens at the first call's symbol lookup; with CUDA_MODULE_LOADING=EAGER
// every context that loads the library reserves it at once, whether or not it
// ever calls fk_gpp_static.
__device__ __align__(256) unsigned char g_gpp_scratch[FK_GPP_STATIC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
// The scratch address and SM count of each device, found by the first call
// that succeeds there (base == nullptr: not set up yet).  A failed set-up is
// not kept: the next call on that device tries again.
struct DevScratch {
    void* base = nullptr;
    int sms = 0;
};
DevScratch g_scratch[MAX_DEVICES];
std::mutex g_setup_mu;

// Device (or managed) memory that a kernel may read where it lies: the
// kernels move rows with 16-byte and bulk copies, so it must start on a
// 16-byte boundary.
bool device_array(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && ((uintptr_t)p & 15) == 0;
}

bool host_array(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged;
}

}  // namespace

extern "C" fk_status fk_gpp_static(void* stream, int nb, int nv, int nc, int ng, const fk_c128* aqsmtemp,
                                   const fk_c128* aqsntemp, const fk_c128* I_eps_array,
                                   const fk_c128* wtilde_array, const double* vcoul, const int* inv_igp_index,
                                   const int* indinv, const double* wx_array, unsigned flags, fk_c128* achtemp,
                                   fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp) {
    // the argument rules of fk_gpp
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb) return FK_EINVAL;
    if (!aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !inv_igp_index || !indinv ||
        !wx_array || !achtemp || !asxtemp)
        return FK_EINVAL;
    if (flags & ~(FK_GPP_ROOT_QUIRKS | FK_GPP_ACHSTEMP)) return FK_EINVAL;
    if ((flags & FK_GPP_ROOT_QUIRKS) && ng > nc) return FK_EINVAL;
    if (ng > 65535) return FK_ENOTSUP;
    // inputs are read where they lie: staging them would need memory
    const void* ins[8] = {aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul, inv_igp_index, indinv, wx_array};
    for (const void* p : ins)
        if (!device_array(p)) return FK_EINVAL;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        cudaGetLastError();
        return FK_ECUDA;
    }
    // set-up, once per device (until it succeeds): the scratch array's address
    // and the SM count.  The address stays valid for the life of the primary
    // context; a cudaDeviceReset after the first call is not supported.
    DevScratch s;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        DevScratch& g = g_scratch[dev];
        if (!g.base) {
            void* base = nullptr;
            int sms = 0;
            cudaError_t e = cudaGetSymbolAddress(&base, g_gpp_scratch);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess || !base) {
                cudaGetLastError();
                return FK_ECUDA;
            }
            g.sms = sms;
            g.base = base;
        }
        s = g;
    }

    fk::Ctx c;
    c.device = dev;
    c.sms = s.sms;
    c.stream = (cudaStream_t)stream;
    c.use_graphs = false;
    c.ws.base = s.base;
    c.ws.cap = FK_GPP_STATIC_SCRATCH_BYTES;

    fk::GppDev r{};
    r.nb = nb; r.nv = nv; r.nc = nc; r.ng = ng;
    r.prec = FK_FP64; r.flags = flags;
    r.aqsm = (const double2*)aqsmtemp; r.aqsn = (const double2*)aqsntemp;
    r.eps = (const double2*)I_eps_array; r.wt = (const double2*)wtilde_array;
    r.ldm = nc; r.aqsm_compact = false;
    r.vcoul = vcoul; r.inv = inv_igp_index; r.indinv = indinv; r.wx = wx_array;
    const size_t outn = 7 + (size_t)nb;
    // the whole request must fit before anything is queued
    const size_t need = fk::gpp_workspace(c, r) + outn * sizeof(double2) + 4096;
    if (need > c.ws.cap) return FK_ENOMEM;
    c.ws.reset();
    r.out = (double2*)c.ws.take(outn * sizeof(double2));
    if (!r.out) return FK_ENOMEM;
    fk_status st = fk::gpp_run(c, r);
    if (st != FK_OK) return st;

    // outputs: device pointers get an enqueued copy, host pointers a copy and a wait
    bool host_out = false;
    struct Out {
        fk_c128* dst;
        size_t off, n;
    } outs[4] = {{achtemp, 0, 3}, {asxtemp, 3, 3}, {achstemp, 6, 1}, {acht_n1_loc, 7, (size_t)nb}};
    for (const Out& o : outs) {
        if (!o.dst) continue;
        host_out = host_out || host_array(o.dst);
        if (cudaMemcpyAsync(o.dst, r.out + o.off, o.n * sizeof(double2), cudaMemcpyDefault, c.stream) != cudaSuccess) {
            cudaGetLastError();
            return FK_ECUDA;
        }
    }
    if (host_out && cudaStreamSynchronize(c.stream) != cudaSuccess) {
        cudaGetLastError();
        return FK_ECUDA;
    }
    return FK_OK;
}
