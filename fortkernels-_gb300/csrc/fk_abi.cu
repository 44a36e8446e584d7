// fk_abi.cu -- implementation of the C ABI declared in include/fk_abi.h:
// contexts, argument checks, host/device residency of the caller's arrays,
// input staging, workspace management and output delivery.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fk_internal.h"
#include "fk_tc.cuh"

namespace fk {

fk_status fail(Ctx& c, fk_status s, const std::string& msg) {
    c.err = msg;
    return s;
}

fk_status cuda_fail(Ctx& c, cudaError_t e, const char* where) {
    c.err = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? FK_ENOMEM : FK_ECUDA;
}

void phase_mark(Ctx& c, int i) {
    if (i == 0) c.nk = 0;
    if (c.profiling && i >= 0 && i < 5) cudaEventRecord(c.ev[i], c.stream);
}

void kernel_begin(Ctx& c) {
    if (c.profiling && c.nk < Ctx::KEV && c.kev[2 * c.nk]) cudaEventRecord(c.kev[2 * c.nk], c.stream);
}

void kernel_end(Ctx& c) {
    if (c.profiling && c.nk < Ctx::KEV && c.kev[2 * c.nk + 1]) cudaEventRecord(c.kev[2 * c.nk + 1], c.stream);
    ++c.nk;
}

void phase_close(Ctx& c, int nphases) {
    if (!c.profiling) return;
    if (cudaEventSynchronize(c.ev[nphases]) != cudaSuccess) return;
    for (int i = 0; i < nphases && i < 4; ++i) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c.ev[i], c.ev[i + 1]) == cudaSuccess) c.timings[i] = ms;
    }
    c.kernel_ms = 0.f;
    c.kernel_launches = 0;
    for (int k = 0; k < c.nk && k < Ctx::KEV; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c.kev[2 * k], c.kev[2 * k + 1]) == cudaSuccess) {
            c.kernel_ms += ms;
            ++c.kernel_launches;
        }
    }
}

namespace {

// Restores the caller's current device when a call returns.
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the sticky-free error of a failed query
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
    return st != cudaStreamCaptureStatusNone;
}

void drop_graphs(Ctx& c) {
    for (auto& kv : c.graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    c.graphs.clear();
}

// FNV-1a over a word sequence (graph cache key).
uint64_t fnv(const uint64_t* w, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i)
        for (int b = 0; b < 8; ++b) {
            h ^= (w[i] >> (8 * b)) & 0xFF;
            h *= 1099511628211ull;
        }
    return h;
}

fk_status ensure_workspace(Ctx& c, size_t need) {
    if (c.ws.cap >= need) return FK_OK;
    drop_graphs(c);  // captured graphs refer to the old workspace
    if (capturing(c.stream))
        return fail(c, FK_ENOMEM, "workspace must grow, which is not allowed during stream capture: call fk_reserve first");
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "workspace: synchronize");
    if (c.ws.base) cudaFree(c.ws.base);
    c.ws.base = nullptr;
    c.ws.cap = 0;
    size_t cap = need + need / 4 + (1u << 20);
    e = cudaMalloc(&c.ws.base, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(c, e, "workspace: cudaMalloc");
    }
    c.ws.cap = cap;
    return FK_OK;
}

// An input array: used in place when it is device memory, staged otherwise.
struct In {
    const void* user;
    size_t bytes;
    bool dev;
    const void* d;
};

// A device array is used where it lies when it starts on a 16-byte boundary
// (the kernels move it with 16-byte and bulk copies); host arrays and
// misaligned device arrays are copied into the workspace.
bool in_place(const In* i) { return !i->user || (i->dev && ((uintptr_t)i->user & 15) == 0); }

size_t staged_bytes(const std::vector<In*>& v) {
    size_t s = 0;
    for (auto* i : v)
        if (!in_place(i)) s += (i->bytes + 255) & ~size_t(255);
    return s;
}

fk_status stage(Ctx& c, const std::vector<In*>& v) {
    for (auto* i : v) {
        if (in_place(i)) {
            i->d = i->user;
            continue;
        }
        void* d = c.ws.take(i->bytes);
        if (!d) return fail(c, FK_ENOMEM, "workspace: staging");
        cudaError_t e = cudaMemcpyAsync(d, i->user, i->bytes, i->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                        c.stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "staging copy");
        if (!i->dev) c.h2d_bytes += i->bytes;
        i->d = d;
    }
    return FK_OK;
}

// Copies out[off..off+n) to a caller pointer (host or device).
fk_status deliver(Ctx& c, void* dst, const double2* out, size_t off, size_t n, bool& host_out) {
    if (!dst || n == 0) return FK_OK;
    if (!is_device_ptr(dst)) {
        host_out = true;
        c.d2h_bytes += n * sizeof(double2);
    }
    cudaError_t e = cudaMemcpyAsync(dst, out + off, n * sizeof(double2), cudaMemcpyDefault, c.stream);
    return e == cudaSuccess ? FK_OK : cuda_fail(c, e, "output copy");
}

// Pinned host buffer of at least `bytes`, safe to overwrite (its previous
// contents have been copied out).
void* pinned_buffer(Ctx& c, size_t bytes) {
    if (c.pinned_ev) cudaEventSynchronize(c.pinned_ev);
    if (c.pinned_cap < bytes) {
        if (c.pinned) cudaFreeHost(c.pinned);
        c.pinned = nullptr;
        c.pinned_cap = 0;
        size_t cap = bytes + bytes / 4 + 4096;
        if (cudaHostAlloc(&c.pinned, cap, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        c.pinned_cap = cap;
    }
    return c.pinned;
}

// After a synchronize: a nonzero error word means a bounded device-side wait
// of the tensor-core kernels gave up (fk_wait_error_status decodes it).
fk_status check_errword(Ctx& c) {
    int w = 0;
    cudaError_t e = cudaMemcpy(&w, c.errword, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "reading the device error word");
    if (w != 0) {
        cudaMemset(c.errword, 0, sizeof(int));
        char buf[512];
        const fk_status s = fk_wait_error_status(w, buf, sizeof buf);
        return fail(c, s, buf);
    }
    return FK_OK;
}

// One thread initialises an mbarrier that expects one arrival, which never
// comes, and waits on it with the bounded wait of the tensor-core kernels; the
// wait gives up after `limit` cycles and the thread records code 0x100 in the
// error word, as a timed-out wait of those kernels does.  No copy or MMA is
// in flight, so giving up is always safe.
__global__ void selftest_wait_kernel(int* err, long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    tc::mbar_init(&bar, 1);
    tc::fence_barrier_init();
    if (!tc::mbar_wait(&bar, 0, limit)) atomicOr(err, 0x100);
}

}  // namespace
}  // namespace fk

using fk::Ctx;

extern "C" {

const char* fk_version(void) { return "fk_gb300 1.0 sm_103a"; }

const char* fk_strerror(fk_status s) {
    switch (s) {
        case FK_OK: return "ok";
        case FK_EINVAL: return "invalid argument";
        case FK_ENOMEM: return "out of memory";
        case FK_ECUDA: return "CUDA error";
        case FK_ETIMEOUT: return "device wait timed out";
        case FK_EBUSY: return "busy: request not admitted";
        case FK_ENOTSUP: return "not supported";
        case FK_ECANCELED: return "cancelled";
    }
    return "unknown status";
}

const char* fk_last_error(fk_ctx_t ctx) { return ctx ? ctx->err.c_str() : "null context"; }

fk_status fk_wait_error_status(int word, char* msg, size_t msg_len) {
    // the bits the kernels set (fk_tc_contract.cuh, selftest_wait_kernel)
    static const struct {
        int bit;
        const char* what;
    } roles[] = {{0x1, "MMA issuer waiting for a free accumulator buffer"},
                 {0x2, "MMA issuer waiting for an operand stage"},
                 {0x4, "MMA issuer waiting for its last MMAs"},
                 {0x8, "copy warp waiting for a free operand stage"},
                 {0x10, "epilogue waiting for an accumulator"},
                 {0x20, "converter warps waiting for operand rows"},
                 {0x40, "copy warp waiting for a free staging half"},
                 {0x80, "copy warp waiting for its last copies"},
                 {0x100, "self-test wait"},
                 {0x200, "plane conversion waiting for its row copy"},
                 {0x400, "-B_im warp waiting for an operand stage"}};
    std::string m;
    if (word == 0) {
        m = "no device-side wait gave up";
    } else {
        char head[64];
        std::snprintf(head, sizeof head, "a device-side wait timed out (code 0x%x):", (unsigned)word);
        m = head;
        int known = 0;
        for (const auto& r : roles)
            if (word & r.bit) {
                m += std::string(known++ ? "; " : " ") + r.what;
            }
        if (word & ~0x7FF) m += std::string(known ? "; " : " ") + "unknown bits";
    }
    if (msg && msg_len) {
        std::strncpy(msg, m.c_str(), msg_len - 1);
        msg[msg_len - 1] = '\0';
    }
    return word == 0 ? FK_OK : FK_ETIMEOUT;
}

fk_status fk_create(int device, fk_ctx_t* out) {
    if (!out) return FK_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return FK_ECUDA;
    }
    fk_ctx* c = new (std::nothrow) fk_ctx();
    if (!c) return FK_ENOMEM;
    c->device = device;
    fk::DeviceGuard g(device);
    if (!g.ok || cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return FK_ECUDA;
    }
    c->stream = c->own_stream;
    // from here on a failure releases everything created so far (fk_destroy
    // skips the members that are still null)
    auto undo = [c]() {
        cudaGetLastError();
        fk_destroy(c);
        cudaGetLastError();
        return FK_ECUDA;
    };
    if (cudaMalloc(&c->errword, 256) != cudaSuccess || cudaMemset(c->errword, 0, 256) != cudaSuccess) return undo();
    if (cudaEventCreateWithFlags(&c->pinned_ev, cudaEventDisableTiming) != cudaSuccess) return undo();
    for (auto& e : c->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return undo();
    for (auto& e : c->kev)
        if (cudaEventCreate(&e) != cudaSuccess) return undo();
    *out = c;
    return FK_OK;
}

fk_status fk_destroy(fk_ctx_t c) {
    if (!c) return FK_EINVAL;
    {
        fk::DeviceGuard g(c->device);
        if (c->stream) cudaStreamSynchronize(c->stream);
        fk::drop_graphs(*c);
        if (c->ws.base) cudaFree(c->ws.base);
        if (c->errword) cudaFree(c->errword);
        if (c->est_dev) cudaFree(c->est_dev);
        if (c->pinned) cudaFreeHost(c->pinned);
        if (c->pinned_ev) cudaEventDestroy(c->pinned_ev);
        for (auto& e : c->ev)
            if (e) cudaEventDestroy(e);
        for (auto& e : c->kev)
            if (e) cudaEventDestroy(e);
        if (c->own_stream) cudaStreamDestroy(c->own_stream);
        if (c->copy_stream) {
            cudaStreamSynchronize(c->copy_stream);
            cudaStreamDestroy(c->copy_stream);
        }
        for (auto& e : c->pipe_ev)
            if (e) cudaEventDestroy(e);
    }
    delete c;
    return FK_OK;
}

fk_status fk_set_stream(fk_ctx_t c, void* stream) {
    if (!c) return FK_EINVAL;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return FK_OK;
}

fk_status fk_synchronize(fk_ctx_t c) {
    if (!c) return FK_EINVAL;
    fk::DeviceGuard g(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fk::cuda_fail(*c, e, "synchronize");
    return fk::check_errword(*c);
}

fk_status fk_reserve(fk_ctx_t c, size_t bytes) {
    if (!c) return FK_EINVAL;
    fk::DeviceGuard g(c->device);
    return fk::ensure_workspace(*c, bytes);
}

fk_status fk_set_wait_limit(fk_ctx_t c, long long cycles) {
    if (!c) return FK_EINVAL;
    const long long v = cycles < 0 ? 4000000000LL : cycles;
    if (v != c->wait_limit) {
        fk::DeviceGuard g(c->device);
        if (c->stream) cudaStreamSynchronize(c->stream);
        fk::drop_graphs(*c);  // captured launches carry the old bound
        c->wait_limit = v;
    }
    return FK_OK;
}

fk_status fk_selftest_timeout(fk_ctx_t c, long long cycles) {
    if (!c) return FK_EINVAL;
    if (cycles < 0 || cycles > 4000000000LL)
        return fk::fail(*c, FK_EINVAL, "selftest_timeout: cycles must lie in [0, 4e9]");
    fk::DeviceGuard g(c->device);
    if (!g.ok) return fk::fail(*c, FK_ECUDA, "selftest_timeout: cannot select device");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->errword, 0, sizeof(int), c->stream);
    if (e != cudaSuccess) return fk::cuda_fail(*c, e, "selftest_timeout");
    fk::selftest_wait_kernel<<<1, 32, 0, c->stream>>>(c->errword, cycles);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fk::cuda_fail(*c, e, "selftest_timeout: kernel");
    return fk::check_errword(*c);
}

fk_status fk_set_profiling(fk_ctx_t c, int enable) {
    if (!c) return FK_EINVAL;
    c->profiling = enable != 0;
    return FK_OK;
}

fk_status fk_last_timings(fk_ctx_t c, float ms[4]) {
    if (!c || !ms) return FK_EINVAL;
    for (int i = 0; i < 4; ++i) ms[i] = c->timings[i];
    return FK_OK;
}

int fk_last_launches(fk_ctx_t c) { return c ? c->launches : -1; }

fk_status fk_last_transfer(fk_ctx_t c, unsigned long long* h2d, unsigned long long* d2h) {
    if (!c) return FK_EINVAL;
    if (h2d) *h2d = c->h2d_bytes;
    if (d2h) *d2h = c->d2h_bytes;
    return FK_OK;
}

fk_status fk_last_kernel_time(fk_ctx_t c, float* ms, int* launches) {
    if (!c || !ms || !launches) return FK_EINVAL;
    *ms = c->kernel_ms;
    *launches = c->kernel_launches;
    return FK_OK;
}

namespace fk {
namespace {

// fk_gpp for large host arrays (mixed precision).  Everything crosses the host
// link on one copy stream, in the order the GPU needs it: the small inputs
// (packed into one pinned block), eps and wtilde, the first row block of
// aqsntemp (with the flag bands), the igp columns of aqsmtemp (gathered on the
// host while that block is in flight: the gather's scattered reads take longer
// than the eps and wtilde copies, and the link would otherwise wait for it),
// then the other row blocks.  The compute stream runs the prep once the first
// block and the columns have landed and each block's contraction as soon as
// that block has; the outputs come back through pinned memory in one copy.
fk_status gpp_host_pipelined(Ctx& x, GppDev r, const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                             const fk_c128* I_eps_array, const fk_c128* wtilde_array, const double* vcoul,
                             const int* inv_igp_index, const int* indinv, const double* wx_array, fk_c128* achtemp,
                             fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp) {
    const int nb = r.nb, nc = r.nc, ng = r.ng;
    const size_t e16 = sizeof(double2), band = (size_t)nb * nc * e16, col = (size_t)ng * nc * e16;
    auto r256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
    // small inputs: device arrays on a 16-byte boundary are used in place, host ones packed
    struct Small {
        const void* user;
        size_t bytes;
        bool dev;
        size_t off;
    } sm[4] = {{vcoul, (size_t)nc * 8, false, 0}, {inv_igp_index, (size_t)ng * 4, false, 0},
               {indinv, (size_t)nc * 4, false, 0}, {wx_array, 24, false, 0}};
    size_t packed = 0;
    for (auto& q : sm) {
        q.dev = is_device_ptr(q.user) && ((uintptr_t)q.user & 15) == 0;
        if (!q.dev) {
            q.off = packed;
            packed += r256(q.bytes);
        }
    }
    const bool aqm_dev = is_device_ptr(aqsmtemp) && ((uintptr_t)aqsmtemp & 15) == 0;
    const bool compact = !aqm_dev && (long)ng * 128 <= (long)nc;
    const size_t aqm_off = packed;
    const size_t aqm_bytes = compact ? (size_t)nb * ng * e16 : 0;
    const size_t outn = 7 + (size_t)nb, out_off = r256(packed + aqm_bytes);
    const size_t pinned_bytes = out_off + outn * e16;
    if (compact) {
        r.aqsm_compact = true;
        r.ldm = ng;
    }
    const size_t need = 2 * r256(col) + r256(band) + r256(packed + aqm_bytes) +
                        (!aqm_dev && !compact ? r256(band) : 0) + gpp_workspace(x, r, true) + outn * e16 + 4096;
    fk_status st = ensure_workspace(x, need);
    if (st != FK_OK) return st;
    x.ws.reset();
    double2* out = (double2*)x.ws.take(outn * e16);
    GppPipe pipe{};
    pipe.aqsn = (const double2*)aqsntemp;
    pipe.eps = (const double2*)I_eps_array;
    pipe.wt = (const double2*)wtilde_array;
    pipe.eps_d = (double2*)x.ws.take(col);
    pipe.wt_d = (double2*)x.ws.take(col);
    pipe.aqsn_d = (double2*)x.ws.take(band);
    uint8_t* small_d = (packed + aqm_bytes) ? (uint8_t*)x.ws.take(packed + aqm_bytes) : nullptr;
    double2* aqsm_full = (!aqm_dev && !compact) ? (double2*)x.ws.take(band) : nullptr;
    if (!out || !pipe.eps_d || !pipe.wt_d || !pipe.aqsn_d || ((packed + aqm_bytes) && !small_d) ||
        (!aqm_dev && !compact && !aqsm_full))
        return fail(x, FK_ENOMEM, "workspace: pipeline");
    r.aqsn = pipe.aqsn_d;
    r.eps = pipe.eps_d;
    r.wt = pipe.wt_d;
    phase_mark(x, 0);
    uint8_t* pb = (uint8_t*)pinned_buffer(x, pinned_bytes);  // waits until the last call's outputs were read
    if (!pb) return fail(x, FK_ENOMEM, "gpp: pinned staging");
    if ((st = pipe_begin(x)) != FK_OK) return st;
    cudaStream_t cs = x.copy_stream;
    // 1. small inputs
    for (auto& q : sm)
        if (!q.dev) {
            std::memcpy(pb + q.off, q.user, q.bytes);
            x.h2d_bytes += q.bytes;
        }
    if (packed && cudaMemcpyAsync(small_d, pb, packed, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        return cuda_fail(x, cudaGetLastError(), "gpp: small inputs");
    // 2. eps and wtilde
    if (cudaMemcpyAsync(pipe.eps_d, I_eps_array, col, cudaMemcpyHostToDevice, cs) != cudaSuccess ||
        cudaMemcpyAsync(pipe.wt_d, wtilde_array, col, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        return cuda_fail(x, cudaGetLastError(), "gpp: eps / wtilde");
    x.h2d_bytes += 2 * col;
    // 3. the first row block of aqsntemp, then aqsmtemp: its igp columns gathered
    // on the host while that block is in flight (or the whole array)
    const int chunks = gpp_pipe_chunks(x, r);
    if ((st = gpp_pipe_copy(x, r, &pipe, 0, 1)) != FK_OK) return st;
    if (compact) {
        std::vector<int> invh, indh;
        const int* ip = inv_igp_index;
        const int* dp = indinv;
        if (sm[1].dev) {
            invh.resize(ng);
            if (cudaMemcpy(invh.data(), inv_igp_index, ng * sizeof(int), cudaMemcpyDefault) != cudaSuccess)
                return cuda_fail(x, cudaGetLastError(), "gpp: reading inv_igp_index");
            ip = invh.data();
        }
        if (sm[2].dev) {
            indh.resize(nc);
            if (cudaMemcpy(indh.data(), indinv, nc * sizeof(int), cudaMemcpyDefault) != cudaSuccess)
                return cuda_fail(x, cudaGetLastError(), "gpp: reading indinv");
            dp = indh.data();
        }
        std::vector<int> gcol(ng);
        for (int h = 0; h < ng; ++h) {  // BGW-Kernels/gppKer.cpp:322-325
            const int ind_ = ip[h];
            int g = -1;
            if (ind_ == nc) g = nc - 1;
            else if (ind_ >= 0 && ind_ < nc) g = dp[ind_];
            gcol[h] = g >= nc ? -1 : g;
        }
        fk_c128* buf = (fk_c128*)(pb + aqm_off);
        for (int n1 = 0; n1 < nb; ++n1) {
            const fk_c128* row = aqsmtemp + (size_t)n1 * nc;
            for (int h = 0; h < ng; ++h) buf[(size_t)n1 * ng + h] = gcol[h] >= 0 ? row[gcol[h]] : fk_c128{0.0, 0.0};
        }
        if (cudaMemcpyAsync(small_d + aqm_off, pb + aqm_off, aqm_bytes, cudaMemcpyHostToDevice, cs) != cudaSuccess)
            return cuda_fail(x, cudaGetLastError(), "gpp: aqsmtemp columns");
        x.h2d_bytes += aqm_bytes;
        r.aqsm = (const double2*)(small_d + aqm_off);
    } else if (aqm_dev) {
        r.aqsm = (const double2*)aqsmtemp;
    } else {
        if (cudaMemcpyAsync(aqsm_full, aqsmtemp, band, cudaMemcpyHostToDevice, cs) != cudaSuccess)
            return cuda_fail(x, cudaGetLastError(), "gpp: staging aqsmtemp");
        x.h2d_bytes += band;
        r.aqsm = aqsm_full;
    }
    if (cudaEventRecord(x.pipe_ev[PIPE_READY], cs) != cudaSuccess)
        return cuda_fail(x, cudaGetLastError(), "gpp: pipeline");
    // 4. the other row blocks of aqsntemp
    if ((st = gpp_pipe_copy(x, r, &pipe, 1, chunks)) != FK_OK) return st;
    r.vcoul = sm[0].dev ? vcoul : (const double*)(small_d + sm[0].off);
    r.inv = sm[1].dev ? inv_igp_index : (const int*)(small_d + sm[1].off);
    r.indinv = sm[2].dev ? indinv : (const int*)(small_d + sm[2].off);
    r.wx = sm[3].dev ? wx_array : (const double*)(small_d + sm[3].off);
    r.out = out;
    if ((st = gpp_run(x, r, &pipe)) != FK_OK) return st;
    // outputs through pinned memory
    double2* po = (double2*)(pb + out_off);
    cudaError_t e = cudaMemcpyAsync(po, out, outn * e16, cudaMemcpyDeviceToHost, x.stream);
    x.d2h_bytes += outn * e16;
    if (e == cudaSuccess) e = cudaEventRecord(x.pinned_ev, x.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(x.stream);
    if (e != cudaSuccess) return cuda_fail(x, e, "gpp: synchronize");
    phase_close(x, 4);
    if ((st = check_errword(x)) != FK_OK) return st;
    struct O {
        fk_c128* dst;
        size_t off, n;
    } outs[4] = {{achtemp, 0, 3}, {asxtemp, 3, 3}, {achstemp, 6, 1}, {acht_n1_loc, 7, (size_t)nb}};
    for (const O& o : outs) {
        if (!o.dst) continue;
        if (is_device_ptr(o.dst)) {
            if (cudaMemcpy(o.dst, po + o.off, o.n * e16, cudaMemcpyHostToDevice) != cudaSuccess)
                return cuda_fail(x, cudaGetLastError(), "gpp: output copy");
        } else {
            std::memcpy(o.dst, po + o.off, o.n * e16);
        }
    }
    return FK_OK;
}

}  // namespace
}  // namespace fk

namespace {
fk_status gpp_call(fk_ctx_t c, int nb, int nv, int nc, int ng, const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                   const fk_c128* I_eps_array, const fk_c128* wtilde_array, const double* vcoul,
                   const int* inv_igp_index, const int* indinv, const double* wx_array, fk_precision precision,
                   unsigned flags, fk_c128* achtemp, fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp) {
    Ctx& x = *c;
    x.h2d_bytes = x.d2h_bytes = 0;
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb)
        return fk::fail(x, FK_EINVAL, "gpp: need number_bands, ncouls, ngpown > 0 and 0 <= nvband <= number_bands");
    if (!aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !inv_igp_index || !indinv ||
        !wx_array || !achtemp || !asxtemp)
        return fk::fail(x, FK_EINVAL, "gpp: null required pointer");
    if (precision != FK_FP64 && precision != FK_MIXED) return fk::fail(x, FK_EINVAL, "gpp: bad precision");
    if (flags & ~(FK_GPP_ROOT_QUIRKS | FK_GPP_ACHSTEMP | FK_GPP_HALF_SUM | FK_GPP_PHYSICS))
        return fk::fail(x, FK_EINVAL, "gpp: unknown flag");
    if ((flags & FK_GPP_PHYSICS) && (flags & (FK_GPP_ROOT_QUIRKS | FK_GPP_HALF_SUM)))
        return fk::fail(x, FK_EINVAL, "gpp: FK_GPP_PHYSICS follows the Fortran source, not the root or half-sum drivers");
    if ((flags & FK_GPP_HALF_SUM) && (flags & FK_GPP_ROOT_QUIRKS))
        return fk::fail(x, FK_EINVAL, "gpp: FK_GPP_HALF_SUM and FK_GPP_ROOT_QUIRKS are different drivers");
    if ((flags & FK_GPP_HALF_SUM) && (flags & FK_GPP_ACHSTEMP))
        return fk::fail(x, FK_ENOTSUP, "gpp: achstemp of the half sum is not provided");
    if ((flags & FK_GPP_ROOT_QUIRKS) && ng > nc)
        return fk::fail(x, FK_EINVAL, "gpp: FK_GPP_ROOT_QUIRKS indexes I_eps[my_igp*ngpown+ig] and needs ngpown <= ncouls");
    if (ng > 65535) return fk::fail(x, FK_ENOTSUP, "gpp: ngpown > 65535");
    fk::DeviceGuard g(x.device);
    if (!g.ok) return fk::fail(x, FK_ECUDA, "gpp: cannot select device");

    const size_t band = (size_t)nb * nc * sizeof(double2), col = (size_t)ng * nc * sizeof(double2);
    fk::In aqm{aqsmtemp, band}, aqn{aqsntemp, band}, eps{I_eps_array, col}, wt{wtilde_array, col},
        vc{vcoul, (size_t)nc * sizeof(double)}, inv{inv_igp_index, (size_t)ng * sizeof(int)},
        ind{indinv, (size_t)nc * sizeof(int)}, wx{wx_array, 3 * sizeof(double)};
    std::vector<fk::In*> ins{&aqm, &aqn, &eps, &wt, &vc, &inv, &ind, &wx};
    for (auto* i : ins) i->dev = fk::is_device_ptr(i->user);

    fk::GppDev r{};
    r.nb = nb; r.nv = nv; r.nc = nc; r.ng = ng; r.prec = precision; r.flags = flags;
    r.ldm = nc;
    r.aqsm_compact = false;
    // Large host arrays of a mixed-precision call: stream eps, wtilde and aqsntemp in
    // k-chunks and compute each chunk as it lands (the host link is the bottleneck).
    // Over four or more n-tiles (ngpown >= 64) the contraction on CTA pairs with a
    // pre-split A image, after all inputs have landed, is faster than streaming
    // single-CTA contractions that split the A rows again for every n-tile.
    if (precision == FK_MIXED && !(flags & FK_GPP_HALF_SUM) && !aqn.dev && !eps.dev && !wt.dev && nb > nv &&
        band >= ((size_t)64 << 20) && ng < 64)
        return fk::gpp_host_pipelined(x, r, aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul, inv_igp_index,
                                      indinv, wx_array, achtemp, asxtemp, acht_n1_loc, achstemp);
    // Host aqsmtemp: the sum reads only its ngpown columns igp(my_igp)
    // (BGW-Kernels/gppKer.cpp:322-325), so when those are few, gather them on
    // the host and stage nb x ngpown values instead of nb x ncouls.
    if (!aqm.dev && !(flags & FK_GPP_HALF_SUM) && (long)ng * 128 <= (long)nc) {
        std::vector<int> invh(ng), indh(nc);
        const int* ip = inv_igp_index;
        const int* dp = indinv;
        bool ok = true;
        if (inv.dev) { ok = ok && cudaMemcpy(invh.data(), inv_igp_index, ng * sizeof(int), cudaMemcpyDefault) == cudaSuccess; ip = invh.data(); }
        if (ind.dev) { ok = ok && cudaMemcpy(indh.data(), indinv, nc * sizeof(int), cudaMemcpyDefault) == cudaSuccess; dp = indh.data(); }
        fk_c128* buf = ok ? (fk_c128*)fk::pinned_buffer(x, band / nc * ng) : nullptr;
        if (buf) {
            for (int h = 0; h < ng; ++h) {
                const int ind_ = ip[h];
                int g = -1;
                if (ind_ == nc) g = nc - 1;
                else if (ind_ >= 0 && ind_ < nc) g = dp[ind_];
                if (g >= nc) g = -1;
                for (int n1 = 0; n1 < nb; ++n1)
                    buf[(size_t)n1 * ng + h] = g >= 0 ? aqsmtemp[(size_t)n1 * nc + g] : fk_c128{0.0, 0.0};
            }
            aqm.user = buf;
            aqm.bytes = (size_t)nb * ng * sizeof(double2);
            r.ldm = ng;
            r.aqsm_compact = true;
        } else {
            cudaGetLastError();
        }
    }
    const size_t outn = 7 + (size_t)nb;
    const size_t need = fk::staged_bytes(ins) + fk::gpp_workspace(x, r) + outn * sizeof(double2) + 4096;
    fk_status s = fk::ensure_workspace(x, need);
    if (s != FK_OK) return s;

    // Repeated calls whose arrays are all device memory replay a captured
    // CUDA graph of the whole sequence (one launch instead of ~12).
    bool all_dev = !x.profiling && x.use_graphs;
    for (auto* i : ins) all_dev = all_dev && i->dev;
    const void* outs[4] = {achtemp, asxtemp, acht_n1_loc, achstemp};
    for (auto* o : outs) all_dev = all_dev && (o == nullptr || fk::is_device_ptr(o));
    uint64_t key = 0;
    fk::Ctx::GraphEntry* ge = nullptr;
    if (all_dev) {
        uint64_t w[24] = {(uint64_t)nb, (uint64_t)nv, (uint64_t)nc, (uint64_t)ng, (uint64_t)precision, flags,
                          (uint64_t)(uintptr_t)x.stream, (uint64_t)(uintptr_t)x.ws.base, (uint64_t)x.est_on};
        int n = 9;
        for (auto* i : ins) w[n++] = (uint64_t)(uintptr_t)i->user;
        for (auto* o : outs) w[n++] = (uint64_t)(uintptr_t)o;
        key = fk::fnv(w, n);
        ge = &x.graphs[key];
        if (ge->exec) {
            cudaError_t e = cudaGraphLaunch(ge->exec, x.stream);
            if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp: graph launch");
            return FK_OK;
        }
    }
    const bool capture = ge && ge->seen >= 1 && x.graphs.size() <= 64;
    if (ge) ++ge->seen;
    if (capture) {
        cudaError_t e = cudaStreamBeginCapture(x.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp: begin capture");
    }
    auto enqueue = [&]() -> fk_status {
        x.ws.reset();
        x.h2d_bytes = x.d2h_bytes = 0;
        double2* out = (double2*)x.ws.take(outn * sizeof(double2));
        fk::phase_mark(x, 0);
        fk_status st = fk::stage(x, ins);
        if (st != FK_OK) return st;
        if (r.aqsm_compact) cudaEventRecord(x.pinned_ev, x.stream);
        r.aqsm = (const double2*)aqm.d; r.aqsn = (const double2*)aqn.d;
        r.eps = (const double2*)eps.d; r.wt = (const double2*)wt.d;
        r.vcoul = (const double*)vc.d; r.inv = (const int*)inv.d; r.indinv = (const int*)ind.d;
        r.wx = (const double*)wx.d; r.out = out;
        if ((st = fk::gpp_run(x, r)) != FK_OK) return st;
        bool host_out = false;
        if ((st = fk::deliver(x, achtemp, out, 0, 3, host_out)) != FK_OK) return st;
        if ((st = fk::deliver(x, asxtemp, out, 3, 3, host_out)) != FK_OK) return st;
        if ((st = fk::deliver(x, achstemp, out, 6, 1, host_out)) != FK_OK) return st;
        if ((st = fk::deliver(x, acht_n1_loc, out, 7, nb, host_out)) != FK_OK) return st;
        if (host_out || x.profiling) {
            cudaError_t e = cudaStreamSynchronize(x.stream);
            if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp: synchronize");
            fk::phase_close(x, 4);
            if ((st = fk::check_errword(x)) != FK_OK) return st;
        }
        return FK_OK;
    };
    s = enqueue();
    if (capture) {
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(x.stream, &graph);
        cudaError_t ei = cudaErrorUnknown;
        if (s == FK_OK && e == cudaSuccess && graph) ei = cudaGraphInstantiate(&ge->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ei == cudaSuccess) {
            e = cudaGraphLaunch(ge->exec, x.stream);
            if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp: graph launch");
            return FK_OK;
        }
        // The sequence could not be captured: never try again for this key and
        // run it directly (the captured work, if any, was discarded).
        cudaGetLastError();
        ge->exec = nullptr;
        ge->seen = -(1 << 30);
        s = enqueue();
    }
    return s;
}
}  // namespace

fk_status fk_gpp(fk_ctx_t c, int nb, int nv, int nc, int ng, const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                 const fk_c128* I_eps_array, const fk_c128* wtilde_array, const double* vcoul,
                 const int* inv_igp_index, const int* indinv, const double* wx_array, fk_precision precision,
                 unsigned flags, fk_c128* achtemp, fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp) {
    if (!c) return FK_EINVAL;
    c->est_valid = false;
    const fk_status s = gpp_call(c, nb, nv, nc, ng, aqsmtemp, aqsntemp, I_eps_array, wtilde_array, vcoul,
                                 inv_igp_index, indinv, wx_array, precision, flags, achtemp, asxtemp, acht_n1_loc,
                                 achstemp);
    // the mixed sums other than the half sum carry the estimate (fk_gpp_error_estimate)
    c->est_valid = s == FK_OK && c->est_on && c->est_dev && precision == FK_MIXED && !(flags & FK_GPP_HALF_SUM);
    return s;
}

fk_status fk_set_error_estimate(fk_ctx_t c, int enable) {
    if (!c) return FK_EINVAL;
    c->est_valid = false;
    if (enable && !c->est_dev) {
        fk::DeviceGuard g(c->device);
        if (!g.ok) return fk::fail(*c, FK_ECUDA, "set_error_estimate: cannot select device");
        if (cudaMalloc(&c->est_dev, 4 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            c->est_dev = nullptr;
            return fk::fail(*c, FK_ENOMEM, "set_error_estimate: cannot allocate the estimate's result");
        }
    }
    c->est_on = enable != 0;
    return FK_OK;
}

fk_status fk_gpp_error_estimate(fk_ctx_t c, double* max_err_est) {
    if (!c) return FK_EINVAL;
    if (!max_err_est) return fk::fail(*c, FK_EINVAL, "gpp_error_estimate: null max_err_est");
    if (!c->est_valid)
        return fk::fail(*c, FK_ENOTSUP, "gpp_error_estimate: the last fk_gpp call on this context was not a "
                                        "mixed-precision call made with fk_set_error_estimate(ctx, 1) (the half "
                                        "sum has no estimate)");
    fk::DeviceGuard g(c->device);
    if (!g.ok) return fk::fail(*c, FK_ECUDA, "gpp_error_estimate: cannot select device");
    double h[3];
    cudaError_t e = cudaMemcpyAsync(h, c->est_dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fk::cuda_fail(*c, e, "gpp_error_estimate");
    fk_status st = fk::check_errword(*c);
    if (st != FK_OK) return st;
    for (int i = 0; i < 3; ++i) max_err_est[i] = h[i];
    return FK_OK;
}

fk_status fk_gpp_real(fk_ctx_t c, int nb, int nv, int nc, int ng, const double* aqsmtemp, const double* aqsntemp,
                      const double* I_eps_array, const double* wtilde_array, const double* vcoul,
                      const int* inv_igp_index, const int* indinv, const double* wx_array, fk_precision precision,
                      unsigned flags, double* achtemp, double* asxtemp, double* acht_n1_loc) {
    if (!c) return FK_EINVAL;
    Ctx& x = *c;
    x.h2d_bytes = x.d2h_bytes = 0;
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb)
        return fk::fail(x, FK_EINVAL, "gpp_real: need number_bands, ncouls, ngpown > 0 and 0 <= nvband <= number_bands");
    if (!aqsmtemp || !aqsntemp || !I_eps_array || !wtilde_array || !vcoul || !inv_igp_index || !indinv ||
        !wx_array || !achtemp || !asxtemp)
        return fk::fail(x, FK_EINVAL, "gpp_real: null required pointer");
    if (precision != FK_FP64 && precision != FK_MIXED) return fk::fail(x, FK_EINVAL, "gpp_real: bad precision");
    if (flags & ~FK_GPP_REAL_ZERO_MASKED) return fk::fail(x, FK_EINVAL, "gpp_real: unknown flag");
    if (ng > 65535) return fk::fail(x, FK_ENOTSUP, "gpp_real: ngpown > 65535");
    fk::DeviceGuard g(x.device);
    if (!g.ok) return fk::fail(x, FK_ECUDA, "gpp_real: cannot select device");

    const size_t band = (size_t)nb * nc * sizeof(double), col = (size_t)ng * nc * sizeof(double);
    fk::In aqm{aqsmtemp, band}, eps{I_eps_array, col}, wt{wtilde_array, col}, vc{vcoul, (size_t)nc * sizeof(double)},
        inv{inv_igp_index, (size_t)ng * sizeof(int)}, ind{indinv, (size_t)nc * sizeof(int)},
        wx{wx_array, 3 * sizeof(double)};
    std::vector<fk::In*> ins{&aqm, &eps, &wt, &vc, &inv, &ind, &wx};
    for (auto* i : ins) i->dev = fk::is_device_ptr(i->user);
    // aqsntemp is read as rows of complex pairs: in place when its rows have an
    // even length and start on 16-byte boundaries, else copied with a padded
    // (even) row stride whose pad column is zero
    const bool aqn_dev = fk::is_device_ptr(aqsntemp);
    const bool aqn_in_place = aqn_dev && (nc % 2 == 0) && ((uintptr_t)aqsntemp & 15) == 0;
    const long lda = nc + (nc & 1);
    const size_t aqn_bytes = aqn_in_place ? 0 : ((size_t)nb * lda * sizeof(double) + 255) & ~(size_t)255;

    fk::GppRealDev r{};
    r.nb = nb; r.nv = nv; r.nc = nc; r.ng = ng; r.prec = precision; r.flags = flags;
    r.lda = aqn_in_place ? nc : lda;
    const size_t outn = 6 + (size_t)nb;
    const size_t need = fk::staged_bytes(ins) + aqn_bytes + fk::gpp_real_workspace(x, r) + outn * sizeof(double) + 4096;
    fk_status s = fk::ensure_workspace(x, need);
    if (s != FK_OK) return s;
    x.ws.reset();
    double* out = (double*)x.ws.take(outn * sizeof(double));
    fk::phase_mark(x, 0);
    if ((s = fk::stage(x, ins)) != FK_OK) return s;
    if (aqn_in_place) {
        r.aqsn = aqsntemp;
    } else {
        double* d = (double*)x.ws.take(aqn_bytes);
        if (!out || !d) return fk::fail(x, FK_ENOMEM, "workspace: staging");
        cudaError_t e = cudaMemcpy2DAsync(d, lda * sizeof(double), aqsntemp, nc * sizeof(double), nc * sizeof(double),
                                          nb, aqn_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, x.stream);
        if (e == cudaSuccess && (nc & 1))
            e = cudaMemset2DAsync(d + nc, lda * sizeof(double), 0, sizeof(double), nb, x.stream);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp_real: staging aqsntemp");
        if (!aqn_dev) x.h2d_bytes += (size_t)nb * nc * sizeof(double);
        r.aqsn = d;
    }
    r.aqsm = (const double*)aqm.d; r.eps = (const double*)eps.d; r.wt = (const double*)wt.d;
    r.vcoul = (const double*)vc.d; r.inv = (const int*)inv.d; r.indinv = (const int*)ind.d;
    r.wx = (const double*)wx.d; r.out = out;
    if ((s = fk::gpp_real_run(x, r)) != FK_OK) return s;
    bool host_out = false;
    struct Out {
        double* dst;
        size_t off, n;
    } outs[3] = {{achtemp, 0, 3}, {asxtemp, 3, 3}, {acht_n1_loc, 6, (size_t)nb}};
    for (const Out& o : outs) {
        if (!o.dst) continue;
        if (!fk::is_device_ptr(o.dst)) {
            host_out = true;
            x.d2h_bytes += o.n * sizeof(double);
        }
        cudaError_t e = cudaMemcpyAsync(o.dst, out + o.off, o.n * sizeof(double), cudaMemcpyDefault, x.stream);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp_real: output copy");
    }
    if (host_out || x.profiling) {
        cudaError_t e = cudaStreamSynchronize(x.stream);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "gpp_real: synchronize");
        fk::phase_close(x, 4);
        if ((s = fk::check_errword(x)) != FK_OK) return s;
    }
    return FK_OK;
}

fk_status fk_ff(fk_ctx_t c, int nb, int nv, int nc, int ng, int nf, int ne, const fk_c128* aqsmtemp,
                const fk_c128* aqsntemp, const fk_c128* I_epsR_array, const fk_c128* I_epsA_array,
                const double* vcoul, const int* inv_igp_index, const int* indinv, const double* ekq,
                const double* dFreqGrid, const fk_c128* dFreqBrd, const double* pref, double pref_zb,
                double freqevalmin, double freqevalstep, double occ, fk_precision precision, unsigned flags,
                fk_c128* achsDtemp, fk_c128* asxDtemp, fk_c128* achDtemp, fk_c128* achDtemp_cor,
                fk_c128* ach2Dtemp, fk_c128* schDt_matrix) {
    if (!c) return FK_EINVAL;
    Ctx& x = *c;
    x.h2d_bytes = x.d2h_bytes = 0;
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb || nf < 2 || ne < 1)
        return fk::fail(x, FK_EINVAL, "ff: need sizes > 0, nFreq >= 2, 0 <= nvband <= number_bands");
    if (ng > nc) return fk::fail(x, FK_EINVAL, "ff: ngpown cannot be greater than ncouls");
    if (!aqsmtemp || !aqsntemp || !I_epsR_array || !I_epsA_array || !vcoul || !inv_igp_index || !indinv || !ekq ||
        !dFreqGrid || !dFreqBrd || !pref || !achsDtemp || !asxDtemp || !achDtemp_cor)
        return fk::fail(x, FK_EINVAL, "ff: null required pointer");
    if (precision != FK_FP64 && precision != FK_MIXED) return fk::fail(x, FK_EINVAL, "ff: bad precision");
    if (flags & ~(FK_FF_SCHDT_GEMM | FK_FF_PHYSICS | FK_FF_SPLIT_ACHD)) return fk::fail(x, FK_EINVAL, "ff: unknown flag");
    fk::DeviceGuard g(x.device);
    if (!g.ok) return fk::fail(x, FK_ECUDA, "ff: cannot select device");

    const size_t band = (size_t)nb * nc * sizeof(double2), planes = (size_t)nf * ng * nc * sizeof(double2);
    fk::In aqm{aqsmtemp, band}, aqn{aqsntemp, band}, er{I_epsR_array, planes}, ea{I_epsA_array, planes},
        vc{vcoul, (size_t)nc * sizeof(double)}, inv{inv_igp_index, (size_t)ng * sizeof(int)},
        ind{indinv, (size_t)nc * sizeof(int)}, ek{ekq, (size_t)nb * sizeof(double)},
        gr{dFreqGrid, (size_t)nf * sizeof(double)}, br{dFreqBrd, (size_t)nf * sizeof(double2)},
        pr{pref, (size_t)nf * sizeof(double)};
    std::vector<fk::In*> ins{&aqm, &aqn, &er, &ea, &vc, &inv, &ind, &ek, &gr, &br, &pr};
    for (auto* i : ins) i->dev = fk::is_device_ptr(i->user);

    fk::FfDev r{};
    r.nb = nb; r.nv = nv; r.nc = nc; r.ng = ng; r.nf = nf; r.ne = ne;
    r.pref_zb = pref_zb; r.fmin = freqevalmin; r.fstep = freqevalstep; r.occ = occ;
    r.prec = precision; r.flags = flags;
    r.ekq = ekq; r.grid = dFreqGrid;  // host or device; only read by the planner
    // host I_epsR / I_epsA of a large request: streamed in plane groups while
    // the groups already copied are being computed (fk::FfPipe)
    const bool pipelined = !er.dev && !ea.dev && planes >= ((size_t)64 << 20) && !fk::capturing(x.stream);
    const size_t wsb = fk::ff_workspace(x, r, pipelined);
    if (wsb == (size_t)-1) return fk::fail(x, FK_ECUDA, "ff: reading ekq/dFreqGrid");
    const size_t outn = 1 + 4 * (size_t)ne + (size_t)nb * nf;
    auto r256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
    std::vector<fk::In*> small{&vc, &inv, &ind, &ek, &gr, &br, &pr}, bands{&aqm, &aqn};
    size_t packed = 0;
    for (auto* i : small)
        if (!fk::in_place(i)) packed += r256(i->bytes);
    const size_t need = (pipelined ? fk::staged_bytes(bands) + 2 * r256(planes) + r256(packed) : fk::staged_bytes(ins)) +
                        wsb + outn * sizeof(double2) + 4096;
    fk_status s = fk::ensure_workspace(x, need);
    if (s != FK_OK) return s;
    x.ws.reset();
    double2* out = (double2*)x.ws.take(outn * sizeof(double2));
    fk::phase_mark(x, 0);
    fk::FfPipe pipe{};
    std::vector<double> ekq_h, grid_h;
    if (!pipelined) {
        if ((s = fk::stage(x, ins)) != FK_OK) return s;
    } else {
        // small inputs packed into pinned memory, then aqsmtemp and aqsntemp, on
        // the copy stream ahead of the planes; the planner reads ekq and dFreqGrid on the host
        pipe.ekq_h = ekq;
        pipe.grid_h = dFreqGrid;
        if (ek.dev || gr.dev) {
            ekq_h.resize(nb);
            grid_h.resize(nf);
            if (cudaMemcpy(ekq_h.data(), ekq, nb * sizeof(double), cudaMemcpyDefault) != cudaSuccess ||
                cudaMemcpy(grid_h.data(), dFreqGrid, nf * sizeof(double), cudaMemcpyDefault) != cudaSuccess)
                return fk::cuda_fail(x, cudaGetLastError(), "ff: reading ekq/dFreqGrid");
            pipe.ekq_h = ekq_h.data();
            pipe.grid_h = grid_h.data();
        }
        pipe.epsR = (const double2*)I_epsR_array;
        pipe.epsA = (const double2*)I_epsA_array;
        pipe.epsR_d = (double2*)x.ws.take(planes);
        pipe.epsA_d = (double2*)x.ws.take(planes);
        uint8_t* small_d = packed ? (uint8_t*)x.ws.take(packed) : nullptr;
        if (!out || !pipe.epsR_d || !pipe.epsA_d || (packed && !small_d)) return fk::fail(x, FK_ENOMEM, "workspace: pipeline");
        uint8_t* pb = packed ? (uint8_t*)fk::pinned_buffer(x, packed) : nullptr;  // free once its last copy is done
        if (packed && !pb) return fk::fail(x, FK_ENOMEM, "ff: pinned staging");
        if ((s = fk::pipe_begin(x)) != FK_OK) return s;
        cudaStream_t cs = x.copy_stream;
        size_t off = 0;
        for (auto* i : small) {
            if (fk::in_place(i)) {
                i->d = i->user;
                continue;
            }
            std::memcpy(pb + off, i->user, i->bytes);
            x.h2d_bytes += i->bytes;
            i->d = small_d + off;
            off += r256(i->bytes);
        }
        cudaError_t e = cudaSuccess;
        if (packed) {
            e = cudaMemcpyAsync(small_d, pb, packed, cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess) e = cudaEventRecord(x.pinned_ev, cs);
        }
        for (auto* i : bands) {
            if (e != cudaSuccess) break;
            if (fk::in_place(i)) {
                i->d = i->user;
                continue;
            }
            void* d = x.ws.take(i->bytes);
            if (!d) return fk::fail(x, FK_ENOMEM, "workspace: staging");
            e = cudaMemcpyAsync(d, i->user, i->bytes, i->dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, cs);
            if (!i->dev) x.h2d_bytes += i->bytes;
            i->d = d;
        }
        if (e == cudaSuccess) e = cudaEventRecord(x.pipe_ev[fk::PIPE_READY], cs);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "ff: staging copies");
        er.d = pipe.epsR_d;
        ea.d = pipe.epsA_d;
    }
    r.aqsm = (const double2*)aqm.d; r.aqsn = (const double2*)aqn.d;
    r.epsR = (const double2*)er.d; r.epsA = (const double2*)ea.d; r.brd = (const double2*)br.d;
    r.vcoul = (const double*)vc.d; r.ekq = (const double*)ek.d; r.grid = (const double*)gr.d;
    r.pref = (const double*)pr.d; r.inv = (const int*)inv.d; r.indinv = (const int*)ind.d; r.out = out;
    if ((s = fk::ff_run(x, r, pipelined ? &pipe : nullptr)) != FK_OK) return s;
    bool host_out = false;
    if ((s = fk::deliver(x, achsDtemp, out, 0, 1, host_out)) != FK_OK) return s;
    if ((s = fk::deliver(x, asxDtemp, out, 1, ne, host_out)) != FK_OK) return s;
    if ((s = fk::deliver(x, achDtemp, out, 1 + ne, ne, host_out)) != FK_OK) return s;
    if ((s = fk::deliver(x, achDtemp_cor, out, 1 + 2 * (size_t)ne, ne, host_out)) != FK_OK) return s;
    if ((s = fk::deliver(x, ach2Dtemp, out, 1 + 3 * (size_t)ne, ne, host_out)) != FK_OK) return s;
    if ((s = fk::deliver(x, schDt_matrix, out, 1 + 4 * (size_t)ne, (size_t)nb * nf, host_out)) != FK_OK) return s;
    if (host_out || x.profiling) {
        cudaError_t e = cudaStreamSynchronize(x.stream);
        if (e != cudaSuccess) return fk::cuda_fail(x, e, "ff: synchronize");
        fk::phase_close(x, 4);
        if ((s = fk::check_errword(x)) != FK_OK) return s;
    }
    return FK_OK;
}

}  // extern "C"
