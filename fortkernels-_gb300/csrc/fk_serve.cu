// fk_serve.cu -- the GPP request server.
//
// A worker thread owns one GPU stream and runs steps.  Each step admits
// waiting requests whose device footprint fits in the server's memory budget
// (first fit, in arrival order; a later request may pass one that does not fit
// yet for a few steps), stages their host inputs, and hands every active
// request a fair share of the step's contraction work: a large request advances
// a slice of its k-range per step while small ones finish in one.  The step
// itself is one replay of a captured graph whose kernels read a table of the
// step's requests (fk_gpp.cu: gpp_step_launch).  Epsilon and wtilde can be put
// once under a key and stay resident across requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fk_firstfit.h"
#include "fk_internal.h"

namespace fk {
namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Makes `device` current for the scope and restores the caller's device.
struct DevScope {
    int prev = -1;
    explicit DevScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(device);
    }
    ~DevScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// First-fit allocator over one device block, coalescing on release (the
// bookkeeping by offsets is FirstFit's).
class Arena {
  public:
    ~Arena() {
        if (base_) cudaFree(base_);
    }
    bool init(size_t bytes) {
        ff_.reset(bytes);
        if (cudaMalloc(&base_, ff_.capacity()) != cudaSuccess) {
            cudaGetLastError();
            base_ = nullptr;
            ff_.reset(0);
            return false;
        }
        return true;
    }
    void* alloc(size_t bytes) {
        const size_t off = ff_.alloc(bytes);
        return off == FirstFit::NONE ? nullptr : (char*)base_ + off;
    }
    void release(void* p) {
        if (p) ff_.release((size_t)((char*)p - (char*)base_));
    }
    size_t capacity() const { return ff_.capacity(); }
    size_t peak() const { return ff_.peak(); }

  private:
    void* base_ = nullptr;
    FirstFit ff_;
};

struct Resident {
    void* dev = nullptr;
    size_t bytes = 0;
    int refs = 0;
    bool evicted = false;
};

struct Request {
    uint64_t id = 0;
    fk_gpp_request q{};
    double t_submit = 0, t_done = 0;
    int state = 0;  // 0 waiting, 1 active, 2 done
    fk_status status = FK_OK;
    void* mem = nullptr;  // arena block: staged inputs, then the workspace
    size_t mem_bytes = 0;
    GppJob* job = nullptr;
    int units = 0, next = 0, spu = 1;
    bool first = true;
    int waited = 0;
    uint64_t key[2] = {0, 0};
    bool keyed[2] = {false, false};
};

bool dev_ptr(const void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// An input is used in place when it is device memory on a 16-byte boundary.
bool in_place(const void* p) { return dev_ptr(p) && ((uintptr_t)p & 15) == 0; }

}  // namespace
}  // namespace fk

struct fk_server {
    fk_ctx_t ctx = nullptr;
    fk::Arena arena;
    fk::GppStep* step = nullptr;
    int max_active = 16;
    long step_stages = 96;  // per SM
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    std::thread worker;
    bool stop = false;
    std::deque<fk::Request*> waiting;
    std::vector<fk::Request*> active;
    std::unordered_map<uint64_t, fk::Request*> reqs;
    std::unordered_map<uint64_t, fk::Resident> resident;
    uint64_t next_id = 1;
    // statistics
    std::vector<double> lat;
    double terms = 0, first_submit = -1, last_done = 0;
    unsigned long long submitted = 0, completed = 0, steps = 0, step_reqs = 0;
    int peak_active = 0;
    // pinned staging of finished outputs
    double2* pinned = nullptr;
    size_t pinned_n = 0;
    // autotuned k-slice counts by request shape (nb, nvband, ncouls, ngpown, flags)
    std::map<std::vector<long>, int> tuned;
    int ks_for(const fk_gpp_request& q) const {
        auto it = tuned.find({q.number_bands, q.nvband, q.ncouls, q.ngpown, (long)q.flags});
        return it == tuned.end() ? 0 : it->second;
    }

    void run();
    bool admit(fk::Request* r);
    void release(fk::Request* r);
};

namespace fk {
namespace {

const size_t kElt = sizeof(double2);

// Device bytes a request needs besides its workspace: its inputs that are not
// usable in place.
size_t staged_bytes(const fk_server& s, const fk_gpp_request& q) {
    const size_t nb = q.number_bands, nc = q.ncouls, ng = q.ngpown;
    size_t b = 0;
    auto add = [&](const void* p, size_t bytes) {
        if (!in_place(p)) b += round256(bytes);
    };
    add(q.aqsmtemp, nb * nc * kElt);
    add(q.aqsntemp, nb * nc * kElt);
    if (q.I_eps_array) add(q.I_eps_array, ng * nc * kElt);
    if (q.wtilde_array) add(q.wtilde_array, ng * nc * kElt);
    add(q.vcoul, nc * sizeof(double));
    add(q.inv_igp_index, ng * sizeof(int));
    add(q.indinv, nc * sizeof(int));
    add(q.wx_array, 3 * sizeof(double));
    (void)s;
    return b;
}

GppDev request_dev(const fk_gpp_request& q) {
    GppDev r{};
    r.nb = q.number_bands; r.nv = q.nvband; r.nc = q.ncouls; r.ng = q.ngpown;
    r.prec = FK_MIXED; r.flags = q.flags; r.ldm = q.ncouls; r.aqsm_compact = false;
    return r;
}

}  // namespace
}  // namespace fk

bool fk_server::admit(fk::Request* r) {
    using namespace fk;
    const fk_gpp_request& q = r->q;
    GppDev d = request_dev(q);
    const int ks = ks_for(q);
    const size_t ws = gpp_job_bytes(*ctx, d, ks);
    const size_t need = staged_bytes(*this, q) + ws + 4096;
    void* mem = arena.alloc(need);
    if (!mem) return false;
    r->mem = mem;
    r->mem_bytes = need;
    Workspace w;
    w.base = mem;
    w.cap = need;
    cudaStream_t st = ctx->stream;
    bool ok = true;
    auto stage = [&](const void* p, size_t bytes) -> const void* {
        if (in_place(p)) return p;
        void* dst = w.take(bytes);
        if (!dst || cudaMemcpyAsync(dst, p, bytes, cudaMemcpyDefault, st) != cudaSuccess) ok = false;
        return dst;
    };
    const size_t nb = q.number_bands, nc = q.ncouls, ng = q.ngpown;
    d.aqsm = (const double2*)stage(q.aqsmtemp, nb * nc * kElt);
    d.aqsn = (const double2*)stage(q.aqsntemp, nb * nc * kElt);
    const void* eps = q.I_eps_array ? stage(q.I_eps_array, ng * nc * kElt) : resident[r->key[0]].dev;
    const void* wt = q.wtilde_array ? stage(q.wtilde_array, ng * nc * kElt) : resident[r->key[1]].dev;
    d.eps = (const double2*)eps;
    d.wt = (const double2*)wt;
    d.vcoul = (const double*)stage(q.vcoul, nc * sizeof(double));
    d.inv = (const int*)stage(q.inv_igp_index, ng * sizeof(int));
    d.indinv = (const int*)stage(q.indinv, nc * sizeof(int));
    d.wx = (const double*)stage(q.wx_array, 3 * sizeof(double));
    fk_status st2 = FK_OK;
    void* wsp = ok ? w.take(ws) : nullptr;
    if (ok && wsp) r->job = gpp_job_create(*ctx, d, ks, wsp, ws, &st2);
    if (!ok || !wsp || !r->job) {
        r->status = !ok ? FK_ECUDA : (st2 != FK_OK ? st2 : FK_ENOMEM);
        cudaGetLastError();
        return true;  // admitted only to be completed with its error
    }
    r->units = gpp_job_units(r->job);
    r->spu = std::max(1, gpp_job_stages_per_unit(r->job));
    return true;
}

void fk_server::release(fk::Request* r) {
    if (r->job) fk::gpp_job_destroy(r->job);
    r->job = nullptr;
    arena.release(r->mem);
    r->mem = nullptr;
    for (int i = 0; i < 2; ++i) {
        if (!r->keyed[i]) continue;
        auto it = resident.find(r->key[i]);
        if (it == resident.end()) continue;
        if (--it->second.refs <= 0 && it->second.evicted) {
            arena.release(it->second.dev);
            resident.erase(it);
        }
    }
}

void fk_server::run() {
    using namespace fk;
    cudaSetDevice(ctx->device);
    Ctx& c = *ctx;
    std::vector<GppStepItem> items;
    std::vector<Request*> in_step, finishing;
    for (;;) {
        std::vector<Request*> failed;
        {
            std::unique_lock<std::mutex> lk(mu);
            work_cv.wait(lk, [&] { return stop || !waiting.empty() || !active.empty(); });
            if (stop && waiting.empty() && active.empty()) break;
            // admission: arrival order, while slots and memory last
            for (auto it = waiting.begin(); it != waiting.end() && (int)active.size() < max_active;) {
                Request* r = *it;
                if (admit(r)) {
                    it = waiting.erase(it);
                    if (r->status != FK_OK) {
                        failed.push_back(r);
                    } else {
                        r->state = 1;
                        active.push_back(r);
                    }
                } else {
                    // the head waits; later requests may pass it for a few steps
                    if (it == waiting.begin() && ++r->waited > 8) break;
                    ++it;
                }
            }
            peak_active = std::max(peak_active, (int)active.size());
        }
        // requests that failed during admission complete at once
        if (!failed.empty()) {
            cudaStreamSynchronize(c.stream);
            std::lock_guard<std::mutex> lk(mu);
            for (Request* r : failed) {
                release(r);
                r->state = 2;
                r->t_done = now_s();
            }
            done_cv.notify_all();
        }
        if (active.empty()) continue;

        // fair share of the step's work (k-stages), then leftovers in arrival order
        items.clear();
        in_step.clear();
        finishing.clear();
        const long budget = step_stages * c.sms;
        const int n = std::min((int)active.size(), gpp_step_capacity());
        std::vector<int> take(n, 0);
        long left = budget;
        int open = 0;
        for (int i = 0; i < n; ++i) open += active[i]->next < active[i]->units;
        for (int round = 0; round < 2 && left > 0 && open > 0; ++round) {
            const long share = std::max(1L, left / std::max(1, open));
            for (int i = 0; i < n && left > 0; ++i) {
                Request* r = active[i];
                const int rem = r->units - r->next - take[i];
                if (rem <= 0) continue;
                const long cap = round == 0 ? share : left;
                const int k = (int)std::min<long>(rem, std::max(1L, cap / r->spu));
                take[i] += k;
                left -= (long)k * r->spu;
            }
        }
        for (int i = 0; i < n; ++i) {
            Request* r = active[i];
            GppStepItem it{r->job, r->next, r->next + take[i], r->first, r->next + take[i] >= r->units};
            if (it.u1 == it.u0 && !it.first && !it.last) continue;
            items.push_back(it);
            in_step.push_back(r);
            if (it.last) finishing.push_back(r);
        }
        fk_status st = gpp_step_launch(c, step, items.data(), (int)items.size());
        // finished outputs to pinned staging
        size_t need = 0;
        for (Request* r : finishing) need += 7 + (size_t)r->q.number_bands;
        if (need > pinned_n) {
            if (pinned) cudaFreeHost(pinned);
            pinned = nullptr;
            pinned_n = 0;
            if (cudaMallocHost(&pinned, need * sizeof(double2) * 2) == cudaSuccess) pinned_n = need * 2;
            else st = FK_ENOMEM;
        }
        size_t off = 0;
        if (st == FK_OK)
            for (Request* r : finishing) {
                const size_t nout = 7 + (size_t)r->q.number_bands;
                cudaMemcpyAsync(pinned + off, gpp_job_out(r->job), nout * sizeof(double2), cudaMemcpyDeviceToHost,
                                c.stream);
                off += nout;
            }
        cudaError_t e = cudaStreamSynchronize(c.stream);
        int word = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&word, c.errword, sizeof(int), cudaMemcpyDeviceToHost);
        if (st == FK_OK && e != cudaSuccess) st = FK_ECUDA;
        if (st == FK_OK && word != 0) st = FK_ETIMEOUT;
        const double t = now_s();
        std::lock_guard<std::mutex> lk(mu);
        ++steps;
        step_reqs += in_step.size();
        for (size_t i = 0; i < items.size(); ++i) {
            Request* r = in_step[i];
            r->first = false;
            r->next = items[i].u1;
            if (st != FK_OK) r->status = st;
        }
        off = 0;
        for (Request* r : finishing) {
            const size_t nb = r->q.number_bands, nout = 7 + nb;
            if (r->status == FK_OK) {
                const double2* o = pinned + off;
                auto put = [&](fk_c128* dst, const double2* src, size_t n) {
                    if (!dst) return;
                    if (dev_ptr(dst)) cudaMemcpy(dst, src, n * sizeof(double2), cudaMemcpyHostToDevice);
                    else std::memcpy(dst, src, n * sizeof(double2));
                };
                put(r->q.achtemp, o, 3);
                put(r->q.asxtemp, o + 3, 3);
                put(r->q.acht_n1_loc, o + 7, nb);
                terms += 3.0 * nb * r->q.ngpown * r->q.ncouls;
            }
            off += nout;
            release(r);
            r->state = 2;
            r->t_done = t;
            last_done = t;
            lat.push_back(t - r->t_submit);
            ++completed;
        }
        if (st != FK_OK) {
            // a failed step leaves its requests' partial sums undefined: end them all
            for (Request* r : in_step)
                if (r->state != 2) {
                    release(r);
                    r->state = 2;
                    r->t_done = t;
                }
        }
        active.erase(std::remove_if(active.begin(), active.end(), [](Request* r) { return r->state == 2; }),
                     active.end());
        done_cv.notify_all();
    }
}

// --------------------------------------------------------------- C ABI
extern "C" {

fk_status fk_server_create(int device, const fk_server_config* cfg, fk_server_t* out) {
    if (!out || !cfg) return FK_EINVAL;
    *out = nullptr;
    if (cfg->hbm_bytes == 0 || cfg->max_active < 1 || cfg->max_active > fk::gpp_step_capacity() ||
        cfg->step_stages < 0)
        return FK_EINVAL;
    fk_server* s = new (std::nothrow) fk_server();
    if (!s) return FK_ENOMEM;
    fk_status st = fk_create(device, &s->ctx);
    if (st != FK_OK) {
        delete s;
        return st;
    }
    fk::DevScope dev(s->ctx->device);
    s->max_active = cfg->max_active;
    if (cfg->step_stages > 0) s->step_stages = cfg->step_stages;
    if (!s->arena.init(cfg->hbm_bytes)) {
        fk_destroy(s->ctx);
        delete s;
        return FK_ENOMEM;
    }
    s->step = fk::gpp_step_create(*s->ctx, &st);
    if (!s->step) {
        fk_destroy(s->ctx);
        delete s;
        return st;
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return FK_OK;
}

fk_status fk_server_destroy(fk_server_t s) {
    if (!s) return FK_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->work_cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    fk::DevScope dev(s->ctx->device);
    fk::gpp_step_destroy(s->step);
    for (auto& kv : s->reqs) delete kv.second;
    if (s->pinned) cudaFreeHost(s->pinned);
    s->resident.clear();
    fk_ctx_t ctx = s->ctx;
    delete s;  // frees the arena
    fk_destroy(ctx);
    return FK_OK;
}

fk_status fk_server_resident_put(fk_server_t s, unsigned long long key, const void* data, size_t bytes) {
    if (!s || !data || bytes == 0) return FK_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->resident.find(key);
    if (it != s->resident.end())  // in use, or evicted but still read by running requests
        return it->second.evicted ? FK_EBUSY : FK_EINVAL;
    void* dev = s->arena.alloc(bytes);
    if (!dev) return FK_ENOMEM;
    fk::DevScope scope(s->ctx->device);
    if (cudaMemcpy(dev, data, bytes, cudaMemcpyDefault) != cudaSuccess) {
        cudaGetLastError();
        s->arena.release(dev);
        return FK_ECUDA;
    }
    fk::Resident r;
    r.dev = dev;
    r.bytes = bytes;
    s->resident[key] = r;
    return FK_OK;
}

fk_status fk_server_resident_evict(fk_server_t s, unsigned long long key) {
    if (!s) return FK_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->resident.find(key);
    if (it == s->resident.end() || it->second.evicted) return FK_EINVAL;
    if (it->second.refs > 0) {
        it->second.evicted = true;  // freed when its last request ends
        return FK_OK;
    }
    s->arena.release(it->second.dev);
    s->resident.erase(it);
    return FK_OK;
}

fk_status fk_server_submit(fk_server_t s, const fk_gpp_request* q, unsigned long long* ticket) {
    if (!s || !q || !ticket) return FK_EINVAL;
    const int nb = q->number_bands, nv = q->nvband, nc = q->ncouls, ng = q->ngpown;
    if (nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb) return FK_EINVAL;
    if (!q->aqsmtemp || !q->aqsntemp || !q->vcoul || !q->inv_igp_index || !q->indinv || !q->wx_array ||
        !q->achtemp || !q->asxtemp)
        return FK_EINVAL;
    if (q->flags & ~(unsigned)FK_GPP_ROOT_QUIRKS) return FK_EINVAL;
    if ((q->flags & FK_GPP_ROOT_QUIRKS) && ng > nc) return FK_EINVAL;
    if (ng > 65535) return FK_ENOTSUP;
    fk::Request* r = new (std::nothrow) fk::Request();
    if (!r) return FK_ENOMEM;
    r->q = *q;
    std::lock_guard<std::mutex> lk(s->mu);
    const unsigned long long keys[2] = {q->eps_key, q->wtilde_key};
    const void* ptrs[2] = {q->I_eps_array, q->wtilde_array};
    for (int i = 0; i < 2; ++i) {
        if (ptrs[i]) continue;
        auto it = s->resident.find(keys[i]);
        const size_t want = (size_t)ng * nc * fk::kElt;
        if (it == s->resident.end() || it->second.evicted || it->second.bytes < want) {
            delete r;
            return FK_EINVAL;  // no resident array of that size under the key
        }
        r->key[i] = keys[i];
        r->keyed[i] = true;
    }
    // a request that could never fit is refused now
    fk::DevScope scope(s->ctx->device);
    fk::GppDev d = fk::request_dev(*q);
    const size_t need = fk::staged_bytes(*s, *q) + fk::gpp_job_bytes(*s->ctx, d, s->ks_for(*q)) + 4096;
    if (fk::round256(need) > s->arena.capacity()) {
        delete r;
        return FK_ENOMEM;
    }
    for (int i = 0; i < 2; ++i)
        if (r->keyed[i]) ++s->resident[r->key[i]].refs;
    r->id = s->next_id++;
    r->t_submit = fk::now_s();
    if (s->first_submit < 0) s->first_submit = r->t_submit;
    s->reqs[r->id] = r;
    s->waiting.push_back(r);
    ++s->submitted;
    *ticket = r->id;
    s->work_cv.notify_all();
    return FK_OK;
}

fk_status fk_server_wait(fk_server_t s, unsigned long long ticket, double timeout_s, double* latency_s) {
    if (!s) return FK_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return FK_EINVAL;
    fk::Request* r = it->second;
    auto pred = [&] { return r->state == 2; };
    if (timeout_s < 0) s->done_cv.wait(lk, pred);
    else if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return FK_EBUSY;
    const fk_status st = r->status;
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    s->reqs.erase(it);
    delete r;
    return st;
}

fk_status fk_server_cancel(fk_server_t s, unsigned long long ticket) {
    if (!s) return FK_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return FK_EINVAL;
    fk::Request* r = it->second;
    if (r->state != 0) return FK_EBUSY;  // admitted (or finished): it completes as usual
    auto w = std::find(s->waiting.begin(), s->waiting.end(), r);
    if (w == s->waiting.end()) return FK_EBUSY;
    s->waiting.erase(w);
    s->release(r);  // drops its resident references (it holds no memory yet)
    r->status = FK_ECANCELED;
    r->state = 2;
    r->t_done = fk::now_s();
    s->done_cv.notify_all();
    return FK_OK;
}

fk_status fk_server_tune(fk_server_t s, int nb, int nv, int nc, int ng, unsigned flags, int* chosen_ks) {
    if (!s || nb <= 0 || nc <= 0 || ng <= 0 || nv < 0 || nv > nb || ng > 65535) return FK_EINVAL;
    if (flags & ~(unsigned)FK_GPP_ROOT_QUIRKS) return FK_EINVAL;
    if ((flags & FK_GPP_ROOT_QUIRKS) && ng > nc) return FK_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->waiting.empty() || !s->active.empty()) return FK_EBUSY;  // tune while idle
    fk::DevScope scope(s->ctx->device);
    fk::Ctx& c = *s->ctx;
    // synthetic inputs of the shape: zeros, with an index map that stays in range
    const size_t kE = sizeof(double2);
    const size_t in_bytes = fk::round256((size_t)nb * nc * kE) * 2 + fk::round256((size_t)ng * nc * kE) * 2 +
                            fk::round256((size_t)nc * 8) + fk::round256((size_t)ng * 4) + fk::round256((size_t)nc * 4) +
                            256;
    fk::GppDev d{};
    d.nb = nb; d.nv = nv; d.nc = nc; d.ng = ng; d.prec = FK_MIXED; d.flags = flags; d.ldm = nc;
    // candidates: the default plan, and k-slices of 16..256 k-stages
    const int ks0 = fk::gpp_default_ks(c, d);
    const int kst = (nc + 31) / 32;
    std::vector<int> cand{ks0};
    for (int L = 16; L <= 256; L *= 2) {
        const int k = std::max(1, (kst + L - 1) / L);
        if (std::find(cand.begin(), cand.end(), k) == cand.end()) cand.push_back(k);
    }
    size_t ws_max = 0;
    for (int k : cand) ws_max = std::max(ws_max, fk::gpp_job_bytes(c, d, k));
    void* mem = s->arena.alloc(in_bytes + ws_max + 4096);
    if (!mem) return FK_ENOMEM;
    fk::Workspace w;
    w.base = mem;
    w.cap = in_bytes + ws_max + 4096;
    d.aqsm = (const double2*)w.take((size_t)nb * nc * kE);
    d.aqsn = (const double2*)w.take((size_t)nb * nc * kE);
    d.eps = (const double2*)w.take((size_t)ng * nc * kE);
    d.wt = (const double2*)w.take((size_t)ng * nc * kE);
    d.vcoul = (const double*)w.take((size_t)nc * 8);
    d.inv = (const int*)w.take((size_t)ng * 4);
    d.indinv = (const int*)w.take((size_t)nc * 4);
    d.wx = (const double*)w.take(256);
    cudaMemsetAsync(mem, 0, in_bytes, c.stream);
    const double wx[3] = {9.0, 10.0, 11.0};
    cudaMemcpyAsync((void*)d.wx, wx, sizeof(wx), cudaMemcpyHostToDevice, c.stream);
    void* ws = w.take(ws_max);
    // the fastest plan for the request served alone in this server's steps
    std::vector<float> ms(cand.size(), 0.f);
    std::vector<int> units(cand.size(), 0);
    fk_status st = FK_OK;
    for (size_t i = 0; i < cand.size() && st == FK_OK; ++i)
        st = fk::gpp_time_plan(c, s->step, d, cand[i], s->step_stages * c.sms, ws, ws_max, &ms[i], &units[i]);
    cudaStreamSynchronize(c.stream);
    s->arena.release(mem);
    if (st != FK_OK) return st;
    int pick = ks0;
    float best = 1e30f;
    for (size_t i = 0; i < cand.size(); ++i)
        if (ms[i] < best) {
            best = ms[i];
            pick = cand[i];
        }
    s->tuned[{nb, nv, nc, ng, (long)flags}] = pick;
    if (chosen_ks) *chosen_ks = pick;
    return FK_OK;
}

fk_status fk_server_stats(fk_server_t s, fk_server_info* out) {
    if (!s || !out) return FK_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->steps = s->steps;
    out->peak_active = s->peak_active;
    out->hbm_peak_bytes = s->arena.peak();
    out->mean_active = s->steps ? (double)s->step_reqs / (double)s->steps : 0.0;
    if (!s->lat.empty()) {
        std::vector<double> v = s->lat;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            const double x = p * (double)(v.size() - 1);
            const size_t i = (size_t)x;
            const double f = x - (double)i;
            return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
        };
        out->p50_s = pct(0.50);
        out->p99_s = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_s = sum / (double)v.size();
    }
    const double span = s->last_done - s->first_submit;
    out->terms_per_s = span > 0 ? s->terms / span : 0.0;
    return FK_OK;
}

}  // extern "C"
