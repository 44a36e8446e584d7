// fk_internal.h -- host-side declarations shared by the C ABI and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <unordered_map>

#include "../../include/fk_abi.h"

namespace fk {

// Device workspace: a bump allocator over one grow-only cudaMalloc block.
struct Workspace {
    void* base = nullptr;
    size_t cap = 0, used = 0;
    void reset() { used = 0; }
    void* take(size_t bytes) {  // 256-byte aligned; nullptr when it does not fit
        size_t off = (used + 255) & ~size_t(255);
        if (off + bytes > cap) return nullptr;
        used = off + bytes;
        return (char*)base + off;
    }
};

struct Ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    Workspace ws;
    void* pinned = nullptr;      // pinned host staging (column gathers)
    size_t pinned_cap = 0;
    cudaEvent_t pinned_ev = nullptr;  // last copy out of `pinned`
    std::string err;
    bool profiling = false;
    cudaEvent_t ev[5] = {};
    float timings[4] = {0, 0, 0, 0};
    int launches = 0;
    // profiling: events around each launch of the dominant (contraction) kernel
    static constexpr int KEV = 8;
    cudaEvent_t kev[2 * KEV] = {};
    int nk = 0;                 // launches bracketed in the current call
    float kernel_ms = 0.f;      // their summed device time in the last profiled call
    int kernel_launches = 0;
    // host-link bytes of the last fk_gpp / fk_gpp_real / fk_ff call
    unsigned long long h2d_bytes = 0, d2h_bytes = 0;
    int* errword = nullptr;      // device error word of the tensor-core kernels (bounded waits)
    long long wait_limit = 4000000000LL;  // bound of their waits between roles, SM clock cycles (~2 s)
    // a-priori error estimate of mixed fk_gpp calls (fk_set_error_estimate): on/off,
    // its device result [3], and whether the last fk_gpp call on the context made one
    bool est_on = false;
    double* est_dev = nullptr;
    bool est_valid = false;
    // Graphs of repeated fully device-resident calls: key -> (times seen, executable graph).
    struct GraphEntry {
        int seen = 0;
        cudaGraphExec_t exec = nullptr;
    };
    std::unordered_map<uint64_t, GraphEntry> graphs;
    bool use_graphs = true;
    // host-input pipelining: a copy stream and events (one per k-chunk, plus
    // "buffers free" and "small inputs ready"), created on first use
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t pipe_ev[10] = {};
};

// Set the context's last error and return the status.
fk_status fail(Ctx& c, fk_status s, const std::string& msg);
fk_status cuda_fail(Ctx& c, cudaError_t e, const char* where);

// Resolved GPP request: every pointer is device memory.
struct GppDev {
    int nb, nv, nc, ng;
    const double2 *aqsm, *aqsn, *eps, *wt;
    long ldm;           // row stride of aqsm: ncouls, or ngpown when only the igp columns were staged
    bool aqsm_compact;  // aqsm holds column igp(my_igp) at position my_igp
    const double* vcoul;
    const int *inv, *indinv;
    const double* wx;  // device [3]
    fk_precision prec;
    unsigned flags;
    double2* out;      // device [3 achtemp | 3 asxtemp | 1 achstemp | nb acht_n1_loc]
};
// Host arrays of a mixed-precision request streamed to the device in row
// blocks while the blocks already copied are being computed (the host link is
// far slower than HBM, so the copy is the call's critical path).
struct GppPipe {
    const double2 *aqsn, *eps, *wt;  // host sources, row-major as in GppDev
    double2 *aqsn_d, *eps_d, *wt_d;  // device destinations (r.aqsn, r.eps, r.wt point at them)
};
// Bytes of workspace gpp_run needs for this request (excluding staged inputs).
size_t gpp_workspace(const Ctx& c, const GppDev& r, bool pipelined = false);
// Pipelined calls: aqsntemp moves in row blocks (chunk 0: the flag bands and the
// first block of m-tiles; then one block per chunk); gpp_pipe_chunks gives their
// number; pipe_begin makes c.copy_stream wait for the work already queued on
// c.stream (the destinations' last users); gpp_pipe_copy queues the row blocks
// [q0, q1) on c.copy_stream, each followed by its event.  The caller copies
// eps, wtilde and the small inputs first and records pipe_ev[PIPE_READY].
constexpr int PIPE_FREE = 8, PIPE_READY = 9;
int gpp_pipe_chunks(const Ctx& c, const GppDev& r);
fk_status pipe_begin(Ctx& c);
fk_status gpp_pipe_copy(Ctx& c, const GppDev& r, const GppPipe* pipe, int q0, int q1);
fk_status gpp_run(Ctx& c, const GppDev& r, const GppPipe* pipe = nullptr);

// The real-valued GPP sum (gppKer_real.cpp) on device arrays.
struct GppRealDev {
    int nb, nv, nc, ng;
    const double *aqsm, *aqsn, *eps, *wt;  // [nb][nc] (aqsn: row stride lda), [ng][nc]
    long lda;          // row stride of aqsn in doubles: even, >= nc; the pad column (if any) is 0
    const double* vcoul;
    const int *inv, *indinv;
    const double* wx;  // device [3]
    fk_precision prec;
    unsigned flags;
    double* out;       // device [3 achtemp | 3 asxtemp | nb acht_n1_loc]
};
size_t gpp_real_workspace(const Ctx& c, const GppRealDev& r);
fk_status gpp_real_run(Ctx& c, const GppRealDev& r);

// Served GPP requests (mixed precision): a request's plan, workspace and
// descriptors, and the captured step that runs several of them at once.
struct GppJob;
struct GppStep;
struct GppStepItem {
    GppJob* job;
    int u0, u1;   // contraction units [u0, u1) of the request run in this step
    bool first;   // index map, weights and prep run in this step (the request's first)
    bool last;    // the reduction runs in this step (all units done)
};
// Device bytes of a request's workspace (plan with ks k-slices per tile, 0: default).
size_t gpp_job_bytes(const Ctx& c, const GppDev& r, int ks);
// r's pointers are device memory; the workspace is [ws, ws+bytes).  Clears the
// request's image on c.stream.
GppJob* gpp_job_create(Ctx& c, const GppDev& r, int ks, void* ws, size_t bytes, fk_status* st);
void gpp_job_destroy(GppJob* j);
int gpp_job_units(const GppJob* j);
int gpp_job_stages_per_unit(const GppJob* j);
int gpp_job_ks(const GppJob* j);
double2* gpp_job_out(const GppJob* j);  // device [3 achtemp | 3 asxtemp | 1 | nb acht_n1_loc]
GppStep* gpp_step_create(Ctx& c, fk_status* st);
void gpp_step_destroy(GppStep* s);
int gpp_step_capacity();
// Runs one step on c.stream (waits for the previous step's table upload first).
fk_status gpp_step_launch(Ctx& c, GppStep* s, const GppStepItem* items, int n);
// The k-slice count the default plan picks, and the device time (ms) of a
// request run alone through served steps of step_budget k-stages with ks
// k-slices per tile (r: device inputs; [ws, ws+bytes) its workspace).
int gpp_default_ks(const Ctx& c, const GppDev& r);
fk_status gpp_time_plan(Ctx& c, GppStep* s, const GppDev& r, int ks, long step_budget, void* ws, size_t bytes,
                        float* ms, int* units);

struct FfDev {
    int nb, nv, nc, ng, nf, ne;
    const double2 *aqsm, *aqsn, *epsR, *epsA, *brd;
    const double *vcoul, *ekq, *grid, *pref;
    const int *inv, *indinv;
    double pref_zb, fmin, fstep, occ;
    fk_precision prec;
    unsigned flags;
    // outputs (device): [achsDtemp | asx[ne] | achD[ne] | cor[ne] | a2[ne] | schDt[nb*nf]]
    double2* out;
};
// Host I_epsR / I_epsA arrays of an FF request streamed to the device in plane
// groups on c.copy_stream, each group followed by its event (pipe_ev[0..7]);
// the compute stream waits for pipe_ev[PIPE_READY] (the caller's copies of
// aqsmtemp, aqsntemp and the small inputs) and then runs each group's
// conversion and contraction as soon as that group has landed.  The device
// arrays hold all nFreq planes; only the planes the request reads are copied.
struct FfPipe {
    const double2 *epsR, *epsA;      // host sources [nFreq][ngpown][ncouls]
    double2 *epsR_d, *epsA_d;        // device destinations (r.epsR, r.epsA point at them)
    const double *ekq_h, *grid_h;    // host copies of ekq and dFreqGrid (the planner reads them)
};
size_t ff_workspace(const Ctx& c, const FfDev& r, bool pipelined = false);
fk_status ff_run(Ctx& c, const FfDev& r, const FfPipe* pipe = nullptr);

// Phase timing helpers (no-ops unless profiling is on).
void phase_mark(Ctx& c, int i);
void phase_close(Ctx& c, int nphases);
// Bracket one launch of the dominant kernel (profiling only).
void kernel_begin(Ctx& c);
void kernel_end(Ctx& c);

}  // namespace fk

// The public context handle is the internal context.
struct fk_ctx : public fk::Ctx {};
