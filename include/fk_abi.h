/*
 * fk_abi.h -- C ABI of the GB300 (sm_103a) GPP / FF self-energy library.
 *
 * The reference mini-apps have no library boundary: each hot path is a loop
 * nest inside a driver main() that fills its own arrays.  Every entry point
 * below replaces one of those loop nests with a call that takes the same
 * arrays in the same layouts:
 *
 *   fk_gpp  <- the n1 x my_igp x ig x iw nest of BGW-Kernels/gppKer.cpp:303-439
 *              (flagOCC_solver :130-159 + ssxt_scht_solver :19-65 for n1 < nvband,
 *              the cache-blocked noflag block :349-413 otherwise), and its
 *              repo-root variant gppKer.cpp:266-345 (FK_GPP_ROOT_QUIRKS).
 *   fk_ff   <- the kernel sequence of FFKer_cori/ffKernel.cpp:480-503
 *              (achsDtemp_Kernel :107-131, asxDtemp_Kernel :133-153,
 *              achDtemp_Kernel :155-210, achDtemp_cor_Kernel :212-246) plus the
 *              band x G x G' contraction of ffkernel.deslippe.best.f90.back1:402-418.
 *
 * Conventions
 *   - Complex numbers are fk_c128 = {double re, im}, bit-compatible with
 *     std::complex<double> and with the reference's GPUComplex.
 *   - Arrays are row-major exactly as in the reference:
 *       aqsmtemp/aqsntemp [number_bands][ncouls]
 *       I_eps_array/wtilde_array [ngpown][ncouls]
 *       I_epsR_array/I_epsA_array [nFreq][ngpown][ncouls]
 *   - Every array pointer may be host memory or device memory of the
 *     context's GPU; the library detects which.  Host inputs are staged to the
 *     device; host outputs are copied back and the call returns after the
 *     stream has finished.  When every output pointer is device memory the
 *     call only enqueues work on the context's stream and returns at once.
 *   - The caller owns all buffers; no pointer is kept after a call returns.
 *   - Errors are reported by status code only; nothing aborts or throws.
 *   - A context is bound to one device and one stream and is not thread-safe:
 *     use one context per host thread.
 *   - There is no CPU fallback: without a usable GPU every compute call
 *     returns FK_ECUDA.
 */
#ifndef FK_ABI_H
#define FK_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fk_ctx* fk_ctx_t;

typedef enum {
    FK_OK = 0,
    FK_EINVAL = 1,    /* bad sizes, null required pointer, bad flags          */
    FK_ENOMEM = 2,    /* device or pinned-host allocation failed              */
    FK_ECUDA = 3,     /* a CUDA call failed (no device, launch error, ...)    */
    FK_ETIMEOUT = 4,  /* a bounded device-side wait gave up                   */
    FK_EBUSY = 5,     /* admission refused (serving: over the memory budget)  */
    FK_ENOTSUP = 6,   /* valid request the library does not support          */
    FK_ECANCELED = 7  /* serving: the request was cancelled before it ran     */
} fk_status;

typedef enum {
    FK_FP64 = 0,   /* plain path: FP64 everywhere; matches the reference C++ to 1e-12 */
    FK_MIXED = 1   /* branch tests and near-pole divisions in FP64, bulk
                      contractions in reduced precision with FP32 accumulation
                      and FP64 block reductions; <= 1e-6 relative to FP64 */
} fk_precision;

typedef struct { double re, im; } fk_c128;

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device` with its own non-blocking stream. */
fk_status fk_create(int device, fk_ctx_t* out);
fk_status fk_destroy(fk_ctx_t ctx);
/* Use `stream` (a cudaStream_t of the context's device) for later calls;
 * NULL restores the context's own stream. */
fk_status fk_set_stream(fk_ctx_t ctx, void* stream);
/* Wait for all work enqueued by the context. */
fk_status fk_synchronize(fk_ctx_t ctx);
/* Grow the device workspace to at least `bytes` now (e.g. before capturing
 * a CUDA graph, during which the library must not allocate). */
fk_status fk_reserve(fk_ctx_t ctx, size_t bytes);
/* Static description of a status code, and the last detailed message. */
const char* fk_strerror(fk_status s);
const char* fk_last_error(fk_ctx_t ctx);
/* Library version string, e.g. "fk_gb300 1.0 sm_103a". */
const char* fk_version(void);

/* ------------------------------------------------------------------- GPP */

/* Flags for fk_gpp */
#define FK_GPP_ROOT_QUIRKS 0x1u /* semantics of the repo-root gppKer.cpp: every noflag
                                   term is summed (no |wdiff|/|delw| mask, gppKer.cpp:336)
                                   and flagOCC's sch uses I_eps[my_igp*ngpown+ig]
                                   (gppKer.cpp:139) */
#define FK_GPP_ACHSTEMP    0x2u /* also compute the static-CH remainder achstemp
                                   (gppkernel.deslippe.09.30.2014.f90:195-229) */
#define FK_GPP_HALF_SUM    0x4u /* gppsum == 1 of gppKerSeq.cpp: for column igp the
                                   sum over ig runs below igp and each term carries its
                                   conjugate pair (noflagOCC_solver :206-242 with the
                                   driver's 512-wide blocks :430-447, flagOCC_solver
                                   :90-139); not with FK_GPP_ROOT_QUIRKS or FK_GPP_ACHSTEMP */
#define FK_GPP_PHYSICS     0x8u /* the Fortran source of the kernel where it differs from
                                   the C++ ("physics" mode; the default is the C++):
                                   branch-A ssx with cden = wx**2 - wtilde**2
                                   (gppkernel.deslippe.09.30.2014.f90:302-305, C++:
                                   pow(wx,2), BGW-Kernels/gppKer.cpp:41-44), the sexcut
                                   test applied when wx < 0 (f90:319-320; the C++ test
                                   abs(wx) < 0 never fires), and asxtemp subtracted
                                   (f90:393; C++ adds, :419); not with
                                   FK_GPP_ROOT_QUIRKS or FK_GPP_HALF_SUM */
#define FK_GPP_REAL_ZERO_MASKED 0x10u /* fk_gpp_real only: a masked noflag term
                                   contributes 0 (the else left commented out at
                                   gppKer_real.cpp:371-372) instead of the value the
                                   driver's scha[ig] still holds */

/*
 * GPP self-energy sum (BGW-Kernels/gppKer.cpp:303-439).
 *
 *   inv_igp_index[ngpown], indinv[ncouls] (int32): column map
 *       igp = indinv[inv_igp_index[my_igp]], with inv_igp_index == ncouls
 *       mapped to igp = ncouls-1 (BGW-Kernels/gppKer.cpp:322-325); entries that
 *       map outside [0, ncouls) are skipped as the reference skips them (:328).
 *   wx_array[3]: the evaluation frequencies (the reference computes
 *       e_lk - e_n1kq + dw*(iw-1), clamped away from 0, :310-314).
 *   Outputs: achtemp[3], asxtemp[3]; acht_n1_loc[number_bands] and achstemp[1]
 *       may be NULL.
 */
fk_status fk_gpp(fk_ctx_t ctx, int number_bands, int nvband, int ncouls, int ngpown,
                 const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                 const fk_c128* I_eps_array, const fk_c128* wtilde_array,
                 const double* vcoul, const int* inv_igp_index, const int* indinv,
                 const double* wx_array, fk_precision precision, unsigned flags,
                 fk_c128* achtemp, fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp);

/*
 * A-priori error estimate of the mixed path (no counterpart in the reference,
 * whose sums are FP64).  fk_set_error_estimate(ctx, 1) makes every later
 * mixed-precision fk_gpp call on ctx (not the half sum) also compute, on the
 * device, an estimate of the absolute error of its outputs against exact
 * arithmetic; the cost is one more pass over aqsntemp and a few small
 * kernels (off by default).  fk_gpp_error_estimate then returns, for the last
 * fk_gpp call on ctx, max_err_est[0] for achtemp (the largest over the three
 * frequencies), [1] for asxtemp and [2] for acht_n1_loc (the largest over the
 * bands).  The model: every term w*a*x of a sum (w the band-column weight, a
 * an aqsntemp element, x the branch factor) carries a few FP32 roundings of
 * random sign, so the error is about C * 2^-24 * sqrt(sum |w a x|^2); the sum
 * of squares is bounded from the row norms of aqsntemp and the column norms
 * of the branch factors (so the estimate is at least the model's value), and
 * C = 64 lies above every ratio measured in the tests.  achstemp
 * (FK_GPP_ACHSTEMP) is not covered.  FK_ENOTSUP when the last fk_gpp call on
 * ctx failed, was FP64 or the half sum, or ran with the estimate off.
 * fk_gpp_error_estimate waits for the context's stream.
 */
fk_status fk_set_error_estimate(fk_ctx_t ctx, int enable);
fk_status fk_gpp_error_estimate(fk_ctx_t ctx, double* max_err_est /* [3] */);

/*
 * Real-valued GPP sum (gppKer_real.cpp:297-412): the same loop nest on double
 * arrays, aqsmtemp/aqsntemp [number_bands][ncouls], I_eps_array/wtilde_array
 * [ngpown][ncouls], with the index map and frequencies of fk_gpp.  As in the
 * reference, a masked noflag term leaves the value of the last unmasked term
 * at its offset in the 512-wide block (gppKer_real.cpp:341-383) in the block
 * sums; FK_GPP_REAL_ZERO_MASKED counts it as 0 instead.  Outputs: achtemp[3],
 * asxtemp[3], acht_n1_loc[number_bands] (may be NULL).  aqsntemp is read in
 * place when it is device memory on a 16-byte boundary with an even ncouls;
 * otherwise it is staged.  Flags: 0 or FK_GPP_REAL_ZERO_MASKED.
 */
fk_status fk_gpp_real(fk_ctx_t ctx, int number_bands, int nvband, int ncouls, int ngpown,
                      const double* aqsmtemp, const double* aqsntemp,
                      const double* I_eps_array, const double* wtilde_array,
                      const double* vcoul, const int* inv_igp_index, const int* indinv,
                      const double* wx_array, fk_precision precision, unsigned flags,
                      double* achtemp, double* asxtemp, double* acht_n1_loc);

/* Device scratch compiled into the library for fk_gpp_static, per GPU. */
#define FK_GPP_STATIC_SCRATCH_BYTES (64u << 20)

/*
 * fk_gpp_static: the FP64 GPP sum of fk_gpp (same arguments and results as
 * fk_gpp with precision FK_FP64) for callers that must not allocate device
 * memory: a process whose GPU memory is already owned by another allocator
 * (a framework's caching pool that has reserved the device), or a loop that
 * cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  No
 * counterpart in the reference.
 *
 * Memory: every intermediate lives in one fixed array of
 * FK_GPP_STATIC_SCRATCH_BYTES (64 MiB) of device memory per GPU, module data
 * of the library; the call makes no cudaMalloc, cudaFree or other allocating
 * call.  A request needs 48*ngpown*ncouls bytes plus its partial sums and
 * per-band rows (about 1 MB at number_bands = 512; the benchmark size
 * 512 2 32768 20 needs about 33 MB in all).  A request that does not fit
 * returns FK_ENOMEM before any work is queued.  Nothing in the scratch needs
 * to start at zero: every value a call reads was written earlier in the same
 * call.
 *
 * When the memory is taken: under lazy module loading (CUDA's default since
 * 12.2) the array is reserved on a GPU when the first fk_gpp_static call
 * there looks it up; with CUDA_MODULE_LOADING=EAGER every process that loads
 * the library reserves 64 MiB on each GPU it uses, even if it never calls
 * fk_gpp_static.
 *
 * Set-up: the first call on each device looks up the array's address
 * (cudaGetSymbolAddress), which may load that part of the library onto the
 * GPU; make the first call on a device before any stream capture.  A set-up
 * that fails returns FK_ECUDA and is tried again by the next call.  The
 * address is kept for the life of the process: calling cudaDeviceReset on a
 * device after its first fk_gpp_static call is not supported.
 *
 * Concurrency: all calls on one GPU share the one array.  Calls whose work
 * overlaps in time (from different threads, or on different streams without
 * an event between them) overwrite each other's intermediates and return
 * wrong results: serialise them.
 *
 * Arguments: stream is a cudaStream_t of the calling thread's current device
 * (NULL: the legacy default stream).  Every input array must be device memory
 * starting on a 16-byte boundary (else FK_EINVAL: staging a host array would
 * need memory).  Outputs may be device memory (the call only enqueues work)
 * or host memory (the call waits for the stream).  Errors are status codes
 * only (there is no context to hold a message).
 */
fk_status fk_gpp_static(void* stream, int number_bands, int nvband, int ncouls, int ngpown,
                        const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                        const fk_c128* I_eps_array, const fk_c128* wtilde_array,
                        const double* vcoul, const int* inv_igp_index, const int* indinv,
                        const double* wx_array, unsigned flags,
                        fk_c128* achtemp, fk_c128* asxtemp, fk_c128* acht_n1_loc, fk_c128* achstemp);

/* -------------------------------------------------------------------- FF */

/* Flags for fk_ff */
#define FK_FF_SCHDT_GEMM  0x1u /* schDt_matrix[n1][f] = sum_igp conj(aqsm[n1][igp]) *
                                  sum_ig I_epsR[f][my_igp][ig]*aqsn[n1][ig]
                                  (ffkernel.deslippe.best.f90.back1:402-418); without it
                                  schDt_matrix is zero as in FFKer_cori/ffKernel.cpp:421-422 */
#define FK_FF_PHYSICS     0x2u /* calculate_schDt_lin3 gets freqevalmin/freqevalstep as
                                  doubles; the reference C++ truncates them to int
                                  (FFKer_cori/ffKernel.cpp:10) */
#define FK_FF_SPLIT_ACHD  0x4u /* return achDtemp separately; the reference main passes
                                  asxDtemp as achDtemp_Kernel's output (ffKernel.cpp:495),
                                  so by default the sum lands in asxDtemp */

/*
 * FF full-frequency kernels (FFKer_cori/ffKernel.cpp:480-503).
 *   ekq[number_bands], dFreqGrid[nFreq], pref[nFreq] (float64),
 *   dFreqBrd[nFreq] (complex), vcoul[ncouls], inv_igp_index[ngpown], indinv[ncouls].
 *   Outputs: achsDtemp[1], asxDtemp[nfreqeval], achDtemp_cor[nfreqeval];
 *   achDtemp[nfreqeval], ach2Dtemp[nfreqeval] and schDt_matrix[number_bands][nFreq]
 *   may be NULL.  Requires nFreq >= 2 and ngpown <= ncouls (ffKernel.cpp:320).
 */
fk_status fk_ff(fk_ctx_t ctx, int number_bands, int nvband, int ncouls, int ngpown,
                int nFreq, int nfreqeval,
                const fk_c128* aqsmtemp, const fk_c128* aqsntemp,
                const fk_c128* I_epsR_array, const fk_c128* I_epsA_array,
                const double* vcoul, const int* inv_igp_index, const int* indinv,
                const double* ekq, const double* dFreqGrid, const fk_c128* dFreqBrd,
                const double* pref, double pref_zb, double freqevalmin, double freqevalstep,
                double occ, fk_precision precision, unsigned flags,
                fk_c128* achsDtemp, fk_c128* asxDtemp, fk_c128* achDtemp,
                fk_c128* achDtemp_cor, fk_c128* ach2Dtemp, fk_c128* schDt_matrix);

/* ---------------------------------------------------------------- serving */

/*
 * A GPP request server: a worker thread on one GPU takes requests of any
 * (number_bands, ncouls, ngpown) as they are submitted, admits them while its
 * device memory budget and active slots allow, and runs them in steps.  Each
 * step is one replay of a captured CUDA graph whose kernels (index map and
 * weights, prep, one persistent tcgen05 contraction over every request's
 * units, reductions) read a table of the step's requests; a large request
 * advances part of its k-range per step, a small one finishes in one step.
 * A request's arithmetic (its k-slices and summation order) depends only on
 * its own shape, so its result is the same alone and in any mix.  Mixed
 * precision (FK_MIXED semantics of fk_gpp).  No counterpart in the reference
 * (which runs one evaluation per process).
 */
typedef struct fk_server* fk_server_t;

typedef struct {
    size_t hbm_bytes; /* device memory for resident arrays and requests (one block) */
    int max_active;   /* requests on the GPU at once, 1..64 */
    int step_stages;  /* contraction work per step, in 32-wide k-stages per SM (0: 96) */
} fk_server_config;

typedef struct {
    int number_bands, nvband, ncouls, ngpown;
    const fk_c128* aqsmtemp;     /* [number_bands][ncouls], host or device */
    const fk_c128* aqsntemp;     /* [number_bands][ncouls], host or device */
    const fk_c128* I_eps_array;  /* [ngpown][ncouls], host or device; NULL: eps_key */
    const fk_c128* wtilde_array; /* [ngpown][ncouls], host or device; NULL: wtilde_key */
    unsigned long long eps_key, wtilde_key; /* fk_server_resident_put keys */
    const double* vcoul;         /* [ncouls] */
    const int* inv_igp_index;    /* [ngpown] */
    const int* indinv;           /* [ncouls] */
    const double* wx_array;      /* [3] */
    unsigned flags;              /* 0 or FK_GPP_ROOT_QUIRKS */
    fk_c128* achtemp;            /* [3] outputs, host or device, written at completion */
    fk_c128* asxtemp;            /* [3] */
    fk_c128* acht_n1_loc;        /* [number_bands] or NULL */
} fk_gpp_request;

typedef struct {
    unsigned long long submitted, completed, steps;
    double p50_s, p99_s, mean_s; /* submit-to-completion latency of completed requests */
    double terms_per_s;          /* completed terms / (last completion - first submission) */
    double mean_active;          /* requests per step */
    int peak_active;
    size_t hbm_peak_bytes;       /* most of the budget in use at once */
} fk_server_info;

fk_status fk_server_create(int device, const fk_server_config* cfg, fk_server_t* out);
/* Finishes every submitted request, then stops the worker and frees the GPU memory. */
fk_status fk_server_destroy(fk_server_t srv);
/* Copies an array (host or device) to the server's memory under `key`, for
 * requests that name it instead of passing I_eps_array / wtilde_array.
 * FK_EINVAL if the key is in use, FK_EBUSY if it was evicted but running
 * requests still read it. */
fk_status fk_server_resident_put(fk_server_t srv, unsigned long long key, const void* data, size_t bytes);
/* Frees a resident array once no admitted or waiting request uses it. */
fk_status fk_server_resident_evict(fk_server_t srv, unsigned long long key);
/* Queues a request (the input arrays must stay valid until it completes).
 * FK_ENOMEM: the request can never fit in the server's memory budget. */
fk_status fk_server_submit(fk_server_t srv, const fk_gpp_request* req, unsigned long long* ticket);
/* Waits for a request (timeout_s < 0: no limit; FK_EBUSY on timeout) and
 * returns its status; latency_s (may be NULL) gets submit-to-completion time.
 * The ticket is consumed when the request has completed. */
fk_status fk_server_wait(fk_server_t srv, unsigned long long ticket, double timeout_s, double* latency_s);
/* Cancels a request that is still waiting for admission: it leaves the queue
 * without running (its outputs are not written), its references to resident
 * arrays are dropped, and fk_server_wait on its ticket returns FK_ECANCELED
 * at once.  A request already admitted runs to completion: FK_EBUSY (wait for
 * it as usual).  FK_EINVAL for an unknown ticket. */
fk_status fk_server_cancel(fk_server_t srv, unsigned long long ticket);
/* The server's counters since it was created: requests submitted and
 * completed, steps run, latency percentiles, throughput, requests per step
 * and the peak of its memory budget in use (fk_server_info). */
fk_status fk_server_stats(fk_server_t srv, fk_server_info* out);
/* Autotunes the plan of one request shape (while the server is idle, else
 * FK_EBUSY): runs the shape with synthetic inputs through the server's steps
 * under each candidate k-split (the default plan's, and k-slices of 16, 32,
 * ..., 256 k-stages) and keeps the fastest for later requests of that shape.
 * chosen_ks (may be NULL) gets its k-slice count. */
fk_status fk_server_tune(fk_server_t srv, int number_bands, int nvband, int ncouls, int ngpown, unsigned flags,
                         int* chosen_ks);

/* ------------------------------------------------------------ measurement */

/* Kernel-level timing of the most recent fk_gpp/fk_ff call, measured with
 * CUDA events on the launch stream when enabled with fk_set_profiling(ctx,1).
 * Phases: 0 = input staging, 1 = prep / branch kernel, 2 = contraction
 * (the dominant kernel), 3 = reduction + epilogue.  Milliseconds. */
fk_status fk_set_profiling(fk_ctx_t ctx, int enable);
fk_status fk_last_timings(fk_ctx_t ctx, float ms[4]);
/* Number of kernels the most recent call launched. */
int fk_last_launches(fk_ctx_t ctx);
/* Device time of the dominant kernel alone in the most recent profiled call:
 * the milliseconds summed over its launches (CUDA events recorded on the
 * launch stream right before and after each launch) and their count. */
fk_status fk_last_kernel_time(fk_ctx_t ctx, float* ms, int* launches);
/* Bytes the most recent fk_gpp / fk_gpp_real / fk_ff call moved over the host
 * link: its host inputs copied to the device (a host array is sent in full,
 * except where the call reads a part of it: the igp columns of aqsmtemp,
 * the frequency planes of I_epsR/I_epsA the request reads) and its outputs
 * copied to host arrays.  Device arrays move nothing. */
fk_status fk_last_transfer(fk_ctx_t ctx, unsigned long long* h2d, unsigned long long* d2h);

/* ------------------------------------------------------------ diagnostics */

/* Bound, in SM clock cycles, of every wait between the warp roles of the
 * tensor-core kernels (default 4e9, about 2 s at 2 GHz; a negative value
 * restores the default).  A wait that runs out makes its kernel record a
 * code in the context's error word, let the copies and MMAs it has already
 * started finish, and return; the call then returns FK_ETIMEOUT and clears
 * the error word, so the context stays usable.  Lowering the bound is a test
 * hook: with 0 cycles any wait not satisfied on its first test gives up.  No
 * counterpart in the reference (its loops never wait on another part of the
 * GPU). */
fk_status fk_set_wait_limit(fk_ctx_t ctx, long long cycles);
/* Runs a one-warp kernel that waits, through the same bounded wait, on a
 * barrier that nothing arrives on, giving up after `cycles` (0 .. 4e9)
 * cycles: returns FK_ETIMEOUT through the same error-word path as a
 * timed-out contraction and leaves the context usable.  No counterpart in the
 * reference. */
fk_status fk_selftest_timeout(fk_ctx_t ctx, long long cycles);
/* Decodes a device error word of the tensor-core kernels: FK_OK for 0, else
 * FK_ETIMEOUT, with a description naming each kind of wait that gave up
 * written to msg (msg_len bytes, NUL-terminated; msg may be NULL).  Calls
 * that see a nonzero word return this status and keep this description as
 * their fk_last_error.  No GPU needed.  No counterpart in the reference. */
fk_status fk_wait_error_status(int word, char* msg, size_t msg_len);

#ifdef __cplusplus
}
#endif
#endif /* FK_ABI_H */
