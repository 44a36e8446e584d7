// fk_gemm.cuh -- complex "band x G" contraction engines with a fused,
// weighted row reduction.
//
// Both hot paths reduce to the same shape.  For a batch b (FF frequency
// plane, or the single GPP plane), band rows m and columns n:
//
//     S[m][n]  = sum_k  A[m][k] * B[b][n][k]                 (complex, K = ig)
//     P[m][g] += sum_n  w(m, n) * S[m][n]   for the groups g of column n
//
//   GPP: A = aqsntemp, B = D[(my_igp,iw)][ig] = mask * delw * I_eps (built by
//        the prep kernel), w = 0.5 * vcoul[igp] * conj(aqsmtemp[m][igp]),
//        g = iw.  (BGW-Kernels/gppKer.cpp:387-424 with the n1-independent
//        factor hoisted out of the n1 loop.)
//   FF:  A = aqsntemp, B = I_eps[f], t = conj(aqsmtemp[m][igp]) * S,
//        g0 += vcoul[igp] * t, g1 += t  (FFKer_cori/ffKernel.cpp:107-131,
//        ffkernel.deslippe.best.f90.back1:402-418).
//   STAT: A = aqsntemp, B = I_eps, w = -0.5 * vcoul[igp] * conj(aqsm[m][igp])
//        (gppkernel.deslippe.09.30.2014.f90:213-228).
//
// Each CTA owns a (m-tile, n-tile, k-slice, batch) block and writes one
// partial P per (slot, m, g) with slot = (batch*KS + ks)*NT + nt; a separate
// kernel sums the slots in a fixed order, so results are bit-reproducible.
#pragma once
#include "fk_common.cuh"

namespace fk {

enum EpiKind { EPI_GPP = 0, EPI_FF = 1, EPI_STAT = 2 };

struct ContractArgs {
    const double2* A;       // row m at A + (m0 + m) * lda
    long lda;
    int m0, M;              // rows [m0, m0+M) of A; P rows are indexed m in [0, M)
    const void* B;          // double2 (FP64 engine, FF in mixed) or float2 (GPP mixed)
    long ldb;               // row stride of B
    long bstride;           // batch stride of B (elements)
    int N, K;
    int KS;                 // k-slices
    int kchunk;             // k per slice (multiple of 16)
    int batches;
    const int* batch_plane; // batch index -> plane index in B (nullable = identity)
    // epilogue
    const double2* aqsm;    // [nb][ncouls]
    long ldm;
    const double* vcoul;
    const int* igp;         // column h -> igp (-1: skipped); indexes vcoul
    const int* acol;        // column h -> column of the aqsm array passed (igp, or h when compacted)
    double wscale;
    int G;                  // groups per row in P
    double2* P;             // [slots][M][G]
};

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// Weight of column n of row m and the group it feeds (GPP / STAT).
FK_DEV double2 epi_weight(const ContractArgs& a, int m, int h) {
    int g = a.igp[h];
    if (g < 0) return make_double2(0.0, 0.0);
    double2 am = a.aqsm[(long)(a.m0 + m) * a.ldm + a.acol[h]];
    double s = a.wscale * a.vcoul[g];
    return make_double2(am.x * s, -am.y * s);
}

// Per-thread accumulation of one S element into the row's group sums gs[G].
template <int EPI>
FK_DEV void epi_accum(const ContractArgs& a, int m, int n, double2 c, double2* gs) {
    if (m >= a.M || n >= a.N) return;
    if (EPI == EPI_GPP) {
        int g = n % 3;
        gs[g] = cadd(gs[g], cmul(epi_weight(a, m, n / 3), c));
    } else if (EPI == EPI_FF) {
        int ig = a.igp[n];
        if (ig < 0) return;
        double2 am = a.aqsm[(long)(a.m0 + m) * a.ldm + a.acol[n]];
        double2 t = cmul(cconj(am), c);
        gs[0] = cadd(gs[0], cscale(t, a.vcoul[ig]));
        gs[1] = cadd(gs[1], t);
    } else {
        gs[0] = cadd(gs[0], cmul(epi_weight(a, m, n), c));
    }
}

// Fixed-order sum over the SLOTS per-thread partials of each (row, group)
// held in smem part[(row*SLOTS + slot)*G + g], written to P.
template <int BM, int SLOTS>
FK_DEV void epi_reduce_store(const ContractArgs& a, const double2* part, int mt, int slot) {
    const int G = a.G;
    for (int idx = threadIdx.x; idx < BM * G; idx += blockDim.x) {
        int ml = idx / G, g = idx % G;
        int m = mt * BM + ml;
        if (m >= a.M) continue;
        double2 s = make_double2(0.0, 0.0);
        for (int j = 0; j < SLOTS; ++j) s = cadd(s, part[(ml * SLOTS + j) * G + g]);
        a.P[((long)slot * a.M + m) * G + g] = s;
    }
}
constexpr int GMAX = 3;

// ============================================================ FP64 (DMMA)
// CTA tile 64 x 32 complex, 4 warps (2 x 2), warp tile 32 x 16, k-step 16.
// Each 8x8x4 block uses mma.sync.m8n8k4.f64 four times:
//   Sr += Ar*Br + Ai*(-Bi),  Si += Ar*Bi + Ai*Br.
namespace d64 {
constexpr int BM = 64, BN = 32, BK = 16, PAD = 4, LDS = BK + PAD, STAGES = 3, THREADS = 128;
constexpr size_t SMEM = (size_t)STAGES * (BM + BN) * LDS * sizeof(double2);
static_assert(SMEM >= (size_t)BM * 8 * GMAX * sizeof(double2), "reduction partials must fit in the pipeline buffers");

FK_DEV void dmma(double& c0, double& c1, double a, double b) {
    // not volatile: the scheduler may interleave independent accumulators
    asm("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
        : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
}
FK_DEV void cp_async16(void* smem, const void* gmem, bool pred) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    int n = pred ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
FK_DEV void cp_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N> FK_DEV void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <int EPI>
__global__ void __launch_bounds__(THREADS) contract_kernel(ContractArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2* As = reinterpret_cast<double2*>(smem_raw);
    double2* Bs = As + STAGES * BM * LDS;
    const int NT = ceil_div(a.N, BN);
    const int mt = blockIdx.x, nt = blockIdx.y % NT;
    const int ks = (blockIdx.y / NT) % a.KS, batch = blockIdx.y / (NT * a.KS);
    const int plane = a.batch_plane ? a.batch_plane[batch] : batch;
    const double2* B = reinterpret_cast<const double2*>(a.B) + (long)plane * a.bstride;
    const int k0 = ks * a.kchunk;
    const int k1 = min(a.K, k0 + a.kchunk);
    const int nk = k1 > k0 ? ceil_div(k1 - k0, BK) : 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;

    auto load_stage = [&](int stage, int kt) {
        const int kb = k0 + kt * BK;
        double2* as = As + stage * BM * LDS;
        double2* bs = Bs + stage * BN * LDS;
        for (int i = tid; i < BM * BK; i += THREADS) {
            int r = i / BK, c = i % BK;
            int m = mt * BM + r, k = kb + c;
            bool ok = m < a.M && k < k1;
            const double2* src = ok ? a.A + (long)(a.m0 + m) * a.lda + k : a.A;
            cp_async16(&as[r * LDS + c], src, ok);
        }
        for (int i = tid; i < BN * BK; i += THREADS) {
            int r = i / BK, c = i % BK;
            int n = nt * BN + r, k = kb + c;
            bool ok = n < a.N && k < k1;
            const double2* src = ok ? B + (long)n * a.ldb + k : B;
            cp_async16(&bs[r * LDS + c], src, ok);
        }
    };

    double cr[4][2][2], ci[4][2][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) cr[i][j][0] = cr[i][j][1] = ci[i][j][0] = ci[i][j][1] = 0.0;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nk) load_stage(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < nk; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        if (kt + STAGES - 1 < nk) load_stage((kt + STAGES - 1) % STAGES, kt + STAGES - 1);
        cp_commit();
        const double2* as = As + (kt % STAGES) * BM * LDS;
        const double2* bs = Bs + (kt % STAGES) * BN * LDS;
#pragma unroll
        for (int kk = 0; kk < BK; kk += 4) {
            double2 af[4], bf[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) af[i] = as[(wm * 32 + i * 8 + (lane >> 2)) * LDS + kk + (lane & 3)];
#pragma unroll
            for (int j = 0; j < 2; ++j) bf[j] = bs[(wn * 16 + j * 8 + (lane >> 2)) * LDS + kk + (lane & 3)];
            double nbi[2] = {-bf[0].y, -bf[1].y};
            // four passes over the 8 accumulator tiles: consecutive updates of
            // one accumulator are 8 independent DMMAs apart
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) dmma(cr[i][j][0], cr[i][j][1], af[i].x, bf[j].x);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) dmma(ci[i][j][0], ci[i][j][1], af[i].x, bf[j].y);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) dmma(cr[i][j][0], cr[i][j][1], af[i].y, nbi[j]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) dmma(ci[i][j][0], ci[i][j][1], af[i].y, bf[j].x);
        }
    }
    cp_wait<0>();
    __syncthreads();

    // epilogue: weighted group sums per thread -> smem -> fixed-order row sums
    double2* part = reinterpret_cast<double2*>(smem_raw);  // [BM][8 slots][G]
    const int slot = wn * 4 + (lane & 3);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int ml = wm * 32 + i * 8 + (lane >> 2);
        double2 gs[GMAX] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                int nl = wn * 16 + j * 8 + (lane & 3) * 2 + e;
                epi_accum<EPI>(a, mt * BM + ml, nt * BN + nl, make_double2(cr[i][j][e], ci[i][j][e]), gs);
            }
        for (int g = 0; g < a.G; ++g) part[(ml * 8 + slot) * a.G + g] = gs[g];
    }
    __syncthreads();
    epi_reduce_store<BM, 8>(a, part, mt, (batch * a.KS + ks) * NT + nt);
}
}  // namespace d64

// ================================================== FP32 SIMT (mixed, v1)
// CTA tile 64 x 64 complex, 256 threads, 4 x 4 complex per thread, k-step
// 16.  FP64 inputs are rounded to FP32 with the integer conversion; products
// accumulate in FP32 for one 16-value k-step, then into a float-float (hi, lo)
// accumulator (TwoSum), so the FP32 rounding error does not grow with K.
namespace f32 {
constexpr int BM = 64, BN = 64, BK = 16, THREADS = 256, FLUSH_TILES = 1;
constexpr int LDA = BM + 1, LDB = BN + 1;
constexpr size_t SMEM_PIPE = (size_t)2 * BK * (LDA + LDB) * sizeof(float2);
constexpr size_t SMEM_RED = (size_t)BM * 16 * GMAX * sizeof(double2);
constexpr size_t SMEM = SMEM_PIPE > SMEM_RED ? SMEM_PIPE : SMEM_RED;

template <class TB> FK_DEV float2 to_f2(TB v);
template <> FK_DEV float2 to_f2<double2>(double2 v) { return c64_to_f32(v); }
template <> FK_DEV float2 to_f2<float2>(float2 v) { return v; }

template <int EPI, class TB>
__global__ void __launch_bounds__(THREADS) contract_kernel(ContractArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* As = reinterpret_cast<float2*>(smem_raw);  // [2][BK][LDA]
    float2* Bs = As + 2 * BK * LDA;                     // [2][BK][LDB]
    const int NT = ceil_div(a.N, BN);
    const int mt = blockIdx.x, nt = blockIdx.y % NT;
    const int ks = (blockIdx.y / NT) % a.KS, batch = blockIdx.y / (NT * a.KS);
    const int plane = a.batch_plane ? a.batch_plane[batch] : batch;
    const TB* B = reinterpret_cast<const TB*>(a.B) + (long)plane * a.bstride;
    const int k0 = ks * a.kchunk;
    const int k1 = min(a.K, k0 + a.kchunk);
    const int nk = k1 > k0 ? ceil_div(k1 - k0, BK) : 0;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

    // register staging: 4 A and 4 B complex values per thread per k-step
    float2 ra[4], rb[4];
    auto gload = [&](int kt) {
        const int kb = k0 + kt * BK;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int idx = tid + i * THREADS;
            int r = idx / BK, c = idx % BK;
            int m = mt * BM + r, k = kb + c;
            ra[i] = (m < a.M && k < k1) ? c64_to_f32(a.A[(long)(a.m0 + m) * a.lda + k]) : make_float2(0.f, 0.f);
            int n = nt * BN + r;
            rb[i] = (n < a.N && k < k1) ? to_f2<TB>(B[(long)n * a.ldb + k]) : make_float2(0.f, 0.f);
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int idx = tid + i * THREADS;
            int r = idx / BK, c = idx % BK;
            As[(buf * BK + c) * LDA + r] = ra[i];
            Bs[(buf * BK + c) * LDB + r] = rb[i];
        }
    };

    float2 acc[4][4];
    ff32 hr[4][4], hi_[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            acc[i][j] = make_float2(0.f, 0.f);
            hr[i][j] = {0.f, 0.f};
            hi_[i][j] = {0.f, 0.f};
        }

    if (nk > 0) { gload(0); sstore(0); }
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int buf = kt & 1;
        if (kt + 1 < nk) gload(kt + 1);
        const float2* as = As + buf * BK * LDA;
        const float2* bs = Bs + buf * BK * LDB;
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            float2 av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = as[k * LDA + ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = bs[k * LDB + tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) cfmaf(acc[i][j], av[i], bv[j]);
        }
        if ((kt + 1) % FLUSH_TILES == 0 || kt + 1 == nk) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    ff_add(hr[i][j], acc[i][j].x);
                    ff_add(hi_[i][j], acc[i][j].y);
                    acc[i][j] = make_float2(0.f, 0.f);
                }
        }
        if (kt + 1 < nk) sstore(buf ^ 1);
        __syncthreads();
    }

    double2* part = reinterpret_cast<double2*>(smem_raw);  // [BM][16 slots][G]
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int ml = ty + 16 * i;
        double2 gs[GMAX] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int nl = tx + 16 * j;
            double2 c = make_double2((double)hr[i][j].hi + (double)hr[i][j].lo,
                                     (double)hi_[i][j].hi + (double)hi_[i][j].lo);
            epi_accum<EPI>(a, mt * BM + ml, nt * BN + nl, c, gs);
        }
        for (int g = 0; g < a.G; ++g) part[(ml * 16 + tx) * a.G + g] = gs[g];
    }
    __syncthreads();
    epi_reduce_store<BM, 16>(a, part, mt, (batch * a.KS + ks) * NT + nt);
}
}  // namespace f32

}  // namespace fk
