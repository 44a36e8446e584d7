// fk_tc_contract.cuh -- tensor-core (tcgen05) form of the band x G
// contraction with the fused weighted row reduction of fk_gemm.cuh.
//
//   S[m][n] = sum_k A[m][k] * B[n][k]        (complex; A = aqsntemp, FP64 in HBM)
//   P[slot][m][g] = sum_n w(m, n) * S[m][n]  (FP64 partials, fixed order)
//
// Precision scheme (mixed path): every FP64 operand is rounded to FP32 with
// integer instructions and split exactly into three BF16 pieces
// x = x_h + x_m + x_l.  A complex product uses the six piece products whose
// order is at least 2^-16 (hh, hm, mh, hl, lh, mm).  Tensor-core FP32
// accumulation truncates, so its error grows with the number of MMA results
// added into one accumulator: the hh products go to their own (re, im)
// accumulators, which receive 2 MMA results per 16 k-values, the five
// smaller piece products to separate correction accumulators (2^-8 smaller,
// so their truncation is negligible), and all four are drained into the
// FP64 epilogue every CHUNK_STAGES*32 k-values.
//
// CTA organisation (one persistent CTA per SM):
//   warp 0      TMEM allocation, MMA issue (one lane)
//   warp 1      copies: pre-split B tiles (and FF's pre-split A tiles) by bulk
//               copy, GPP's FP64 A rows by tensor-map TMA (one lane issues)
//   GPP, 448 threads: warps 4..7 epilogue (TMEM lanes 0..127 = tile rows,
//               weighted sums), warps 2,3,8..13 converters (FP64 A rows ->
//               swizzled BF16 pieces in smem); two operand stages
//   FF, 576 threads: warps 2..17 epilogue, one per (lane quarter, 16-column
//               group), weights in registers; three operand stages
// Work units are (m-tile, n-tile, k-slice, batch); CTA i takes units
// i, i + gridDim.x, ...  Every wait is bounded; on timeout the CTA records
// an error code and unwinds without further waits of unbounded length.
#pragma once
#include <cuda.h>

#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fk_gemm.cuh"
#include "fk_tc.cuh"

namespace fk {
namespace tcx {

constexpr int BM = 128;
constexpr int BK = 32;            // complex k-values per stage (64 B of bf16 per row)
constexpr int NSPLIT = 3;         // bf16 pieces per real value
constexpr int NSUB = 2 * NSPLIT;  // sub-tiles per operand: re h/m/l, im h/m/l
constexpr int THREADS = 448;     // GPP: MMA, producer, 8 converter warps, 4 epilogue warps
constexpr int THREADS_FF = 608;  // FF: MMA, producer, 16 epilogue warps, the -B_im warp
// FF (A operand pre-split, no converter work): the 16 warps 2..17 all drain
// TMEM, four per lane quarter, each over one 16-column group with its own
// weights in registers and its own partial-sum slot; GPP: warps 4..7, one per
// quarter, all columns.
constexpr int FF_EPI_WARPS = 4;
constexpr int NCONV = 8;          // converter warps
// Default bound of every wait on another role of the CTA (SM clock cycles,
// ~2 s at 2 GHz); a launch may pass a different one (TcArgs::wait_limit).
constexpr long long WAIT_LIMIT = 4000000000LL;
// Bound of the waits at the end of a CTA for its own asynchronous work (bulk
// copies still landing, issued MMAs): these always run to completion, so they
// keep the default bound whatever limit the launch passes.
constexpr long long DRAIN_LIMIT = 4000000000LL;

template <int BN, bool WSMEM = false, bool PAIR = false, bool APRE = WSMEM>
struct Cfg {
    static_assert(BN == 64, "the accumulator buffers fill the 512 TMEM columns at BN = 64");
    // Operand stages: FF three (its epilogue keeps the per-unit weights in
    // registers, so shared memory holds operands only), GPP two.  GPP: a 64 KB staging buffer receives
    // FP64 A rows by TMA in two halves of BK/2 k-values, so that one half is in
    // flight while the converters read the other.  (Two full stagings do not fit
    // beside two operand stages; one operand stage with two stagings measured
    // slower: the converters then wait for each stage's MMAs.)
    static constexpr int CHUNK_STAGES = 1;  // k-values per TMEM accumulation = 32
    // FF operands are FP16 hi/lo pieces (two per real value; every row scaled by
    // a power of two that brings its largest magnitude just below 2^15, three
    // piece products per complex product: hh, hl, lh), GPP operands BF16
    // hi/mid/lo pieces (three per value, six piece products)
    static constexpr bool F16 = WSMEM;
    static constexpr int NPIECE = F16 ? 2 : NSPLIT;
    static constexpr int ASUB = 2 * NPIECE;  // A sub-tiles: the re pieces, then the im pieces
    // (GPP with a pre-split A image: no FP64 staging, so three operand stages)
    static constexpr int STAGES = WSMEM ? (F16 ? 4 : 3) : (APRE ? 3 : 2);
    static constexpr uint32_t A_BYTES = ASUB * BM * 64;
    // The pre-split B image, one k-stage of an n-tile: GPP six sub-tiles (re h,
    // im h, re m, im m, re l, im l); FF four (re, im of each piece h, l).  FF's
    // one-accumulator layout also needs -B_im: the -B_im warp writes it into
    // the stage after the copy lands (IMGN).
    static constexpr bool IMGN = WSMEM;
    static constexpr uint32_t B_BYTES = (IMGN ? 2 * NPIECE : NSUB) * BN * 64;
    // SL (FF): one accumulator D = A_re x [B_re|B_im] + A_im x [-B_im|B_re] =
    // [S_re | S_im], 2*BN columns, in four buffers; otherwise (GPP) two
    // accumulators X = A_re x [B_re|B_im], Y = A_im x [B_re|B_im] in two buffers.
    static constexpr bool SL = WSMEM;
    // B in one CTA's stage, per piece: GPP single CTA [B_re; B_im], GPP pair the
    // even CTA's B_re and the odd CTA's B_im; FF single CTA the image's three
    // sub-tiles [-B_im; B_re; B_im] ([B_re; B_im] from the second, [-B_im; B_re]
    // from the first), FF pair the even CTA's [B_re; -B_im], the odd CTA's [B_im; B_re]
    static constexpr uint32_t B_SMEM = (SL ? (PAIR ? 2 : 3) : (PAIR ? 1 : 2)) * NPIECE * BN * 64;
    static constexpr uint32_t STAGE_BYTES = A_BYTES + B_SMEM;
    // B bytes the copies of one stage bring (FF single CTA: [re; im] of each
    // piece, the -B_im warp writes the third sub-tile)
    static constexpr uint32_t B_COPY = IMGN ? 2 * NPIECE * BN * 64 : B_SMEM;
    static constexpr int NBUF = SL ? 4 : 2;
    // SL: the accumulator buffers are handed over in groups of two (consecutive
    // chunks), one full and one empty barrier per group: the MMA issuer waits,
    // fences and commits once per group, the epilogue drains a group in one pass
    static constexpr int GRP = SL ? 2 : 1;
    static constexpr int NSLOT = NBUF / GRP;
    static constexpr uint32_t ACC_COLS = SL ? 2 * BN : 4 * BN;
    static constexpr uint32_t TMEM_COLS = NBUF * ACC_COLS;
    static constexpr uint32_t W_BYTES = 0u;
    static constexpr uint32_t F64_BYTES = APRE ? 0u : (uint32_t)(BM * BK * sizeof(double2));
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + W_BYTES + F64_BYTES + 1024 + 512;
};

struct TcArgs {
    CUtensorMap amap;     // GPP: A (FP64 complex rows) as a 2-D FP64 tensor, box 32 x BM (half a stage), zero fill
    ContractArgs c;       // shapes, partial buffer (same meaning as fk_gemm.cuh)
    const uint8_t* Bimg;  // pre-split B tiles: [plane][nt][kstage][NSUB][BN rows][64 B]
    const uint8_t* Aimg;  // pre-split A tiles [mt][kstage][ASUB][BM rows][64 B] (APRE kernels only)
    const float* ascale;  // FF: 2^-k of each A image row (the row was scaled by 2^k before its split)
    const float* bscale;  // FF: 2^-k of each B row, [batch][N]
    const float2* W1;     // epilogue weights, column-major [h][ldw] (GPP: 0.5 vcoul conj(aqsm); FF: vcoul conj(aqsm))
    const float2* W2;     // FF only: conj(aqsm), [h][ldw]
    int ldw;              // = M (rows are contiguous, so a warp's 32 rows load coalesced)
    const float* vcol;    // FF: vcoul[igp(n)] per column n (FP32)
    int gpp_cols;         // GPP: igp columns per n-tile (21: complete (igp, iw) triples)
    int kstages_total;    // k-stages per (plane, nt) in Bimg = ceil(K/32)
    int MT, NT, units;
    int mt0;              // first m-tile of the launch (its units cover m-tiles mt0 .. mt0+MT-1)
    int* err;             // device error word (nonzero: a wait timed out)
    long long wait_limit; // bound of the waits between roles, cycles (0 is allowed: any wait that
                          // is not satisfied on its first test gives up)
    int chunk_stages;     // k-stages accumulated in TMEM between drains (0: 1)
    int ff_no_rs;         // FF: the unweighted sum (partial 1) is not needed; only the vcoul-weighted one
};

// Split an FP32 value into three BF16 pieces (exact: 8+8+8 significand bits).
__device__ __forceinline__ void split3(float f, uint16_t& h, uint16_t& m, uint16_t& l) {
    const uint32_t fb = __float_as_uint(f);
    const uint32_t hb = fb & 0xFFFF0000u;
    const float r1 = f - __uint_as_float(hb);
    const uint32_t mb = __float_as_uint(r1) & 0xFFFF0000u;
    const float r2 = r1 - __uint_as_float(mb);
    h = (uint16_t)(hb >> 16);
    m = (uint16_t)(mb >> 16);
    l = (uint16_t)(__float_as_uint(r2) >> 16);  // r2 has at most 8 significant bits: exact
}

// Image element writer shared by the prep/conversion kernels: complex value
// (re, im) of row `row` (within its ROWS-row tile) at k-value k of a tile
// column whose k-stages are ROWS*NSUB*64 bytes apart.  A tiles keep the
// sub-tile order re h, m, l, im h, m, l (each one is an MMA A operand);
// B tiles (PAIRED) put re and im of a piece next to each other -- re h, im h,
// re m, im m, re l, im l -- so that [B_re | B_im] of a piece is one 2*ROWS-row
// operand.
template <int ROWS, bool PAIRED = false>
__device__ __forceinline__ void img_store(uint8_t* img_tile, int row, int k, float re, float im) {
    uint8_t* st = img_tile + (long)(k / BK) * (ROWS * NSUB * 64);
    const uint32_t off = tc::sw64_offset(row, k % BK);
    constexpr int RE0 = 0, RS = PAIRED ? 2 : 1, IM0 = PAIRED ? 1 : 3;
    uint16_t h, m, l;
    split3(re, h, m, l);
    *(uint16_t*)(st + (RE0 + 0 * RS) * ROWS * 64 + off) = h;
    *(uint16_t*)(st + (RE0 + 1 * RS) * ROWS * 64 + off) = m;
    *(uint16_t*)(st + (RE0 + 2 * RS) * ROWS * 64 + off) = l;
    split3(im, h, m, l);
    *(uint16_t*)(st + (IM0 + 0 * RS) * ROWS * 64 + off) = h;
    *(uint16_t*)(st + (IM0 + 1 * RS) * ROWS * 64 + off) = m;
    *(uint16_t*)(st + (IM0 + 2 * RS) * ROWS * 64 + off) = l;
}
template <int BN>
__device__ __forceinline__ void bimg_store(uint8_t* img_nt, int kstage_total_unused, int n_in_tile, int k,
                                           float re, float im) {
    (void)kstage_total_unused;
    img_store<BN, true>(img_nt, n_in_tile, k, re, im);
}

// One half of a paired B element: the three pieces of its real (part 0) or
// imaginary (part 1) component, for writers that produce the two halves
// separately.
template <int BN>
__device__ __forceinline__ void bimg_store_part(uint8_t* img_nt, int n_in_tile, int k, int part, float v) {
    uint8_t* st = img_nt + (long)(k / BK) * (BN * NSUB * 64);
    const uint32_t off = tc::sw64_offset(n_in_tile, k % BK);
    uint16_t h, m, l;
    split3(v, h, m, l);
    *(uint16_t*)(st + (part + 0) * BN * 64 + off) = h;
    *(uint16_t*)(st + (part + 2) * BN * 64 + off) = m;
    *(uint16_t*)(st + (part + 4) * BN * 64 + off) = l;
}

// Where a kernel's units come from.  OneReq: every unit belongs to the one
// request in the launch parameters.  TableReqs: units of several requests,
// laid end to end; request r owns global units [ustart[r], ustart[r+1]) and
// they are its local units ulocal0[r], ulocal0[r]+1, ... (a step of a served
// request may cover only part of its k-slices).  Each warp role walks units
// in increasing order, so a cursor finds the request without a search.
constexpr int TC_MAXREQ = 64;
struct TcTable {
    TcArgs req[TC_MAXREQ];
    int nreq, units;
    int ustart[TC_MAXREQ + 1];
    int ulocal0[TC_MAXREQ];
};
struct OneReq {
    const TcArgs& t;
    __device__ int units() const { return t.units; }
    __device__ const TcArgs& at(int u, int& lu) {
        lu = u;
        return t;
    }
    static constexpr bool kTable = false;
};
struct TableReqs {
    const TcTable* tab;
    int r;
    __device__ int units() const { return tab->units; }
    __device__ const TcArgs& at(int u, int& lu) {
        while (r + 1 < tab->nreq && u >= tab->ustart[r + 1]) ++r;
        lu = tab->ulocal0[r] + (u - tab->ustart[r]);
        return tab->req[r];
    }
    static constexpr bool kTable = true;
};

// PAIR: a cluster of two CTAs computes M = 256 rows per unit (128 per CTA)
// with MMAs the even CTA issues for both (see fk_tc.cuh): each CTA loads its
// own A rows and its half of B; the odd CTA's "stage landed" and "accumulator
// drained" signals go to the even CTA's barriers (a relay thread and remote
// arrivals); the MMA commits reach both CTAs' barriers.
// Units of several batches (FF frequency planes) with their own row-tile
// ranges in one launch: plane r owns units [u0[r], u0[r+1]) over row tiles
// [mt0[r], mt0[r] + MT[r]); its B image and partial sums sit islab / pslab
// bytes / elements after the previous plane's.  Each warp role keeps a copy
// of the current plane's arguments, updated when it moves to the next plane.
constexpr int TC_MAXPL = 64;
struct PlaneTab {
    int n;
    int u0[TC_MAXPL + 1], mt0[TC_MAXPL], MT[TC_MAXPL];
    long islab, pslab;
};
struct PlaneSeq {
    const TcArgs* base;
    const PlaneTab* tab;
    TcArgs cur;
    int r;
    __device__ int units() const { return tab->u0[tab->n]; }
    __device__ const TcArgs& at(int u, int& lu) {
        if (r < 0 || u >= tab->u0[r + 1]) {
            if (r < 0) r = 0;
            while (r + 1 < tab->n && u >= tab->u0[r + 1]) ++r;
            cur = *base;
            cur.mt0 = tab->mt0[r];
            cur.MT = tab->MT[r];
            cur.units = tab->u0[r + 1] - tab->u0[r];
            cur.Bimg = base->Bimg + (long)r * tab->islab;
            if (base->bscale) cur.bscale = base->bscale + (long)r * base->c.N;
            cur.c.P = base->c.P + (long)r * tab->pslab;
        }
        lu = u - tab->u0[r];
        return cur;
    }
    static constexpr bool kTable = false;
};

// AIMG: the FF layout (16 epilogue warps over 16-column groups, no converter
// warps); APRE: the A operand arrives as a pre-split image (bulk copies onto the
// stage's B barrier) instead of FP64 rows split by the converter warps.  FF has
// both; GPP on CTA pairs over many n-tiles has APRE alone (its converter warps idle).
template <int EPI, int BN, bool AIMG, bool PAIR, class Src, bool APRE = AIMG>
__device__ __forceinline__ void tc_contract_body(Src src0, int* err, const long long wait_limit) {
    using C = Cfg<BN, EPI == EPI_FF, PAIR, APRE>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-aligned operand area
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    double2* sF = (double2*)(base + C::STAGES * C::STAGE_BYTES + C::W_BYTES);  // GPP: FP64 rows [BM][BK]
    uint64_t* bars = (uint64_t*)(base + C::STAGES * C::STAGE_BYTES + C::W_BYTES + C::F64_BYTES);
    uint64_t* fullA = bars;
    uint64_t* fullB = bars + C::STAGES;
    uint64_t* empty = bars + 2 * C::STAGES;
    uint64_t* accFull = bars + 3 * C::STAGES;  // [NBUF]
    uint64_t* accEmpty = accFull + C::NBUF;    // [NBUF]
    uint64_t* done = accEmpty + C::NBUF;
    uint64_t* fFull = done + 1;    // [2] GPP: FP64 staging half filled (tx bytes)
    uint64_t* fEmpty = done + 3;   // [2] GPP: FP64 staging half read by all converter warps
    uint64_t* peerFull = done + 5; // [STAGES] PAIR, even CTA: the odd CTA's half of the stage has landed
    uint64_t* negFull = done + 5 + C::STAGES;  // [STAGES] FF: the stage's -B_im is written
    uint32_t* tslot = (uint32_t*)(done + 5 + 2 * C::STAGES);
    __shared__ int s_abort_flag;
    volatile int& s_abort = s_abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // a CTA pair takes units together: pair id, pair count, rank in the pair
    const uint32_t rank = PAIR ? tc::cluster_rank() : 0u;
    const int pid = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int npairs = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
    constexpr int EPI_WARPS = AIMG ? 4 * FF_EPI_WARPS : 4;

    if (tid == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            tc::mbar_init(&fullA[s], APRE ? 1 : NCONV);
            tc::mbar_init(&fullB[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < C::NBUF; ++b) {
            tc::mbar_init(&accFull[b], 1);
            tc::mbar_init(&accEmpty[b], PAIR ? 2 * EPI_WARPS : EPI_WARPS);  // both CTAs' epilogues drain
        }
        for (int s = 0; s < C::STAGES; ++s) {
            tc::mbar_init(&peerFull[s], 1);
            tc::mbar_init(&negFull[s], 1);
        }
        tc::mbar_init(done, 1);
        for (int h = 0; h < 2; ++h) {
            tc::mbar_init(&fFull[h], 1);
            tc::mbar_init(&fEmpty[h], NCONV);
        }
        tc::fence_barrier_init();
        s_abort = 0;
    }
    if (warp == 0) {
        if constexpr (PAIR) {
            tc::tmem_alloc_pair(tslot, C::TMEM_COLS);
            tc::tmem_relinquish_pair();
        } else {
            tc::tmem_alloc(tslot, C::TMEM_COLS);
            tc::tmem_relinquish();
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if constexpr (PAIR) tc::cluster_sync();  // both CTAs' barriers and TMEM exist before any MMA
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;

    // local unit -> (m-tile, n-tile, k-slice, batch) and the slice's k range
    // (PAIR: MT counts 256-row tiles; mt is this CTA's 128-row tile)
    auto unit_coords = [&](const TcArgs& t, int u, int& mt, int& nt, int& ks, int& batch) {
        mt = t.mt0 + u % t.MT;
        if (PAIR) mt = 2 * mt + (int)rank;
        int r = u / t.MT;
        nt = r % t.NT;
        r /= t.NT;
        ks = r % t.c.KS;
        batch = r / t.c.KS;
    };
    auto krange = [&](const TcArgs& t, int ks, int& k0, int& k1) {
        k0 = ks * t.c.kchunk;
        k1 = min(t.c.K, k0 + t.c.kchunk);
    };
    auto fail = [&](int code) {
        atomicOr(err, code);
        s_abort = 1;
    };

    Src src = src0;  // per-role cursor
    if (warp == 0) {
        if (PAIR && rank == 1 && lane == 0) {
            // ------------------------------------------------- relay (odd CTA)
            // each stage's operands of this CTA have landed -> the even CTA's peerFull
            int g = 0;
            bool ok = true;
            for (int u = pid; u < src.units() && ok; u += npairs) {
                int lu;
                const TcArgs& t = src.at(u, lu);
                int mt, nt, ks, batch, k0, k1;
                unit_coords(t, lu, mt, nt, ks, batch);
                krange(t, ks, k0, k1);
                const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
                const bool ua = APRE || (Src::kTable && t.Aimg != nullptr);  // A pre-split: on fullB
                for (int st = 0; st < nst; ++st, ++g) {
                    const int s = g % C::STAGES;
                    const uint32_t par = (g / C::STAGES) & 1;
                    if ((!ua && !tc::mbar_wait(&fullA[s], par, wait_limit)) || !tc::mbar_wait(&fullB[s], par, wait_limit) ||
                        s_abort) {
                        fail(2);
                        ok = false;
                        break;
                    }
                    tc::mbar_arrive_remote(&peerFull[s], 0);
                }
            }
        } else if (lane == 0 && (!PAIR || rank == 0)) {
            // ------------------------------------------------------------ MMA
            int g = 0, grp = 0;
            bool ok = true;
            const uint32_t idp = C::F16 ? tc::idesc_f16(PAIR ? 2 * BM : BM, 2 * BN)
                                        : tc::idesc_bf16(PAIR ? 2 * BM : BM, 2 * BN, false);
            for (int u = pid; u < src.units() && ok; u += npairs) {
                int lu;
                const TcArgs& t = src.at(u, lu);
                int mt, nt, ks, batch, k0, k1;
                unit_coords(t, lu, mt, nt, ks, batch);
                krange(t, ks, k0, k1);
                const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
                const int CH = t.chunk_stages > 0 ? t.chunk_stages : 1;
                // a served request may carry a pre-split A image (its stages' A lands on fullB)
                const bool ua = APRE || (Src::kTable && t.Aimg != nullptr);
                for (int sg0 = 0; sg0 < nst && ok; sg0 += C::GRP * CH, ++grp) {
                    // a group: up to GRP chunks of CH stages, each into its own buffer of the slot
                    const int slot = grp % C::NSLOT;
                    const uint32_t bpar = ((grp / C::NSLOT) & 1) ^ 1;
                    const bool freed = PAIR ? tc::mbar_wait_cluster(&accEmpty[slot], bpar, wait_limit)
                                            : tc::mbar_wait(&accEmpty[slot], bpar, wait_limit);
                    if (!freed) { fail(1); ok = false; break; }
                    tc::tc_fence_after();
                    const int sg1 = min(nst, sg0 + C::GRP * CH);
                    for (int st0 = sg0, b = slot * C::GRP; st0 < sg1 && ok; st0 += CH, ++b) {
                        // X, Y (two accumulators) or, SL, the one accumulator D = dX
                        const uint32_t dX = tmem + (uint32_t)(b * C::ACC_COLS), dY = dX + 2 * BN;
                        const int st1 = min(nst, st0 + CH);
                        for (int st = st0; st < st1; ++st, ++g) {
                            const int s = g % C::STAGES;
                            const uint32_t par = (g / C::STAGES) & 1;
                            // pre-split A: the A image lands on fullB too (one barrier per stage);
                            // FF: negFull follows fullB once the -B_im warp has written -B_im
                            if ((!ua && !tc::mbar_wait(&fullA[s], par, wait_limit)) ||
                                !tc::mbar_wait(C::IMGN ? &negFull[s] : &fullB[s], par, wait_limit) ||
                                (PAIR && !tc::mbar_wait_cluster(&peerFull[s], par, wait_limit))) {
                                fail(2);
                                ok = false;
                                break;
                            }
                            tc::tc_fence_after();
                            // the descriptor's start-address field is address / 16 in its low 14 bits and
                            // shared addresses stay below 2^18, so every operand's descriptor is the stage's
                            // base descriptor plus a constant: one add per MMA for the single issuing thread
                            const uint64_t dA = tc::sdesc_sw64(tc::smem_u32(base + s * C::STAGE_BYTES));
                            const uint64_t dB = dA + (C::A_BYTES >> 4);
                            // A sub-tile (re h,m,l, im h,m,l) and B piece, k offset kk*16.  A CTA's B
                            // piece is 2*BN rows ([B_re; B_im], or SL [B_re; -B_im] / [B_im; B_re]),
                            // or BN rows (pair without SL: its half [B_re] or [B_im])
                            auto ad = [&](int sub, int kk) { return dA + (uint64_t)((sub * BM * 64) >> 4) + 2 * kk; };
                            auto bd = [&](int piece, int kk) {
                                constexpr int SUBS = C::SL ? (PAIR ? 2 : 3) : (PAIR ? 1 : 2);  // sub-tiles per piece
                                return dB + (uint64_t)((piece * SUBS * BN * 64) >> 4) + 2 * kk;
                            };
                            constexpr uint64_t B_HALF = (uint64_t)(BN * 64) >> 4;  // SL: the piece's second BN rows
                            auto mma2 = [&](int pa, int pb, int kk, uint32_t accumulate) {
                                // X += A_re,pa x [B_re|B_im]_pb, Y += A_im,pa x [B_re|B_im]_pb; SL:
                                // D += A_re,pa x [B_re|B_im]_pb + A_im,pa x [-B_im|B_re]_pb
                                if constexpr (C::SL && PAIR) {
                                    tc::mma_bf16_pair(dX, ad(pa, kk), bd(pb, kk), idp, accumulate);
                                    tc::mma_bf16_pair(dX, ad(C::NPIECE + pa, kk), bd(pb, kk) + B_HALF, idp, 1u);
                                } else if constexpr (C::SL) {
                                    // [B_re; B_im] from the piece's second sub-tile, [-B_im; B_re] from its first
                                    tc::mma_bf16(dX, ad(pa, kk), bd(pb, kk) + B_HALF, idp, accumulate);
                                    tc::mma_bf16(dX, ad(C::NPIECE + pa, kk), bd(pb, kk), idp, 1u);
                                } else if constexpr (PAIR) {
                                    tc::mma_bf16_pair(dX, ad(pa, kk), bd(pb, kk), idp, accumulate);
                                    tc::mma_bf16_pair(dY, ad(C::NPIECE + pa, kk), bd(pb, kk), idp, accumulate);
                                } else {
                                    tc::mma_bf16(dX, ad(pa, kk), bd(pb, kk), idp, accumulate);
                                    tc::mma_bf16(dY, ad(C::NPIECE + pa, kk), bd(pb, kk), idp, accumulate);
                                }
                            };
                            // The accumulators truncate each addition to FP32 at the magnitude they
                            // hold, so the small piece products (BF16: mm, lh, hl, mh, hm, 2^-8 and
                            // below of the sum; FP16: lh, hl, 2^-11) of both k-steps go in first,
                            // while the accumulator is small, and the two hh products last: two
                            // full-scale roundings per stage.
                            constexpr int NQ = C::F16 ? 2 : 5;
                            constexpr int PA[5] = {1, C::F16 ? 0 : 2, 0, 1, 0};
                            constexpr int PB[5] = {C::F16 ? 0 : 1, C::F16 ? 1 : 0, 2, 0, 1};
#pragma unroll
                            for (int kk = 0; kk < 2; ++kk)
#pragma unroll
                                for (int q = 0; q < NQ; ++q) mma2(PA[q], PB[q], kk, (st > st0 || kk > 0 || q > 0) ? 1u : 0u);
                            mma2(0, 0, 0, 1u);
                            mma2(0, 0, 1, 1u);
                            if constexpr (PAIR) tc::mma_commit_pair(&empty[s], 3);  // frees the stage in both CTAs
                            else tc::mma_commit(&empty[s]);
                        }
                    }
                    if (!ok) break;
                    // one commit tracks every earlier MMA of this thread: the whole group
                    if constexpr (PAIR) tc::mma_commit_pair(&accFull[slot], 3);  // both CTAs' epilogues
                    else tc::mma_commit(&accFull[slot]);
                }
            }
            // drain: every issued MMA has completed before TMEM is released
            if constexpr (PAIR) tc::mma_commit_pair(done, 1);
            else tc::mma_commit(done);
            if (!tc::mbar_wait(done, 0, DRAIN_LIMIT)) fail(4);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ bulk copies
        // lane 0: pre-split B (and, for a pre-split A, A) tiles into the operand stage;
        // all lanes (GPP): the next stage's FP64 A rows into the staging buffer.
        // g counts stage uses, gf the stage uses staged in FP64 (the staging
        // halves' barriers complete once per such use)
        int g = 0, gf = 0;
        bool ok = true;
        // the last copy issued into each stage / staging half (-1: none), so
        // that the CTA can wait for every copy it started before it exits
        int last_st[C::STAGES], last_f[2] = {-1, -1};
#pragma unroll
        for (int s = 0; s < C::STAGES; ++s) last_st[s] = -1;
        for (int u = pid; u < src.units() && ok; u += npairs) {
            int lu;
            const TcArgs& t = src.at(u, lu);
            const ContractArgs& a = t.c;
            int mt, nt, ks, batch, k0, k1;
            unit_coords(t, lu, mt, nt, ks, batch);
            krange(t, ks, k0, k1);
            const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
            const int plane = a.batch_plane ? a.batch_plane[batch] : batch;
            const bool ua = APRE || (Src::kTable && t.Aimg != nullptr);
            if (Src::kTable && !ua && lane == 0) {
                // the table was written by copies before the launch: make its
                // tensor map visible to the tensor-memory-access unit
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&t.amap) : "memory");
            }
            for (int st = 0; st < nst; ++st, ++g) {
                const int s = g % C::STAGES;
                const long kst = (long)(k0 / BK) + st;
                if (!ua) {
                    // FP64 rows in two halves of BK/2 k-values, each into its own half of the
                    // staging buffer as soon as the converters have read that half of the last stage
                    for (int h = 0; h < 2 && ok; ++h) {
                        if (!tc::warp_all(tc::mbar_wait(&fEmpty[h], (gf & 1) ^ 1, wait_limit) && !s_abort)) {
                            fail(64);
                            ok = false;
                            break;
                        }
                        if (lane == 0) {
                            tc::mbar_arrive_expect_tx(&fFull[h], C::F64_BYTES / 2);
                            tc::tma_load_2d(sF + h * (BM * BK / 2), &t.amap, 2 * (k0 + st * BK + h * (BK / 2)),
                                            a.m0 + mt * BM, &fFull[h]);
                            last_f[h] = gf;
                        }
                    }
                    if (!ok) break;
                    ++gf;
                }
                if (lane == 0) {
                    if (!tc::mbar_wait(&empty[s], ((g / C::STAGES) & 1) ^ 1, wait_limit) || s_abort) {
                        fail(8);
                        ok = false;
                    } else {
                        const uint8_t* src =
                            t.Bimg + (((long)plane * t.NT + nt) * t.kstages_total + kst) * (long)C::B_BYTES;
                        tc::mbar_arrive_expect_tx(&fullB[s], C::B_COPY + (ua ? C::A_BYTES : 0u));
                        uint8_t* bdst = base + s * C::STAGE_BYTES + C::A_BYTES;
                        if constexpr (C::SL && !PAIR) {
                            // single CTA: [re; im] of each piece into sub-tiles 1, 2 of its three
                            // (the -B_im warp writes -im into sub-tile 0)
                            for (int pc = 0; pc < C::NPIECE; ++pc)
                                tc::bulk_g2s(bdst + (3 * pc + 1) * BN * 64, src + (2 * pc) * BN * 64, 2 * BN * 64,
                                             &fullB[s]);
                        } else if constexpr (C::SL) {
                            // image re, im per piece: the even CTA takes [re; im] (its -B_im warp
                            // negates im in place), the odd [im; re]
                            for (int pc = 0; pc < C::NPIECE; ++pc) {
                                if (rank == 0) {
                                    tc::bulk_g2s(bdst + (2 * pc) * BN * 64, src + (2 * pc) * BN * 64, 2 * BN * 64, &fullB[s]);
                                } else {
                                    tc::bulk_g2s(bdst + (2 * pc) * BN * 64, src + (2 * pc + 1) * BN * 64, BN * 64, &fullB[s]);
                                    tc::bulk_g2s(bdst + (2 * pc + 1) * BN * 64, src + (2 * pc) * BN * 64, BN * 64,
                                                 &fullB[s]);
                                }
                            }
                        } else if constexpr (PAIR) {
                            // the even CTA's B_re, the odd CTA's B_im of each piece (paired image layout:
                            // re h, im h, re m, im m, re l, im l), BN rows each
                            for (int pc = 0; pc < NSPLIT; ++pc)
                                tc::bulk_g2s(bdst + pc * BN * 64, src + (2 * pc + (int)rank) * BN * 64, BN * 64, &fullB[s]);
                        } else {
                            tc::bulk_g2s(base + s * C::STAGE_BYTES + C::A_BYTES, src, C::B_BYTES, &fullB[s]);
                        }
                        if (ua) {
                            const uint8_t* asrc = t.Aimg + ((long)mt * t.kstages_total + kst) * (long)C::A_BYTES;
                            tc::bulk_g2s(base + s * C::STAGE_BYTES, asrc, C::A_BYTES, &fullB[s]);
                        }
                        last_st[s] = g;
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                if (!ok) break;
            }
        }
        // Every copy this warp started lands before the CTA exits (after a
        // timed-out wait elsewhere, the consumers may never have waited for
        // them).  A stage's copies start only after its previous phase was
        // consumed, so each barrier owes at most its last issued phase.
        if (lane == 0) {
            bool drained = true;
#pragma unroll
            for (int s = 0; s < C::STAGES; ++s)
                if (last_st[s] >= 0) {
                    const uint32_t par = (uint32_t)(last_st[s] / C::STAGES) & 1u;
                    drained = tc::mbar_wait(&fullB[s], par, DRAIN_LIMIT) && drained;  // a pre-split A image too
                }
            if (!APRE)
                for (int h = 0; h < 2; ++h)
                    if (last_f[h] >= 0) drained = tc::mbar_wait(&fFull[h], (uint32_t)last_f[h] & 1u, DRAIN_LIMIT) && drained;
            if (!drained) fail(128);
        }
    } else if (C::IMGN && warp == THREADS_FF / 32 - 1) {
        // ------------------------------------------------------- -B_im warp
        // FF (the MMA-issuing CTA of a pair, or a single CTA): once a stage's
        // copies have landed, write -im of each B piece (the FP16 sign bits
        // flipped: the swizzle permutes whole 16-byte chunks, so no position
        // moves), in place for a pair's even CTA, into sub-tile 0 for a single
        // CTA; then fence toward the tensor cores' proxy and arrive on negFull.
        if (!PAIR || rank == 0) {
            int g = 0;
            bool ok = true;
            for (int u = pid; u < src.units() && ok; u += npairs) {
                int lu;
                const TcArgs& t = src.at(u, lu);
                int mt, nt, ks, batch, k0, k1;
                unit_coords(t, lu, mt, nt, ks, batch);
                krange(t, ks, k0, k1);
                const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
                for (int st = 0; st < nst; ++st, ++g) {
                    const int s = g % C::STAGES;
                    if (!tc::warp_all(tc::mbar_wait(&fullB[s], (g / C::STAGES) & 1, wait_limit) && !s_abort)) {
                        fail(0x400);
                        ok = false;
                        break;
                    }
                    uint8_t* bsm = base + s * C::STAGE_BYTES + C::A_BYTES;
#pragma unroll
                    for (int pc = 0; pc < C::NPIECE; ++pc) {
                        const uint4* from = (const uint4*)(bsm + (PAIR ? 2 * pc + 1 : 3 * pc + 2) * BN * 64);
                        uint4* to = (uint4*)(bsm + (PAIR ? 2 * pc + 1 : 3 * pc) * BN * 64);
                        for (int i = lane; i < BN * 64 / 16; i += 32) {
                            uint4 v = from[i];
                            v.x ^= 0x80008000u;
                            v.y ^= 0x80008000u;
                            v.z ^= 0x80008000u;
                            v.w ^= 0x80008000u;
                            to[i] = v;
                        }
                    }
                    tc::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&negFull[s]);
                }
            }
        }
    } else if ((warp >= 4 && warp < 8) || AIMG) {
        // ------------------------------------------------------- epilogue
        // Weights are fetched once per unit into registers: GPP all 64
        // columns of the row (a 64-wide tile holds complete (igp, iw) triples
        // of GPP_COLS igp), FF the warp's 16 columns (and their vcoul).
        // Columns are fully unrolled so every register index is a compile-time
        // constant.
        constexpr int EW = AIMG ? FF_EPI_WARPS : 1;  // warps per lane quarter
        const int q4 = warp & 3;                     // TMEM lane quarter
        const int ej = AIMG ? (warp - 2) >> 2 : 0;   // FF: this warp's 16-column group
        const int row = q4 * 32 + lane;
        int grp = 0;
        bool ok = true;
        constexpr int GC = BN / 3;  // 21 igp per GPP tile
        for (int u = pid; u < src.units() && ok; u += npairs) {
            int lu;
            const TcArgs& t = src.at(u, lu);
            const ContractArgs& a = t.c;
            int mt, nt, ks, batch, k0, k1;
            unit_coords(t, lu, mt, nt, ks, batch);
            krange(t, ks, k0, k1);
            const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
            const int m = mt * BM + row;
            const int mc = min(m, a.M - 1);
            float2 wreg[EPI == EPI_GPP ? GC : 16];
            float vreg[EPI == EPI_GPP ? 1 : 16];
            if (EPI == EPI_GPP) {
#pragma unroll
                for (int i = 0; i < GC; ++i) {
                    const int h = nt * t.gpp_cols + i;
                    wreg[i] = (i < t.gpp_cols && h < a.N / 3) ? t.W1[(long)h * t.ldw + mc] : make_float2(0.f, 0.f);
                }
            } else {
                // conj(aqsm) of this thread's row and vcoul of the warp's 16 columns; the
                // weights carry 2^-k of the row's and the column's scales (powers of two: exact)
                const float sa = (t.ascale && m < a.M) ? t.ascale[m] : 1.f;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = nt * BN + ej * 16 + j;
                    wreg[j] = (n < a.N && m < a.M) ? t.W2[(long)n * t.ldw + m] : make_float2(0.f, 0.f);
                    vreg[j] = n < a.N ? t.vcol[n] : 0.f;
                    if (t.bscale) {
                        const float sc = sa * (n < a.N ? t.bscale[(long)batch * a.N + n] : 0.f);
                        wreg[j].x *= sc;
                        wreg[j].y *= sc;
                    }
                }
            }
            // per-unit sums as FP32 float-float pairs (TwoSum): no FP64 instruction per drain
            // (GB300's FP64 pipe takes ~16 cycles per warp instruction); widened once per unit
            ff32 accx[GMAX] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, accy[GMAX] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            const int CH = t.chunk_stages > 0 ? t.chunk_stages : 1;
            const bool rs = !t.ff_no_rs;
            // a pass drains one group of accumulator buffers (SL: two consecutive chunks,
            // added in registers with one round-to-nearest FP32 addition before the
            // weighted sums: half the arithmetic, waits and returns per chunk)
            for (int st0 = 0; st0 < nst; ++grp) {
                const int npass = min(C::GRP, (nst - st0 + CH - 1) / CH);  // chunks in the group
                const int slot = grp % C::NSLOT;
                const int b = slot * C::GRP, b2 = b + 1;
                if (!tc::warp_all(tc::mbar_wait(&accFull[slot], (grp / C::NSLOT) & 1, wait_limit) && !s_abort)) {
                    fail(16);
                    ok = false;
                    break;
                }
                st0 += npass * CH;
                tc::tc_fence_after();
                const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b * C::ACC_COLS);
                const uint32_t tl2 = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b2 * C::ACC_COLS);
                float2 gsum[GMAX] = {make_float2(0, 0), make_float2(0, 0), make_float2(0, 0)};
                // the pass's buffers go back to the MMA issuer as soon as this warp's
                // last TMEM load of them has landed, before the arithmetic on those values
                auto release = [&]() {
                    tc::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) {
                        // the MMA issuer's barrier; the loads of the group have completed, so
                        // no cluster-wide release is needed (it cost ~2000 cycles per drain)
                        if (PAIR && rank == 1) tc::mbar_arrive_peer(&accEmpty[slot], 0);
                        else tc::mbar_arrive(&accEmpty[slot]);
                    }
                };
                if constexpr (EPI == EPI_FF) {
                    // the warp's 16 columns of D = [S_re | S_im] of each buffer (the real
                    // parts of both, added, then the imaginary parts: 48 registers of
                    // values live instead of 64), the buffers go back, then the weighted sums
                    const int c0 = ej * 16;
                    float sr[16], si[16];
                    if (npass == 2) {
                        float tx[16];
                        tc::tmem_ld16(tl + c0, sr);
                        tc::tmem_ld16(tl2 + c0, tx);
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 16; ++j) sr[j] += tx[j];
                        tc::tmem_ld16(tl + BN + c0, si);
                        tc::tmem_ld16(tl2 + BN + c0, tx);
                        tc::tmem_ld_wait();
                        release();
#pragma unroll
                        for (int j = 0; j < 16; ++j) si[j] += tx[j];
                    } else {
                        tc::tmem_ld16(tl + c0, sr);
                        tc::tmem_ld16(tl + BN + c0, si);
                        tc::tmem_ld_wait();
                        release();
                    }
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float2 t2 = cmulf(wreg[j], make_float2(sr[j], si[j]));
                        gsum[0].x = fmaf(vreg[j], t2.x, gsum[0].x);
                        gsum[0].y = fmaf(vreg[j], t2.y, gsum[0].y);
                        if (rs) {
                            gsum[1].x += t2.x;
                            gsum[1].y += t2.y;
                        }
                    }
                    for (int gg = 0; gg < 2; ++gg) {
                        ff_add(accx[gg], gsum[gg].x);
                        ff_add(accy[gg], gsum[gg].y);
                        gsum[gg] = make_float2(0.f, 0.f);
                    }
                }
#pragma unroll
                for (int c0 = 0; c0 < BN && EPI == EPI_GPP; c0 += 16) {
                    // X = [A_re B_re | A_re B_im], Y = [A_im B_re | A_im B_im]
                    float xr[16], xi[16], yr[16], yi[16];
                    tc::tmem_ld16(tl + c0, xr);
                    tc::tmem_ld16(tl + BN + c0, xi);
                    tc::tmem_ld16(tl + 2 * BN + c0, yr);
                    tc::tmem_ld16(tl + 3 * BN + c0, yi);
                    tc::tmem_ld_wait();
                    if (c0 + 16 >= BN) release();
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int c = c0 + j;
                        const float2 sv = make_float2(xr[j] - yi[j], xi[j] + yr[j]);
                        // tile column c = 3*(igp offset) + iw; column 63 is padding
                        if (c < 3 * GC) cfmaf(gsum[c % 3], wreg[c / 3], sv);
                    }
                }
                if (EPI == EPI_GPP) {
#pragma unroll
                    for (int gg = 0; gg < 3; ++gg) {
                        ff_add(accx[gg], gsum[gg].x);
                        ff_add(accy[gg], gsum[gg].y);
                    }
                }
            }
            if (!ok) break;
            if (m < a.M) {
                const int slot = ((batch * a.KS + ks) * t.NT + nt) * EW + ej * (EW > 1);
                for (int gg = 0; gg < a.G; ++gg)
                    a.P[((long)slot * a.M + m) * a.G + gg] =
                        make_double2((double)accx[gg].hi + (double)accx[gg].lo, (double)accy[gg].hi + (double)accy[gg].lo);
            }
        }
    } else {
        // ----------------------------------------------------- converters
        // warp cw converts rows cw*16 .. cw*16+15 of each stage.  The staging
        // buffer holds the stage in two halves of BK/2 k-values, each filled by
        // its own TMA box: read a half (lane = (row pair, k), one conflict-free
        // 512-byte read per instruction), release it so that the next stage's
        // half is copied while the other half is read, then split everything
        // into BF16 pieces and store it into the operand stage.
        if (!APRE) {
            const int cw = warp < 4 ? warp - 2 : warp - 6;  // 0..7
            constexpr int RPW = BM / NCONV;                  // rows per converter warp
            int g = 0, gf = 0;  // stage uses, FP64-staged stage uses (as the copy warp counts them)
            bool ok = true;
            for (int u = pid; u < src.units() && ok; u += npairs) {
                int lu;
                const TcArgs& t = src.at(u, lu);
                const ContractArgs& a = t.c;
                int mt, nt, ks, batch, k0, k1;
                unit_coords(t, lu, mt, nt, ks, batch);
                krange(t, ks, k0, k1);
                const int nst = k1 > k0 ? (k1 - k0 + BK - 1) / BK : 0;
                const bool ua = Src::kTable && t.Aimg != nullptr;  // the request's A is pre-split
                for (int st = 0; st < nst; ++st, ++g) {
                    const int s = g % C::STAGES;
                    if (ua) {
                        // the stage's A arrives by bulk copy: only complete this use's phase of
                        // fullA (no data), after the stage is free, so that every use of a
                        // stage completes one phase whichever way its A arrives
                        if (!tc::warp_all(tc::mbar_wait(&empty[s], ((g / C::STAGES) & 1) ^ 1, wait_limit) && !s_abort)) {
                            fail(32);
                            ok = false;
                            break;
                        }
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(&fullA[s]);
                        continue;
                    }
                    if (!tc::warp_all(tc::mbar_wait(&fFull[0], gf & 1, wait_limit) && !s_abort)) {
                        fail(32);
                        ok = false;
                        break;
                    }
                    // lane -> (row pair offset lane>>4, k within the half lane&15)
                    double2 v[RPW];
                    const int kk = lane & 15, rr = lane >> 4;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (h == 1 && !tc::warp_all(tc::mbar_wait(&fFull[1], gf & 1, wait_limit) && !s_abort)) {
                            fail(32);
                            ok = false;
                            break;
                        }
                        const double2* sh = sF + h * (BM * BK / 2);
                        const int kh = k0 + st * BK + h * (BK / 2) + kk;
#pragma unroll
                        for (int i = 0; i < RPW / 2; ++i) {
                            const int r = cw * RPW + 2 * i + rr;
                            v[h * (RPW / 2) + i] = (mt * BM + r < a.M && kh < k1) ? sh[r * (BK / 2) + kk] : make_double2(0.0, 0.0);
                        }
                        __syncwarp();
                        if (lane == 0) tc::mbar_arrive(&fEmpty[h]);
                    }
                    if (!ok) break;
                    if (!tc::warp_all(tc::mbar_wait(&empty[s], ((g / C::STAGES) & 1) ^ 1, wait_limit) && !s_abort)) {
                        fail(32);
                        ok = false;
                        break;
                    }
                    uint8_t* sa = base + s * C::STAGE_BYTES;
#pragma unroll
                    for (int i = 0; i < RPW; ++i) {
                        // v[i]: half i / (RPW/2), row pair i % (RPW/2)
                        const uint32_t off =
                            tc::sw64_offset(cw * RPW + 2 * (i % (RPW / 2)) + rr, (i / (RPW / 2)) * (BK / 2) + kk);
                        uint16_t hh, mm, ll;
                        split3(f64_to_f32_bits(v[i].x), hh, mm, ll);
                        *(uint16_t*)(sa + 0 * BM * 64 + off) = hh;
                        *(uint16_t*)(sa + 1 * BM * 64 + off) = mm;
                        *(uint16_t*)(sa + 2 * BM * 64 + off) = ll;
                        split3(f64_to_f32_bits(v[i].y), hh, mm, ll);
                        *(uint16_t*)(sa + 3 * BM * 64 + off) = hh;
                        *(uint16_t*)(sa + 4 * BM * 64 + off) = mm;
                        *(uint16_t*)(sa + 5 * BM * 64 + off) = ll;
                    }
                    tc::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&fullA[s]);
                    ++gf;
                }
            }
        }
    }

    tc::tc_fence_before();
    __syncthreads();
    // PAIR: the even CTA's MMAs read this CTA's shared memory and write its
    // TMEM; neither CTA releases either before both are done
    if constexpr (PAIR) tc::cluster_sync();
    if (warp == 0) {
        __syncwarp();
        if constexpr (PAIR) tc::tmem_dealloc_pair(tmem, C::TMEM_COLS);
        else tc::tmem_dealloc(tmem, C::TMEM_COLS);
    }
}

template <int EPI, int BN, bool AIMG>
__global__ void __launch_bounds__(AIMG ? THREADS_FF : THREADS, 1) tc_contract_kernel(const __grid_constant__ TcArgs t) {
    tc_contract_body<EPI, BN, AIMG, false>(OneReq{t}, t.err, t.wait_limit);
}

// The same over CTA pairs (M = 256 per unit; t.MT counts 256-row tiles and
// the grid is an even number of CTAs).
template <int EPI, int BN, bool AIMG>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(AIMG ? THREADS_FF : THREADS, 1)
    tc_contract_pair_kernel(const __grid_constant__ TcArgs t) {
    tc_contract_body<EPI, BN, AIMG, true>(OneReq{t}, t.err, t.wait_limit);
}

// GPP on CTA pairs with aqsntemp pre-split into an A image (over many n-tiles
// the converter warps would split the same A rows again for every n-tile).
template <int EPI, int BN>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    tc_contract_pair_apre_kernel(const __grid_constant__ TcArgs t) {
    tc_contract_body<EPI, BN, false, true, OneReq, true>(OneReq{t}, t.err, t.wait_limit);
}

// The batches of a PlaneTab in one launch (single CTAs).
template <int EPI, int BN, bool AIMG>
__global__ void __launch_bounds__(AIMG ? THREADS_FF : THREADS, 1)
    tc_contract_planes_kernel(const __grid_constant__ TcArgs t, const __grid_constant__ PlaneTab pt) {
    tc_contract_body<EPI, BN, AIMG, false>(PlaneSeq{&t, &pt, t, -1}, t.err, t.wait_limit);
}

// Units of several requests from a device table (the served step).
template <int EPI, int BN, bool AIMG>
__global__ void __launch_bounds__(AIMG ? THREADS_FF : THREADS, 1) tc_contract_table_kernel(const TcTable* tab, int* err, long long wait_limit) {
    tc_contract_body<EPI, BN, AIMG, false>(TableReqs{tab, 0}, err, wait_limit);
}

// Epilogue weight tables in FP32, column-major (row m contiguous):
// W1[h][m] = wscale*vcoul[igp]*conj(aqsm[r][igp]), W2[h][m] = conj(aqsm[r][igp]),
// r = m0 + m, or rowmap[m] when the rows are in another order.
__device__ __forceinline__ float2 weight_w1(const double2 am, double s) {
    return make_float2(f64_to_f32_bits(am.x * s), f64_to_f32_bits(-am.y * s));
}
static __global__ void weight_table_kernel(int M, int m0, int ncols, const double2* aqsm, long ldm, const double* vcoul,
                                    const int* igp, const int* acol, double wscale, float2* W1, float2* W2,
                                    float* vcol, const int* rowmap = nullptr) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y;
    if (h >= ncols || m >= M) return;
    const int g = igp[h];
    float2 w1 = make_float2(0.f, 0.f), w2 = w1;
    if (g >= 0) {
        const double2 am = aqsm[(long)(rowmap ? rowmap[m] : m0 + m) * ldm + acol[h]];
        w1 = weight_w1(am, wscale * vcoul[g]);
        w2 = make_float2(f64_to_f32_bits(am.x), f64_to_f32_bits(-am.y));
    }
    W1[(long)h * M + m] = w1;
    if (W2) W2[(long)h * M + m] = w2;
    if (vcol && m == 0) vcol[h] = g >= 0 ? f64_to_f32_bits(vcoul[g]) : 0.f;
}

// FF operands in FP16 pieces.  A row is scaled by 2^k, k from its largest
// magnitude |re| or |im| (its FP64 exponent e: k = 14 - e, so the row's values
// lie below 2^15, within FP16's range, and its largest ones use FP16's full
// precision); a scaled FP32 value v splits into h = fp16(v) and l = fp16(v - h)
// (v - h is exact in FP32), v = h + l to 22 bits.  k is clamped to [-126, 126]
// (2^k and 2^-k stay normal FP32 numbers): rows whose largest magnitude lies
// outside [2^-112, 2^140] keep fewer bits.  Rows of zeros get k = 0.
__device__ __forceinline__ int f16_row_shift(unsigned long long maxbits) {
    const int e = (int)((maxbits >> 52) & 0x7ff);
    if (e == 0) return 0;
    return min(126, max(-126, 14 - (e - 1023)));
}
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float((uint32_t)(127 + k) << 23); }
__device__ __forceinline__ void split_f16(float v, uint16_t& h, uint16_t& l) {
    const __half hh = __float2half_rn(v);
    h = __half_as_ushort(hh);
    l = __half_as_ushort(__float2half_rn(v - __half2float(hh)));
}
// Largest |re| or |im| bit pattern of an FP64 complex row (integer compares:
// the FP64 pipe is narrow on this GPU), over the block; every thread gets it.
__device__ __forceinline__ unsigned long long row_max_bits(const double2* row, int K) {
    unsigned long long mx = 0;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const double2 v = row[k];
        const unsigned long long a = (unsigned long long)__double_as_longlong(v.x) & 0x7fffffffffffffffull;
        const unsigned long long b = (unsigned long long)__double_as_longlong(v.y) & 0x7fffffffffffffffull;
        mx = max(mx, max(a, b));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    __shared__ unsigned long long wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = max(mx, wm[w]);
    return mx;
}

// FF B images: four sub-tiles per k-stage (re, im of pieces h and l)
constexpr int FF_BSUB = 4;
// FF B image writer: the 16-byte swizzle chunk of each of the four sub-tiles
// for the 8 consecutive k-values k0.. of row n (k0 % 8 == 0; values past K, if
// any, are zeros), scaled by s.
template <int BN>
__device__ __forceinline__ void bimg_chunk_f16(uint8_t* img_nt, int n, int k0, const double2 (&v)[8], float s) {
    constexpr long STAGE = (long)FF_BSUB * BN * 64;
    uint32_t pk[4][4];  // piece (part + 2*level) x four fp16 pairs
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
        uint16_t h0, l0, h1, l1;
        split_f16(f64_to_f32_bits(v[j].x) * s, h0, l0);
        split_f16(f64_to_f32_bits(v[j + 1].x) * s, h1, l1);
        pk[0][j / 2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        pk[2][j / 2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
        split_f16(f64_to_f32_bits(v[j].y) * s, h0, l0);
        split_f16(f64_to_f32_bits(v[j + 1].y) * s, h1, l1);
        pk[1][j / 2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        pk[3][j / 2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
    uint8_t* st = img_nt + (long)(k0 / BK) * STAGE;
    const uint32_t off = tc::sw64_offset(n % BN, k0 % BK);  // 16-byte aligned: k0 % 8 == 0
#pragma unroll
    for (int q = 0; q < 4; ++q)  // sub-tiles re h, im h, re l, im l
        *(uint4*)(st + q * BN * 64 + off) = make_uint4(pk[q][0], pk[q][1], pk[q][2], pk[q][3]);
}
// Stage of a rotation of eight values: when `on`, w[i] takes w[(i - B) & 7].
template <int B>
__device__ __forceinline__ void rot8_stage(double2 (&w)[8], bool on) {
    double2 t[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) t[i] = on ? w[(i - B) & 7] : w[i];
#pragma unroll
    for (int i = 0; i < 8; ++i) w[i] = t[i];
}
// The values k0 .. k0+7 of a row held in shared memory (zeros at and past n).
// A thread's eight values are 128 contiguous bytes, so the eight threads of a
// quarter-warp read 128 bytes apart: read in order, every 16-byte load would
// hit the same four banks (eight-way conflict).  Thread t reads element
// (j + t) & 7 in step j instead, which puts the quarter-warp's eight loads on
// eight different 16-byte bank groups, and rotates the values back (three
// conditional stages by 1, 2 and 4 positions).
__device__ __forceinline__ void smem_chunk8(const double2* rowbuf, int k0, int n, double2 (&v)[8]) {
    const int r = threadIdx.x & 7;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int e = (j + r) & 7;
        v[j] = k0 + e < n ? rowbuf[k0 + e] : make_double2(0.0, 0.0);
    }
    // v[j] holds element (j + r) & 7, so element i is v[(i - r) & 7]
    rot8_stage<1>(v, (r & 1) != 0);
    rot8_stage<2>(v, (r & 2) != 0);
    rot8_stage<4>(v, (r & 4) != 0);
}
__device__ __forceinline__ unsigned long long abs_bits2(double2 v) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(v.x) & 0x7fffffffffffffffull;
    const unsigned long long b = (unsigned long long)__double_as_longlong(v.y) & 0x7fffffffffffffffull;
    return max(a, b);
}
// Largest of the block's per-thread values (every thread gets it).
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long mx) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    __shared__ unsigned long long wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = max(mx, wm[w]);
    return mx;
}

// FP64 planes [plane][rows][K] -> the FF B images
// [plane][nt][kstage][re h, im h, re l, im l][BN][64 B], each row scaled by its
// own 2^k (scale[plane][row] = 2^-k).  One block of 512 threads per (row, plane), each thread holding
// NCH chunks of 8 consecutive k-values (128 contiguous bytes) in registers: the
// row's largest magnitude over the block, then the pieces of the held values,
// one 16-byte swizzle chunk of each sub-tile per chunk (the swizzle permutes
// whole 16-byte chunks).  Rows up to 4096 * NCH k-values; NCH = 0: any length,
// the row read twice (its largest magnitude, then the pieces).  Grid (rows, planes).
template <int BN, int NCH>
__global__ void __launch_bounds__(512) bimg_convert_kernel(const double2* src, long plane_stride, int rows, int K,
                                                           const int* planes, int kstages, uint8_t* img,
                                                           float* scale) {
    constexpr int T = 512;
    const int n = blockIdx.x, b = blockIdx.y;
    const int f = planes ? planes[b] : b;
    const double2* row = src + (long)f * plane_stride + (long)n * K;
    const int NT = (rows + BN - 1) / BN;
    uint8_t* img_nt = img + (((long)b * NT + n / BN) * kstages) * ((long)FF_BSUB * BN * 64);
    double2 v[NCH > 0 ? NCH : 1][8];
    unsigned long long mx = 0;
    auto load = [&](int k0, double2 (&w)[8]) {
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = k0 + j < K ? row[k0 + j] : make_double2(0.0, 0.0);
    };
    if constexpr (NCH > 0) {
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const int k0 = 8 * (threadIdx.x + c * T);
            if (k0 < K) {
                load(k0, v[c]);
#pragma unroll
                for (int j = 0; j < 8; ++j) mx = max(mx, abs_bits2(v[c][j]));
            }
        }
    } else {
        for (int k = threadIdx.x; k < K; k += T) mx = max(mx, abs_bits2(row[k]));
    }
    const int k2 = f16_row_shift(block_max_u64(mx));
    const float s = pow2f(k2);
    if (threadIdx.x == 0) scale[(long)b * rows + n] = pow2f(-k2);
    if constexpr (NCH > 0) {
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const int k0 = 8 * (threadIdx.x + c * T);
            if (k0 < K) bimg_chunk_f16<BN>(img_nt, n, k0, v[c], s);
        }
    } else {
        for (int k0 = 8 * threadIdx.x; k0 < K; k0 += 8 * T) {
            load(k0, v[0]);
            bimg_chunk_f16<BN>(img_nt, n, k0, v[0], s);
        }
    }
}
// The same conversion with the row in shared memory: one thread copies the
// whole row there with bulk copies (one request per 16 KB; no register staging,
// so three 256-thread blocks per SM overlap their copies with the others'
// conversion), then the block takes the row's largest magnitude and writes its
// pieces.  Rows of at most FF_ROW_SMEM_K k-values (64 KB); the row must start on
// a 16-byte boundary (double2 rows do).  A copy that does not land within
// `wait_limit` cycles sets bit 0x200 of *err and the block writes nothing.
constexpr int FF_ROW_SMEM_K = 4096;
template <int BN>
__global__ void __launch_bounds__(256) bimg_convert_smem_kernel(const double2* src, long plane_stride, int rows, int K,
                                                                const int* planes, int kstages, uint8_t* img,
                                                                float* scale, int* err, long long wait_limit) {
    extern __shared__ __align__(16) uint8_t smem_row[];
    double2* rowbuf = (double2*)smem_row;
    __shared__ __align__(8) uint64_t bar;
    __shared__ int ok;
    const int n = blockIdx.x, b = blockIdx.y;
    const int f = planes ? planes[b] : b;
    const double2* row = src + (long)f * plane_stride + (long)n * K;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
        const uint32_t bytes = (uint32_t)K * 16u;
        tc::mbar_arrive_expect_tx(&bar, bytes);
        for (uint32_t o = 0; o < bytes; o += 16384u)
            tc::bulk_g2s(smem_row + o, (const uint8_t*)row + o, min(16384u, bytes - o), &bar);
        // the block exits only after its copy has landed (the bound applies to a
        // copy that never completes, which leaves the block's result unwritten)
        ok = tc::mbar_wait(&bar, 0, wait_limit) ? 1 : 0;
        if (!ok) {
            atomicOr(err, 0x200);
            tc::mbar_wait(&bar, 0, DRAIN_LIMIT);
        }
    }
    __syncthreads();
    if (!ok) return;
    unsigned long long mx = 0;
    for (int k = threadIdx.x; k < K; k += 256) mx = max(mx, abs_bits2(rowbuf[k]));
    const int k2 = f16_row_shift(block_max_u64(mx));
    const float s = pow2f(k2);
    if (threadIdx.x == 0) scale[(long)b * rows + n] = pow2f(-k2);
    const int NT = (rows + BN - 1) / BN;
    uint8_t* img_nt = img + (((long)b * NT + n / BN) * kstages) * ((long)FF_BSUB * BN * 64);
    for (int k0 = 8 * threadIdx.x; k0 < K; k0 += 8 * 256) {
        double2 v[8];
        smem_chunk8(rowbuf, k0, K, v);
        bimg_chunk_f16<BN>(img_nt, n, k0, v, s);
    }
}

// Rows of up to 2 * FF_ROW_SMEM_K k-values on CTA pairs: each CTA of the pair
// copies its half of the row (a multiple of 8 k-values; at most 64 KB) into its
// shared memory, takes the half's largest magnitude, and the two exchange them
// through distributed shared memory, so that three CTAs per SM overlap their
// copies with the others' conversion.  Both CTAs pass both cluster barriers on
// every path (a copy that does not land within `wait_limit` cycles sets bit
// 0x200 of *err, and that CTA writes nothing).  Grid (2 * rows, planes).
template <int BN>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(256)
    bimg_convert_pair_kernel(const double2* src, long plane_stride, int rows, int K, const int* planes, int kstages,
                             uint8_t* img, float* scale, int* err, long long wait_limit) {
    extern __shared__ __align__(16) uint8_t smem_row[];
    double2* rowbuf = (double2*)smem_row;
    __shared__ __align__(8) uint64_t bar;
    __shared__ unsigned long long half_max;
    __shared__ int ok;
    const uint32_t rank = tc::cluster_rank();
    const int n = blockIdx.x >> 1, b = blockIdx.y;
    const int f = planes ? planes[b] : b;
    const double2* row = src + (long)f * plane_stride + (long)n * K;
    const int Kh = ((K + 15) / 16) * 8;  // the first half: a multiple of 8 k-values
    const int k0 = rank ? Kh : 0, k1 = rank ? K : min(K, Kh), nk = max(0, k1 - k0);
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
        const uint32_t bytes = (uint32_t)nk * 16u;
        int good = 1;
        if (bytes) {
            tc::mbar_arrive_expect_tx(&bar, bytes);
            for (uint32_t o = 0; o < bytes; o += 16384u)
                tc::bulk_g2s(smem_row + o, (const uint8_t*)(row + k0) + o, min(16384u, bytes - o), &bar);
            good = tc::mbar_wait(&bar, 0, wait_limit) ? 1 : 0;
            if (!good) {
                atomicOr(err, 0x200);
                tc::mbar_wait(&bar, 0, DRAIN_LIMIT);
            }
        }
        ok = good;
    }
    __syncthreads();
    unsigned long long mx = 0;
    if (ok)
        for (int k = threadIdx.x; k < nk; k += 256) mx = max(mx, abs_bits2(rowbuf[k]));
    mx = block_max_u64(mx);
    if (threadIdx.x == 0) half_max = mx;
    tc::cluster_sync();  // both halves' maxima are in shared memory
    uint32_t peer;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(peer) : "r"(tc::smem_u32(&half_max)), "r"(rank ^ 1u));
    unsigned long long other;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(other) : "r"(peer) : "memory");
    tc::cluster_sync();  // the peer's value was read before either CTA may exit
    const int k2 = f16_row_shift(max(mx, other));
    const float s = pow2f(k2);
    if (rank == 0 && threadIdx.x == 0) scale[(long)b * rows + n] = pow2f(-k2);
    if (!ok) return;
    const int NT = (rows + BN - 1) / BN;
    uint8_t* img_nt = img + (((long)b * NT + n / BN) * kstages) * ((long)FF_BSUB * BN * 64);
    for (int j0 = 8 * threadIdx.x; j0 < nk; j0 += 8 * 256) {
        double2 v[8];
        smem_chunk8(rowbuf, j0, nk, v);
        bimg_chunk_f16<BN>(img_nt, n, k0 + j0, v, s);
    }
}

// Zeros the image positions that no converter writes: rows past a tile's
// valid rows and k-values past K.  Valid rows of tile nt: 3*min(gpp_cols,
// cols - gpp_cols*nt) when gpp_cols > 0 (GPP: gpp_cols igp triples per tile),
// else min(ROWS, cols - ROWS*nt).  NS sub-tiles per stage (six for the GPP
// images and the FF B images, four for FF's A image).  Grid (kstages, NT, planes).
template <int ROWS, int NS = NSUB>
__global__ void img_pad_kernel(uint8_t* img, int NT, int kstages, int cols, int gpp_cols, int K) {
    const int kst = blockIdx.x, nt = blockIdx.y, pl = blockIdx.z;
    const int vr = gpp_cols > 0 ? 3 * min(gpp_cols, cols - gpp_cols * nt) : min(ROWS, cols - ROWS * nt);
    const int kv = min(BK, K - kst * BK);  // valid k-values of this stage
    if (vr >= ROWS && kv >= BK) return;
    uint8_t* st = img + (((long)pl * NT + nt) * kstages + kst) * (long)(ROWS * NS * 64);
    for (int i = threadIdx.x; i < ROWS * BK; i += blockDim.x) {
        const int row = i / BK, k = i % BK;
        if (row < vr && k < kv) continue;
        const uint32_t off = tc::sw64_offset(row, k);
#pragma unroll
        for (int q = 0; q < NS; ++q) *(uint16_t*)(st + q * ROWS * 64 + off) = 0;
    }
}
// True when some image position needs img_pad_kernel.
inline bool img_needs_pad(int rows_per_tile, int cols, int gpp_cols, int K) {
    if (K % BK) return true;
    if (gpp_cols > 0) return 3 * gpp_cols < rows_per_tile || cols % gpp_cols;
    return cols % rows_per_tile != 0;
}

// FF: FP64 rows [rows][K] -> the A image [mt][kstage][re h, re l, im h, im l][BM][64 B],
// image row m holding source row rowmap[m] (or m) scaled by its own 2^k
// (scale[m] = 2^-k).  One block of 256 threads per row.
static __global__ void __launch_bounds__(256) aimg_convert_kernel(const double2* src, int rows, int K, int kstages,
                                                                  uint8_t* img, const int* rowmap, float* scale) {
    const int m = blockIdx.x;
    const double2* row = src + (long)(rowmap ? rowmap[m] : m) * K;
    const int k2 = f16_row_shift(row_max_bits(row, K));
    const float s = pow2f(k2);
    if (threadIdx.x == 0) scale[m] = pow2f(-k2);
    uint8_t* tile = img + ((long)(m / BM) * kstages) * (long)(BM * 4 * 64);
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const double2 v = row[k];
        uint8_t* st = tile + (long)(k / BK) * (BM * 4 * 64);
        const uint32_t off = tc::sw64_offset(m % BM, k % BK);
        uint16_t h, l;
        split_f16(f64_to_f32_bits(v.x) * s, h, l);
        *(uint16_t*)(st + 0 * BM * 64 + off) = h;
        *(uint16_t*)(st + 1 * BM * 64 + off) = l;
        split_f16(f64_to_f32_bits(v.y) * s, h, l);
        *(uint16_t*)(st + 2 * BM * 64 + off) = h;
        *(uint16_t*)(st + 3 * BM * 64 + off) = l;
    }
}

// The BF16 A image [mt][kstage][re h, m, l, im h, m, l][BM][64 B] of 8
// consecutive k-values k0.. (k0 % 8 == 0) of image row m: the pieces the
// converter warps make (the same FP32 rounding and split), one 16-byte swizzle
// chunk per sub-tile.
__device__ __forceinline__ void aimg_chunk_split3(uint8_t* img, int kstages, int m, int k0, const double2 (&v)[8]) {
    uint32_t pk[6][4];  // sub-tile (re h, m, l, im h, m, l) x four bf16 pairs
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
        uint16_t a0, b0, c0, a1, b1, c1;
        split3(f64_to_f32_bits(v[j].x), a0, b0, c0);
        split3(f64_to_f32_bits(v[j + 1].x), a1, b1, c1);
        pk[0][j / 2] = (uint32_t)a0 | ((uint32_t)a1 << 16);
        pk[1][j / 2] = (uint32_t)b0 | ((uint32_t)b1 << 16);
        pk[2][j / 2] = (uint32_t)c0 | ((uint32_t)c1 << 16);
        split3(f64_to_f32_bits(v[j].y), a0, b0, c0);
        split3(f64_to_f32_bits(v[j + 1].y), a1, b1, c1);
        pk[3][j / 2] = (uint32_t)a0 | ((uint32_t)a1 << 16);
        pk[4][j / 2] = (uint32_t)b0 | ((uint32_t)b1 << 16);
        pk[5][j / 2] = (uint32_t)c0 | ((uint32_t)c1 << 16);
    }
    uint8_t* st = img + ((long)(m / BM) * kstages + k0 / BK) * (long)(BM * NSUB * 64);
    const uint32_t off = tc::sw64_offset(m % BM, k0 % BK);  // 16-byte aligned: k0 % 8 == 0
#pragma unroll
    for (int q = 0; q < NSUB; ++q) *(uint4*)(st + q * BM * 64 + off) = make_uint4(pk[q][0], pk[q][1], pk[q][2], pk[q][3]);
}

// GPP over many n-tiles: FP64 rows [rows][K] -> the BF16 A image, every
// position of the padded extent (rows up to a whole number of 128-row tiles,
// kstages * 32 k-values) written, zeros outside the rows and K.  One thread per
// 8 k-values; grid (ceil(kstages * 4 / blockDim), padded rows).
static __global__ void aimg_split3_kernel(const double2* src, int rows, int K, int kstages, uint8_t* img) {
    const int k0 = 8 * (blockIdx.x * blockDim.x + threadIdx.x), m = blockIdx.y;
    if (k0 >= kstages * BK) return;
    double2 v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (m < rows && k0 + j < K) ? src[(long)m * K + k0 + j] : make_double2(0.0, 0.0);
    aimg_chunk_split3(img, kstages, m, k0, v);
}

// Host: how many CTA pairs of a pair kernel can be resident at once with
// `smem` bytes of dynamic shared memory (at most `cap`), so that a persistent
// launch never leaves pairs waiting for a second wave.  (Callers keep the
// answer: it depends only on the kernel and the device.)
template <class K>
inline int resident_pairs(K kernel, size_t smem, int threads, int cap) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * (unsigned)cap);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    int m = 0;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveClusters(&m, (const void*)kernel, &cfg) != cudaSuccess || m <= 0) {
        cudaGetLastError();
        m = cap;
    }
    return std::max(1, std::min(m, cap));
}

// Host: A (rows of complex FP64, row stride lda complex elements) as a 2-D FP64
// tensor map for tma_load_2d: inner extent 2*K doubles, `rows` rows, box
// BK doubles (half a stage) x BM rows, elements outside the extents read as zero.  The
// encoder comes from the CUDA driver API through the runtime, so the library links
// only the CUDA runtime.
inline cudaError_t encode_rows_map(CUtensorMap* map, const double2* A, long lda, int K, int rows) {
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static const Encode fn = []() -> Encode {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (Encode)f;
    }();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)2 * K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)lda * sizeof(double2)};
    const cuuint32_t box[2] = {BK, BM};  // half a stage: BK/2 complex values of BM rows
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void*)A, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace tcx
}  // namespace fk
