// fk_ff.cu -- FF full-frequency self-energy on sm_103a.
//
// Reference: the kernel sequence of FFKer_cori/ffKernel.cpp:480-503.  Every
// band sum there is a contraction over ig of aqsntemp[n1][ig] with a
// frequency plane of I_epsR / I_epsA, weighted by conj(aqsmtemp[n1][igp]) (and
// vcoul[igp]) and summed over igp:
//   achsDtemp_Kernel (:107-131)         plane 1 of I_epsR, all bands
//   asxDtemp_Kernel  (:133-153)         planes ifreq, ifreq+1 of I_epsR, n1 < nvband
//   achDtemp_cor_Kernel (:212-300)      planes ifreq, ifreq+1 of I_epsR - I_epsA
//   schDt_matrix (.back1 :402-418)      every plane of I_epsR, no vcoul
// so the library runs one batched complex contraction per eps array over the
// planes that are needed (fk_gemm.cuh, EPI_FF), producing per (n1, plane)
//   RW = sum_igp vcoul*conj(aqsm)*S,   RS = sum_igp conj(aqsm)*S,
// and then evaluates the reference's scalar epilogues (compute_fact,
// calculate_schDt_lin3, achDtemp_Kernel's frequency sums) in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fk_gemm.cuh"
#include "fk_internal.h"
#include "fk_tc_contract.cuh"
#include <cstdlib>

namespace fk {
namespace {

__global__ void ff_igp_kernel(int ng, int nc, const int* inv, const int* indinv, int* igp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    int ind = inv[i];
    int g = (ind >= 0 && ind < nc) ? indinv[ind] : -1;
    igp[i] = (g >= 0 && g < nc) ? g : -1;
}

// Sum the (KS x NT) partial slots of each (batch, row, group) and scatter into
// the per-plane tables RW/RS [nb][nf]; partial row i belongs to band order[i]
// (or i).  One warp per (row, batch); lane 4g + c takes component c (RW re, RW
// im, RS re, RS im) of slots g, g+8, .. in order, so that the four lanes of a
// slot read its 32-byte (RW, RS) record as one sector, then three shuffle
// levels add the eight slot groups (fixed order: deterministic).  GB300's FP64
// pipe retires one warp instruction per 64 cycles per sub-partition: this takes
// slots/8 + 3 FP64 adds per warp.
__global__ void ff_rows_kernel(int nb, int nf, int batches, int slots_per_batch, const int* planes,
                               const double2* P, double2* RW, double2* RS, const int* order) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), b = blockIdx.y, lane = threadIdx.x & 31;
    if (i >= nb || b >= batches) return;  // warp-uniform
    const int g = lane >> 2, comp = lane & 3;
    const double* q = (const double*)(P + ((long)b * slots_per_batch * nb + i) * 2) + comp;
    const long sstride = 4L * nb;  // doubles per slot
    const int ns = slots_per_batch;
    double v = 0.0;
    for (int s0 = g; s0 < ns; s0 += 64) {
        double a[8];  // eight loads in flight; clamped indices, +0.0 past the end (exact)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = q[(long)min(s0 + 8 * j, ns - 1) * sstride];
#pragma unroll
        for (int j = 0; j < 8; ++j) v = __dadd_rn(v, s0 + 8 * j < ns ? a[j] : 0.0);
    }
#pragma unroll
    for (int off = 4; off < 32; off <<= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (lane >= 4) return;
    const int n1 = order ? order[i] : i;
    const int f = planes[b];
    if (comp < 2) ((double*)(RW + (long)n1 * nf + f))[comp] = v;
    else if (RS) ((double*)(RS + (long)n1 * nf + f))[comp - 2] = v;
}

struct FactRow {
    int ifq_a, ifq_c, kind;  // kind: 0 none, 1 schDttt_corKernel1, 2 schDttt_corKernel2
    double fa1, fa2, fc1, fc2;
};

struct EpiArgs {
    int nb, nv, nf, ne;
    const double2 *RW, *RS, *AW;  // [nb][nf]
    const FactRow* fact;
    const double *ekq, *grid, *pref;
    const double2* brd;
    double pref_zb, fmin, fstep, fminI, fstepI, occ;
    unsigned flags;
    double2* SD;   // [ne][nb] achDtemp per band
    double2* out;  // [achs | asx ne | achD ne | cor ne | a2 ne | schDt nb*nf]
};

// schDt value used by achDtemp_Kernel: RS when the band x G x G' contraction
// is requested, zero otherwise (FFKer_cori/ffKernel.cpp:421-422).
FK_DEV double2 schdt_of(const EpiArgs& a, int n1, int f) {
    return (a.flags & FK_FF_SCHDT_GEMM) ? a.RS[(long)n1 * a.nf + f] : make_double2(0.0, 0.0);
}

// GPUComplex_divide(a, b), FFKer_cori/Complex.h:201-211.
FK_DEV double2 gc_div(double2 a, double2 b) {
    double2 bc = cconj(b);
    double2 num = cmul(a, bc), den = cmul(b, bc);
    return make_double2(__ddiv_rn(num.x, den.x), __ddiv_rn(num.y, den.x));
}

// achDtemp_Kernel's schDi sum (FFKer_cori/ffKernel.cpp:199-206): for each
// (iw, n1), sum over ifreq of -((0, pref[f]) x schDt[n1][f]) / (wx - coh[f]),
// coh[f] = (grid[f] - brd[f].re, 0 - brd[f].im), wx = freqevalmin - ekq[n1] +
// (iw-1)*freqevalstep.  The (n1, f) numerator and the f terms do not depend on
// iw: they are formed once here (same FP64 operations as inside the loop), and
// for the mixed path also as FP32 tables, with coh.re split into a float-float
// pair so that the nearly cancelling difference wx - coh.re keeps its accuracy.
struct SchdiTab {
    double2 *num, *coh;  // [nb][nf], [nf]
    float4* f32;         // [nb][nf]: (num.re, num.im, -coh.im, 0) as FP32
    float2* cohr;        // [nf]: coh.re as (hi, lo)
};

__global__ void ff_schdi_tables_kernel(EpiArgs a, SchdiTab t) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x, n1 = blockIdx.y;
    if (f >= a.nf) return;
    const double2 coh = make_double2(__dsub_rn(a.grid[f], a.brd[f].x), 0.0 - a.brd[f].y);
    const double2 num = cmul(make_double2(0.0, a.pref[f]), schdt_of(a, n1, f));
    t.num[(long)n1 * a.nf + f] = num;
    if (n1 == 0) t.coh[f] = coh;
    if (t.f32) {
        t.f32[(long)n1 * a.nf + f] =
            make_float4(f64_to_f32_bits(num.x), f64_to_f32_bits(num.y), f64_to_f32_bits(0.0 - coh.y), 0.f);
        if (n1 == 0) {
            const float hi = f64_to_f32_bits(coh.x);
            t.cohr[f] = make_float2(hi, f64_to_f32_bits(coh.x - (double)hi));
        }
    }
}

// FP64: the reference's operations per term (GPUComplex_divide), block = one band,
// threads = consecutive iw, so every f-table load is uniform across the warp.
__global__ void ff_schdi_kernel(EpiArgs a, SchdiTab t) {
    const int iw = blockIdx.x * blockDim.x + threadIdx.x, n1 = blockIdx.y;
    if (iw >= a.ne) return;
    double2 s = make_double2(0.0, 0.0);
    const double wx = a.fmin - a.ekq[n1] + (iw - 1) * a.fstep;
    const double2* num = t.num + (long)n1 * a.nf;
    for (int f = 0; f < a.nf; ++f) {
        const double2 coh = t.coh[f];
        const double2 q = gc_div(num[f], make_double2(__dsub_rn(wx, coh.x), 0 - coh.y));
        s = cadd(s, make_double2(0.0 - q.x, 0.0 - q.y));
    }
    a.SD[(long)iw * a.nb + n1] = s;
}

// Mixed: the same sum in FP32.  wx - coh.re = (wx_hi - coh_hi) + (wx_lo - coh_lo):
// the first difference is exact when the two are close (Sterbenz), so the
// denominator keeps full relative accuracy where it is small; terms are added
// in FP32 over 32 frequencies, then into a float-float (TwoSum) accumulator.
__global__ void ff_schdi32_kernel(EpiArgs a, SchdiTab t) {
    const int iw = blockIdx.x * blockDim.x + threadIdx.x, n1 = blockIdx.y;
    if (iw >= a.ne) return;
    const double wx = a.fmin - a.ekq[n1] + (iw - 1) * a.fstep;
    const float wh = f64_to_f32_bits(wx), wl = f64_to_f32_bits(wx - (double)wh);
    const float4* tab = t.f32 + (long)n1 * a.nf;
    ff32 ar{0.f, 0.f}, ai{0.f, 0.f};
    for (int f0 = 0; f0 < a.nf; f0 += 32) {
        float sr = 0.f, si = 0.f;
        const int f1 = min(a.nf, f0 + 32);
        for (int f = f0; f < f1; ++f) {
            const float4 c = tab[f];
            const float2 ch = t.cohr[f];
            const float dr = (wh - ch.x) + (wl - ch.y), di = c.z;
            const float r = __frcp_rn(fmaf(dr, dr, di * di));
            // -(c / d) = -(c * conj(d)) / |d|^2
            sr -= fmaf(c.x, dr, c.y * di) * r;
            si -= fmaf(c.y, dr, -(c.x * di)) * r;
        }
        ff_add(ar, sr);
        ff_add(ai, si);
    }
    a.SD[(long)iw * a.nb + n1] = make_double2((double)ar.hi + (double)ar.lo, (double)ai.hi + (double)ai.lo);
}

FK_DEV void bsum(double2& v, double2* sm) {
    for (int off = 16; off > 0; off >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, off);
        v.y += __shfl_down_sync(0xffffffffu, v.y, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = cadd(s, sm[w]);
        v = s;
    }
}

// One block per output iw (blockIdx.x < ne) plus one block for the
// iw-independent scalars (blockIdx.x == ne).
__global__ void ff_epilogue_kernel(EpiArgs a) {
    __shared__ double2 sm[32];
    const int tid = threadIdx.x, iw = blockIdx.x;
    // iw-independent sums, computed redundantly per block (tiny)
    double2 achs = make_double2(0, 0), asx = achs, cor = achs;
    for (int n1 = tid; n1 < a.nb; n1 += blockDim.x) {
        achs = cadd(achs, a.RW[(long)n1 * a.nf + 1]);
        const FactRow fr = a.fact[n1];
        if (n1 < a.nv) {
            double2 v = cadd(cscale(a.RW[(long)n1 * a.nf + fr.ifq_a], fr.fa1),
                             cscale(a.RW[(long)n1 * a.nf + fr.ifq_a + 1], fr.fa2));
            asx = cadd(asx, cscale(v, a.occ));
        }
        if (fr.kind) {
            const double2 d0 = csub(a.RW[(long)n1 * a.nf + fr.ifq_c], a.AW[(long)n1 * a.nf + fr.ifq_c]);
            const double2 d1 = csub(a.RW[(long)n1 * a.nf + fr.ifq_c + 1], a.AW[(long)n1 * a.nf + fr.ifq_c + 1]);
            double2 v = cadd(cscale(d0, fr.fc1), cscale(d1, fr.fc2));
            if (fr.kind == 2) v = cscale(v, -0.5);
            cor = cadd(cor, v);
        }
    }
    bsum(achs, sm);
    bsum(asx, sm);
    bsum(cor, sm);
    if (iw == a.ne) {
        if (tid == 0) a.out[0] = cscale(achs, -0.5);
        // schDt_matrix output
        for (long i = tid; i < (long)a.nb * a.nf; i += blockDim.x)
            a.out[1 + 4L * a.ne + i] = (a.flags & FK_FF_SCHDT_GEMM) ? a.RS[i] : make_double2(0.0, 0.0);
        return;
    }
    double2 achd = make_double2(0, 0);
    for (int n1 = tid; n1 < a.nb; n1 += blockDim.x) achd = cadd(achd, a.SD[(long)iw * a.nb + n1]);
    bsum(achd, sm);
    if (tid == 0) {
        // sch2Di after achDtemp_Kernel holds the value of its last (n1, ifreq)
        // iteration, which achDtemp_cor_Kernel adds once per band (:191-192, :241).
        double2 last = make_double2(0.0, 0.0);
        const int n1 = a.nb - 1, f = a.nf - 1;
        if (f >= 1) {
            const double right = a.grid[f], left = a.grid[f - 1];
            const double2 R = schdt_of(a, n1, f), L = schdt_of(a, n1, f - 1);
            const double2 avg = cscale(cadd(R, L), 0.5);
            const double ew = a.fminI - a.ekq[n1] + (double)(iw - 1) * a.fstepI;
            double intfact = __ddiv_rn(__dsub_rn(ew, right), __dsub_rn(ew, left));
            if (intfact < 0.0001) intfact = 0.0001;
            if (intfact > 10000) intfact = 10000;
            intfact = -log(intfact);
            last = csub(make_double2(0.0, 0.0), cscale(cmul(make_double2(0.0, a.pref_zb), avg), intfact));
        }
        const int ne = a.ne;
        double2 asx_iw = asx;
        if (!(a.flags & FK_FF_SPLIT_ACHD)) asx_iw = cadd(asx_iw, achd);  // ffKernel.cpp:495
        a.out[1 + iw] = asx_iw;
        a.out[1 + ne + iw] = (a.flags & FK_FF_SPLIT_ACHD) ? achd : make_double2(0.0, 0.0);
        a.out[1 + 2 * ne + iw] = cor;
        a.out[1 + 3 * ne + iw] = cscale(last, (double)a.nb);
    }
}

// compute_fact, FFKer_cori/ffKernel.cpp:30-78 (host copy; the oracle holds
// the same restatement).
void compute_fact(double wx, int nFreq, const double* g, double& fact1, double& fact2, int& ifreq, int loop,
                  bool flag_occ) {
    if (loop == 1 && wx > 0.00) {
        for (int k = 0; k < nFreq - 1; ++k)
            if (wx > g[k] && wx < g[k + 1]) ifreq = k;
        if (ifreq == 0) ifreq = nFreq - 2;
        fact1 = (g[ifreq + 1] - wx) / (g[ifreq + 1] - g[ifreq]);
        fact2 = (wx - g[ifreq]) / (g[ifreq + 1] - g[ifreq]);
    } else if (loop == 1) {
        for (int k = 0; k < nFreq - 1; ++k)
            if (-wx > g[k] && -wx < g[k + 1]) ifreq = k;
        if (ifreq == 0) ifreq = nFreq - 2;
        fact1 = (g[ifreq + 1] + wx) / (g[ifreq + 1] - g[ifreq]);
        fact2 = (-g[ifreq] - wx) / (g[ifreq + 1] - g[ifreq]);
    }
    if (loop == 2 && wx > 0.00) {
        for (int k = 0; k < nFreq - 1; ++k)
            if (wx > g[k] && wx < g[k + 1]) ifreq = k;
        if (ifreq == -1) ifreq = nFreq - 2;
        fact1 = -0.5 * (g[ifreq + 1] - wx) / (g[ifreq + 1] - g[ifreq]);
        fact2 = -0.5 * (wx - g[ifreq]) / (g[ifreq + 1] - g[ifreq]);
    } else if (loop == 2 && flag_occ) {
        wx = -wx;
        ifreq = 0;
        for (int k = 0; k < nFreq - 1; ++k)
            if (wx > g[k] && wx < g[k + 1]) ifreq = k;
        if (ifreq == 0) ifreq = nFreq - 2;
        fact1 = (g[ifreq + 1] - wx) / (g[ifreq + 1] - g[ifreq]);
        fact2 = (wx - g[ifreq]) / (g[ifreq + 1] - g[ifreq]);
    }
}

struct FfPlan {
    std::vector<FactRow> fact;
    std::vector<int> planesR, planesA;
    std::vector<int> groups;      // pipelined requests: copy group q = R planes (q < ngR) or A planes, of the
    int ngR;                      // combined list [planesR | planesA], is [groups[q], groups[q+1])
    int MT, NT, KS, kchunk;
    int BN, kstages;              // tensor-core path (mixed)
    // Mixed path: bands in the order of the A image and the partial sums --
    // those with a correction term grouped by its bracket plane, then the
    // others -- and for each A plane the rows [aLo, aHi) of the bands that read
    // it, contracted with KSa k-slices of kchunka.
    std::vector<int> order, aLo, aHi;
    int KSa = 0, kchunka = 0;
    bool mixed;
    size_t bytes, bytesImgR, bytesImgA, bytesW, bytesAimg;
    size_t bytesScale;  // mixed: 2^-k of every A image row and of every row of the converted planes
};

// k-slices for the persistent tensor-core kernel (see fk_gpp.cu)
void ff_pick_split_tc(long tiles, int K, int sms, int& KS, int& kchunk) {
    const int kmax = std::max(1, K / 256);
    int best = 1;
    double best_cost = 1e30;
    for (int ks = 1; ks <= std::min(kmax, 64); ++ks) {
        const long units = tiles * ks;
        const long waves = (units + sms - 1) / sms;
        const double eff = (double)units / (double)(waves * sms);
        const double cost = (1.0 / eff) * (1.0 + 0.002 * ks);
        if (cost < best_cost - 1e-9) { best_cost = cost; best = ks; }
        if (eff > 0.92 && units >= sms) break;
    }
    kchunk = ((K + best - 1) / best + tcx::BK - 1) / tcx::BK * tcx::BK;
    KS = (K + kchunk - 1) / kchunk;
}

constexpr int FF_PIPE_GROUPS = 8;  // copy groups of a pipelined request at most (events 0..7 of Ctx::pipe_ev)

FfPlan make_plan(const Ctx& c, const FfDev& r, const double* ekq_h, const double* grid_h, bool pipelined) {
    FfPlan p;
    p.mixed = r.prec == FK_MIXED;
    p.fact.resize(r.nb);
    std::vector<char> needR(r.nf, 0), needA(r.nf, 0);
    needR[1] = 1;
    const bool all = (r.flags & FK_FF_SCHDT_GEMM) != 0;
    for (int n1 = 0; n1 < r.nb; ++n1) {
        FactRow fr{0, 0, 0, 0.0, 0.0, 0.0, 0.0};
        const double wx = r.fmin - ekq_h[n1] + r.fstep;
        if (n1 < r.nv) {
            compute_fact(wx, r.nf, grid_h, fr.fa1, fr.fa2, fr.ifq_a, 1, false);
            needR[fr.ifq_a] = needR[fr.ifq_a + 1] = 1;
        }
        const bool occ = n1 < r.nv;
        compute_fact(wx, r.nf, grid_h, fr.fc1, fr.fc2, fr.ifq_c, 2, occ);
        if (wx > 0) fr.kind = occ ? 0 : 1;
        else fr.kind = occ ? 2 : 0;
        if (fr.kind) needR[fr.ifq_c] = needR[fr.ifq_c + 1] = needA[fr.ifq_c] = needA[fr.ifq_c + 1] = 1;
        p.fact[n1] = fr;
    }
    for (int f = 0; f < r.nf; ++f) {
        if (all || needR[f]) p.planesR.push_back(f);
        if (needA[f]) p.planesA.push_back(f);
    }
    // copy groups: the R and A planes share FF_PIPE_GROUPS groups in proportion
    // to their counts.  The first group (computing cannot start before it has
    // landed) and the last (computed after the last copy) are one plane each;
    // the others split the rest evenly.  Each group is one contraction launch,
    // so the k-split is chosen for the largest group.
    const int nR = (int)p.planesR.size(), nA = (int)p.planesA.size();
    p.ngR = 0;
    int gmax = std::max(nR, 1);
    if (pipelined) {
        int gR = nR ? std::max(1, std::min(nR, (FF_PIPE_GROUPS * nR + (nR + nA) / 2) / (nR + nA))) : 0;
        const int gA = nA ? std::max(1, std::min(nA, FF_PIPE_GROUPS - gR)) : 0;
        gR = std::min(gR, FF_PIPE_GROUPS - gA);
        // sizes of n planes in g groups, with a one-plane group at the front (first) or back (last)
        auto split = [](int n, int g, bool one_first, bool one_last, std::vector<int>& out) {
            std::vector<int> sz;
            int lead = 0, tail = 0;
            if (one_first && g >= 2 && n >= 2) { sz.push_back(1); lead = 1; --g; }
            if (one_last && g >= 2 && n - lead >= 2) tail = 1, --g;
            const int rest = n - lead - tail;
            for (int i = 0; i < g; ++i) sz.push_back(rest / g + (i < rest % g ? 1 : 0));
            if (tail) sz.push_back(1);
            for (int s : sz)
                if (s > 0) out.push_back(s);
        };
        std::vector<int> szR, szA;
        split(nR, gR, true, nA == 0, szR);
        split(nA, gA, nR == 0, true, szA);
        p.groups.push_back(0);
        for (int s : szR) p.groups.push_back(p.groups.back() + s);
        p.ngR = (int)szR.size();
        for (int s : szA) p.groups.push_back(p.groups.back() + s);
        gmax = 1;
        for (int s : szR) gmax = std::max(gmax, s);
        for (int s : szA) gmax = std::max(gmax, s);
    }
    const int nplanes = gmax;
    p.bytesImgR = p.bytesImgA = p.bytesW = p.bytesAimg = p.bytesScale = 0;
    if (p.mixed) {
        // the contraction runs on CTA pairs: units of 256 bands (p.MT counts them),
        // over an A image of an even number of 128-row tiles
        p.BN = 64;
        p.kstages = ceil_div(r.nc, tcx::BK);
        p.MT = ceil_div(r.nb, 2 * tcx::BM);
        p.NT = ceil_div(r.ng, p.BN);
        ff_pick_split_tc((long)p.MT * p.NT * nplanes, r.nc, c.sms / 2, p.KS, p.kchunk);
        const size_t bb = tcx::Cfg<64, true>::B_BYTES;
        p.bytesImgR = p.planesR.size() * (size_t)p.NT * p.kstages * bb;
        p.bytesImgA = p.planesA.size() * (size_t)p.NT * p.kstages * bb;
        p.bytesW = 2 * (size_t)r.nb * r.ng * sizeof(float2) + (size_t)r.ng * sizeof(float) + 256;
        p.bytesAimg = (size_t)2 * p.MT * p.kstages * tcx::Cfg<64, true>::A_BYTES;
        p.bytesScale = ((size_t)r.nb + (p.planesR.size() + p.planesA.size()) * (size_t)r.ng) * sizeof(float);
    } else {
        p.BN = d64::BN;
        p.kstages = 0;
        p.MT = ceil_div(r.nb, d64::BM);
        p.NT = ceil_div(r.ng, d64::BN);
        const int tiles = p.MT * p.NT * nplanes;
        p.KS = std::max(1, std::min((c.sms * 2 + tiles - 1) / tiles, std::max(1, r.nc / 256)));
        p.kchunk = ((r.nc + p.KS - 1) / p.KS + 15) / 16 * 16;
        p.KS = (r.nc + p.kchunk - 1) / p.kchunk;
    }
    if (p.mixed) {
        // the correction term of band n1 reads the A planes ifq_c and ifq_c + 1 only
        // (achDtemp_cor_Kernel, FFKer_cori/ffKernel.cpp:212-246): sort the bands by that
        // bracket so that each A plane is contracted over the row tiles of its bands only
        p.order.resize(r.nb);
        for (int i = 0; i < r.nb; ++i) p.order[i] = i;
        std::stable_sort(p.order.begin(), p.order.end(), [&](int a, int b) {
            const int ka = p.fact[a].kind ? p.fact[a].ifq_c : 1 << 30, kb = p.fact[b].kind ? p.fact[b].ifq_c : 1 << 30;
            return ka < kb;
        });
        long tiles = 0;
        for (int f : p.planesA) {
            int lo = -1, hi = -1;
            for (int i = 0; i < r.nb; ++i) {
                const FactRow& fr = p.fact[p.order[i]];
                if (fr.kind && (fr.ifq_c == f || fr.ifq_c + 1 == f)) {
                    if (lo < 0) lo = i;
                    hi = i + 1;
                }
            }
            if (lo < 0) lo = hi = 0;
            p.aLo.push_back(lo);
            p.aHi.push_back(hi);
            tiles += hi > lo ? (hi - 1) / tcx::BM - lo / tcx::BM + 1 : 0;
        }
        // k-slices for the one launch over all A planes' (row tile, n-tile) pairs
        ff_pick_split_tc(std::max(1L, tiles) * p.NT, r.nc, c.sms, p.KSa, p.kchunka);
    }
    const size_t slots = (size_t)p.KS * p.NT * (p.mixed ? tcx::FF_EPI_WARPS : 1);  // partial slots per plane
    const size_t slotsA = p.mixed ? (size_t)p.KSa * p.NT * tcx::FF_EPI_WARPS : slots;
    p.bytes = ((slots * p.planesR.size() + slotsA * p.planesA.size()) * r.nb * 2 + 3 * (size_t)r.nb * r.nf +
               (size_t)r.ne * r.nb + (size_t)r.nb * r.nf + r.nf) * sizeof(double2) +
              (p.mixed ? (size_t)r.nb * r.nf * sizeof(float4) + r.nf * sizeof(float2) : 0) + 4 * 256 +
              r.nb * sizeof(FactRow) + (p.planesR.size() + p.planesA.size()) * sizeof(int) + r.ng * sizeof(int) +
              r.nb * sizeof(int) +
              p.bytesImgR + p.bytesImgA + p.bytesW + p.bytesAimg + p.bytesScale + 20 * 256;
    return p;
}

}  // namespace

size_t ff_workspace(const Ctx& c, const FfDev& r, bool pipelined) {
    std::vector<double> ekq(r.nb), grid(r.nf);
    if (cudaMemcpy(ekq.data(), r.ekq, r.nb * sizeof(double), cudaMemcpyDefault) != cudaSuccess ||
        cudaMemcpy(grid.data(), r.grid, r.nf * sizeof(double), cudaMemcpyDefault) != cudaSuccess)
        return (size_t)-1;
    return make_plan(c, r, ekq.data(), grid.data(), pipelined).bytes;
}

fk_status ff_run(Ctx& c, const FfDev& r, const FfPipe* pipe) {
    std::vector<double> ekq, grid;
    cudaError_t e = cudaSuccess;
    if (!pipe) {
        ekq.resize(r.nb);
        grid.resize(r.nf);
        e = cudaMemcpyAsync(ekq.data(), r.ekq, r.nb * sizeof(double), cudaMemcpyDefault, c.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(grid.data(), r.grid, r.nf * sizeof(double), cudaMemcpyDefault, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "ff: reading ekq/dFreqGrid");
    }
    const FfPlan p = pipe ? make_plan(c, r, pipe->ekq_h, pipe->grid_h, true)
                          : make_plan(c, r, ekq.data(), grid.data(), false);
    cudaStream_t st = c.stream;
    const int nR = (int)p.planesR.size(), nA = (int)p.planesA.size();
    const size_t slots = (size_t)p.KS * p.NT * (p.mixed ? tcx::FF_EPI_WARPS : 1);  // partial slots per plane
    const size_t slotsA = p.mixed ? (size_t)p.KSa * p.NT * tcx::FF_EPI_WARPS : slots;
    int* igp = (int*)c.ws.take(r.ng * sizeof(int));
    int* order = p.mixed ? (int*)c.ws.take(r.nb * sizeof(int)) : nullptr;
    int* planes = (int*)c.ws.take((nR + nA) * sizeof(int));
    FactRow* fact = (FactRow*)c.ws.take(r.nb * sizeof(FactRow));
    double2* PR = (double2*)c.ws.take(slots * std::max(nR, 1) * r.nb * 2 * sizeof(double2));
    double2* PA = nA ? (double2*)c.ws.take(slotsA * nA * r.nb * 2 * sizeof(double2)) : nullptr;
    double2* tabs = (double2*)c.ws.take(3 * (size_t)r.nb * r.nf * sizeof(double2));
    double2* SD = (double2*)c.ws.take((size_t)r.ne * r.nb * sizeof(double2));
    SchdiTab stab{};
    stab.num = (double2*)c.ws.take((size_t)r.nb * r.nf * sizeof(double2));
    stab.coh = (double2*)c.ws.take((size_t)r.nf * sizeof(double2));
    if (p.mixed) {
        stab.f32 = (float4*)c.ws.take((size_t)r.nb * r.nf * sizeof(float4));
        stab.cohr = (float2*)c.ws.take((size_t)r.nf * sizeof(float2));
    }
    uint8_t* imgR = p.bytesImgR ? (uint8_t*)c.ws.take(p.bytesImgR) : nullptr;
    uint8_t* imgA = p.bytesImgA ? (uint8_t*)c.ws.take(p.bytesImgA) : nullptr;
    float2* W = p.bytesW ? (float2*)c.ws.take(p.bytesW) : nullptr;
    uint8_t* Aimg = p.bytesAimg ? (uint8_t*)c.ws.take(p.bytesAimg) : nullptr;
    float* scales = p.bytesScale ? (float*)c.ws.take(p.bytesScale) : nullptr;
    float* ascale = scales;                                              // [nb], image row order
    float* bscaleR = scales ? scales + r.nb : nullptr;                   // [nR][ng]
    float* bscaleA = scales ? bscaleR + (size_t)nR * r.ng : nullptr;     // [nA][ng]
    if (!igp || (p.mixed && !order) || !planes || !fact || !PR || (nA && !PA) || !tabs || !SD || (p.bytesImgR && !imgR) ||
        (p.bytesImgA && !imgA) || (p.bytesW && !W) || (p.bytesAimg && !Aimg) || (p.bytesScale && !scales))
        return fail(c, FK_ENOMEM, "workspace too small for FF request");
    double2 *RW = tabs, *RS = tabs + (size_t)r.nb * r.nf, *AW = tabs + 2 * (size_t)r.nb * r.nf;
    // host tables -> device (pageable source; the copy completes before return of the call's sync)
    std::vector<int> pl(p.planesR);
    pl.insert(pl.end(), p.planesA.begin(), p.planesA.end());
    e = cudaMemcpyAsync(planes, pl.data(), pl.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fact, p.fact.data(), r.nb * sizeof(FactRow), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && order)
        e = cudaMemcpyAsync(order, p.order.data(), r.nb * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(tabs, 0, 3 * (size_t)r.nb * r.nf * sizeof(double2), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "ff: tables");
    c.launches = 0;
    // pipelined request: the planes each group reads, in runs of consecutive
    // planes, on the copy stream; group q is followed by pipe_ev[q]
    const int ngroups = pipe ? (int)p.groups.size() - 1 : 0;
    if (pipe) {
        const size_t plane = (size_t)r.ng * r.nc;
        auto copy_group = [&](const std::vector<int>& pls, int i0, int i1, const double2* src, double2* dst, int q) {
            cudaError_t ce = cudaSuccess;
            for (int i = i0; i < i1 && ce == cudaSuccess;) {
                int j = i + 1;
                while (j < i1 && pls[j] == pls[j - 1] + 1) ++j;
                const size_t off = (size_t)pls[i] * plane;
                ce = cudaMemcpyAsync(dst + off, src + off, (size_t)(j - i) * plane * sizeof(double2),
                                     cudaMemcpyHostToDevice, c.copy_stream);
                c.h2d_bytes += (size_t)(j - i) * plane * sizeof(double2);
                i = j;
            }
            if (ce == cudaSuccess) ce = cudaEventRecord(c.pipe_ev[q], c.copy_stream);
            return ce;
        };
        for (int q = 0; q < ngroups && e == cudaSuccess; ++q) {
            const bool isR = q < p.ngR;
            const int off = isR ? 0 : nR;  // group bounds count R planes, then A planes
            e = copy_group(isR ? p.planesR : p.planesA, p.groups[q] - off, p.groups[q + 1] - off,
                           isR ? pipe->epsR : pipe->epsA, isR ? pipe->epsR_d : pipe->epsA_d, q);
        }
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, c.pipe_ev[PIPE_READY], 0);
        if (e != cudaSuccess) return cuda_fail(c, e, "ff: plane copies");
    }

    phase_mark(c, 1);
    ff_igp_kernel<<<ceil_div(r.ng, 128), 128, 0, st>>>(r.ng, r.nc, r.inv, r.indinv, igp);
    ++c.launches;
    phase_mark(c, 2);
    if (p.mixed) {
        tcx::weight_table_kernel<<<dim3(ceil_div(r.nb, 128), r.ng), 128, 0, st>>>(r.nb, 0, r.ng, r.aqsm, r.nc, r.vcoul,
                                                                                igp, igp, 1.0, W, W + (size_t)r.nb * r.ng,
                                                                                (float*)(W + 2 * (size_t)r.nb * r.ng), order);
        // aqsntemp is reused by every (plane, n-tile): split it to FP16 pieces once
        // (an even number of 128-row tiles: rows past number_bands are zeros)
        const int MTa = 2 * p.MT;
        if (tcx::img_needs_pad(tcx::BM, r.nb, 0, r.nc) || MTa * tcx::BM > r.nb) {
            tcx::img_pad_kernel<tcx::BM, 4><<<dim3(p.kstages, MTa, 1), 256, 0, st>>>(Aimg, MTa, p.kstages, r.nb, 0, r.nc);
            ++c.launches;
        }
        tcx::aimg_convert_kernel<<<r.nb, 256, 0, st>>>(r.aqsn, r.nb, r.nc, p.kstages, Aimg, order, ascale);
        c.launches += 2;
        cudaMemsetAsync(c.errword, 0, sizeof(int), st);
    }
    // a0 < 0: R planes, all bands on CTA pairs; a0 >= 0: the A planes a0 .. a0+nb_-1
    // of planesA, each over the row tiles of the bands that read it
    auto contract = [&](const double2* eps, const int* pls, int nb_, double2* P, uint8_t* img, float* bsc,
                        int a0) {
        ContractArgs a{};
        a.A = r.aqsn; a.lda = r.nc; a.m0 = 0; a.M = r.nb;
        a.B = eps; a.ldb = r.nc; a.bstride = (long)r.ng * r.nc; a.N = r.ng; a.K = r.nc;
        a.KS = p.KS; a.kchunk = p.kchunk; a.batches = nb_; a.batch_plane = pls;
        a.aqsm = r.aqsm; a.ldm = r.nc; a.vcoul = r.vcoul; a.igp = igp; a.acol = igp; a.wscale = 1.0; a.G = 2; a.P = P;
        if (p.mixed) {
            // pre-split B planes (FP16 hi/lo, rows scaled), then the tensor-core contraction
            const int NTb = ceil_div(r.ng, 64);
            if (tcx::img_needs_pad(64, r.ng, 0, r.nc)) {
                tcx::img_pad_kernel<64, tcx::FF_BSUB><<<dim3(p.kstages, NTb, nb_), 256, 0, st>>>(img, NTb, p.kstages, r.ng, 0, r.nc);
                ++c.launches;
            }
            // rows up to 4096 k-values through shared memory (bulk copies: the planes
            // start on a 16-byte boundary), else held in registers up to 8192 k-values
            // (one or two chunks of 8 per thread), else read twice
            const dim3 gconv(r.ng, nb_);
            if (r.nc <= tcx::FF_ROW_SMEM_K && ((uintptr_t)eps & 15) == 0) {
                auto kc = tcx::bimg_convert_smem_kernel<64>;
                const int sm = r.nc * 16;
                cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, tcx::FF_ROW_SMEM_K * 16);
                kc<<<gconv, 256, sm, st>>>(eps, a.bstride, r.ng, r.nc, pls, p.kstages, img, bsc, c.errword, c.wait_limit);
            } else if (r.nc <= 2 * tcx::FF_ROW_SMEM_K && ((uintptr_t)eps & 15) == 0) {
                // longer rows: half a row per CTA of a pair, the halves' maxima exchanged
                auto kc = tcx::bimg_convert_pair_kernel<64>;
                const int sm = ((r.nc + 15) / 16) * 8 * 16;
                cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, tcx::FF_ROW_SMEM_K * 16);
                kc<<<dim3(2 * r.ng, nb_), 256, sm, st>>>(eps, a.bstride, r.ng, r.nc, pls, p.kstages, img, bsc, c.errword,
                                                         c.wait_limit);
            } else if (r.nc <= 4096)
                tcx::bimg_convert_kernel<64, 1><<<gconv, 512, 0, st>>>(eps, a.bstride, r.ng, r.nc, pls, p.kstages, img, bsc);
            else if (r.nc <= 8192)
                tcx::bimg_convert_kernel<64, 2><<<gconv, 512, 0, st>>>(eps, a.bstride, r.ng, r.nc, pls, p.kstages, img, bsc);
            else
                tcx::bimg_convert_kernel<64, 0><<<gconv, 512, 0, st>>>(eps, a.bstride, r.ng, r.nc, pls, p.kstages, img, bsc);
            tcx::TcArgs t{};
            t.c = a;
            t.c.batch_plane = nullptr;  // the image is indexed by batch position
            t.Bimg = img;
            t.W1 = W; t.W2 = W + (size_t)r.nb * r.ng; t.ldw = r.nb; t.Aimg = Aimg; t.gpp_cols = 0;
            t.ascale = ascale; t.bscale = bsc;
            t.vcol = (const float*)(W + 2 * (size_t)r.nb * r.ng);
            t.kstages_total = p.kstages;
            t.MT = p.MT; t.NT = p.NT; t.units = p.MT * p.NT * p.KS * nb_;
            t.err = c.errword;
            t.wait_limit = c.wait_limit;
            if (a0 >= 0) {
                // the A planes in one persistent launch (up to 64 planes each): every plane over
                // the row tiles of the bands that read it, with the A k-split, and only the
                // vcoul-weighted sum (AW).  Not bracketed by the kernel timer: the timed launches
                // are the R-plane contraction, whose algorithmic flops the caller counts.
                t.ff_no_rs = 1;
                t.c.batches = 1;
                t.c.KS = p.KSa;
                t.c.kchunk = p.kchunka;
                auto k = tcx::tc_contract_planes_kernel<EPI_FF, 64, true>;
                constexpr size_t smem = tcx::Cfg<64, true>::SMEM;
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                for (int j0 = 0; j0 < nb_; j0 += tcx::TC_MAXPL) {
                    tcx::PlaneTab pt{};
                    pt.islab = (long)p.NT * p.kstages * tcx::Cfg<64, true>::B_BYTES;
                    pt.pslab = (long)slotsA * r.nb * 2;
                    pt.u0[0] = 0;
                    for (int j = j0; j < std::min(nb_, j0 + tcx::TC_MAXPL); ++j) {
                        const int lo = p.aLo[a0 + j], hi = p.aHi[a0 + j], q = pt.n++;
                        pt.mt0[q] = hi > lo ? lo / tcx::BM : 0;
                        pt.MT[q] = hi > lo ? (hi - 1) / tcx::BM - pt.mt0[q] + 1 : 0;
                        pt.u0[q + 1] = pt.u0[q] + pt.MT[q] * p.NT * p.KSa;
                    }
                    if (pt.u0[pt.n] == 0) continue;
                    t.Bimg = img + (long)j0 * pt.islab;
                    t.bscale = bsc + (long)j0 * r.ng;
                    t.c.P = P + (long)j0 * pt.pslab;
                    k<<<std::min(pt.u0[pt.n], c.sms), tcx::THREADS_FF, smem, st>>>(t, pt);
                    ++c.launches;
                }
                ++c.launches;  // the conversion
                return;
            }
            auto k = tcx::tc_contract_pair_kernel<EPI_FF, 64, true>;
            constexpr size_t smem = tcx::Cfg<64, true, true>::SMEM;
            static const int pairs = tcx::resident_pairs(k, smem, tcx::THREADS_FF, c.sms / 2);
            const int grid1 = 2 * std::min(t.units, pairs);
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kernel_begin(c);
            k<<<grid1, tcx::THREADS_FF, smem, st>>>(t);
            kernel_end(c);
            c.launches += 2;
        } else {
            dim3 grid(p.MT, p.NT * p.KS * nb_);
            auto k = d64::contract_kernel<EPI_FF>;
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d64::SMEM);
            kernel_begin(c);
            k<<<grid, d64::THREADS, d64::SMEM, st>>>(a);
            kernel_end(c);
            ++c.launches;
        }
    };
    if (!pipe) {
        if (nR) contract(r.epsR, planes, nR, PR, imgR, bscaleR, -1);
        if (nA) contract(r.epsA, planes + nR, nA, PA, imgA, bscaleA, 0);  // A planes: AW only
    } else {
        // one launch pair per copy group, each after its planes have landed;
        // a group's partials and pre-split image sit at its batch offset
        const size_t pslab = slots * r.nb * 2, pslabA = slotsA * r.nb * 2;
        const size_t islab = (size_t)p.NT * p.kstages * tcx::Cfg<64, true>::B_BYTES;
        for (int q = 0; q < ngroups; ++q) {
            const bool isR = q < p.ngR;
            const int g0 = p.groups[q] - (isR ? 0 : nR), n = p.groups[q + 1] - p.groups[q];
            if (cudaStreamWaitEvent(st, c.pipe_ev[q], 0) != cudaSuccess)
                return cuda_fail(c, cudaGetLastError(), "ff: pipeline wait");
            uint8_t* img = isR ? imgR : imgA;
            float* bs = isR ? bscaleR : bscaleA;
            contract(isR ? r.epsR : r.epsA, planes + (isR ? 0 : nR) + g0, n, isR ? PR + g0 * pslab : PA + g0 * pslabA,
                     img ? img + g0 * islab : nullptr, bs ? bs + (size_t)g0 * r.ng : nullptr, isR ? -1 : g0);
        }
    }
    phase_mark(c, 3);
    if (nR) {
        ff_rows_kernel<<<dim3(ceil_div(r.nb, 4), nR), 128, 0, st>>>(r.nb, r.nf, nR, (int)slots, planes, PR, RW, RS,
                                                                     order);
        ++c.launches;
    }
    if (nA) {
        // (rows outside a plane's tiles give values no band reads)
        ff_rows_kernel<<<dim3(ceil_div(r.nb, 4), nA), 128, 0, st>>>(r.nb, r.nf, nA, (int)slotsA, planes + nR, PA, AW,
                                                                     nullptr, order);
        ++c.launches;
    }
    EpiArgs ea{};
    ea.nb = r.nb; ea.nv = r.nv; ea.nf = r.nf; ea.ne = r.ne;
    ea.RW = RW; ea.RS = RS; ea.AW = AW; ea.fact = fact;
    ea.ekq = r.ekq; ea.grid = r.grid; ea.pref = r.pref; ea.brd = r.brd;
    ea.pref_zb = r.pref_zb; ea.fmin = r.fmin; ea.fstep = r.fstep; ea.occ = r.occ; ea.flags = r.flags;
    const bool phys = (r.flags & FK_FF_PHYSICS) != 0;
    ea.fminI = phys ? r.fmin : (double)(int)r.fmin;
    ea.fstepI = phys ? r.fstep : (double)(int)r.fstep;
    ea.SD = SD; ea.out = r.out;
    ff_schdi_tables_kernel<<<dim3(ceil_div(r.nf, 128), r.nb), 128, 0, st>>>(ea, stab);
    if (p.mixed) ff_schdi32_kernel<<<dim3(ceil_div(r.ne, 128), r.nb), 128, 0, st>>>(ea, stab);
    else ff_schdi_kernel<<<dim3(ceil_div(r.ne, 128), r.nb), 128, 0, st>>>(ea, stab);
    c.launches += 1;
    ff_epilogue_kernel<<<r.ne + 1, 256, 0, st>>>(ea);
    c.launches += 2;
    phase_mark(c, 4);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "ff kernels");
    return FK_OK;
}

}  // namespace fk
