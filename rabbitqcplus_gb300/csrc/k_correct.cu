// Per-anchor correction: shifted-Hamming alignment of every candidate in both
// orientations, orientation choice, candidate filters, MSA build, region
// refinement and the anchor correction decision.
//
// reference: src/cpu_alignment.cpp:32-497 (alignment),
// include/alignmentorientation.hpp:10-92 (orientation),
// include/corrector.hpp:982-1211 (flag and mismatch-ratio filters),
// :1260-1421 (weights, MSA build, refinement), src/msa.cpp:9-173,304-453,532-734
// (MSA, properties, corrected anchor, different-region search).
//
// Float work keeps the reference's operand order and uses explicitly rounded
// intrinsics (the library is also built with --fmad=false): every compare the
// decision makes sees the same float values as the reference's host code.

#include <algorithm>
#include <type_traits>

#include "care_device.cuh"
#include "care_internal.h"

namespace cg {

namespace {

// ---------------------------------------------------------------- alignment

constexpr int kAlignWarps = 4;  // warps per block, one anchor per warp
constexpr unsigned kFull = 0xffffffffu;

struct AlnRes {
    int score, overlap, shift, nOps;
    bool valid;
};

// Warp-cooperative shifted Hamming alignment of one candidate orientation.
//
// Each lane evaluates shifts t = lane, lane+32, ... in the reference's scan
// order (0, 1, .., La-minov, then -1, -2, .., -(Lc-minov)).  The winner is the
// first shift with the smallest score among those whose mismatch count stays
// below int(overlap * maxErrorRate); the reference's early exits only skip
// shifts that cannot win, so evaluating all of them returns its (score, shift).
//
// The non-shifted side of every comparison lives in registers (aR: anchor,
// cR: candidate, hi and lo planes); the shifted side streams from shared
// memory one word per step.  A lane stops once its mismatch count reaches its
// limit (the count only grows), and the warp leaves the word loop when no lane
// is still running.
template <int MAXW>
__device__ __forceinline__ AlnRes align_warp(const uint32_t* __restrict__ aS, const uint32_t* __restrict__ cS, int wp,
                                             const uint32_t (&aR)[2][MAXW], const uint32_t (&cR)[2][MAXW], int La,
                                             int Lc, int minov, float rate) {
    const int tb = La + Lc;
    const int n1 = max(0, La - minov + 1);
    const int n2 = max(0, Lc - minov);
    const int lane = (int)lane_id();
    uint32_t best = 0xffffffffu;
    for (int t0 = 0; t0 < n1 + n2; t0 += 32) {
        const int t = t0 + lane;
        int s = 0, ov = 0;
        if (t < n1) {
            s = t;
            ov = min(La - s, Lc);
        } else if (t < n1 + n2) {
            s = -(t - n1 + 1);
            ov = min(La, Lc + s);
        }
        const int maxErr = (int)__fmul_rn((float)ov, rate);
        bool run = t < n1 + n2 && maxErr > 0 && ov > 0;
        const bool fwdShift = s >= 0;
        const int sl = fwdShift ? s : -s;
        const int parts = (ov + 31) >> 5;
        const int rem = (parts << 5) - ov;
        const int ws = sl >> 5, bs = sl & 31;
        const uint32_t* sh = fwdShift ? aS : cS;
        uint32_t curH = 0, curL = 0;
        if (run) {
            curH = sh[ws];
            curL = sh[wp + ws];
        }
        int m = 0;
#pragma unroll
        for (int i = 0; i < MAXW; i++) {
            const bool act = run && i < parts;
            if (!__any_sync(kFull, act)) break;
            if (act) {
                const uint32_t nxH = sh[ws + i + 1];
                const uint32_t nxL = sh[wp + ws + i + 1];
                const uint32_t hi = __funnelshift_l(nxH, curH, bs);
                const uint32_t lo = __funnelshift_l(nxL, curL, bs);
                const uint32_t oh = fwdShift ? cR[0][i] : aR[0][i];
                const uint32_t ol = fwdShift ? cR[1][i] : aR[1][i];
                uint32_t x = (hi ^ oh) | (lo ^ ol);
                if (i == parts - 1 && rem != 0) x &= 0xffffffffu << rem;
                m += __popc(x);
                curH = nxH;
                curL = nxL;
                if (m >= maxErr) run = false;
            }
        }
        if (run) {
            const int score = m + tb - 2 * ov;
            if (score < tb) {
                const uint32_t key = ((uint32_t)score << 16) | (uint32_t)t;
                best = key < best ? key : best;
            }
        }
    }
    best = __reduce_min_sync(kFull, best);
    AlnRes r;
    int bestShift, bestScore;
    if (best == 0xffffffffu) {
        bestShift = -Lc;
        bestScore = tb;
    } else {
        const int t = (int)(best & 0xffffu);
        bestScore = (int)(best >> 16);
        bestShift = t < n1 ? t : -(t - n1 + 1);
    }
    r.valid = bestShift != -Lc;
    const int cb = max(-bestShift, 0);
    const int ce = min(Lc, La - bestShift);
    r.overlap = ce - cb;
    r.score = bestScore;
    r.shift = bestShift;
    r.nOps = bestScore - tb + 2 * r.overlap;
    return r;
}

// Register-resident variant for reads of at most 32*MAXW bases.
//
// Shifts are split by direction and lane l takes shifts 32k+l (right, anchor
// shifted) and 32k+l+1 (left, candidate shifted), so a lane's bit offset is
// the same in every iteration k and only its word offset advances.  Each lane
// therefore funnel-shifts the shifted sequence once (SA: per anchor, SC: per
// candidate orientation) and iteration k, word i reads SA[k+i] / SC[k+i]
// from registers; the inner loop is XOR/OR/POPC only.  The words compared are
// exactly those of align_warp (padding words are zero), so the result is the
// same.  maxErrTab[ov] holds int(float(ov) * maxErrorRate).
template <int MAXW>
struct ShiftedRegs {
    uint32_t h[2 * MAXW - 1], l[2 * MAXW - 1];
};

template <int MAXW>
__device__ __forceinline__ void load_shifted(ShiftedRegs<MAXW>& r, const uint32_t* __restrict__ hi,
                                             const uint32_t* __restrict__ lo, int wp, int wordOff, int bs) {
#pragma unroll
    for (int j = 0; j < 2 * MAXW - 1; j++) {
        const int x = j + wordOff;
        const uint32_t h0 = x < wp ? hi[x] : 0u, h1 = x + 1 < wp ? hi[x + 1] : 0u;
        const uint32_t l0 = x < wp ? lo[x] : 0u, l1 = x + 1 < wp ? lo[x + 1] : 0u;
        r.h[j] = __funnelshift_l(h1, h0, bs);
        r.l[j] = __funnelshift_l(l1, l0, bs);
    }
}

template <int MAXW, bool LEFT>
__device__ __forceinline__ void scan_direction(const ShiftedRegs<MAXW>& S, const uint32_t (&O)[2][MAXW], int n,
                                               int La, int Lc, int tb, int tBase, const int16_t* maxErrTab,
                                               uint32_t& best) {
    const int lane = (int)lane_id();
#pragma unroll
    for (int k = 0; k < MAXW; k++) {
        if (32 * k >= n) break;
        const int tl = 32 * k + lane;
        const bool active = tl < n;
        const int sl = LEFT ? tl + 1 : tl;
        const int ov = active ? (LEFT ? min(La, Lc - sl) : min(La - sl, Lc)) : 0;
        const int maxErr = maxErrTab[ov];
        const int parts = (ov + 31) >> 5;
        const int rem = (parts << 5) - ov;
        const uint32_t last = 0xffffffffu << rem;  // rem < 32
        // words 0 and 1 without branches: a word past the overlap has mask 0
        const uint32_t mask0 = parts > 1 ? 0xffffffffu : (parts == 1 ? last : 0u);
        const uint32_t mask1 = parts > 2 ? 0xffffffffu : (parts == 2 ? last : 0u);
        int m = __popc(((S.h[k] ^ O[0][0]) | (S.l[k] ^ O[1][0])) & mask0) +
                __popc(((S.h[k + 1] ^ O[0][1]) | (S.l[k + 1] ^ O[1][1])) & mask1);
        bool run = active && maxErr > 0 && m < maxErr;
        // the rest only while some lane of the warp can still be valid
        if (__any_sync(kFull, run && parts > 2)) {
#pragma unroll
            for (int i = 2; i < MAXW; i++) {
                const bool act = run && i < parts;
                if (!__any_sync(kFull, act)) break;
                if (act) {
                    const uint32_t mask = i == parts - 1 ? last : 0xffffffffu;
                    m += __popc(((S.h[k + i] ^ O[0][i]) | (S.l[k + i] ^ O[1][i])) & mask);
                    run = m < maxErr;
                }
            }
        }
        if (run) {
            const int score = m + tb - 2 * ov;
            if (score < tb) {
                const uint32_t key = ((uint32_t)score << 16) | (uint32_t)(tBase + tl);
                best = key < best ? key : best;
            }
        }
    }
}

template <int MAXW>
__device__ __forceinline__ AlnRes align_regs(const ShiftedRegs<MAXW>& SA, const uint32_t (&A)[2][MAXW],
                                             const uint32_t* __restrict__ cHi, const uint32_t* __restrict__ cLo,
                                             int wp, int La, int Lc, int minov, const int16_t* maxErrTab) {
    const int tb = La + Lc;
    const int n1 = max(0, La - minov + 1);
    const int n2 = max(0, Lc - minov);
    const int lane = (int)lane_id();
    uint32_t C[2][MAXW];
#pragma unroll
    for (int i = 0; i < MAXW; i++) {
        C[0][i] = i < wp ? cHi[i] : 0u;
        C[1][i] = i < wp ? cLo[i] : 0u;
    }
    uint32_t best = 0xffffffffu;
    scan_direction<MAXW, false>(SA, C, n1, La, Lc, tb, 0, maxErrTab, best);
    if (n2 > 0) {
        ShiftedRegs<MAXW> SC;
        load_shifted<MAXW>(SC, cHi, cLo, wp, lane == 31 ? 1 : 0, (lane + 1) & 31);
        scan_direction<MAXW, true>(SC, A, n2, La, Lc, tb, n1, maxErrTab, best);
    }
    best = __reduce_min_sync(kFull, best);
    AlnRes r;
    int bestShift, bestScore;
    if (best == 0xffffffffu) {
        bestShift = -Lc;
        bestScore = tb;
    } else {
        const int t = (int)(best & 0xffffu);
        bestScore = (int)(best >> 16);
        bestShift = t < n1 ? t : -(t - n1 + 1);
    }
    r.valid = bestShift != -Lc;
    const int cb = max(-bestShift, 0);
    const int ce = min(Lc, La - bestShift);
    r.overlap = ce - cb;
    r.score = bestScore;
    r.shift = bestShift;
    r.nOps = bestScore - tb + 2 * r.overlap;
    return r;
}

// reference: include/alignmentorientation.hpp:12-66; 1 fwd, 2 rc, 3 none
__device__ int choose_orientation(const AlnRes& f, const AlnRes& r, int La, float ratioParam, int minOverlap,
                                  float maxErr) {
    const int byRatio = (int)__fmul_rn((float)La, ratioParam);
    const int minimumOverlap = byRatio > minOverlap ? byRatio : minOverlap;
    int ret = 3;
    if (f.valid && f.overlap >= minimumOverlap) {
        if (r.valid && r.overlap >= minimumOverlap) {
            const float ratio = __fdiv_rn((float)f.nOps, (float)f.overlap);
            const float rratio = __fdiv_rn((float)r.nOps, (float)r.overlap);
            if (ratio < rratio) {
                if (ratio < maxErr) ret = 1;
            } else if (rratio < ratio) {
                if (rratio < maxErr) ret = 2;
            } else {
                if (ratio < maxErr) ret = f.overlap > r.overlap ? 1 : 2;
            }
        } else {
            if (__fdiv_rn((float)f.nOps, (float)f.overlap) < maxErr) ret = 1;
        }
    } else if (r.valid && r.overlap >= minimumOverlap) {
        if (__fdiv_rn((float)r.nOps, (float)r.overlap) < maxErr) ret = 2;
    }
    return ret;
}

__device__ __forceinline__ uint2 pack_aln(const AlnRes& r, int ori) {
    return make_uint2((uint32_t)(uint16_t)(int16_t)r.shift | ((uint32_t)r.overlap << 16),
                      (uint32_t)(uint16_t)r.nOps | ((uint32_t)ori << 16));
}

// Mismatch-ratio filter of one anchor (include/corrector.hpp:1053-1149 single
// end, 1151-1211 paired end) over its aligned candidates b.aln[base, base+nc),
// writing the kept candidates in order; one warp.
__device__ void filter_anchor(const StoreArg& st, const Params& p, const BatchArg& b, int a, uint32_t base,
                              uint32_t nc) {
    const int lane = (int)lane_id();
    float thr;
    if (!p.paired) {
        uint32_t c0 = 0, c1 = 0, c2 = 0;
        for (uint32_t j = lane; j < nc; j += 32) {
            const uint2 v = b.aln[base + j];
            if ((v.y >> 16) != 3u) {
                const float ratio = __fdiv_rn((float)(int)(int16_t)(v.y & 0xffffu), (float)(v.x >> 16));
                c0 += ratio < p.mm2;
                c1 += ratio < p.mm3;
                c2 += ratio < p.mm4;
            }
        }
        c0 = __reduce_add_sync(kFull, c0);
        c1 = __reduce_add_sync(kFull, c1);
        c2 = __reduce_add_sync(kFull, c2);
        thr = -3.402823466e+38f;  // std::numeric_limits<float>::lowest()
        if (c0 > 0 || c1 > 0 || c2 > 0) {
            if ((float)c0 >= p.goodAlignmentsCountThreshold) thr = p.mm2;
            else if ((float)c1 >= p.goodAlignmentsCountThreshold) thr = p.mm3;
            else if ((float)c2 >= p.goodAlignmentsCountThreshold) thr = p.mm4;
        }
    } else {
        thr = p.pairedThreshold;
    }
    uint32_t kept = 0, aligned = 0;
    for (uint32_t j0 = 0; j0 < nc; j0 += 32) {
        const uint32_t j = j0 + lane;
        bool keep = false, isAligned = false;
        uint2 v = make_uint2(0, 0);
        if (j < nc) {
            v = b.aln[base + j];
            const int ori = (int)(v.y >> 16);
            if (ori != 3) {
                isAligned = true;
                const int ov = (int)(v.x >> 16);
                const int nOps = (int)(int16_t)(v.y & 0xffffu);
                const float ratio = __fdiv_rn((float)nOps, (float)ov);
                keep = ratio < thr;
                if (p.paired && b.paired[base + j]) keep = true;
            }
        }
        const uint32_t m = __ballot_sync(kFull, keep);
        aligned += __popc(__ballot_sync(kFull, isAligned));
        if (keep) {
            const uint32_t pos = kept + __popc(m & ((1u << lane) - 1u));
            const int ov = (int)(v.x >> 16);
            const int nOps = (int)(int16_t)(v.y & 0xffffu);
            const uint32_t cid = b.cand[base + j];
            b.fid[base + pos] = cid;
            b.fshift[base + pos] = (int16_t)(v.x & 0xffffu);
            b.forient[base + pos] = (uint8_t)(v.y >> 16);
            b.flen[base + pos] = st.len[cid];
            // reference: include/hostdevicefunctions.cuh:93-95 (calculateOverlapWeight)
            b.fweight[base + pos] =
                __fsub_rn(1.0f, __fsqrt_rn(__fdiv_rn((float)nOps, __fmul_rn((float)ov, p.maxErrorRate))));
        }
        kept += __popc(m);
    }
    if (lane == 0) {
        b.nfinal[a] = kept;
        atomicAdd(&b.counters[kCounterAligned], (unsigned long long)aligned);
        atomicAdd(&b.counters[kCounterMsaCands], (unsigned long long)kept);
    }
}

// One warp per anchor: align all candidates, choose orientations, apply the
// mismatch-ratio filter and write the filtered candidate list in order.
// Shared memory per warp: anchor hi/lo, candidate fwd hi/lo, rc hi/lo planes.
template <int MAXW, bool REGS>
__global__ void __launch_bounds__(kAlignWarps * 32, REGS ? (MAXW <= 5 ? 6 : 4) : 1) align_filter_kernel(StoreArg st, Params p, BatchArg b,
                                                                        const uint32_t* __restrict__ rawOff) {
    extern __shared__ uint32_t smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = (int)lane_id();
    const int wp = st.wp;
    int16_t* maxErrTab = reinterpret_cast<int16_t*>(smem + kAlignWarps * 6 * wp);
    if (REGS) {
        for (int i = threadIdx.x; i <= st.lmax; i += blockDim.x)
            maxErrTab[i] = (int16_t)(int)__fmul_rn((float)i, p.maxErrorRate);
        __syncthreads();
    }
    const int a = blockIdx.x * kAlignWarps + warp;
    if (a >= b.count) return;
    uint32_t* aS = smem + warp * 6 * wp;
    uint32_t* cS = aS + 2 * wp;
    const uint64_t aid = batch_first(b) + (uint64_t)a;
    const int La = st.len[aid];
    const uint32_t nc = b.ncand[a];
    const uint32_t base = rawOff[a];
    if (nc == 0) {
        if (lane == 0) b.nfinal[a] = 0;
        return;
    }
    const uint32_t* ahl = st.hilo + aid * 4 * (uint64_t)wp;  // forward planes
    for (int i = lane; i < 2 * wp; i += 32) aS[i] = ahl[i];
    __syncwarp();
    uint32_t aR[2][MAXW];
#pragma unroll
    for (int i = 0; i < MAXW; i++) {
        aR[0][i] = i < wp ? aS[i] : 0u;
        aR[1][i] = i < wp ? aS[wp + i] : 0u;
    }
    const int minov = max(p.minOverlap, (int)__fmul_rn((float)La, p.minOverlapRatio));
    ShiftedRegs<MAXW> SA;
    if (REGS) load_shifted<MAXW>(SA, aS, aS + wp, wp, 0, lane);
    for (uint32_t j = 0; j < nc; j++) {
        const uint32_t id = b.cand[base + j];
        const int Lc = st.len[id];
        const uint32_t* chl = st.hilo + (uint64_t)id * 4 * wp;
        __syncwarp();
        for (int i = lane; i < 4 * wp; i += 32) cS[i] = chl[i];
        __syncwarp();
        if (REGS) {
            const AlnRes f = align_regs<MAXW>(SA, aR, cS, cS + wp, wp, La, Lc, minov, maxErrTab);
            const AlnRes r = align_regs<MAXW>(SA, aR, cS + 2 * wp, cS + 3 * wp, wp, La, Lc, minov, maxErrTab);
            const int ori = choose_orientation(f, r, La, p.minOverlapRatio, p.minOverlap, p.orientMaxErrorRate);
            if (lane == 0) b.aln[base + j] = pack_aln(ori == 2 ? r : f, ori);
            continue;
        }
        uint32_t cR[2][MAXW];
#pragma unroll
        for (int i = 0; i < MAXW; i++) {
            cR[0][i] = i < wp ? cS[i] : 0u;
            cR[1][i] = i < wp ? cS[wp + i] : 0u;
        }
        const AlnRes f = align_warp<MAXW>(aS, cS, wp, aR, cR, La, Lc, minov, p.maxErrorRate);
#pragma unroll
        for (int i = 0; i < MAXW; i++) {
            cR[0][i] = i < wp ? cS[2 * wp + i] : 0u;
            cR[1][i] = i < wp ? cS[3 * wp + i] : 0u;
        }
        const AlnRes r = align_warp<MAXW>(aS, cS + 2 * wp, wp, aR, cR, La, Lc, minov, p.maxErrorRate);
        const int ori = choose_orientation(f, r, La, p.minOverlapRatio, p.minOverlap, p.orientMaxErrorRate);
        if (lane == 0) b.aln[base + j] = pack_aln(ori == 2 ? r : f, ori);
    }
    __syncwarp();
    filter_anchor(st, p, b, a, base, nc);
}

// ---------------------------------------------------------------- lane per candidate

// Both reads' planes for the lane kernel: words 0..MAXW (a read of at most
// 32 * MAXW bases and the zero word after it).  Every word a shift reads lies
// at index <= MAXW.
template <int MAXW>
__device__ __forceinline__ void load_planes(uint32_t (&R)[2][MAXW + 1], const uint32_t* __restrict__ hilo, int wp) {
#pragma unroll
    for (int i = 0; i <= MAXW; i++) {
        R[0][i] = i < wp ? hilo[i] : 0u;
        R[1][i] = i < wp ? hilo[wp + i] : 0u;
    }
}

// One direction of the reference's sequential shift scan for one lane
// (src/cpu_alignment.cpp:324-397 right, 408-481 left; the same max_errors,
// score and break).  S: words of the shifted sequence, O: words of the other
// one (hi, lo planes, zero past the read).  Right scan (LEFT false): shift
// sl = 0..n-1 moves the anchor; left scan: sl = 1..n moves the candidate.
//
// A fast rejection for shifts whose overlap has at least 32 bases: with at
// least 64 bases, the mismatches of the overlap's first two words (complete,
// so no masks) against the error limit of the scan's longest overlap, tabMax;
// with 32 to 63 bases, those of the first word against the limit at overlap
// min(63, La, Lc), tab63.  The reference's limit at any shift is
// min(maxErrTab[ov], ...) and the table is non-decreasing, so it is at most
// the bound used, and the words' mismatches are part of the shift's: a shift
// rejected here is rejected there too.  Every other shift takes the
// reference's step.  The direction ends where the reference's does: at the
// first shift whose limit is <= 0, i.e. whose overlap is at most
// max((tb - best) / 2, ovPos - 1), ovPos being the smallest overlap with a
// positive table entry; that point moves only when the best score improves.
// Overlap at shift sl: min(X - sl, Y), X = La and Y = Lc for the right scan
// (anchor shifted), the other way round for the left.
//
// Shifts go by word groups W (sl = 32 W + bb); after each group the shifted
// read's words move down by one, so that word W + i is always S[.][i] and one
// copy of the loop body serves every group (S is consumed).  The lanes of
// `lanes` (one candidate each) walk the shifts in step: every loop bound is
// the same for all of them (warp minimum or maximum of the lanes' own
// bounds), so the common loops carry one test per shift and no per-lane
// exits.  A lane past its own end only sees shifts that its step rejects
// (beyond the end the limit is <= 0, and the step checks the end).
template <int MAXW, bool LEFT>
__device__ __forceinline__ void seq_scan_fast(uint32_t (&S)[2][MAXW + 1], const uint32_t (&O)[2][MAXW + 1], int La,
                                              int Lc, int n, int tb, const int16_t* __restrict__ maxErrTab,
                                              int tabMax, int tab63, int ovPos, unsigned lanes, int& bestScore,
                                              int& bestShift) {
    const int X = LEFT ? Lc : La, Y = LEFT ? La : Lc;
    const int slFast = Y >= 64 ? X - 64 : -1;   // overlap >= 64 up to here
    const int slFast1 = Y >= 32 ? X - 32 : -1;  // overlap >= 32 up to here
    auto stopAt = [&](int best) {
        const int dv = max((tb - best) >> 1, ovPos - 1);  // done once the overlap is <= dv
        return Y <= dv ? 0 : X - dv;
    };
    int stop = min(LEFT ? n + 1 : n, stopAt(bestScore));
    const int fastAll = __reduce_min_sync(lanes, slFast);    // every lane in the two-word tier up to here
    const int fastAny = __reduce_max_sync(lanes, slFast);    // no lane in it past here
    const int fast1All = __reduce_min_sync(lanes, slFast1);  // every lane in a word tier up to here
    auto diff = [&](int bb, int i) {
        return (__funnelshift_l(S[0][i + 1], S[0][i], bb) ^ O[0][i]) |
               (__funnelshift_l(S[1][i + 1], S[1][i], bb) ^ O[1][i]);
    };
    int bb = LEFT ? 1 : 0;
#pragma unroll 1
    for (int base = 0; base < 32 * MAXW; base += 32, bb = 0) {
        const int wStop = __reduce_max_sync(lanes, stop);
        if (base >= wStop) break;
        const int ge = min(32, wStop - base);
        // the reference's step at shift base + bb
        auto step = [&](int bb) {
            const int sl = base + bb;
            if (sl >= stop) return;
            const int ov = min(X - sl, Y);
            const int maxErr = min((int)maxErrTab[ov], bestScore - tb + 2 * ov);  // > 0 before `stop`
            const int parts = (ov + 31) >> 5;
            const uint32_t last = 0xffffffffu << ((parts << 5) - ov);
            const uint32_t mask0 = parts > 1 ? 0xffffffffu : last;
            const uint32_t mask1 = parts > 2 ? 0xffffffffu : (parts == 2 ? last : 0u);
            int m = __popc(diff(bb, 0) & mask0) + __popc(diff(bb, 1) & mask1);
            if (m < maxErr && parts > 2) {
#pragma unroll
                for (int i = 2; i < MAXW; i++) {
                    if (i >= parts || m >= maxErr) break;
                    m += __popc(diff(bb, i) & (i == parts - 1 ? last : 0xffffffffu));
                }
            }
            if (m < maxErr) {
                const int score = m + tb - 2 * ov;
                if (score < bestScore) {
                    bestScore = score;
                    bestShift = LEFT ? -sl : sl;
                    stop = min(stop, stopAt(bestScore));
                }
            }
        };
        // The fast tests only record whether each shift passes (shifted into
        // `pass` from the bottom, so the group's last shift is bit 0); the
        // steps run after the group's tests, each lane's in shift order.
        // The tests do not depend on the best score, so this is the
        // reference's sequence of steps, and lanes that pass at different
        // shifts take their steps together instead of one shift at a time.
        uint32_t pass = 0u;
        // x < 0: the shift passes (its sign bit moves into pass)
        auto record = [&](int x) { pass = __funnelshift_l((uint32_t)x, pass, 1); };
        // shifts where the lanes' tiers differ: each lane tests its own
        // (selected, not branched on, so the lanes stay together)
        auto mixed = [&](int e) {
            for (; bb < e; bb++) {
                const int sl = base + bb;
                const bool two = sl <= slFast, one = sl <= slFast1;
                const int m = __popc(diff(bb, 0)) + (two ? __popc(diff(bb, 1)) : 0);
                record(m - (two ? tabMax : one ? tab63 : 0x7fffffff));
            }
        };
        {  // all lanes: two words
            const int e = min(ge, fastAll + 1 - base);
            if (MAXW <= 5) {  // two shifts per iteration: independent tests, steps in order
                for (; bb + 1 < e; bb += 2) {
                    const int ma = __popc(diff(bb, 0)) + __popc(diff(bb, 1)) - tabMax;
                    const int mb = __popc(diff(bb + 1, 0)) + __popc(diff(bb + 1, 1)) - tabMax;
                    record(ma);
                    record(mb);
                }
            }
            for (; bb < e; bb++) record(__popc(diff(bb, 0)) + __popc(diff(bb, 1)) - tabMax);
        }
        mixed(min(ge, max(bb, fastAny + 1 - base)));
        {  // all lanes: one word
            const int e = min(ge, fast1All + 1 - base);
            if (MAXW <= 5) {  // two shifts per iteration
                for (; bb + 1 < e; bb += 2) {
                    const int ma = __popc(diff(bb, 0)) - tab63, mb = __popc(diff(bb + 1, 0)) - tab63;
                    record(ma);
                    record(mb);
                }
            }
            for (; bb < e; bb++) record(__popc(diff(bb, 0)) - tab63);
        }
        mixed(ge);
        while (__any_sync(lanes, pass != 0u)) {
            if (pass != 0u) {
                const int q = 31 - __clz(pass);  // the earliest shift left
                pass ^= 1u << q;
                step(ge - 1 - q);
            }
        }
#pragma unroll
        for (int k = 0; k < MAXW; k++) {
            S[0][k] = S[0][k + 1];
            S[1][k] = S[1][k + 1];
        }
        S[0][MAXW] = S[1][MAXW] = 0u;
    }
}

// Both directions for one orientation of the candidate (planes at cPlanes);
// A and C are working copies that the scans consume.
template <int MAXW>
__device__ __forceinline__ AlnRes align_seq_fast(const uint32_t* __restrict__ aPlanes,
                                                 const uint32_t* __restrict__ cPlanes, int wp, uint32_t (&A)[2][MAXW + 1],
                                                 uint32_t (&C)[2][MAXW + 1], int La, int Lc, int minov,
                                                 const int16_t* maxErrTab, int ovPos, unsigned lanes) {
    const int tb = La + Lc;
    const int tabMax = maxErrTab[min(La, Lc)];
    const int tab63 = maxErrTab[min(63, min(La, Lc))];
    int bestScore = tb, bestShift = -Lc;
    load_planes<MAXW>(A, aPlanes, wp);
    load_planes<MAXW>(C, cPlanes, wp);
    seq_scan_fast<MAXW, false>(A, C, La, Lc, La - minov + 1, tb, maxErrTab, tabMax, tab63, ovPos, lanes, bestScore,
                               bestShift);
    load_planes<MAXW>(A, aPlanes, wp);
    seq_scan_fast<MAXW, true>(C, A, La, Lc, Lc - minov, tb, maxErrTab, tabMax, tab63, ovPos, lanes, bestScore,
                              bestShift);
    AlnRes r;
    r.valid = bestShift != -Lc;
    const int cb = max(-bestShift, 0);
    const int ce = min(Lc, La - bestShift);
    r.overlap = ce - cb;
    r.score = bestScore;
    r.shift = bestShift;
    r.nOps = bestScore - tb + 2 * r.overlap;
    return r;
}

constexpr int kLaneThreads = 128;

// Whether some shift of one candidate orientation could still tie or beat
// the other orientation's result in the orientation rule.  Every shift whose
// overlap has at least minov (>= 32) bases is tested, both directions (right
// shifts 0 .. La - minov move the anchor against the candidate's first word,
// left shifts 1 .. Lc - minov the candidate against the anchor's): the hi
// plane mismatches of the overlap's first 32 bases, a lower bound of the
// shift's mismatches, against L.  Shifts are tested 32 at a time, fully
// unrolled: each outcome's sign bit moves into a pass word, which is then
// masked to the lane's own shifts.  aHi, cHi: the hi planes (wp words).
template <int MAXW>
__device__ __forceinline__ bool exists_close_shift(const uint32_t* __restrict__ aHi, const uint32_t* __restrict__ cHi,
                                                   int wp, int La, int Lc, int minov, int L, unsigned lanes) {
    bool found = false;
#pragma unroll 1
    for (int dir = 0; dir < 2; dir++) {
        const uint32_t* sh = dir == 0 ? aHi : cHi;
        const uint32_t o0 = dir == 0 ? cHi[0] : aHi[0];
        const int n = dir == 0 ? (Lc >= minov ? La - minov + 1 : 0) : (La >= minov ? Lc - minov + 1 : 0);
        uint32_t R[MAXW + 1];
#pragma unroll
        for (int i = 0; i <= MAXW; i++) R[i] = i < wp ? sh[i] : 0u;
        const int wn = __reduce_max_sync(lanes, n);
#pragma unroll 1
        for (int base = 0; base < wn; base += 32) {
            uint32_t pass = 0u;  // bit 31 - bb: shift base + bb has at most L
#pragma unroll
            for (int bb = 0; bb < 32; bb++) {
                const uint32_t x = __funnelshift_l(R[1], R[0], bb) ^ o0;
                pass = __funnelshift_l((uint32_t)((int)__popc(x) - L - 1), pass, 1);
            }
            const int lo = max(dir - base, 0), hi = min(n - base, 32);  // this lane's shifts [lo, hi)
            const uint32_t mine = lo < hi ? (0xffffffffu >> lo) & ~(hi >= 32 ? 0u : 0xffffffffu >> hi) : 0u;
            found |= (pass & mine) != 0u;
            if (__all_sync(lanes, found)) return true;
#pragma unroll
            for (int k = 0; k < MAXW; k++) R[k] = R[k + 1];
            R[MAXW] = 0u;
        }
    }
    return found;
}

// A deferred candidate: its slot, anchor, and the result of the orientation
// scanned first (shift | overlap << 16, nOps | valid << 16 | orientation << 17).
__device__ __forceinline__ uint4 defer_entry(uint32_t slot, int a, const AlnRes& x, int o) {
    return make_uint4(slot, (uint32_t)a, (uint32_t)(uint16_t)(int16_t)x.shift | ((uint32_t)x.overlap << 16),
                      (uint32_t)(uint16_t)(int16_t)x.nOps | ((uint32_t)x.valid << 16) | ((uint32_t)o << 17));
}

// One thread per (anchor, candidate), warps taking 32-candidate chunks; the
// packed result of the reference's orientation choice at the candidate's
// slot.  uoff = exclusive scan of the per-anchor candidate counts.
//
// The reference aligns both orientations (its sequential shift scan) and
// chooses by the mismatch ratios (choose_orientation).  Here each candidate's
// orientation predicted by its shared minimum (bit 31 of its b.perm entry) is
// scanned first, x1.  If x1 alone would be chosen and no shift of the other
// orientation has at most L = floor(nOps1 * min(La, Lc) / overlap1) + 1
// mismatches (exists_close_shift), the other orientation's best shift, at
// overlap ov <= min(La, Lc), has a ratio of at least nOps1 / overlap1 + 1 /
// ov: more than the float rounding of either ratio, so the rule chooses x1
// as it would with both scans.  Otherwise the candidate is deferred: its
// warp queues it and later scans the other orientation fully in a round of
// 32 deferred candidates, and chooses from both results exactly as the
// reference.  Either way the packed result is the reference's.
template <int MAXW>
__global__ void __launch_bounds__(kLaneThreads, 8) align_lane_kernel(StoreArg st, Params p, BatchArg b,
                                                                  const uint32_t* __restrict__ rawOff,
                                                                  const uint32_t* __restrict__ uoff, uint32_t total) {
    __shared__ int16_t maxErrTab[CG_MAX_READ_LENGTH + 2];
    __shared__ int ovPos;  // smallest overlap whose error limit is positive
    __shared__ uint4 deferred[kLaneThreads / 32][64];
    if (threadIdx.x == 0) ovPos = st.lmax + 1;
    for (int i = threadIdx.x; i <= st.lmax; i += blockDim.x)
        maxErrTab[i] = (int16_t)(int)__fmul_rn((float)i, p.maxErrorRate);
    __syncthreads();
    for (int i = threadIdx.x; i <= st.lmax; i += blockDim.x)  // the table is non-decreasing
        if (maxErrTab[i] > 0 && (i == 0 || maxErrTab[i - 1] <= 0)) ovPos = i;
    __syncthreads();
    const uint64_t first = batch_first(b);
    const int lane = (int)lane_id(), warp = (int)(threadIdx.x >> 5);
    uint4* dq = deferred[warp];
    int queued = 0;  // the warp's deferred candidates (the same in every lane)
    // persistent form: warps take 32-candidate chunks from a shared counter
    // until the batch's candidates (uoff[count], on the device) are done;
    // otherwise one chunk per warp
    unsigned int* const work = b.work ? b.work : b.laneWork;
    if (work) total = uoff[b.count];
    bool chunks = true;
    uint32_t t0 = blockIdx.x * kLaneThreads + warp * 32;
    const int wp = st.wp;
    while (true) {
        // a round: 32 deferred candidates when as many wait, else the next
        // chunk, else what is left deferred
        bool second = queued >= 32;
        if (!second && chunks) {
            if (work) {
                uint32_t c = 0;
                if (lane == 0) c = atomicAdd(&work[0], 32u);
                t0 = __shfl_sync(kFull, c, 0);
            }
            if (t0 >= total) chunks = false;
        }
        if (!second && !chunks) {
            if (queued == 0) return;
            second = true;
        }
        bool has = false, defer = false;
        uint32_t slot = 0;
        int a = 0, o = 0;
        AlnRes x1{};
        if (second) {
            const int cnt = min(queued, 32);
            uint4 e = make_uint4(0u, 0u, 0u, 0u);
            if (lane < cnt) e = dq[lane];
            __syncwarp();
            if (lane + 32 < queued) dq[lane] = dq[lane + 32];
            __syncwarp();
            queued -= cnt;
            has = lane < cnt;
            slot = e.x;
            a = (int)e.y;
            x1.shift = (int)(int16_t)(e.z & 0xffffu);
            x1.overlap = (int)(e.z >> 16);
            x1.nOps = (int)(int16_t)(e.w & 0xffffu);
            x1.valid = ((e.w >> 16) & 1u) != 0u;
            o = 1 - (int)((e.w >> 17) & 1u);  // the orientation not yet scanned
        } else {
            const uint32_t t = t0 + (uint32_t)lane;
            has = t < total;
            if (has) {
                int lo = 0, hi = b.count;  // last anchor with uoff[a] <= t
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (uoff[mid] <= t) lo = mid;
                    else hi = mid;
                }
                a = lo;
                const uint32_t j = t - uoff[a];
                const uint32_t pe = b.perm ? b.perm[rawOff[a] + j] : j;  // position, predicted orientation
                slot = rawOff[a] + (pe & 0x7fffffffu);
                o = (int)(pe >> 31);
            }
        }
        const unsigned lanes = __ballot_sync(kFull, has);  // the warp's lanes with a candidate
        if (has) {
            const uint64_t aid = first + (uint64_t)a;
            const uint32_t id = b.cand[slot];
            const int La = st.len[aid], Lc = st.len[id];
            const int minov = max(p.minOverlap, (int)__fmul_rn((float)La, p.minOverlapRatio));
            const uint32_t* aPl = st.hilo + aid * 4 * (uint64_t)wp;
            const uint32_t* cPl = st.hilo + (uint64_t)id * 4 * wp;
            uint32_t A[2][MAXW + 1], C[2][MAXW + 1];
            const AlnRes x = align_seq_fast<MAXW>(aPl, cPl + 2 * wp * o, wp, A, C, La, Lc, minov, maxErrTab, ovPos,
                                                  lanes);
            if (second) {
                const AlnRes& f = o == 0 ? x : x1;
                const AlnRes& r = o == 0 ? x1 : x;
                const int ori = choose_orientation(f, r, La, p.minOverlapRatio, p.minOverlap, p.orientMaxErrorRate);
                b.aln[slot] = pack_aln(ori == 2 ? r : f, ori);
            } else {
                AlnRes none{};
                none.valid = false;
                const int solo = o == 0 ? choose_orientation(x, none, La, p.minOverlapRatio, p.minOverlap,
                                                             p.orientMaxErrorRate)
                                        : choose_orientation(none, x, La, p.minOverlapRatio, p.minOverlap,
                                                             p.orientMaxErrorRate);
                const bool test = solo != 3 && minov >= 32;
                const unsigned tlanes = __ballot_sync(lanes, test);
                bool close = true;
                if (test) {
                    const int L = (int)(((uint32_t)x.nOps * (uint32_t)min(La, Lc)) / (uint32_t)x.overlap) + 1;
                    close = exists_close_shift<MAXW>(aPl, cPl + 2 * wp * (1 - o), wp, La, Lc, minov, L, tlanes);
                }
                if (!close) b.aln[slot] = pack_aln(x, solo);
                defer = close;
                x1 = x;
            }
        }
        if (!second) {  // queue the deferred candidates of the chunk
            const unsigned dm = __ballot_sync(kFull, defer);
            if (defer) dq[queued + __popc(dm & ((1u << lane) - 1u))] = defer_entry(slot, a, x1, o);
            queued += __popc(dm);
            __syncwarp();
            if (!work) chunks = false;  // one chunk per warp
        }
    }
}

// one warp per anchor: the mismatch-ratio filter after align_lane_kernel
__global__ void __launch_bounds__(128) filter_kernel(StoreArg st, Params p, BatchArg b,
                                                     const uint32_t* __restrict__ rawOff) {
    const int a = (int)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (a >= b.count) return;
    const uint32_t nc = b.ncand[a];
    if (nc == 0) {
        if (lane_id() == 0) b.nfinal[a] = 0;
        return;
    }
    filter_anchor(st, p, b, a, rawOff[a], nc);
}

// ---------------------------------------------------------------- MSA

constexpr int kMsaThreadsMin = 128;
constexpr int kMsaCols = 4;  // columns owned per thread
constexpr int kMsaChunkRows = 512;

struct RowMeta {
    const uint32_t* enc;  // candidate's 2-bit row
    const uint8_t* qual;  // candidate's qualities (or null)
    float weight;
    int16_t shift;
    uint16_t len;
    uint8_t rc;
    uint8_t pad[7];
};
static_assert(sizeof(RowMeta) == 32, "row meta layout");

template <class T>
__device__ __forceinline__ T block_reduce(T v, T* red, int op /*0 min 1 max 2 sum*/) {
    for (int d = 16; d > 0; d >>= 1) {
        const T o = __shfl_xor_sync(kFull, v, d);
        v = op == 0 ? (o < v ? o : v) : op == 1 ? (o > v ? o : v) : v + o;
    }
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    T r = red[0];
    for (int w = 1; w < nw; w++) r = op == 0 ? (red[w] < r ? red[w] : r) : op == 1 ? (red[w] > r ? red[w] : r) : r + red[w];
    return r;
}

// One block per anchor; column c belongs to thread c % blockDim (at most
// kMsaCols columns per thread, kept in registers while the rows stream by).
// Every column adds its rows in list order -- anchor first, then the kept
// candidates as the filters left them -- so each float sum is the
// reference's sequence of additions.  Row metadata is staged in shared memory
// in chunks of kMsaChunkRows rows; removed rows are a shared bitset.
// reference: include/classification.hpp:748-797 (extract_anchor_v3) and
// include/forest.hpp:70-81,217-226 (tree walk; decide: running mean of the
// trees' probabilities, true as soon as it reaches the threshold)
__device__ bool forest_decide(const Params& p, const float* f) {
    float sum = 0.0f;
    for (int t = 0; t < p.numTrees; t++) {
        const ForestNode* tree = p.forestNodes + p.treeOffsets[t];
        uint32_t i = 0;
        float prob = 0.0f;
        for (int guard = 0; guard < (1 << 20); guard++) {
            const ForestNode n = tree[i];
            if ((double)f[n.att] <= n.split) {
                if (n.flag & 2u) { prob = __uint_as_float(n.lhs); break; }
                i = n.lhs;
            } else {
                if (n.flag & 1u) { prob = __uint_as_float(n.rhs); break; }
                i = n.rhs;
            }
        }
        sum = __fadd_rn(sum, prob);
        if (__fdiv_rn(sum, (float)p.numTrees) >= p.forestThreshold) return true;
    }
    return false;
}

__device__ __forceinline__ int base_index(char c) { return c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3; }

// ---------------------------------------------------------------- candidate correction
//
// reference: src/msa.cpp:457-522 (getCorrectedCandidates), include/corrector.hpp
// :293-299 and 1504-1512 (HQ anchors correct their candidates), :1674-1748 (the
// record: the consensus slice, reverse complemented back for a reverse-
// complement candidate).  A row of the final MSA with shift s and length len
// qualifies when -nc <= s <= nc and s + len <= La + nc (nc =
// new_columns_to_correct; the support and coverage test computed there is
// overwritten by `candidateShouldBeCorrected = true`).  Its record votes for
// read `id` (see Params::candVotes).

__device__ __forceinline__ void vote_word(const Params& p, uint64_t read, int w, unsigned long long v) {
    const uint64_t i = read * (uint64_t)p.candPitch + (uint64_t)w;
    atomicAnd(&p.candAnd[i], v);
    atomicOr(&p.candOr[i], v);
}

// One thread votes for one row: cons(col) gives the consensus base code of
// column col (relative to the anchor's first column).  Returns 1 if it voted.
template <class Cons>
__device__ __forceinline__ int vote_candidate(const Params& p, int s, int len, bool rc, uint32_t id, uint64_t aid,
                                              int La, Cons cons) {
    const int nc = p.newColumns;
    if (s < -nc || s > nc || s + len > La + nc) return 0;
    for (int w = 0; w * 32 < len; w++) {
        unsigned long long v = 0;
        const int pe = min(len, w * 32 + 32);
        for (int q = w * 32; q < pe; q++) {
            uint32_t bb = cons(s + (rc ? len - 1 - q : q));
            if (rc) bb = 3u - bb;
            v |= (unsigned long long)bb << (62 - 2 * (q & 31));
        }
        vote_word(p, id, w, v);
    }
    atomicAdd((uint64_t)id > aid ? &p.candVotes[id].x : &p.candVotes[id].y, 1u);
    return 1;
}

// Quality score of position `pos` (aligned orientation) of a candidate row
// (reference: include/corrector.hpp:1214-1239).  Rows hold Lmax scores; past
// the read's end the store holds what the reference's decoded row holds there
// (zero, or the first bin's score with lossy qualities; include/
// chunkedreadstorage.hpp:532-610), and a reverse-complement candidate's whole
// row is reversed, so a read shorter than Lmax starts with that padding: its
// position pos reads score Lmax - 1 - pos.
__device__ __forceinline__ uint8_t row_quality(const uint8_t* q, int lmax, bool rc, int pos) {
    return q[rc ? lmax - 1 - pos : pos];
}

__global__ void __launch_bounds__(1024) msa_correct_kernel(StoreArg st, Params p, BatchArg b,
                                                          const uint32_t* __restrict__ rawOff, int maxCols,
                                                          int bitsetWords, int storeWeights) {
    extern __shared__ __align__(16) unsigned char sm[];
    RowMeta* rows = reinterpret_cast<RowMeta*>(sm);
    uint32_t* removed = reinterpret_cast<uint32_t*>(rows + kMsaChunkRows);
    float* qw = reinterpret_cast<float*>(removed + bitsetWords);
    int* cntA = reinterpret_cast<int*>(qw + 256);
    int* cntC = cntA + maxCols;
    int* cntG = cntC + maxCols;
    int* cntT = cntG + maxCols;
    int* cov = cntT + maxCols;
    int* origCov = cov + maxCols;
    float* sup = reinterpret_cast<float*>(origCov + maxCols);
    // column weights, kept only for the forest's features
    float* colWA = storeWeights ? sup + maxCols : nullptr;
    float* colWC = storeWeights ? colWA + maxCols : nullptr;
    float* colWG = storeWeights ? colWC + maxCols : nullptr;
    float* colWT = storeWeights ? colWG + maxCols : nullptr;
    char* cons = reinterpret_cast<char*>(sup + maxCols + (storeWeights ? 4 * maxCols : 0));
    __shared__ float redf[32];
    __shared__ int redi[32];
    __shared__ int sCol, sFound, sByConsensus;

    const int a = blockIdx.x;
    const int tid = threadIdx.x;
    const int bd = blockDim.x;
    const uint64_t first = batch_first(b);
    const uint64_t aid = first + (uint64_t)a;
    const uint64_t oi = (first - out_first(b)) + (uint64_t)a;  // output row
    const uint32_t nf = b.nfinal[a];
    char* out = b.out + oi * b.outPitch;
    if (nf == 0) {
        if (tid == 0) b.flags[oi] = 0;
        return;
    }
    const uint32_t base = rawOff[a];
    const int La = st.len[aid];
    const uint32_t* aenc = st.enc + aid * (uint64_t)st.pitch;
    const uint8_t* aq = p.useQuality ? st.qual + aid * (uint64_t)st.lmax : nullptr;
    for (int i = tid; i < bitsetWords; i += bd) removed[i] = 0u;
    if (p.useQuality)
        for (int i = tid; i < 256; i += bd) qw[i] = p.qweight[i];
    const bool oneChunk = nf <= (uint32_t)kMsaChunkRows;
    auto loadRows = [&](uint32_t j0, uint32_t cnt) {
        for (uint32_t r = tid; r < cnt; r += bd) {
            const uint32_t j = base + j0 + r;
            const uint32_t id = b.fid[j];
            RowMeta m;
            m.enc = st.enc + (uint64_t)id * st.pitch;
            m.qual = p.useQuality ? st.qual + (uint64_t)id * st.lmax : nullptr;
            m.weight = b.fweight[j];
            m.shift = b.fshift[j];
            m.len = b.flen[j];
            m.rc = b.forient[j] == 2;
            rows[r] = m;
        }
    };
    if (oneChunk) loadRows(0, nf);
    __syncthreads();
    auto isRemoved = [&](uint32_t j) { return (removed[j >> 5] >> (j & 31)) & 1u; };

    int aBegin = 0, nActive = (int)nf, builds = 0;
    for (int iter = 0;; iter++) {
        // columns of the current MSA (src/msa.cpp:19-33)
        int lo = 0, hi = La, act = 0;
        for (uint32_t j = tid; j < nf; j += bd) {
            if (!isRemoved(j)) {
                const int s = b.fshift[base + j];
                lo = min(lo, s);
                hi = max(hi, s + (int)b.flen[base + j]);
                act++;
            }
        }
        lo = block_reduce<int>(lo, redi, 0);
        hi = block_reduce<int>(hi, redi, 1);
        nActive = block_reduce<int>(act, redi, 2);
        const int nCols = hi - lo;
        aBegin = -lo;
        const int aEnd = aBegin + La;
        // build: counts, weights (src/msa.cpp:93-112)
        int nA[kMsaCols], nC[kMsaCols], nG[kMsaCols], nT[kMsaCols];
        float wA[kMsaCols], wC[kMsaCols], wG[kMsaCols], wT[kMsaCols];
#pragma unroll
        for (int k = 0; k < kMsaCols; k++) {
            nA[k] = nC[k] = nG[k] = nT[k] = 0;
            wA[k] = wC[k] = wG[k] = wT[k] = 0.0f;
        }
        auto add = [&](int k, uint32_t bb, float w) {
            if (bb == 0) { nA[k]++; wA[k] = __fadd_rn(wA[k], w); }
            else if (bb == 1) { nC[k]++; wC[k] = __fadd_rn(wC[k], w); }
            else if (bb == 2) { nG[k]++; wG[k] = __fadd_rn(wG[k], w); }
            else { nT[k]++; wT[k] = __fadd_rn(wT[k], w); }
        };
#pragma unroll
        for (int k = 0; k < kMsaCols; k++) {
            const int c = tid + k * bd;
            if (c >= aBegin && c < aEnd) {
                const int pos = c - aBegin;
                const float w = p.useQuality ? __fmul_rn(1.0f, qw[aq[pos]]) : 1.0f;
                add(k, get2bit(aenc, pos), w);
            }
        }
        for (uint32_t j0 = 0; j0 < nf; j0 += kMsaChunkRows) {
            const uint32_t cnt = min((uint32_t)kMsaChunkRows, nf - j0);
            if (!oneChunk) {
                __syncthreads();
                loadRows(j0, cnt);
                __syncthreads();
            }
            for (uint32_t r = 0; r < cnt; r++) {
                if (isRemoved(j0 + r)) continue;
                const RowMeta m = rows[r];
                const int rb = aBegin + m.shift;
                const int re = rb + (int)m.len;
#pragma unroll
                for (int k = 0; k < kMsaCols; k++) {
                    const int c = tid + k * bd;
                    if (c >= rb && c < re) {
                        const int pos = c - rb;
                        const int sp = m.rc ? (int)m.len - 1 - pos : pos;
                        uint32_t bb = get2bit(m.enc, sp);
                        if (m.rc) bb = 3u - bb;
                        float w = m.weight;
                        if (p.useQuality) w = __fmul_rn(w, qw[row_quality(m.qual, st.lmax, m.rc, pos)]);
                        add(k, bb, w);
                    }
                }
            }
        }
        // findConsensus (src/msa.cpp:135-157), findOrigWeightAndCoverage (:159-173)
#pragma unroll
        for (int k = 0; k < kMsaCols; k++) {
            const int c = tid + k * bd;
            if (c < nCols) {
                char cs = 'A';
                float cw = wA[k];
                if (wC[k] > cw) { cs = 'C'; cw = wC[k]; }
                if (wG[k] > cw) { cs = 'G'; cw = wG[k]; }
                if (wT[k] > cw) { cs = 'T'; cw = wT[k]; }
                const float colW = __fadd_rn(__fadd_rn(__fadd_rn(wA[k], wC[k]), wG[k]), wT[k]);
                cntA[c] = nA[k]; cntC[c] = nC[k]; cntG[c] = nG[k]; cntT[c] = nT[k];
                cov[c] = nA[k] + nC[k] + nG[k] + nT[k];
                sup[c] = __fdiv_rn(cw, colW);
                cons[c] = cs;
                if (storeWeights) {
                    colWA[c] = wA[k]; colWC[c] = wC[k]; colWG[c] = wG[k]; colWT[c] = wT[k];
                }
                if (c >= aBegin && c < aEnd) {
                    const uint32_t ab = get2bit(aenc, c - aBegin);
                    origCov[c] = ab == 0 ? nA[k] : ab == 1 ? nC[k] : ab == 2 ? nG[k] : nT[k];
                }
            }
        }
        builds++;
        __syncthreads();
        if (iter == 5 || nActive == 0) break;
        // findCandidatesOfDifferentRegion (src/msa.cpp:532-734)
        bool mism = false;
        for (int c = aBegin + tid; c < aEnd; c += bd) mism |= cons[c] != "ACGT"[get2bit(aenc, c - aBegin)];
        if (!__syncthreads_or(mism)) break;
        if (tid == 0) sCol = 0x7fffffff;
        __syncthreads();
        for (int c = aBegin + tid; c < aEnd; c += bd) {
            const int counts[4] = {cntA[c], cntC[c], cntG[c], cntT[c]};
            const int ci = cons[c] == 'A' ? 0 : cons[c] == 'C' ? 1 : cons[c] == 'G' ? 2 : 3;
            bool sig = false;
            for (int i = 0; i < 4; i++) sig |= (i != ci && p.significantCount <= counts[i]);
            if (sig) atomicMin(&sCol, c);
        }
        __syncthreads();
        const int col = sCol;
        if (col == 0x7fffffff) break;
        if (tid == 0) {
            const int counts[4] = {cntA[col], cntC[col], cntG[col], cntT[col]};
            const int ci = cons[col] == 'A' ? 0 : cons[col] == 'C' ? 1 : cons[col] == 'G' ? 2 : 3;
            int si = -1;
            for (int i = 0; i < 4; i++)
                if (i != ci && p.significantCount <= counts[i]) si = i;
            sFound = si;
        }
        __syncthreads();
        const uint32_t found = (uint32_t)sFound;
        const uint32_t orig = get2bit(aenc, col - aBegin);
        const bool keepMatching = orig == found;
        auto differs = [&](uint32_t j) -> bool {  // row j lies on `col` and is to be removed
            const uint32_t g = base + j;
            const int rb = aBegin + b.fshift[g];
            const int len = b.flen[g];
            if (col < rb || col >= rb + len) return false;
            const uint32_t* e = st.enc + (uint64_t)b.fid[g] * st.pitch;
            const int pos = col - rb;
            const bool rc = b.forient[g] == 2;
            uint32_t bb = get2bit(e, rc ? len - 1 - pos : pos);
            if (rc) bb = 3u - bb;
            return keepMatching ? (bb != found) : (bb == found);
        };
        bool veto = false, any = false;
        for (uint32_t j = tid; j < nf; j += bd) {
            if (isRemoved(j) || !differs(j)) continue;
            any = true;
            veto |= b.fweight[base + j] >= 0.90f;
        }
        const bool anyVeto = __syncthreads_or(veto);
        const bool anyRemove = __syncthreads_or(any);
        // a veto (or nothing to remove) leaves the MSA as it is; the
        // reference then rebuilds the same MSA and reaches the same decision
        if (anyVeto || !anyRemove) break;
        for (uint32_t j = tid; j < nf; j += bd) {
            if (!isRemoved(j) && differs(j)) atomicOr(&removed[j >> 5], 1u << (j & 31));
        }
        __syncthreads();
    }
    // getMSAProperties (src/msa.cpp:304-376) and getCorrectedAnchor (:379-453)
    const int aEnd = aBegin + La;
    float mins = 3.402823466e+38f;
    int minc = 0x7fffffff, maxc = -1;
    for (int c = aBegin + tid; c < aEnd; c += bd) {
        mins = fminf(mins, sup[c]);
        minc = min(minc, cov[c]);
        maxc = max(maxc, cov[c]);
    }
    mins = block_reduce<float>(mins, redf, 0);
    minc = block_reduce<int>(minc, redi, 0);
    maxc = block_reduce<int>(maxc, redi, 1);
    __shared__ float sAvg;
    __shared__ int sHQ;
    if (tid == 0) {
        float sum = 0.0f;
        for (int c = aBegin; c < aEnd; c++) sum = __fadd_rn(sum, sup[c]);
        const float avg = __fdiv_rn(sum, (float)La);
        const bool good = fgeq(avg, p.avgSupportThreshold) && fgeq(mins, p.minSupportThreshold) &&
                          fgeq((float)minc, p.minCoverageThreshold);
        bool hq = false;
        if (good) {
            int smallest = 100;
            for (int percent = p.errPercent; percent >= 0; percent--) {
                if (fgeq(avg, p.hqAvg[percent]) && fgeq(mins, p.hqMin[percent])) smallest = percent;
            }
            hq = fgeq((float)minc, p.minCoverageThreshold) && fleq((float)smallest, p.hqPercentLimit);
        }
        sByConsensus = good;
        sAvg = avg;
        sHQ = hq;
        // the forest decision corrects every anchor that reached the MSA
        // (include/corrector.hpp:1448-1472); the classic one needs candidates
        const bool corrected = p.correctionType == CG_CORR_FOREST || nActive > 0;
        if (corrected) {
            atomicAdd(&b.counters[kCounterCorrected], 1ull);
            if (hq) atomicAdd(&b.counters[kCounterHQ], 1ull);
        }
        atomicAdd(&b.counters[kCounterMsaBuilds], (unsigned long long)builds);
        b.flags[oi] = corrected ? (uint8_t)(CG_RESULT_CORRECTED | (hq ? CG_RESULT_HQ : 0)) : (uint8_t)0;
    }
    __syncthreads();
    if (p.candidates && sHQ) {
        // candidate correction: one thread per row of the final MSA, whose
        // consensus covers every column of the rows
        int votes = 0;
        for (uint32_t j = tid; j < nf; j += bd) {
            if (isRemoved(j)) continue;
            const uint32_t g = base + j;
            votes += vote_candidate(p, b.fshift[g], b.flen[g], b.forient[g] == 2, b.fid[g], aid, La,
                                    [&](int col) { return (uint32_t)base_index(cons[aBegin + col]); });
        }
        votes = block_reduce<int>(votes, redi, 2);
        if (tid == 0 && votes) atomicAdd(&b.counters[kCounterCandidateVotes], (unsigned long long)votes);
    }
    if (p.correctionType == CG_CORR_FOREST) {
        const bool hq = sHQ;
        const float avg = sAvg;
        for (int i = tid; i < La; i += bd) {
            const int c = aBegin + i;
            const uint32_t ab = get2bit(aenc, i);
            const char orig = "ACGT"[ab];
            char r = cons[c];
            if (!hq && r != orig) {
                const float wsum = __fadd_rn(__fadd_rn(__fadd_rn(colWA[c], colWC[c]), colWG[c]), colWT[c]);
                float wCons, nCons;
                switch (r) {
                    case 'A': wCons = colWA[c]; nCons = (float)cntA[c]; break;
                    case 'C': wCons = colWC[c]; nCons = (float)cntC[c]; break;
                    case 'G': wCons = colWG[c]; nCons = (float)cntG[c]; break;
                    default: wCons = colWT[c]; nCons = (float)cntT[c]; break;
                }
                const float wOrig = ab == 0 ? colWA[c] : ab == 1 ? colWC[c] : ab == 2 ? colWG[c] : colWT[c];
                const float cv = (float)cov[c];
                const float oc = (float)origCov[c];
                const float ec = p.estimatedCoverage;
                const float f[13] = {__fdiv_rn(oc, cv),           __fdiv_rn(wOrig, wsum), __fdiv_rn(wOrig, oc),
                                     __fdiv_rn(nCons, cv),        sup[c],                 __fdiv_rn(wCons, nCons),
                                     __fdiv_rn(wsum, cv),         __fdiv_rn(cv, ec),      __fdiv_rn(wsum, ec),
                                     avg,                         mins,                   __fdiv_rn((float)maxc, ec),
                                     __fdiv_rn((float)minc, ec)};
                if (!forest_decide(p, f)) r = orig;
            }
            out[i] = r;
        }
        return;
    }
    if (nActive == 0) return;
    const bool byCons = sByConsensus;
    for (int i = tid; i < La; i += bd) {
        const int c = aBegin + i;
        char r;
        if (byCons) {
            r = cons[c];
        } else {
            r = (sup[c] > 0.90f && origCov[c] <= 2) ? cons[c] : "ACGT"[get2bit(aenc, i)];
        }
        out[i] = r;
    }
}

// ---------------------------------------------------------------- MSA, warp per anchor

// A column's weights and counts and the statistics derived from them
// (src/msa.cpp:135-157).
struct ColInfo {
    float w[4];
    uint32_t n[4];
    char cons;
    float consW, colW;
    __device__ float wOf(uint32_t i) const { return i == 0 ? w[0] : i == 1 ? w[1] : i == 2 ? w[2] : w[3]; }
    __device__ uint32_t nOf(uint32_t i) const { return i == 0 ? n[0] : i == 1 ? n[1] : i == 2 ? n[2] : n[3]; }
    __device__ int cov() const { return (int)(n[0] + n[1] + n[2] + n[3]); }
};

// wc[q * cp + c]: weight bits (x) and count (y) of base q in column c, read
// as one 8-byte entry per base
__device__ __forceinline__ ColInfo col_info(const uint2* wc, int cp, int c) {
    ColInfo r;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const uint2 v = wc[q * cp + c];
        r.w[q] = __uint_as_float(v.x);
        r.n[q] = v.y;
    }
    const float wA = r.w[0], wC = r.w[1], wG = r.w[2], wT = r.w[3];
    r.cons = 'A';
    r.consW = wA;
    if (wC > r.consW) { r.cons = 'C'; r.consW = wC; }
    if (wG > r.consW) { r.cons = 'G'; r.consW = wG; }
    if (wT > r.consW) { r.cons = 'T'; r.consW = wT; }
    r.colW = __fadd_rn(__fadd_rn(__fadd_rn(wA, wC), wG), wT);
    return r;
}

// One warp per anchor (one warp per block) for reads up to 256 bp.
//
// Everything the path reads from an MSA -- the different-region search, the
// properties and both decisions -- lies in the anchor's columns, so only the
// part of each row that overlaps the anchor is accumulated, in anchor
// coordinates (column = anchor position).  Shared memory holds per anchor
// position and base the weight and the count side by side (one 8-byte
// access per addition); rows are added one at a time
// (anchor, then the kept candidates in list order) with the lanes over the
// row's positions, so every column receives its additions in the reference's
// order.  Lane l owns the columns c with c % 32 == l in every pass (rows,
// consensus, properties, decision), so consecutive rows need no warp sync.
// The 2-bit words and the metadata of 32 rows are staged in shared memory per
// chunk.
//
// `sm` is the warp's own slice of shared memory (msa_warp_slice_bytes), `qw`
// the block's quality weights.
// Walk of the chunk staging loop: word i0 + lane of a chunk's rows is word
// off of row r (r = (i0 + lane) / pitch); (r0, off0) at i0 = 0 and the step
// (dr, doff) per 32 words, so that the loop divides nothing.
struct StageWalk {
    int r0, off0, dr, doff;
};

template <bool QUAL>
__device__ __forceinline__ void msa_warp_anchor(const StoreArg& st, const Params& p, const BatchArg& b,
                                             const uint32_t* __restrict__ rawOff, int lp, int a, uint64_t first,
                                             unsigned char* sm, const float* qw, const StageWalk sw) {
    const int lane = (int)lane_id();
    uint2* wc = reinterpret_cast<uint2*>(sm);                    // [4][lp]: weight bits, count
    float* sup = reinterpret_cast<float*>(wc + 4 * lp);          // [lp]
    uint32_t* stage = reinterpret_cast<uint32_t*>(sup + lp);     // [32][pitch]
    int4* meta = reinterpret_cast<int4*>(stage + 32 * st.pitch);  // [32]: shift, len | orient << 16, weight, id
    const uint64_t aid = first + (uint64_t)a;
    const uint64_t oi = (first - out_first(b)) + (uint64_t)a;   // output row
    const uint32_t nf = b.nfinal[a];
    char* out = b.out + oi * b.outPitch;
    if (nf == 0) {
        if (lane == 0) b.flags[oi] = 0;
        return;
    }
    const uint32_t base = rawOff[a];
    const int La = st.len[aid];
    const int pitch = st.pitch;
    const uint32_t* aenc = st.enc + aid * (uint64_t)pitch;
    const uint8_t* aq = QUAL ? st.qual + aid * (uint64_t)st.lmax : nullptr;
    constexpr uint8_t kRm = 0x80;

    // Rows are added (sign +1: every row still in the MSA, after the anchor
    // row) or taken out again (sign -1: the rows just removed, marked kNew).
    // Returns the number of rows added or taken out.
    constexpr uint8_t kNew = 0x40;
    auto rowsPass = [&](auto addTag) -> int {
        constexpr bool add = decltype(addTag)::value;
        int selected = 0;
        for (uint32_t j0 = 0; j0 < nf; j0 += 32) {
            const uint32_t jr = j0 + lane;
            const int rows = (int)min(32u, nf - j0);
            uint32_t mo = kRm, mid = 0;
            int mshift = 0, mlen = 0;
            float mw = 0.0f;
            if (jr < nf) {
                mo = b.forient[base + jr];
                mshift = b.fshift[base + jr];
                mlen = b.flen[base + jr];
                mid = b.fid[base + jr];
                mw = b.fweight[base + jr];
            }
            const bool sel = jr < nf && (add ? !(mo & kRm) : (mo & kNew) != 0);
            const unsigned selRows = __ballot_sync(kFull, sel);
            if (!selRows) continue;
            selected += __popc(selRows);
            if (!add && sel) b.forient[base + jr] = (uint8_t)(mo & ~kNew);
            // the selected rows' 2-bit words, copied without a register round
            // trip and waited for once
            {
                const int total = rows * pitch;
                int r = sw.r0, off = sw.off0;
                for (int i0 = 0; i0 < total; i0 += 32) {  // warp-uniform trip count
                    const int rr = min(r, rows - 1);
                    const uint32_t rid = __shfl_sync(kFull, mid, rr);
                    if (i0 + lane < total && ((selRows >> rr) & 1u))
                        cp_async4(stage + i0 + lane, st.enc + (uint64_t)rid * pitch + off);
                    r += sw.dr;
                    off += sw.doff;
                    if (off >= pitch) {
                        off -= pitch;
                        r++;
                    }
                }
            }
            meta[lane] = make_int4(mshift, mlen | (int)((mo & 3u) << 16), __float_as_int(mw), (int)mid);
            cp_async_wait_all();
            __syncwarp();
            for (int r = 0; r < rows; r++) {
                if (!((selRows >> r) & 1u)) continue;
                const int4 md = meta[r];
                const bool rc = ((uint32_t)md.y >> 16) == 2;
                const int shift = md.x, len = md.y & 0xffff;
                const float weight = __int_as_float(md.z);
                const uint32_t* e = stage + r * pitch;
                const uint8_t* q = QUAL ? st.qual + (uint64_t)(uint32_t)md.w * st.lmax : nullptr;
                const int c0 = max(shift, 0), c1 = min(La, shift + len);  // overlap with the anchor
                int c = c0 + ((lane - c0) & 31);                           // this lane's first column
                // the row position moves by 32 per column step of the lane, so
                // its word moves by 2 and its bit offset stays
                int sp = rc ? len - 1 - (c - shift) : c - shift;
                const int dsp = rc ? -32 : 32, dwi = rc ? -2 : 2;
                const uint32_t sh = 30u - 2u * (uint32_t)(sp & 15), flip = rc ? 3u : 0u;
                // quality index: sp, or for a reverse complement row Lmax - 1 - (c - shift)
                const int qd = rc ? st.lmax - len : 0;
                // padding past the read's end is read as stored
                auto wtAt = [&](int s) -> float { return QUAL ? __fmul_rn(weight, qw[q[s + qd]]) : weight; };
                auto upd = [&](uint2& v, float wt) {
                    if (add) {
                        v.x = __float_as_uint(__fadd_rn(__uint_as_float(v.x), wt));
                        v.y++;
                    } else {
                        v.x = __float_as_uint(__fsub_rn(__uint_as_float(v.x), wt));
                        v.y--;
                    }
                };
                int wi = sp >> 4;
                // two of the lane's columns (c and c + 32) per iteration: both
                // words and both entries are read before either is written
                // (distinct columns, distinct entries)
                for (; c + 32 < c1; c += 64, wi += 2 * dwi, sp += 2 * dsp) {
                    const uint32_t b0 = ((e[wi] >> sh) & 3u) ^ flip;
                    const uint32_t b1 = ((e[wi + dwi] >> sh) & 3u) ^ flip;
                    const float w0 = wtAt(sp), w1 = wtAt(sp + dsp);
                    uint2* p0 = wc + b0 * lp + c;
                    uint2* p1 = wc + b1 * lp + (c + 32);
                    uint2 v0 = *p0, v1 = *p1;
                    upd(v0, w0);
                    upd(v1, w1);
                    *p0 = v0;
                    *p1 = v1;
                }
                if (c < c1) {
                    const uint32_t b0 = ((e[wi] >> sh) & 3u) ^ flip;
                    uint2* p0 = wc + b0 * lp + c;
                    uint2 v0 = *p0;
                    upd(v0, wtAt(sp));
                    *p0 = v0;
                }
            }
            __syncwarp();  // the next chunk overwrites the staged rows
        }
        return selected;
    };
    // The MSA of the rows still in it, built as the reference builds it: the
    // anchor row (weight 1 times the quality weight), then the rows in order.
    // Returns the number of rows it holds besides the anchor.
    auto build = [&]() -> int {
        for (int pos = lane; pos < La; pos += 32) {
            const uint32_t bb = get2bit(aenc, pos);
            const float wt = QUAL ? __fmul_rn(1.0f, qw[aq[pos]]) : 1.0f;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                wc[q * lp + pos] = (uint32_t)q == bb ? make_uint2(__float_as_uint(__fadd_rn(0.0f, wt)), 1u)
                                                     : make_uint2(__float_as_uint(0.0f), 0u);
            }
        }
        __syncwarp();
        return rowsPass(std::true_type{});
    };

    int builds = 0;
    bool exact = true, haveS = false;
    int nActive = build();
    const float tol = __fmul_rn(2.5f * 5.9604645e-8f, (float)(3 * nf + 4));  // 2 E_c / S_c with slack
    for (int iter = 0;; iter++) {
        builds++;
        if (iter == 5 || nActive == 0) break;
        if (!exact) {
            bool close = false;
            for (int c = lane; c < La; c += 32) {
                float t1 = 0.0f, t2 = 0.0f;  // the two largest weights
                const ColInfo ci = col_info(wc, lp, c);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float v = ci.w[q];
                    t2 = fmaxf(t2, fminf(t1, v));
                    t1 = fmaxf(t1, v);
                }
                close |= !(__fsub_rn(t1, t2) > __fmul_rn(tol, sup[c]));
            }
            if (__any_sync(kFull, close)) {
                build();
                exact = true;
            }
        }
        // findCandidatesOfDifferentRegion (src/msa.cpp:532-734), in anchor coordinates
        bool mism = false;
        int firstSig = 0x7fffffff;
        for (int c = lane; c < La; c += 32) {
            const ColInfo ci = col_info(wc, lp, c);
            mism |= ci.cons != "ACGT"[get2bit(aenc, c)];
            const int cidx = base_index(ci.cons);
            bool sig = false;
#pragma unroll
            for (int i = 0; i < 4; i++) sig |= (i != cidx && p.significantCount <= (int)ci.n[i]);
            if (sig && c < firstSig) firstSig = c;
        }
        if (!__any_sync(kFull, mism)) break;
        const int col = __reduce_min_sync(kFull, firstSig);
        if (col == 0x7fffffff) break;
        int found;
        {
            const ColInfo ci = col_info(wc, lp, col);
            const int cidx = base_index(ci.cons);
            found = -1;
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (i != cidx && p.significantCount <= (int)ci.n[i]) found = i;
        }
        const uint32_t orig = get2bit(aenc, col);
        const bool keepMatching = orig == (uint32_t)found;
        auto differs = [&](uint32_t j) -> bool {
            const uint32_t g = base + j;
            const int sh = b.fshift[g];
            const int len = b.flen[g];
            if (col < sh || col >= sh + len) return false;
            const uint32_t* e = st.enc + (uint64_t)b.fid[g] * pitch;
            const int pos = col - sh;
            const bool rc = (b.forient[g] & 3) == 2;
            uint32_t bb = get2bit(e, rc ? len - 1 - pos : pos);
            if (rc) bb = 3u - bb;
            return keepMatching ? (bb != (uint32_t)found) : (bb == (uint32_t)found);
        };
        bool veto = false, any = false;
        for (uint32_t j = lane; j < nf; j += 32) {
            if ((b.forient[base + j] & kRm) || !differs(j)) continue;
            any = true;
            veto |= b.fweight[base + j] >= 0.90f;
        }
        // a veto (or nothing to remove) leaves the MSA as it is; the
        // reference then rebuilds the same MSA and reaches the same decision
        if (__any_sync(kFull, veto) || !__any_sync(kFull, any)) break;
        int act = 0;
        for (uint32_t j = lane; j < nf; j += 32) {
            const uint8_t o = b.forient[base + j];
            if (!(o & kRm) && differs(j)) b.forient[base + j] = o | kRm | kNew;
            else act += !(o & kRm);
        }
        nActive = __reduce_add_sync(kFull, act);
        if (!haveS) {  // S_c (the first build, which wc still holds), kept in `sup` until the properties
            for (int c = lane; c < La; c += 32) sup[c] = col_info(wc, lp, c).colW;
            haveS = true;
        }
        __syncwarp();
        rowsPass(std::false_type{});
        exact = false;
    }
    if (!exact) build();
    // getMSAProperties (src/msa.cpp:304-376) and the decision
    float mins = 3.402823466e+38f;
    int minc = 0x7fffffff, maxc = -1;
    for (int c = lane; c < La; c += 32) {
        const ColInfo ci = col_info(wc, lp, c);
        const float s = __fdiv_rn(ci.consW, ci.colW);
        sup[c] = s;
        mins = fminf(mins, s);
        const int cv = ci.cov();
        minc = min(minc, cv);
        maxc = max(maxc, cv);
    }
    for (int d = 16; d > 0; d >>= 1) mins = fminf(mins, __shfl_xor_sync(kFull, mins, d));
    minc = __reduce_min_sync(kFull, minc);
    maxc = __reduce_max_sync(kFull, maxc);
    __syncwarp();
    float avg = 0.0f;
    if (lane == 0) {  // in column order, four columns per shared-memory load
        float sum = 0.0f;
        const float4* s4 = reinterpret_cast<const float4*>(sup);
        int i = 0;
        for (; i + 4 <= La; i += 4) {
            const float4 v = s4[i >> 2];
            sum = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(sum, v.x), v.y), v.z), v.w);
        }
        for (; i < La; i++) sum = __fadd_rn(sum, sup[i]);
        avg = __fdiv_rn(sum, (float)La);
    }
    avg = __shfl_sync(kFull, avg, 0);
    const bool good = fgeq(avg, p.avgSupportThreshold) && fgeq(mins, p.minSupportThreshold) &&
                      fgeq((float)minc, p.minCoverageThreshold);
    bool hq = false;
    if (good) {
        int smallest = 100;
        for (int percent = p.errPercent; percent >= 0; percent--) {
            if (fgeq(avg, p.hqAvg[percent]) && fgeq(mins, p.hqMin[percent])) smallest = percent;
        }
        hq = fgeq((float)minc, p.minCoverageThreshold) && fleq((float)smallest, p.hqPercentLimit);
    }
    const bool forest = p.correctionType == CG_CORR_FOREST;
    const bool corrected = forest || nActive > 0;
    if (lane == 0) {
        if (corrected) {
            atomicAdd(&b.counters[kCounterCorrected], 1ull);
            if (hq) atomicAdd(&b.counters[kCounterHQ], 1ull);
        }
        atomicAdd(&b.counters[kCounterMsaBuilds], (unsigned long long)builds);
        b.flags[oi] = corrected ? (uint8_t)(CG_RESULT_CORRECTED | (hq ? CG_RESULT_HQ : 0)) : (uint8_t)0;
    }
    if (!corrected) return;
    for (int c = lane; c < La; c += 32) {
        const uint32_t ab = get2bit(aenc, c);
        const char orig = "ACGT"[ab];
        const ColInfo ci = col_info(wc, lp, c);
        const int origCov = (int)ci.nOf(ab);
        char r;
        if (forest) {
            // correctAnchorClf (include/corrector.hpp:1448-1472), features of
            // include/classification.hpp:748-797
            r = ci.cons;
            if (!hq && r != orig) {
                const int ci_ = base_index(ci.cons);
                const float wCons = ci.wOf((uint32_t)ci_);
                const float nCons = (float)ci.nOf((uint32_t)ci_);
                const float wOrig = ci.wOf(ab);
                const float cv = (float)ci.cov();
                const float oc = (float)origCov;
                const float ec = p.estimatedCoverage;
                const float f[13] = {__fdiv_rn(oc, cv),      __fdiv_rn(wOrig, ci.colW), __fdiv_rn(wOrig, oc),
                                     __fdiv_rn(nCons, cv),   sup[c],                    __fdiv_rn(wCons, nCons),
                                     __fdiv_rn(ci.colW, cv), __fdiv_rn(cv, ec),         __fdiv_rn(ci.colW, ec),
                                     avg,                    mins,                      __fdiv_rn((float)maxc, ec),
                                     __fdiv_rn((float)minc, ec)};
                if (!forest_decide(p, f)) r = orig;
            }
        } else if (good) {
            r = ci.cons;
        } else {
            r = (sup[c] > 0.90f && origCov <= 2) ? ci.cons : orig;
        }
        out[c] = r;
    }
    if (p.candidates && hq) {
        // Candidate correction.  The MSA above holds the anchor's columns
        // only; the consensus of the nc columns on either side is summed here,
        // rows in list order, lane e0 + lane owning extension column e (column
        // e - nc left of the anchor, or La + e - nc right of it).  cons8[x] =
        // consensus base code of column x - nc, for x in [0, La + 2 nc).
        const int nc = p.newColumns;
        uint8_t* cons8 = reinterpret_cast<uint8_t*>(meta + 32);
        for (int c = lane; c < La; c += 32) cons8[nc + c] = (uint8_t)base_index(col_info(wc, lp, c).cons);
        for (int e0 = 0; e0 < 2 * nc; e0 += 32) {  // warp-uniform trip count
            const int e = e0 + lane;
            const int col = e < nc ? e - nc : La + (e - nc);
            float w4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (uint32_t j0 = 0; j0 < nf; j0 += 32) {
                const uint32_t jr = j0 + lane;
                const int rows = (int)min(32u, nf - j0);
                uint32_t mo = kRm, mid = 0;
                int mshift = 0, mlen = 0;
                float mw = 0.0f;
                if (jr < nf) {
                    mo = b.forient[base + jr];
                    mshift = b.fshift[base + jr];
                    mlen = b.flen[base + jr];
                    mid = b.fid[base + jr];
                    mw = b.fweight[base + jr];
                }
                // rows still in the MSA that reach past either end of the anchor
                const bool sel = jr < nf && !(mo & kRm) && (mshift < 0 || mshift + mlen > La);
                const unsigned selRows = __ballot_sync(kFull, sel);
                if (!selRows) continue;
                for (int i0 = 0; i0 < rows * pitch; i0 += 32) {
                    const int idx = i0 + lane;
                    const int r = min(idx / pitch, rows - 1);
                    const uint32_t rid = __shfl_sync(kFull, mid, r);
                    if (idx < rows * pitch && ((selRows >> r) & 1u))
                        stage[idx] = st.enc[(uint64_t)rid * pitch + (idx - r * pitch)];
                }
                meta[lane] = make_int4(mshift, mlen | (int)((mo & 3u) << 16), __float_as_int(mw), (int)mid);
                __syncwarp();
                for (int r = 0; r < rows; r++) {
                    if (!((selRows >> r) & 1u)) continue;
                    const int4 md = meta[r];
                    const bool rc = ((uint32_t)md.y >> 16) == 2;
                    const int len = md.y & 0xffff;
                    const int pos = col - md.x;
                    if (e >= 2 * nc || pos < 0 || pos >= len) continue;
                    const int sp = rc ? len - 1 - pos : pos;
                    const uint32_t bb = ((stage[r * pitch + (sp >> 4)] >> (30u - 2u * (uint32_t)(sp & 15))) & 3u) ^
                                        (rc ? 3u : 0u);
                    float wt = __int_as_float(md.z);
                    if (QUAL)
                        wt = __fmul_rn(wt, qw[row_quality(st.qual + (uint64_t)(uint32_t)md.w * st.lmax, st.lmax, rc,
                                                          pos)]);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if ((uint32_t)q == bb) w4[q] = __fadd_rn(w4[q], wt);
                }
                __syncwarp();  // the next chunk overwrites the staged rows
            }
            if (e < 2 * nc) {  // src/msa.cpp:135-157: the first largest weight, A C G T
                int cb = 0;
                float cw = w4[0];
#pragma unroll
                for (int q = 1; q < 4; q++)
                    if (w4[q] > cw) {
                        cb = q;
                        cw = w4[q];
                    }
                cons8[e < nc ? e : La + e] = (uint8_t)cb;
            }
        }
        __syncwarp();
        // The consensus packed 32 columns per word, forward (fw: column x at
        // position x) and reverse complemented (rv: position y holds the
        // complement of column X - 1 - y), one zero word past each; a row's
        // slice is then a run of whole words at a bit offset in one of them.
        const int X = La + 2 * nc, nw = (X + 31) / 32;
        unsigned long long* fw =
            reinterpret_cast<unsigned long long*>(cons8 + ((size_t)lp + 2 * (size_t)nc + 15) / 16 * 16);
        unsigned long long* rv = fw + nw + 1;
        __syncwarp();
        for (int u = lane; u <= nw; u += 32) {
            unsigned long long f = 0, r = 0;
            for (int t = 0; t < 32; t++) {
                const int x = 32 * u + t;
                if (x < X) {
                    f |= (unsigned long long)cons8[x] << (62 - 2 * t);
                    r |= (unsigned long long)(3u - cons8[X - 1 - x]) << (62 - 2 * t);
                }
            }
            fw[u] = f;
            rv[u] = r;
        }
        __syncwarp();
        // one row per lane
        int votes = 0;
        for (uint32_t j = lane; j < nf; j += 32) {
            const uint32_t g = base + j;
            const uint8_t o = b.forient[g];
            if (o & kRm) continue;
            const int s = b.fshift[g], len = b.flen[g];
            if (s < -nc || s > nc || s + len > La + nc) continue;
            const bool rc = (o & 3) == 2;
            const unsigned long long* src = rc ? rv : fw;
            const int y0 = rc ? X - (nc + s) - len : nc + s;  // the slice's first position in src
            const uint32_t id = b.fid[g];
            for (int w = 0; w * 32 < len; w++) {
                const int y = y0 + 32 * w, u = y >> 5, off = 2 * (y & 31);
                unsigned long long v = src[u] << off;
                if (off) v |= src[u + 1] >> (64 - off);
                const int rest = len - 32 * w;
                if (rest < 32) v &= ~0ull << (64 - 2 * rest);
                vote_word(p, id, w, v);
            }
            atomicAdd((uint64_t)id > aid ? &p.candVotes[id].x : &p.candVotes[id].y, 1u);
            votes++;
        }
        votes = __reduce_add_sync(kFull, votes);
        if (lane == 0 && votes) atomicAdd(&b.counters[kCounterCandidateVotes], (unsigned long long)votes);
        return;
    }
    if (p.correctionType != CG_CORR_LEARNED || hq) return;
    // Learned decision: record every column whose consensus differs from the
    // anchor's base, with its features; the classifier then replaces the
    // decision written above (the fallback) where it is confident.
    int nd = 0;
    for (int c = lane; c < La; c += 32) nd += col_info(wc, lp, c).cons != "ACGT"[get2bit(aenc, c)];
    nd = __reduce_add_sync(kFull, nd);
    const float ec = p.estimatedCoverage;
    const float invLa = __fdiv_rn(1.0f, (float)La);
    for (int c0 = 0; c0 < La; c0 += 32) {  // warp-uniform trip count
        const int c = c0 + lane;
        bool rec = false;
        ColInfo ci{};
        uint32_t ab = 0;
        if (c < La) {
            ab = get2bit(aenc, c);
            ci = col_info(wc, lp, c);
            rec = ci.cons != "ACGT"[ab];
        }
        const unsigned m = __ballot_sync(kFull, rec);
        if (!m) continue;
        unsigned slot = 0;
        if (lane == 0) slot = atomicAdd(b.colCount, (unsigned)__popc(m));
        slot = __shfl_sync(kFull, slot, 0) + (unsigned)__popc(m & ((1u << lane) - 1u));
        if (!rec || slot >= b.colCap) continue;
        const int cb = base_index(ci.cons);
        float n4[4], w4[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            n4[q] = (float)ci.n[q];
            w4[q] = ci.w[q];
        }
        auto pick = [](const float (&v)[4], uint32_t i) {
            return i == 0 ? v[0] : i == 1 ? v[1] : i == 2 ? v[2] : v[3];
        };
        const float cov = __fadd_rn(__fadd_rn(__fadd_rn(n4[0], n4[1]), n4[2]), n4[3]);
        const float icov = __fdiv_rn(1.0f, cov);
        const float icw = ci.colW > 0.0f ? __fdiv_rn(1.0f, ci.colW) : 0.0f;
        // Ratios that sit near 1 enter as 1 - ratio: BF16 keeps about three
        // significant digits, so 0.983 and 0.987 would be the same value but
        // 0.017 and 0.013 are not.
        const float na = pick(n4, ab), nc = pick(n4, (uint32_t)cb);
        float second = 0.0f;  // the second largest base weight
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (q != cb) second = fmaxf(second, w4[q]);
        float f[kLearnedFeatures];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            f[q] = __fmul_rn(n4[q], icov);                 // base counts / coverage
            f[4 + q] = __fmul_rn(w4[q], icw);              // weights / column weight
            f[18 + q] = q == cb ? 1.0f : 0.0f;             // consensus base
        }
        f[8] = __fdiv_rn(cov, ec);
        f[9] = __fdiv_rn(ci.colW, ec);
        f[10] = __fsub_rn(1.0f, sup[c]);
        f[11] = __fmul_rn(pick(w4, ab), icw);
        f[12] = __fmul_rn(na, icov);
        f[13] = __fsub_rn(1.0f, __fmul_rn(nc, icov));
        f[14] = __fsub_rn(1.0f, __fdiv_rn(pick(w4, ab), na));                   // mean weight of the anchor base's rows
        f[15] = nc > 0.0f ? __fsub_rn(1.0f, __fdiv_rn(ci.consW, nc)) : 1.0f;   // ... of the consensus base's rows
        f[16] = __fsub_rn(1.0f, __fmul_rn(ci.colW, icov));                      // ... of all rows
        f[17] = __fmul_rn(second, icw);                                          // runner-up weight / column weight
        f[22] = __fmul_rn((float)c, invLa);
        f[23] = __fmul_rn((float)min(c, La - 1 - c), invLa);
        f[24] = __fsub_rn(1.0f, avg);
        f[25] = __fsub_rn(1.0f, mins);
        f[26] = __fdiv_rn((float)minc, ec);
        f[27] = __fdiv_rn((float)maxc, ec);
        f[28] = __fmul_rn((float)La, 1.0f / 256.0f);
        f[29] = __fmul_rn((float)nd, invLa);
        f[30] = __fdiv_rn((float)nActive, ec);
        f[31] = QUAL ? qw[aq[c]] : 1.0f;
        uint32_t wd[kLearnedFeatures / 2];
#pragma unroll
        for (int k = 0; k < kLearnedFeatures / 2; k++) {
            const __nv_bfloat162 v = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
            wd[k] = *reinterpret_cast<const uint32_t*>(&v);
        }
        uint4* dst = reinterpret_cast<uint4*>(b.colFeat + (uint64_t)slot * kLearnedFeatures);
#pragma unroll
        for (int k = 0; k < kLearnedFeatures / 8; k++)
            dst[k] = make_uint4(wd[4 * k], wd[4 * k + 1], wd[4 * k + 2], wd[4 * k + 3]);
        b.colMeta[slot] = make_uint2((uint32_t)oi, (uint32_t)c | ((uint32_t)(uint8_t)ci.cons << 16));
    }
}

// Bytes of shared memory one warp of msa_warp_kernel works in (with candidate
// correction, the consensus codes of Lmax + 2 new_columns_to_correct columns
// follow the row metadata).
__host__ __device__ inline size_t msa_warp_slice_bytes(int lp, int pitch, const Params& p) {
    const size_t cols = (size_t)lp + 2 * (size_t)p.newColumns;
    const size_t cand = p.candidates ? (cols + 15) / 16 * 16 + 2 * ((cols + 31) / 32 + 1) * sizeof(uint64_t) : 0;
    return (size_t)lp * (9 * sizeof(float)) + (size_t)32 * pitch * sizeof(uint32_t) + 32 * sizeof(int4) + cand;
}

// `warps` warps per block, each on its own anchors.  Plain form: anchor
// blockIdx.x * warps + warp.  Persistent form (b.work set): warps take the
// next anchor from the counter b.work[1] until the batch is done.
__global__ void __launch_bounds__(256, 4) msa_warp_kernel(StoreArg st, Params p, BatchArg b,
                                                       const uint32_t* __restrict__ rawOff, int lp) {
    extern __shared__ __align__(16) unsigned char sm[];
    float* qw = reinterpret_cast<float*>(sm);  // [256] (quality scores only)
    const int warp = (int)(threadIdx.x >> 5), warps = (int)(blockDim.x >> 5);
    const size_t qbytes = p.useQuality ? 256 * sizeof(float) : 0;
    unsigned char* slice = sm + qbytes + (size_t)warp * msa_warp_slice_bytes(lp, st.pitch, p);
    if (p.useQuality) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) qw[i] = p.qweight[i];
        __syncthreads();
    }
    const uint64_t first = batch_first(b);
    const int lane = (int)lane_id(), pitch = st.pitch;
    const StageWalk sw{lane / pitch, lane % pitch, 32 / pitch, 32 % pitch};
    auto anchor = [&](int i) {
        const int a = b.order ? (int)b.order[i] : i;
        if (p.useQuality) msa_warp_anchor<true>(st, p, b, rawOff, lp, a, first, slice, qw, sw);
        else msa_warp_anchor<false>(st, p, b, rawOff, lp, a, first, slice, qw, sw);
    };
    if (!b.work) {
        const int i = blockIdx.x * warps + warp;
        if (i < b.count) anchor(i);
        return;
    }
    while (true) {
        int i = 0;
        if (lane == 0) i = (int)atomicAdd(&b.work[1], 1u);
        i = __shfl_sync(kFull, i, 0);
        if (i >= b.count) return;
        anchor(i);
        __syncwarp();
    }
}

constexpr int kOrderBuckets = 16;

// bucket 0 holds the anchors with the most kept rows (nf >= 2^14), bucket 15
// those with none
__device__ __forceinline__ int order_bucket(uint32_t nf) { return 15 - min(15, 32 - __clz(nf)); }

__global__ void msa_order_hist_kernel(const uint32_t* __restrict__ nfinal, int count, unsigned int* hist) {
    __shared__ unsigned int h[kOrderBuckets];
    if (threadIdx.x < kOrderBuckets) h[threadIdx.x] = 0;
    __syncthreads();
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < count; a += gridDim.x * blockDim.x)
        atomicAdd(&h[order_bucket(nfinal[a])], 1u);
    __syncthreads();
    if (threadIdx.x < kOrderBuckets && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Each block reserves its slots of every bucket with one global atomic per
// bucket per round (the per-anchor tickets come from shared memory).
__global__ void msa_order_scatter_kernel(const uint32_t* __restrict__ nfinal, int count,
                                         const unsigned int* __restrict__ hist, unsigned int* cursor,
                                         uint32_t* __restrict__ order) {
    __shared__ unsigned int start[kOrderBuckets], local[kOrderBuckets], base[kOrderBuckets];
    if (threadIdx.x == 0) {
        unsigned int acc = 0;
        for (int i = 0; i < kOrderBuckets; i++) {
            start[i] = acc;
            acc += hist[i];
        }
    }
    for (int a0 = blockIdx.x * blockDim.x; a0 < count; a0 += gridDim.x * blockDim.x) {
        if (threadIdx.x < kOrderBuckets) local[threadIdx.x] = 0;
        __syncthreads();
        const int a = a0 + threadIdx.x;
        int k = 0;
        unsigned int ticket = 0;
        if (a < count) {
            k = order_bucket(nfinal[a]);
            ticket = atomicAdd(&local[k], 1u);
        }
        __syncthreads();
        if (threadIdx.x < kOrderBuckets && local[threadIdx.x])
            base[threadIdx.x] = start[threadIdx.x] + atomicAdd(&cursor[threadIdx.x], local[threadIdx.x]);
        __syncthreads();
        if (a < count) order[base[k] + ticket] = (uint32_t)a;
        __syncthreads();
    }
}

template <int MAXW, bool REGS>
cudaError_t launch_align_t(StoreArg st, Params p, BatchArg b, cudaStream_t s) {
    const size_t smem = (size_t)kAlignWarps * 6 * st.wp * sizeof(uint32_t) +
                        (REGS ? ((size_t)st.lmax + 2) * sizeof(int16_t) : 0);
    const unsigned blocks = (unsigned)((b.count + kAlignWarps - 1) / kAlignWarps);
    align_filter_kernel<MAXW, REGS><<<blocks, kAlignWarps * 32, smem, s>>>(st, p, b, b.rawCount);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_align_filter(StoreArg st, Params p, BatchArg b, const uint32_t* uoff, uint32_t totalUnique,
                                cudaEvent_t between, cudaStream_t s, const Shape* shape) {
    const int need = st.wp - 1;  // words per plane that hold bases
    if (need <= 8 && uoff) {
        const bool persistent = shape && b.work;
        if (persistent || totalUnique > 0) {
            // persistent: the warps take 32-candidate chunks until uoff[count];
            // with b.laneWork (plain form) as many blocks as fit the GPU do the same
            unsigned blocks =
                persistent ? (unsigned)shape->alignBlocks : (totalUnique + kLaneThreads - 1) / kLaneThreads;
            if (!persistent && b.laneWork) {
                int dev = 0, sms = 1, occ = 1;
                if (cudaGetDevice(&dev) == cudaSuccess)
                    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                occ = std::max(align_lane_occupancy(st), 1);
                blocks = std::min(blocks, (unsigned)(std::max(sms, 1) * occ));
            }
            if (need <= 5)
                align_lane_kernel<5><<<blocks, kLaneThreads, 0, s>>>(st, p, b, b.rawCount, uoff, totalUnique);
            else
                align_lane_kernel<8><<<blocks, kLaneThreads, 0, s>>>(st, p, b, b.rawCount, uoff, totalUnique);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        if (between) {
            cudaError_t e = cudaEventRecord(between, s);
            if (e != cudaSuccess) return e;
        }
        filter_kernel<<<(unsigned)(((uint64_t)b.count * 32 + 127) / 128), 128, 0, s>>>(st, p, b, b.rawCount);
        return cudaGetLastError();
    }
    if (between) {
        cudaError_t e = cudaEventRecord(between, s);  // the fused kernel below aligns and filters
        if (e != cudaSuccess) return e;
    }
    if (need <= 5) return launch_align_t<5, true>(st, p, b, s);
    if (need <= 8) return launch_align_t<8, true>(st, p, b, s);
    if (need <= 16) return launch_align_t<16, false>(st, p, b, s);
    return launch_align_t<32, false>(st, p, b, s);
}

int msa_threads(int maxCols) {
    int t = kMsaThreadsMin;
    while (t * kMsaCols < maxCols) t += 32;
    return t;
}

size_t msa_smem_bytes(int maxCols, int bitsetWords, int storeWeights) {
    return sizeof(RowMeta) * kMsaChunkRows + sizeof(uint32_t) * bitsetWords + 256 * sizeof(float) +
           (size_t)maxCols * (7 * sizeof(int) + 1 + (storeWeights ? 4 * sizeof(float) : 0));
}

namespace {

size_t msa_warp_smem(StoreArg st, Params p, int warps) {
    const int lp = (st.lmax + 31) / 32 * 32;
    return (p.useQuality ? 256 * sizeof(float) : 0) + (size_t)warps * msa_warp_slice_bytes(lp, st.pitch, p);
}

cudaError_t msa_warp_prepare(size_t smem) {
    if (smem <= 40 * 1024) return cudaSuccess;  // leaves room for the kernel's static shared memory
    return cudaFuncSetAttribute(msa_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace

int align_lane_occupancy(StoreArg st) {
    const int need = st.wp - 1;
    if (need > 8) return 0;
    int blocks = 0;
    const cudaError_t e = need <= 5
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, align_lane_kernel<5>, kLaneThreads, 0)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, align_lane_kernel<8>, kLaneThreads, 0);
    return e == cudaSuccess ? blocks : 0;
}

int msa_warp_occupancy(StoreArg st, Params p, int warps) {
    if (st.lmax > 256 || warps < 1 || warps > 8) return 0;
    const size_t smem = msa_warp_smem(st, p, warps);
    if (msa_warp_prepare(smem) != cudaSuccess) return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, msa_warp_kernel, warps * 32, smem) != cudaSuccess)
        return 0;
    return blocks;
}

cudaError_t launch_msa_correct(StoreArg st, Params p, BatchArg b, int maxRows, cudaStream_t s, const Shape* shape) {
    const int maxCols = 3 * st.lmax + 4;
    if (st.lmax <= 256) {
        const int lp = (st.lmax + 31) / 32 * 32;
        const bool persistent = shape && b.work;
        const int warps = persistent ? shape->msaWarps : 1;
        const size_t smem = msa_warp_smem(st, p, warps);
        cudaError_t e = msa_warp_prepare(smem);
        if (e != cudaSuccess) return e;
        const unsigned blocks = persistent ? (unsigned)shape->msaBlocks : (unsigned)b.count;
        if (blocks == 0) return cudaSuccess;
        msa_warp_kernel<<<blocks, warps * 32, smem, s>>>(st, p, b, b.rawCount, lp);
        return cudaGetLastError();
    }
    const int bitsetWords = (maxRows + 31) / 32 + 1;
    const int storeWeights = p.correctionType == CG_CORR_FOREST;
    const size_t smem = msa_smem_bytes(maxCols, bitsetWords, storeWeights);
    if (smem > 40 * 1024) {  // leaves room for the kernel's static shared memory
        cudaError_t e = cudaFuncSetAttribute(msa_correct_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    if (b.count == 0) return cudaSuccess;
    msa_correct_kernel<<<b.count, msa_threads(maxCols), smem, s>>>(st, p, b, b.rawCount, maxCols, bitsetWords,
                                                                    storeWeights);
    return cudaGetLastError();
}

cudaError_t launch_msa_order(BatchArg b, unsigned int* scratch, uint32_t* order, cudaStream_t s) {
    if (b.count <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scratch, 0, 2 * kOrderBuckets * sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)min((b.count + 255) / 256, 304);
    msa_order_hist_kernel<<<blocks, 256, 0, s>>>(b.nfinal, b.count, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    msa_order_scatter_kernel<<<blocks, 256, 0, s>>>(b.nfinal, b.count, scratch, scratch + kOrderBuckets, order);
    return cudaGetLastError();
}

namespace {

// one warp per anchor of the batch; lane w packs word w of a low-quality
// anchor correction (the output row's bases) and votes with it
__global__ void __launch_bounds__(256) anchor_vote_kernel(StoreArg st, Params p, BatchArg b) {
    const int a = (int)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (a >= b.count) return;
    const uint64_t first = batch_first(b);
    const uint64_t aid = first + (uint64_t)a;
    const uint64_t oi = (first - out_first(b)) + (uint64_t)a;
    const uint8_t f = b.flags[oi];
    if (!(f & CG_RESULT_CORRECTED) || (f & CG_RESULT_HQ)) return;
    const int len = st.len[aid];
    const int w = (int)lane_id();
    if (w * 32 >= len) return;
    const char* o = b.out + oi * (uint64_t)b.outPitch;
    unsigned long long v = 0;
    const int pe = min(len, w * 32 + 32);
    for (int q = w * 32; q < pe; q++) v |= (unsigned long long)base_index(o[q]) << (62 - 2 * (q & 31));
    vote_word(p, aid, w, v);
}

// reference: src/correctionresultoutput.cpp:1256-1551 (combine), with the
// record filter of include/corrector.hpp:1678-1681 in a single-threaded run's
// order: read c's candidate records from anchors above c are not saved when c
// is a corrected HQ anchor.  One thread per read.
__global__ void combine_kernel(StoreArg st, Params p, uint64_t first, uint64_t n, uint8_t* __restrict__ flags,
                               unsigned long long* __restrict__ records) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long k = 0;
    if (i < n) {
        const uint64_t r = first + i;
        uint8_t f = flags[i];
        const uint2 v = p.candVotes[r];
        const bool hqAnchor = (f & CG_RESULT_CORRECTED) && (f & CG_RESULT_HQ);
        k = (unsigned long long)v.x + (hqAnchor ? 0ull : (unsigned long long)v.y);
        if (k) f |= CG_RESULT_CANDIDATE_RECORD;
        if ((f & CG_RESULT_CORRECTED) && !(f & CG_RESULT_HQ) && k >= 2) {
            const int words = (st.len[r] + 31) / 32;
            bool same = true;
            for (int w = 0; w < words; w++) {
                const uint64_t j = r * (uint64_t)p.candPitch + (uint64_t)w;
                same &= p.candAnd[j] == p.candOr[j];
            }
            f |= same ? CG_RESULT_CANDIDATES : CG_RESULT_REJECTED;
        }
        flags[i] = f;
    }
    for (int d = 16; d > 0; d >>= 1) k += __shfl_xor_sync(kFull, k, d);
    if ((threadIdx.x & 31) == 0 && k) atomicAdd(records, k);
}

__global__ void batch_advance_kernel(unsigned long long* cursor, unsigned int* work, unsigned long long stride) {
    cursor[0] += stride;
    work[0] = 0;
    work[1] = 0;
}
}  // namespace

cudaError_t launch_anchor_vote(StoreArg st, Params p, BatchArg b, cudaStream_t s) {
    if (b.count <= 0) return cudaSuccess;
    anchor_vote_kernel<<<(unsigned)((b.count + 7) / 8), 256, 0, s>>>(st, p, b);
    return cudaGetLastError();
}

cudaError_t launch_combine(StoreArg st, Params p, uint64_t first, uint64_t n, uint8_t* flags,
                           unsigned long long* records, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st, p, first, n, flags, records);
    return cudaGetLastError();
}

cudaError_t launch_batch_advance(unsigned long long* cursor, unsigned int* work, unsigned long long stride,
                                 cudaStream_t s) {
    batch_advance_kernel<<<1, 1, 0, s>>>(cursor, work, stride);
    return cudaGetLastError();
}

}  // namespace cg
