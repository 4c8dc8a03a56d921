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

#include "care_device.cuh"
#include "care_internal.h"

namespace cg {

namespace {

// ---------------------------------------------------------------- alignment

constexpr int kAlignWarps = 4;  // warps per block, one anchor per warp

// mismatches between `sh` shifted left by `sl` bases and `ot`, over `ov` bases
__device__ __forceinline__ int mismatches(const uint32_t* __restrict__ shHi, const uint32_t* __restrict__ shLo,
                                          const uint32_t* __restrict__ otHi, const uint32_t* __restrict__ otLo,
                                          int sl, int ov) {
    const int parts = (ov + 31) >> 5;
    const int rem = (parts << 5) - ov;
    const int ws = sl >> 5, bs = sl & 31;
    int m = 0;
    for (int i = 0; i < parts; i++) {
        const uint32_t hi = __funnelshift_l(shHi[i + ws + 1], shHi[i + ws], bs);
        const uint32_t lo = __funnelshift_l(shLo[i + ws + 1], shLo[i + ws], bs);
        uint32_t x = (hi ^ otHi[i]) | (lo ^ otLo[i]);
        if (i == parts - 1 && rem != 0) x &= 0xffffffffu << rem;
        m += __popc(x);
    }
    return m;
}

struct AlnRes {
    int score, overlap, shift, nOps;
    bool valid;
};

// Warp-cooperative shifted Hamming alignment.  Every lane evaluates a subset
// of the shifts; the winner is the first shift in the reference's scan order
// (0, 1, .., La-minov, then -1, -2, .., -(Lc-minov)) among those with the
// smallest score whose mismatch count is below int(overlap * maxErrorRate).
// The reference's early exits only skip shifts that cannot win, so this
// full evaluation returns the same (score, shift).
__device__ AlnRes align_warp(const uint32_t* aHi, const uint32_t* aLo, int La, const uint32_t* cHi,
                             const uint32_t* cLo, int Lc, int minov, float rate) {
    const int tb = La + Lc;
    const int n1 = max(0, La - minov + 1);
    const int n2 = max(0, Lc - minov);
    uint32_t best = 0xffffffffu;
    for (int t = (int)lane_id(); t < n1 + n2; t += 32) {
        int s, ov;
        if (t < n1) {
            s = t;
            ov = min(La - s, Lc);
        } else {
            s = -(t - n1 + 1);
            ov = min(La, Lc + s);
        }
        const int maxErr = (int)__fmul_rn((float)ov, rate);
        if (maxErr > 0 && ov > 0) {
            const int m = s >= 0 ? mismatches(aHi, aLo, cHi, cLo, s, ov) : mismatches(cHi, cLo, aHi, aLo, -s, ov);
            const int score = m + tb - 2 * ov;
            if (m < maxErr && score < tb) {
                const uint32_t key = ((uint32_t)score << 16) | (uint32_t)t;
                best = key < best ? key : best;
            }
        }
    }
    best = __reduce_min_sync(0xffffffffu, best);
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

// One warp per anchor: align all candidates, choose orientations, apply the
// mismatch-ratio filter and write the filtered candidate list in order.
__global__ void __launch_bounds__(kAlignWarps * 32) align_filter_kernel(StoreArg st, Params p, BatchArg b,
                                                                        const uint32_t* __restrict__ rawOff) {
    extern __shared__ uint32_t smem[];
    const int warp = threadIdx.x >> 5;
    const uint32_t lane = lane_id();
    const int a = blockIdx.x * kAlignWarps + warp;
    if (a >= b.count) return;
    const int wp = st.wp;
    uint32_t* aHL = smem + warp * 6 * wp;  // anchor hi, lo; candidate fwd hi, lo, rc hi, lo
    uint32_t* cHL = aHL + 2 * wp;
    const uint64_t aid = b.first + (uint64_t)a;
    const int La = st.len[aid];
    const uint32_t nc = b.ncand[a];
    const uint32_t base = rawOff[a];
    if (nc == 0) {
        if (lane == 0) b.nfinal[a] = 0;
        return;
    }
    const uint32_t* ahl = st.hilo + aid * 4 * (uint64_t)wp;  // forward planes
    for (int i = (int)lane; i < 2 * wp; i += 32) aHL[i] = ahl[i];
    const int minov = max(p.minOverlap, (int)__fmul_rn((float)La, p.minOverlapRatio));
    for (uint32_t j = 0; j < nc; j++) {
        const uint32_t id = b.cand[base + j];
        const int Lc = st.len[id];
        const uint32_t* chl = st.hilo + (uint64_t)id * 4 * wp;
        __syncwarp();
        for (int i = (int)lane; i < 4 * wp; i += 32) cHL[i] = chl[i];
        __syncwarp();
        const AlnRes f = align_warp(aHL, aHL + wp, La, cHL, cHL + wp, Lc, minov, p.maxErrorRate);
        const AlnRes r = align_warp(aHL, aHL + wp, La, cHL + 2 * wp, cHL + 3 * wp, Lc, minov, p.maxErrorRate);
        const int ori = choose_orientation(f, r, La, p.minOverlapRatio, p.minOverlap, p.orientMaxErrorRate);
        if (lane == 0) b.aln[base + j] = pack_aln(ori == 2 ? r : f, ori);
    }
    __syncwarp();
    // mismatch-ratio filter (include/corrector.hpp:1053-1149 single end, 1151-1211 paired end)
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
        c0 = __reduce_add_sync(0xffffffffu, c0);
        c1 = __reduce_add_sync(0xffffffffu, c1);
        c2 = __reduce_add_sync(0xffffffffu, c2);
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
        const uint32_t m = __ballot_sync(0xffffffffu, keep);
        aligned += __popc(__ballot_sync(0xffffffffu, isAligned));
        if (keep) {
            const uint32_t pos = kept + __popc(m & ((1u << lane) - 1u));
            const int ov = (int)(v.x >> 16);
            const int nOps = (int)(int16_t)(v.y & 0xffffu);
            b.fid[base + pos] = b.cand[base + j];
            b.fshift[base + pos] = (int16_t)(v.x & 0xffffu);
            b.forient[base + pos] = (uint8_t)(v.y >> 16);
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

// ---------------------------------------------------------------- MSA

constexpr int kMsaThreads = 128;
constexpr uint8_t kRemoved = 0x80;

__device__ __forceinline__ float block_min_f(float v, float* red) {
    for (int d = 16; d > 0; d >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, d));
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    float r = red[0];
    for (int w = 1; w < kMsaThreads / 32; w++) r = fminf(r, red[w]);
    return r;
}

__device__ __forceinline__ int block_reduce_i(int v, int* red, int op /*0 min 1 max 2 sum*/) {
    for (int d = 16; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(0xffffffffu, v, d);
        v = op == 0 ? min(v, o) : op == 1 ? max(v, o) : v + o;
    }
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    int r = red[0];
    for (int w = 1; w < kMsaThreads / 32; w++) r = op == 0 ? min(r, red[w]) : op == 1 ? max(r, red[w]) : r + red[w];
    return r;
}

// One block per anchor.  Columns are owned by threads (column c by thread
// c % blockDim), and every column sums its rows in list order: anchor first,
// then the kept candidates as the filters left them, so each float sum is
// the reference's sequence of additions.
__global__ void __launch_bounds__(kMsaThreads) msa_correct_kernel(StoreArg st, Params p, BatchArg b,
                                                                  const uint32_t* __restrict__ rawOff, int maxCols) {
    extern __shared__ unsigned char sm[];
    int* cntA = reinterpret_cast<int*>(sm);
    int* cntC = cntA + maxCols;
    int* cntG = cntC + maxCols;
    int* cntT = cntG + maxCols;
    int* cov = cntT + maxCols;
    int* origCov = cov + maxCols;
    float* sup = reinterpret_cast<float*>(origCov + maxCols);
    char* cons = reinterpret_cast<char*>(sup + maxCols);
    __shared__ float redf[kMsaThreads / 32];
    __shared__ int redi[kMsaThreads / 32];
    __shared__ int sCol, sFound;

    const int a = blockIdx.x;
    const int tid = threadIdx.x;
    const uint64_t aid = b.first + (uint64_t)a;
    const uint32_t nf = b.nfinal[a];
    char* out = b.out + (uint64_t)a * b.outPitch;
    if (nf == 0) {
        if (tid == 0) b.flags[a] = 0;
        return;
    }
    const uint32_t base = rawOff[a];
    const uint32_t* fid = b.fid + base;
    const int16_t* fshift = b.fshift + base;
    uint8_t* forient = b.forient + base;
    const float* fweight = b.fweight + base;
    const int La = st.len[aid];
    const uint32_t* aenc = st.enc + aid * (uint64_t)st.pitch;
    const uint8_t* aq = p.useQuality ? st.qual + aid * (uint64_t)st.lmax : nullptr;

    int aBegin = 0, nCols = 0, nActive = (int)nf, builds = 0;
    for (int iter = 0;; iter++) {
        // columns of the current MSA (src/msa.cpp:19-33)
        int lo = 0, hi = La, act = 0;
        for (uint32_t j = tid; j < nf; j += kMsaThreads) {
            if (!(forient[j] & kRemoved)) {
                const int s = fshift[j];
                lo = min(lo, s);
                hi = max(hi, s + (int)st.len[fid[j]]);
                act++;
            }
        }
        lo = block_reduce_i(lo, redi, 0);
        hi = block_reduce_i(hi, redi, 1);
        nActive = block_reduce_i(act, redi, 2);
        nCols = hi - lo;
        aBegin = -lo;
        const int aEnd = aBegin + La;
        // build: counts, weights, consensus, support, original-base coverage
        for (int c = tid; c < nCols; c += kMsaThreads) {
            int nA = 0, nC = 0, nG = 0, nT = 0, cv = 0;
            float wA = 0.0f, wC = 0.0f, wG = 0.0f, wT = 0.0f;
            auto add = [&](uint32_t bb, float w) {
                switch (bb) {
                    case 0: nA++; wA = __fadd_rn(wA, w); break;
                    case 1: nC++; wC = __fadd_rn(wC, w); break;
                    case 2: nG++; wG = __fadd_rn(wG, w); break;
                    default: nT++; wT = __fadd_rn(wT, w); break;
                }
                cv++;
            };
            uint32_t anchorBase = 0;
            if (c >= aBegin && c < aEnd) {
                const int pos = c - aBegin;
                anchorBase = get2bit(aenc, pos);
                const float w = p.useQuality ? __fmul_rn(1.0f, p.qweight[aq[pos]]) : 1.0f;
                add(anchorBase, w);
            }
            for (uint32_t j = 0; j < nf; j++) {
                const uint8_t o = forient[j];
                if (o & kRemoved) continue;
                const int rb = aBegin + fshift[j];
                const uint32_t id = fid[j];
                const int Lc = st.len[id];
                if (c < rb || c >= rb + Lc) continue;
                const int pos = c - rb;
                const bool rc = o == 2;
                const uint32_t bb = oriented_base(st.enc + (uint64_t)id * st.pitch, Lc, rc, pos);
                float w = fweight[j];
                if (p.useQuality) {
                    const uint8_t q = st.qual[(uint64_t)id * st.lmax + (rc ? Lc - 1 - pos : pos)];
                    w = __fmul_rn(w, p.qweight[q]);
                }
                add(bb, w);
            }
            // findConsensus (src/msa.cpp:135-157)
            char cs = 'A';
            float cw = wA;
            if (wC > cw) { cs = 'C'; cw = wC; }
            if (wG > cw) { cs = 'G'; cw = wG; }
            if (wT > cw) { cs = 'T'; cw = wT; }
            const float colW = __fadd_rn(__fadd_rn(__fadd_rn(wA, wC), wG), wT);
            cntA[c] = nA; cntC[c] = nC; cntG[c] = nG; cntT[c] = nT;
            cov[c] = cv;
            sup[c] = __fdiv_rn(cw, colW);
            cons[c] = cs;
            if (c >= aBegin && c < aEnd) {
                origCov[c] = anchorBase == 0 ? nA : anchorBase == 1 ? nC : anchorBase == 2 ? nG : nT;
            }
        }
        builds++;
        __syncthreads();
        if (iter == 5 || nActive == 0) break;
        // findCandidatesOfDifferentRegion (src/msa.cpp:532-734)
        bool mism = false;
        for (int c = aBegin + tid; c < aEnd; c += kMsaThreads) {
            const char ab = "ACGT"[get2bit(aenc, c - aBegin)];
            mism |= cons[c] != ab;
        }
        if (!__syncthreads_or(mism)) break;
        if (tid == 0) sCol = 0x7fffffff;
        __syncthreads();
        for (int c = aBegin + tid; c < aEnd; c += kMsaThreads) {
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
        bool veto = false, any = false;
        for (uint32_t j = tid; j < nf; j += kMsaThreads) {
            const uint8_t o = forient[j];
            if (o & kRemoved) continue;
            const int rb = aBegin + fshift[j];
            const uint32_t id = fid[j];
            const int Lc = st.len[id];
            if (col < rb || col >= rb + Lc) continue;
            const uint32_t bb = oriented_base(st.enc + (uint64_t)id * st.pitch, Lc, o == 2, col - rb);
            const bool rm = keepMatching ? (bb != found) : (bb == found);
            if (rm) {
                any = true;
                veto |= fweight[j] >= 0.90f;
            }
        }
        const bool anyVeto = __syncthreads_or(veto);
        const bool anyRemove = __syncthreads_or(any);
        // a veto (or nothing to remove) leaves the MSA as it is; the
        // reference then rebuilds the same MSA and reaches the same decision
        if (anyVeto || !anyRemove) break;
        for (uint32_t j = tid; j < nf; j += kMsaThreads) {
            const uint8_t o = forient[j];
            if (o & kRemoved) continue;
            const int rb = aBegin + fshift[j];
            const uint32_t id = fid[j];
            const int Lc = st.len[id];
            if (col < rb || col >= rb + Lc) continue;
            const uint32_t bb = oriented_base(st.enc + (uint64_t)id * st.pitch, Lc, o == 2, col - rb);
            const bool rm = keepMatching ? (bb != found) : (bb == found);
            if (rm) forient[j] = o | kRemoved;
        }
        __syncthreads();
    }
    // getMSAProperties (src/msa.cpp:304-376) and getCorrectedAnchor (:379-453)
    const int aEnd = aBegin + La;
    float mins = 3.402823466e+38f;
    int minc = 0x7fffffff, maxc = -1;
    for (int c = aBegin + tid; c < aEnd; c += kMsaThreads) {
        mins = fminf(mins, sup[c]);
        minc = min(minc, cov[c]);
        maxc = max(maxc, cov[c]);
    }
    mins = block_min_f(mins, redf);
    minc = block_reduce_i(minc, redi, 0);
    maxc = block_reduce_i(maxc, redi, 1);
    __shared__ int sByConsensus, sHQ;
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
        sHQ = hq;
        if (nActive > 0) {
            atomicAdd(&b.counters[kCounterCorrected], 1ull);
            if (hq) atomicAdd(&b.counters[kCounterHQ], 1ull);
        }
        atomicAdd(&b.counters[kCounterMsaBuilds], (unsigned long long)builds);
        b.flags[a] = nActive > 0 ? (uint8_t)(CG_RESULT_CORRECTED | (hq ? CG_RESULT_HQ : 0)) : (uint8_t)0;
    }
    __syncthreads();
    (void)maxc;
    if (nActive == 0) return;
    const bool byCons = sByConsensus;
    for (int i = tid; i < La; i += kMsaThreads) {
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

}  // namespace

cudaError_t launch_align_filter(StoreArg st, Params p, BatchArg b, cudaStream_t s) {
    const size_t smem = (size_t)kAlignWarps * 6 * st.wp * sizeof(uint32_t);
    const unsigned blocks = (unsigned)((b.count + kAlignWarps - 1) / kAlignWarps);
    align_filter_kernel<<<blocks, kAlignWarps * 32, smem, s>>>(st, p, b, b.rawCount);
    return cudaGetLastError();
}

size_t msa_smem_bytes(int maxCols) { return (size_t)maxCols * (7 * sizeof(int) + 1); }

cudaError_t launch_msa_correct(StoreArg st, Params p, BatchArg b, cudaStream_t s) {
    const int maxCols = 3 * st.lmax + 4;
    const size_t smem = msa_smem_bytes(maxCols);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(msa_correct_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    msa_correct_kernel<<<b.count, kMsaThreads, smem, s>>>(st, p, b, b.rawCount, maxCols);
    return cudaGetLastError();
}

}  // namespace cg
