// ORACLE -- test infrastructure, not product code.
//
// A plain C++ restatement of the reference CARE correction path (RabbitQCPlus
// --correctWithCare, correctionType Classic) used only as the checker of the
// GPU path in tests/, in __graft_entry__.smoke() and as bench.py's CPU
// baseline.  The product library never links or calls it.
//
// Parity pin: its outputs are checked against fixtures produced by the
// reference itself (oracle/ref.mk builds the reference's own sources here;
// tests/golden/make_golden.py runs them), see tests/test_oracle_golden.py.
//
// Each function names the reference code it restates (paths relative to the
// reference project).  Floating-point expressions keep the reference's
// operand order; the file is compiled as ISO C++17 with -ffp-contract=off, as
// the reference is.

#include <care_gpu.h>

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------- helpers

// reference: include/hostdevicefunctions.cuh:9-28 (feq / fleq / fgeq)
inline bool feq(float l, float r) {
    const float d = l - r < 0 ? -(l - r) : l - r;
    return d < 1e-5f;
}
inline bool fleq(float l, float r) { return (l < r) || feq(l, r); }
inline bool fgeq(float l, float r) { return (l > r) || feq(l, r); }

// reference: include/hpc_helpers/include/hashers.cuh:129-136 (64-bit Murmur finalizer)
inline uint64_t murmur64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

inline int sdiv(int a, int b) { return (a + b - 1) / b; }

const char kBase[4] = {'A', 'C', 'G', 'T'};

inline uint32_t baseCode(char c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return 0;
    }
}

inline char complementChar(char c) {
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T': return 'A';
        default: return c;
    }
}

// reference: include/sequencehelpers.hpp:151-186 (encodeSequence2Bit):
// 16 bases per 32-bit word, first base in the two most significant bits,
// the last word left-aligned.
void encode2bit(uint32_t* out, const char* s, int len) {
    const int words = sdiv(len, 16);
    for (int w = 0; w < words; w++) out[w] = 0;
    for (int i = 0; i < len; i++) out[i / 16] |= baseCode(s[i]) << (30 - 2 * (i % 16));
}

inline uint32_t get2bit(const uint32_t* enc, int i) { return (enc[i / 16] >> (30 - 2 * (i % 16))) & 3u; }

void decode2bit(char* out, const uint32_t* enc, int len) {
    for (int i = 0; i < len; i++) out[i] = kBase[get2bit(enc, i)];
}

// ---------------------------------------------------------------- read store

struct Store {
    uint64_t n = 0;
    int Lmax = 0;
    int pitch = 0;  // words of 16 bases per read
    std::vector<uint32_t> enc;
    std::vector<int> len;
    std::vector<char> qual;  // n * Lmax
    std::vector<uint8_t> ambig;
    bool hasQual = false;
    // hi/lo planes of every read, forward then reverse complement, W words per
    // plane (reference: include/sequencehelpers.hpp:264-324 and 645-691,
    // reverseComplementSequence2Bit and convert2BitTo2BitHiLo: hi plane = high
    // bit of each base code, lo plane = low bit, 32 bases per word, first base
    // in the most significant bit).  The reference converts them per call
    // (include/corrector.hpp:880-922); kept here once per read: same bits.
    int W = 0;
    std::vector<uint32_t> hilo;  // n * 4 * W: fwd hi, fwd lo, rc hi, rc lo
    const uint32_t* planes(uint64_t id, bool rc) const { return &hilo[(id * 4 + (rc ? 2 : 0)) * size_t(W)]; }
};

struct Tables {
    int k = 20;
    int nmaps = 48;
    int maxValuesPerKey = 75;
    uint64_t kmask = 0;
    // per map: the kept keys in an open-addressing lookup (reference:
    // include/cpuhashtable.hpp:30-292, AoSCpuSingleValueHashTable: murmur64 of
    // the key, linear probing) to the range of their read ids in `values`
    struct Slot {
        uint64_t key;
        uint32_t begin, count;  // count 0: empty slot (kept keys have 2 or more ids)
    };
    std::vector<std::vector<Slot>> slots;
    std::vector<std::vector<uint32_t>> values;
    // signatures are not kept: a query recomputes its anchor's, as the
    // reference's query does (include/ordinaryminhasher.hpp:155-169)
};

// reference: include/forest.hpp:21-67 (node layout, preorder file format)
struct ForestNode {
    uint8_t att;
    uint8_t flag;  // bit 1: lhs is a leaf, bit 0: rhs is a leaf
    double split;
    uint32_t lhs, rhs;  // child index, or the leaf's float bits
};

struct Forest {
    std::vector<std::vector<ForestNode>> trees;
    float thresh = 0.5f;
};

// A candidate correction record (reference: TempCorrectedSequence of type
// Candidate, include/corrector.hpp:1674-1748): read `read` corrected by the
// MSA of anchor `anchor`, in the read's forward orientation.
struct CandRec {
    uint32_t read;
    uint32_t anchor;
    std::string seq;
};

struct Oracle {
    cg_options o;
    Forest forest;
    Store s;
    Tables t;
    float qweight[256];
    double buildSeconds = 0;
};

// reference: include/cpusequencehasher.hpp:86-125 (hashInto) with the canonical
// k-mer walk of include/sequencehelpers.hpp:842-930: for each hash function h,
// the minimum over canonical k-mers of murmur64(kmer + h), masked to 2k bits.
// Reads shorter than k keep the all-ones value (masked).  Maps [h0, h1) only;
// out[h - h0].
void signatureMaps(const uint32_t* enc, int len, int k, int h0, int h1, uint64_t* out) {
    const uint64_t kmask = k == 32 ? ~0ull : ((1ull << (2 * k)) - 1);
    uint64_t mins[CG_MAX_HASHMAPS];
    for (int h = h0; h < h1; h++) mins[h - h0] = ~0ull;
    if (len >= k) {
        uint64_t fwd = 0, rc = 0;
        for (int i = 0; i < len; i++) {
            const uint64_t b = get2bit(enc, i);
            fwd = ((fwd << 2) | b) & kmask;
            rc = (rc >> 2) | ((3ull - b) << (2 * (k - 1)));
            if (i >= k - 1) {
                const uint64_t canon = std::min(fwd, rc);
                for (int h = h0; h < h1; h++)
                    mins[h - h0] = std::min(mins[h - h0], murmur64(canon + uint64_t(h)));
            }
        }
    }
    for (int h = h0; h < h1; h++) out[h - h0] = mins[h - h0] & kmask;
}

void signature(const uint32_t* enc, int len, int k, int nmaps, uint64_t* out) {
    signatureMaps(enc, len, k, 0, nmaps, out);
}

// reference: include/chunkedreadstorageconstruction.hpp:67-92 (preprocessSequence),
// :243-282 (the encoder loop: the round-robin counter restarts for every batch of
// 65536 parsed reads) and include/qualityscorecompression.hpp:337 (8-bit
// qualities are stored unchanged).
void buildStore(Oracle& O, const char* seqs, const uint64_t* offs, const char* quals, uint64_t n) {
    Store& s = O.s;
    s.n = n;
    s.Lmax = 0;
    for (uint64_t i = 0; i < n; i++) s.Lmax = std::max<int>(s.Lmax, int(offs[i + 1] - offs[i]));
    s.pitch = sdiv(std::max(s.Lmax, 1), 16);
    s.enc.assign(n * s.pitch, 0);
    s.len.resize(n);
    s.ambig.assign(n, 0);
    s.hasQual = quals != nullptr;
    if (s.hasQual) s.qual.assign(n * size_t(s.Lmax), 0);
    int Ncount = 0;
    std::string tmp;
    for (uint64_t i = 0; i < n; i++) {
        if (i % 65536 == 0) Ncount = 0;
        const int L = int(offs[i + 1] - offs[i]);
        tmp.assign(seqs + offs[i], L);
        bool amb = false;
        for (auto& c : tmp) {
            if (c == 'a') c = 'A';
            else if (c == 'c') c = 'C';
            else if (c == 'g') c = 'G';
            else if (c == 't') c = 'T';
            else if (c != 'A' && c != 'C' && c != 'G' && c != 'T') {
                c = kBase[Ncount];
                Ncount = (Ncount + 1) % 4;
                amb = true;
            }
        }
        s.len[i] = L;
        s.ambig[i] = amb;
        encode2bit(&s.enc[i * s.pitch], tmp.data(), L);
        if (s.hasQual) std::memcpy(&s.qual[i * size_t(s.Lmax)], quals + offs[i], L);
    }
    s.W = sdiv(std::max(s.Lmax, 1), 32) + 1;
    s.hilo.assign(n * 4 * size_t(s.W), 0);
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < int64_t(n); i++) {
        const int L = s.len[i];
        const uint32_t* enc = &s.enc[i * s.pitch];
        uint32_t* fh = &s.hilo[uint64_t(i) * 4 * s.W];
        uint32_t* fl = fh + s.W;
        uint32_t* rh = fl + s.W;
        uint32_t* rl = rh + s.W;
        for (int p = 0; p < L; p++) {
            const uint32_t b = get2bit(enc, p);
            const uint32_t c = 3u - b;  // complement; reverse-complement position L-1-p
            const int q = L - 1 - p;
            fh[p / 32] |= (b >> 1) << (31 - (p % 32));
            fl[p / 32] |= (b & 1u) << (31 - (p % 32));
            rh[q / 32] |= (c >> 1) << (31 - (q % 32));
            rl[q / 32] |= (c & 1u) << (31 - (q % 32));
        }
    }
    // reference: include/qualityscorecompression.hpp:25-140 (QualityCompressorConfig<1|2>,
    // encodeQualityString: the first bin whose boundary is >= Q, Q = int(char) - 33;
    // decodeQualityToString: the bin's score) as include/chunkedreadstorage.hpp:532-607
    // decodes a whole Lmax row, so positions past a read's end (zero bits in
    // the reference's row) decode to the first bin's score.
    const int bits = O.o.quality_score_bits == 0 ? 8 : O.o.quality_score_bits;
    if (s.hasQual && (bits == 1 || bits == 2)) {
        static const int bound1[2] = {13, 256}, bound2[4] = {4, 13, 20, 256};
        static const char score1[2] = {'(', '5'}, score2[4] = {'$', '(', '1', '9'};
        const int* bound = bits == 1 ? bound1 : bound2;
        const char* score = bits == 1 ? score1 : score2;
        for (uint64_t i = 0; i < n; i++) {
            char* row = &s.qual[i * size_t(s.Lmax)];
            for (int p = 0; p < s.Lmax; p++) {
                int bin = 0;
                if (p < s.len[i]) {
                    const int Q = int(int8_t(row[p])) - 33;
                    while (Q > bound[bin]) bin++;
                }
                row[p] = score[bin];
            }
        }
    }
}

// reference: src/cpuminhasherconstruction.cpp:27-165 with
// include/ordinaryminhasher.hpp:376-426 (insert), :223-254 (compact) and
// include/groupbykey.hpp:69-250: per map, (key, readId) pairs grouped by key,
// read ids ascending; keys with fewer than 2 or more than maxValuesPerKey ids
// keep no values.  maxValuesPerKey = calculateResultsPerMapThreshold(int(coverage))
// (include/minhasherlimit.hpp:9-15).
void buildTables(Oracle& O, int threads) {
    const Store& s = O.s;
    Tables& t = O.t;
    t.k = O.o.kmerlength;
    if (t.k == 0) t.k = s.Lmax < 160 ? 20 : 32;  // src/dispatch_care_correct_cpu.cpp:81-95
    t.nmaps = O.o.num_hash_functions;
    t.kmask = t.k == 32 ? ~0ull : ((1ull << (2 * t.k)) - 1);
    {
        const int cov = int(O.o.estimated_coverage);
        int r = int(cov * 2.5f);
        r = std::min(r, 65535);
        r = std::max(10, r);
        t.maxValuesPerKey = r;
    }
    t.slots.assign(t.nmaps, {});
    t.values.assign(t.nmaps, {});
    // maps in waves of up to 8: the (key, read id) pairs of a wave's maps are
    // the only per-read data held (16 bytes per read and map)
    const int wave = std::max(1, std::min(8, t.nmaps));
    const uint32_t upper = uint32_t(std::min(t.maxValuesPerKey, 65535));
    for (int h0 = 0; h0 < t.nmaps; h0 += wave) {
        const int h1 = std::min(t.nmaps, h0 + wave);
        const int w = h1 - h0;
        std::vector<std::vector<std::pair<uint64_t, uint32_t>>> kv(w);
        for (auto& v : kv) v.resize(s.n);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1024)
        for (int64_t i = 0; i < int64_t(s.n); i++) {
            uint64_t sig[CG_MAX_HASHMAPS];
            signatureMaps(&s.enc[i * s.pitch], s.len[i], t.k, h0, h1, sig);
            for (int j = 0; j < w; j++) kv[j][i] = {sig[j], uint32_t(i)};
        }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
        for (int j = 0; j < w; j++) {
            const int h = h0 + j;
            auto& v = kv[j];
            std::sort(v.begin(), v.end());
            uint64_t kept = 0;
            for (uint64_t a = 0; a < v.size();) {
                uint64_t b = a;
                while (b < v.size() && v[b].first == v[a].first) b++;
                if (b - a >= 2 && b - a <= upper) kept++;
                a = b;
            }
            uint64_t cap = 16;
            while (cap < 2 * kept) cap <<= 1;
            auto& sl = t.slots[h];
            sl.assign(cap, Tables::Slot{0, 0, 0});
            for (uint64_t a = 0; a < v.size();) {
                uint64_t b = a;
                while (b < v.size() && v[b].first == v[a].first) b++;
                const uint64_t num = b - a;
                if (num >= 2 && num <= upper) {
                    uint64_t i = murmur64(v[a].first) & (cap - 1);
                    while (sl[i].count) i = (i + 1) & (cap - 1);
                    sl[i] = Tables::Slot{v[a].first, uint32_t(t.values[h].size()), uint32_t(num)};
                    for (uint64_t q = a; q < b; q++) t.values[h].push_back(v[q].second);
                }
                a = b;
            }
            std::vector<std::pair<uint64_t, uint32_t>>().swap(v);
            t.values[h].shrink_to_fit();
        }
    }
}

// ---------------------------------------------------------------- alignment

struct Aln {
    int score, overlap, shift, nOps;
    bool isValid;
};

// reference: src/cpu_alignment.cpp:32-497 (cpuShiftedHammingDistancePopcount2BitHiLo):
// right shifts 0..La-minov (anchor shifted), then left shifts -1..-(Lc-minov)
// (candidate shifted); per shift the mismatch count over the overlap, the
// first shift with the smallest score wins; each direction stops once no later
// shift can win (max_errors <= 0).
Aln align(const uint32_t* aHi, const uint32_t* aLo, int La, const uint32_t* cHi, const uint32_t* cLo, int Lc,
          int min_overlap, float maxErrorRate, float min_overlap_ratio) {
    const int totalbases = La + Lc;
    const int minoverlap = std::max(min_overlap, int(float(La) * min_overlap_ratio));
    int bestScore = totalbases;
    int bestShift = -Lc;
    auto mismatches = [&](const uint32_t* shHi, const uint32_t* shLo, int shiftLen, const uint32_t* oHi,
                          const uint32_t* oLo, int ov, int maxErrors) {
        const int parts = (ov + 31) >> 5;
        const int rem = (parts << 5) - ov;
        const int ws = shiftLen >> 5, bs = shiftLen & 31;
        int result = 0;
        auto word = [&](const uint32_t* p, int i) {
            const uint32_t a = p[i + ws] << bs;
            const uint32_t b = bs == 0 ? 0u : (p[i + ws + 1] >> (32 - bs));
            return a | b;
        };
        for (int i = 0; i < parts - 1 && result < maxErrors; i++) {
            result += __builtin_popcount((word(shHi, i) ^ oHi[i]) | (word(shLo, i) ^ oLo[i]));
        }
        if (result < maxErrors) {
            const uint32_t mask = rem == 0 ? 0xFFFFFFFFu : 0xFFFFFFFFu << rem;
            result += __builtin_popcount(((word(shHi, parts - 1) ^ oHi[parts - 1]) |
                                          (word(shLo, parts - 1) ^ oLo[parts - 1])) & mask);
        }
        return result;
    };
    for (int shift = 0; shift < La - minoverlap + 1; ++shift) {
        const int ov = std::min(La - shift, Lc);
        const int maxErr = std::min(int(float(ov) * maxErrorRate), bestScore - totalbases + 2 * ov);
        if (maxErr <= 0) break;
        const int m = mismatches(aHi, aLo, shift, cHi, cLo, ov, maxErr);
        const int score = m < maxErr ? m + totalbases - 2 * ov : std::numeric_limits<int>::max();
        if (score < bestScore) {
            bestScore = score;
            bestShift = shift;
        }
    }
    for (int shift = -1; shift >= -Lc + minoverlap; --shift) {
        const int ov = std::min(La, Lc + shift);
        const int maxErr = std::min(int(float(ov) * maxErrorRate), bestScore - totalbases + 2 * ov);
        if (maxErr <= 0) break;
        const int m = mismatches(cHi, cLo, -shift, aHi, aLo, ov, maxErr);
        const int score = m < maxErr ? m + totalbases - 2 * ov : std::numeric_limits<int>::max();
        if (score < bestScore) {
            bestScore = score;
            bestShift = shift;
        }
    }
    Aln r;
    r.isValid = bestShift != -Lc;
    const int cb = std::max(-bestShift, 0);
    const int ce = std::min(Lc, La - bestShift);
    const int ov = ce - cb;
    r.score = bestScore;
    r.overlap = ov;
    r.shift = bestShift;
    r.nOps = bestScore - totalbases + 2 * ov;
    return r;
}

// reference: include/alignmentorientation.hpp:10-92 (chooseBestAlignmentOrientation):
// 1 = forward, 2 = reverse complement, 3 = none
int orientation(const Aln& f, const Aln& r, int La, float min_overlap_ratio, int min_overlap, float maxErrorRate) {
    const int minimumOverlap = int(La * min_overlap_ratio) > min_overlap ? int(La * min_overlap_ratio) : min_overlap;
    int ret = 3;
    if (f.isValid && f.overlap >= minimumOverlap) {
        if (r.isValid && r.overlap >= minimumOverlap) {
            const float ratio = (float)f.nOps / f.overlap;
            const float revcomplratio = (float)r.nOps / r.overlap;
            if (ratio < revcomplratio) {
                if (ratio < maxErrorRate) ret = 1;
            } else if (revcomplratio < ratio) {
                if (revcomplratio < maxErrorRate) ret = 2;
            } else {
                if (ratio < maxErrorRate) ret = f.overlap > r.overlap ? 1 : 2;
            }
        } else {
            if ((float)f.nOps / f.overlap < maxErrorRate) ret = 1;
        }
    } else {
        if (r.isValid && r.overlap >= minimumOverlap) {
            if ((float)r.nOps / r.overlap < maxErrorRate) ret = 2;
        }
    }
    return ret;
}

// ---------------------------------------------------------------- MSA

struct Cand {
    uint32_t id;
    int len;
    int orient;  // 1 fwd, 2 rc
    Aln aln;
    bool paired;
    float weight;
    std::string seq;   // bases in aligned orientation
    std::string qual;  // qualities in aligned orientation (reversed for rc)
};

struct Msa {
    int nColumns = 0, begin = 0, end = 0, nCand = 0;
    std::vector<int> cA, cC, cG, cT, cov, origCov;
    std::vector<float> wA, wC, wG, wT, support, origW;
    std::string cons;
};

// reference: src/msa.cpp:9-173 (build, addSequence, findConsensus,
// findOrigWeightAndCoverage).  Column weights are accumulated anchor first,
// then candidates in list order.
void buildMsa(Msa& m, const std::string& anchor, const std::string& aqual, const std::vector<Cand>& cs,
              bool useQ, const float* qw) {
    int startindex = 0, endindex = int(anchor.size());
    for (const auto& c : cs) {
        startindex = std::min(c.aln.shift, startindex);
        endindex = std::max(c.len + c.aln.shift, endindex);
    }
    m.nColumns = endindex - startindex;
    m.begin = std::max(-startindex, 0);
    m.end = m.begin + int(anchor.size());
    m.nCand = int(cs.size());
    const int C = m.nColumns;
    for (auto* v : {&m.cA, &m.cC, &m.cG, &m.cT, &m.cov, &m.origCov}) v->assign(C, 0);
    for (auto* v : {&m.wA, &m.wC, &m.wG, &m.wT, &m.support, &m.origW}) v->assign(C, 0.0f);
    m.cons.assign(C, 0);
    auto add = [&](const std::string& seq, const std::string& q, int shift, float f) {
        for (int i = 0; i < int(seq.size()); i++) {
            const int g = m.begin + shift + i;
            const float w = f * (useQ ? qw[(unsigned char)q[i]] : 1.0f);
            switch (seq[i]) {
                case 'A': m.cA[g]++; m.wA[g] += w; break;
                case 'C': m.cC[g]++; m.wC[g] += w; break;
                case 'G': m.cG[g]++; m.wG[g] += w; break;
                case 'T': m.cT[g]++; m.wT[g] += w; break;
            }
            m.cov[g]++;
        }
    };
    add(anchor, aqual, 0, 1.0f);
    for (const auto& c : cs) add(c.seq, c.qual, c.aln.shift, c.weight);
    for (int col = 0; col < C; col++) {
        char cons = 'A';
        float cw = m.wA[col];
        if (m.wC[col] > cw) { cons = 'C'; cw = m.wC[col]; }
        if (m.wG[col] > cw) { cons = 'G'; cw = m.wG[col]; }
        if (m.wT[col] > cw) { cons = 'T'; cw = m.wT[col]; }
        m.cons[col] = cons;
        const float colW = m.wA[col] + m.wC[col] + m.wG[col] + m.wT[col];
        m.support[col] = cw / colW;
    }
    for (int col = m.begin; col < m.end; col++) {
        switch (anchor[col - m.begin]) {
            case 'A': m.origW[col] = m.wA[col]; m.origCov[col] = m.cA[col]; break;
            case 'C': m.origW[col] = m.wC[col]; m.origCov[col] = m.cC[col]; break;
            case 'G': m.origW[col] = m.wG[col]; m.origCov[col] = m.cG[col]; break;
            case 'T': m.origW[col] = m.wT[col]; m.origCov[col] = m.cT[col]; break;
        }
    }
}

// reference: src/msa.cpp:532-734 (findCandidatesOfDifferentRegion); returns
// false when no minimization is performed, else fills `remove`.
bool differentRegion(const Msa& m, const std::string& anchor, const std::vector<Cand>& cs, int datasetCoverage,
                     std::vector<char>& remove) {
    if (anchor.compare(0, anchor.size(), m.cons, m.begin, anchor.size()) == 0) return false;
    const int thr = int(datasetCoverage * 0.3f);
    int col = -1, foundIdx = -1, consIdx = -1;
    for (int c = m.begin; c < m.end && col < 0; c++) {
        const int counts[4] = {m.cA[c], m.cC[c], m.cG[c], m.cT[c]};
        const char cons = m.cons[c];
        consIdx = cons == 'A' ? 0 : cons == 'C' ? 1 : cons == 'G' ? 2 : 3;
        int sig = -1;
        for (int i = 0; i < 4; i++)
            if (i != consIdx && thr <= counts[i]) sig = i;
        if (sig != -1) {
            col = c;
            foundIdx = sig;
        }
    }
    if (col < 0) return false;
    const char foundBase = kBase[foundIdx];
    const char origBase = anchor[col - m.begin];
    const bool keepMatching = origBase == foundBase;
    remove.assign(cs.size(), 0);
    for (size_t i = 0; i < cs.size(); i++) {
        const int rb = m.begin + cs[i].aln.shift;
        const int re = rb + cs[i].len;
        if (col < rb || re <= col) continue;
        const char b = cs[i].seq[col - rb];
        if (keepMatching ? (b != foundBase) : (b == foundBase)) remove[i] = 1;
    }
    for (size_t i = 0; i < cs.size(); i++) {
        if (remove[i] && cs[i].weight >= 0.90f) {
            std::fill(remove.begin(), remove.end(), 0);
            break;
        }
    }
    return true;
}

struct Props {
    float avg_support, min_support;
    int min_coverage, max_coverage;
    bool isHQ;
};

// reference: src/msa.cpp:304-376 (getMSAProperties)
Props msaProperties(const Msa& m, float err, float cov, float mcov) {
    const float avgThr = 1.0f - 1.0f * err;
    const float minThr = 1.0f - 3.0f * err;
    const float covThr = mcov / 6.0f * cov;
    const int first = m.begin, last = m.end, dist = last - first;
    Props p;
    p.min_support = *std::min_element(m.support.begin() + first, m.support.begin() + last);
    float sum = 0.0f;
    for (int c = first; c < last; c++) sum += m.support[c];
    p.avg_support = sum / dist;
    p.min_coverage = *std::min_element(m.cov.begin() + first, m.cov.begin() + last);
    p.max_coverage = *std::max_element(m.cov.begin() + first, m.cov.begin() + last);
    p.isHQ = false;
    const bool allGood = fgeq(p.avg_support, avgThr) && fgeq(p.min_support, minThr) && fgeq(float(p.min_coverage), covThr);
    if (allGood) {
        int smallest = 100;
        const int pct = int(std::ceil(err * 100.0f));
        for (int percent = pct; percent >= 0; percent--) {
            const float factor = percent / 100.0f;
            if (fgeq(p.avg_support, 1.0f - 1.0f * factor) && fgeq(p.min_support, 1.0f - 3.0f * factor)) smallest = percent;
        }
        p.isHQ = fgeq(float(p.min_coverage), covThr) && fleq(float(smallest), pct * 0.5f);
    }
    return p;
}

// reference: src/msa.cpp:379-453 (getCorrectedAnchor)
bool correctedAnchor(const Msa& m, const Props& p, const std::string& anchor, float err, float cov, float mcov,
                     std::string& out) {
    if (m.nCand == 0) return false;
    const float avgThr = 1.0f - 1.0f * err;
    const float minThr = 1.0f - 3.0f * err;
    const float covThr = mcov / 6.0f * cov;
    const bool byConsensus = fgeq(p.avg_support, avgThr) && fgeq(p.min_support, minThr) && fgeq(float(p.min_coverage), covThr);
    out.resize(anchor.size());
    if (byConsensus) {
        for (size_t i = 0; i < anchor.size(); i++) out[i] = m.cons[m.begin + i];
    } else {
        for (size_t i = 0; i < anchor.size(); i++) {
            const int c = m.begin + int(i);
            out[i] = (m.support[c] > 0.90f && m.origCov[c] <= 2) ? m.cons[c] : anchor[i];
        }
    }
    return true;
}

// reference: include/classification.hpp:748-797 (extract_anchor_v3)
void anchorFeatures(const Msa& m, const Props& p, int i, float cov, float out[13]) {
    const int pos = m.begin + i;
    const float wsum = m.wA[pos] + m.wC[pos] + m.wG[pos] + m.wT[pos];
    float weightCons = 0, countCons = 0;
    switch (m.cons[pos]) {
        case 'A': weightCons = m.wA[pos]; countCons = m.cA[pos]; break;
        case 'C': weightCons = m.wC[pos]; countCons = m.cC[pos]; break;
        case 'G': weightCons = m.wG[pos]; countCons = m.cG[pos]; break;
        case 'T': weightCons = m.wT[pos]; countCons = m.cT[pos]; break;
    }
    out[0] = float(m.origCov[pos]) / m.cov[pos];
    out[1] = m.origW[pos] / wsum;
    out[2] = m.origW[pos] / m.origCov[pos];
    out[3] = countCons / m.cov[pos];
    out[4] = m.support[pos];
    out[5] = weightCons / countCons;
    out[6] = wsum / m.cov[pos];
    out[7] = m.cov[pos] / cov;
    out[8] = wsum / cov;
    out[9] = p.avg_support;
    out[10] = p.min_support;
    out[11] = float(p.max_coverage) / cov;
    out[12] = float(p.min_coverage) / cov;
}

// reference: include/forest.hpp:70-81 (prob) and 217-226 (decide)
bool forestDecide(const Forest& f, const float* feats) {
    float sum = 0.f;
    for (const auto& tree : f.trees) {
        size_t i = 0;
        float prob;
        while (true) {
            const ForestNode& n = tree[i];
            if (feats[n.att] <= n.split) {
                if (n.flag / 2) { std::memcpy(&prob, &n.lhs, 4); break; }
                i = n.lhs;
            } else {
                if (n.flag % 2) { std::memcpy(&prob, &n.rhs, 4); break; }
                i = n.rhs;
            }
        }
        sum += prob;
        if (sum / f.trees.size() >= f.thresh) return true;
    }
    return false;
}

// ---------------------------------------------------------------- per anchor

std::string decodeRead(const Store& s, uint64_t id) {
    std::string r(s.len[id], 'A');
    decode2bit(&r[0], &s.enc[id * s.pitch], s.len[id]);
    return r;
}

// reference: include/corrector.hpp:571-650 (determineCandidateReadIds) with
// include/ordinaryminhasher.hpp:135-221,437-449 (determineNumValues, retrieveValues, queryMap)
void candidates(const Oracle& O, uint64_t anchor, std::vector<uint32_t>& out, uint64_t* rawCount) {
    const Store& s = O.s;
    const Tables& t = O.t;
    out.clear();
    if (O.o.exclude_ambiguous_reads && s.ambig[anchor]) return;
    if (s.len[anchor] >= t.k) {
        uint64_t sig[CG_MAX_HASHMAPS];
        signature(&s.enc[anchor * s.pitch], s.len[anchor], t.k, t.nmaps, sig);
        for (int h = 0; h < t.nmaps; h++) {
            const auto& sl = t.slots[h];
            const uint64_t mask = sl.size() - 1;
            for (uint64_t i = murmur64(sig[h]) & mask; sl[i].count; i = (i + 1) & mask) {
                if (sl[i].key != sig[h]) continue;
                out.insert(out.end(), t.values[h].begin() + sl[i].begin,
                           t.values[h].begin() + sl[i].begin + sl[i].count);
                break;
            }
        }
    }
    if (rawCount) *rawCount += out.size();
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    auto it = std::lower_bound(out.begin(), out.end(), uint32_t(anchor));
    if (it != out.end() && *it == uint32_t(anchor)) out.erase(it);
    if (O.o.exclude_ambiguous_reads) {
        out.erase(std::remove_if(out.begin(), out.end(), [&](uint32_t c) { return s.ambig[c] != 0; }), out.end());
    }
}

// reference: include/util.hpp:1005-1143 (flagPairedCandidates via
// findPositionsOfPairedReadIds, :1151-1200): positions of ids in range 1 whose
// mate (id/2 equal) is in range 2 and vice versa.
void pairFlags(const std::vector<uint32_t>& r1, const std::vector<uint32_t>& r2, std::vector<char>& f1,
               std::vector<char>& f2) {
    f1.assign(r1.size(), 0);
    f2.assign(r2.size(), 0);
    size_t a = 0, b = 0;
    while (a < r1.size() && b < r2.size()) {
        const int e1 = (a + 1 < r1.size() && r1[a] / 2 == r1[a + 1] / 2) ? 2 : 1;
        const int e2 = (b + 1 < r2.size() && r2[b] / 2 == r2[b + 1] / 2) ? 2 : 1;
        const bool same = r1[a] / 2 == r2[b] / 2;
        if (e1 == 1 && e2 == 1) {
            if (same) {
                if (r1[a] != r2[b]) { f1[a] = 1; f2[b] = 1; }
                a++; b++;
            } else {
                if (r1[a] < r2[b]) a++; else b++;
            }
        } else if (e1 == 2 && e2 == 2) {
            if (same) {
                f1[a] = 1; f2[b] = 1; f1[a + 1] = 1; f2[b + 1] = 1;
                a += 2; b += 2;
            } else {
                if (r1[a] < r2[b]) a += 2; else b += 2;
            }
        } else if (e1 == 2 && e2 == 1) {
            if (same) {
                if (r1[a] == r2[b]) { a++; f1[a] = 1; f2[b] = 1; a++; b++; }
                else { f1[a] = 1; f2[b] = 1; a++; b++; a++; }
            } else {
                if (r1[a] < r2[b]) a += 2; else b++;
            }
        } else {
            if (same) {
                if (r1[a] == r2[b]) { b++; f1[a] = 1; f2[b] = 1; a++; b++; }
                else { f1[a] = 1; f2[b] = 1; a++; b++; b++; }
            } else {
                if (r1[a] < r2[b]) a++; else b += 2;
            }
        }
    }
}

struct Counters {
    uint64_t raw = 0, uniq = 0, aligned = 0, msaCands = 0, msaBuilds = 0, corrected = 0, hq = 0;
};

// reference: include/corrector.hpp:1504-1512 (correctCandidatesClassic) and
// src/msa.cpp:457-522 (getCorrectedCandidates): every candidate of the final
// MSA whose first column lies within nc columns of the anchor's first column
// and whose last column ends at most nc columns past the anchor's end gets
// the consensus of its columns (the support and coverage test computed there
// is overwritten by `candidateShouldBeCorrected = true`).  A reverse-
// complement candidate's record holds the reverse complement of that slice
// (include/corrector.hpp:1686-1702).
void candidateCorrections(const Msa& m, const std::vector<Cand>& kept, int nc, uint64_t anchor,
                          std::vector<CandRec>& out) {
    for (const auto& c : kept) {
        const int qb = m.begin + c.aln.shift;
        const int qe = qb + c.len;
        if (!(m.begin - nc <= qb && qb <= m.begin + nc && qe <= m.end + nc)) continue;
        std::string s(m.cons.begin() + qb, m.cons.begin() + qe);
        if (c.orient == 2) {
            std::string f(s.size(), 'A');
            for (size_t i = 0; i < s.size(); i++) f[i] = complementChar(s[s.size() - 1 - i]);
            s.swap(f);
        }
        out.push_back(CandRec{c.id, uint32_t(anchor), std::move(s)});
    }
}

// reference: include/corrector.hpp:145-312 (process) and 325-513 (processMulti):
// candidates -> alignments -> orientation -> filters -> MSA -> refinement ->
// anchor correction.  Returns the CG_RESULT_* flags.
uint8_t correctOne(const Oracle& O, uint64_t anchor, const std::vector<uint32_t>& candIds,
                   const std::vector<char>& paired, std::string& corrected, Counters& cnt,
                   std::vector<CandRec>& recs) {
    const Store& s = O.s;
    const cg_options& o = O.o;
    const int La = s.len[anchor];
    if (candIds.empty()) return 0;
    cnt.uniq += candIds.size();
    const uint32_t* aHi = s.planes(anchor, false);
    const uint32_t* aLo = aHi + s.W;
    const std::string anchorStr = decodeRead(s, anchor);
    std::string anchorQ;
    if (o.use_quality_scores) anchorQ.assign(&s.qual[anchor * size_t(s.Lmax)], La);
    thread_local std::vector<Cand> cs, kept, next;  // reused across anchors
    thread_local std::vector<char> remove;
    cs.clear();
    for (size_t i = 0; i < candIds.size(); i++) {
        const uint32_t id = candIds[i];
        const int Lc = s.len[id];
        const uint32_t* cHi = s.planes(id, false);
        const uint32_t* rHi = s.planes(id, true);
        const Aln f = align(aHi, aLo, La, cHi, cHi + s.W, Lc, o.min_overlap, o.max_error_rate, o.min_overlap_ratio);
        const Aln r = align(aHi, aLo, La, rHi, rHi + s.W, Lc, o.min_overlap, o.max_error_rate, o.min_overlap_ratio);
        const int ori = orientation(f, r, La, o.min_overlap_ratio, o.min_overlap, o.estimated_errorrate * 4.0f);
        if (ori == 3) continue;
        Cand c;
        c.id = id;
        c.len = Lc;
        c.orient = ori;
        c.aln = ori == 1 ? f : r;
        c.paired = paired.empty() ? false : paired[i] != 0;
        cs.push_back(std::move(c));
    }
    cnt.aligned += cs.size();
    if (cs.empty()) return 0;
    // mismatch ratio filter: include/corrector.hpp:1053-1149 (SE), 1151-1211 (PE)
    kept.clear();
    if (o.pair_mode == CG_PAIR_PE) {
        for (auto& c : cs) {
            if (c.paired) kept.push_back(std::move(c));
            else if (float(c.aln.nOps) / float(c.aln.overlap) < o.paired_filter_threshold) kept.push_back(std::move(c));
        }
    } else {
        const float base = o.estimated_errorrate * 1.0f;
        const float goodThr = o.estimated_coverage * o.m_coverage;
        int counts[3] = {0, 0, 0};
        for (const auto& c : cs) {
            const float r = float(c.aln.nOps) / float(c.aln.overlap);
            if (r < 2 * base) counts[0]++;
            if (r < 3 * base) counts[1]++;
            if (r < 4 * base) counts[2]++;
        }
        float thr = std::numeric_limits<float>::lowest();
        if (counts[0] > 0 || counts[1] > 0 || counts[2] > 0) {
            if (counts[0] >= goodThr) thr = 2 * base;
            else if (counts[1] >= goodThr) thr = 3 * base;
            else if (counts[2] >= goodThr) thr = 4 * base;
        }
        for (auto& c : cs) {
            if (float(c.aln.nOps) / float(c.aln.overlap) < thr) kept.push_back(std::move(c));
        }
    }
    if (kept.empty()) return 0;
    // overlap weights: include/corrector.hpp:1260-1280, include/hostdevicefunctions.cuh:93-95
    for (auto& c : kept) c.weight = 1.0f - std::sqrt(c.aln.nOps / (c.aln.overlap * o.max_error_rate));
    // candidate strings in aligned orientation (include/corrector.hpp:1242-1258)
    // and their qualities (include/corrector.hpp:1214-1239: rows of Lmax
    // qualities, zero -- or the first bin with lossy qualities -- past the
    // read's end; a reverse-complement candidate's whole row is reversed, so a
    // read shorter than Lmax takes the padding first)
    for (auto& c : kept) {
        c.seq = decodeRead(s, c.id);
        if (c.orient == 2) {
            std::reverse(c.seq.begin(), c.seq.end());
            for (auto& ch : c.seq) ch = complementChar(ch);
        }
        if (o.use_quality_scores) {
            const char* row = &s.qual[c.id * size_t(s.Lmax)];
            if (c.orient == 2) {
                c.qual.assign(size_t(c.len), 0);
                for (int i = 0; i < c.len; i++) c.qual[i] = row[s.Lmax - 1 - i];
            } else {
                c.qual.assign(row, c.len);
            }
        }
    }
    cnt.msaCands += kept.size();
    thread_local Msa m;  // buffers reused across anchors
    buildMsa(m, anchorStr, anchorQ, kept, o.use_quality_scores != 0, O.qweight);
    cnt.msaBuilds++;
    // refinement: include/corrector.hpp:1307-1421
    for (int it = 0; it < 5; it++) {
        if (!differentRegion(m, anchorStr, kept, int(o.estimated_coverage), remove)) break;
        next.clear();
        for (size_t i = 0; i < kept.size(); i++)
            if (!remove[i]) next.push_back(std::move(kept[i]));
        const bool changed = next.size() != kept.size();
        kept.swap(next);
        if (!changed) break;  // an unchanged rebuild repeats the same MSA and decision
        buildMsa(m, anchorStr, anchorQ, kept, o.use_quality_scores != 0, O.qweight);
        cnt.msaBuilds++;
    }
    const Props p = msaProperties(m, o.estimated_errorrate, o.estimated_coverage, o.m_coverage);
    // include/corrector.hpp:293-299: candidates are corrected by HQ anchors
    if (o.correct_candidates && p.isHQ) candidateCorrections(m, kept, o.new_columns_to_correct, anchor, recs);
    if (o.correction_type == CG_CORR_FOREST) {
        // correctAnchorClf: include/corrector.hpp:1448-1472
        corrected.assign(m.cons.begin() + m.begin, m.cons.begin() + m.end);
        if (!p.isHQ) {
            float feats[13];
            for (int i = 0; i < La; i++) {
                if (anchorStr[i] != m.cons[m.begin + i]) {
                    anchorFeatures(m, p, i, o.estimated_coverage, feats);
                    if (!forestDecide(O.forest, feats)) corrected[i] = anchorStr[i];
                }
            }
        }
        cnt.corrected++;
        if (p.isHQ) cnt.hq++;
        return uint8_t(CG_RESULT_CORRECTED | (p.isHQ ? CG_RESULT_HQ : 0));
    }
    // correctAnchorClassic: include/corrector.hpp:1423-1446
    if (!correctedAnchor(m, p, anchorStr, o.estimated_errorrate, o.estimated_coverage, o.m_coverage, corrected)) return 0;
    cnt.corrected++;
    if (p.isHQ) cnt.hq++;
    return uint8_t(CG_RESULT_CORRECTED | (p.isHQ ? CG_RESULT_HQ : 0));
}

// reference: src/correctionresultoutput.cpp:1256-1551
// (combineMultipleCorrectionResults1_rawtcs2) over the records of a whole run,
// with the record filter of include/corrector.hpp:1678-1681 as a
// single-threaded run applies it (anchors in id order; a candidate record of
// read c made by anchor a is dropped when c < a and c was corrected as an HQ
// anchor).  Only a low-quality anchor correction with two or more candidate
// records changes: it stays if every record equals it, else the read is
// written unchanged.  Returns the number of saved candidate records.
uint64_t combine(std::vector<CandRec>& recs, uint8_t* flags, const char* out, size_t pitch, const Store& s) {
    std::sort(recs.begin(), recs.end(), [](const CandRec& x, const CandRec& y) {
        return x.read != y.read ? x.read < y.read : x.anchor < y.anchor;
    });
    uint64_t saved = 0;
    for (size_t i = 0; i < recs.size();) {
        size_t j = i;
        while (j < recs.size() && recs[j].read == recs[i].read) j++;
        const uint32_t r = recs[i].read;
        const uint8_t f = flags[r];
        const bool hqAnchor = (f & CG_RESULT_CORRECTED) && (f & CG_RESULT_HQ);
        uint64_t k = 0;
        bool same = true;
        for (size_t t = i; t < j; t++) {
            if (hqAnchor && r < recs[t].anchor) continue;
            k++;
            if (f & CG_RESULT_CORRECTED) same &= recs[t].seq.compare(0, std::string::npos, out + r * pitch, s.len[r]) == 0;
        }
        saved += k;
        if (k > 0) flags[r] |= CG_RESULT_CANDIDATE_RECORD;
        if ((f & CG_RESULT_CORRECTED) && !(f & CG_RESULT_HQ) && k >= 2)
            flags[r] |= same ? CG_RESULT_CANDIDATES : CG_RESULT_REJECTED;
        i = j;
    }
    return saved;
}

}  // namespace

extern "C" {

void* orc_create(const cg_options* o, const char* seqs, const uint64_t* offsets, const char* quals, uint64_t n,
                 int threads) {
    if (!o || !seqs || !offsets || n == 0) return nullptr;
    if (o->use_quality_scores && !quals) return nullptr;
    Oracle* O = new Oracle();
    O->o = *o;
    // reference: include/qualityscoreweights.hpp:17-33
    for (int i = 0; i < 256; i++) {
        const float p = i < 33 ? 1.0f : std::pow(10.0f, -(i - 33) / 10.0f);
        O->qweight[i] = std::max(0.001f, 1.0f - p);
    }
    const auto t0 = std::chrono::steady_clock::now();
    buildStore(*O, seqs, offsets, quals, n);
    buildTables(*O, threads);
    O->buildSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return O;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

// Forest in the reference's file format (include/forest.hpp:38-55, 141-162);
// returns 0, or -1 on a malformed file.
int orc_load_forest(void* h, const uint8_t* data, uint64_t size, uint32_t maxTrees, float thresh) {
    Oracle* O = static_cast<Oracle*>(h);
    uint64_t pos = 0;
    auto rd = [&](void* dst, uint64_t n) {
        if (pos + n > size) throw 1;
        std::memcpy(dst, data + pos, n);
        pos += n;
    };
    try {
        uint64_t dl;
        rd(&dl, 8);
        std::string desc(dl, 0);
        rd(&desc[0], dl);
        if (desc != "13 extract_anchor_v3") return -1;
        uint32_t nt;
        rd(&nt, 4);
        nt = std::min(nt, maxTrees);
        O->forest.trees.assign(nt, {});
        O->forest.thresh = thresh;
        for (auto& tree : O->forest.trees) {
            uint32_t nn;
            rd(&nn, 4);
            std::vector<std::pair<uint32_t, int>> stack;  // (node, side to fill: 0 lhs 1 rhs)
            auto readNode = [&]() -> uint32_t {
                ForestNode n;
                rd(&n.att, 1);
                rd(&n.split, 8);
                rd(&n.flag, 1);
                n.lhs = n.rhs = 0;
                tree.push_back(n);
                return uint32_t(tree.size() - 1);
            };
            // preorder: node, lhs subtree (or leaf prob), rhs subtree (or leaf prob)
            std::vector<uint32_t> path;
            uint32_t root = readNode();
            path.push_back(root);
            std::vector<int> state{0};
            while (!path.empty()) {
                const uint32_t cur = path.back();
                int& st = state.back();
                if (st == 2) {
                    path.pop_back();
                    state.pop_back();
                    continue;
                }
                const bool leaf = st == 0 ? (tree[cur].flag / 2) != 0 : (tree[cur].flag % 2) != 0;
                const int side = st;
                st++;
                if (leaf) {
                    uint32_t bits;
                    rd(&bits, 4);
                    (side == 0 ? tree[cur].lhs : tree[cur].rhs) = bits;
                } else {
                    const uint32_t child = readNode();
                    (side == 0 ? tree[cur].lhs : tree[cur].rhs) = child;
                    path.push_back(child);
                    state.push_back(0);
                }
            }
        }
    } catch (int) {
        return -1;
    }
    return 0;
}

int orc_info(void* h, uint64_t* nreads, int* lmax, int* k, int* nmaps, double* buildSeconds) {
    const Oracle* O = static_cast<Oracle*>(h);
    *nreads = O->s.n;
    *lmax = O->s.Lmax;
    *k = O->t.k;
    *nmaps = O->t.nmaps;
    *buildSeconds = O->buildSeconds;
    return 0;
}

int orc_signatures(void* h, uint64_t first, uint64_t n, uint64_t* out) {
    const Oracle* O = static_cast<Oracle*>(h);
    if (first + n > O->s.n) return CG_ERR_INVALID_ARGUMENT;
    for (uint64_t i = first; i < first + n; i++)
        signature(&O->s.enc[i * O->s.pitch], O->s.len[i], O->t.k, O->t.nmaps, out + (i - first) * O->t.nmaps);
    return 0;
}

int orc_candidates(void* h, uint64_t anchor, uint32_t* out, uint32_t cap, uint32_t* count) {
    const Oracle* O = static_cast<Oracle*>(h);
    if (anchor >= O->s.n) return CG_ERR_INVALID_ARGUMENT;
    std::vector<uint32_t> c;
    candidates(*O, anchor, c, nullptr);
    *count = uint32_t(c.size());
    std::memcpy(out, c.data(), std::min<size_t>(cap, c.size()) * 4);
    return 0;
}

// Check of the device alignment's orientation shortcut (not part of the
// reference: the GPU kernel align_lane_kernel scans one orientation first and
// skips the other where a one-plane test rules out a tie).  For every
// candidate of the anchors [first, first + count) and for each orientation
// taken as the one scanned first: the shortcut decides when that
// orientation's result would be chosen on its own (choose it against an
// invalid other), the minimum overlap is at least 32, and no shift of the
// other orientation with at least that overlap has at most L = floor(nOps *
// min(La, Lc) / overlap) + 1 hi-plane mismatches in its overlap's first 32
// bases.  out[0] = (candidate, first orientation) cases, out[1] = cases the
// shortcut decides, out[2] = decided cases where the reference's choice from
// both scans differs from the first orientation (the shortcut's claim: 0).
int orc_check_orientation_shortcut(void* h, uint64_t first, uint64_t count, int threads, uint64_t* out) {
    const Oracle* O = static_cast<Oracle*>(h);
    const Store& s = O->s;
    const cg_options& o = O->o;
    if (first + count > s.n) return CG_ERR_INVALID_ARGUMENT;
    auto bits32 = [&](const uint32_t* p, int sh) {  // bases sh .. sh + 31 of a plane
        const int w = sh >> 5, b = sh & 31;
        return b ? (p[w] << b) | (p[w + 1] >> (32 - b)) : p[w];
    };
    uint64_t cases = 0, decided = 0, wrong = 0;
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) reduction(+ : cases, decided, wrong)
    for (long long ai = 0; ai < (long long)count; ai++) {
        const uint64_t anchor = first + (uint64_t)ai;
        std::vector<uint32_t> ids;
        candidates(*O, anchor, ids, nullptr);
        const int La = s.len[anchor];
        const uint32_t* aHi = s.planes(anchor, false);
        const int minov = std::max(o.min_overlap, int(float(La) * o.min_overlap_ratio));
        for (const uint32_t id : ids) {
            const int Lc = s.len[id];
            const uint32_t* pl[2] = {s.planes(id, false), s.planes(id, true)};
            const Aln f = align(aHi, aHi + s.W, La, pl[0], pl[0] + s.W, Lc, o.min_overlap, o.max_error_rate,
                                o.min_overlap_ratio);
            const Aln r = align(aHi, aHi + s.W, La, pl[1], pl[1] + s.W, Lc, o.min_overlap, o.max_error_rate,
                                o.min_overlap_ratio);
            const float mer = o.estimated_errorrate * 4.0f;
            const int ori = orientation(f, r, La, o.min_overlap_ratio, o.min_overlap, mer);
            Aln none{};
            none.isValid = false;
            for (int po = 0; po < 2; po++) {
                cases++;
                const Aln& x1 = po == 0 ? f : r;
                const int solo = po == 0 ? orientation(x1, none, La, o.min_overlap_ratio, o.min_overlap, mer)
                                         : orientation(none, x1, La, o.min_overlap_ratio, o.min_overlap, mer);
                if (solo == 3 || minov < 32) continue;
                const int L = int((uint32_t(x1.nOps) * uint32_t(std::min(La, Lc))) / uint32_t(x1.overlap)) + 1;
                const uint32_t* oHi = pl[1 - po];
                bool close = false;
                if (Lc >= minov)
                    for (int sh = 0; sh <= La - minov && !close; sh++)
                        close = __builtin_popcount(bits32(aHi, sh) ^ oHi[0]) <= L;
                if (La >= minov)
                    for (int sh = 1; sh <= Lc - minov && !close; sh++)
                        close = __builtin_popcount(bits32(oHi, sh) ^ aHi[0]) <= L;
                if (close) continue;
                decided++;
                if (ori != solo) wrong++;
            }
        }
    }
    out[0] = cases;
    out[1] = decided;
    out[2] = wrong;
    return 0;
}

// Corrects anchors [first, first+count); flags and corrected sequences as in
// cg_correct.  With candidate correction the range must be the whole read set
// and the flags come out as cg_combine_results leaves them.  counters (8
// entries, may be NULL): raw ids, unique candidates, aligned, msa candidates,
// msa builds, corrected, hq, saved candidate records.
int orc_correct(void* h, uint64_t first, uint64_t count, uint8_t* flags, char* out, size_t pitch, int threads,
                uint64_t* counters) {
    const Oracle* O = static_cast<Oracle*>(h);
    if (first + count > O->s.n) return CG_ERR_INVALID_ARGUMENT;
    const bool pe = O->o.pair_mode == CG_PAIR_PE;
    if (pe && ((first | count) & 1)) return CG_ERR_INVALID_ARGUMENT;
    if (O->o.correct_candidates && (first != 0 || count != O->s.n)) return CG_ERR_INVALID_ARGUMENT;
    Counters total;
    std::vector<CandRec> allRecs;
    const int64_t units = int64_t(pe ? count / 2 : count);
    // reference: include/options.hpp:126-133 (getNumReadsToProcess) with
    // src/correct_cpu.cpp:97-102: only anchors below fixedNumberOfReads run
    const uint64_t limit = O->o.fixed_number_of_reads ? std::min<uint64_t>(O->o.fixed_number_of_reads, O->s.n)
                                                      : O->s.n;
#pragma omp parallel num_threads(threads)
    {
        Counters cnt;
        std::vector<uint32_t> c1, c2;
        std::vector<char> f1, f2, none;
        std::string corr;
        std::vector<CandRec> recs;
#pragma omp for schedule(dynamic, 8)
        for (int64_t u = 0; u < units; u++) {
            if (!pe) {
                const uint64_t a = first + uint64_t(u);
                if (a >= limit) {
                    flags[a - first] = 0;
                    continue;
                }
                candidates(*O, a, c1, &cnt.raw);
                const uint8_t f = correctOne(*O, a, c1, none, corr, cnt, recs);
                flags[a - first] = f;
                if (f & CG_RESULT_CORRECTED) std::memcpy(out + (a - first) * pitch, corr.data(), corr.size());
            } else {
                const uint64_t a = first + 2 * uint64_t(u);
                if (a >= limit) {
                    flags[a - first] = flags[a + 1 - first] = 0;
                    continue;
                }
                candidates(*O, a, c1, &cnt.raw);
                candidates(*O, a + 1, c2, &cnt.raw);
                pairFlags(c1, c2, f1, f2);
                const uint8_t fa = correctOne(*O, a, c1, f1, corr, cnt, recs);
                flags[a - first] = fa;
                if (fa & CG_RESULT_CORRECTED) std::memcpy(out + (a - first) * pitch, corr.data(), corr.size());
                const uint8_t fb = correctOne(*O, a + 1, c2, f2, corr, cnt, recs);
                flags[a + 1 - first] = fb;
                if (fb & CG_RESULT_CORRECTED) std::memcpy(out + (a + 1 - first) * pitch, corr.data(), corr.size());
            }
        }
#pragma omp critical
        {
            total.raw += cnt.raw; total.uniq += cnt.uniq; total.aligned += cnt.aligned;
            total.msaCands += cnt.msaCands; total.msaBuilds += cnt.msaBuilds;
            total.corrected += cnt.corrected; total.hq += cnt.hq;
            for (auto& r : recs) allRecs.push_back(std::move(r));
        }
    }
    const uint64_t saved = O->o.correct_candidates ? combine(allRecs, flags, out, pitch, O->s) : 0;
    if (counters) {
        counters[0] = total.raw; counters[1] = total.uniq; counters[2] = total.aligned;
        counters[3] = total.msaCands; counters[4] = total.msaBuilds; counters[5] = total.corrected;
        counters[6] = total.hq; counters[7] = saved;
    }
    return 0;
}

}  // extern "C"
