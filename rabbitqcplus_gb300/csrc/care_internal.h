// Internal declarations shared by the CUDA kernel files and the C ABI layer.
//
// Device layout (one context, one GPU):
//   read store      enc   u32 [N][pitch]      2-bit bases, 16 per word, first base in the MSBs
//                   len   u16 [N]
//                   hilo  u32 [N][2][2][wp]   hi/lo bit planes (32 bases per word) of the forward
//                                             and reverse-complement read, wp = ceil(Lmax/32)+1
//                                             (one zero word of padding for shifted reads)
//                   qual  u8  [N][Lmax]       Phred+33 (only with quality scores)
//                   ambig u8  [N]             read had a non-ACGT base
//   signatures      sig   u64 [maps][N]       minhash key of every read for every map
//   hash tables     per map: open-addressing slots {key, offset, count} and the
//                   read ids of every kept key, ascending
//   per batch       candidate lists, alignment results, filtered lists and the
//                   corrected anchors, all addressed by per-anchor offsets
#ifndef CARE_INTERNAL_H
#define CARE_INTERNAL_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "care_gpu.h"

namespace cg {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr int kSegmentReads = 65536;  // N-replacement counter restarts per parser batch
constexpr int kMaxMaps = CG_MAX_HASHMAPS;
constexpr int kMaxBucket = 65535;     // BucketSize is uint16 in the reference
constexpr int kLearnedFeatures = 32;  // features of one MSA column for the learned decision

struct Slot {
    unsigned long long key;
    uint32_t offset;
    uint32_t count;
};
static_assert(sizeof(Slot) == 16, "slot layout");

// All maps' lookup tables, passed by value to the query kernels.
struct TablesArg {
    const Slot* slots[kMaxMaps];
    const uint32_t* values[kMaxMaps];
    uint32_t mask[kMaxMaps];
    int nmaps;
    int maxValuesPerKey;
    // With strand set (fewer than 2^31 reads): the read id is the low 31 bits
    // of every bucket value; in maps 0-15 bit 31 is the value read's strand bit
    // for that map (launch_signatures) and strand[anchor] holds the anchor's
    // bits (zero elsewhere: no prediction).
    const uint16_t* strand;
};

// Read store view.
struct StoreArg {
    const uint32_t* enc;
    const uint16_t* len;
    const uint32_t* hilo;
    const uint8_t* qual;
    const uint8_t* ambig;
    int pitch;      // u32 words per read in enc
    int wp;         // u32 words per plane in hilo
    int lmax;
    uint64_t n;
};

// Float constants of the correction decision, computed once on the host in
// the reference's operand order (ISO C++, no contraction).
struct Params {
    int k;
    int nmaps;
    int minOverlap;
    float maxErrorRate;        // maxErrorRate (alignment)
    float minOverlapRatio;
    float orientMaxErrorRate;  // estimatedErrorrate * 4.0f
    float mmBase;              // estimatedErrorrate * 1.0f
    float mm2, mm3, mm4;       // 2/3/4 * mmBase
    float goodAlignmentsCountThreshold;  // estimatedCoverage * m_coverage
    float pairedThreshold;
    float avgSupportThreshold;  // 1 - 1*err
    float minSupportThreshold;  // 1 - 3*err
    float minCoverageThreshold; // m_coverage / 6 * cov
    int errPercent;             // ceil(err * 100)
    float hqPercentLimit;       // errPercent * 0.5f
    float hqAvg[101];           // 1 - 1*percent/100 for percent 0..100
    float hqMin[101];           // 1 - 3*percent/100
    int significantCount;       // int(int(cov) * 0.3f)
    int useQuality;
    int excludeAmbiguous;
    int paired;
    int correctionType;         // CG_CORR_*
    float estimatedCoverage;
    // forest decision (correctionType == CG_CORR_FOREST)
    const struct ForestNode* forestNodes;
    const uint32_t* treeOffsets;  // first node of each tree
    int numTrees;
    float forestThreshold;
    float qweight[256];
    // Candidate correction (correct_candidates).  Per read: votes = {number of
    // candidate corrections made by anchors with a smaller id, by anchors with a
    // larger id}; candAnd / candOr = bitwise AND / OR of every sequence voted
    // for the read (its candidate corrections and its own low-quality anchor
    // correction), 2 bits per base, 32 bases per word, first base in the most
    // significant bits, zero past the read's end.  All of them are equal
    // exactly when AND == OR over the read's words.
    int candidates;
    int newColumns;               // new_columns_to_correct
    int candPitch;                // words per read = ceil(Lmax / 32)
    uint2* candVotes;             // [N]
    unsigned long long* candAnd;  // [N][candPitch]
    unsigned long long* candOr;   // [N][candPitch]
};

// One forest node (reference: include/forest.hpp:21-30): go left when
// feature[att] <= split; flag bit 1 = lhs is a leaf, bit 0 = rhs is a leaf;
// a leaf side holds the float probability's bits, an inner side the index of
// the child within the tree.
struct ForestNode {
    double split;
    uint32_t lhs, rhs;
    uint8_t att, flag;
    uint8_t pad[6];
};
static_assert(sizeof(ForestNode) == 24, "forest node layout");

// ---------------------------------------------------------------- launches
// Every launcher enqueues on `s` and returns the launch status.

// exclusive scans, in place; `tmp` needs scan_tmp_bytes(n) bytes
size_t scan_tmp_bytes(size_t n);
cudaError_t scan_exclusive_u32(uint32_t* data, size_t n, void* tmp, cudaStream_t s);
cudaError_t scan_exclusive_u64(unsigned long long* data, size_t n, void* tmp, cudaStream_t s);
// kernels one scan of n elements launches
uint64_t scan_launches(uint64_t n);

// read store
// offs[i] -= base for i < count
cudaError_t launch_rebase_offsets(uint64_t* offs, uint64_t count, uint64_t base, cudaStream_t s);
cudaError_t launch_count_invalid(const char* chars, const uint64_t* offs, uint64_t n, uint32_t* invalid,
                                 cudaStream_t s);
cudaError_t launch_encode(const char* chars, const uint64_t* offs, const char* quals, uint64_t n,
                          uint64_t firstId, const uint32_t* invalidScan, const uint64_t* segStart,
                          uint32_t* enc, uint16_t* len, uint8_t* qual, uint8_t* ambig, int pitch, int lmax,
                          cudaStream_t s);
cudaError_t launch_hilo(StoreArg st, uint32_t* hilo, cudaStream_t s);
// sig[maps][N]; with strand set also strand[N], bit q of strand[r] = map
// q's minimum of read r came from a reverse complement canonical k-mer (maps
// 0-15)
cudaError_t launch_signatures(StoreArg st, int k, int nmaps, unsigned long long* sig, uint16_t* strand,
                              cudaStream_t s);
// out[0] = shortest, out[1] = longest read of the store (out preset to {~0, 0})
cudaError_t launch_len_range(const uint16_t* len, uint64_t n, unsigned int* out, cudaStream_t s);
// qualityScoreBits 1 or 2: bins the stored scores of reads [0, n) in place
// (rows of lmax bytes) and fills each row past its read's end with the first bin
cudaError_t launch_quality_bins(uint8_t* qual, const uint16_t* len, uint64_t n, int lmax, int bits, cudaStream_t s);

// hash tables
cudaError_t launch_table_init(Slot* t, uint64_t cap, cudaStream_t s);
// one map's (key, read id) pairs sorted by key (read ids ascending within a
// key) into keys/vals, from the first `bits` bits of keysIn's keys (values
// 0 .. n - 1; with tags, n < 2^31 and bit tagBit of tags[i] rides in bit 31
// of value i); keysAlt/valsAlt hold n pairs of scratch, temp
// radix_sort_temp_bytes(n) bytes
size_t radix_sort_temp_bytes(uint64_t n);
cudaError_t radix_sort_pairs(const unsigned long long* keysIn, uint64_t n, int bits, unsigned long long* keys,
                             uint32_t* vals, unsigned long long* keysAlt, uint32_t* valsAlt, void* temp,
                             cudaStream_t s, const uint16_t* tags = nullptr, int tagBit = 0);
// runs of equal keys in sorted pairs: runOf[0..n] (scanned in place by the
// caller into run indices, runOf[n] = number of runs R), start[0..R],
// packed[0..R] (scanned by the caller into value offsets and totals), then
// the kept runs' ids into values and their keys into the final table (and,
// with rawAll, each kept id's bucket size added to rawAll[id])
cudaError_t launch_run_heads(const unsigned long long* keys, uint64_t n, uint32_t* runOf, cudaStream_t s);
cudaError_t launch_run_starts(const unsigned long long* keys, uint64_t n, const uint32_t* runOf, uint32_t* start,
                              cudaStream_t s);
cudaError_t launch_run_pack(const unsigned long long* keys, const uint32_t* start, uint32_t runs, int maxValues,
                            unsigned long long* packed, cudaStream_t s);
cudaError_t launch_run_fill(const unsigned long long* keys, const uint32_t* ids, uint64_t n, const uint32_t* runOf,
                            const uint32_t* start, uint32_t runs, const unsigned long long* packedScan, int maxValues,
                            uint32_t* values, Slot* fin, uint32_t finMask, cudaStream_t s,
                            uint32_t* rawAll = nullptr, uint32_t idMask = 0xffffffffu);

// correction batch
struct BatchArg {
    uint64_t first;         // first anchor id
    int count;              // anchors in batch
    const unsigned long long* sig;  // [nmaps][N]
    uint2* qrange;          // [count][nmaps] (offset, count) per map
    uint32_t* rawCount;     // [count+2]: raw counts, exclusive-scanned in place into offsets
                            // ([count] = total after the scan); [count+1] = batch maximum
    uint32_t* cand;         // [totalRaw] unique candidate ids
    uint32_t* ncand;        // [count]
    uint8_t* paired;        // [totalRaw] pair flags (PE)
    uint2* aln;             // [totalRaw] packed alignment results
    uint32_t* fid;          // [totalRaw] filtered candidates: id
    int16_t* fshift;        // [totalRaw]
    uint8_t* forient;       // [totalRaw] 1 fwd, 2 rc
    float* fweight;         // [totalRaw]
    uint16_t* flen;         // [totalRaw] candidate length
    uint32_t* nfinal;       // [count]
    // [totalRaw] or null: per anchor, its candidates' positions in the order
    // the alignment takes them (lane j of an anchor gets candidate perm[j]),
    // with each one's predicted orientation in bit 31; with lenOrder the
    // positions are grouped by length, so that a warp's lanes see similar
    // lengths
    uint32_t* perm;
    int lenOrder;
    uint8_t* flags;         // [count] CG_RESULT_*
    char* out;              // [count][outPitch]
    int outPitch;
    unsigned long long* counters;  // device counters, see kCounter*
    // Output rows: anchor first + a goes to row (first - outFirst) + a of out
    // and flags.  The plain form sets outFirst = first.
    unsigned long long outFirst;
    // Batched form (graph replays), null in the plain form:
    //   cursor[0] = the batch's first anchor id, cursor[1] = outFirst, both
    //     read on the device so that one captured graph serves every batch
    //   rangeOff = exclusive scan of the raw id counts of the anchors
    //     outFirst, outFirst+1, ...; the candidate kernel takes the batch's raw
    //     offsets from it instead of a count pass and a scan per batch
    //   work[0], work[1] = the persistent alignment and MSA kernels'
    //     work-stealing counters (zero at the start of a batch)
    // laneWork (plain form, optional): the alignment's own work-stealing
    // counter, zero before its launch
    const unsigned long long* cursor;
    const unsigned long long* rangeOff;
    unsigned int* work;
    unsigned int* laneWork;
    // Learned decision (correctionType CG_CORR_LEARNED): the MSA kernel records
    // every column of a non-HQ anchor whose consensus differs from the anchor's
    // base: 32 BF16 features (colFeat) and {output row, position | consensus
    // base << 16} (colMeta), at index atomicAdd(colCount); indexes past colCap
    // are not stored (those columns keep the fallback decision).
    __nv_bfloat16* colFeat;
    uint2* colMeta;
    unsigned int* colCount;
    unsigned int colCap;
    // MSA order: anchors by decreasing number of kept rows (null: batch order);
    // the heavy MSAs start first, so that none of them is left for the end
    const uint32_t* order;
};
enum {
    kCounterRaw = 0,
    kCounterUnique,
    kCounterAligned,
    kCounterMsaCands,
    kCounterMsaBuilds,
    kCounterCorrected,
    kCounterHQ,
    kCounterTimeouts,
    kCounterColumns,         // learned decision: columns recorded for the classifier
    kCounterColumnOverflow,  // columns beyond the buffer (decided by the fallback rule)
    kCounterLearnedTaken,    // columns the classifier corrected
    kCounterCandidateVotes,  // candidate corrections made by HQ anchors
    kNumCounters
};

cudaError_t launch_query_count(StoreArg st, TablesArg tb, Params p, BatchArg b, cudaStream_t s);
// with b.rangeOff set the kernel looks the buckets up itself and writes the
// batch's raw offsets into b.rawCount (no query_count pass, no scan)
// bigScratch (optional, count + 1 words): anchors with more than 1024 raw ids
// run in a second, large-table pass instead of sizing every block for them
cudaError_t launch_gather_unique(StoreArg st, TablesArg tb, Params p, BatchArg b, int maxRawPerAnchor,
                                 cudaStream_t s, uint32_t* bigScratch = nullptr);
cudaError_t launch_pair_flags(BatchArg b, cudaStream_t s);
// raw id count of every read as an anchor, raw[N]: raw holds every read's
// kept bucket sizes summed by launch_run_fill over all maps; reads that
// cannot be anchors get zero
cudaError_t launch_raw_count(StoreArg st, Params p, uint32_t* raw, cudaStream_t s);
// off[num+1] = exclusive scan of raw[0..num); maxima[0] = the largest raw
// total of a batch of `batch` anchors, maxima[1] = the largest raw count of
// one anchor; tmp needs scan_tmp_bytes(num + 1) bytes
cudaError_t launch_range_offsets(const uint32_t* raw, uint64_t num, uint64_t batch, unsigned long long* off,
                                 void* tmp, unsigned long long* maxima, cudaStream_t s);

// Launch shapes of the batched form's persistent kernels (b.work set).
struct Shape {
    int alignBlocks;  // persistent alignment blocks of 128 threads
    int msaWarps;     // warps (anchors in flight) per MSA block
    int msaBlocks;    // persistent MSA blocks
};

// uoff: exclusive scan of the per-anchor candidate counts (count+1 entries),
// totalUnique = uoff[count] (unused with a shape: the persistent kernel reads
// uoff[count]); with uoff null the warp-per-anchor kernel runs
cudaError_t launch_align_filter(StoreArg st, Params p, BatchArg b, const uint32_t* uoff, uint32_t totalUnique,
                                cudaEvent_t between, cudaStream_t s,  // `between` (optional) after the alignment
                                const Shape* shape = nullptr);
cudaError_t launch_msa_correct(StoreArg st, Params p, BatchArg b, int maxRows, cudaStream_t s,
                               const Shape* shape = nullptr);
// resident 128-thread blocks per SM of the thread-per-candidate alignment
// (0: it does not apply to this store's read length)
int align_lane_occupancy(StoreArg st);
// warp-per-anchor MSA blocks of `warps` warps that fit one SM (0: the warp
// MSA does not apply to this store)
int msa_warp_occupancy(StoreArg st, Params p, int warps);
// order[count] = the batch's anchors by decreasing b.nfinal (log2 buckets);
// scratch = 32 words, cleared by the launcher
cudaError_t launch_msa_order(BatchArg b, unsigned int* scratch, uint32_t* order, cudaStream_t s);
// candidate correction: the batch's low-quality anchor corrections join their
// reads' votes (after the MSA and any classifier pass)
cudaError_t launch_anchor_vote(StoreArg st, Params p, BatchArg b, cudaStream_t s);
// the combine step for reads [first, first + n): flags[i] of read first + i is
// rewritten (CG_RESULT_CANDIDATES / _REJECTED / _CANDIDATE_RECORD), *records
// (zeroed by the caller) gains the number of saved candidate records
cudaError_t launch_combine(StoreArg st, Params p, uint64_t first, uint64_t n, uint8_t* flags,
                           unsigned long long* records, cudaStream_t s);
// cursor[0] += stride, work[0] = work[1] = 0 (the last node of a batch)
cudaError_t launch_batch_advance(unsigned long long* cursor, unsigned int* work, unsigned long long stride,
                                 cudaStream_t s);

}  // namespace cg

#endif
