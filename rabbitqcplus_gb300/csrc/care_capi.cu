// C ABI of the CARE correction engine (include/care_gpu.h): context, device
// memory, and the order of the kernels.
//
// reference: care::performCorrection's STEP1 and STEP2
// (src/dispatch_care_correct_cpu.cpp:52-170) -- read store and minhasher
// construction, then cpu::correct_cpu (src/correct_cpu.cpp:47-348) -- with the
// per-anchor pipeline of CpuErrorCorrector (include/corrector.hpp:145-513)
// split into batched device stages.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <new>
#include <string>
#include <vector>

#include "care_capi_internal.h"
#include "care_gpu.h"
#include "care_internal.h"
#include "care_learned.h"

using namespace cg;

namespace {

// Device blocks released by the contexts of this process, kept for reuse
// (like a caching allocator): a later context of the same shapes allocates
// without cudaMalloc and frees without cudaFree.  A block is cached only after
// the device has finished every queued kernel (the release synchronises, as
// cudaFree would), and the cache is emptied before an allocation fails.
// Simulated device out-of-memory (cg_set_allocation_fault): requests left
// before every request fails; < 0 = off.
std::atomic<long long> g_allocFault{-1};

bool simulated_out_of_memory() {
    long long v = g_allocFault.load();
    while (v >= 0) {
        if (v == 0) return true;
        if (g_allocFault.compare_exchange_weak(v, v - 1)) return false;
    }
    return false;
}

class BlockCache {
public:
    cudaError_t alloc(void** p, size_t n, size_t* got) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (simulated_out_of_memory()) {
            // as a real failure: the cache is emptied before the request fails
            trim(dev);
            return cudaErrorMemoryAllocation;
        }
        {
            std::lock_guard<std::mutex> lock(mu_);
            // the smallest cached block of this device that holds n bytes, if
            // it is at most twice as large and still a live allocation (a
            // cudaDeviceReset of the program's would have released it)
            for (auto it = free_.lower_bound(n); it != free_.end() && it->first <= 2 * n + 4096;) {
                if (it->second.first != dev) {
                    ++it;
                    continue;
                }
                cudaPointerAttributes attr{};
                const bool live = cudaPointerGetAttributes(&attr, it->second.second) == cudaSuccess &&
                                  attr.type == cudaMemoryTypeDevice && attr.device == dev;
                if (!live) {
                    cudaGetLastError();
                    it = free_.erase(it);
                    continue;
                }
                *p = it->second.second;
                *got = it->first;
                free_.erase(it);
                return cudaSuccess;
            }
        }
        cudaError_t e = cudaMalloc(p, n);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            trim(dev);
            e = cudaMalloc(p, n);
        }
        if (e == cudaSuccess) *got = n;
        return e;
    }
    void release(void* p, size_t bytes) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceSynchronize();
        std::lock_guard<std::mutex> lock(mu_);
        free_.emplace(bytes, std::make_pair(dev, p));
    }
    // frees the cached blocks of device dev (every device if dev < 0)
    void trim(int dev) {
        std::lock_guard<std::mutex> lock(mu_);
        int cur = 0;
        cudaGetDevice(&cur);
        for (auto it = free_.begin(); it != free_.end();) {
            if (dev < 0 || it->second.first == dev) {
                cudaSetDevice(it->second.first);
                cudaFree(it->second.second);
                it = free_.erase(it);
            } else {
                ++it;
            }
        }
        cudaSetDevice(cur);
    }

private:
    std::mutex mu_;
    std::multimap<size_t, std::pair<int, void*>> free_;
};

BlockCache& block_cache() {
    static BlockCache* c = new BlockCache();  // never destroyed: the driver may be gone at exit
    return *c;
}

// grow-only device buffer; blocks come from and go back to the block cache,
// except adopted ones (cached = false), which are freed
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    bool cached = true;
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        size_t want = std::max(n, bytes + bytes / 2), got = 0;
        release();
        cudaError_t e = block_cache().alloc(&p, want, &got);
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = block_cache().alloc(&p, n, &got);
            if (e != cudaSuccess) {
                p = nullptr;
                return e;
            }
        }
        bytes = got;
        return cudaSuccess;
    }
    void release() {
        if (p) {
            if (cached) block_cache().release(p, bytes);
            else cudaFree(p);
        }
        p = nullptr;
        bytes = 0;
        cached = true;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct MapTable {
    Slot* slots = nullptr;
    uint32_t* values = nullptr;
    uint64_t cap = 0;
    uint64_t keys = 0;
    uint64_t nvalues = 0;
};

// What a captured batch graph depends on; a change means a new capture.
struct GraphSig {
    int count = 0;
    unsigned long long stride = 0;
    Shape shape{};
    int tableRaw = 0, maxRows = 0;
    std::vector<const void*> ptrs;
    bool operator==(const GraphSig& o) const {
        return count == o.count && stride == o.stride && shape.alignBlocks == o.shape.alignBlocks &&
               shape.msaWarps == o.shape.msaWarps && shape.msaBlocks == o.shape.msaBlocks &&
               tableRaw == o.tableRaw && maxRows == o.maxRows && ptrs == o.ptrs;
    }
};

// One batch pipeline of the batched driver: its buffers, stream and graph.
struct BatchSet {
    DevBuf rawCount, cand, ncand, paired, aln, fid, fshift, forient, fweight, flen, nfinal, uoff, scanTmp, cursor,
        work, colFeat, colMeta, colCount, order, orderScratch, bigScratch, perm;
    cudaStream_t stream = nullptr;
    cudaEvent_t joined = nullptr;
    cudaGraphExec_t exec = nullptr;
    GraphSig sig;
    int kernels = 0;  // kernel nodes of one replay
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (joined) cudaEventDestroy(joined);
        joined = nullptr;
        for (DevBuf* b : {&rawCount, &cand, &ncand, &paired, &aln, &fid, &fshift, &forient, &fweight, &flen, &nfinal,
                          &uoff, &scanTmp, &cursor, &work, &colFeat, &colMeta, &colCount, &order, &orderScratch,
                          &bigScratch, &perm})
            b->release();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

// Batch size and launch shapes of the batched driver.
struct Plan {
    int batch = 0;
    Shape shape{};
    int streams = 0;
};

constexpr int kMaxSets = 2;

// Drops the cached device address of the no-allocation lookup's scratch array
// for `device` (every device if < 0); defined with that entry point below.
void forget_noalloc_scratch(int device);

}  // namespace

struct cg_ctx {
    cg_options o{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t st0 = nullptr, st1 = nullptr, st1b = nullptr, st2 = nullptr, st3 = nullptr;  // stage boundaries
    std::string err;

    // appended reads, one device chunk per cg_append_reads call (uploaded by
    // the call itself; encoded and released by cg_build_tables)
    struct Chunk {
        DevBuf chars, offs, qual;  // bases, offsets rebased to 0 (u64 [m+1]), qualities
        uint64_t first = 0, reads = 0;
    };
    std::vector<Chunk> chunks;
    uint64_t appended = 0;
    int appendLmax = 0;
    bool haveQual = true;

    // device read store
    bool built = false;
    uint64_t n = 0;
    int lmax = 0, pitch = 0, wp = 0, k = 20, nmaps = 48, maxValuesPerKey = 75;
    DevBuf enc, len, hilo, qual, ambig, sig;
    // strand bits of every read's minima in maps 0-15 (u16 [N]) and the read
    // ids in those maps' buckets tagged with them: fewer than 2^31 reads
    DevBuf strand;
    bool strandTags = false;
    std::vector<MapTable> maps;    // views into tableSlabs
    std::vector<DevBuf> tableSlabs;
    TablesArg tables{};
    Params params{};
    // where cg_correct's results go: host memory, or device memory for the
    // device file path (cg::correct_into_device)
    cudaMemcpyKind outKind = cudaMemcpyDeviceToHost;
    uint64_t paramsVersion = 0;

    // batch buffers
    DevBuf qrange, rawCount, cand, ncand, paired, aln, fid, fshift, forient, fweight, flen, nfinal, flags, out, counters;
    DevBuf scanTmp, uoff, msaOrder, orderScratch, bigScratch, perm, lenRange, laneWork;
    uint32_t* hPinned = nullptr;  // 2 words: total raw, max raw
    bool lenVaries = false;       // reads of different lengths: candidates aligned in length order

    // batched driver
    BatchSet sets[kMaxSets];
    DevBuf rawAll, rangeOff, rangeTmp, maxima, outRange, flagsRange, counterSave;
    unsigned long long* hBatched = nullptr;  // pinned: [0..1] maxima, then two cursor words per set
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evPro = nullptr, evStart = nullptr;
    std::vector<cudaEvent_t> batchDone;
    bool haveRawAll = false;

    // learned classifier (CG_CORR_LEARNED): model and the plain driver's column records
    DevBuf mlp, colFeat, colMeta, colCount;
    bool haveMlp = false;
    bool collecting = false;  // cg_get_columns: record the columns, do not score them
    float minLogit = 0.0f;    // logit of threshold_anchor
    unsigned long long timeoutsSeen = 0;  // classifier blocks whose MMA wait ran out, already reported

    // forest classifier (CG_CORR_FOREST)
    DevBuf forestNodes, treeOffsets;
    int numTrees = 0;

    // candidate correction (correct_candidates): per-read votes (Params) and
    // the anchors the current pass has corrected, one bit per read
    DevBuf candVotes, candAnd, candOr, combineFlags, combineCount;
    std::vector<uint64_t> candPass;

    cg_stats stats{};
};

namespace {

int fail(cg_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CG_CUDA(ctx, call)                                                                              \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA,    \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);    \
        }                                                                                               \
    } while (0)

uint64_t pow2_at_least(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Float constants in the reference's operand order (host, no contraction).
void make_params(cg_ctx* c) {
    c->paramsVersion++;  // captured batch graphs hold the parameters by value
    Params& p = c->params;
    const cg_options& o = c->o;
    p.k = c->k;
    p.nmaps = c->nmaps;
    p.minOverlap = o.min_overlap;
    p.maxErrorRate = o.max_error_rate;
    p.minOverlapRatio = o.min_overlap_ratio;
    p.orientMaxErrorRate = o.estimated_errorrate * 4.0f;              // alignmentorientation.hpp:90
    p.mmBase = o.estimated_errorrate * 1.0f;                          // corrector.hpp:1063
    p.mm2 = 2 * p.mmBase;
    p.mm3 = 3 * p.mmBase;
    p.mm4 = 4 * p.mmBase;
    p.goodAlignmentsCountThreshold = o.estimated_coverage * o.m_coverage;  // corrector.hpp:1064
    p.pairedThreshold = o.paired_filter_threshold;
    p.avgSupportThreshold = 1.0f - 1.0f * o.estimated_errorrate;     // msa.cpp:314-316
    p.minSupportThreshold = 1.0f - 3.0f * o.estimated_errorrate;
    p.minCoverageThreshold = o.m_coverage / 6.0f * o.estimated_coverage;
    p.errPercent = (int)std::ceil(o.estimated_errorrate * 100.0f);  // msa.cpp:361
    p.hqPercentLimit = p.errPercent * 0.5f;
    for (int pc = 0; pc <= 100; pc++) {
        const float factor = pc / 100.0f;
        p.hqAvg[pc] = 1.0f - 1.0f * factor;
        p.hqMin[pc] = 1.0f - 3.0f * factor;
    }
    p.significantCount = int(int(o.estimated_coverage) * 0.3f);     // msa.cpp:536-540
    p.useQuality = o.use_quality_scores != 0;
    p.excludeAmbiguous = o.exclude_ambiguous_reads != 0;
    p.paired = o.pair_mode == CG_PAIR_PE;
    p.correctionType = o.correction_type;
    p.estimatedCoverage = o.estimated_coverage;
    p.forestNodes = c->forestNodes.as<ForestNode>();
    p.treeOffsets = c->treeOffsets.as<uint32_t>();
    p.numTrees = c->numTrees;
    p.forestThreshold = o.threshold_anchor;
    p.candidates = o.correct_candidates != 0;
    p.newColumns = o.new_columns_to_correct;
    p.candPitch = (c->lmax + 31) / 32;
    p.candVotes = c->candVotes.as<uint2>();
    p.candAnd = c->candAnd.as<unsigned long long>();
    p.candOr = c->candOr.as<unsigned long long>();
    // include/qualityscoreweights.hpp:17-33
    for (int i = 0; i < 256; i++) {
        const float e = i < 33 ? 1.0f : std::pow(10.0f, -(i - 33) / 10.0f);
        p.qweight[i] = std::max(0.001f, 1.0f - e);
    }
}

// A new candidate-correction pass: no votes, no anchors corrected.
int reset_candidates(cg_ctx* c) {
    const size_t words = c->n * (size_t)((c->lmax + 31) / 32);
    CG_CUDA(c, cudaMemsetAsync(c->candVotes.p, 0, c->n * sizeof(uint2), c->stream));
    CG_CUDA(c, cudaMemsetAsync(c->candAnd.p, 0xff, words * sizeof(unsigned long long), c->stream));
    CG_CUDA(c, cudaMemsetAsync(c->candOr.p, 0, words * sizeof(unsigned long long), c->stream));
    c->candPass.assign((c->n + 63) / 64, 0ull);
    return CG_OK;
}

// Marks anchors [first, first + num) as corrected by the current pass; one
// that the pass already corrected starts a new pass first.
int mark_pass(cg_ctx* c, uint64_t first, uint64_t num) {
    auto bits = [&](bool set) {
        bool any = false;
        for (uint64_t i = first; i < first + num;) {
            const uint64_t w = i >> 6, b0 = i & 63;
            const uint64_t cnt = std::min<uint64_t>(64 - b0, first + num - i);
            const uint64_t m = (cnt == 64 ? ~0ull : ((1ull << cnt) - 1)) << b0;
            any |= (c->candPass[w] & m) != 0;
            if (set) c->candPass[w] |= m;
            i += cnt;
        }
        return any;
    };
    if (bits(false)) {
        const int rc = reset_candidates(c);
        if (rc != CG_OK) return rc;
    }
    bits(true);
    return CG_OK;
}

StoreArg store_arg(const cg_ctx* c) {
    StoreArg s;
    s.enc = c->enc.as<uint32_t>();
    s.len = c->len.as<uint16_t>();
    s.hilo = c->hilo.as<uint32_t>();
    s.qual = c->qual.as<uint8_t>();
    s.ambig = c->ambig.as<uint8_t>();
    s.pitch = c->pitch;
    s.wp = c->wp;
    s.lmax = c->lmax;
    s.n = c->n;
    return s;
}

void release_tables(cg_ctx* c) {
    c->maps.clear();
    for (DevBuf& d : c->tableSlabs) d.release();
    c->tableSlabs.clear();
}

int build_store(cg_ctx* c) {
    const uint64_t n = c->appended;
    c->n = n;
    const int lmax = c->appendLmax;
    c->lmax = std::max(lmax, 1);
    c->pitch = (c->lmax + 15) / 16;
    c->wp = (c->lmax + 31) / 32 + 1;
    c->k = c->o.kmerlength == 0 ? (lmax < 160 ? 20 : 32) : c->o.kmerlength;  // dispatch_care_correct_cpu.cpp:81-95
    c->nmaps = c->o.num_hash_functions;
    {
        // include/minhasherlimit.hpp:9-15 (the coverage argument is an int)
        const int cov = int(c->o.estimated_coverage);
        int r = int(cov * 2.5f);
        r = std::min(r, 65535);
        r = std::max(10, r);
        c->maxValuesPerKey = r;
    }
    const bool q = c->o.use_quality_scores != 0;
    CG_CUDA(c, c->enc.ensure(n * c->pitch * sizeof(uint32_t)));
    CG_CUDA(c, c->len.ensure(n * sizeof(uint16_t)));
    CG_CUDA(c, c->ambig.ensure(n));
    CG_CUDA(c, c->hilo.ensure(n * 4 * (uint64_t)c->wp * sizeof(uint32_t)));
    if (q) CG_CUDA(c, c->qual.ensure(n * (uint64_t)c->lmax));
    CG_CUDA(c, cudaMemsetAsync(c->enc.p, 0, n * c->pitch * sizeof(uint32_t), c->stream));
    if (q) CG_CUDA(c, cudaMemsetAsync(c->qual.p, 0, n * (uint64_t)c->lmax, c->stream));
    // encode per append call (the N counter restarts per call)
    DevBuf dInv, tmp;
    for (cg_ctx::Chunk& ch : c->chunks) {
        const uint64_t m = ch.reads;
        CG_CUDA(c, dInv.ensure((m + 1) * sizeof(uint32_t)));
        CG_CUDA(c, tmp.ensure(scan_tmp_bytes(m + 1)));
        CG_CUDA(c, launch_count_invalid(ch.chars.as<char>(), ch.offs.as<uint64_t>(), m, dInv.as<uint32_t>(),
                                        c->stream));
        CG_CUDA(c, scan_exclusive_u32(dInv.as<uint32_t>(), m, tmp.p, c->stream));
        CG_CUDA(c, launch_encode(ch.chars.as<char>(), ch.offs.as<uint64_t>(), q ? ch.qual.as<char>() : nullptr, m,
                                 ch.first, dInv.as<uint32_t>(), nullptr, c->enc.as<uint32_t>(), c->len.as<uint16_t>(),
                                 c->qual.as<uint8_t>(), c->ambig.as<uint8_t>(), c->pitch, c->lmax, c->stream));
        // the chunks and staging buffers are freed below only after the stream drained
    }
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    dInv.release();
    tmp.release();
    for (cg_ctx::Chunk& ch : c->chunks) {
        ch.chars.release();
        ch.offs.release();
        ch.qual.release();
    }
    c->chunks.clear();
    StoreArg st = store_arg(c);
    const int qbits = c->o.quality_score_bits == 0 ? 8 : c->o.quality_score_bits;
    if (q && qbits != 8) {
        CG_CUDA(c, launch_quality_bins(c->qual.as<uint8_t>(), c->len.as<uint16_t>(), n, c->lmax, qbits, c->stream));
        c->stats.kernel_launches += 1;
    }
    CG_CUDA(c, launch_hilo(st, c->hilo.as<uint32_t>(), c->stream));
    // shortest and longest read (read back once the build has finished)
    CG_CUDA(c, c->lenRange.ensure(2 * sizeof(unsigned int)));
    CG_CUDA(c, cudaMemsetAsync(c->lenRange.p, 0xff, sizeof(unsigned int), c->stream));
    CG_CUDA(c, cudaMemsetAsync(c->lenRange.as<unsigned int>() + 1, 0, sizeof(unsigned int), c->stream));
    CG_CUDA(c, launch_len_range(st.len, st.n, c->lenRange.as<unsigned int>(), c->stream));
    return CG_OK;
}

int build_tables(cg_ctx* c) {
    const uint64_t n = c->n;
    CG_CUDA(c, c->sig.ensure(n * c->nmaps * sizeof(unsigned long long)));
    StoreArg st = store_arg(c);
    c->strandTags = n <= 0x7fffffffull;
    uint16_t* strand = nullptr;
    if (c->strandTags) {
        CG_CUDA(c, c->strand.ensure((size_t)n * sizeof(uint16_t)));
        strand = c->strand.as<uint16_t>();
    }
    CG_CUDA(c, launch_signatures(st, c->k, c->nmaps, c->sig.as<unsigned long long>(), strand, c->stream));
    if (n > 0x40000000ull) return fail(c, CG_ERR_UNSUPPORTED, "too many reads for one table (%llu)",
                                       (unsigned long long)n);
    // The maps are built in waves of up to kTableStreams maps, one stream and
    // one set of sorting buffers per map of a wave (as many as a quarter of the
    // free memory holds).  A wave sorts its maps' (key, read id) pairs and
    // marks their runs of equal keys; one synchronisation reads the run
    // counts, a second the kept keys' and values' totals, which size one slab
    // for the wave's slots and values; then the wave fills its maps.  The
    // next wave's sorts follow on the same streams.
    constexpr int kTableStreams = 8;
    const int bits = std::min(64, 2 * c->k);  // the signatures keep 2k bits
    const size_t perStream = n * (2 * sizeof(unsigned long long) + 2 * sizeof(uint32_t)) +
                             2 * (n + 1) * sizeof(uint32_t) + (n + 1) * sizeof(unsigned long long) +
                             radix_sort_temp_bytes(n) + scan_tmp_bytes(n + 1);
    size_t freeB = 0, totalB = 0;
    CG_CUDA(c, cudaMemGetInfo(&freeB, &totalB));
    const int S = (int)std::max<size_t>(1, std::min<size_t>({(size_t)kTableStreams, (size_t)c->nmaps,
                                                            freeB / 4 / std::max<size_t>(perStream, 1)}));
    struct Lane {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        DevBuf keys, ids, keysAlt, idsAlt, runOf, start, packed, sortTmp, scanTmp;
    };
    std::vector<Lane> lanes(S);
    unsigned long long* hTot = nullptr;  // per map: (kept keys << 32) | values, then the runs (u32)
    release_tables(c);
    c->maps.resize(c->nmaps);
    c->stats.table_keys = 0;
    c->stats.table_values = 0;
    cudaEvent_t sigDone = nullptr;
    int rc = CG_OK;
    auto cuda = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == CG_OK)
            rc = fail(c, e == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA, "tables (%s): %s",
                      what, cudaGetErrorString(e));
        return rc == CG_OK;
    };
    // the batched driver's raw id count of every read, summed as the maps are
    // filled (finished by ensure_batched_state); cleared before the lanes start
    uint32_t* rawAll = nullptr;
    c->haveRawAll = false;
    if (c->o.driver == CG_DRIVER_BATCHED &&
        cuda(c->rawAll.ensure(std::max<uint64_t>(n, 1) * sizeof(uint32_t)), "raw counts") &&
        cuda(cudaMemsetAsync(c->rawAll.p, 0, n * sizeof(uint32_t), c->stream), "raw counts"))
        rawAll = c->rawAll.as<uint32_t>();
    if (rc == CG_OK &&
        cuda(cudaMallocHost(&hTot, 2 * (size_t)c->nmaps * sizeof(unsigned long long)), "host totals") &&
        cuda(cudaEventCreateWithFlags(&sigDone, cudaEventDisableTiming), "event") &&
        cuda(cudaEventRecord(sigDone, c->stream), "event")) {
        for (Lane& l : lanes) {
            if (!cuda(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking), "stream") ||
                !cuda(cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming), "event") ||
                !cuda(cudaStreamWaitEvent(l.stream, sigDone, 0), "wait") ||
                !cuda(l.keys.ensure(std::max<uint64_t>(n, 1) * sizeof(unsigned long long)), "sorted keys") ||
                !cuda(l.ids.ensure(std::max<uint64_t>(n, 1) * sizeof(uint32_t)), "sorted ids") ||
                !cuda(l.keysAlt.ensure(std::max<uint64_t>(n, 1) * sizeof(unsigned long long)), "sort keys") ||
                !cuda(l.idsAlt.ensure(std::max<uint64_t>(n, 1) * sizeof(uint32_t)), "sort ids") ||
                !cuda(l.runOf.ensure((n + 1) * sizeof(uint32_t)), "runs") ||
                !cuda(l.start.ensure((n + 1) * sizeof(uint32_t)), "run starts") ||
                !cuda(l.packed.ensure((n + 1) * sizeof(unsigned long long)), "run lengths") ||
                !cuda(l.sortTmp.ensure(radix_sort_temp_bytes(n)), "sort") ||
                !cuda(l.scanTmp.ensure(scan_tmp_bytes(n + 1)), "scan"))
                break;
        }
    }
    uint32_t* hRuns = reinterpret_cast<uint32_t*>(hTot + c->nmaps);
    for (int w0 = 0; w0 < c->nmaps && rc == CG_OK; w0 += S) {
        const int w1 = std::min(c->nmaps, w0 + S);
        for (int h = w0; h < w1 && rc == CG_OK; h++) {
            Lane& l = lanes[h - w0];
            const unsigned long long* keys = c->sig.as<unsigned long long>() + (uint64_t)h * n;
            cudaError_t e = radix_sort_pairs(keys, n, bits, l.keys.as<unsigned long long>(), l.ids.as<uint32_t>(),
                                             l.keysAlt.as<unsigned long long>(), l.idsAlt.as<uint32_t>(),
                                             l.sortTmp.p, l.stream, h < 16 ? strand : nullptr, h);
            if (e == cudaSuccess) e = launch_run_heads(l.keys.as<unsigned long long>(), n, l.runOf.as<uint32_t>(),
                                                       l.stream);
            if (e == cudaSuccess) e = scan_exclusive_u32(l.runOf.as<uint32_t>(), n + 1, l.scanTmp.p, l.stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(hRuns + h, l.runOf.as<uint32_t>() + n, sizeof(uint32_t),
                                                      cudaMemcpyDeviceToHost, l.stream);
            cuda(e, "sort");
        }
        for (int h = w0; h < w1 && rc == CG_OK; h++) cuda(cudaStreamSynchronize(lanes[h - w0].stream), "sort");
        for (int h = w0; h < w1 && rc == CG_OK; h++) {
            Lane& l = lanes[h - w0];
            const uint32_t runs = hRuns[h];
            cudaError_t e = launch_run_starts(l.keys.as<unsigned long long>(), n, l.runOf.as<uint32_t>(),
                                              l.start.as<uint32_t>(), l.stream);
            if (e == cudaSuccess) e = launch_run_pack(l.keys.as<unsigned long long>(), l.start.as<uint32_t>(), runs,
                                                      c->maxValuesPerKey, l.packed.as<unsigned long long>(), l.stream);
            if (e == cudaSuccess) e = scan_exclusive_u64(l.packed.as<unsigned long long>(), (size_t)runs + 1,
                                                         l.scanTmp.p, l.stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(hTot + h, l.packed.as<unsigned long long>() + runs,
                                                      sizeof(unsigned long long), cudaMemcpyDeviceToHost, l.stream);
            cuda(e, "runs");
        }
        for (int h = w0; h < w1 && rc == CG_OK; h++) cuda(cudaStreamSynchronize(lanes[h - w0].stream), "runs");
        if (rc != CG_OK) break;
        uint64_t slotTotal = 0, valueTotal = 0;
        std::vector<uint64_t> valueOff(w1 - w0);
        for (int h = w0; h < w1; h++) {
            MapTable& mt = c->maps[h];
            mt.keys = hTot[h] >> 32;
            mt.nvalues = hTot[h] & 0xffffffffull;
            mt.cap = pow2_at_least(std::max<uint64_t>(2 * mt.keys, 64));
            slotTotal += mt.cap;
        }
        for (int h = w0; h < w1; h++) {
            valueOff[h - w0] = valueTotal;
            valueTotal += (std::max<uint64_t>(c->maps[h].nvalues, 1) + 3) / 4 * 4;  // 16-byte aligned per map
        }
        c->tableSlabs.emplace_back();
        DevBuf& slab = c->tableSlabs.back();
        if (!cuda(slab.ensure(slotTotal * sizeof(Slot) + valueTotal * sizeof(uint32_t)), "slab")) break;
        Slot* slotBase = slab.as<Slot>();
        uint32_t* valueBase = reinterpret_cast<uint32_t*>(slotBase + slotTotal);
        for (int h = w0; h < w1 && rc == CG_OK; h++) {
            Lane& l = lanes[h - w0];
            MapTable& mt = c->maps[h];
            mt.slots = slotBase;
            slotBase += mt.cap;
            mt.values = valueBase + valueOff[h - w0];
            cudaError_t e = launch_table_init(mt.slots, mt.cap, l.stream);
            if (e == cudaSuccess) e = launch_run_fill(l.keys.as<unsigned long long>(), l.ids.as<uint32_t>(), n,
                                                      l.runOf.as<uint32_t>(), l.start.as<uint32_t>(),
                                                      hRuns[h], l.packed.as<unsigned long long>(),
                                                      c->maxValuesPerKey, mt.values, mt.slots,
                                                      (uint32_t)(mt.cap - 1), l.stream, rawAll,
                                                      strand ? 0x7fffffffu : 0xffffffffu);
            if (!cuda(e, "build")) break;
            c->stats.table_keys += mt.keys;
            c->stats.table_values += mt.nvalues;
            c->tables.slots[h] = mt.slots;
            c->tables.values[h] = mt.values;
            c->tables.mask[h] = (uint32_t)(mt.cap - 1);
        }
    }
    // the context's stream continues after every wave's last work
    for (Lane& l : lanes) {
        if (l.stream && l.done && cudaEventRecord(l.done, l.stream) == cudaSuccess)
            cuda(cudaStreamWaitEvent(c->stream, l.done, 0), "join");
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    for (Lane& l : lanes) {
        if (l.stream) cudaStreamSynchronize(l.stream);
        for (DevBuf* d : {&l.keys, &l.ids, &l.keysAlt, &l.idsAlt, &l.runOf, &l.start, &l.packed, &l.sortTmp,
                          &l.scanTmp})
            d->release();
        if (l.done) cudaEventDestroy(l.done);
        if (l.stream) cudaStreamDestroy(l.stream);
    }
    if (sigDone) cudaEventDestroy(sigDone);
    if (hTot) cudaFreeHost(hTot);
    if (rc != CG_OK) return rc;
    CG_CUDA(c, e);
    c->tables.nmaps = c->nmaps;
    c->tables.maxValuesPerKey = c->maxValuesPerKey;
    c->tables.strand = strand;
    return CG_OK;
}

BatchArg batch_arg(cg_ctx* c, uint64_t first, int count) {
    BatchArg b{};
    b.first = first;
    b.outFirst = first;
    b.count = count;
    b.sig = c->sig.as<unsigned long long>();
    b.qrange = c->qrange.as<uint2>();
    b.rawCount = c->rawCount.as<uint32_t>();
    b.cand = c->cand.as<uint32_t>();
    b.ncand = c->ncand.as<uint32_t>();
    b.paired = c->paired.as<uint8_t>();
    b.aln = c->aln.as<uint2>();
    b.fid = c->fid.as<uint32_t>();
    b.fshift = c->fshift.as<int16_t>();
    b.forient = c->forient.as<uint8_t>();
    b.fweight = c->fweight.as<float>();
    b.flen = c->flen.as<uint16_t>();
    b.nfinal = c->nfinal.as<uint32_t>();
    b.perm = c->lenVaries || c->strandTags ? c->perm.as<uint32_t>() : nullptr;
    b.lenOrder = c->lenVaries;
    b.flags = c->flags.as<uint8_t>();
    b.out = c->out.as<char>();
    b.outPitch = c->lmax;
    b.counters = c->counters.as<unsigned long long>();
    return b;
}

// Learned decision: column records per anchor of a batch (columns past this
// keep the fallback decision and are counted as overflow)
constexpr uint64_t kColumnsPerAnchor = 32;

int ensure_columns(cg_ctx* c, DevBuf& feat, DevBuf& meta, DevBuf& cnt, int count) {
    const size_t cap = (size_t)count * kColumnsPerAnchor;
    CG_CUDA(c, feat.ensure(cap * kLearnedFeatures * sizeof(__nv_bfloat16)));
    CG_CUDA(c, meta.ensure(cap * sizeof(uint2)));
    CG_CUDA(c, cnt.ensure(sizeof(unsigned int)));
    return CG_OK;
}

void set_columns(BatchArg& b, const DevBuf& feat, const DevBuf& meta, const DevBuf& cnt, int count) {
    b.colFeat = feat.as<__nv_bfloat16>();
    b.colMeta = meta.as<uint2>();
    b.colCount = cnt.as<unsigned int>();
    b.colCap = (unsigned int)((uint64_t)count * kColumnsPerAnchor);
}

// classifier blocks: two per SM (each holds 128 of an SM's 512 tensor-memory columns)
int infer_blocks(cg_ctx* c) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) sms = 1;
    return std::max(sms, 1) * 2;
}

// Candidate ids of a batch (query, scan, gather/unique).  On return
// c->hPinned[0] holds the batch's raw id total.
int run_candidates(cg_ctx* c, uint64_t first, int count) {
    const StoreArg st = store_arg(c);
    CG_CUDA(c, cudaEventRecord(c->st0, c->stream));
    CG_CUDA(c, c->qrange.ensure((size_t)count * c->nmaps * sizeof(uint2)));
    CG_CUDA(c, c->rawCount.ensure((size_t)(count + 2) * sizeof(uint32_t)));
    CG_CUDA(c, c->ncand.ensure((size_t)count * sizeof(uint32_t)));
    CG_CUDA(c, c->scanTmp.ensure(scan_tmp_bytes(count + 1)));
    CG_CUDA(c, cudaMemsetAsync(c->rawCount.p, 0, (size_t)(count + 2) * sizeof(uint32_t), c->stream));
    BatchArg b = batch_arg(c, first, count);
    CG_CUDA(c, launch_query_count(st, c->tables, c->params, b, c->stream));
    CG_CUDA(c, scan_exclusive_u32(b.rawCount, (size_t)count + 1, c->scanTmp.p, c->stream));
    c->stats.kernel_launches += 1 + scan_launches(count + 1);
    CG_CUDA(c, cudaMemcpyAsync(c->hPinned, b.rawCount + count, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    const uint64_t total = c->hPinned[0];
    const uint32_t maxRaw = c->hPinned[1];
    const size_t cap = std::max<uint64_t>(total, 1);
    CG_CUDA(c, c->cand.ensure(cap * sizeof(uint32_t)));
    if (c->lenVaries || c->strandTags) CG_CUDA(c, c->perm.ensure(cap * sizeof(uint32_t)));
    CG_CUDA(c, c->paired.ensure(cap));
    CG_CUDA(c, c->aln.ensure(cap * sizeof(uint2)));
    CG_CUDA(c, c->fid.ensure(cap * sizeof(uint32_t)));
    CG_CUDA(c, c->fshift.ensure(cap * sizeof(int16_t)));
    CG_CUDA(c, c->forient.ensure(cap));
    CG_CUDA(c, c->fweight.ensure(cap * sizeof(float)));
    CG_CUDA(c, c->flen.ensure(cap * sizeof(uint16_t)));
    b = batch_arg(c, first, count);
    CG_CUDA(c, c->bigScratch.ensure((size_t)(count + 1) * sizeof(uint32_t)));
    CG_CUDA(c, launch_gather_unique(st, c->tables, c->params, b, (int)std::max<uint32_t>(maxRaw, 1), c->stream,
                                    c->bigScratch.as<uint32_t>()));
    if (maxRaw > 1024) c->stats.kernel_launches += 1;
    c->stats.kernel_launches += 1;
    return CG_OK;
}

int run_batch(cg_ctx* c, uint64_t first, int count, uint8_t* hFlags, char* hOut, size_t outPitch) {
    int rc = run_candidates(c, first, count);
    if (rc != CG_OK) return rc;
    const StoreArg st = store_arg(c);
    CG_CUDA(c, c->nfinal.ensure((size_t)count * sizeof(uint32_t)));
    CG_CUDA(c, c->flags.ensure((size_t)count));
    CG_CUDA(c, c->out.ensure((size_t)count * c->lmax));
    const bool learned = c->params.correctionType == CG_CORR_LEARNED;
    if (learned) {
        rc = ensure_columns(c, c->colFeat, c->colMeta, c->colCount, count);
        if (rc != CG_OK) return rc;
    }
    BatchArg b = batch_arg(c, first, count);
    if (learned) {
        set_columns(b, c->colFeat, c->colMeta, c->colCount, count);
        CG_CUDA(c, cudaMemsetAsync(b.colCount, 0, sizeof(unsigned int), c->stream));
    }
    if (c->params.paired) {
        CG_CUDA(c, launch_pair_flags(b, c->stream));
        c->stats.kernel_launches += 1;
    }
    // dense candidate numbering for the thread-per-candidate alignment
    CG_CUDA(c, c->uoff.ensure((size_t)(count + 1) * sizeof(uint32_t)));
    CG_CUDA(c, cudaMemsetAsync(c->uoff.as<uint32_t>() + count, 0, sizeof(uint32_t), c->stream));
    CG_CUDA(c, cudaMemcpyAsync(c->uoff.p, b.ncand, (size_t)count * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                               c->stream));
    CG_CUDA(c, scan_exclusive_u32(c->uoff.as<uint32_t>(), (size_t)count + 1, c->scanTmp.p, c->stream));
    CG_CUDA(c, cudaMemcpyAsync(c->hPinned + 2, c->uoff.as<uint32_t>() + count, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->stats.kernel_launches += scan_launches(count + 1) + 1;
    // the alignment's warps take their candidates from a counter (deferred
    // second orientations are then scanned in full warps)
    CG_CUDA(c, c->laneWork.ensure(sizeof(unsigned int)));
    CG_CUDA(c, cudaMemsetAsync(c->laneWork.p, 0, sizeof(unsigned int), c->stream));
    b.laneWork = c->laneWork.as<unsigned int>();
    CG_CUDA(c, cudaEventRecord(c->st1, c->stream));
    CG_CUDA(c, launch_align_filter(st, c->params, b, c->uoff.as<uint32_t>(), c->hPinned[2], c->st1b, c->stream));
    CG_CUDA(c, cudaEventRecord(c->st2, c->stream));
    CG_CUDA(c, c->msaOrder.ensure((size_t)count * sizeof(uint32_t)));
    CG_CUDA(c, c->orderScratch.ensure(32 * sizeof(unsigned int)));
    CG_CUDA(c, launch_msa_order(b, c->orderScratch.as<unsigned int>(), c->msaOrder.as<uint32_t>(), c->stream));
    c->stats.kernel_launches += 2;
    b.order = c->msaOrder.as<uint32_t>();
    CG_CUDA(c, launch_msa_correct(st, c->params, b, (int)std::max<uint32_t>(c->hPinned[1], 1), c->stream));
    if (learned && !c->collecting) {
        CG_CUDA(c, launch_mlp_infer(c->mlp.as<unsigned char>(), b.colFeat, b.colMeta, b.colCount, 0, b.colCap,
                                    c->minLogit, b.out, b.outPitch, nullptr, b.counters, infer_blocks(c),
                                    c->stream));
        c->stats.kernel_launches += 1;
    }
    if (c->params.candidates) {
        CG_CUDA(c, launch_anchor_vote(st, c->params, b, c->stream));
        c->stats.kernel_launches += 1;
    }
    CG_CUDA(c, cudaEventRecord(c->st3, c->stream));
    c->stats.kernel_launches += 3;
    c->stats.align_launches += 1;
    c->stats.msa_launches += 1;
    CG_CUDA(c, cudaMemcpyAsync(hFlags, b.flags, (size_t)count, c->outKind, c->stream));
    CG_CUDA(c, cudaMemcpy2DAsync(hOut, outPitch, b.out, (size_t)c->lmax, std::min<size_t>(outPitch, c->lmax),
                                 (size_t)count, c->outKind, c->stream));
    CG_CUDA(c, cudaEventSynchronize(c->st3));
    float t01 = 0, t11 = 0, t12 = 0, t23 = 0;
    cudaEventElapsedTime(&t01, c->st0, c->st1);
    cudaEventElapsedTime(&t11, c->st1, c->st1b);
    cudaEventElapsedTime(&t12, c->st1b, c->st2);
    cudaEventElapsedTime(&t23, c->st2, c->st3);
    c->stats.seconds_candidates += t01 / 1000.0;
    c->stats.seconds_align += t11 / 1000.0;
    c->stats.seconds_filter += t12 / 1000.0;
    c->stats.seconds_msa += t23 / 1000.0;
    return CG_OK;
}

// ---------------------------------------------------------------- batched driver
//
// One CUDA graph per batch pipeline, captured once per shape and replayed for
// every batch: the candidate kernel (bucket lookup, gather, unique), the
// candidate numbering scan, the persistent alignment kernel, the filter, the
// persistent MSA/correction kernel and a one-thread kernel that advances the
// pipeline's device cursor to its next batch.  Nothing in a replay depends on
// a host value: the batch's first anchor is read from the cursor, its raw id
// offsets come from one scan over the whole range (raw counts per read are
// computed once, with the tables), and the buffers are sized before the
// replays from the range's largest batch.  With two pipelines, batches
// alternate between two streams so that one batch's memory-bound candidate
// stage runs beside the other's compute-bound alignment.

BatchArg set_arg(cg_ctx* c, BatchSet& s, int count) {
    BatchArg b{};
    b.count = count;
    b.sig = c->sig.as<unsigned long long>();
    b.rawCount = s.rawCount.as<uint32_t>();
    b.cand = s.cand.as<uint32_t>();
    b.ncand = s.ncand.as<uint32_t>();
    b.paired = s.paired.as<uint8_t>();
    b.aln = s.aln.as<uint2>();
    b.fid = s.fid.as<uint32_t>();
    b.fshift = s.fshift.as<int16_t>();
    b.forient = s.forient.as<uint8_t>();
    b.fweight = s.fweight.as<float>();
    b.flen = s.flen.as<uint16_t>();
    b.nfinal = s.nfinal.as<uint32_t>();
    b.perm = c->lenVaries || c->strandTags ? s.perm.as<uint32_t>() : nullptr;
    b.lenOrder = c->lenVaries;
    b.flags = c->flagsRange.as<uint8_t>();
    b.out = c->outRange.as<char>();
    b.outPitch = c->lmax;
    b.counters = c->counters.as<unsigned long long>();
    b.cursor = s.cursor.as<unsigned long long>();
    b.rangeOff = c->rangeOff.as<unsigned long long>();
    b.work = s.work.as<unsigned int>();
    if (c->params.correctionType == CG_CORR_LEARNED) set_columns(b, s.colFeat, s.colMeta, s.colCount, count);
    b.order = s.order.as<uint32_t>();
    return b;
}

int ensure_set(cg_ctx* c, BatchSet& s, int count, uint64_t capRaw) {
    if (!s.stream) CG_CUDA(c, cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
    if (!s.joined) CG_CUDA(c, cudaEventCreateWithFlags(&s.joined, cudaEventDisableTiming));
    const size_t n = (size_t)count;
    CG_CUDA(c, s.rawCount.ensure((n + 2) * sizeof(uint32_t)));
    CG_CUDA(c, s.ncand.ensure(n * sizeof(uint32_t)));
    CG_CUDA(c, s.uoff.ensure((n + 1) * sizeof(uint32_t)));
    CG_CUDA(c, s.nfinal.ensure(n * sizeof(uint32_t)));
    CG_CUDA(c, s.scanTmp.ensure(scan_tmp_bytes(n + 1)));
    CG_CUDA(c, s.cand.ensure(capRaw * sizeof(uint32_t)));
    if (c->lenVaries || c->strandTags) CG_CUDA(c, s.perm.ensure(capRaw * sizeof(uint32_t)));
    CG_CUDA(c, s.paired.ensure(capRaw));
    CG_CUDA(c, s.aln.ensure(capRaw * sizeof(uint2)));
    CG_CUDA(c, s.fid.ensure(capRaw * sizeof(uint32_t)));
    CG_CUDA(c, s.fshift.ensure(capRaw * sizeof(int16_t)));
    CG_CUDA(c, s.forient.ensure(capRaw));
    CG_CUDA(c, s.fweight.ensure(capRaw * sizeof(float)));
    CG_CUDA(c, s.flen.ensure(capRaw * sizeof(uint16_t)));
    CG_CUDA(c, s.cursor.ensure(2 * sizeof(unsigned long long)));
    CG_CUDA(c, s.work.ensure(2 * sizeof(unsigned int)));
    CG_CUDA(c, s.order.ensure(n * sizeof(uint32_t)));
    CG_CUDA(c, s.orderScratch.ensure(32 * sizeof(unsigned int)));
    CG_CUDA(c, s.bigScratch.ensure((n + 1) * sizeof(uint32_t)));
    if (c->params.correctionType == CG_CORR_LEARNED) return ensure_columns(c, s.colFeat, s.colMeta, s.colCount, count);
    return CG_OK;
}

// The kernels of one batch, enqueued on the set's stream (captured).
cudaError_t enqueue_batch(cg_ctx* c, BatchSet& s, int count, unsigned long long stride, const Shape& sh,
                          int tableRaw, int maxRows, int* kernels) {
    const StoreArg st = store_arg(c);
    const BatchArg b = set_arg(c, s, count);
    uint32_t* uoff = s.uoff.as<uint32_t>();
    int k = 0;
    const bool learned = c->params.correctionType == CG_CORR_LEARNED;
    cudaError_t e = learned ? cudaMemsetAsync(b.colCount, 0, sizeof(unsigned int), s.stream) : cudaSuccess;
    if (e == cudaSuccess)
        e = launch_gather_unique(st, c->tables, c->params, b, tableRaw, s.stream, s.bigScratch.as<uint32_t>());
    k += tableRaw > 1024 ? 2 : 1;
    if (e == cudaSuccess && c->params.paired) {
        e = launch_pair_flags(b, s.stream);
        k++;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(uoff, b.ncand, (size_t)count * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(uoff + count, 0, sizeof(uint32_t), s.stream);
    if (e == cudaSuccess) {
        e = scan_exclusive_u32(uoff, (size_t)count + 1, s.scanTmp.p, s.stream);
        k += (int)scan_launches((uint64_t)count + 1);
    }
    if (e == cudaSuccess) {
        e = launch_align_filter(st, c->params, b, uoff, 0, nullptr, s.stream, &sh);
        k += st.wp - 1 <= 8 ? 2 : 1;
    }
    if (e == cudaSuccess) {
        e = launch_msa_order(b, s.orderScratch.as<unsigned int>(), s.order.as<uint32_t>(), s.stream);
        k += 2;
    }
    if (e == cudaSuccess) {
        e = launch_msa_correct(st, c->params, b, maxRows, s.stream, &sh);
        k++;
    }
    if (e == cudaSuccess && learned) {
        e = launch_mlp_infer(c->mlp.as<unsigned char>(), b.colFeat, b.colMeta, b.colCount, 0, b.colCap, c->minLogit,
                             b.out, b.outPitch, nullptr, b.counters, infer_blocks(c), s.stream);
        k++;
    }
    if (e == cudaSuccess && c->params.candidates) {
        e = launch_anchor_vote(st, c->params, b, s.stream);
        k++;
    }
    if (e == cudaSuccess) {
        e = launch_batch_advance(s.cursor.as<unsigned long long>(), s.work.as<unsigned int>(), stride, s.stream);
        k++;
    }
    *kernels = k;
    return e;
}

int capture_set(cg_ctx* c, BatchSet& s, int count, unsigned long long stride, const Shape& sh, int tableRaw,
                int maxRows) {
    GraphSig g;
    g.count = count;
    g.stride = stride;
    g.shape = sh;
    g.tableRaw = tableRaw;
    g.maxRows = maxRows;
    for (const DevBuf* d : {&s.rawCount, &s.cand, &s.ncand, &s.paired, &s.aln, &s.fid, &s.fshift, &s.forient,
                            &s.fweight, &s.flen, &s.nfinal, &s.uoff, &s.scanTmp, &s.cursor, &s.work, &s.colFeat,
                            &s.colMeta, &s.colCount, &s.order, &s.orderScratch, &s.bigScratch, &s.perm, &c->mlp,
                            &c->outRange,
                            &c->flagsRange, &c->rangeOff, &c->counters, &c->sig})
        g.ptrs.push_back(d->p);
    g.ptrs.push_back(reinterpret_cast<const void*>(static_cast<uintptr_t>(c->paramsVersion)));
    if (s.exec && g == s.sig) return CG_OK;
    if (s.exec) cudaGraphExecDestroy(s.exec);
    s.exec = nullptr;
    CG_CUDA(c, cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    int kernels = 0;
    const cudaError_t e = enqueue_batch(c, s, count, stride, sh, tableRaw, maxRows, &kernels);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s.stream, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return fail(c, CG_ERR_CUDA, "batch graph capture failed: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    const cudaError_t e3 = cudaGraphInstantiate(&s.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) {
        s.exec = nullptr;
        return fail(c, CG_ERR_CUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e3));
    }
    s.sig = g;
    s.kernels = kernels;
    return CG_OK;
}

int ensure_batched_state(cg_ctx* c) {
    if (!c->hBatched) CG_CUDA(c, cudaMallocHost(&c->hBatched, (2 + 2 * kMaxSets) * sizeof(unsigned long long)));
    if (!c->copyStream) CG_CUDA(c, cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking));
    if (!c->evPro) CG_CUDA(c, cudaEventCreateWithFlags(&c->evPro, cudaEventDisableTiming));
    if (!c->evStart) CG_CUDA(c, cudaEventCreate(&c->evStart));
    if (!c->haveRawAll) {
        // the table build summed the bucket sizes (batched driver only)
        if (!c->rawAll.p) return fail(c, CG_ERR_STATE, "raw counts were not built with the tables");
        CG_CUDA(c, launch_raw_count(store_arg(c), c->params, c->rawAll.as<uint32_t>(), c->stream));
        c->stats.kernel_launches += 1;
        c->haveRawAll = true;
    }
    return CG_OK;
}

// Enqueue the `nb` full batches of `pl.batch` anchors starting at `first`:
// prologue on c->stream (one host round trip for the buffer sizes), then the
// graph replays on the sets' streams.  Batch j's outputs land in rows
// j * batch .. of c->outRange / c->flagsRange; if `done` is given, event
// done[j] follows batch j.  The caller orders c->stream after the sets.
int run_batched(cg_ctx* c, uint64_t first, uint64_t nb, const Plan& pl, const std::vector<cudaEvent_t>* done) {
    const uint64_t B = (uint64_t)pl.batch;
    const uint64_t num = nb * B;
    CG_CUDA(c, c->rangeOff.ensure((num + 1) * sizeof(unsigned long long)));
    CG_CUDA(c, c->rangeTmp.ensure(scan_tmp_bytes(num + 1)));
    CG_CUDA(c, c->maxima.ensure(2 * sizeof(unsigned long long)));
    CG_CUDA(c, launch_range_offsets(c->rawAll.as<uint32_t>() + first, num, B, c->rangeOff.as<unsigned long long>(),
                                    c->rangeTmp.p, c->maxima.as<unsigned long long>(), c->stream));
    c->stats.kernel_launches += 2 + scan_launches(num + 1);
    CG_CUDA(c, cudaMemcpyAsync(c->hBatched, c->maxima.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    const uint64_t capRaw = std::max<unsigned long long>(c->hBatched[0], 1);
    const int maxRaw = (int)std::max<unsigned long long>(c->hBatched[1], 1);
    if (capRaw > 0xffffffffull) return fail(c, CG_ERR_UNSUPPORTED, "batch of %llu raw ids exceeds 2^32",
                                            (unsigned long long)capRaw);
    CG_CUDA(c, c->outRange.ensure(num * c->lmax));
    CG_CUDA(c, c->flagsRange.ensure(num));
    const int S = pl.streams;
    for (int k = 0; k < S; k++) {
        BatchSet& s = c->sets[k];
        int rc = ensure_set(c, s, pl.batch, capRaw);
        if (rc != CG_OK) return rc;
        rc = capture_set(c, s, pl.batch, B * S, pl.shape, maxRaw, maxRaw);
        if (rc != CG_OK) return rc;
        c->hBatched[2 + 2 * k] = first + (uint64_t)k * B;
        c->hBatched[3 + 2 * k] = first;
        CG_CUDA(c, cudaMemcpyAsync(s.cursor.p, c->hBatched + 2 + 2 * k, 2 * sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, c->stream));
        CG_CUDA(c, cudaMemsetAsync(s.work.p, 0, 2 * sizeof(unsigned int), c->stream));
    }
    CG_CUDA(c, cudaEventRecord(c->evPro, c->stream));
    CG_CUDA(c, cudaEventRecord(c->evStart, c->stream));  // replays start (after any capture)
    for (int k = 0; k < S; k++) CG_CUDA(c, cudaStreamWaitEvent(c->sets[k].stream, c->evPro, 0));
    for (uint64_t j = 0; j < nb; j++) {
        BatchSet& s = c->sets[j % S];
        CG_CUDA(c, cudaGraphLaunch(s.exec, s.stream));
        if (done) CG_CUDA(c, cudaEventRecord((*done)[j], s.stream));
        c->stats.kernel_launches += (uint64_t)s.kernels;
        c->stats.align_launches += 1;
        c->stats.msa_launches += 1;
        c->stats.graph_replays += 1;
    }
    return CG_OK;
}

// `to` waits for everything enqueued so far on the first S sets' streams
int join_sets(cg_ctx* c, int S, cudaStream_t to) {
    for (int k = 0; k < S; k++) {
        CG_CUDA(c, cudaEventRecord(c->sets[k].joined, c->sets[k].stream));
        CG_CUDA(c, cudaStreamWaitEvent(to, c->sets[k].joined, 0));
    }
    return CG_OK;
}

// A learned-decision call whose classifier blocks gave up waiting for their
// MMAs (counters[kCounterTimeouts] grew) left those blocks' columns to the
// fallback decision: the call reports CG_ERR_TIMEOUT instead of CG_OK.
int check_classifier_timeouts(cg_ctx* c) {
    if (c->params.correctionType != CG_CORR_LEARNED || c->collecting) return CG_OK;
    unsigned long long n = 0;
    CG_CUDA(c, cudaMemcpy(&n, c->counters.as<unsigned long long>() + kCounterTimeouts, sizeof(n),
                          cudaMemcpyDeviceToHost));
    if (n > c->timeoutsSeen) {
        const unsigned long long grew = n - c->timeoutsSeen;
        c->timeoutsSeen = n;
        return fail(c, CG_ERR_TIMEOUT,
                    "%llu classifier block(s) timed out waiting for the tensor cores; their columns kept the "
                    "fallback decision",
                    grew);
    }
    return CG_OK;
}

// ---- autotuner
//
// The batch size, the persistent grids and the number of pipelines change
// only the speed (every candidate and anchor is computed the same way in any
// shape), so they are picked by timing: coordinate descent over a few values
// per dimension, each trial running the same sample of anchors (the first
// anchors of the range) end to end through run_batched.  The counters are
// saved before and restored after.  The result is kept for the process, keyed
// by what decides the kernels' cost.

using TuneKey = std::tuple<int, int, int, int, int, int, int, int>;
std::mutex gTuneMu;
std::map<TuneKey, Plan> gTuned;

TuneKey tune_key(const cg_ctx* c) {
    int lg = 0;
    while ((1ull << lg) < c->n) lg++;
    return TuneKey(c->device, c->lmax, c->params.useQuality, c->params.correctionType, c->params.paired, c->nmaps,
                   c->maxValuesPerKey, lg);
}

int sm_count(cg_ctx* c) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) sms = 1;
    return std::max(sms, 1);
}

// complete a shape: unset grids become the resident maximum
Plan fill_plan(cg_ctx* c, Plan p) {
    const StoreArg st = store_arg(c);
    const int sms = sm_count(c);
    if (p.batch <= 0) p.batch = 65536;
    if (c->params.paired && (p.batch & 1)) p.batch++;
    if (p.streams <= 0) p.streams = 2;
    p.streams = std::min(p.streams, kMaxSets);
    if (p.shape.msaWarps <= 0) p.shape.msaWarps = 4;
    p.shape.msaWarps = std::min(std::max(p.shape.msaWarps, 1), 8);
    if (p.shape.alignBlocks <= 0) p.shape.alignBlocks = sms * std::max(align_lane_occupancy(st), 1);
    if (p.shape.msaBlocks <= 0) p.shape.msaBlocks = sms * std::max(msa_warp_occupancy(st, c->params, p.shape.msaWarps), 1);
    return p;
}

// device seconds of one run of `pl` over the sample [first, first + sample)
int time_plan(cg_ctx* c, uint64_t first, uint64_t sample, const Plan& pl, double* sec) {
    const uint64_t nb = sample / (uint64_t)pl.batch;
    if (nb == 0) {
        *sec = 1e30;
        return CG_OK;
    }
    int rc = run_batched(c, first, nb, pl, nullptr);
    if (rc != CG_OK) return rc;
    rc = join_sets(c, pl.streams, c->stream);
    if (rc != CG_OK) return rc;
    CG_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    CG_CUDA(c, cudaEventSynchronize(c->ev1));
    float ms = 0;  // the replays only: the graph capture of a new shape is not timed
    CG_CUDA(c, cudaEventElapsedTime(&ms, c->evStart, c->ev1));
    *sec = ms / 1000.0 / (double)(nb * (uint64_t)pl.batch);  // per anchor
    return CG_OK;
}

int plan_for(cg_ctx* c, uint64_t first, uint64_t num, Plan* out) {
    Plan want;
    want.batch = c->o.batch_anchors;
    want.shape.alignBlocks = c->o.align_blocks;
    want.shape.msaWarps = c->o.msa_warps;
    want.streams = c->o.streams;
    const bool fixed = want.batch > 0 && want.shape.alignBlocks > 0 && want.shape.msaWarps > 0 && want.streams > 0;
    const uint64_t sample = std::min<uint64_t>(num, 262144);
    if (fixed || sample < 2 * 32768) {
        *out = fill_plan(c, want);
        return CG_OK;
    }
    const TuneKey key = tune_key(c);
    {
        std::lock_guard<std::mutex> lk(gTuneMu);
        auto it = gTuned.find(key);
        if (it != gTuned.end()) {
            Plan p = it->second;
            if (want.batch > 0) p.batch = want.batch;
            if (want.shape.alignBlocks > 0) p.shape.alignBlocks = want.shape.alignBlocks;
            if (want.shape.msaWarps > 0) {
                p.shape.msaWarps = want.shape.msaWarps;
                p.shape.msaBlocks = 0;
            }
            if (want.streams > 0) p.streams = want.streams;
            *out = fill_plan(c, p);
            return CG_OK;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    const size_t cbytes = kNumCounters * sizeof(unsigned long long);
    CG_CUDA(c, c->counterSave.ensure(cbytes));
    CG_CUDA(c, cudaMemcpyAsync(c->counterSave.p, c->counters.p, cbytes, cudaMemcpyDeviceToDevice, c->stream));
    // the trials run without candidate correction: their votes would join the pass
    const int cand = c->params.candidates;
    if (cand) {
        c->params.candidates = 0;
        c->paramsVersion++;
    }
    const StoreArg st = store_arg(c);
    const int sms = sm_count(c);
    const int occA = std::max(align_lane_occupancy(st), 1);
    Plan best = fill_plan(c, want);
    double bestSec = 0;
    int rc = time_plan(c, first, sample, best, &bestSec);
    auto trial = [&](Plan p) -> int {
        p = fill_plan(c, p);
        double sec = 0;
        const int r = time_plan(c, first, sample, p, &sec);
        if (r == CG_OK && sec < bestSec) {
            best = p;
            bestSec = sec;
        }
        return r;
    };
    if (rc == CG_OK && want.shape.msaWarps <= 0) {
        for (int w : {1, 2, 8}) {
            Plan p = best;
            p.shape.msaWarps = w;
            p.shape.msaBlocks = 0;
            if ((rc = trial(p)) != CG_OK) break;
        }
    }
    if (rc == CG_OK && want.shape.alignBlocks <= 0 && occA > 1) {
        Plan p = best;
        p.shape.alignBlocks = sms * std::max(occA / 2, 1);
        rc = trial(p);
    }
    if (rc == CG_OK && want.streams <= 0) {
        Plan p = best;
        p.streams = 1;
        rc = trial(p);
    }
    if (rc == CG_OK && want.batch <= 0) {
        for (int bsz : {32768, 131072}) {
            Plan p = best;
            p.batch = bsz;
            if ((rc = trial(p)) != CG_OK) break;
        }
    }
    if (cand) {
        c->params.candidates = cand;
        c->paramsVersion++;
    }
    CG_CUDA(c, cudaMemcpyAsync(c->counters.p, c->counterSave.p, cbytes, cudaMemcpyDeviceToDevice, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (rc != CG_OK) return rc;
    c->stats.seconds_tune += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    {
        std::lock_guard<std::mutex> lk(gTuneMu);
        gTuned[key] = best;
    }
    *out = best;
    return CG_OK;
}

// cg_correct with the batched driver: full batches as graph replays, the
// remainder (fewer anchors than a batch) through the plain driver on the
// context's own stream, concurrently.
int correct_batched(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* out_flags, char* out_seq, size_t out_pitch) {
    int rc = ensure_batched_state(c);
    if (rc != CG_OK) return rc;
    Plan pl;
    rc = plan_for(c, first, num, &pl);
    if (rc != CG_OK) return rc;
    c->stats.batch_anchors = pl.batch;
    c->stats.align_blocks = pl.shape.alignBlocks;
    c->stats.msa_warps = pl.shape.msaWarps;
    c->stats.streams = pl.streams;
    const uint64_t B = (uint64_t)pl.batch;
    const uint64_t nb = num / B;
    const uint64_t done = nb * B;
    CG_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if (nb > 0) {
        while (c->batchDone.size() < nb) {
            cudaEvent_t ev = nullptr;
            CG_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            c->batchDone.push_back(ev);
        }
        rc = run_batched(c, first, nb, pl, &c->batchDone);
        if (rc != CG_OK) return rc;
    }
    if (done < num) {
        // the remainder runs beside the replays; its own syncs wait only for it
        int B2 = pl.batch;
        for (uint64_t a = done; a < num; a += (uint64_t)B2) {
            const int cnt = (int)std::min<uint64_t>((uint64_t)B2, num - a);
            rc = run_batch(c, first + a, cnt, out_flags + a, out_seq + a * out_pitch, out_pitch);
            if (rc != CG_OK) return rc;
        }
    }
    // results of each batch to the host as soon as the batch is done
    for (uint64_t j = 0; j < nb; j++) {
        CG_CUDA(c, cudaStreamWaitEvent(c->copyStream, c->batchDone[j], 0));
        CG_CUDA(c, cudaMemcpyAsync(out_flags + j * B, c->flagsRange.as<uint8_t>() + j * B, B, c->outKind,
                                   c->copyStream));
        CG_CUDA(c, cudaMemcpy2DAsync(out_seq + j * B * out_pitch, out_pitch, c->outRange.as<char>() + j * B * c->lmax,
                                     (size_t)c->lmax, (size_t)c->lmax, B, c->outKind, c->copyStream));
    }
    if (nb > 0) {  // the pipelines exist only once a full batch ran
        rc = join_sets(c, pl.streams, c->stream);
        if (rc != CG_OK) return rc;
    }
    CG_CUDA(c, cudaEventRecord(c->evPro, c->copyStream));
    CG_CUDA(c, cudaStreamWaitEvent(c->stream, c->evPro, 0));
    CG_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    CG_CUDA(c, cudaEventSynchronize(c->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.seconds_correct = ms / 1000.0;
    c->stats.num_anchors_processed += num;
    return check_classifier_timeouts(c);
}

}  // namespace

extern "C" {

void cg_default_options(cg_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->kmerlength = 20;
    o->num_hash_functions = 48;
    o->estimated_coverage = 1.0f;
    o->estimated_errorrate = 0.06f;
    o->m_coverage = 0.6f;
    o->max_error_rate = 0.2f;
    o->min_overlap_ratio = 0.30f;
    o->min_overlap = 30;
    o->paired_filter_threshold = 0.06f;
    o->new_columns_to_correct = 15;
    o->pair_mode = CG_PAIR_SE;
    o->correction_type = CG_CORR_CLASSIC;
    o->threshold_anchor = 0.5f;
    o->quality_score_bits = 8;
}

int cg_create(const cg_options* o, cg_ctx** out) {
    if (!o || !out) return CG_ERR_INVALID_ARGUMENT;
    if (o->num_hash_functions < 1 || o->num_hash_functions > CG_MAX_HASHMAPS) return CG_ERR_INVALID_ARGUMENT;
    if (o->kmerlength < 0 || o->kmerlength > 32) return CG_ERR_INVALID_ARGUMENT;
    if (!(o->estimated_coverage > 0.0f)) return CG_ERR_INVALID_ARGUMENT;
    if (o->pair_mode != CG_PAIR_SE && o->pair_mode != CG_PAIR_PE) return CG_ERR_INVALID_ARGUMENT;
    if (o->correct_candidates && (o->new_columns_to_correct < 0 || o->new_columns_to_correct > 256))
        return CG_ERR_UNSUPPORTED;
    if (o->correction_type != CG_CORR_CLASSIC && o->correction_type != CG_CORR_FOREST &&
        o->correction_type != CG_CORR_LEARNED)
        return CG_ERR_UNSUPPORTED;
    if (o->correction_type == CG_CORR_LEARNED && !(o->threshold_anchor > 0.0f && o->threshold_anchor < 1.0f))
        return CG_ERR_INVALID_ARGUMENT;
    if (o->driver != CG_DRIVER_PLAIN && o->driver != CG_DRIVER_BATCHED) return CG_ERR_INVALID_ARGUMENT;
    if (o->quality_score_bits != 0 && o->quality_score_bits != 1 && o->quality_score_bits != 2 &&
        o->quality_score_bits != 8)
        return CG_ERR_UNSUPPORTED;  // the reference's QualityCompressorWrapper knows 1, 2 and 8
    if (o->pair_mode == CG_PAIR_PE && (o->fixed_number_of_reads & 1u)) return CG_ERR_INVALID_ARGUMENT;
    if (o->batch_anchors < 0 || o->align_blocks < 0 || o->msa_warps < 0 || o->msa_warps > 8 || o->streams < 0 ||
        o->streams > kMaxSets)
        return CG_ERR_INVALID_ARGUMENT;
    cg_ctx* c = new (std::nothrow) cg_ctx();
    if (!c) return CG_ERR_OUT_OF_MEMORY;
    c->o = *o;
    if (o->correction_type == CG_CORR_LEARNED)  // p >= t  <=>  logit >= log(t / (1 - t))
        c->minLogit = (float)std::log((double)o->threshold_anchor / (1.0 - (double)o->threshold_anchor));
    c->device = o->device;
    auto bail = [&](cudaError_t e) {
        cudaGetLastError();
        cg_destroy(c);  // streams, events and blocks made so far
        return e == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return bail(e);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(e);
    e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    for (cudaEvent_t* ev : {&c->st0, &c->st1, &c->st1b, &c->st2, &c->st3})
        if (e == cudaSuccess) e = cudaEventCreate(ev);
    if (e == cudaSuccess) e = cudaMallocHost(&c->hPinned, 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = c->counters.ensure(kNumCounters * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(c->counters.p, 0, kNumCounters * sizeof(unsigned long long));
    if (e != cudaSuccess) return bail(e);
    *out = c;
    return CG_OK;
}

int cg_release_cached_memory(int device) {
    block_cache().trim(device);
    forget_noalloc_scratch(device);
    return cudaGetLastError() == cudaSuccess ? CG_OK : CG_ERR_CUDA;
}

int cg_set_allocation_fault(int64_t after) {
    g_allocFault.store(after < 0 ? -1 : (long long)after);
    return CG_OK;
}

int cg_set_classifier_wait_limit(int device, int64_t polls) {
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return CG_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return CG_ERR_INVALID_ARGUMENT;
    }
    const uint32_t p = polls < 0 ? (1u << 20) : (uint32_t)std::min<int64_t>(polls, 0xffffffffll);
    const cudaError_t e = set_classifier_wait_limit(p);
    cudaSetDevice(cur);
    return e == cudaSuccess ? CG_OK : CG_ERR_CUDA;
}

void cg_destroy(cg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    release_tables(c);
    for (DevBuf* b : {&c->enc, &c->len, &c->hilo, &c->qual, &c->ambig, &c->sig, &c->strand, &c->qrange, &c->rawCount,
                      &c->cand,
                      &c->ncand, &c->paired, &c->aln, &c->fid, &c->fshift, &c->forient, &c->fweight, &c->flen, &c->nfinal,
                      &c->flags, &c->out, &c->counters, &c->scanTmp, &c->uoff, &c->forestNodes, &c->treeOffsets,
                      &c->msaOrder, &c->orderScratch, &c->bigScratch, &c->perm, &c->lenRange, &c->laneWork})
        b->release();
    for (cg_ctx::Chunk& ch : c->chunks) {
        ch.chars.release();
        ch.offs.release();
        ch.qual.release();
    }
    for (BatchSet& bs : c->sets) bs.release();
    for (DevBuf* b : {&c->rawAll, &c->rangeOff, &c->rangeTmp, &c->maxima, &c->outRange, &c->flagsRange,
                      &c->counterSave, &c->mlp, &c->colFeat, &c->colMeta, &c->colCount})
        b->release();
    for (cudaEvent_t ev : c->batchDone) cudaEventDestroy(ev);
    if (c->evPro) cudaEventDestroy(c->evPro);
    if (c->evStart) cudaEventDestroy(c->evStart);
    if (c->copyStream) cudaStreamDestroy(c->copyStream);
    if (c->hBatched) cudaFreeHost(c->hBatched);
    if (c->hPinned) cudaFreeHost(c->hPinned);
    for (cudaEvent_t ev : {c->ev0, c->ev1, c->st0, c->st1, c->st1b, c->st2, c->st3})
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* cg_last_error(const cg_ctx* c) { return c ? c->err.c_str() : "no context"; }

int cg_append_reads(cg_ctx* c, const char* sequences, const uint64_t* offsets, const char* qualities,
                    uint64_t num_reads) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (c->built) return fail(c, CG_ERR_STATE, "reads cannot be appended after cg_build_tables");
    if (!sequences || !offsets || num_reads == 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "empty read batch");
    if (c->o.use_quality_scores && !qualities)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "quality scores requested but not given");
    // the first read whose offsets descend or span more than the longest read
    // (in read order, as a sequential check finds it), and the longest read
    uint64_t badOrder = ~0ull, badLength = ~0ull;
    int lmax = 0;
#pragma omp parallel for reduction(min : badOrder, badLength) reduction(max : lmax) if (num_reads > (1u << 16))
    for (uint64_t i = 0; i < num_reads; i++) {
        if (offsets[i + 1] < offsets[i]) badOrder = std::min(badOrder, i);
        else if (offsets[i + 1] - offsets[i] > CG_MAX_READ_LENGTH) badLength = std::min(badLength, i);
        else lmax = std::max(lmax, (int)(offsets[i + 1] - offsets[i]));
    }
    if (badOrder < badLength)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "offsets not ascending at %llu", (unsigned long long)badOrder);
    if (badLength != ~0ull)
        return fail(c, CG_ERR_UNSUPPORTED, "read %llu longer than %d", (unsigned long long)badLength,
                    CG_MAX_READ_LENGTH);
    if (c->appended + num_reads > 0xffffffffull) return fail(c, CG_ERR_UNSUPPORTED, "more than 2^32-1 reads");
    CG_CUDA(c, cudaSetDevice(c->device));
    const uint64_t bytes = offsets[num_reads] - offsets[0];
    c->chunks.emplace_back();
    cg_ctx::Chunk& ch = c->chunks.back();
    ch.first = c->appended;
    ch.reads = num_reads;
    // straight from the caller's memory to the device: no host staging copy
    CG_CUDA(c, ch.chars.ensure(std::max<uint64_t>(bytes, 1)));
    CG_CUDA(c, ch.offs.ensure((num_reads + 1) * sizeof(uint64_t)));
    CG_CUDA(c, cudaMemcpyAsync(ch.chars.p, sequences + offsets[0], bytes, cudaMemcpyHostToDevice, c->stream));
    // the caller's offsets as they are, made relative to the chunk on the device
    CG_CUDA(c, cudaMemcpyAsync(ch.offs.p, offsets, (num_reads + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                               c->stream));
    CG_CUDA(c, launch_rebase_offsets(ch.offs.as<uint64_t>(), num_reads + 1, offsets[0], c->stream));
    if (c->o.use_quality_scores) {
        CG_CUDA(c, ch.qual.ensure(std::max<uint64_t>(bytes, 1)));
        CG_CUDA(c, cudaMemcpyAsync(ch.qual.p, qualities + offsets[0], bytes, cudaMemcpyHostToDevice, c->stream));
    }
    CG_CUDA(c, cudaStreamSynchronize(c->stream));  // the caller's buffers may go away
    c->appended += num_reads;
    c->appendLmax = std::max(c->appendLmax, lmax);
    return CG_OK;
}

int cg_build_tables(cg_ctx* c) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (c->appended == 0) return fail(c, CG_ERR_STATE, "no reads appended");
    if (c->o.pair_mode == CG_PAIR_PE && (c->appended & 1))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "paired mode needs an even number of reads");
    if (c->o.hashtable_memory_bytes) {
        // reference: include/ordinaryminhasher.hpp:350-372 -- maps of the first
        // construction round: limit / ((sizeof key + sizeof read id) x reads) - 2
        const long long fit = (long long)(c->o.hashtable_memory_bytes / (12ull * c->appended)) - 2;
        if (fit < c->o.num_hash_functions)
            return fail(c, CG_ERR_UNSUPPORTED,
                        "memoryForHashtables %llu bytes holds %lld maps of %llu reads in the reference's first "
                        "construction round, fewer than the %d requested; the reference's final map count would "
                        "depend on its host tables' sizes",
                        (unsigned long long)c->o.hashtable_memory_bytes, fit, (unsigned long long)c->appended,
                        c->o.num_hash_functions);
    }
    CG_CUDA(c, cudaSetDevice(c->device));
    CG_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    int rc = build_store(c);
    if (rc != CG_OK) return rc;
    rc = build_tables(c);
    if (rc != CG_OK) return rc;
    if (c->o.correct_candidates) {
        const size_t words = c->n * (size_t)((c->lmax + 31) / 32);
        CG_CUDA(c, c->candVotes.ensure(c->n * sizeof(uint2)));
        CG_CUDA(c, c->candAnd.ensure(words * sizeof(unsigned long long)));
        CG_CUDA(c, c->candOr.ensure(words * sizeof(unsigned long long)));
        rc = reset_candidates(c);
        if (rc != CG_OK) return rc;
    }
    make_params(c);
    if (c->o.driver == CG_DRIVER_BATCHED) {
        // raw id counts per read: part of the index the batched driver reads
        rc = ensure_batched_state(c);
        if (rc != CG_OK) return rc;
    }
    CG_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    CG_CUDA(c, cudaEventSynchronize(c->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.seconds_build = ms / 1000.0;
    {
        unsigned int range[2] = {0, 0};
        CG_CUDA(c, cudaMemcpy(range, c->lenRange.p, sizeof(range), cudaMemcpyDeviceToHost));
        c->lenVaries = range[0] != range[1];
    }
    c->stats.num_reads = c->n;
    c->stats.kmerlength = c->k;
    c->stats.num_maps = c->nmaps;
    c->stats.max_read_length = c->lmax;
    c->built = true;
    return CG_OK;
}

int cg_correct(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* out_flags, char* out_seq, size_t out_pitch) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (first + num > c->n || first + num < first) return fail(c, CG_ERR_INVALID_ARGUMENT, "anchor range out of bounds");
    if (num == 0) return CG_OK;
    if (!out_flags || !out_seq || out_pitch < (size_t)c->lmax)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "output buffers missing or pitch below %d", c->lmax);
    if (c->params.paired && ((first | num) & 1)) return fail(c, CG_ERR_INVALID_ARGUMENT, "paired mode needs even ranges");
    if (c->o.correction_type == CG_CORR_FOREST && c->numTrees == 0)
        return fail(c, CG_ERR_STATE, "forest correction requested but no forest loaded (cg_load_forest)");
    if (c->o.correction_type == CG_CORR_LEARNED && !c->haveMlp)
        return fail(c, CG_ERR_STATE, "learned correction requested but no classifier loaded (cg_load_classifier)");
    if (c->o.correction_type == CG_CORR_LEARNED && c->lmax > 256)
        return fail(c, CG_ERR_UNSUPPORTED, "learned correction supports reads up to 256 bp (longest is %d)", c->lmax);
    CG_CUDA(c, cudaSetDevice(c->device));
    {
        // fixedNumberOfReads: anchors past the limit are not corrected
        const uint64_t limit =
            c->o.fixed_number_of_reads ? std::min<uint64_t>(c->o.fixed_number_of_reads, c->n) : c->n;
        const uint64_t run = first >= limit ? 0 : std::min(num, limit - first);
        if (run < num) {
            if (c->outKind == cudaMemcpyDeviceToDevice)
                CG_CUDA(c, cudaMemsetAsync(out_flags + run, 0, num - run, c->stream));
            else
                std::memset(out_flags + run, 0, num - run);
        }
        if (run == 0) {
            CG_CUDA(c, cudaStreamSynchronize(c->stream));
            c->stats.seconds_correct = 0.0;
            return CG_OK;
        }
        num = run;
    }
    if (c->params.candidates) {
        const int rc = mark_pass(c, first, num);
        if (rc != CG_OK) return rc;
    }
    if (c->o.driver == CG_DRIVER_BATCHED) return correct_batched(c, first, num, out_flags, out_seq, out_pitch);
    int B = c->o.batch_anchors > 0 ? c->o.batch_anchors : 65536;
    if (c->params.paired && (B & 1)) B++;
    CG_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    for (uint64_t a = 0; a < num; a += (uint64_t)B) {
        const int cnt = (int)std::min<uint64_t>((uint64_t)B, num - a);
        const int rc = run_batch(c, first + a, cnt, out_flags + a, out_seq + a * out_pitch, out_pitch);
        if (rc != CG_OK) return rc;
    }
    CG_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    CG_CUDA(c, cudaEventSynchronize(c->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.seconds_correct = ms / 1000.0;
    c->stats.num_anchors_processed += num;
    return check_classifier_timeouts(c);
}

int cg_combine_results(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* flags, uint64_t* num_candidate_records) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (!c->params.candidates) return fail(c, CG_ERR_STATE, "candidate correction is off (correct_candidates)");
    if (first + num > c->n || first + num < first) return fail(c, CG_ERR_INVALID_ARGUMENT, "read range out of bounds");
    if (num_candidate_records) *num_candidate_records = 0;
    if (num == 0) return CG_OK;
    if (!flags) return fail(c, CG_ERR_INVALID_ARGUMENT, "flags missing");
    CG_CUDA(c, cudaSetDevice(c->device));
    CG_CUDA(c, c->combineFlags.ensure(num));
    CG_CUDA(c, cudaMemcpyAsync(c->combineFlags.p, flags, num, cudaMemcpyHostToDevice, c->stream));
    const int rc = cg::combine_into_device(c, first, num, c->combineFlags.as<uint8_t>(), num_candidate_records);
    if (rc != CG_OK) return rc;
    CG_CUDA(c, cudaMemcpy(flags, c->combineFlags.p, num, cudaMemcpyDeviceToHost));
    return CG_OK;
}

int cg_get_stats(const cg_ctx* c, cg_stats* out) {
    if (!c || !out) return CG_ERR_INVALID_ARGUMENT;
    cg_stats s = c->stats;
    unsigned long long cnt[kNumCounters] = {0};
    if (c->counters.p) {
        cudaSetDevice(c->device);
        if (cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost) != cudaSuccess)
            return CG_ERR_CUDA;
    }
    s.raw_candidate_ids = cnt[kCounterRaw];
    s.unique_candidates = cnt[kCounterUnique];
    s.aligned_candidates = cnt[kCounterAligned];
    s.msa_candidates = cnt[kCounterMsaCands];
    s.msa_builds = cnt[kCounterMsaBuilds];
    s.corrected_anchors = cnt[kCounterCorrected];
    s.hq_anchors = cnt[kCounterHQ];
    s.learned_columns = cnt[kCounterColumns];
    s.learned_corrections = cnt[kCounterLearnedTaken];
    s.learned_overflow = cnt[kCounterColumnOverflow];
    s.candidate_corrections = cnt[kCounterCandidateVotes];
    s.classifier_timeouts = cnt[kCounterTimeouts];
    *out = s;
    return CG_OK;
}

int cg_get_read_info(const cg_ctx* c, uint64_t* num_reads, int32_t* max_length) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (num_reads) *num_reads = c->built ? c->n : c->appended;
    if (max_length) *max_length = c->lmax;
    return CG_OK;
}

int cg_get_signatures(cg_ctx* c, uint64_t first, uint64_t n, uint64_t* out) {
    if (!c || !out) return CG_ERR_INVALID_ARGUMENT;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (first + n > c->n) return fail(c, CG_ERR_INVALID_ARGUMENT, "read range out of bounds");
    std::vector<uint64_t> col(n);
    for (int h = 0; h < c->nmaps; h++) {
        CG_CUDA(c, cudaMemcpy(col.data(), c->sig.as<unsigned long long>() + (uint64_t)h * c->n + first,
                              n * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < n; i++) out[i * c->nmaps + h] = col[i];
    }
    return CG_OK;
}

int cg_load_forest(cg_ctx* c, const void* data, size_t size, uint32_t max_trees) {
    if (!c || !data) return CG_ERR_INVALID_ARGUMENT;
    // reference file format: include/forest.hpp:38-55 (preorder nodes) and 141-162
    const uint8_t* d = static_cast<const uint8_t*>(data);
    size_t pos = 0;
    auto rd = [&](void* dst, size_t n) {
        if (pos + n > size) return false;
        std::memcpy(dst, d + pos, n);
        pos += n;
        return true;
    };
    uint64_t dl = 0;
    if (!rd(&dl, 8) || dl > 4096 || pos + dl > size) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: bad header");
    const std::string desc(reinterpret_cast<const char*>(d + pos), dl);
    pos += dl;
    if (desc != "13 extract_anchor_v3")
        return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: descriptor '%s' is not 13 extract_anchor_v3", desc.c_str());
    uint32_t nt = 0;
    if (!rd(&nt, 4) || nt == 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: no trees");
    nt = std::min(nt, max_trees == 0 ? nt : max_trees);
    std::vector<ForestNode> nodes;
    std::vector<uint32_t> offsets;
    for (uint32_t t = 0; t < nt; t++) {
        uint32_t reserve = 0;
        if (!rd(&reserve, 4)) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: truncated tree %u", t);
        const uint32_t base = (uint32_t)nodes.size();
        offsets.push_back(base);
        // iterative preorder: node, then lhs (leaf prob or subtree), then rhs
        std::vector<std::pair<uint32_t, int>> stack;
        auto readNode = [&](uint32_t& idx) {
            ForestNode n{};
            if (!rd(&n.att, 1) || !rd(&n.split, 8) || !rd(&n.flag, 1) || n.att >= 13 || n.flag > 3) return false;
            nodes.push_back(n);
            idx = (uint32_t)nodes.size() - 1 - base;
            return true;
        };
        uint32_t root;
        if (!readNode(root)) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: bad node in tree %u", t);
        stack.push_back({root, 0});
        while (!stack.empty()) {
            auto& top = stack.back();
            if (top.second == 2) {
                stack.pop_back();
                continue;
            }
            const uint32_t cur = top.first;
            const int side = top.second++;
            const bool leaf = side == 0 ? (nodes[base + cur].flag & 2u) : (nodes[base + cur].flag & 1u);
            if (leaf) {
                uint32_t bits;
                if (!rd(&bits, 4)) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: truncated leaf");
                (side == 0 ? nodes[base + cur].lhs : nodes[base + cur].rhs) = bits;
            } else {
                uint32_t child;
                if (!readNode(child)) return fail(c, CG_ERR_INVALID_ARGUMENT, "forest: bad node in tree %u", t);
                (side == 0 ? nodes[base + cur].lhs : nodes[base + cur].rhs) = child;
                stack.push_back({child, 0});
            }
        }
    }
    CG_CUDA(c, cudaSetDevice(c->device));
    CG_CUDA(c, c->forestNodes.ensure(nodes.size() * sizeof(ForestNode)));
    CG_CUDA(c, c->treeOffsets.ensure(offsets.size() * sizeof(uint32_t)));
    CG_CUDA(c, cudaMemcpy(c->forestNodes.p, nodes.data(), nodes.size() * sizeof(ForestNode), cudaMemcpyHostToDevice));
    CG_CUDA(c, cudaMemcpy(c->treeOffsets.p, offsets.data(), offsets.size() * sizeof(uint32_t),
                          cudaMemcpyHostToDevice));
    c->numTrees = (int)nt;
    if (c->built) make_params(c);
    return CG_OK;
}

int cg_load_classifier(cg_ctx* c, const void* data, size_t size) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    std::vector<unsigned char> blob;
    if (!cg_parse_classifier(data, size, &blob))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "not a classifier of %zu bytes with a 32-64-64-1 layout",
                    cg_classifier_size());
    CG_CUDA(c, cudaSetDevice(c->device));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    CG_CUDA(c, c->mlp.ensure(kMlpBytes));
    CG_CUDA(c, cudaMemcpy(c->mlp.p, blob.data(), kMlpBytes, cudaMemcpyHostToDevice));
    c->haveMlp = true;
    return CG_OK;
}

int cg_get_columns(cg_ctx* c, uint64_t first, uint64_t num, float* features, uint64_t* anchors, uint16_t* positions,
                   char* consensus, uint64_t capacity, uint64_t* count) {
    if (!c || !count) return CG_ERR_INVALID_ARGUMENT;
    *count = 0;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (c->o.correction_type != CG_CORR_LEARNED)
        return fail(c, CG_ERR_STATE, "columns are recorded only with correction_type CG_CORR_LEARNED");
    if (c->lmax > 256)
        return fail(c, CG_ERR_UNSUPPORTED, "learned correction supports reads up to 256 bp (longest is %d)", c->lmax);
    if (first + num > c->n || first + num < first) return fail(c, CG_ERR_INVALID_ARGUMENT, "anchor range out of bounds");
    if (capacity && (!features || !anchors || !positions || !consensus))
        return fail(c, CG_ERR_INVALID_ARGUMENT, "output arrays missing");
    if (c->params.paired && ((first | num) & 1)) return fail(c, CG_ERR_INVALID_ARGUMENT, "paired mode needs even ranges");
    CG_CUDA(c, cudaSetDevice(c->device));
    int B = c->o.batch_anchors > 0 ? c->o.batch_anchors : 65536;
    if (c->params.paired && (B & 1)) B++;
    std::vector<uint8_t> hFlags(B);
    std::vector<char> hOut((size_t)B * std::max(c->lmax, 1));
    std::vector<uint16_t> hf;
    std::vector<uint2> hm;
    uint64_t total = 0;
    c->collecting = true;
    // no candidate votes: this is not a correction pass
    const int cand = c->params.candidates;
    c->params.candidates = 0;
    int rc = CG_OK;
    for (uint64_t a = 0; a < num && rc == CG_OK; a += (uint64_t)B) {
        const int cnt = (int)std::min<uint64_t>((uint64_t)B, num - a);
        rc = run_batch(c, first + a, cnt, hFlags.data(), hOut.data(), (size_t)std::max(c->lmax, 1));
        if (rc != CG_OK) break;
        unsigned int k = 0;
        if (cudaMemcpy(&k, c->colCount.p, sizeof(k), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(c, CG_ERR_CUDA, "reading the column count failed");
            break;
        }
        const uint64_t cap = (uint64_t)cnt * kColumnsPerAnchor;
        if (k > cap) {
            rc = fail(c, CG_ERR_UNSUPPORTED, "batch at anchor %llu has %u columns, more than the %llu recorded",
                      (unsigned long long)(first + a), k, (unsigned long long)cap);
            break;
        }
        if (total + k > capacity) {
            total += k;
            continue;  // keep counting
        }
        hf.resize((size_t)k * kLearnedFeatures);
        hm.resize(k);
        if (k && (cudaMemcpy(hf.data(), c->colFeat.p, hf.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost) !=
                      cudaSuccess ||
                  cudaMemcpy(hm.data(), c->colMeta.p, k * sizeof(uint2), cudaMemcpyDeviceToHost) != cudaSuccess)) {
            rc = fail(c, CG_ERR_CUDA, "reading the columns failed");
            break;
        }
        for (uint64_t i = 0; i < k; i++) {
            for (int f = 0; f < kLearnedFeatures; f++) {
                const uint32_t u = (uint32_t)hf[i * kLearnedFeatures + f] << 16;
                std::memcpy(&features[(total + i) * kLearnedFeatures + f], &u, 4);
            }
            anchors[total + i] = first + a + hm[i].x;
            positions[total + i] = (uint16_t)(hm[i].y & 0xffffu);
            consensus[total + i] = (char)((hm[i].y >> 16) & 0xffu);
        }
        total += k;
    }
    c->collecting = false;
    c->params.candidates = cand;
    if (rc != CG_OK) return rc;
    *count = total;
    if (total > capacity)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "%llu columns, capacity %llu", (unsigned long long)total,
                    (unsigned long long)capacity);
    return CG_OK;
}

int cg_get_candidates(cg_ctx* c, uint64_t anchor, uint32_t* out, uint32_t capacity, uint32_t* count) {
    if (!c || !count) return CG_ERR_INVALID_ARGUMENT;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (anchor >= c->n) return fail(c, CG_ERR_INVALID_ARGUMENT, "anchor out of bounds");
    CG_CUDA(c, cudaSetDevice(c->device));
    int rc = run_candidates(c, anchor, 1);
    if (rc != CG_OK) return rc;
    uint32_t nc = 0;
    CG_CUDA(c, cudaMemcpyAsync(&nc, c->ncand.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    *count = nc;
    const uint32_t w = std::min(nc, capacity);
    if (w && out) CG_CUDA(c, cudaMemcpy(out, c->cand.p, w * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return CG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- no-allocation candidate lookup
//
// cg_get_candidates_noalloc: the candidate ids of one anchor, like
// cg_get_candidates, for callers that cannot allocate device memory -- a host
// application that hands its whole device-memory budget to its own pool, or
// one that looks up single reads in a latency-sensitive loop and must not pay
// the device-wide synchronisation that cudaMalloc/cudaFree can imply.  The call
// allocates nothing: its scratch (the anchor's per-map bucket ranges, the raw
// hit count, the unique-id list and counters) is the file-scope device array
// below, which every GPU that loads this library holds until the process
// exits.  All calls share it and it keeps the last call's contents; the call
// clears what must start at zero itself.  Calls that overlap on the GPU race
// on it, so callers must not run two of them at once on any device.
namespace {

constexpr uint32_t kNoallocMaxRaw = 8192;  // raw bucket hits per anchor the scratch holds
constexpr size_t kNoallocQrange = 0;       // uint2[kMaxMaps]
constexpr size_t kNoallocRaw = 512;        // uint32_t[4]: raw count, scanned total, batch maximum
constexpr size_t kNoallocNcand = 576;      // uint32_t
constexpr size_t kNoallocCounters = 640;   // unsigned long long[kNumCounters]
constexpr size_t kNoallocCand = 1024;      // uint32_t[kNoallocMaxRaw]
constexpr size_t kNoallocBytes = kNoallocCand + sizeof(uint32_t) * kNoallocMaxRaw;
static_assert(kNoallocQrange + sizeof(uint2) * CG_MAX_HASHMAPS <= kNoallocRaw, "scratch layout: bucket ranges");
static_assert(kNoallocRaw + 4 * sizeof(uint32_t) <= kNoallocNcand, "scratch layout: raw counts");
static_assert(kNoallocNcand + sizeof(uint32_t) <= kNoallocCounters, "scratch layout: unique count");
static_assert(kNoallocCounters + sizeof(unsigned long long) * kNumCounters <= kNoallocCand, "scratch layout");

static __device__ __align__(256) unsigned char g_noallocScratch[kNoallocBytes];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noallocMutex;
unsigned char* g_noallocPtr[kNoallocMaxDevices] = {nullptr};

void forget_noalloc_scratch(int device) {
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    for (int d = 0; d < kNoallocMaxDevices; d++)
        if (device < 0 || d == device) g_noallocPtr[d] = nullptr;
}

// Device address of the scratch array on the current device (set up once per
// device; cg_release_cached_memory forgets it, as a device reset moves it).
int noalloc_scratch(cg_ctx* c, unsigned char** out) {
    int dev = 0;
    CG_CUDA(c, cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoallocMaxDevices) return fail(c, CG_ERR_UNSUPPORTED, "device ordinal %d too large", dev);
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocPtr[dev]) {
        void* p = nullptr;
        CG_CUDA(c, cudaGetSymbolAddress(&p, g_noallocScratch));
        g_noallocPtr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noallocPtr[dev];
    return CG_OK;
}

}  // namespace

extern "C" int cg_get_candidates_noalloc(cg_ctx* c, uint64_t anchor, uint32_t* out, uint32_t capacity,
                                         uint32_t* count) {
    if (!c || !count) return CG_ERR_INVALID_ARGUMENT;
    if (!c->built) return fail(c, CG_ERR_STATE, "cg_build_tables has not run");
    if (anchor >= c->n) return fail(c, CG_ERR_INVALID_ARGUMENT, "anchor out of bounds");
    CG_CUDA(c, cudaSetDevice(c->device));
    unsigned char* s = nullptr;
    const int rc = noalloc_scratch(c, &s);
    if (rc != CG_OK) return rc;
    BatchArg b{};
    b.first = anchor;
    b.count = 1;
    b.sig = c->sig.as<unsigned long long>();
    b.qrange = reinterpret_cast<uint2*>(s + kNoallocQrange);
    b.rawCount = reinterpret_cast<uint32_t*>(s + kNoallocRaw);
    b.ncand = reinterpret_cast<uint32_t*>(s + kNoallocNcand);
    b.counters = reinterpret_cast<unsigned long long*>(s + kNoallocCounters);
    b.cand = reinterpret_cast<uint32_t*>(s + kNoallocCand);
    const StoreArg st = store_arg(c);
    // the raw count slots and the batch maximum must start at zero
    CG_CUDA(c, cudaMemsetAsync(b.rawCount, 0, 4 * sizeof(uint32_t), c->stream));
    CG_CUDA(c, launch_query_count(st, c->tables, c->params, b, c->stream));
    CG_CUDA(c, scan_exclusive_u32(b.rawCount, 2, nullptr, c->stream));  // one tile: no scan scratch
    uint32_t raw[3] = {0, 0, 0};
    CG_CUDA(c, cudaMemcpyAsync(raw, b.rawCount, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (raw[1] > kNoallocMaxRaw)
        return fail(c, CG_ERR_INVALID_ARGUMENT,
                    "anchor %llu has %u raw bucket hits; cg_get_candidates_noalloc holds at most %u "
                    "(use cg_get_candidates)",
                    (unsigned long long)anchor, raw[1], kNoallocMaxRaw);
    CG_CUDA(c, launch_gather_unique(st, c->tables, c->params, b, (int)std::max<uint32_t>(raw[1], 1), c->stream));
    uint32_t nc = 0;
    CG_CUDA(c, cudaMemcpyAsync(&nc, b.ncand, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    *count = nc;
    const uint32_t w = std::min(nc, capacity);
    if (w && out) {
        CG_CUDA(c, cudaMemcpyAsync(out, b.cand, w * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        CG_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return CG_OK;
}

// ---------------------------------------------------------------- device file path hooks
namespace cg {

int append_device_chunk(cg_ctx* c, void* dChars, uint64_t* dOffs, void* dQual, uint64_t n, int lmax) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    if (c->built) return fail(c, CG_ERR_STATE, "reads cannot be appended after cg_build_tables");
    if (n == 0) return fail(c, CG_ERR_INVALID_ARGUMENT, "empty read batch");
    if (c->o.use_quality_scores && !dQual)
        return fail(c, CG_ERR_INVALID_ARGUMENT, "quality scores requested but not given");
    if (lmax > CG_MAX_READ_LENGTH) return fail(c, CG_ERR_UNSUPPORTED, "reads longer than %d", CG_MAX_READ_LENGTH);
    if (c->appended + n > 0xffffffffull) return fail(c, CG_ERR_UNSUPPORTED, "more than 2^32-1 reads");
    c->chunks.emplace_back();
    cg_ctx::Chunk& ch = c->chunks.back();
    ch.first = c->appended;
    ch.reads = n;
    ch.chars.p = dChars;  // the chunk owns the buffers from here on (freed after the build)
    ch.chars.bytes = 1;
    ch.chars.cached = false;
    ch.offs.p = dOffs;
    ch.offs.bytes = (n + 1) * sizeof(uint64_t);
    ch.offs.cached = false;
    if (c->o.use_quality_scores) {
        ch.qual.p = dQual;
        ch.qual.bytes = 1;
        ch.qual.cached = false;
    } else if (dQual) {
        cudaFree(dQual);
    }
    c->appended += n;
    c->appendLmax = std::max(c->appendLmax, lmax);
    return CG_OK;
}

int combine_into_device(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* dFlags, uint64_t* records) {
    if (!c || !c->params.candidates) return CG_ERR_STATE;
    CG_CUDA(c, c->combineCount.ensure(sizeof(unsigned long long)));
    CG_CUDA(c, cudaMemsetAsync(c->combineCount.p, 0, sizeof(unsigned long long), c->stream));
    CG_CUDA(c, launch_combine(store_arg(c), c->params, first, num, dFlags, c->combineCount.as<unsigned long long>(),
                              c->stream));
    c->stats.kernel_launches += 1;
    unsigned long long n = 0;
    CG_CUDA(c, cudaMemcpyAsync(&n, c->combineCount.p, sizeof(n), cudaMemcpyDeviceToHost, c->stream));
    CG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (records) *records = n;
    return CG_OK;
}

int correct_into_device(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* dFlags, char* dSeq, size_t pitch) {
    if (!c) return CG_ERR_INVALID_ARGUMENT;
    c->outKind = cudaMemcpyDeviceToDevice;
    const int rc = cg_correct(c, first, num, dFlags, dSeq, pitch);
    c->outKind = cudaMemcpyDeviceToHost;
    return rc;
}

}  // namespace cg
