// File-to-file correction with the FASTQ parsing (STEP1) and the output
// records (STEP3) on the device; see care_files.h.
//
// Input: each file is copied to the device once.  A newline index is built
// by counting '\n' per 64 KiB block, scanning the counts and writing every
// newline's offset in order; record r of a plain FASTQ file is then lines
// 4r..4r+3, checked for the layout the host reader would parse the same way
// ('@' header, a sequence line not starting with '+', a '+' line, a quality
// line of the sequence's length, no '\r').  The sequences (and qualities) of
// each group of reads are gathered into one device chunk and handed to the
// context without visiting host memory.
//
// Output: after the correction (results kept in device memory), one thread
// per read applies the record rules of the host layer (reads with a non-ACGT
// base take the corrected sequence whole; others take the corrected bases as
// edits when at most length/7 positions change, else whole; a high-quality
// read without edits has no record), sizes its FASTQ record, a scan gives the
// record offsets of each output file, and one warp per read writes its record.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "care_capi_internal.h"
#include "care_files.h"
#include "care_gpu.h"
#include "care_internal.h"

namespace cg {

namespace {

constexpr int kIdxThreads = 256;
constexpr int kIdxBytes = 256;  // bytes per thread (16 x 16-byte loads)
constexpr uint64_t kIdxBlockBytes = (uint64_t)kIdxThreads * kIdxBytes;

enum : unsigned { kBadCR = 1u, kBadLayout = 2u, kBadLength = 4u };

// '\n' count of the thread's 256 bytes (and whether a '\r' occurs)
__device__ __forceinline__ uint32_t count_segment(const unsigned char* __restrict__ data, uint64_t size, uint64_t b0,
                                                  bool& cr) {
    uint32_t c = 0;
    if (b0 + kIdxBytes <= size) {
        const uint4* v = reinterpret_cast<const uint4*>(data + b0);
#pragma unroll 4
        for (int k = 0; k < kIdxBytes / 16; k++) {
            const uint4 x = v[k];
            const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                c += __popc(__vcmpeq4(w[j], 0x0a0a0a0au)) >> 3;
                cr |= __vcmpeq4(w[j], 0x0d0d0d0du) != 0u;
            }
        }
    } else {
        for (uint64_t i = b0; i < size; i++) {
            c += data[i] == '\n';
            cr |= data[i] == '\r';
        }
    }
    return c;
}

__global__ void __launch_bounds__(kIdxThreads) nl_count_kernel(const unsigned char* __restrict__ data, uint64_t size,
                                                               unsigned long long* __restrict__ counts,
                                                               unsigned int* bad) {
    __shared__ uint32_t ws[kIdxThreads / 32];
    const uint64_t b0 = (uint64_t)blockIdx.x * kIdxBlockBytes + (uint64_t)threadIdx.x * kIdxBytes;
    bool cr = false;
    const uint32_t c = __reduce_add_sync(0xffffffffu, count_segment(data, size, b0, cr));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    if (__syncthreads_or(cr) && threadIdx.x == 0) atomicOr(bad, kBadCR);
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kIdxThreads / 32; w++) t += ws[w];
        counts[blockIdx.x] = t;
    }
}

// every newline's byte offset, in file order (blockBase: exclusive scan of the counts)
__global__ void __launch_bounds__(kIdxThreads) nl_write_kernel(const unsigned char* __restrict__ data, uint64_t size,
                                                               const unsigned long long* __restrict__ blockBase,
                                                               unsigned long long* __restrict__ nl) {
    __shared__ uint32_t ws[kIdxThreads / 32];
    const uint64_t b0 = (uint64_t)blockIdx.x * kIdxBlockBytes + (uint64_t)threadIdx.x * kIdxBytes;
    bool cr = false;
    const uint32_t c = count_segment(data, size, b0, cr);
    // exclusive prefix of the counts over the block's threads
    const uint32_t lane = threadIdx.x & 31;
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += o;
    }
    if (lane == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    uint32_t warpBase = 0;
    for (uint32_t w = 0; w < (threadIdx.x >> 5); w++) warpBase += ws[w];
    unsigned long long pos = blockBase[blockIdx.x] + warpBase + incl - c;
    const uint64_t e = b0 + kIdxBytes < size ? b0 + kIdxBytes : size;
    for (uint64_t i = b0; i < e; i++)
        if (data[i] == '\n') nl[pos++] = i;
}

struct ReadIdx {
    const char* hdr;   // header without the '@'
    const char* seq;
    const char* qual;
    uint32_t hdrLen, seqLen;
};
static_assert(sizeof(ReadIdx) == 32, "read index layout");

// Record r = lines 4r..4r+3 of one file -> read dst0 + r * stride.
__global__ void records_kernel(const char* __restrict__ data, const unsigned long long* __restrict__ nl, uint64_t nrec,
                               uint64_t dst0, uint32_t stride, uint8_t outFile, ReadIdx* __restrict__ reads,
                               uint8_t* __restrict__ readOut, unsigned int* bad, unsigned int* maxLen) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const uint64_t hs = r == 0 ? 0 : nl[4 * r - 1] + 1, he = nl[4 * r];
    const uint64_t ss = he + 1, se = nl[4 * r + 1];
    const uint64_t ps = se + 1, pe = nl[4 * r + 2];
    const uint64_t qs = pe + 1, qe = nl[4 * r + 3];
    bool ok = he > hs && data[hs] == '@' && pe > ps && data[ps] == '+' && qe - qs == se - ss;
    if (ok && se > ss && data[ss] == '+') ok = false;  // the host reader would take it for the '+' line
    if (!ok) {
        atomicOr(bad, kBadLayout);
        return;
    }
    const uint64_t len = se - ss;
    if (len > CG_MAX_READ_LENGTH) {
        atomicOr(bad, kBadLength);
        return;
    }
    const uint64_t i = dst0 + r * stride;
    ReadIdx x;
    x.hdr = data + hs + 1;
    x.seq = data + ss;
    x.qual = data + qs;
    x.hdrLen = (uint32_t)(he - hs - 1);
    x.seqLen = (uint32_t)len;
    reads[i] = x;
    readOut[i] = outFile;
    atomicMax(maxLen, (unsigned int)len);
}

__global__ void lengths_kernel(const ReadIdx* __restrict__ reads, uint64_t n, unsigned long long* __restrict__ off) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) off[i] = i < n ? reads[i].seqLen : 0ull;
}

// one warp per read: bases (and qualities) back to back at the scanned offsets
__global__ void gather_kernel(const ReadIdx* __restrict__ reads, uint64_t n, const unsigned long long* __restrict__ off,
                              char* __restrict__ chars, char* __restrict__ quals) {
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    const uint32_t lane = threadIdx.x & 31;
    const ReadIdx r = reads[i];
    char* d = chars + off[i];
    for (uint32_t p = lane; p < r.seqLen; p += 32) d[p] = r.seq[p];
    if (quals) {
        char* q = quals + off[i];
        for (uint32_t p = lane; p < r.seqLen; p += 32) q[p] = r.qual[p];
    }
}

__device__ __forceinline__ bool is_ambiguous(char ch) {
    return !(ch == 'A' || ch == 'C' || ch == 'G' || ch == 'T' || ch == 'a' || ch == 'c' || ch == 'g' || ch == 't');
}

__device__ __forceinline__ char upper_acgt(char ch) {
    return ch == 'a' ? 'A' : ch == 'c' ? 'C' : ch == 'g' ? 'G' : ch == 't' ? 'T' : ch;
}

constexpr int kLabelLen = 9;  // " care:q=N"

// Record rules per read: mode 0 original sequence, 1 corrected bases as
// edits, 2 corrected sequence whole; status = the quality label (0 none, 1 LQ
// anchor only, 2 LQ confirmed by candidates, 3 HQ); the size of the read's
// FASTQ record without the label.  *last = 1 + the index (base + i) of the
// last read with a correction record (anchor or candidate): the reference
// labels no read after it (src/correctionresultoutput.cpp:370-377, 896-901).
__global__ void plan_kernel(const ReadIdx* __restrict__ reads, uint64_t n, const uint8_t* __restrict__ flags,
                            const char* __restrict__ corr, int pitch, uint8_t* __restrict__ mode,
                            uint8_t* __restrict__ status, unsigned long long* __restrict__ size,
                            unsigned long long* records, unsigned int* last, uint64_t base) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t rec = 0, lastHere = 0;
    if (i < n) {
        const ReadIdx r = reads[i];
        const int len = (int)r.seqLen;
        uint8_t md = 0, st = 0;
        const uint8_t f = flags[i];
        if (f & CG_RESULT_CORRECTED) {
            const bool hq = (f & CG_RESULT_HQ) != 0;
            const char* c = corr + (uint64_t)i * pitch;
            bool amb = false;
            for (int p = 0; p < len && !amb; p++) amb = is_ambiguous(r.seq[p]);
            if (amb) {  // include/corrector.hpp:1651-1667: no edit list for reads with N
                md = 2;
                st = hq ? 3 : 1;
            } else {
                const int maxEdits = len / 7;
                int edits = 0;
                for (int p = 0; p < len && edits <= maxEdits; p++) edits += c[p] != upper_acgt(r.seq[p]);
                if (edits > maxEdits) {
                    md = 2;
                    st = hq ? 3 : 1;
                } else if (!(hq && edits == 0)) {  // src/correct_cpu.cpp:263-273 drops such records
                    md = 1;
                    st = hq ? 3 : 1;
                }
            }
        }
        rec = st != 0;
        // the combine step (candidate correction): a rejected LQ correction
        // keeps its record but writes the read unchanged
        if (f & CG_RESULT_REJECTED) {
            md = 0;
            st = 0;
        } else if (st == 1 && (f & CG_RESULT_CANDIDATES)) {
            st = 2;
        }
        mode[i] = md;
        status[i] = st;
        if (rec || (f & CG_RESULT_CANDIDATE_RECORD)) lastHere = (uint32_t)(base + i + 1);
        size[i] = 2ull * len + r.hdrLen + 6;
    }
    rec = __reduce_add_sync(0xffffffffu, rec);
    lastHere = __reduce_max_sync(0xffffffffu, lastHere);
    if ((threadIdx.x & 31) == 0 && rec) atomicAdd(records, (unsigned long long)rec);
    if ((threadIdx.x & 31) == 0 && lastHere) atomicMax(last, lastHere);
}

// labelled(k) = labels and read k is not after the last record
__device__ __forceinline__ bool labelled(int labels, uint64_t k, const unsigned int* last) {
    return labels && k < (uint64_t)*last;
}

__global__ void mask_kernel(const unsigned long long* __restrict__ size, const uint8_t* __restrict__ readOut,
                            uint64_t n, uint8_t f, int labels, const unsigned int* __restrict__ last, uint64_t base,
                            unsigned long long* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n)
        out[i] = i < n && readOut[i] == f ? size[i] + (labelled(labels, base + i, last) ? kLabelLen : 0) : 0ull;
}

// one warp per read of output f: "@header[ care:q=N]\nSEQ\n+\nQUAL\n"
__global__ void write_kernel(const ReadIdx* __restrict__ reads, uint64_t n, const uint8_t* __restrict__ readOut,
                             uint8_t f, const unsigned long long* __restrict__ pos, const uint8_t* __restrict__ mode,
                             const uint8_t* __restrict__ status, const char* __restrict__ corr, int pitch, int labels,
                             const unsigned int* __restrict__ last, uint64_t base, char* __restrict__ out) {
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n || readOut[i] != f) return;
    const uint32_t lane = threadIdx.x & 31;
    const ReadIdx r = reads[i];
    char* o = out + pos[i];
    const uint32_t hl = r.hdrLen, lab = labelled(labels, base + i, last) ? kLabelLen : 0;
    const char st = (char)('0' + status[i]);
    const char* label = " care:q=";  // src/correctionresultoutput.cpp:403-414
    for (uint32_t k = lane; k < hl + lab + 2; k += 32) {
        char ch;
        if (k == 0) ch = '@';
        else if (k <= hl) ch = r.hdr[k - 1];
        else if (k < hl + lab) ch = label[k - 1 - hl];
        else if (k == hl + lab) ch = st;
        else ch = '\n';
        o[k] = ch;
    }
    o += hl + lab + 2;
    const uint8_t md = mode[i];
    const char* c = corr + (uint64_t)i * pitch;
    const uint32_t len = r.seqLen;
    for (uint32_t p = lane; p < len; p += 32) {
        const char orig = r.seq[p];
        o[p] = md == 0 ? orig : md == 2 ? c[p] : (c[p] != upper_acgt(orig) ? c[p] : orig);
    }
    o += len;
    if (lane < 3) o[lane] = lane == 1 ? '+' : '\n';
    o += 3;
    for (uint32_t p = lane; p < len; p += 32) o[p] = r.qual[p];
    if (lane == 0) o[len] = '\n';
}

// device buffer freed on scope exit (unless released)
struct DMem {
    void* p = nullptr;
    DMem() = default;
    DMem(const DMem&) = delete;
    DMem& operator=(const DMem&) = delete;
    ~DMem() { free(); }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n < 16 ? 16 : n); }
    void* release() {
        void* q = p;
        p = nullptr;
        return q;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() {
        if (s) cudaStreamDestroy(s);
    }
};

struct Ctx {
    cg_ctx* c = nullptr;
    ~Ctx() {
        if (c) cg_destroy(c);
    }
};

int failf(std::string* error, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (error) *error = buf;
    return code;
}

#define DCHECK(call)                                                                                  \
    do {                                                                                              \
        const cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                      \
            cudaGetLastError();                                                                       \
            return failf(error, e_ == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA, \
                         "%s: %s", #call, cudaGetErrorString(e_));                                    \
        }                                                                                             \
    } while (0)

#define LCHECK(ctx, call)                                                                     \
    do {                                                                                      \
        const int rc_ = (call);                                                               \
        if (rc_ != CG_OK) return failf(error, rc_, "%s: %s", #call, cg_last_error((ctx)));   \
    } while (0)

unsigned grid_for(uint64_t threads, int block) { return (unsigned)((threads + block - 1) / block); }

}  // namespace

int correct_fastq_on_device(const cg_options& options, const std::vector<ByteSpan>& inputs,
                            bool paired, bool qualityLabels, int numOutputs, const std::vector<char>* forest,
                            uint32_t maxTrees, const std::vector<char>* classifier, FastqRun* run,
                            std::string* error) {
    if (!run || inputs.empty() || numOutputs < 1 || (paired && inputs.size() != 2))
        return failf(error, CG_ERR_INVALID_ARGUMENT, "bad arguments");
    DCHECK(cudaSetDevice(options.device));
    Stream st;
    DCHECK(cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking));
    const cudaStream_t s = st.s;
    const size_t nf = inputs.size();
    DMem flagsDev;  // bad-layout flags and the longest read
    DCHECK(flagsDev.alloc(2 * sizeof(unsigned int)));
    DCHECK(cudaMemsetAsync(flagsDev.p, 0, 2 * sizeof(unsigned int), s));
    unsigned int* bad = flagsDev.as<unsigned int>();
    unsigned int* maxLen = bad + 1;

    // ---- STEP1: files to the device, newline index, records
    std::vector<DMem> fileDev(nf), nlDev(nf);
    std::vector<uint64_t> recs(nf);
    for (size_t k = 0; k < nf; k++) {
        const ByteSpan f = inputs[k];
        const bool needNl = f.size == 0 || f.data[f.size - 1] != '\n';
        const uint64_t size = f.size + (needNl ? 1 : 0);
        DCHECK(fileDev[k].alloc(size));
        if (f.size) DCHECK(cudaMemcpyAsync(fileDev[k].p, f.data, f.size, cudaMemcpyHostToDevice, s));
        if (needNl) DCHECK(cudaMemsetAsync(fileDev[k].as<char>() + f.size, '\n', 1, s));
        const uint64_t blocks = (size + kIdxBlockBytes - 1) / kIdxBlockBytes;
        DMem counts, tmp;
        DCHECK(counts.alloc((blocks + 1) * sizeof(unsigned long long)));
        DCHECK(tmp.alloc(scan_tmp_bytes(blocks + 1)));
        DCHECK(cudaMemsetAsync(counts.as<unsigned long long>() + blocks, 0, sizeof(unsigned long long), s));
        nl_count_kernel<<<(unsigned)blocks, kIdxThreads, 0, s>>>(fileDev[k].as<unsigned char>(), size,
                                                                 counts.as<unsigned long long>(), bad);
        DCHECK(cudaGetLastError());
        DCHECK(scan_exclusive_u64(counts.as<unsigned long long>(), blocks + 1, tmp.p, s));
        unsigned long long lines = 0;
        unsigned int hbad = 0;
        DCHECK(cudaMemcpyAsync(&lines, counts.as<unsigned long long>() + blocks, sizeof(lines),
                               cudaMemcpyDeviceToHost, s));
        DCHECK(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, s));
        DCHECK(cudaStreamSynchronize(s));
        if (hbad || lines % 4 != 0) return failf(error, CG_ERR_UNSUPPORTED, "input %zu is not plain 4-line FASTQ", k);
        recs[k] = lines / 4;
        DCHECK(nlDev[k].alloc(lines * sizeof(unsigned long long)));
        nl_write_kernel<<<(unsigned)blocks, kIdxThreads, 0, s>>>(fileDev[k].as<unsigned char>(), size,
                                                                 counts.as<unsigned long long>(),
                                                                 nlDev[k].as<unsigned long long>());
        DCHECK(cudaGetLastError());
        DCHECK(cudaStreamSynchronize(s));  // counts/tmp go out of scope
    }
    uint64_t n = 0;
    std::vector<uint64_t> groupStart;  // first read of every group (one append call each)
    if (paired) {
        const uint64_t pairs = std::min(recs[0], recs[1]);
        n = 2 * pairs;
        groupStart.push_back(0);
    } else {
        for (size_t k = 0; k < nf; k++) {
            groupStart.push_back(n);
            n += recs[k];
        }
    }
    groupStart.push_back(n);
    if (n == 0) return failf(error, CG_ERR_INVALID_ARGUMENT, "input contains no reads");
    DMem readsDev, readOut;
    DCHECK(readsDev.alloc(n * sizeof(ReadIdx)));
    DCHECK(readOut.alloc(n));
    ReadIdx* reads = readsDev.as<ReadIdx>();
    for (size_t k = 0; k < nf; k++) {
        const uint64_t nrec = paired ? n / 2 : recs[k];
        if (nrec == 0) continue;
        const uint64_t dst0 = paired ? k : groupStart[k];
        const uint32_t stride = paired ? 2 : 1;
        const uint8_t out = (uint8_t)std::min<int>((int)k, numOutputs - 1);
        records_kernel<<<grid_for(nrec, 256), 256, 0, s>>>(fileDev[k].as<char>(), nlDev[k].as<unsigned long long>(),
                                                           nrec, dst0, stride, out, reads, readOut.as<uint8_t>(), bad,
                                                           maxLen);
        DCHECK(cudaGetLastError());
    }
    unsigned int hflags[2] = {0, 0};
    DCHECK(cudaMemcpyAsync(hflags, bad, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    DCHECK(cudaStreamSynchronize(s));
    if (hflags[0]) return failf(error, CG_ERR_UNSUPPORTED, "input is not plain 4-line FASTQ (flags %u)", hflags[0]);
    for (size_t k = 0; k < nf; k++) nlDev[k].free();  // the index is no longer needed
    const int lmax = std::max<int>((int)hflags[1], 1);

    // ---- the context: one device chunk per group, build, correction into device memory
    Ctx ctx;
    {
        const int rc = cg_create(&options, &ctx.c);
        if (rc != CG_OK) return failf(error, rc, "cg_create failed");
    }
    const bool quals = options.use_quality_scores != 0;
    for (size_t g = 0; g + 1 < groupStart.size(); g++) {
        const uint64_t g0 = groupStart[g], m = groupStart[g + 1] - g0;
        if (m == 0) continue;
        DMem off, tmp, chars, qual;
        DCHECK(off.alloc((m + 1) * sizeof(unsigned long long)));
        DCHECK(tmp.alloc(scan_tmp_bytes(m + 1)));
        lengths_kernel<<<grid_for(m + 1, 256), 256, 0, s>>>(reads + g0, m, off.as<unsigned long long>());
        DCHECK(cudaGetLastError());
        DCHECK(scan_exclusive_u64(off.as<unsigned long long>(), m + 1, tmp.p, s));
        unsigned long long bytes = 0;
        DCHECK(cudaMemcpyAsync(&bytes, off.as<unsigned long long>() + m, sizeof(bytes), cudaMemcpyDeviceToHost, s));
        DCHECK(cudaStreamSynchronize(s));
        DCHECK(chars.alloc(bytes));
        if (quals) DCHECK(qual.alloc(bytes));
        gather_kernel<<<grid_for(m * 32, 256), 256, 0, s>>>(reads + g0, m, off.as<unsigned long long>(),
                                                            chars.as<char>(), quals ? qual.as<char>() : nullptr);
        DCHECK(cudaGetLastError());
        DCHECK(cudaStreamSynchronize(s));
        const int rc = append_device_chunk(ctx.c, chars.p, off.as<uint64_t>(), quals ? qual.p : nullptr, m, lmax);
        if (rc != CG_OK) return failf(error, rc, "append_device_chunk: %s", cg_last_error(ctx.c));
        chars.release();  // owned by the context now
        off.release();
        if (quals) qual.release();
    }
    LCHECK(ctx.c, cg_build_tables(ctx.c));
    if (forest) LCHECK(ctx.c, cg_load_forest(ctx.c, forest->data(), forest->size(), maxTrees));
    if (classifier) LCHECK(ctx.c, cg_load_classifier(ctx.c, classifier->data(), classifier->size()));
    int32_t pitch = 0;
    uint64_t nr = 0;
    LCHECK(ctx.c, cg_get_read_info(ctx.c, &nr, &pitch));
    pitch = std::max(pitch, 1);
    DMem flagsOut, seqOut;
    DCHECK(flagsOut.alloc(n));
    DCHECK(seqOut.alloc(n * (uint64_t)pitch));

    // ---- STEP2 and STEP3 per range of reads (one range unless the caller
    // takes the output range by range): correction into device memory, then
    // the range's records of every output file
    DMem mode, status, size, recCount, lastRec, pos, tmp;
    DCHECK(mode.alloc(n));
    DCHECK(status.alloc(n));
    DCHECK(size.alloc(n * sizeof(unsigned long long)));
    DCHECK(recCount.alloc(sizeof(unsigned long long)));
    DCHECK(cudaMemsetAsync(recCount.p, 0, sizeof(unsigned long long), s));
    DCHECK(lastRec.alloc(sizeof(unsigned int)));
    DCHECK(cudaMemsetAsync(lastRec.p, 0, sizeof(unsigned int), s));
    DCHECK(pos.alloc((n + 1) * sizeof(unsigned long long)));
    DCHECK(tmp.alloc(scan_tmp_bytes(n + 1)));
    run->outputs.clear();
    run->outputs.resize((size_t)numOutputs);
    run->outputSizes.assign((size_t)numOutputs, 0);
    run->deviceOutputs.clear();
    run->deviceOutputs.resize((size_t)numOutputs);
    // One range when a read's output depends on reads after it: candidate
    // corrections come from any anchor, and the labels stop after the last
    // record of the whole run.
    const bool oneRange = !run->onChunk || qualityLabels || options.correct_candidates;
    const uint64_t range = oneRange ? n : std::max<uint64_t>(262144, (n / 4 + 1) & ~1ull);  // even
    uint64_t candRecords = 0;
    for (uint64_t r0 = 0; r0 < n; r0 += range) {
        const uint64_t m = std::min(range, n - r0);
        uint8_t* fl = flagsOut.as<uint8_t>() + r0;
        char* sq = seqOut.as<char>() + r0 * (uint64_t)pitch;
        LCHECK(ctx.c, correct_into_device(ctx.c, r0, m, fl, sq, (size_t)pitch));
        if (options.correct_candidates) LCHECK(ctx.c, combine_into_device(ctx.c, r0, m, fl, &candRecords));
        plan_kernel<<<grid_for(m, 256), 256, 0, s>>>(reads + r0, m, fl, sq, pitch, mode.as<uint8_t>() + r0,
                                                     status.as<uint8_t>() + r0, size.as<unsigned long long>() + r0,
                                                     recCount.as<unsigned long long>(),
                                                     lastRec.as<unsigned int>(), r0);
        DCHECK(cudaGetLastError());
        for (int f = 0; f < numOutputs; f++) {
            mask_kernel<<<grid_for(m + 1, 256), 256, 0, s>>>(size.as<unsigned long long>() + r0,
                                                             readOut.as<uint8_t>() + r0, m, (uint8_t)f,
                                                             qualityLabels ? 1 : 0, lastRec.as<unsigned int>(), r0,
                                                             pos.as<unsigned long long>());
            DCHECK(cudaGetLastError());
            DCHECK(scan_exclusive_u64(pos.as<unsigned long long>(), m + 1, tmp.p, s));
            unsigned long long total = 0;
            DCHECK(cudaMemcpyAsync(&total, pos.as<unsigned long long>() + m, sizeof(total), cudaMemcpyDeviceToHost,
                                   s));
            DCHECK(cudaStreamSynchronize(s));
            if (total == 0) continue;
            DMem outDev;
            DCHECK(outDev.alloc(total));
            write_kernel<<<grid_for(m * 32, 256), 256, 0, s>>>(reads + r0, m, readOut.as<uint8_t>() + r0, (uint8_t)f,
                                                               pos.as<unsigned long long>(), mode.as<uint8_t>() + r0,
                                                               status.as<uint8_t>() + r0, sq, pitch,
                                                               qualityLabels ? 1 : 0, lastRec.as<unsigned int>(), r0,
                                                               outDev.as<char>());
            DCHECK(cudaGetLastError());
            if (run->queueChunkBytes && !run->onChunk) {
                // queue chunks: cut at record ends, each chunk the longest run of
                // whole records under queueChunkBytes (src/correctionresultoutput.cpp:
                // 733-745); the bytes stay on the device until emit_queue_chunks
                std::vector<unsigned long long> ends(m + 1);
                DCHECK(cudaMemcpyAsync(ends.data(), pos.p, (m + 1) * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, s));
                DCHECK(cudaStreamSynchronize(s));
                const size_t cap = run->queueChunkBytes;
                auto& dout = run->deviceOutputs[(size_t)f];
                size_t begin = 0;
                for (uint64_t i = 0; i < m; i++) {
                    const size_t a = ends[i], b = ends[i + 1];
                    if (b == a) continue;  // a read of another output file
                    if (b - a >= cap) return failf(error, CG_ERR_INVALID_ARGUMENT, "record larger than a chunk");
                    if (b - begin >= cap) {
                        dout.chunks.emplace_back(begin, a);
                        begin = a;
                    }
                }
                dout.chunks.emplace_back(begin, (size_t)total);
                dout.bytes = outDev.release();
                continue;
            }
            std::unique_ptr<char[]> bytes(new char[total]);  // left uninitialised: the copy fills it
            DCHECK(cudaMemcpyAsync(bytes.get(), outDev.p, total, cudaMemcpyDeviceToHost, s));
            DCHECK(cudaStreamSynchronize(s));
            if (run->onChunk) {
                run->onChunk(f, std::move(bytes), total);
            } else {
                run->outputs[f] = std::move(bytes);
                run->outputSizes[f] = total;
            }
        }
    }
    LCHECK(ctx.c, cg_get_stats(ctx.c, &run->stats));
    unsigned long long records = 0;
    DCHECK(cudaMemcpyAsync(&records, recCount.p, sizeof(records), cudaMemcpyDeviceToHost, s));
    DCHECK(cudaStreamSynchronize(s));
    run->reads = n;
    run->records = records + candRecords;
    return CG_OK;
}

FastqRun::~FastqRun() {
    for (auto& d : deviceOutputs)
        if (d.bytes) cudaFree(d.bytes);
}

int emit_queue_chunks(FastqRun* run, const std::function<bool(int f, char* chunk, int size)>& sink,
                      std::string* error) {
    const size_t cap = run->queueChunkBytes;
    int rc = CG_OK;
    bool stop = false;
    for (size_t k = 0; !stop && rc == CG_OK; k++) {
        bool any = false;
        for (size_t f = 0; f < run->deviceOutputs.size() && !stop && rc == CG_OK; f++) {
            const auto& d = run->deviceOutputs[f];
            if (k >= d.chunks.size()) continue;
            any = true;
            const size_t b = d.chunks[k].first, e = d.chunks[k].second;
            char* chunk = new char[cap];
            const cudaError_t ce = cudaMemcpy(chunk, static_cast<const char*>(d.bytes) + b, e - b,
                                              cudaMemcpyDeviceToHost);
            if (ce != cudaSuccess) {
                delete[] chunk;
                rc = failf(error, CG_ERR_CUDA, "chunk copy: %s", cudaGetErrorString(ce));
            } else if (!sink((int)f, chunk, (int)(e - b))) {
                stop = true;  // the consumer is gone
            }
        }
        if (!any) break;
    }
    for (auto& d : run->deviceOutputs) {
        if (d.bytes) cudaFree(d.bytes);
        d.bytes = nullptr;
        d.chunks.clear();
    }
    return rc;
}

}  // namespace cg
