// Read store construction and minhash signatures.
//
// reference: include/chunkedreadstorageconstruction.hpp:29-485 (parse, N
// replacement, 2-bit encode), include/sequencehelpers.hpp:151-193 (encoding),
// :645-697 (hi/lo planes), include/cpusequencehasher.hpp:86-125 and
// include/sequencehelpers.hpp:842-930 (signatures over canonical k-mers).

#include "care_device.cuh"
#include "care_internal.h"

namespace cg {

// ---------------------------------------------------------------- scan
// Exclusive prefix sum, three phases: per-block scan + block totals, scan of
// the totals (recursively), add back.  4096 elements per block.

namespace {
constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

template <class T>
__global__ void scan_tile_kernel(T* __restrict__ data, size_t n, T* __restrict__ tileSums) {
    __shared__ T warpTot[kScanBlock / 32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T run = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        const T x = (base + i < n) ? data[base + i] : T(0);
        v[i] = run;
        run += x;
    }
    // inclusive warp scan of thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        T w = lane < kScanBlock / 32 ? warpTot[lane] : T(0);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < kScanBlock / 32) warpTot[lane] = w;  // inclusive
    }
    __syncthreads();
    const T warpPrefix = warp == 0 ? T(0) : warpTot[warp - 1];
    const T threadPrefix = warpPrefix + incl - run;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) data[base + i] = threadPrefix + v[i];
    }
    if (tileSums && threadIdx.x == kScanBlock - 1) tileSums[blockIdx.x] = warpTot[kScanBlock / 32 - 1];
}

template <class T>
__global__ void scan_add_kernel(T* __restrict__ data, size_t n, const T* __restrict__ tileSums) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += tileSums[i / kScanTile];
}

size_t tiles_of(size_t n) { return (n + kScanTile - 1) / kScanTile; }

template <class T>
cudaError_t scan_impl(T* data, size_t n, T* tmp, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const size_t tiles = tiles_of(n);
    if (tiles == 1) {
        scan_tile_kernel<T><<<1, kScanBlock, 0, s>>>(data, n, nullptr);
        return cudaGetLastError();
    }
    scan_tile_kernel<T><<<(unsigned)tiles, kScanBlock, 0, s>>>(data, n, tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_impl<T>(tmp, tiles, tmp + tiles, s);
    if (e != cudaSuccess) return e;
    scan_add_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data, n, tmp);
    return cudaGetLastError();
}
}  // namespace

size_t scan_tmp_bytes(size_t n) {
    size_t total = 0;
    while (n > 1) {
        n = tiles_of(n);
        total += n;
    }
    return (total + 16) * sizeof(unsigned long long);
}

uint64_t scan_launches(uint64_t n) {
    uint64_t k = 0;
    while (true) {
        const uint64_t tiles = tiles_of(n);
        if (tiles <= 1) return k + 1;
        k += 2;
        n = tiles;
    }
}

cudaError_t scan_exclusive_u32(uint32_t* data, size_t n, void* tmp, cudaStream_t s) {
    return scan_impl<uint32_t>(data, n, static_cast<uint32_t*>(tmp), s);
}
cudaError_t scan_exclusive_u64(unsigned long long* data, size_t n, void* tmp, cudaStream_t s) {
    return scan_impl<unsigned long long>(data, n, static_cast<unsigned long long*>(tmp), s);
}

// ---------------------------------------------------------------- encode

namespace {

__device__ __forceinline__ char upcase_acgt(char c) {
    switch (c) {
        case 'a': return 'A';
        case 'c': return 'C';
        case 'g': return 'G';
        case 't': return 'T';
        default: return c;
    }
}
__device__ __forceinline__ int code_of(char c) {  // -1 for a non-ACGT character
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

__global__ void rebase_kernel(uint64_t* __restrict__ offs, uint64_t count, uint64_t base) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) offs[i] -= base;
}

// one warp per read: number of characters outside ACGTacgt
__global__ void count_invalid_kernel(const char* __restrict__ chars, const uint64_t* __restrict__ offs, uint64_t n,
                                     uint32_t* __restrict__ invalid) {
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    const uint32_t lane = lane_id();
    const uint64_t b = offs[r], L = offs[r + 1] - b;
    uint32_t cnt = 0;
    for (uint64_t c = lane; c < L; c += 32) cnt += code_of(upcase_acgt(chars[b + c])) < 0;
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0) invalid[r] = cnt;
}

// One warp per read.  Non-ACGT characters become A,C,G,T in turn; the turn
// counter starts at 0 at every multiple of 65536 reads of this call, as the
// reference's encoder threads restart it per parsed batch
// (include/chunkedreadstorageconstruction.hpp:243-282).  `invalidScan` is the
// exclusive scan of per-read invalid counts of this call (mod 2^32, which keeps
// the count mod 4).
__global__ void encode_kernel(const char* __restrict__ chars, const uint64_t* __restrict__ offs,
                              const char* __restrict__ quals, uint64_t n, uint64_t firstId,
                              const uint32_t* __restrict__ invalidScan, uint32_t* __restrict__ enc,
                              uint16_t* __restrict__ len, uint8_t* __restrict__ qual, uint8_t* __restrict__ ambig,
                              int pitch, int lmax) {
    const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    const uint32_t lane = lane_id();
    const uint64_t b = offs[r];
    const int L = (int)(offs[r + 1] - b);
    const uint64_t seg = (r / kSegmentReads) * kSegmentReads;
    uint32_t ctr = invalidScan[r] - invalidScan[seg];
    const uint32_t ctr0 = ctr;
    const uint64_t id = firstId + r;
    uint32_t* row = enc + id * (uint64_t)pitch;
    for (int c = 0; c < L; c += 32) {
        const int p = c + (int)lane;
        const bool in = p < L;
        const int code0 = in ? code_of(upcase_acgt(chars[b + p])) : 0;
        const bool inval = in && code0 < 0;
        const uint32_t m = __ballot_sync(0xffffffffu, inval);
        const uint32_t rank = __popc(m & ((1u << lane) - 1u));
        const uint32_t code = inval ? ((ctr + rank) & 3u) : (uint32_t)code0;
        ctr += __popc(m);
        uint32_t v = in ? code << (30 - 2 * (lane & 15)) : 0u;
        v |= __shfl_xor_sync(0xffffffffu, v, 1);
        v |= __shfl_xor_sync(0xffffffffu, v, 2);
        v |= __shfl_xor_sync(0xffffffffu, v, 4);
        v |= __shfl_xor_sync(0xffffffffu, v, 8);
        const int word = (c >> 4) + (lane >> 4);
        if ((lane & 15) == 0 && word * 16 < L) row[word] = v;
        if (quals && in) qual[id * (uint64_t)lmax + p] = (uint8_t)quals[b + p];
    }
    if (lane == 0) {
        len[id] = (uint16_t)L;
        ambig[id] = ctr != ctr0;
    }
}

// one thread per read and orientation: hi/lo bit planes, 32 bases per word
__global__ void hilo_kernel(StoreArg st, uint32_t* __restrict__ hilo) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t r = t >> 1;
    const int rc = (int)(t & 1);
    if (r >= st.n) return;
    const int L = st.len[r];
    const uint32_t* e = st.enc + r * (uint64_t)st.pitch;
    uint32_t* hi = hilo + (r * 2 + rc) * 2 * (uint64_t)st.wp;
    uint32_t* lo = hi + st.wp;
    for (int w = 0; w < st.wp; w++) {
        uint32_t h = 0, l = 0;
        for (int j = 0; j < 32; j++) {
            const int p = w * 32 + j;
            if (p < L) {
                const uint32_t bb = rc ? 3u - get2bit(e, L - 1 - p) : get2bit(e, p);
                h |= (bb >> 1) << (31 - j);
                l |= (bb & 1u) << (31 - j);
            }
        }
        hi[w] = h;
        lo[w] = l;
    }
}

// Signatures: one thread per (read, group of 16 maps); threads of a warp take
// consecutive reads of the same group so the map-major stores coalesce.
// With `strand`, bit q of strand[read] tells whether map q's minimum (maps
// 0-15 only) came from a k-mer whose canonical form is its reverse
// complement: two reads that share that minimum overlap in the same
// orientation when their bits agree, which the alignment uses to choose which
// orientation to scan first (a prediction only: the result does not depend on
// it).  The threads of the other maps skip the bookkeeping.
constexpr int kSigReads = 128;
constexpr int kSigGroup = 16;

__global__ void __launch_bounds__(kSigReads * 3) signature_kernel(StoreArg st, int k, int nmaps,
                                                                  unsigned long long* __restrict__ sig,
                                                                  uint16_t* __restrict__ strand) {
    const uint64_t r = (uint64_t)blockIdx.x * kSigReads + (threadIdx.x % kSigReads);
    const int g = threadIdx.x / kSigReads;
    const int m0 = g * kSigGroup;
    if (r >= st.n || m0 >= nmaps) return;
    const uint64_t kmask = k == 32 ? ~0ull : ((1ull << (2 * k)) - 1ull);
    uint64_t mins[kSigGroup];
#pragma unroll
    for (int j = 0; j < kSigGroup; j++) mins[j] = ~0ull;
    uint32_t sb = 0;  // strand bit of each map's minimum
    const bool track = strand && g == 0;
    const int L = st.len[r];
    if (L >= k) {
        const uint32_t* e = st.enc + r * (uint64_t)st.pitch;
        uint64_t fwd = 0, rc = 0;
        const int rcShift = 2 * (k - 1);
        for (int w = 0; w * 16 < L; w++) {
            const uint32_t word = e[w];
            const int lim = min(16, L - w * 16);
            for (int j = 0; j < lim; j++) {
                const uint64_t bb = (word >> (30 - 2 * j)) & 3u;
                fwd = ((fwd << 2) | bb) & kmask;
                rc = (rc >> 2) | ((3ull - bb) << rcShift);
                if (w * 16 + j >= k - 1) {
                    const uint64_t canon = fwd < rc ? fwd : rc;
                    if (track) {  // the same for every thread of a warp
                        const uint32_t rcBits = rc < fwd ? 0xffffu : 0u;
#pragma unroll
                        for (int q = 0; q < kSigGroup; q++) {
                            const uint64_t hv = murmur64(canon + (uint64_t)(m0 + q));
                            const bool lower = hv < mins[q];
                            mins[q] = lower ? hv : mins[q];
                            const uint32_t m = lower ? 1u << q : 0u;  // bit q takes this k-mer's strand
                            sb = (sb & ~m) | (rcBits & m);
                        }
                    } else {
#pragma unroll
                        for (int q = 0; q < kSigGroup; q++) {
                            const uint64_t hv = murmur64(canon + (uint64_t)(m0 + q));
                            mins[q] = hv < mins[q] ? hv : mins[q];
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kSigGroup; q++) {
        if (m0 + q < nmaps) sig[(uint64_t)(m0 + q) * st.n + r] = mins[q] & kmask;
    }
    if (track) strand[r] = (uint16_t)sb;
}

}  // namespace

cudaError_t launch_rebase_offsets(uint64_t* offs, uint64_t count, uint64_t base, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    rebase_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(offs, count, base);
    return cudaGetLastError();
}

cudaError_t launch_count_invalid(const char* chars, const uint64_t* offs, uint64_t n, uint32_t* invalid,
                                 cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t threads = n * 32;
    count_invalid_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(chars, offs, n, invalid);
    return cudaGetLastError();
}

cudaError_t launch_encode(const char* chars, const uint64_t* offs, const char* quals, uint64_t n, uint64_t firstId,
                          const uint32_t* invalidScan, const uint64_t* /*segStart*/, uint32_t* enc, uint16_t* len,
                          uint8_t* qual, uint8_t* ambig, int pitch, int lmax, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t threads = n * 32;
    encode_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(chars, offs, quals, n, firstId, invalidScan, enc,
                                                                    len, qual, ambig, pitch, lmax);
    return cudaGetLastError();
}

cudaError_t launch_hilo(StoreArg st, uint32_t* hilo, cudaStream_t s) {
    const uint64_t threads = st.n * 2;
    hilo_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(st, hilo);
    return cudaGetLastError();
}

namespace {
__global__ void len_range_kernel(const uint16_t* __restrict__ len, uint64_t n, unsigned int* out) {
    unsigned int lo = 0xffffffffu, hi = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        lo = min(lo, (unsigned int)len[i]);
        hi = max(hi, (unsigned int)len[i]);
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&out[0], lo);
        atomicMax(&out[1], hi);
    }
}
}  // namespace

namespace {
// Lossy quality store (qualityScoreBits 1 or 2): the binned score of every
// base, and the first bin's score past the read's end, where the reference's
// zero-filled encoded row decodes to bin 0 (include/qualityscorecompression.hpp:
// 25-140; scores are read as signed chars, as the reference's `int(quality[p])`
// on x86-64).  Four bytes per thread, rows of lmax bytes.
__global__ void quality_bin_kernel(uint8_t* __restrict__ qual, const uint16_t* __restrict__ len, uint64_t n,
                                   int lmax, int bits) {
    const uint64_t total = n * (uint64_t)lmax;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / (uint64_t)lmax;
        const int p = (int)(i - r * (uint64_t)lmax);
        const int q = (int)(int8_t)qual[i] - 33;
        uint8_t b;
        if (bits == 1) {
            b = (p >= len[r] || q <= 13) ? '(' : '5';
        } else {
            b = (p >= len[r] || q <= 4) ? '$' : q <= 13 ? '(' : q <= 20 ? '1' : '9';
        }
        qual[i] = b;
    }
}
}  // namespace

cudaError_t launch_quality_bins(uint8_t* qual, const uint16_t* len, uint64_t n, int lmax, int bits, cudaStream_t s) {
    if (n == 0 || (bits != 1 && bits != 2)) return cudaSuccess;
    const uint64_t total = n * (uint64_t)lmax;
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 152 * 16);
    quality_bin_kernel<<<blocks, 256, 0, s>>>(qual, len, n, lmax, bits);
    return cudaGetLastError();
}

cudaError_t launch_len_range(const uint16_t* len, uint64_t n, unsigned int* out, cudaStream_t s) {
    len_range_kernel<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 1216), 256, 0, s>>>(len, n, out);
    return cudaGetLastError();
}

cudaError_t launch_signatures(StoreArg st, int k, int nmaps, unsigned long long* sig, uint16_t* strand,
                              cudaStream_t s) {
    const unsigned blocks = (unsigned)((st.n + kSigReads - 1) / kSigReads);
    signature_kernel<<<blocks, kSigReads * 3, 0, s>>>(st, k, nmaps, sig, strand);
    return cudaGetLastError();
}

}  // namespace cg
