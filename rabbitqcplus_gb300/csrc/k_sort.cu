// Stable LSD radix sort of (64-bit key, 32-bit value) pairs, for the minhash
// tables' build: one map's (key, read id) pairs sorted by key with the read
// ids ascending within a key, so that every bucket comes out in the order the
// reference's group-by-key gives it (include/groupbykey.hpp:69-250).
//
// Per 8-bit digit, three launches: (1) the digit counts of every tile of
// 2048 elements, (2) an exclusive scan of the counts in (digit, tile) order,
// (3) a scatter.  The scatter ranks each element among the tile's elements
// of the same digit in element order -- warps take contiguous sub-tiles,
// lanes with equal digits find each other with a warp match, each warp keeps
// its digit counts in shared memory -- stages the tile in digit order in
// shared memory and writes it out, so consecutive threads store consecutive
// elements of a digit's run.

#include <algorithm>

#include "care_internal.h"

namespace cg {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kDigits = 256;
static_assert(kSortThreads == kDigits, "one thread per digit in the per-tile steps");

__device__ __forceinline__ uint32_t digit_of(unsigned long long k, int shift) {
    return (uint32_t)(k >> shift) & (kDigits - 1);
}

// counts[d * tiles + t] = elements of tile t whose digit is d
__global__ void __launch_bounds__(kSortThreads) radix_count_kernel(const unsigned long long* __restrict__ keys,
                                                                   uint64_t n, int shift, uint32_t* __restrict__ counts,
                                                                   uint32_t tiles) {
    __shared__ uint32_t h[kDigits];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        const uint64_t i = base + (uint64_t)(j * kSortThreads) + threadIdx.x;
        if (i < n) atomicAdd(&h[digit_of(keys[i], shift)], 1u);
    }
    __syncthreads();
    counts[(uint64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// One tile per block.  offsets = the exclusive scan of radix_count_kernel's
// counts; vals == nullptr stands for the values 0, 1, ..., n - 1, each with
// bit tagBit of tags[i] in bit 31 when tags is set.
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ vals, uint64_t n, int shift,
    const uint32_t* __restrict__ offsets, uint32_t tiles, unsigned long long* __restrict__ keysOut,
    uint32_t* __restrict__ valsOut, const uint16_t* __restrict__ tags, int tagBit) {
    __shared__ uint32_t wcount[kSortWarps][kDigits];  // per warp: digit counts, then the warp's start in the digit
    __shared__ uint32_t tileStart[kDigits];           // digit d's first position in the staged tile
    __shared__ uint32_t globalStart[kDigits];         // and in the output
    __shared__ uint32_t warpSum[kSortWarps];
    __shared__ unsigned long long skey[kSortTile];
    __shared__ uint32_t sval[kSortTile];
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    for (int i = threadIdx.x; i < kSortWarps * kDigits; i += kSortThreads) (&wcount[0][0])[i] = 0;
    __syncthreads();
    // warp w: elements tile + w * 32 * kSortItems + 32 j + lane, j = 0 .. kSortItems - 1
    // (element order = (warp, j, lane) order)
    const uint64_t tile0 = (uint64_t)blockIdx.x * kSortTile;
    const uint64_t base = tile0 + (uint64_t)warp * 32 * kSortItems;
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long k[kSortItems];
    uint32_t v[kSortItems], rank[kSortItems];
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        const uint64_t i = base + (uint64_t)(32 * j + lane);
        const bool valid = i < n;
        k[j] = valid ? keys[i] : 0ull;
        v[j] = valid ? (vals ? vals[i] : ((uint32_t)i | (tags ? ((uint32_t)(tags[i] >> tagBit) & 1u) << 31 : 0u)))
                     : 0u;
        rank[j] = 0;
        const unsigned act = __ballot_sync(kFull, valid);
        if (valid) {
            const uint32_t d = digit_of(k[j], shift);
            const unsigned peers = __match_any_sync(act, d);
            const uint32_t before = wcount[warp][d];
            rank[j] = before + (uint32_t)__popc(peers & lt);
            __syncwarp(act);
            if (lane == __ffs(peers) - 1) wcount[warp][d] = before + (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // thread d: the warps' starts within digit d, the digit's tile count, and
    // the exclusive scan of the tile counts over the digits
    const int d = (int)threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) {
        const uint32_t c = wcount[w][d];
        wcount[w][d] = run;
        run += c;
    }
    uint32_t incl = run;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, s);
        if (lane >= s) incl += y;
    }
    if (lane == 31) warpSum[warp] = incl;
    globalStart[d] = offsets[(uint64_t)d * tiles + blockIdx.x];
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; w++) before += warpSum[w];
    tileStart[d] = before + incl - run;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        if (base + (uint64_t)(32 * j + lane) < n) {
            const uint32_t dj = digit_of(k[j], shift);
            const uint32_t pos = tileStart[dj] + wcount[warp][dj] + rank[j];
            skey[pos] = k[j];
            sval[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t count = (uint32_t)min((uint64_t)kSortTile, n - tile0);
    for (uint32_t p = threadIdx.x; p < count; p += kSortThreads) {
        const unsigned long long key = skey[p];
        const uint32_t dp = digit_of(key, shift);
        const uint32_t dst = globalStart[dp] + (p - tileStart[dp]);
        keysOut[dst] = key;
        valsOut[dst] = sval[p];
    }
}

size_t align16(size_t b) { return (b + 15) / 16 * 16; }

}  // namespace

size_t radix_sort_temp_bytes(uint64_t n) {
    const uint64_t tiles = (n + kSortTile - 1) / kSortTile;
    const size_t counts = (size_t)kDigits * (size_t)std::max<uint64_t>(tiles, 1);
    return align16(counts * sizeof(uint32_t)) + scan_tmp_bytes(counts);
}

cudaError_t radix_sort_pairs(const unsigned long long* keysIn, uint64_t n, int bits, unsigned long long* keys,
                             uint32_t* vals, unsigned long long* keysAlt, uint32_t* valsAlt, void* temp,
                             cudaStream_t s, const uint16_t* tags, int tagBit) {
    if (n == 0) return cudaSuccess;
    if (n > 0xffffffffull || (tags && n > 0x7fffffffull)) return cudaErrorInvalidValue;
    const uint32_t tiles = (uint32_t)((n + kSortTile - 1) / kSortTile);
    const size_t ncounts = (size_t)kDigits * tiles;
    uint32_t* counts = static_cast<uint32_t*>(temp);
    void* scanTmp = static_cast<unsigned char*>(temp) + align16(ncounts * sizeof(uint32_t));
    const int passes = std::max(1, (std::min(bits, 64) + 7) / 8);
    const unsigned long long* ki = keysIn;
    const uint32_t* vi = nullptr;  // pass 0: the values are the element indices
    for (int p = 0; p < passes; p++) {
        // the last pass writes keys/vals
        const bool toMain = ((passes - 1 - p) & 1) == 0;
        unsigned long long* ko = toMain ? keys : keysAlt;
        uint32_t* vo = toMain ? vals : valsAlt;
        radix_count_kernel<<<tiles, kSortThreads, 0, s>>>(ki, n, 8 * p, counts, tiles);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = scan_exclusive_u32(counts, ncounts, scanTmp, s);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(ki, vi, n, 8 * p, counts, tiles, ko, vo, tags, tagBit);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ki = ko;
        vi = vo;
    }
    return cudaSuccess;
}

}  // namespace cg
