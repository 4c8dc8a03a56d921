// Minhash tables: build and query.
//
// reference: include/ordinaryminhasher.hpp:135-254,376-449 and
// include/groupbykey.hpp:69-250 (per map: group (key, readId) by key, read ids
// ascending, drop keys with fewer than 2 or more than maxValuesPerKey ids),
// include/corrector.hpp:571-650 (candidate ids: union of the anchor's buckets,
// sorted, unique, self removed, optionally ambiguous reads removed) and
// include/util.hpp:1005-1200 (pair flags of paired-end candidates).
//
// Build, per map: (1) sort the (key, read id) pairs by key, read ids
// ascending within a key (k_sort.cu), (2) find the runs of equal keys,
// (3) keep the keys with 2 to maxValuesPerKey ids and scan their lengths into
// value offsets, (4) copy each kept run's read ids into its bucket and place
// its key in a compact open-addressing table.  The bucket contents -- the only
// thing a query observes -- equal the reference's.

#include <algorithm>

#include "care_device.cuh"
#include "care_internal.h"

namespace cg {

namespace {

__global__ void table_init_kernel(Slot* __restrict__ t, uint64_t cap) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < cap) {
        t[s].key = kEmptyKey;
        t[s].offset = 0;
        t[s].count = 0;
    }
}

// ---------------------------------------------------------------- runs of sorted pairs
//
// keys/ids: one map's pairs sorted by key.  runOf[i] = 1 where element i
// starts a run (runOf[n] = 0); after an exclusive scan over n + 1 entries,
// runOf[i + 1] - 1 is element i's run and runOf[n] the number of runs R.
// start[r] = first element of run r, start[R] = n.

__device__ __forceinline__ bool run_kept(unsigned long long key, uint32_t len, int maxValues) {
    const uint32_t upper = (uint32_t)min(maxValues, kMaxBucket);
    return key != kEmptyKey && len >= 2u && len <= upper;
}

__global__ void run_head_kernel(const unsigned long long* __restrict__ keys, uint64_t n,
                                uint32_t* __restrict__ runOf) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    runOf[i] = (i < n && (i == 0 || keys[i] != keys[i - 1])) ? 1u : 0u;
}

__global__ void run_start_kernel(const unsigned long long* __restrict__ keys, uint64_t n,
                                 const uint32_t* __restrict__ runOf, uint32_t* __restrict__ start) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) start[runOf[n]] = (uint32_t)n;
    else if (i == 0 || keys[i] != keys[i - 1]) start[runOf[i]] = (uint32_t)i;
}

// packed[r] = (1 << 32) | length for a kept run, else 0; packed[R] = 0
__global__ void run_pack_kernel(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ start,
                                uint32_t runs, int maxValues, unsigned long long* __restrict__ packed) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r > runs) return;
    if (r == runs) {
        packed[r] = 0;
        return;
    }
    const uint32_t s0 = start[r], len = start[r + 1] - s0;
    packed[r] = run_kept(keys[s0], len, maxValues) ? ((1ull << 32) | len) : 0ull;
}

// packedScan = exclusive scan of run_pack_kernel's output: the read ids of
// every kept run, in order, at its value offset.  With rawAll set, each kept
// id also adds its run's length -- its bucket's size, the ids a query of that
// read finds in this map -- to rawAll[id & idMask] (atomic: the maps of a
// build wave run concurrently; idMask drops a strand tag in bit 31).
__global__ void run_values_kernel(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ ids,
                                  uint64_t n, const uint32_t* __restrict__ runOf, const uint32_t* __restrict__ start,
                                  const unsigned long long* __restrict__ packedScan, int maxValues,
                                  uint32_t* __restrict__ values, uint32_t* __restrict__ rawAll, uint32_t idMask) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = runOf[i + 1] - 1u;
    const uint32_t s0 = start[r], len = start[r + 1] - s0;
    if (!run_kept(keys[i], len, maxValues)) return;
    const uint32_t id = ids[i];
    values[(uint32_t)(packedScan[r] & 0xffffffffull) + ((uint32_t)i - s0)] = id;
    if (rawAll) atomicAdd(&rawAll[id & idMask], len);
}

// every kept run's key into the final table with its value offset and length
__global__ void run_place_kernel(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ start,
                                 uint32_t runs, const unsigned long long* __restrict__ packedScan, int maxValues,
                                 Slot* __restrict__ fin, uint32_t finMask) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= runs) return;
    const uint32_t s0 = start[r], len = start[r + 1] - s0;
    const unsigned long long key = keys[s0];
    if (!run_kept(key, len, maxValues)) return;
    uint32_t f = slot_of(key, finMask);
    for (uint32_t probe = 0; probe <= finMask; probe++) {
        const unsigned long long old = atomicCAS(&fin[f].key, kEmptyKey, key);
        if (old == kEmptyKey) {
            fin[f].offset = (uint32_t)(packedScan[r] & 0xffffffffull);
            fin[f].count = len;
            return;
        }
        f = (f + 1) & finMask;
    }
}

// ---------------------------------------------------------------- query

__device__ __forceinline__ uint2 lookup(const Slot* __restrict__ slots, uint32_t mask, unsigned long long key) {
    if (key == kEmptyKey) return make_uint2(0, 0);
    uint32_t s = slot_of(key, mask);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const Slot t = slots[s];
        if (t.key == key) return make_uint2(t.offset, t.count);
        if (t.key == kEmptyKey) return make_uint2(0, 0);
        s = (s + 1) & mask;
    }
    return make_uint2(0, 0);
}

// One warp per anchor: the anchor's bucket of every map.
__global__ void query_count_kernel(StoreArg st, TablesArg tb, Params p, BatchArg b) {
    const int a = (int)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (a >= b.count) return;
    const uint32_t lane = lane_id();
    const uint64_t aid = batch_first(b) + (uint64_t)a;
    const bool active = st.len[aid] >= p.k && !(p.excludeAmbiguous && st.ambig[aid]);
    uint32_t total = 0;
    for (int m = (int)lane; m < tb.nmaps; m += 32) {
        uint2 r = make_uint2(0, 0);
        if (active) {
            r = lookup(tb.slots[m], tb.mask[m], b.sig[(uint64_t)m * st.n + aid]);
            if ((int)r.y > tb.maxValuesPerKey) r = make_uint2(0, 0);
        }
        b.qrange[(uint64_t)a * tb.nmaps + m] = r;
        total += r.y;
    }
    total = __reduce_add_sync(0xffffffffu, total);
    if (lane == 0) {
        b.rawCount[a] = total;
        atomicMax(&b.rawCount[b.count + 1], total);  // batch maximum
    }
}

// The raw id count of every read as an anchor (the sum of
// query_count_kernel's bucket sizes), for the batched form's range offsets:
// the table build has summed every read's kept buckets into raw; a read that
// cannot be an anchor (shorter than k, or ambiguous and excluded) queries
// nothing.
__global__ void raw_count_kernel(StoreArg st, Params p, uint32_t* __restrict__ raw) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= st.n) return;
    if (st.len[i] < p.k || (p.excludeAmbiguous && st.ambig[i])) raw[i] = 0u;
}

// Raw counts of the anchors [first, first + num) widened to u64, with a zero
// after the last, ready for the exclusive scan into range offsets; also the
// largest count of one anchor.
__global__ void range_widen_kernel(const uint32_t* __restrict__ raw, uint64_t num,
                                   unsigned long long* __restrict__ off, unsigned long long* __restrict__ maxima) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;  // blockDim: a multiple of 32
    const uint32_t v = i < num ? raw[i] : 0u;
    if (i <= num) off[i] = v;
    const uint32_t m = __reduce_max_sync(0xffffffffu, v);
    if (lane_id() == 0 && m > 0) atomicMax(&maxima[1], (unsigned long long)m);
}

// After the scan: the largest raw total of one batch of `batch` anchors.
__global__ void range_batch_max_kernel(const unsigned long long* __restrict__ off, uint64_t num, uint64_t batch,
                                       unsigned long long* __restrict__ maxima) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t b0 = j * batch;
    if (b0 >= num) return;
    const uint64_t b1 = b0 + batch < num ? b0 + batch : num;
    atomicMax(&maxima[0], off[b1] - off[b0]);
}

constexpr int kGatherThreads = 128;

// One block per anchor: the union of the anchor's buckets, ascending, without
// the anchor itself (and without ambiguous reads if requested).  The raw ids
// go into a shared-memory hash set (duplicates vanish on insert, the first
// copy of an id joins the unique list); the unique ids are then put in
// ascending order by rank (or a bitonic sort when there are many).  rawOff =
// exclusive scan of the raw counts; the table holds tableSize >= 2 * raw
// slots.
// Raw id range (offset, count) of anchor a.  In the batched form it comes
// from the range scan; the small-table pass also writes the offset into
// b.rawCount for the later stages.
__device__ __forceinline__ uint2 gather_range(const BatchArg& b, const uint32_t* __restrict__ rawOff, int a,
                                              uint64_t first, bool writeOffsets) {
    if (b.rangeOff) {
        const uint64_t r0 = first - out_first(b);
        const unsigned long long* ro = b.rangeOff + r0;
        const uint32_t off = (uint32_t)(ro[a] - ro[0]);
        if (writeOffsets && threadIdx.x == 0) {
            b.rawCount[a] = off;
            if (a == b.count - 1) b.rawCount[b.count] = (uint32_t)(ro[b.count] - ro[0]);
        }
        return make_uint2(off, (uint32_t)(ro[a + 1] - ro[a]));
    }
    return make_uint2(rawOff[a], rawOff[a + 1] - rawOff[a]);
}

// The union of anchor a's buckets (all threads of the block), raw > 0; the
// shared-memory table holds tableSize >= 2 * raw slots and a list of half that.
// Groups of 16 threads take the maps in turn (a bucket's first 16 ids with one
// load per thread, all maps' loads issued before the inserts); an id joins the
// unique list when its first copy enters the hash set.
__device__ void gather_one(const StoreArg& st, const TablesArg& tb, const Params& p, const BatchArg& b, int a,
                           uint64_t aid, uint32_t off, uint32_t raw, uint32_t* table, int tableSize, uint2* rng,
                           uint32_t* nUniqueS) {
    uint32_t* list = table + tableSize;
    uint32_t& nUnique = *nUniqueS;
    const int tid = threadIdx.x;
    uint32_t T = 64;
    while (T < raw + raw / 2) T <<= 1;  // at most two thirds full
    const uint32_t mask = T - 1;
    if (tid < tb.nmaps) {
        if (b.rangeOff) {
            // the rule of query_count_kernel; raw > 0 means the anchor is active
            uint2 r = lookup(tb.slots[tid], tb.mask[tid], b.sig[(uint64_t)tid * st.n + aid]);
            if ((int)r.y > tb.maxValuesPerKey) r = make_uint2(0, 0);
            rng[tid] = r;
        } else {
            rng[tid] = b.qrange[(uint64_t)a * tb.nmaps + tid];
        }
    }
    for (uint32_t i = tid; i < T; i += kGatherThreads) table[i] = 0xffffffffu;
    if (tid == 0) nUnique = 0;
    // With strand-tagged values (tb.strand set) a unique candidate's list
    // entry is its sort key id << 1 | o, o = the orientation predicted by the
    // map whose bucket brought its first copy: its strand bit against the
    // anchor's for that map (0 forward, 1 reverse complement).  The ids are
    // distinct, so sorting the keys sorts the ids.
    const bool tagged = tb.strand != nullptr;
    constexpr int kGroup = 16, kGroups = kGatherThreads / kGroup, kMapsPer = (kMaxMaps + kGroups - 1) / kGroups;
    const int g = tid / kGroup, gl = tid % kGroup;
    // this thread's maps g + k kGroups: bit k = the anchor's strand bit there
    // (maps 0-15 only; the others carry no prediction)
    uint32_t aStrand = 0;
    if (tagged) {
        const uint32_t bits = tb.strand[aid];
#pragma unroll
        for (int k = 0; k < kMapsPer; k++) {
            const int m = g + k * kGroups;
            if (m < 16) aStrand |= ((bits >> m) & 1u) << k;
        }
    }
    __syncthreads();
    auto insert = [&](uint32_t tv, int k) {  // a value of map g + k kGroups
        const uint32_t v = tagged ? tv & 0x7fffffffu : tv;
        uint32_t h = (v * 0x9E3779B1u) & mask;
        for (uint32_t probe = 0; probe < T; probe++) {
            const uint32_t old = atomicCAS(&table[h], 0xffffffffu, v);
            if (old == 0xffffffffu) {  // the first copy of v
                if ((uint64_t)v != aid && !(p.excludeAmbiguous && st.ambig[v]))
                    list[atomicAdd(&nUnique, 1u)] = tagged ? (v << 1) | ((tv >> 31) ^ ((aStrand >> k) & 1u)) : v;
                return;
            }
            if (old == v) return;
            h = (h + 1) & mask;
        }
    };
    uint32_t vals[kMapsPer];
#pragma unroll
    for (int k = 0; k < kMapsPer; k++) {
        const int m = g + k * kGroups;
        vals[k] = 0xffffffffu;
        if (m < tb.nmaps && (uint32_t)gl < rng[m].y) vals[k] = tb.values[m][rng[m].x + gl];
    }
#pragma unroll
    for (int k = 0; k < kMapsPer; k++)
        if (vals[k] != 0xffffffffu) insert(vals[k], k);
    for (int k = 0; k < kMapsPer; k++) {  // ids past a bucket's first 16
        const int m = g + k * kGroups;
        if (m >= tb.nmaps) break;
        for (uint32_t i = kGroup + gl; i < rng[m].y; i += kGroup) insert(tb.values[m][rng[m].x + i], k);
    }
    __syncthreads();
    const uint32_t U = nUnique;
    uint32_t* out = b.cand + off;
    const int keyShift = tagged ? 1 : 0;
    // the sorted keys stay in shared memory for the alignment order below:
    // in `list` after the register sort, in `table` (free once the ids are
    // in) after the others
    const uint32_t* sk = U <= 64 ? list : table;
    if (U <= 64) {
        // one warp: a bitonic network over 64 slots in registers, ids i and
        // i + 32 in lane i (padding sorts last; the ids are distinct)
        if (tid < 32) {
            constexpr unsigned kFull = 0xffffffffu;
            const uint32_t lane = (uint32_t)tid;
            uint32_t x0 = lane < U ? list[lane] : 0xffffffffu, x1 = lane + 32 < U ? list[lane + 32] : 0xffffffffu;
#pragma unroll
            for (uint32_t k = 2; k <= 64; k <<= 1) {
#pragma unroll
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    if (j == 32) {  // slots i and i + 32 meet in one lane (k == 64: ascending)
                        const uint32_t lo = min(x0, x1), hi = max(x0, x1);
                        x0 = lo;
                        x1 = hi;
                    } else {
                        const uint32_t y0 = __shfl_xor_sync(kFull, x0, j), y1 = __shfl_xor_sync(kFull, x1, j);
                        const bool lower = (lane & j) == 0;
                        const bool asc0 = (lane & k) == 0, asc1 = ((lane + 32) & k) == 0;
                        x0 = lower == asc0 ? min(x0, y0) : max(x0, y0);
                        x1 = lower == asc1 ? min(x1, y1) : max(x1, y1);
                    }
                }
            }
            if (lane < U) out[lane] = x0 >> keyShift;
            if (lane + 32 < U) out[lane + 32] = x1 >> keyShift;
            __syncwarp();  // every lane has read its unsorted keys
            if (lane < U) list[lane] = x0;  // the list holds at least U entries
            if (lane + 32 < U) list[lane + 32] = x1;
        }
    } else if (U <= 512) {
        // rank of each id among the unique ids = its position in ascending order
        for (uint32_t i = tid; i < U; i += kGatherThreads) {
            const uint32_t v = list[i];
            uint32_t rank = 0;
            for (uint32_t k = 0; k < U; k++) rank += list[k] < v;
            out[rank] = v >> keyShift;
            table[rank] = v;
        }
    } else {
        uint32_t S = 1;
        while (S < U) S <<= 1;  // S <= T: the hash table's space becomes the sort buffer
        for (uint32_t i = tid; i < S; i += kGatherThreads) table[i] = i < U ? list[i] : 0xffffffffu;
        __syncthreads();
        for (uint32_t k = 2; k <= S; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < S; i += kGatherThreads) {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        const uint32_t x = table[i], y = table[ixj];
                        const bool asc = (i & k) == 0;
                        if ((x > y) == asc) {
                            table[i] = y;
                            table[ixj] = x;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = tid; i < U; i += kGatherThreads) out[i] = table[i] >> keyShift;
    }
    if (b.perm && !b.lenOrder) {
        // the alignment's order is the list's; an entry is the position with
        // the predicted orientation in bit 31
        __syncthreads();
        for (uint32_t i = tid; i < U; i += kGatherThreads) b.perm[off + i] = i | (tagged ? (sk[i] & 1u) << 31 : 0u);
    } else if (b.perm) {
        // the alignment's order: positions grouped by words per read
        // (length / 32, up to 8) and within that by predicted orientation,
        // in position order within a group -- a counting sort by one warp;
        // the list's space holds the groups.  An entry is the position, with
        // the predicted orientation in bit 31.
        __syncthreads();
        if (tid < 32) {
            constexpr unsigned kFull = 0xffffffffu;
            constexpr int kGroups = 18;
            const int lane = tid;
            uint32_t cnt = 0;  // lane g < kGroups: size of group g, then its start
            for (uint32_t i0 = 0; i0 < U; i0 += 32) {
                const uint32_t i = i0 + (uint32_t)lane;
                uint32_t g = kGroups;
                if (i < U) {
                    const uint32_t key = sk[i];
                    g = 2 * min((uint32_t)st.len[key >> keyShift] >> 5, 8u) + (tagged ? key & 1u : 0u);
                }
                __syncwarp();  // sk may be `list`: every lane has its key before the groups overwrite it
                if (i < U) list[i] = g;
#pragma unroll
                for (int v = 0; v < kGroups; v++) {
                    const uint32_t n = __popc(__ballot_sync(kFull, g == (uint32_t)v));
                    if (lane == v) cnt += n;
                }
            }
            uint32_t start = cnt;  // exclusive scan over the groups
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, start, d);
                if (lane >= d) start += y;
            }
            start -= cnt;
            for (uint32_t i0 = 0; i0 < U; i0 += 32) {
                const uint32_t i = i0 + (uint32_t)lane;
                const uint32_t g = i < U ? list[i] : kGroups;
                uint32_t r = 0;
#pragma unroll
                for (int v = 0; v < kGroups; v++) {
                    const uint32_t m = __ballot_sync(kFull, g == (uint32_t)v);
                    const uint32_t s0 = __shfl_sync(kFull, start, v);
                    if (g == (uint32_t)v) r = s0 + __popc(m & ((1u << lane) - 1u));
                    if (lane == v) start += __popc(m);
                }
                if (i < U) b.perm[off + r] = i | ((g & 1u) << 31);
            }
        }
    }
    if (tid == 0) {
        b.ncand[a] = U;
        atomicAdd(&b.counters[kCounterRaw], (unsigned long long)raw);
        atomicAdd(&b.counters[kCounterUnique], (unsigned long long)U);
    }
}

// One block per anchor of the batch with at most smallCap raw ids (all of them
// when bigList is null); anchors with more go to bigList for gather_big_kernel,
// whose blocks hold tables large enough for them.  The split keeps the few
// repeat anchors' large tables from lowering every block's occupancy.
__global__ void __launch_bounds__(kGatherThreads, 16) gather_unique_kernel(StoreArg st, TablesArg tb, Params p,
                                                                       BatchArg b, const uint32_t* __restrict__ rawOff,
                                                                       int tableSize, uint32_t smallCap,
                                                                       uint32_t* bigList, unsigned int* bigCount) {
    extern __shared__ uint32_t table[];  // [tableSize], then list[tableSize / 2]
    __shared__ uint2 rng[kMaxMaps];
    __shared__ uint32_t nUnique;
    const int a = blockIdx.x;
    const uint64_t first = batch_first(b);
    const uint2 r = gather_range(b, rawOff, a, first, true);
    if (r.y == 0) {
        if (threadIdx.x == 0) b.ncand[a] = 0;
        return;
    }
    if (bigList && r.y > smallCap) {
        if (threadIdx.x == 0) bigList[atomicAdd(bigCount, 1u)] = (uint32_t)a;
        return;
    }
    gather_one(st, tb, p, b, a, first + (uint64_t)a, r.x, r.y, table, tableSize, rng, &nUnique);
}

// Persistent blocks over the deferred anchors of gather_unique_kernel.
__global__ void __launch_bounds__(kGatherThreads) gather_big_kernel(StoreArg st, TablesArg tb, Params p, BatchArg b,
                                                                    const uint32_t* __restrict__ rawOff,
                                                                    int tableSize, const uint32_t* bigList,
                                                                    const unsigned int* bigCount) {
    extern __shared__ uint32_t table[];
    __shared__ uint2 rng[kMaxMaps];
    __shared__ uint32_t nUnique;
    const uint64_t first = batch_first(b);
    const unsigned int n = *bigCount;
    for (unsigned int i = blockIdx.x; i < n; i += gridDim.x) {
        const int a = (int)bigList[i];
        const uint2 r = gather_range(b, rawOff, a, first, false);
        gather_one(st, tb, p, b, a, first + (uint64_t)a, r.x, r.y, table, tableSize, rng, &nUnique);
        __syncthreads();  // the next anchor reuses the shared arrays
    }
}

// One thread per read pair (2i, 2i+1) of the batch: flag candidates whose mate
// is a candidate of the other read of the pair (include/util.hpp:1005-1143).
__global__ void pair_flags_kernel(BatchArg b, const uint32_t* __restrict__ rawOff) {
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    const int a1 = 2 * pr;
    if (a1 + 1 >= b.count) return;
    const uint32_t* r1 = b.cand + rawOff[a1];
    const uint32_t* r2 = b.cand + rawOff[a1 + 1];
    uint8_t* f1 = b.paired + rawOff[a1];
    uint8_t* f2 = b.paired + rawOff[a1 + 1];
    const uint32_t n1 = b.ncand[a1], n2 = b.ncand[a1 + 1];
    for (uint32_t i = 0; i < n1; i++) f1[i] = 0;
    for (uint32_t i = 0; i < n2; i++) f2[i] = 0;
    uint32_t x = 0, y = 0;
    while (x < n1 && y < n2) {
        const int e1 = (x + 1 < n1 && r1[x] / 2 == r1[x + 1] / 2) ? 2 : 1;
        const int e2 = (y + 1 < n2 && r2[y] / 2 == r2[y + 1] / 2) ? 2 : 1;
        const bool same = r1[x] / 2 == r2[y] / 2;
        if (e1 == 1 && e2 == 1) {
            if (same) {
                if (r1[x] != r2[y]) {
                    f1[x] = 1;
                    f2[y] = 1;
                }
                x++;
                y++;
            } else if (r1[x] < r2[y]) {
                x++;
            } else {
                y++;
            }
        } else if (e1 == 2 && e2 == 2) {
            if (same) {
                f1[x] = f1[x + 1] = 1;
                f2[y] = f2[y + 1] = 1;
                x += 2;
                y += 2;
            } else if (r1[x] < r2[y]) {
                x += 2;
            } else {
                y += 2;
            }
        } else if (e1 == 2 && e2 == 1) {
            if (same) {
                if (r1[x] == r2[y]) {
                    x++;
                    f1[x] = 1;
                    f2[y] = 1;
                    x++;
                    y++;
                } else {
                    f1[x] = 1;
                    f2[y] = 1;
                    x += 2;
                    y++;
                }
            } else if (r1[x] < r2[y]) {
                x += 2;
            } else {
                y++;
            }
        } else {
            if (same) {
                if (r1[x] == r2[y]) {
                    y++;
                    f1[x] = 1;
                    f2[y] = 1;
                    x++;
                    y++;
                } else {
                    f1[x] = 1;
                    f2[y] = 1;
                    x++;
                    y += 2;
                }
            } else if (r1[x] < r2[y]) {
                x++;
            } else {
                y += 2;
            }
        }
    }
}

}  // namespace

cudaError_t launch_table_init(Slot* t, uint64_t cap, cudaStream_t s) {
    table_init_kernel<<<(unsigned)std::max<uint64_t>(1, (cap + 255) / 256), 256, 0, s>>>(t, cap);
    return cudaGetLastError();
}

unsigned grid_of(uint64_t threads) { return (unsigned)std::max<uint64_t>(1, (threads + 255) / 256); }

cudaError_t launch_run_heads(const unsigned long long* keys, uint64_t n, uint32_t* runOf, cudaStream_t s) {
    run_head_kernel<<<grid_of(n + 1), 256, 0, s>>>(keys, n, runOf);
    return cudaGetLastError();
}

cudaError_t launch_run_starts(const unsigned long long* keys, uint64_t n, const uint32_t* runOf, uint32_t* start,
                              cudaStream_t s) {
    run_start_kernel<<<grid_of(n + 1), 256, 0, s>>>(keys, n, runOf, start);
    return cudaGetLastError();
}

cudaError_t launch_run_pack(const unsigned long long* keys, const uint32_t* start, uint32_t runs, int maxValues,
                            unsigned long long* packed, cudaStream_t s) {
    run_pack_kernel<<<grid_of((uint64_t)runs + 1), 256, 0, s>>>(keys, start, runs, maxValues, packed);
    return cudaGetLastError();
}

cudaError_t launch_run_fill(const unsigned long long* keys, const uint32_t* ids, uint64_t n, const uint32_t* runOf,
                            const uint32_t* start, uint32_t runs, const unsigned long long* packedScan, int maxValues,
                            uint32_t* values, Slot* fin, uint32_t finMask, cudaStream_t s, uint32_t* rawAll,
                            uint32_t idMask) {
    run_values_kernel<<<grid_of(n), 256, 0, s>>>(keys, ids, n, runOf, start, packedScan, maxValues, values, rawAll,
                                                 idMask);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    run_place_kernel<<<grid_of(runs), 256, 0, s>>>(keys, start, runs, packedScan, maxValues, fin, finMask);
    return cudaGetLastError();
}

cudaError_t launch_query_count(StoreArg st, TablesArg tb, Params p, BatchArg b, cudaStream_t s) {
    const uint64_t threads = (uint64_t)b.count * 32;
    query_count_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(st, tb, p, b);
    return cudaGetLastError();
}

namespace {

constexpr uint32_t kGatherSmallRaw = 1024;  // anchors above this go to the large-table pass
constexpr int kGatherBigBlocksPerSm = 4;

int table_slots(int maxRaw) {
    int T = 64;
    while (T < 2 * maxRaw) T <<= 1;
    return T;
}

template <class K>
cudaError_t gather_smem_attr(K kernel, size_t smem) {
    if (smem <= 40 * 1024) return cudaSuccess;  // leaves room for the kernel's static shared memory
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace

cudaError_t launch_gather_unique(StoreArg st, TablesArg tb, Params p, BatchArg b, int maxRawPerAnchor,
                                 cudaStream_t s, uint32_t* bigScratch) {
    if (b.count <= 0) return cudaSuccess;
    const bool split = bigScratch && (uint32_t)maxRawPerAnchor > kGatherSmallRaw;
    const int T = table_slots(split ? (int)kGatherSmallRaw : maxRawPerAnchor);
    const size_t smem = (size_t)T * sizeof(uint32_t) * 3 / 2;  // table + unique list
    cudaError_t e = gather_smem_attr(gather_unique_kernel, smem);
    if (e != cudaSuccess) return e;
    unsigned int* bigCount = split ? bigScratch : nullptr;
    uint32_t* bigList = split ? bigScratch + 1 : nullptr;
    if (split) {
        e = cudaMemsetAsync(bigCount, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) return e;
    }
    gather_unique_kernel<<<b.count, kGatherThreads, smem, s>>>(st, tb, p, b, b.rawCount, T, kGatherSmallRaw,
                                                                bigList, bigCount);
    e = cudaGetLastError();
    if (e != cudaSuccess || !split) return e;
    const int Tb = table_slots(maxRawPerAnchor);
    const size_t smemB = (size_t)Tb * sizeof(uint32_t) * 3 / 2;
    e = gather_smem_attr(gather_big_kernel, smemB);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned blocks = (unsigned)std::min<int>(b.count, std::max(sms, 1) * kGatherBigBlocksPerSm);
    gather_big_kernel<<<blocks, kGatherThreads, smemB, s>>>(st, tb, p, b, b.rawCount, Tb, bigList, bigCount);
    return cudaGetLastError();
}

cudaError_t launch_raw_count(StoreArg st, Params p, uint32_t* raw, cudaStream_t s) {
    if (st.n == 0) return cudaSuccess;
    raw_count_kernel<<<(unsigned)((st.n + 255) / 256), 256, 0, s>>>(st, p, raw);
    return cudaGetLastError();
}

cudaError_t launch_range_offsets(const uint32_t* raw, uint64_t num, uint64_t batch, unsigned long long* off,
                                 void* tmp, unsigned long long* maxima, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(maxima, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    range_widen_kernel<<<(unsigned)((num + 1 + 255) / 256), 256, 0, s>>>(raw, num, off, maxima);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_exclusive_u64(off, num + 1, tmp, s);
    if (e != cudaSuccess) return e;
    const uint64_t batches = (num + batch - 1) / batch;
    range_batch_max_kernel<<<(unsigned)((batches + 255) / 256), 256, 0, s>>>(off, num, batch, maxima);
    return cudaGetLastError();
}

cudaError_t launch_pair_flags(BatchArg b, cudaStream_t s) {
    const int pairs = b.count / 2;
    if (pairs == 0) return cudaSuccess;
    pair_flags_kernel<<<(pairs + 127) / 128, 128, 0, s>>>(b, b.rawCount);
    return cudaGetLastError();
}

}  // namespace cg
