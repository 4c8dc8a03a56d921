// Device helpers shared by the kernel files.
#ifndef CARE_DEVICE_CUH
#define CARE_DEVICE_CUH

#include <stdint.h>

#include "care_internal.h"

namespace cg {

// 64-bit Murmur finalizer (reference: include/hpc_helpers/include/hashers.cuh:129-136)
__device__ __forceinline__ uint64_t murmur64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// slot index of a key in an open-addressing table with capacity mask+1
__device__ __forceinline__ uint32_t slot_of(uint64_t key, uint32_t mask) {
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 32) & mask;
}

// 2-bit base i of a read (reference: include/sequencehelpers.hpp:195-201)
__device__ __forceinline__ uint32_t get2bit(const uint32_t* enc, int i) {
    return (enc[i >> 4] >> (30 - 2 * (i & 15))) & 3u;
}

// base at position p of a candidate read in its aligned orientation
__device__ __forceinline__ uint32_t oriented_base(const uint32_t* enc, int len, bool rc, int p) {
    return rc ? 3u - get2bit(enc, len - 1 - p) : get2bit(enc, p);
}

// reference: include/hostdevicefunctions.cuh:9-28
__device__ __forceinline__ bool feq(float l, float r) {
    const float d = __fsub_rn(l, r) < 0.0f ? -__fsub_rn(l, r) : __fsub_rn(l, r);
    return d < 1e-5f;
}
__device__ __forceinline__ bool fleq(float l, float r) { return (l < r) || feq(l, r); }
__device__ __forceinline__ bool fgeq(float l, float r) { return (l > r) || feq(l, r); }

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// One 4-byte word from global to shared memory without a register (cp.async,
// L1-cached); complete and visible to the issuing thread after
// cp_async_wait_all(), to the rest of its warp after a __syncwarp() that
// follows.
__device__ __forceinline__ void cp_async4(uint32_t* dst, const uint32_t* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// first anchor of the batch and anchor id of output row 0: kernel parameters,
// or device memory in graph replays
__device__ __forceinline__ uint64_t batch_first(const BatchArg& b) { return b.cursor ? b.cursor[0] : b.first; }
__device__ __forceinline__ uint64_t out_first(const BatchArg& b) { return b.cursor ? b.cursor[1] : b.outFirst; }

}  // namespace cg

#endif
