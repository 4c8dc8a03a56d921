// Library-internal hooks of the C ABI layer (care_capi.cu) for the device
// file path (care_files.cu): reads that are already in device memory, and
// results that stay there.
#ifndef CARE_CAPI_INTERNAL_H
#define CARE_CAPI_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include "care_gpu.h"

namespace cg {

// cg_append_reads for one group of reads already on the device: bases back to
// back (dChars), offsets dOffs[n+1] from 0, qualities like the bases (or
// null).  The context takes ownership of the three cudaMalloc'd buffers.
int append_device_chunk(cg_ctx* c, void* dChars, uint64_t* dOffs, void* dQual, uint64_t n, int lmax);

// cg_correct with flags[num] and sequences[num][pitch] in device memory.
int correct_into_device(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* dFlags, char* dSeq, size_t pitch);

// cg_combine_results with flags[num] in device memory (candidate correction
// on); *records (may be null) gets the saved candidate records of the reads.
int combine_into_device(cg_ctx* c, uint64_t first, uint64_t num, uint8_t* dFlags, uint64_t* records);

}  // namespace cg

#endif
