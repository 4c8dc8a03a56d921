// File-to-file correction with the input parsing (STEP1) and the output
// records (STEP3) on the device.
//
// reference: the input side of care::performCorrection (src/readlibraryio.cpp,
// include/readlibraryio.hpp:121-403: kseq-style FASTQ records, paired files
// read alternately) and its output side (src/correctionresultoutput.cpp:
// 448-970, one "@header\nSEQ\n+\nQUAL\n" record per read, the corrected
// sequence as edits or whole, quality labels " care:q=N").  The host layer
// (host/care_host.cpp) takes this path for FASTQ inputs and falls back to its
// own reader and writer whenever the layout is not the plain one checked here.
#ifndef CARE_FILES_H
#define CARE_FILES_H

#include <stddef.h>
#include <stdint.h>

#include <functional>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "care_gpu.h"

namespace cg {

// A caller's bytes (a whole input file).
struct ByteSpan {
    const char* data;
    size_t size;
};

struct FastqRun {
    uint64_t reads = 0;
    uint64_t records = 0;                    // correction records (changNum)
    cg_stats stats{};
    // bytes of every output file
    std::vector<std::unique_ptr<char[]>> outputs;
    std::vector<size_t> outputSizes;
    // if set, the reads are corrected in a few ranges and each range's bytes
    // of output file f go here in order (outputs stays empty), so that the
    // caller can write one range while the next is corrected
    std::function<void(int f, std::unique_ptr<char[]> bytes, size_t size)> onChunk;
    // Queue protocol: with queueChunkBytes set (and onChunk unset) the output
    // files stay in device memory, cut into chunks of whole records of under
    // queueChunkBytes bytes each (the host writer's cut points), and
    // emit_queue_chunks hands them over (outputs stays empty).
    size_t queueChunkBytes = 0;
    struct DeviceOutput {
        void* bytes = nullptr;                          // device memory
        std::vector<std::pair<size_t, size_t>> chunks;  // [begin, end) byte ranges
    };
    std::vector<DeviceOutput> deviceOutputs;

    FastqRun() = default;
    FastqRun(const FastqRun&) = delete;
    FastqRun& operator=(const FastqRun&) = delete;
    ~FastqRun();  // frees deviceOutputs
};

// Corrects the reads of `inputs` (the bytes of whole FASTQ files) and returns
// the output files' bytes.  Single end: each input is one group of reads (as
// one cg_append_reads call) and read i goes to output min(input, numOutputs-1).
// Paired (two inputs): read 2i is record i of the first file and 2i+1 record i
// of the second, as many pairs as the shorter file holds; read i goes to
// output i & 1 when there are two outputs, else to output 0.
// Returns CG_OK; CG_ERR_UNSUPPORTED when an input is not plain 4-line FASTQ
// (a '\r', an empty or continued line, a record whose sequence line starts
// with '+' or whose quality length differs, a read over CG_MAX_READ_LENGTH) --
// nothing has been written then and the caller takes the host path; any other
// code is an error (message in *error).
int correct_fastq_on_device(const cg_options& options, const std::vector<ByteSpan>& inputs,
                            bool paired, bool qualityLabels, int numOutputs, const std::vector<char>* forest,
                            uint32_t maxTrees, const std::vector<char>* classifier, FastqRun* run,
                            std::string* error);

// Queue protocol, after correct_fastq_on_device with run->queueChunkBytes set:
// sink(f, chunk, size) gets every chunk of output file f, the files' chunks
// alternating (file 0's first, file 1's first, file 0's second, ...); each
// chunk is copied from device memory straight into a new char[queueChunkBytes]
// that the sink owns.  Stops when the sink returns false.  Frees the device
// outputs.  Returns CG_OK or CG_ERR_CUDA (message in *error).
int emit_queue_chunks(FastqRun* run, const std::function<bool(int f, char* chunk, int size)>& sink,
                      std::string* error);

}  // namespace cg

#endif
