// Host side of the drop-in boundary: the reference's two CARE entry points,
// re-implemented over the C ABI of include/care_gpu.h.
//
// reference: include/dispatch_care_correct_cpu.hpp:9-11
//     void care::performCorrection(ProgramOptions);
//     void care::performCorrectionOutToQueue(ProgramOptions, Q1, Q2, producerDone,
//                                            careStartWrite, changNum);
// and the STEP3 output rules of src/correctionresultoutput.cpp:448-970,1256-1551
// (anchor-only correction: a read with a correction record takes its
// corrected sequence -- as edits when it had no ambiguous base and at most
// length/7 positions changed, else whole -- and the record count is the
// changNum of the queue protocol).
#ifndef CARE_HOST_H
#define CARE_HOST_H

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "care_gpu.h"

#include <unistd.h>

namespace care_gb300 {

enum class SequencePairType { Invalid, SingleEnd, PairedEnd };
enum class CorrectionType : int { Classic = 0, Forest = 1, Print = 2, Learned = 3 };

// The fields of care::ProgramOptions (reference include/options.hpp:36-99)
// that the correction path and its output read, with the same names and defaults.
struct ProgramOptions {
    int min_overlap = 30;
    float maxErrorRate = 0.2f;
    float min_overlap_ratio = 0.30f;
    bool excludeAmbiguousReads = false;
    bool correctCandidates = false;
    bool useQualityScores = false;
    bool autodetectKmerlength = false;
    bool outputCorrectionQualityLabels = false;
    bool gzoutput = false;
    float estimatedCoverage = 1.0f;
    float estimatedErrorrate = 0.06f;
    float m_coverage = 0.6f;
    int batchsize = 1000;
    int new_columns_to_correct = 15;
    int kmerlength = 20;
    int numHashFunctions = 48;
    CorrectionType correctionType = CorrectionType::Classic;
    CorrectionType correctionTypeCands = CorrectionType::Classic;
    float thresholdAnchor = .5f;
    float pairedFilterThreshold = 0.06f;
    uint32_t maxForestTreesAnchor = 0xffffffffu;
    std::string mlForestfileAnchor = "";
    // No reference counterpart: the GPU driver (both give identical results;
    // the batched one replays captured per-batch graphs, see cg_options.driver)
    // and the serialized classifier of CorrectionType::Learned.
    bool gpuBatched = true;
    std::string mlClassifierFileAnchor = "";
    // FASTQ inputs parsed and output records written on the device (inputs
    // that are not plain 4-line FASTQ take the host reader and writer anyway)
    bool deviceFileIO = true;
    bool showProgress = false;
    int threads = 1;
    std::vector<int> deviceIds;
    int qualityScoreBits = 8;             // 8, 2 or 1: lossy quality store (cg_options.quality_score_bits)
    std::size_t fixedNumberOfReads = 0;   // only reads [0, n) are corrected as anchors (0 = all)
    // Host memory limits of the reference's table construction: the smaller
    // one goes to cg_options.hashtable_memory_bytes, where a limit that would
    // make the reference build its maps in several rounds is refused
    // (CG_ERR_UNSUPPORTED).  0 = no limit (the device holds the tables).
    std::size_t memoryForHashtables = 0;
    std::size_t memoryTotalLimit = 0;
    bool mustUseAllHashfunctions = false;  // the reference aborts when fewer maps than requested were built
    // candidate classifier (only with correctCandidates; Forest/Print are refused)
    float thresholdCands = .5f;
    uint32_t maxForestTreesCands = 0xffffffffu;
    std::string mlForestfileCands = "";
    // binary read-store / hash-table files of the reference's checkpointing
    // (--save_preprocessedreads_to, --load_preprocessedreads_from,
    // --save_hashtables_to, --load_hashtables_from): not supported, refused
    std::string save_binary_reads_to = "";
    std::string load_binary_reads_from = "";
    std::string save_hashtables_to = "";
    std::string load_hashtables_from = "";
    SequencePairType pairType = SequencePairType::SingleEnd;
    std::string outputdirectory = "";
    std::string tempdirectory = "";
    std::vector<std::string> inputfiles;
    std::vector<std::string> outputfilenames;
};

cg_options toCgOptions(const ProgramOptions& o);

// Throws std::runtime_error for options this engine refuses rather than
// silently computing something else: Print correction (either type), a Forest
// candidate classifier with candidate correction, the checkpoint files, and a
// quality bit count other than 1, 2 or 8.  The hash-table memory limit is
// checked by cg_build_tables once the number of reads is known.
void validateOptions(const ProgramOptions& o);

// One output chunk: `data` (allocated with new char[]) holds whole FASTQ
// records of output file `file`; ownership passes to the sink.
using ChunkSink = std::function<bool(int file, char* data, int size)>;

struct RunReport {
    uint64_t reads = 0;
    uint64_t records = 0;  // correction records (changNum)
    cg_stats stats{};
    bool deviceFileIO = false;  // the files were parsed and written on the device
};

// STEP1-3 into files outputdirectory/outputfilenames[i].  Throws on error.
RunReport performCorrection(const ProgramOptions& programOptions);

// STEP1-3 into 1 MiB chunks; onStart(changNum) is called before the first
// chunk; no chunk is produced when changNum is 0.  Throws on error.
RunReport performCorrectionToSink(const ProgramOptions& programOptions, const std::function<void(int)>& onStart,
                                  const ChunkSink& sink);

// The reference's queue protocol on any queue type with
// try_enqueue(std::pair<char*, int>) (moodycamel::ReaderWriterQueue in RabbitQCPlus).
template <class Queue>
void performCorrectionOutToQueue(ProgramOptions programOptions, Queue* Q1, Queue* Q2, std::atomic_int* producerDone,
                                 std::atomic_int* careStartWrite, int* changNum) {
    performCorrectionToSink(
        programOptions,
        [&](int n) {
            *changNum = n;
            *careStartWrite = 1;
        },
        [&](int file, char* data, int size) {
            Queue* q = file == 0 ? Q1 : Q2;
            while (!q->try_enqueue(std::pair<char*, int>(data, size))) {
                if (*producerDone == 1) {
                    delete[] data;
                    return false;
                }
                usleep(100);
            }
            return true;
        });
}

}  // namespace care_gb300

#endif
