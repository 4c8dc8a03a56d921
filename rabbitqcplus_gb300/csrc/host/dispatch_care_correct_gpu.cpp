// Drop-in replacement for RabbitQCPlus's src/dispatch_care_correct_cpu.cpp:
// the same two entry points (reference: include/dispatch_care_correct_cpu.hpp:
// 9-11), served by the GB300 engine through the host layer of care_host.h.
//
// This file is compiled inside a RabbitQCPlus build, against its headers
// (care::ProgramOptions from include/options.hpp, moodycamel's queue from
// include/concurrencyhelpers.hpp), in place of dispatch_care_correct_cpu.o;
// the binary links libcaregpu.so.  It is not part of libcaregpu.so itself.
//
// Every field of care::ProgramOptions (include/options.hpp:36-99) is either
// forwarded or does not change the corrected output:
//   forwarded  -- the correction parameters, files, pair mode, threads and
//                 devices, quality scores and their bit count, candidate
//                 correction and its classifier fields, forest file and tree
//                 limits, fixedNumberOfReads, the table-memory limits, the
//                 checkpoint file names (refused by the host layer when set);
//   no effect  -- batchsize (the device batches anchors itself), singlehash
//                 (the reference always builds its ordinary minhasher,
//                 src/dispatch_care_correct_cpu.cpp:105-109),
//                 hashtableLoadfactor (the layout of the reference's host
//                 tables, not their contents), showProgress, sampleRateAnchor/
//                 sampleRateCands and mlForestfilePrint* (Print mode only,
//                 which is refused), the GPU-version and extension options
//                 (canUseGpu, replicateGpuData, warpcore, insertSize*,
//                 fixedStddev, fixedStepsize, allowOutwardExtension,
//                 sortedOutput, outputRemainingReads, extendedReadsOutputfilename,
//                 minimum/maximum_sequence_length, nReads), which the CPU
//                 correction path of the reference does not read.
#include <dispatch_care_correct_cpu.hpp>  // care::ProgramOptions, moodycamel::ReaderWriterQueue

#include "care_host.h"

namespace care {

// Exposed (not static) so that an integration test can check the mapping.
care_gb300::ProgramOptions toGb300Options(const ProgramOptions& o) {
    care_gb300::ProgramOptions g;
    g.min_overlap = o.min_overlap;
    g.maxErrorRate = o.maxErrorRate;
    g.min_overlap_ratio = o.min_overlap_ratio;
    g.excludeAmbiguousReads = o.excludeAmbiguousReads;
    g.correctCandidates = o.correctCandidates;
    g.useQualityScores = o.useQualityScores;
    g.autodetectKmerlength = o.autodetectKmerlength;
    g.outputCorrectionQualityLabels = o.outputCorrectionQualityLabels;
    g.gzoutput = o.gzoutput;
    g.estimatedCoverage = o.estimatedCoverage;
    g.estimatedErrorrate = o.estimatedErrorrate;
    g.m_coverage = o.m_coverage;
    g.batchsize = o.batchsize;
    g.new_columns_to_correct = o.new_columns_to_correct;
    g.kmerlength = o.kmerlength;
    g.numHashFunctions = o.numHashFunctions;
    g.correctionType = static_cast<care_gb300::CorrectionType>(static_cast<int>(o.correctionType));
    g.correctionTypeCands = static_cast<care_gb300::CorrectionType>(static_cast<int>(o.correctionTypeCands));
    g.thresholdAnchor = o.thresholdAnchor;
    g.thresholdCands = o.thresholdCands;
    g.pairedFilterThreshold = o.pairedFilterThreshold;
    g.maxForestTreesAnchor = o.maxForestTreesAnchor;
    g.maxForestTreesCands = o.maxForestTreesCands;
    g.mlForestfileAnchor = o.mlForestfileAnchor;
    g.mlForestfileCands = o.mlForestfileCands;
    g.showProgress = o.showProgress;
    g.threads = o.threads;
    g.deviceIds = o.deviceIds;
    g.qualityScoreBits = o.qualityScoreBits;
    g.fixedNumberOfReads = o.fixedNumberOfReads;
    g.memoryForHashtables = o.memoryForHashtables;
    g.memoryTotalLimit = o.memoryTotalLimit;
    g.mustUseAllHashfunctions = o.mustUseAllHashfunctions;
    g.save_binary_reads_to = o.save_binary_reads_to;
    g.load_binary_reads_from = o.load_binary_reads_from;
    g.save_hashtables_to = o.save_hashtables_to;
    g.load_hashtables_from = o.load_hashtables_from;
    g.pairType = o.pairType == SequencePairType::PairedEnd ? care_gb300::SequencePairType::PairedEnd
                                                            : care_gb300::SequencePairType::SingleEnd;
    g.outputdirectory = o.outputdirectory;
    g.tempdirectory = o.tempdirectory;
    g.inputfiles = o.inputfiles;
    g.outputfilenames = o.outputfilenames;
    g.gpuBatched = true;  // the batched driver: the plain driver's output, faster
    return g;
}

void performCorrection(ProgramOptions programOptions) {
    care_gb300::performCorrection(toGb300Options(programOptions));
}

void performCorrectionOutToQueue(ProgramOptions programOptions,
                                 moodycamel::ReaderWriterQueue<std::pair<char*, int>>* Q1,
                                 moodycamel::ReaderWriterQueue<std::pair<char*, int>>* Q2,
                                 std::atomic_int* producerDone, std::atomic_int* careStartWrite, int* changNum) {
    care_gb300::performCorrectionOutToQueue(toGb300Options(programOptions), Q1, Q2, producerDone, careStartWrite,
                                            changNum);
}

}  // namespace care
