// Test driver for the drop-in shim (rabbitqcplus_gb300/csrc/host/
// dispatch_care_correct_gpu.cpp) inside a RabbitQCPlus-shaped program.
//
// Linked (oracle/ref.mk, target care_gpu_dropin) with RabbitQCPlus's own
// main_correction (src/main_correct_cpu.cpp, compiled from the reference's
// source where it lies), the reference's CARE objects minus
// dispatch_care_correct_cpu.o, the shim in its place, and libcaregpu.so.
//
//   care_gpu_dropin --mapping
//       converts a care::ProgramOptions whose every forwarded field differs
//       from its default and prints "mapping ok" when the GB300 options carry
//       each value (exit 1 and the field's name otherwise);
//   care_gpu_dropin --queue <threads> <in.fq> <out.fq>
//       runs the correction the way SeQc::careProcess does (the argument list
//       of src/seqc.cpp:94-262, main_correction on its own std::thread,
//       src/seqc.cpp:659-672) into a moodycamel::ReaderWriterQueue of
//       capacity 1 << 20 (src/seqc.cpp:69-71), drains it the way
//       FileReader::Read does (src/FileReader.h:221-290: try_dequeue, copy,
//       delete[] the chunk) into out.fq and prints "changNum <n> bytes <b>";
//       an exception from the correction thread is printed as
//       "error: <what>" with exit code 3.
#include <dispatch_care_correct_cpu.hpp>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "main_correct_cpu.h"

#include "care_host.h"

namespace care {
care_gb300::ProgramOptions toGb300Options(const ProgramOptions& o);
}

static int checkMapping() {
    care::ProgramOptions o;
    o.min_overlap = 31;
    o.maxErrorRate = 0.25f;
    o.min_overlap_ratio = 0.35f;
    o.excludeAmbiguousReads = true;
    o.correctCandidates = true;
    o.useQualityScores = true;
    o.autodetectKmerlength = true;
    o.outputCorrectionQualityLabels = true;
    o.gzoutput = true;
    o.estimatedCoverage = 17.0f;
    o.estimatedErrorrate = 0.07f;
    o.m_coverage = 0.65f;
    o.batchsize = 7;
    o.new_columns_to_correct = 21;
    o.kmerlength = 19;
    o.numHashFunctions = 33;
    o.correctionType = care::CorrectionType::Forest;
    o.correctionTypeCands = care::CorrectionType::Forest;
    o.thresholdAnchor = 0.55f;
    o.thresholdCands = 0.45f;
    o.pairedFilterThreshold = 0.07f;
    o.maxForestTreesAnchor = 9;
    o.maxForestTreesCands = 8;
    o.mlForestfileAnchor = "anchor.rf";
    o.mlForestfileCands = "cands.rf";
    o.showProgress = true;
    o.threads = 5;
    o.deviceIds = {1};
    o.qualityScoreBits = 2;
    o.fixedNumberOfReads = 1234;
    o.memoryForHashtables = 1ull << 33;
    o.memoryTotalLimit = 1ull << 34;
    o.mustUseAllHashfunctions = true;
    o.save_binary_reads_to = "a";
    o.load_binary_reads_from = "b";
    o.save_hashtables_to = "c";
    o.load_hashtables_from = "d";
    o.pairType = care::SequencePairType::PairedEnd;
    o.outputdirectory = "outdir";
    o.tempdirectory = "tmpdir";
    o.inputfiles = {"in1.fq", "in2.fq"};
    o.outputfilenames = {"o1.fq", "o2.fq"};
    const care_gb300::ProgramOptions g = care::toGb300Options(o);
#define SAME(field, expr)                                   \
    if (!(expr)) {                                          \
        std::printf("mapping differs: %s\n", field);        \
        return 1;                                           \
    }
    SAME("min_overlap", g.min_overlap == 31);
    SAME("maxErrorRate", g.maxErrorRate == 0.25f);
    SAME("min_overlap_ratio", g.min_overlap_ratio == 0.35f);
    SAME("excludeAmbiguousReads", g.excludeAmbiguousReads);
    SAME("correctCandidates", g.correctCandidates);
    SAME("useQualityScores", g.useQualityScores);
    SAME("autodetectKmerlength", g.autodetectKmerlength);
    SAME("outputCorrectionQualityLabels", g.outputCorrectionQualityLabels);
    SAME("gzoutput", g.gzoutput);
    SAME("estimatedCoverage", g.estimatedCoverage == 17.0f);
    SAME("estimatedErrorrate", g.estimatedErrorrate == 0.07f);
    SAME("m_coverage", g.m_coverage == 0.65f);
    SAME("batchsize", g.batchsize == 7);
    SAME("new_columns_to_correct", g.new_columns_to_correct == 21);
    SAME("kmerlength", g.kmerlength == 19);
    SAME("numHashFunctions", g.numHashFunctions == 33);
    SAME("correctionType", g.correctionType == care_gb300::CorrectionType::Forest);
    SAME("correctionTypeCands", g.correctionTypeCands == care_gb300::CorrectionType::Forest);
    SAME("thresholdAnchor", g.thresholdAnchor == 0.55f);
    SAME("thresholdCands", g.thresholdCands == 0.45f);
    SAME("pairedFilterThreshold", g.pairedFilterThreshold == 0.07f);
    SAME("maxForestTreesAnchor", g.maxForestTreesAnchor == 9);
    SAME("maxForestTreesCands", g.maxForestTreesCands == 8);
    SAME("mlForestfileAnchor", g.mlForestfileAnchor == "anchor.rf");
    SAME("mlForestfileCands", g.mlForestfileCands == "cands.rf");
    SAME("showProgress", g.showProgress);
    SAME("threads", g.threads == 5);
    SAME("deviceIds", g.deviceIds.size() == 1 && g.deviceIds[0] == 1);
    SAME("qualityScoreBits", g.qualityScoreBits == 2);
    SAME("fixedNumberOfReads", g.fixedNumberOfReads == 1234);
    SAME("memoryForHashtables", g.memoryForHashtables == (1ull << 33));
    SAME("memoryTotalLimit", g.memoryTotalLimit == (1ull << 34));
    SAME("mustUseAllHashfunctions", g.mustUseAllHashfunctions);
    SAME("save_binary_reads_to", g.save_binary_reads_to == "a");
    SAME("load_binary_reads_from", g.load_binary_reads_from == "b");
    SAME("save_hashtables_to", g.save_hashtables_to == "c");
    SAME("load_hashtables_from", g.load_hashtables_from == "d");
    SAME("pairType", g.pairType == care_gb300::SequencePairType::PairedEnd);
    SAME("outputdirectory", g.outputdirectory == "outdir");
    SAME("tempdirectory", g.tempdirectory == "tmpdir");
    SAME("inputfiles", g.inputfiles == o.inputfiles);
    SAME("outputfilenames", g.outputfilenames == o.outputfilenames);
#undef SAME
    // the options it refuses rather than ignore
    bool refused = false;
    try {
        care_gb300::validateOptions(g);
    } catch (const std::exception&) {
        refused = true;
    }
    if (!refused) {
        std::printf("mapping: refused options were accepted\n");
        return 1;
    }
    std::printf("mapping ok\n");
    return 0;
}

static int runQueue(const char* threads, const char* in, const char* out) {
    // the argument list SeQc::careProcess builds (src/seqc.cpp:94-262) for
    // `--correctWithCare --coverage 30 --pairmode SE`
    std::vector<std::string> args = {"./RabbitQCPlus", "-i", in, "-d", "./", "-o", "tmp.fq", "-c", "30",
                                     "-t", threads, "--pairmode", "SE", "--kmerlength", "20"};
    std::vector<char*> argv;
    for (auto& a : args) argv.push_back(&a[0]);
    moodycamel::ReaderWriterQueue<std::pair<char*, int>> Q(1 << 20);
    std::atomic_int producerDone{0}, careStartWrite{0}, careDone{0};
    int changNum = 0;
    std::string error;
    std::thread carer([&] {
        try {
            main_correction((int)argv.size(), argv.data(), &Q, &Q, &producerDone, &careStartWrite, &changNum);
        } catch (const std::exception& e) {
            error = e.what();
            careStartWrite = 1;
        }
        careDone = 1;
    });
    while (careStartWrite == 0) usleep(100);
    FILE* f = std::fopen(out, "wb");
    unsigned long long bytes = 0;
    if (changNum != 0) {
        std::pair<char*, int> now;
        while (true) {
            if (Q.try_dequeue(now)) {
                if (f) std::fwrite(now.first, 1, (size_t)now.second, f);
                bytes += (unsigned long long)now.second;
                delete[] now.first;
                continue;
            }
            if (careDone == 1 && Q.size_approx() == 0) break;
            usleep(1000);
        }
    }
    carer.join();
    if (f) std::fclose(f);
    if (!error.empty()) {
        std::printf("error: %s\n", error.c_str());
        return 3;
    }
    std::printf("changNum %d bytes %llu\n", changNum, bytes);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && std::strcmp(argv[1], "--mapping") == 0) return checkMapping();
    if (argc >= 5 && std::strcmp(argv[1], "--queue") == 0) return runQueue(argv[2], argv[3], argv[4]);
    std::fprintf(stderr, "usage: care_gpu_dropin --mapping | --queue <threads> <in.fq> <out.fq>\n");
    return 2;
}
