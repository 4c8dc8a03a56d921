// Test infrastructure only: a minimal driver linked against the reference's
// own CARE objects (compiled from their sources by oracle/ref.mk) so that the
// reference's corrected output can be produced for parity fixtures and for the
// CPU baseline.  Nothing in the product path links or runs this file.
//
// It fills care::ProgramOptions (include/options.hpp:36-99 of the reference)
// the way main_correction does (src/main_correct_cpu.cpp:63-158: batchsize
// forced to 16, OMP thread count set) and calls care::performCorrection
// (src/dispatch_care_correct_cpu.cpp:52-252), timing cpu::correct_cpu's STEP2
// region is not possible from outside, so the whole call is timed and the
// reference's own STEP prints are left on stderr.

#include <dispatch_care_correct_cpu.hpp>
#include <options.hpp>

#include <omp.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static void usage() {
    std::fprintf(stderr,
                 "ref_driver -i in1 [-i in2] -o out1 [-o out2] -d outdir -c cov "
                 "[-k 20] [-h 48] [-t threads] [--pe] [-q] [--candidates] "
                 "[--exclude-ambiguous] [--forest file] [--print] [--labels] [--new-columns n] [--tempdir dir] "
                 "[--quality-bits 1|2|8] [--fixed-reads n]\n");
}

int main(int argc, char** argv) {
    care::ProgramOptions o;
    o.batchsize = 16;
    o.threads = 1;
    o.estimatedCoverage = 30.0f;
    o.kmerlength = 20;
    o.autodetectKmerlength = false;
    o.numHashFunctions = 48;
    o.qualityScoreBits = 8;
    o.memoryTotalLimit = std::size_t(24) << 30;
    o.memoryForHashtables = std::size_t(20) << 30;
    o.pairType = care::SequencePairType::SingleEnd;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) { usage(); std::exit(2); }
            return argv[++i];
        };
        if (a == "-i") o.inputfiles.push_back(next());
        else if (a == "-o") o.outputfilenames.push_back(next());
        else if (a == "-d") o.outputdirectory = next();
        else if (a == "-c") o.estimatedCoverage = std::stof(next());
        else if (a == "-k") {
            o.kmerlength = std::stoi(next());
            o.autodetectKmerlength = (o.kmerlength == 0);
        }
        else if (a == "-h") o.numHashFunctions = std::stoi(next());
        else if (a == "-t") o.threads = std::stoi(next());
        else if (a == "--pe") o.pairType = care::SequencePairType::PairedEnd;
        else if (a == "-q") o.useQualityScores = true;
        else if (a == "--candidates") o.correctCandidates = true;
        else if (a == "--exclude-ambiguous") o.excludeAmbiguousReads = true;
        else if (a == "--forest") {
            o.correctionType = care::CorrectionType::Forest;
            o.mlForestfileAnchor = next();
            o.mlForestfileCands = o.mlForestfileAnchor;
        }
        else if (a == "--print") {
            o.correctionType = care::CorrectionType::Print;
        }
        else if (a == "--labels") o.outputCorrectionQualityLabels = true;
        else if (a == "--new-columns") o.new_columns_to_correct = std::stoi(next());
        else if (a == "--tempdir") o.tempdirectory = next();
        else if (a == "--quality-bits") o.qualityScoreBits = std::stoi(next());
        else if (a == "--fixed-reads") o.fixedNumberOfReads = std::stoull(next());
        else { usage(); return 2; }
    }
    if (o.inputfiles.empty() || o.outputfilenames.size() != o.inputfiles.size() ||
        o.outputdirectory.empty()) {
        usage();
        return 2;
    }
    if (o.tempdirectory.empty()) o.tempdirectory = o.outputdirectory;
    omp_set_num_threads(o.threads);
    const auto t0 = std::chrono::steady_clock::now();
    care::performCorrection(o);
    const auto t1 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "REF_DRIVER_SECONDS %.6f\n",
                 std::chrono::duration<double>(t1 - t0).count());
    return 0;
}
