// Test infrastructure only: dumps the reference's per-anchor intermediate
// results (signatures, candidate ids, both alignments, orientation, filtered
// candidates, MSA consensus/support after refinement, anchor correction) for a
// range of anchors, by running the steps of CpuErrorCorrector::process
// (include/corrector.hpp:145-312 of the reference) one by one.  The private
// member functions are reached by compiling the header with `private` mapped
// to `public` in this translation unit only; the reference objects it links
// against are unchanged.  Output is a line-oriented text format read by
// tests/golden/make_golden.py; floats are written as their IEEE-754 bit
// patterns so the comparison is exact.

#include <config.hpp>
#include <options.hpp>
#include <chunkedreadstorageconstruction.hpp>
#include <chunkedreadstorage.hpp>
#include <cpuminhasherconstruction.hpp>
#include <ordinaryminhasher.hpp>
#include <cpusequencehasher.hpp>

#define private public
#include <corrector.hpp>
#undef private

#include <omp.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace care;

static unsigned fbits(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}

int main(int argc, char** argv) {
    ProgramOptions o;
    o.batchsize = 16;
    o.threads = 4;
    o.estimatedCoverage = 30.0f;
    o.kmerlength = 20;
    o.numHashFunctions = 48;
    o.qualityScoreBits = 8;
    o.memoryTotalLimit = std::size_t(24) << 30;
    o.memoryForHashtables = std::size_t(20) << 30;
    long first = 0, last = 100, sigreads = 100;
    std::string outpath;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto next = [&]() -> std::string { return argv[++i]; };
        if (a == "-i") o.inputfiles.push_back(next());
        else if (a == "-c") o.estimatedCoverage = std::stof(next());
        else if (a == "-k") o.kmerlength = std::stoi(next());
        else if (a == "-q") o.useQualityScores = true;
        else if (a == "--first") first = std::stol(next());
        else if (a == "--last") last = std::stol(next());
        else if (a == "--sigreads") sigreads = std::stol(next());
        else if (a == "--out") outpath = next();
    }
    omp_set_num_threads(o.threads);
    FILE* out = outpath.empty() ? stdout : std::fopen(outpath.c_str(), "w");

    std::unique_ptr<ChunkedReadStorage> rs = constructChunkedReadStorageFromFiles(o);
    auto mhpair = constructCpuMinhasherFromCpuReadStorage(o, *rs, CpuMinhasherType::Ordinary);
    CpuMinhasher* mh = mhpair.first.get();

    const int Lmax = rs->getSequenceLengthUpperBound();
    const std::size_t pitch = SequenceHelpers::getEncodedNumInts2Bit(Lmax);
    const read_number nReads = rs->getNumberOfReads();
    std::fprintf(out, "NREADS %u LMAX %d MAPS %d\n", nReads, Lmax, mh->getNumberOfMaps());

    // signatures of the first reads, as CPUSequenceHasher::hash gives them
    {
        CPUSequenceHasher<kmer_type> hasher;
        std::vector<unsigned int> seq(pitch);
        for (long r = 0; r < sigreads && r < long(nReads); r++) {
            read_number id = r;
            int len = 0;
            rs->gatherSequenceLengths(&len, &id, 1);
            rs->gatherSequences(seq.data(), pitch, &id, 1);
            auto h = hasher.hash(seq.data(), len, o.kmerlength, mh->getNumberOfMaps(), 0);
            std::fprintf(out, "SIG %u", id);
            for (auto v : h) std::fprintf(out, " %llx", (unsigned long long)v);
            std::fprintf(out, "\n");
        }
    }

    ReadCorrectionFlags flags(nReads);
    ClfAgent clf(o);
    CpuErrorCorrector ec(pitch, Lmax, Lmax, o, *mh, *rs, flags, clf);
    std::vector<unsigned int> anchorData(pitch);
    std::vector<char> anchorQual(Lmax);
    for (long a = first; a < last && a < long(nReads); a++) {
        read_number id = a;
        int len = 0;
        rs->gatherSequenceLengths(&len, &id, 1);
        rs->gatherSequences(anchorData.data(), pitch, &id, 1);
        if (o.useQualityScores) rs->gatherQualities(anchorQual.data(), Lmax, &id, 1);
        CpuErrorCorrectorInput input;
        input.anchorReadId = id;
        input.encodedAnchor = anchorData.data();
        input.anchorQualityscores = anchorQual.data();
        input.anchorLength = len;
        CpuErrorCorrectorTask task = ec.makeTask(input);
        ec.determineCandidateReadIds(task);
        ec.computePairFlags(task);
        std::fprintf(out, "ANCHOR %u LEN %d\nCAND %zu", id, len, task.candidateReadIds.size());
        for (auto c : task.candidateReadIds) std::fprintf(out, " %u", c);
        std::fprintf(out, "\n");
        if (task.candidateReadIds.empty()) { std::fprintf(out, "END\n"); continue; }
        ec.getCandidateSequenceData(task);
        ec.computeReverseComplementCandidates(task);
        ec.getCandidateAlignments(task);
        for (std::size_t i = 0; i < task.candidateReadIds.size(); i++) {
            const auto& f = task.alignments[i];
            const auto& r = task.revcAlignments[i];
            std::fprintf(out, "ALN %u %d %d %d %d %d %d %d %d %d %d %d\n", task.candidateReadIds[i],
                         f.score, f.overlap, f.shift, f.nOps, int(f.isValid),
                         r.score, r.overlap, r.shift, r.nOps, int(r.isValid),
                         int(task.alignmentFlags[i]));
        }
        ec.filterCandidatesByAlignmentFlag(task);
        if (task.candidateReadIds.empty()) { std::fprintf(out, "END\n"); continue; }
        ec.filterCandidatesByAlignmentMismatchRatio(task);
        std::fprintf(out, "KEPT %zu", task.candidateReadIds.size());
        for (auto c : task.candidateReadIds) std::fprintf(out, " %u", c);
        std::fprintf(out, "\n");
        if (task.candidateReadIds.empty()) { std::fprintf(out, "END\n"); continue; }
        if (o.useQualityScores) {
            ec.getCandidateQualities(task);
            ec.reverseQualitiesOfRCAlignments(task);
        }
        ec.makeCandidateStrings(task);
        ec.alignmentsComputeWeightsAndAoStoSoA(task);
        for (std::size_t i = 0; i < task.candidateReadIds.size(); i++) {
            std::fprintf(out, "W %u %d %x\n", task.candidateReadIds[i], task.alignmentShifts[i],
                         fbits(task.alignmentWeights[i]));
        }
        ec.buildMultipleSequenceAlignment(task);
        ec.refineMSA(task);
        const auto& msa = task.multipleSequenceAlignment;
        std::fprintf(out, "MSA %d %d %d %d\n", msa.nCandidates, msa.nColumns,
                     msa.anchorColumnsBegin_incl, msa.anchorColumnsEnd_excl);
        std::fprintf(out, "CONS %.*s\n", msa.nColumns, msa.consensus.data());
        std::fprintf(out, "SUP");
        for (int c = 0; c < msa.nColumns; c++) std::fprintf(out, " %x", fbits(msa.support[c]));
        std::fprintf(out, "\nCOV");
        for (int c = 0; c < msa.nColumns; c++) std::fprintf(out, " %d", msa.coverage[c]);
        std::fprintf(out, "\n");
        ec.correctAnchor(task);
        std::fprintf(out, "PROP %x %x %d %d %d\n", fbits(task.msaProperties.avg_support),
                     fbits(task.msaProperties.min_support), task.msaProperties.min_coverage,
                     task.msaProperties.max_coverage, int(task.msaProperties.isHQ));
        std::fprintf(out, "CORR %d %s\n", int(task.anchorCorrection.isCorrected),
                     task.anchorCorrection.isCorrected ? task.anchorCorrection.correctedSequence.c_str() : "-");
        std::fprintf(out, "END\n");
    }
    if (out != stdout) std::fclose(out);
    return 0;
}
