// Test driver for the queue protocol of the host layer
// (care_gb300::performCorrectionToSink, the body of performCorrectionOutToQueue):
// collects the chunks of every queue into one file per queue and checks that
// each chunk is under 1 MiB and holds whole FASTQ records.
//
//   queue_driver <device|host> <se|pe> <out_prefix> <input> [input2]
//
// prints "records <changNum> reads <n> chunks <k> device <0|1>"; exit code 1 on
// a malformed chunk.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "care_host.h"

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    care_gb300::ProgramOptions o;
    o.deviceFileIO = std::string(argv[1]) == "device";
    const bool pe = std::string(argv[2]) == "pe";
    const std::string prefix = argv[3];
    for (int i = 4; i < argc; i++) o.inputfiles.push_back(argv[i]);
    o.estimatedCoverage = 30.0f;
    o.kmerlength = 20;
    o.pairType = pe ? care_gb300::SequencePairType::PairedEnd : care_gb300::SequencePairType::SingleEnd;
    std::vector<FILE*> out;
    for (int f = 0; f < (pe ? 2 : 1); f++) out.push_back(std::fopen((prefix + std::to_string(f) + ".fq").c_str(), "wb"));
    int changNum = -1;
    long chunks = 0;
    bool bad = false;
    auto rep = care_gb300::performCorrectionToSink(
        o, [&](int n) { changNum = n; },
        [&](int f, char* data, int size) {
            chunks++;
            if (size <= 0 || size >= (1 << 20) || data[0] != '@' || data[size - 1] != '\n') bad = true;
            long lines = 0;
            for (int i = 0; i < size; i++) lines += data[i] == '\n';
            if (lines % 4) bad = true;
            std::fwrite(data, 1, (size_t)size, out[f]);
            delete[] data;
            return true;
        });
    for (FILE* f : out) std::fclose(f);
    std::printf("records %d reads %llu chunks %ld device %d\n", changNum, (unsigned long long)rep.reads, chunks,
                rep.deviceFileIO ? 1 : 0);
    return bad ? 1 : 0;
}
