// FASTA/FASTQ input and output for the host layer.
//
// reference: include/readlibraryio.hpp:121-403 and src/readlibraryio.cpp
// (kseqpp reader, paired files read alternately so read 2i comes from file 1
// and read 2i+1 from file 2; writers emit "@header\nSEQ\n+\nQUAL\n" or
// ">header\nSEQ\n").  Gzip input/output when zlib is available at build time.
#ifndef CARE_HOST_SEQIO_H
#define CARE_HOST_SEQIO_H

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace care_gb300 {

enum class FileFormat { FASTA, FASTQ, FASTAGZ, FASTQGZ, NONE };

struct ReadRecord {
    std::string header;  // header line without the leading '@' / '>'
    std::string sequence;
    std::string quality;
};

// All reads of a set, sequences and qualities back to back.
struct ReadSet {
    std::vector<std::string> headers;
    std::vector<char> sequences;
    std::vector<char> qualities;
    std::vector<uint64_t> offsets{0};
    std::vector<uint8_t> fileId;  // which input file a read came from
    bool hasQualities = true;

    uint64_t size() const { return offsets.size() - 1; }
    void add(ReadRecord&& r, uint8_t file);
};

FileFormat detectFormat(const std::string& path);

class SequenceReader {
public:
    explicit SequenceReader(const std::string& path);
    ~SequenceReader();
    // false at end of file; throws std::runtime_error on malformed input
    bool next(ReadRecord& out);

private:
    struct Impl;
    std::unique_ptr<Impl> impl;
};

class SequenceWriter {
public:
    SequenceWriter(const std::string& path, FileFormat format);
    ~SequenceWriter();
    void write(const std::string& header, const char* seq, size_t len, const std::string& qual);
    // bytes of already formatted records
    void writeRaw(const char* data, size_t len);

private:
    struct Impl;
    std::unique_ptr<Impl> impl;
};

// The whole (decompressed) content of a plain or gzip file, in a buffer that
// is not zero-filled first; a plain file is read by parallel pread calls.
struct FileBytes {
    std::unique_ptr<char[]> data;
    size_t size = 0;
};
FileBytes readFileBytes(const std::string& path);

// Reads all files of one input group: a single-end file, an interleaved
// paired file, or two paired files read alternately.
void readSingleFile(const std::string& path, ReadSet& out, uint8_t fileId);
void readPairedFiles(const std::string& path1, const std::string& path2, ReadSet& out);

}  // namespace care_gb300

#endif
