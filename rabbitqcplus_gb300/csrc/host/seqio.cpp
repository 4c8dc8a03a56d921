#include "seqio.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <thread>

#ifdef CG_HAVE_ZLIB
#include <zlib.h>
#endif

namespace care_gb300 {

void ReadSet::add(ReadRecord&& r, uint8_t file) {
    headers.push_back(std::move(r.header));
    sequences.insert(sequences.end(), r.sequence.begin(), r.sequence.end());
    if (r.quality.size() != r.sequence.size()) hasQualities = false;
    if (hasQualities) qualities.insert(qualities.end(), r.quality.begin(), r.quality.end());
    offsets.push_back(sequences.size());
    fileId.push_back(file);
}

static bool endsWith(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// line source over a plain or gzip file
struct LineSource {
    FILE* f = nullptr;
#ifdef CG_HAVE_ZLIB
    gzFile gz = nullptr;
#endif
    std::vector<char> buf = std::vector<char>(1 << 20);
    size_t pos = 0, end = 0;
    bool eof = false;

    explicit LineSource(const std::string& path) {
#ifdef CG_HAVE_ZLIB
        gz = gzopen(path.c_str(), "rb");
        if (!gz) throw std::runtime_error("cannot open " + path);
        gzbuffer(gz, 1 << 20);
#else
        if (endsWith(path, ".gz")) throw std::runtime_error("gzip input needs zlib: " + path);
        f = std::fopen(path.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + path);
#endif
    }
    ~LineSource() {
        if (f) std::fclose(f);
#ifdef CG_HAVE_ZLIB
        if (gz) gzclose(gz);
#endif
    }
    bool fill() {
        if (eof) return false;
        if (pos > 0) {
            std::memmove(buf.data(), buf.data() + pos, end - pos);
            end -= pos;
            pos = 0;
        }
        if (end == buf.size()) buf.resize(buf.size() * 2);
        long got;
#ifdef CG_HAVE_ZLIB
        got = gzread(gz, buf.data() + end, (unsigned)(buf.size() - end));
#else
        got = (long)std::fread(buf.data() + end, 1, buf.size() - end, f);
#endif
        if (got <= 0) {
            eof = true;
            return false;
        }
        end += (size_t)got;
        return true;
    }
    // next line without the trailing newline (and '\r'); false at end
    bool line(std::string& out) {
        while (true) {
            const char* s = buf.data() + pos;
            const void* nl = std::memchr(s, '\n', end - pos);
            if (nl) {
                size_t len = (const char*)nl - s;
                out.assign(s, len);
                pos += len + 1;
                if (!out.empty() && out.back() == '\r') out.pop_back();
                return true;
            }
            if (!fill()) {
                if (pos < end) {
                    out.assign(buf.data() + pos, end - pos);
                    pos = end;
                    if (!out.empty() && out.back() == '\r') out.pop_back();
                    return true;
                }
                return false;
            }
        }
    }
    int peek() {
        if (pos == end && !fill()) return -1;
        return (unsigned char)buf[pos];
    }
};

struct SequenceReader::Impl {
    LineSource src;
    std::string line;
    explicit Impl(const std::string& p) : src(p) {}
};

SequenceReader::SequenceReader(const std::string& path) : impl(new Impl(path)) {}
SequenceReader::~SequenceReader() = default;

bool SequenceReader::next(ReadRecord& out) {
    auto& L = impl->line;
    do {
        if (!impl->src.line(L)) return false;
    } while (L.empty());
    if (L[0] == '@') {
        out.header.assign(L, 1, std::string::npos);
        out.sequence.clear();
        // sequence lines until '+'
        while (impl->src.line(L)) {
            if (!L.empty() && L[0] == '+') break;
            out.sequence += L;
        }
        out.quality.clear();
        while (out.quality.size() < out.sequence.size() && impl->src.line(L)) out.quality += L;
        if (out.quality.size() != out.sequence.size())
            throw std::runtime_error("truncated FASTQ record " + out.header);
        return true;
    }
    if (L[0] == '>') {
        out.header.assign(L, 1, std::string::npos);
        out.sequence.clear();
        out.quality.clear();
        while (impl->src.peek() != -1 && impl->src.peek() != '>') {
            if (!impl->src.line(L)) break;
            out.sequence += L;
        }
        return true;
    }
    throw std::runtime_error("not a FASTA/FASTQ record: " + L.substr(0, 40));
}

FileFormat detectFormat(const std::string& path) {
    LineSource s(path);
    std::string first;
    while (s.line(first) && first.empty()) {
    }
    const bool gz = endsWith(path, ".gz");
    if (!first.empty() && first[0] == '@') return gz ? FileFormat::FASTQGZ : FileFormat::FASTQ;
    if (!first.empty() && first[0] == '>') return gz ? FileFormat::FASTAGZ : FileFormat::FASTA;
    return FileFormat::NONE;
}

struct SequenceWriter::Impl {
    FileFormat fmt;
    FILE* f = nullptr;
#ifdef CG_HAVE_ZLIB
    gzFile gz = nullptr;
#endif
    std::string buf;
    void flush() {
        if (buf.empty()) return;
#ifdef CG_HAVE_ZLIB
        if (gz) {
            gzwrite(gz, buf.data(), (unsigned)buf.size());
            buf.clear();
            return;
        }
#endif
        std::fwrite(buf.data(), 1, buf.size(), f);
        buf.clear();
    }
};

SequenceWriter::SequenceWriter(const std::string& path, FileFormat format) : impl(new Impl()) {
    impl->fmt = format;
    if (format == FileFormat::FASTQGZ || format == FileFormat::FASTAGZ) {
#ifdef CG_HAVE_ZLIB
        impl->gz = gzopen(path.c_str(), "wb");
        if (!impl->gz) throw std::runtime_error("cannot open " + path + " for writing");
        return;
#else
        throw std::runtime_error("gzip output needs zlib");
#endif
    }
    impl->f = std::fopen(path.c_str(), "wb");
    if (!impl->f) throw std::runtime_error("cannot open " + path + " for writing");
}

SequenceWriter::~SequenceWriter() {
    impl->flush();
    if (impl->f) std::fclose(impl->f);
#ifdef CG_HAVE_ZLIB
    if (impl->gz) gzclose(impl->gz);
#endif
}

void SequenceWriter::write(const std::string& header, const char* seq, size_t len, const std::string& qual) {
    const bool fq = impl->fmt == FileFormat::FASTQ || impl->fmt == FileFormat::FASTQGZ;
    auto& b = impl->buf;
    b.push_back(fq ? '@' : '>');
    b += header;
    b.push_back('\n');
    b.append(seq, len);
    b.push_back('\n');
    if (fq) {
        b += "+\n";
        b += qual;
        b.push_back('\n');
    }
    if (b.size() > (1u << 22)) impl->flush();
}

namespace {

// len bytes of the file at offset off into buf, as 32 MiB parts read by up to
// 16 threads (one thread copies page-cache data at a few GB/s)
bool parallelRead(int fd, char* buf, size_t len, off_t off) {
    constexpr size_t kPart = size_t(32) << 20;
    const size_t parts = (len + kPart - 1) / kPart;
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nthreads = std::min<size_t>({parts, hw, 16});
    std::atomic<size_t> next{0};
    std::atomic<bool> ok{true};
    auto work = [&]() {
        for (size_t p = next.fetch_add(1); p < parts && ok; p = next.fetch_add(1)) {
            size_t done = p * kPart;
            const size_t end = std::min(len, done + kPart);
            while (done < end) {
                const ssize_t r = ::pread(fd, buf + done, end - done, off + (off_t)done);
                if (r < 0 && errno == EINTR) continue;
                if (r <= 0) {
                    ok = false;
                    return;
                }
                done += (size_t)r;
            }
        }
    };
    std::vector<std::thread> threads;
    for (size_t t = 1; t < nthreads; t++) threads.emplace_back(work);
    work();
    for (std::thread& t : threads) t.join();
    return ok;
}

}  // namespace

void SequenceWriter::writeRaw(const char* data, size_t len) {
    impl->flush();
#ifdef CG_HAVE_ZLIB
    if (impl->gz) {
        const size_t step = 1u << 30;  // gzwrite takes an unsigned count
        for (size_t done = 0; done < len; done += step) {
            const size_t k = len - done < step ? len - done : step;
            if (gzwrite(impl->gz, data + done, (unsigned)k) != (int)k) throw std::runtime_error("gzip write failed");
        }
        return;
    }
#endif
    // plain: one stream (writes to one file do not run in parallel: the
    // kernel serialises them on the file)
    if (len > 0 && std::fwrite(data, 1, len, impl->f) != len) throw std::runtime_error("write failed");
}

FileBytes readFileBytes(const std::string& path) {
    FileBytes out;
    const int fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) throw std::runtime_error("cannot open " + path);
    struct stat sb;
    unsigned char magic[2] = {0, 0};
    const bool gzipped = ::pread(fd, magic, 2, 0) == 2 && magic[0] == 0x1f && magic[1] == 0x8b;
    if (!gzipped) {  // plain: the whole file by parallel reads
        if (::fstat(fd, &sb) != 0) {
            ::close(fd);
            throw std::runtime_error("cannot read " + path);
        }
        out.size = (size_t)sb.st_size;
        out.data.reset(new char[std::max<size_t>(out.size, 1)]);
        const bool ok = parallelRead(fd, out.data.get(), out.size, 0);
        ::close(fd);
        if (!ok) throw std::runtime_error("cannot read " + path);
        return out;
    }
    ::close(fd);
#ifdef CG_HAVE_ZLIB
    gzFile gz = gzopen(path.c_str(), "rb");
    if (!gz) throw std::runtime_error("cannot open " + path);
    gzbuffer(gz, 1 << 20);
    size_t cap = size_t(1) << 24;
    out.data.reset(new char[cap]);
    while (true) {
        if (out.size == cap) {
            std::unique_ptr<char[]> bigger(new char[2 * cap]);
            std::memcpy(bigger.get(), out.data.get(), out.size);
            out.data = std::move(bigger);
            cap *= 2;
        }
        const size_t want = std::min<size_t>(cap - out.size, 1u << 30);
        const int got = gzread(gz, out.data.get() + out.size, (unsigned)want);
        if (got < 0) {
            gzclose(gz);
            throw std::runtime_error("cannot read " + path);
        }
        if (got == 0) break;
        out.size += (size_t)got;
    }
    gzclose(gz);
#else
    throw std::runtime_error("gzip input needs zlib: " + path);
#endif
    return out;
}

void readSingleFile(const std::string& path, ReadSet& out, uint8_t fileId) {
    SequenceReader r(path);
    ReadRecord rec;
    while (r.next(rec)) out.add(std::move(rec), fileId);
}

void readPairedFiles(const std::string& path1, const std::string& path2, ReadSet& out) {
    SequenceReader r1(path1), r2(path2);
    ReadRecord a, b;
    while (true) {
        const bool ga = r1.next(a);
        const bool gb = ga && r2.next(b);
        if (!ga || !gb) break;
        out.add(std::move(a), 0);
        out.add(std::move(b), 1);
    }
}

}  // namespace care_gb300
