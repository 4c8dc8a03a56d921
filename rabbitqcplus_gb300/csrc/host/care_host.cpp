// Host side of the drop-in boundary (see care_host.h).
#include "care_host.h"

#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <exception>
#include <fstream>
#include <iterator>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "care_files.h"
#include "seqio.h"

namespace care_gb300 {

cg_options toCgOptions(const ProgramOptions& o) {
    cg_options c;
    cg_default_options(&c);
    c.kmerlength = o.autodetectKmerlength ? 0 : o.kmerlength;
    c.num_hash_functions = o.numHashFunctions;
    c.estimated_coverage = o.estimatedCoverage;
    c.estimated_errorrate = o.estimatedErrorrate;
    c.m_coverage = o.m_coverage;
    c.max_error_rate = o.maxErrorRate;
    c.min_overlap_ratio = o.min_overlap_ratio;
    c.min_overlap = o.min_overlap;
    c.paired_filter_threshold = o.pairedFilterThreshold;
    c.new_columns_to_correct = o.new_columns_to_correct;
    c.use_quality_scores = o.useQualityScores;
    c.exclude_ambiguous_reads = o.excludeAmbiguousReads;
    c.correct_candidates = o.correctCandidates;
    c.pair_mode = o.pairType == SequencePairType::PairedEnd ? CG_PAIR_PE : CG_PAIR_SE;
    c.correction_type = (int)o.correctionType;
    c.threshold_anchor = o.thresholdAnchor;
    c.device = o.deviceIds.empty() ? 0 : o.deviceIds[0];
    c.driver = o.gpuBatched ? CG_DRIVER_BATCHED : CG_DRIVER_PLAIN;
    c.quality_score_bits = o.qualityScoreBits;
    c.fixed_number_of_reads = (uint32_t)std::min<std::size_t>(o.fixedNumberOfReads, 0xffffffffu);
    std::size_t mem = o.memoryForHashtables;
    if (o.memoryTotalLimit && (!mem || o.memoryTotalLimit < mem)) mem = o.memoryTotalLimit;  // src/options.cpp:296
    c.hashtable_memory_bytes = mem;
    return c;
}

void validateOptions(const ProgramOptions& o) {
    if (o.correctionType == CorrectionType::Print || o.correctionTypeCands == CorrectionType::Print)
        // the reference then writes classifier features instead of an output
        // file (src/dispatch_care_correct_cpu.cpp:180)
        throw std::runtime_error("correction type Print is not supported");
    if (o.correctCandidates && o.correctionTypeCands != CorrectionType::Classic)
        throw std::runtime_error("candidate correction supports correctionTypeCands Classic only");
    if (o.qualityScoreBits != 1 && o.qualityScoreBits != 2 && o.qualityScoreBits != 8)
        throw std::runtime_error("qualityScoreBits must be 1, 2 or 8");
    if (o.fixedNumberOfReads > 0xffffffffull)
        throw std::runtime_error("fixedNumberOfReads above 2^32-1");
    if (!o.save_binary_reads_to.empty() || !o.load_binary_reads_from.empty() || !o.save_hashtables_to.empty() ||
        !o.load_hashtables_from.empty())
        throw std::runtime_error("saving or loading preprocessed reads or hash tables is not supported");
}

namespace {

struct Ctx {
    cg_ctx* c = nullptr;
    ~Ctx() {
        if (c) cg_destroy(c);
    }
};

void check(cg_ctx* c, int rc, const char* what) {
    if (rc != CG_OK) {
        throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " +
                                 (c ? cg_last_error(c) : ""));
    }
}

bool isAmbiguousChar(char ch) {
    switch (ch) {
        case 'A': case 'C': case 'G': case 'T': case 'a': case 'c': case 'g': case 't': return false;
        default: return true;
    }
}

char upper(char ch) {
    switch (ch) {
        case 'a': return 'A';
        case 'c': return 'C';
        case 'g': return 'G';
        case 't': return 'T';
        default: return ch;
    }
}

// STEP1-2: reads of the input group, device build and correction.
// Output per read: final sequence written into `seqOut` (same offsets as the
// input) and its quality label (0 none, 1 LQ anchor correction, 2 LQ
// correction confirmed by candidate corrections, 3 HQ); lastRecord = the last
// read with a correction record (-1: none), after which the reference writes
// no labels (src/correctionresultoutput.cpp:370-377, 896-901).
struct Corrected {
    ReadSet reads;
    std::vector<char> seqOut;
    std::vector<uint8_t> status;
    int64_t lastRecord = -1;
    uint64_t records = 0;
    cg_stats stats{};
};

Corrected runCorrection(const ProgramOptions& o) {
    if (o.inputfiles.empty()) throw std::runtime_error("no input files");
    validateOptions(o);
    Corrected r;
    std::vector<uint64_t> groupStarts;  // one device append call per input group
    if (o.pairType == SequencePairType::PairedEnd && o.inputfiles.size() == 2) {
        groupStarts.push_back(0);
        readPairedFiles(o.inputfiles[0], o.inputfiles[1], r.reads);
    } else {
        for (size_t i = 0; i < o.inputfiles.size(); i++) {
            groupStarts.push_back(r.reads.size());
            readSingleFile(o.inputfiles[i], r.reads, (uint8_t)i);
        }
    }
    const uint64_t n = r.reads.size();
    if (n == 0) throw std::runtime_error("input contains no reads");
    bool useQ = o.useQualityScores && r.reads.hasQualities;  // src/main_correct_cpu.cpp:109-121
    ProgramOptions eff = o;
    eff.useQualityScores = useQ;
    const cg_options co = toCgOptions(eff);
    Ctx ctx;
    check(nullptr, cg_create(&co, &ctx.c), "cg_create");
    for (size_t gi = 0; gi < groupStarts.size(); gi++) {
        const uint64_t a = groupStarts[gi];
        const uint64_t b = gi + 1 < groupStarts.size() ? groupStarts[gi + 1] : n;
        if (b == a) continue;
        check(ctx.c,
              cg_append_reads(ctx.c, r.reads.sequences.data(), r.reads.offsets.data() + a,
                              useQ ? r.reads.qualities.data() : nullptr, b - a),
              "cg_append_reads");
    }
    check(ctx.c, cg_build_tables(ctx.c), "cg_build_tables");
    if (o.correctionType == CorrectionType::Forest) {
        // src/main_correct_cpu.cpp:125-134: a forest file is required
        std::ifstream is(o.mlForestfileAnchor, std::ios::binary);
        if (!is) throw std::runtime_error("Loading classifier file failed! " + o.mlForestfileAnchor);
        std::vector<char> bytes((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
        check(ctx.c, cg_load_forest(ctx.c, bytes.data(), bytes.size(), o.maxForestTreesAnchor), "cg_load_forest");
    }
    if (o.correctionType == CorrectionType::Learned) {
        std::ifstream is(o.mlClassifierFileAnchor, std::ios::binary);
        if (!is) throw std::runtime_error("Loading classifier file failed! " + o.mlClassifierFileAnchor);
        std::vector<char> bytes((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
        check(ctx.c, cg_load_classifier(ctx.c, bytes.data(), bytes.size()), "cg_load_classifier");
    }
    uint64_t nr = 0;
    int32_t lmax = 0;
    check(ctx.c, cg_get_read_info(ctx.c, &nr, &lmax), "cg_get_read_info");
    r.seqOut = r.reads.sequences;
    r.status.assign(n, 0);
    const uint64_t chunk = 1u << 20;
    std::vector<uint8_t> flags(chunk);
    std::vector<char> seqs(chunk * (size_t)lmax);
    std::vector<uint8_t> allFlags(o.correctCandidates ? n : 0);  // for the combine step
    for (uint64_t first = 0; first < n; first += chunk) {
        const uint64_t cnt = std::min(chunk, n - first);
        check(ctx.c, cg_correct(ctx.c, first, cnt, flags.data(), seqs.data(), (size_t)lmax), "cg_correct");
        if (o.correctCandidates) std::memcpy(allFlags.data() + first, flags.data(), cnt);
        for (uint64_t j = 0; j < cnt; j++) {
            if (!(flags[j] & CG_RESULT_CORRECTED)) continue;
            const uint64_t id = first + j;
            const uint64_t off = r.reads.offsets[id];
            const int len = (int)(r.reads.offsets[id + 1] - off);
            const char* orig = r.reads.sequences.data() + off;
            const char* corr = seqs.data() + j * (size_t)lmax;
            const bool hq = (flags[j] & CG_RESULT_HQ) != 0;
            bool ambiguous = false;
            for (int p = 0; p < len && !ambiguous; p++) ambiguous = isAmbiguousChar(orig[p]);
            char* dst = r.seqOut.data() + off;
            if (ambiguous) {
                // include/corrector.hpp:1651-1667: no edit list for reads with N
                std::memcpy(dst, corr, len);
                r.status[id] = hq ? 3 : 1;
                r.records++;
                r.lastRecord = (int64_t)id;
                continue;
            }
            const int maxEdits = len / 7;
            int edits = 0;
            for (int p = 0; p < len && edits <= maxEdits; p++) edits += corr[p] != upper(orig[p]);
            if (edits <= maxEdits) {
                if (hq && edits == 0) continue;  // src/correct_cpu.cpp:263-273 drops such records
                for (int p = 0; p < len; p++)
                    if (corr[p] != upper(orig[p])) dst[p] = corr[p];
            } else {
                std::memcpy(dst, corr, len);
            }
            r.status[id] = hq ? 3 : 1;
            r.records++;
            r.lastRecord = (int64_t)id;
        }
    }
    if (o.correctCandidates) {
        // the combine step (src/correctionresultoutput.cpp:1256-1551)
        uint64_t candRecords = 0;
        check(ctx.c, cg_combine_results(ctx.c, 0, n, allFlags.data(), &candRecords), "cg_combine_results");
        r.records += candRecords;
        for (uint64_t i = 0; i < n; i++) {
            const uint8_t f = allFlags[i];
            if (f & CG_RESULT_CANDIDATE_RECORD) r.lastRecord = std::max(r.lastRecord, (int64_t)i);
            if (f & CG_RESULT_REJECTED) {  // written unchanged
                const uint64_t off = r.reads.offsets[i];
                std::memcpy(r.seqOut.data() + off, r.reads.sequences.data() + off, r.reads.offsets[i + 1] - off);
                r.status[i] = 0;
            } else if (f & CG_RESULT_CANDIDATES) {
                r.status[i] = 2;
            }
        }
    }
    check(ctx.c, cg_get_stats(ctx.c, &r.stats), "cg_get_stats");
    return r;
}

std::vector<char> loadFile(const std::string& path, const char* what) {
    std::ifstream is(path, std::ios::binary);
    if (!is) throw std::runtime_error(std::string("Loading classifier file failed! ") + path);
    (void)what;
    return std::vector<char>((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
}

// STEP1-3 with the FASTQ parsing and the output records on the device
// (care_files.h).  false: the inputs are not all plain 4-line FASTQ (or the
// path is switched off) and nothing was done.
bool correctOnDevice(const ProgramOptions& o, cg::FastqRun* run) {
    if (!o.deviceFileIO || o.inputfiles.empty() || o.outputfilenames.empty()) return false;
    if (o.correctionType == CorrectionType::Print) return false;
    if (o.correctCandidates && o.correctionTypeCands != CorrectionType::Classic) return false;
    for (const auto& f : o.inputfiles) {
        const FileFormat fmt = detectFormat(f);
        if (fmt != FileFormat::FASTQ && fmt != FileFormat::FASTQGZ) return false;
    }
    const bool paired = o.pairType == SequencePairType::PairedEnd && o.inputfiles.size() == 2;
    std::vector<FileBytes> data;
    for (const auto& f : o.inputfiles) data.push_back(readFileBytes(f));
    std::vector<cg::ByteSpan> inputs;
    for (const auto& d : data) inputs.push_back(cg::ByteSpan{d.data.get(), d.size});
    std::vector<char> forest, classifier;
    if (o.correctionType == CorrectionType::Forest) forest = loadFile(o.mlForestfileAnchor, "forest");
    if (o.correctionType == CorrectionType::Learned) classifier = loadFile(o.mlClassifierFileAnchor, "classifier");
    const cg_options co = toCgOptions(o);  // FASTQ carries qualities
    std::string err;
    const int rc = cg::correct_fastq_on_device(co, inputs, paired, o.outputCorrectionQualityLabels,
                                               (int)o.outputfilenames.size(),
                                               o.correctionType == CorrectionType::Forest ? &forest : nullptr,
                                               o.maxForestTreesAnchor,
                                               o.correctionType == CorrectionType::Learned ? &classifier : nullptr,
                                               run, &err);
    if (rc == CG_ERR_UNSUPPORTED) return false;
    if (rc != CG_OK) throw std::runtime_error("device file path failed (" + std::to_string(rc) + "): " + err);
    return true;
}

FileFormat outputFormat(const ProgramOptions& o) {
    FileFormat fmt = detectFormat(o.inputfiles[0]);
    if (o.gzoutput) {
        if (fmt == FileFormat::FASTQ) fmt = FileFormat::FASTQGZ;
        if (fmt == FileFormat::FASTA) fmt = FileFormat::FASTAGZ;
    } else {
        if (fmt == FileFormat::FASTQGZ) fmt = FileFormat::FASTQ;
        if (fmt == FileFormat::FASTAGZ) fmt = FileFormat::FASTA;
    }
    return fmt;
}

std::string labelled(const std::string& header, uint8_t status, bool labels) {
    if (!labels) return header;
    // src/correctionresultoutput.cpp:403-414
    return header + " care:q=" + char('0' + status);
}

}  // namespace

namespace {

// Output files written by a thread of their own, in the order the ranges
// arrive, while the device corrects the next range.
class RangeWriter {
public:
    RangeWriter(const ProgramOptions& o, FileFormat fmt) {
        for (const auto& name : o.outputfilenames)
            writers_.emplace_back(new SequenceWriter(o.outputdirectory + "/" + name, fmt));
        thread_ = std::thread([this] { loop(); });
    }
    ~RangeWriter() { finish(false); }
    void put(int f, std::unique_ptr<char[]> bytes, size_t size) {
        std::lock_guard<std::mutex> lock(mu_);
        queue_.push_back(Item{f, std::move(bytes), size});
        cv_.notify_one();
    }
    // waits for every range to be written; rethrows a write error
    void finish(bool rethrow = true) {
        {
            std::lock_guard<std::mutex> lock(mu_);
            done_ = true;
            cv_.notify_one();
        }
        if (thread_.joinable()) thread_.join();
        if (rethrow && error_) std::rethrow_exception(error_);
    }

private:
    struct Item {
        int f;
        std::unique_ptr<char[]> bytes;
        size_t size;
    };
    void loop() {
        while (true) {
            Item it;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_.wait(lock, [this] { return done_ || !queue_.empty(); });
                if (queue_.empty()) return;
                it = std::move(queue_.front());
                queue_.pop_front();
            }
            if (error_) continue;  // drain after a failure
            try {
                writers_[it.f]->writeRaw(it.bytes.get(), it.size);
            } catch (...) {
                error_ = std::current_exception();
            }
        }
    }
    std::vector<std::unique_ptr<SequenceWriter>> writers_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Item> queue_;
    bool done_ = false;
    std::exception_ptr error_;
    std::thread thread_;
};

}  // namespace

RunReport performCorrection(const ProgramOptions& o) {
    validateOptions(o);
    if (!o.outputfilenames.empty() && !o.inputfiles.empty()) {
        cg::FastqRun dr;
        RangeWriter out(o, outputFormat(o));
        dr.onChunk = [&out](int f, std::unique_ptr<char[]> bytes, size_t size) { out.put(f, std::move(bytes), size); };
        if (correctOnDevice(o, &dr)) {
            out.finish();
            RunReport rep;
            rep.reads = dr.reads;
            rep.records = dr.records;
            rep.stats = dr.stats;
            rep.deviceFileIO = true;
            return rep;
        }
    }
    if (o.inputfiles.empty()) throw std::runtime_error("no input files");
    Corrected r = runCorrection(o);
    const FileFormat fmt = outputFormat(o);
    if (o.outputfilenames.empty()) throw std::runtime_error("no output file names");
    std::vector<std::unique_ptr<SequenceWriter>> writers;
    for (const auto& name : o.outputfilenames)
        writers.emplace_back(new SequenceWriter(o.outputdirectory + "/" + name, fmt));
    const uint64_t n = r.reads.size();
    static const std::string empty;
    for (uint64_t i = 0; i < n; i++) {
        const uint64_t off = r.reads.offsets[i];
        const size_t len = r.reads.offsets[i + 1] - off;
        const int w = writers.size() == 1 ? 0 : std::min<int>(r.reads.fileId[i], (int)writers.size() - 1);
        const std::string q = r.reads.hasQualities ? std::string(r.reads.qualities.data() + off, len) : empty;
        const bool lab = o.outputCorrectionQualityLabels && (int64_t)i <= r.lastRecord;
        writers[w]->write(labelled(r.reads.headers[i], r.status[i], lab), r.seqOut.data() + off, len, q);
    }
    RunReport rep;
    rep.reads = n;
    rep.records = r.records;
    rep.stats = r.stats;
    return rep;
}

RunReport performCorrectionToSink(const ProgramOptions& o, const std::function<void(int)>& onStart,
                                  const ChunkSink& sink) {
    validateOptions(o);
    {
        cg::FastqRun dr;
        dr.queueChunkBytes = 1u << 20;  // the queue protocol's chunks (src/correctionresultoutput.cpp:733-745)
        ProgramOptions od = o;
        const int nfiles = (o.pairType == SequencePairType::PairedEnd && o.inputfiles.size() == 2) ? 2 : 1;
        od.outputfilenames.assign(nfiles, "queue");  // one record stream per queue
        if (correctOnDevice(od, &dr)) {
            RunReport rep;
            rep.reads = dr.reads;
            rep.records = dr.records;
            rep.stats = dr.stats;
            rep.deviceFileIO = true;
            onStart((int)dr.records);  // src/correctionresultoutput.cpp:465-466
            if (dr.records == 0) return rep;
            // whole records into chunks of under 1 MiB (the host writer's cut
            // points), copied from device memory straight into the chunks
            std::string err;
            if (cg::emit_queue_chunks(&dr, sink, &err) != CG_OK)
                throw std::runtime_error("queue chunks: " + err);
            return rep;
        }
    }
    Corrected r = runCorrection(o);
    RunReport rep;
    rep.reads = r.reads.size();
    rep.records = r.records;
    rep.stats = r.stats;
    onStart((int)r.records);  // src/correctionresultoutput.cpp:465-466
    if (r.records == 0) return rep;
    const int cap = 1 << 20;
    const int nfiles = (o.pairType == SequencePairType::PairedEnd && o.inputfiles.size() == 2) ? 2 : 1;
    std::vector<char*> buf(nfiles, nullptr);
    std::vector<int> used(nfiles, 0);
    for (int f = 0; f < nfiles; f++) buf[f] = new char[cap];
    bool ok = true;
    auto put = [&](int f, const char* p, size_t len) {
        std::memcpy(buf[f] + used[f], p, len);
        used[f] += (int)len;
    };
    for (uint64_t i = 0; i < rep.reads && ok; i++) {
        const uint64_t off = r.reads.offsets[i];
        const size_t len = r.reads.offsets[i + 1] - off;
        const int f = nfiles == 1 ? 0 : r.reads.fileId[i];
        const bool lab = o.outputCorrectionQualityLabels && (int64_t)i <= r.lastRecord;
        const std::string hdr = labelled(r.reads.headers[i], r.status[i], lab);
        const size_t need = hdr.size() + 2 * len + 6;
        if (need >= (size_t)cap) throw std::runtime_error("record larger than a 1 MiB chunk");
        if (used[f] + need >= (size_t)cap) {
            ok = sink(f, buf[f], used[f]);
            buf[f] = ok ? new char[cap] : nullptr;
            used[f] = 0;
            if (!ok) break;
        }
        // src/correctionresultoutput.cpp:733-770: '@' header, sequence, '+', quality
        put(f, "@", 1);
        put(f, hdr.data(), hdr.size());
        put(f, "\n", 1);
        put(f, r.seqOut.data() + off, len);
        put(f, "\n+\n", 3);
        if (r.reads.hasQualities) put(f, r.reads.qualities.data() + off, len);
        put(f, "\n", 1);
    }
    for (int f = 0; f < nfiles; f++) {
        if (!buf[f]) continue;
        if (ok && used[f] > 0) {
            ok = sink(f, buf[f], used[f]);
        } else {
            delete[] buf[f];
        }
    }
    return rep;
}

}  // namespace care_gb300

// ---------------------------------------------------------------- C ABI
extern "C" int cg_correct_files(const cg_options* options, const char* const* inputs, int num_inputs,
                                const char* output_directory, const char* const* outputs, int num_outputs,
                                int quality_labels, int gz_output, uint64_t* num_records) {
    using namespace care_gb300;
    if (!options || !inputs || num_inputs < 1 || num_inputs > 2 || !outputs || num_outputs < 1 || !output_directory)
        return CG_ERR_INVALID_ARGUMENT;
    ProgramOptions o;
    o.kmerlength = options->kmerlength;
    o.autodetectKmerlength = options->kmerlength == 0;
    o.numHashFunctions = options->num_hash_functions;
    o.estimatedCoverage = options->estimated_coverage;
    o.estimatedErrorrate = options->estimated_errorrate;
    o.m_coverage = options->m_coverage;
    o.maxErrorRate = options->max_error_rate;
    o.min_overlap_ratio = options->min_overlap_ratio;
    o.min_overlap = options->min_overlap;
    o.pairedFilterThreshold = options->paired_filter_threshold;
    o.new_columns_to_correct = options->new_columns_to_correct;
    o.useQualityScores = options->use_quality_scores;
    o.excludeAmbiguousReads = options->exclude_ambiguous_reads;
    o.correctCandidates = options->correct_candidates;
    o.pairType = options->pair_mode == CG_PAIR_PE ? SequencePairType::PairedEnd : SequencePairType::SingleEnd;
    o.correctionType = (CorrectionType)options->correction_type;
    o.thresholdAnchor = options->threshold_anchor;
    o.deviceIds = {options->device};
    o.gpuBatched = options->driver == CG_DRIVER_BATCHED;
    o.deviceFileIO = options->host_file_io == 0;
    o.qualityScoreBits = options->quality_score_bits == 0 ? 8 : options->quality_score_bits;
    o.fixedNumberOfReads = options->fixed_number_of_reads;
    o.memoryForHashtables = options->hashtable_memory_bytes;
    o.outputCorrectionQualityLabels = quality_labels != 0;
    o.gzoutput = gz_output != 0;
    o.outputdirectory = output_directory;
    for (int i = 0; i < num_inputs; i++) o.inputfiles.push_back(inputs[i]);
    for (int i = 0; i < num_outputs; i++) o.outputfilenames.push_back(outputs[i]);
    try {
        RunReport rep = performCorrection(o);
        if (num_records) *num_records = rep.records;
        return CG_OK;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cg_correct_files: %s\n", e.what());  // the C ABI has no context to hold it
        return CG_ERR_IO;
    }
}
