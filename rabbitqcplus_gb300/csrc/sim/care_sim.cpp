// Seeded synthetic read generator for the CARE correction workloads.
//
// Produces a random genome (optionally with diverged repeat copies), samples
// single-end or paired-end reads from it with substitution (and optional
// indel) errors, Phred qualities, and keeps the error-free truth of every read
// so corrections can be scored base by base (TP/FP/FN).  Every random draw comes
// from a counter-based integer generator (splitmix64 of seed, stream, index), so
// the output is identical on x86-64 and aarch64 and independent of the number
// of threads used.  No floating-point transcendental is used on any draw path.

#include "care_sim.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// A small sequential generator seeded per (seed, stream, index).
struct Rng {
    uint64_t s;
    Rng(uint64_t seed, uint64_t stream, uint64_t index)
        : s(splitmix64(seed ^ splitmix64(stream * 0x100000001b3ull + 0x51ed27) ^ splitmix64(index + 0x2545f4914f6cdd1dull))) {}
    uint64_t next() {
        s += 0x9e3779b97f4a7c15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    // uniform integer in [0, n)
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
    // Bernoulli(p) with p given in double; the comparison is exact integer work.
    bool chance(double p) {
        if (p <= 0.0) return false;
        if (p >= 1.0) return true;
        const uint64_t thr = (uint64_t)(p * 9007199254740992.0);  // p * 2^53
        return (next() >> 11) < thr;
    }
    // Approximately standard-normal draw scaled to (mean, sd), rounded to the
    // nearest integer: Irwin-Hall sum of twelve 24-bit uniforms, integer only.
    int64_t normal_int(int64_t mean, int64_t sd) {
        int64_t sum = 0;
        for (int i = 0; i < 12; i++) sum += (int64_t)(next() >> 40);
        const int64_t z24 = sum - 6 * (int64_t(1) << 24);  // N(0,1) * 2^24
        const int64_t scaled = z24 * sd + (int64_t(1) << 23);
        // floor division by 2^24 for negative values too
        const int64_t q = scaled >= 0 ? (scaled >> 24) : -((-scaled + (int64_t(1) << 24) - 1) >> 24);
        return mean + q;
    }
};

const char kBases[4] = {'A', 'C', 'G', 'T'};

inline char complement(char c) {
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T': return 'A';
        default: return c;
    }
}

struct SimData {
    cgsim_config cfg;
    std::string genome;
    std::vector<uint64_t> offsets;  // read i occupies [offsets[i], offsets[i+1])
    std::vector<char> seq;          // concatenated read sequences
    std::vector<char> qual;         // concatenated qualities (Phred+33)
    std::vector<char> truth;        // concatenated error-free sequences (same orientation)
    std::vector<uint8_t> has_indel; // reads whose truth is not position-aligned
    std::vector<uint64_t> origin;   // genome start of the sampled fragment/read
    std::vector<uint8_t> revcomp;
};

void make_genome(SimData& d) {
    const cgsim_config& c = d.cfg;
    d.genome.resize(c.genome_length);
    // 16 bases per draw, each 2 bits
    const uint64_t G = c.genome_length;
    for (uint64_t blk = 0; blk * 16 < G; blk++) {
        Rng r(c.seed, 1, blk);
        uint64_t v = r.next();
        for (int j = 0; j < 16 && blk * 16 + j < G; j++) {
            d.genome[blk * 16 + j] = kBases[(v >> (2 * j)) & 3];
        }
    }
    // repeat families: a source segment copied (with divergence) over other
    // places of the genome.  Copies are written in family/copy order so the
    // result does not depend on threads.
    if (c.repeat_families > 0 && c.repeat_copies > 0 && G > 2 * (uint64_t)c.repeat_max_len + 2) {
        for (uint32_t f = 0; f < c.repeat_families; f++) {
            Rng r(c.seed, 2, f);
            const uint32_t span = c.repeat_max_len - c.repeat_min_len + 1;
            const uint32_t len = c.repeat_min_len + (uint32_t)r.below(span);
            const uint64_t src = r.below(G - len);
            std::string unit = d.genome.substr(src, len);
            for (uint32_t k = 0; k < c.repeat_copies; k++) {
                const uint64_t dst = r.below(G - len);
                for (uint32_t i = 0; i < len; i++) {
                    char b = unit[i];
                    if (r.chance(c.repeat_divergence)) {
                        b = kBases[((b == 'A' ? 0 : b == 'C' ? 1 : b == 'G' ? 2 : 3) + 1 + r.below(3)) & 3];
                    }
                    d.genome[dst + i] = b;
                }
            }
        }
    }
}

// Sample one read of the given length starting at genome position `start`
// (forward strand), with errors; returns false if the genome is too short.
void emit_read(SimData& d, uint64_t id, uint64_t start, uint32_t len, bool rc, Rng& r,
               char* out_seq, char* out_qual, char* out_truth, uint8_t* indel_flag) {
    const cgsim_config& c = d.cfg;
    const uint64_t G = d.genome.size();
    // truth in read orientation
    std::string fwd_truth(len, 'A');
    std::string fwd_obs;
    fwd_obs.reserve(len);
    bool any_indel = false;
    if (c.indel_rate > 0.0) {
        uint64_t gp = start;
        while (fwd_obs.size() < len) {
            const char gb = d.genome[gp < G ? gp : G - 1];
            if (r.chance(c.indel_rate * 0.5)) {  // insertion of a random base
                fwd_obs.push_back(kBases[r.below(4)]);
                any_indel = true;
                continue;
            }
            if (r.chance(c.indel_rate * 0.5)) {  // deletion of the genome base
                gp++;
                any_indel = true;
                continue;
            }
            fwd_obs.push_back(gb);
            gp++;
        }
    } else {
        fwd_obs = d.genome.substr(start, len);
    }
    for (uint32_t i = 0; i < len; i++) fwd_truth[i] = d.genome[std::min<uint64_t>(start + i, G - 1)];
    std::string obs(len, 'A'), tru(len, 'A');
    if (rc) {
        for (uint32_t i = 0; i < len; i++) {
            obs[i] = complement(fwd_obs[len - 1 - i]);
            tru[i] = complement(fwd_truth[len - 1 - i]);
        }
    } else {
        obs = fwd_obs;
        tru = fwd_truth;
    }
    // substitutions along the read (5' -> 3' in read orientation) and qualities
    for (uint32_t i = 0; i < len; i++) {
        const double frac = len > 1 ? double(i) / double(len - 1) : 0.0;
        const double p = c.sub_rate_5p + (c.sub_rate_3p - c.sub_rate_5p) * frac;
        bool err = false;
        if (r.chance(p)) {
            const char b = obs[i];
            const int bi = b == 'A' ? 0 : b == 'C' ? 1 : b == 'G' ? 2 : 3;
            obs[i] = kBases[(bi + 1 + (int)r.below(3)) & 3];
            err = true;
        }
        int q;
        if (err) {
            q = c.err_qual_min + (int)r.below(uint64_t(c.err_qual_max - c.err_qual_min + 1));
        } else {
            q = (int)r.normal_int(c.qual_mean, c.qual_sd);
            q = std::max(c.qual_min, std::min(c.qual_max, q));
        }
        out_qual[i] = char(33 + q);
    }
    if (c.n_read_fraction > 0.0 && r.chance(c.n_read_fraction)) {
        const uint32_t nn = 1 + (uint32_t)r.below(3);
        for (uint32_t k = 0; k < nn; k++) obs[r.below(len)] = 'N';
    }
    std::memcpy(out_seq, obs.data(), len);
    std::memcpy(out_truth, tru.data(), len);
    *indel_flag = any_indel ? 1 : 0;
    (void)id;
}

void make_reads(SimData& d) {
    const cgsim_config& c = d.cfg;
    const uint64_t n = c.num_reads;
    const uint64_t G = d.genome.size();
    d.offsets.resize(n + 1);
    // lengths first (sequential prefix sum, lengths from per-read streams)
    std::vector<uint32_t> lens(n);
    if (c.paired) {
        for (uint64_t p = 0; p < n / 2; p++) {
            Rng r(c.seed, 3, p);
            const uint32_t span = c.read_len_max - c.read_len_min + 1;
            lens[2 * p] = c.read_len_min + (uint32_t)r.below(span);
            lens[2 * p + 1] = c.read_len_min + (uint32_t)r.below(span);
        }
    } else {
        for (uint64_t i = 0; i < n; i++) {
            Rng r(c.seed, 3, i);
            const uint32_t span = c.read_len_max - c.read_len_min + 1;
            lens[i] = c.read_len_min + (uint32_t)r.below(span);
        }
    }
    d.offsets[0] = 0;
    for (uint64_t i = 0; i < n; i++) d.offsets[i + 1] = d.offsets[i] + lens[i];
    d.seq.resize(d.offsets[n]);
    d.qual.resize(d.offsets[n]);
    d.truth.resize(d.offsets[n]);
    d.has_indel.assign(n, 0);
    d.origin.assign(n, 0);
    d.revcomp.assign(n, 0);
    if (c.paired) {
        const int64_t nPairs = (int64_t)(n / 2);
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < nPairs; p++) {
            Rng r(c.seed, 4, (uint64_t)p);
            const uint32_t l1 = lens[2 * p], l2 = lens[2 * p + 1];
            int64_t ins = r.normal_int((int64_t)c.insert_mean, (int64_t)c.insert_sd);
            ins = std::max<int64_t>(ins, std::max(l1, l2));
            if ((uint64_t)ins + 2 > G) ins = (int64_t)G - 2;
            const uint64_t fstart = r.below(G - (uint64_t)ins);
            const bool flip = r.next() & 1;  // which strand the fragment comes from
            const uint64_t i1 = 2 * p, i2 = 2 * p + 1;
            // read 1: forward from fragment start; read 2: reverse complement of fragment end
            const uint64_t s1 = fstart;
            const uint64_t s2 = fstart + (uint64_t)ins - l2;
            bool rc1 = false, rc2 = true;
            if (flip) { rc1 = true; rc2 = false; }
            const uint64_t st1 = flip ? s2 : s1;
            const uint64_t st2 = flip ? s1 : s2;
            emit_read(d, i1, st1, l1, rc1, r, &d.seq[d.offsets[i1]], &d.qual[d.offsets[i1]], &d.truth[d.offsets[i1]], &d.has_indel[i1]);
            emit_read(d, i2, st2, l2, rc2, r, &d.seq[d.offsets[i2]], &d.qual[d.offsets[i2]], &d.truth[d.offsets[i2]], &d.has_indel[i2]);
            d.origin[i1] = st1; d.origin[i2] = st2;
            d.revcomp[i1] = rc1; d.revcomp[i2] = rc2;
        }
    } else {
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint64_t i = (uint64_t)ii;
            Rng r(c.seed, 5, i);
            const uint32_t len = lens[i];
            const uint64_t start = G > len + 1 ? r.below(G - len - 1) : 0;
            const bool rc = r.next() & 1;
            emit_read(d, i, start, len, rc, r, &d.seq[d.offsets[i]], &d.qual[d.offsets[i]], &d.truth[d.offsets[i]], &d.has_indel[i]);
            d.origin[i] = start;
            d.revcomp[i] = rc;
        }
    }
}

bool write_fastq(const SimData& d, const char* path, int which) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    std::vector<char> buf;
    buf.reserve(1 << 22);
    const uint64_t n = d.cfg.num_reads;
    const uint64_t step = d.cfg.paired && which >= 0 ? 2 : 1;
    const uint64_t first = (d.cfg.paired && which >= 0) ? (uint64_t)which : 0;
    char hdr[64];
    for (uint64_t i = first; i < n; i += step) {
        const uint64_t b = d.offsets[i], e = d.offsets[i + 1];
        int hl;
        if (d.cfg.paired && which >= 0)
            hl = std::snprintf(hdr, sizeof(hdr), "@read%llu/%d\n", (unsigned long long)(i / 2), which + 1);
        else
            hl = std::snprintf(hdr, sizeof(hdr), "@read%llu\n", (unsigned long long)i);
        buf.insert(buf.end(), hdr, hdr + hl);
        buf.insert(buf.end(), d.seq.begin() + b, d.seq.begin() + e);
        buf.push_back('\n');
        buf.push_back('+');
        buf.push_back('\n');
        buf.insert(buf.end(), d.qual.begin() + b, d.qual.begin() + e);
        buf.push_back('\n');
        if (buf.size() > (1u << 22)) {
            std::fwrite(buf.data(), 1, buf.size(), f);
            buf.clear();
        }
    }
    std::fwrite(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    return true;
}

}  // namespace

extern "C" {

void cgsim_default_config(cgsim_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->seed = 7;
    c->genome_length = 1000000;
    c->repeat_families = 0;
    c->repeat_copies = 0;
    c->repeat_min_len = 1000;
    c->repeat_max_len = 5000;
    c->repeat_divergence = 0.02;
    c->num_reads = 200000;
    c->read_len_min = 150;
    c->read_len_max = 150;
    c->paired = 0;
    c->insert_mean = 300;
    c->insert_sd = 30;
    c->sub_rate_5p = 0.01;
    c->sub_rate_3p = 0.01;
    c->indel_rate = 0.0;
    c->n_read_fraction = 0.0;
    c->qual_mean = 34;
    c->qual_sd = 4;
    c->qual_min = 2;
    c->qual_max = 41;
    c->err_qual_min = 2;
    c->err_qual_max = 20;
}

void* cgsim_create(const cgsim_config* cfg) {
    if (!cfg || cfg->genome_length < 64 || cfg->read_len_min == 0 || cfg->read_len_max < cfg->read_len_min ||
        cfg->read_len_max + 2 > cfg->genome_length || (cfg->paired && (cfg->num_reads % 2) != 0))
        return nullptr;
    SimData* d = new SimData();
    d->cfg = *cfg;
    make_genome(*d);
    make_reads(*d);
    return d;
}

void cgsim_destroy(void* h) { delete static_cast<SimData*>(h); }

uint64_t cgsim_num_reads(void* h) { return static_cast<SimData*>(h)->cfg.num_reads; }
uint64_t cgsim_total_bases(void* h) { return static_cast<SimData*>(h)->offsets.back(); }
const uint64_t* cgsim_offsets(void* h) { return static_cast<SimData*>(h)->offsets.data(); }
const char* cgsim_sequences(void* h) { return static_cast<SimData*>(h)->seq.data(); }
const char* cgsim_qualities(void* h) { return static_cast<SimData*>(h)->qual.data(); }
const char* cgsim_truth(void* h) { return static_cast<SimData*>(h)->truth.data(); }
const uint8_t* cgsim_indel_flags(void* h) { return static_cast<SimData*>(h)->has_indel.data(); }

int cgsim_write_fastq(void* h, const char* path1, const char* path2) {
    SimData* d = static_cast<SimData*>(h);
    if (d->cfg.paired && path2) {
        if (!write_fastq(*d, path1, 0)) return -1;
        if (!write_fastq(*d, path2, 1)) return -1;
        return 0;
    }
    return write_fastq(*d, path1, -1) ? 0 : -1;
}

// Base-level scoring of corrected reads against the truth.  `corrected` holds
// the corrected reads concatenated with the same offsets as the input.  Reads
// carrying an indel error are skipped (no position-aligned truth).
void cgsim_score(void* h, const char* corrected, uint64_t* tp, uint64_t* fp, uint64_t* fn, uint64_t* reads_scored) {
    SimData* d = static_cast<SimData*>(h);
    uint64_t TP = 0, FP = 0, FN = 0, R = 0;
    const uint64_t n = d->cfg.num_reads;
    for (uint64_t i = 0; i < n; i++) {
        if (d->has_indel[i]) continue;
        R++;
        for (uint64_t p = d->offsets[i]; p < d->offsets[i + 1]; p++) {
            const char o = d->seq[p], t = d->truth[p], c = corrected[p];
            if (o != t) {
                if (c == t) TP++;
                else FN++;
            } else if (c != t) {
                FP++;
            }
        }
    }
    *tp = TP; *fp = FP; *fn = FN; *reads_scored = R;
}

// The same score for reads [first, first + count) straight from correction
// results: read first + j is row j of `rows` (pitch bytes) when flags[j] has
// bit 1 (corrected) and not bit 8 (rejected by the combine step), else its
// input sequence.
void cgsim_score_results(void* h, uint64_t first, uint64_t count, const uint8_t* flags, const char* rows,
                         uint64_t pitch, uint64_t* tp, uint64_t* fp, uint64_t* fn, uint64_t* reads_scored) {
    SimData* d = static_cast<SimData*>(h);
    uint64_t TP = 0, FP = 0, FN = 0, R = 0;
#pragma omp parallel for reduction(+ : TP, FP, FN, R) schedule(static, 4096)
    for (int64_t j = 0; j < (int64_t)count; j++) {
        const uint64_t i = first + (uint64_t)j;
        if (d->has_indel[i]) continue;
        R++;
        const bool use = (flags[j] & 1u) && !(flags[j] & 8u);
        const char* row = rows + (uint64_t)j * pitch;
        for (uint64_t p = d->offsets[i]; p < d->offsets[i + 1]; p++) {
            const char o = d->seq[p], t = d->truth[p], c = use ? row[p - d->offsets[i]] : o;
            if (o != t) {
                if (c == t) TP++;
                else FN++;
            } else if (c != t) {
                FP++;
            }
        }
    }
    *tp = TP; *fp = FP; *fn = FN; *reads_scored = R;
}

}  // extern "C"
