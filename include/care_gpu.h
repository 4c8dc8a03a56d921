/*
 * care_gpu.h -- C ABI of the GB300-native CARE read error-correction engine.
 *
 * This is the boundary that replaces the CPU engine below RabbitQCPlus's
 * CARE entry points
 *     void care::performCorrection(care::ProgramOptions)
 *     void care::performCorrectionOutToQueue(care::ProgramOptions, Q1, Q2,
 *                                            producerDone, careStartWrite, changNum)
 * (reference: include/dispatch_care_correct_cpu.hpp:9-11,
 *  src/dispatch_care_correct_cpu.cpp:52-249 and 254-457).  Those two C++
 * functions are re-implemented on top of this ABI by the host layer
 * (rabbitqcplus_gb300/csrc/host/care_host.cpp, declared in care_host.h); a
 * RabbitQCPlus build links that object in place of dispatch_care_correct_cpu.o.
 *
 * Rules of the ABI: plain pointers and sizes only; every call returns a status
 * code (CG_OK == 0) and never aborts the process; device memory belongs to the
 * context, host buffers belong to the caller; one context drives one GPU and
 * calls on one context must be serialised by the caller.
 */
#ifndef CARE_GPU_H
#define CARE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CG_OK 0
#define CG_ERR_INVALID_ARGUMENT 1
#define CG_ERR_UNSUPPORTED 2
#define CG_ERR_CUDA 3
#define CG_ERR_OUT_OF_MEMORY 4
#define CG_ERR_STATE 5
#define CG_ERR_IO 6
#define CG_ERR_TIMEOUT 7

/* maximum number of minhash maps (reference: include/config.hpp:30) */
#define CG_MAX_HASHMAPS 48
/* longest read the device kernels accept */
#define CG_MAX_READ_LENGTH 1024

#define CG_PAIR_SE 0
#define CG_PAIR_PE 1

/* correction decision (reference: include/options.hpp:23-28, CorrectionType) */
#define CG_CORR_CLASSIC 0
#define CG_CORR_FOREST 1
#define CG_CORR_PRINT 2
#define CG_CORR_LEARNED 3

/* per-anchor result flags */
#define CG_RESULT_CORRECTED 1u /* anchor has a correction (TempCorrectedSequence exists) */
#define CG_RESULT_HQ 2u        /* MSA properties marked the anchor high quality */
/* set by cg_combine_results (candidate correction only) */
#define CG_RESULT_CANDIDATES 4u      /* LQ correction kept: all of its >= 2 candidate corrections agree */
#define CG_RESULT_REJECTED 8u        /* LQ correction dropped: its >= 2 candidate corrections disagree */
#define CG_RESULT_CANDIDATE_RECORD 16u /* the read has at least one saved candidate correction record */

/*
 * Options: the fields of care::ProgramOptions that change what the correction
 * path computes (reference: include/options.hpp:36-99, parsed in
 * src/options.cpp:55-390).  cg_default_options gives the reference defaults
 * except estimated_coverage, which the caller sets from --coverage.
 */
typedef struct cg_options {
    int32_t kmerlength;               /* kmerlength; 0 = autodetect (20 if max read length < 160, else 32) */
    int32_t num_hash_functions;       /* numHashFunctions, 1..48 */
    float estimated_coverage;         /* estimatedCoverage (--coverage) */
    float estimated_errorrate;        /* estimatedErrorrate (0.06) */
    float m_coverage;                 /* m_coverage (0.6) */
    float max_error_rate;             /* maxErrorRate (0.2) */
    float min_overlap_ratio;          /* min_overlap_ratio (0.3) */
    int32_t min_overlap;              /* min_overlap (30) */
    float paired_filter_threshold;    /* pairedFilterThreshold (0.06) */
    int32_t new_columns_to_correct;   /* new_columns_to_correct (15; 0..256 with candidate correction) */
    int32_t use_quality_scores;       /* useQualityScores */
    int32_t exclude_ambiguous_reads;  /* excludeAmbiguousReads */
    int32_t correct_candidates;       /* correctCandidates (classic candidate correction; cg_combine_results) */
    int32_t pair_mode;                /* CG_PAIR_SE / CG_PAIR_PE (pairType) */
    int32_t correction_type;          /* CG_CORR_* (correctionType) */
    float threshold_anchor;           /* thresholdAnchor for the learned decision (0.5) */
    int32_t device;                   /* CUDA device ordinal */
    int32_t batch_anchors;            /* anchors per device batch; 0 = automatic */
    /* Driver of cg_correct (no reference counterpart; both give identical
     * results).  CG_DRIVER_PLAIN runs each batch as stage kernels with host
     * round trips for its sizes.  CG_DRIVER_BATCHED replays one captured CUDA
     * graph per batch (candidates, alignment, filter, MSA and correction with
     * persistent work-stealing kernels) on up to two streams, with buffers
     * sized once per call from the raw candidate counts of the range; the
     * launch shapes below that are 0 are picked by an autotuner on the first
     * batched call of the process for this kind of data. */
    int32_t driver;                   /* CG_DRIVER_* */
    int32_t align_blocks;             /* batched: persistent alignment blocks (128 threads); 0 = tuned */
    int32_t msa_warps;                /* batched: anchors in flight per MSA block, 1..8; 0 = tuned */
    int32_t streams;                  /* batched: batches in flight, 1 or 2; 0 = tuned */
    /* cg_correct_files only (no reference counterpart): 0 = FASTQ inputs are
     * parsed and the output records written on the device (inputs that are not
     * plain 4-line FASTQ still take the host path), 1 = always parse and write
     * on the host; both give the same files */
    int32_t host_file_io;
    /* qualityScoreBits (8; 0 means 8): bits per quality score in the read
     * store.  With 2 or 1 every score is stored binned -- 2 bits: Q <= 4 -> '$',
     * <= 13 -> '(', <= 20 -> '1', else '9'; 1 bit: Q <= 13 -> '(', else '5' --
     * and a row's positions past its read's end hold the first bin's score
     * (reference: include/qualityscorecompression.hpp:25-73 and 74-140,
     * applied by include/chunkedreadstorageconstruction.hpp:240-268, decoded
     * by include/chunkedreadstorage.hpp:532-607).  Only the scores the
     * correction reads change; output files keep the input's scores. */
    int32_t quality_score_bits;
    /* fixedNumberOfReads (0 = every read): only reads [0, n) are corrected as
     * anchors -- cg_correct returns flags 0 for later reads -- while every read
     * stays in the hash tables and can be a candidate (reference:
     * include/options.hpp:126-133, src/correct_cpu.cpp:97-102).  Above the
     * number of reads it means every read; even in paired mode. */
    uint32_t fixed_number_of_reads;
    int32_t reserved0;
    /* memoryForHashtables (bytes; 0 = no limit).  The reference builds its
     * maps in rounds of (limit / (12 bytes x reads)) - 2 under this limit
     * (src/cpuminhasherconstruction.cpp:27-165, include/ordinaryminhasher.hpp:
     * 350-372); when the first round cannot hold num_hash_functions maps, how
     * many maps it ends with depends on the sizes of its compacted host tables,
     * so cg_build_tables refuses the run with CG_ERR_UNSUPPORTED rather than
     * correct with a different number of maps. */
    uint64_t hashtable_memory_bytes;
} cg_options;

#define CG_DRIVER_PLAIN 0
#define CG_DRIVER_BATCHED 1

typedef struct cg_ctx cg_ctx;

/* Per-run counters (reference: the per-stage counters printed by
 * src/correct_cpu.cpp:314-345, as counts instead of times). */
typedef struct cg_stats {
    uint64_t num_reads;
    uint64_t num_anchors_processed;
    uint64_t raw_candidate_ids;       /* sum over anchors of hash-table hits */
    uint64_t unique_candidates;       /* after sort/unique/self removal */
    uint64_t aligned_candidates;      /* after orientation filter */
    uint64_t msa_candidates;          /* after mismatch-ratio filter */
    uint64_t msa_builds;              /* MSA builds including refinement rebuilds */
    uint64_t corrected_anchors;
    uint64_t hq_anchors;
    uint64_t table_keys;              /* kept keys over all maps */
    uint64_t table_values;            /* stored read ids over all maps */
    int32_t kmerlength;               /* k in use (after autodetect) */
    int32_t num_maps;
    int32_t max_read_length;
    int32_t reserved;
    double seconds_build;             /* device time of the last cg_build_tables */
    double seconds_correct;           /* device time of the last cg_correct */
    double seconds_candidates;        /* device time in candidate stages (query, unique), accumulated */
    double seconds_align;             /* device time in the alignment/filter kernel, accumulated */
    double seconds_msa;               /* device time in the MSA/correction kernel, accumulated */
    uint64_t kernel_launches;         /* kernels this context launched, accumulated */
    uint64_t align_launches;          /* launches of the alignment/filter kernel */
    uint64_t msa_launches;            /* launches of the MSA/correction kernel */
    double seconds_filter;            /* device time in the mismatch-ratio filter kernel, accumulated */
    /* batched driver: the shape in use and the time its tuning took */
    int32_t batch_anchors;
    int32_t align_blocks;
    int32_t msa_warps;
    int32_t streams;
    double seconds_tune;
    uint64_t graph_replays;           /* batches run as graph replays, accumulated */
    /* learned decision (CG_CORR_LEARNED) */
    uint64_t learned_columns;         /* columns scored by the classifier */
    uint64_t learned_corrections;     /* columns it set to the consensus */
    uint64_t learned_overflow;        /* columns beyond the per-batch records (fallback decision) */
    /* candidate correction (correct_candidates) */
    uint64_t candidate_corrections;   /* candidates corrected by HQ anchors, accumulated */
    /* learned decision: classifier blocks that gave up waiting for their
     * tensor-core MMAs, accumulated (each such call returned CG_ERR_TIMEOUT) */
    uint64_t classifier_timeouts;
} cg_stats;

/* Fill *o with the reference defaults. */
void cg_default_options(cg_options* o);

/* Create a context on o->device.  *out is set only on CG_OK. */
int cg_create(const cg_options* o, cg_ctx** out);

/* Release the context.  Its device blocks go to a per-process cache that
 * later contexts allocate from; cg_release_cached_memory returns them. */
void cg_destroy(cg_ctx* ctx);

/* Free the device blocks cached for reuse on `device` (all devices if < 0);
 * an allocation that would fail does the same first.  A program that resets
 * a device (cudaDeviceReset) calls this for it first, as the cached blocks
 * die with the reset.  No counterpart in the reference (its CPU path keeps no
 * device memory). */
int cg_release_cached_memory(int device);

/* Fault injection for tests of the out-of-memory path (no counterpart in
 * the reference): after `after` more requests for context device memory
 * succeed, every later request fails as if the device were full -- the
 * per-process block cache is emptied first, as on a real failure -- and the
 * call that made it returns CG_ERR_OUT_OF_MEMORY.  after < 0 switches it off.
 * Process-wide. */
int cg_set_allocation_fault(int64_t after);

/* Polls (mbarrier try-waits) a learned-decision inference block spends on
 * each of its tensor-core MMAs before it gives up on its remaining columns,
 * on `device`; polls < 0 restores the default (1 << 20, far above what an
 * MMA needs).  A block that gives up leaves its columns to the fallback
 * decision, drains its MMAs and releases its tensor memory; the call that ran
 * it (cg_correct, cg_correct_files, cg_classifier_logits) returns
 * CG_ERR_TIMEOUT and cg_stats.classifier_timeouts counts it.  A diagnostic
 * hook (e.g. polls = 0 makes every such wait give up); no counterpart in the
 * reference. */
int cg_set_classifier_wait_limit(int device, int64_t polls);

/* Message of the last failing call on this context (never NULL). */
const char* cg_last_error(const cg_ctx* ctx);

/*
 * Append reads to the device read store (reference: ChunkedReadStorage built by
 * constructChunkedReadStorageFromFiles, include/chunkedreadstorageconstruction.hpp:29-485).
 * `sequences` holds the reads back to back, read i at [offsets[i], offsets[i+1]).
 * Bases are upper-cased; every other character becomes A,C,G,T in turn, the
 * counter restarting every 65536 reads of one call (one call per input file,
 * or per interleaved file pair), and such reads are marked ambiguous.
 * `qualities` (same offsets, Phred+33) may be NULL unless quality scores are used.
 * Reads get consecutive ids in call order.  Must precede cg_build_tables.
 */
int cg_append_reads(cg_ctx* ctx, const char* sequences, const uint64_t* offsets,
                    const char* qualities, uint64_t num_reads);

/*
 * Build the minhash signatures and the hash tables on the device (reference:
 * constructCpuMinhasherFromCpuReadStorage, src/cpuminhasherconstruction.cpp:27-212,
 * OrdinaryCpuMinhasher::insert/compact, include/ordinaryminhasher.hpp:223-254,376-426).
 */
int cg_build_tables(cg_ctx* ctx);

/*
 * Correct anchors [first_read, first_read + num_anchors) (reference: the body of
 * cpu::correct_cpu, src/correct_cpu.cpp:47-348, per anchor
 * CpuErrorCorrector::process / processMulti, include/corrector.hpp:145-513).
 * For anchor j of the range: out_flags[j] gets CG_RESULT_* bits and, when
 * CG_RESULT_CORRECTED is set, out_sequences[j * out_pitch .. + length) gets the
 * corrected bases as 'A','C','G','T' (reference: TempCorrectedSequence::sequence).
 * In paired mode first_read and num_anchors must be even.
 */
int cg_correct(cg_ctx* ctx, uint64_t first_read, uint64_t num_anchors,
               uint8_t* out_flags, char* out_sequences, size_t out_pitch);

/*
 * Candidate correction (options.correct_candidates): the combine step of the
 * output stage (reference: combineMultipleCorrectionResults1_rawtcs2,
 * src/correctionresultoutput.cpp:1256-1551).  While correct_candidates is
 * set, every anchor whose MSA is high quality also corrects the candidates of
 * its final MSA that start within new_columns_to_correct columns of the
 * anchor and end at most that far past it (reference: src/msa.cpp:457-522,
 * include/corrector.hpp:293-299, 1504-1512, 1674-1748), and cg_correct keeps
 * those candidate corrections in the context.  A pass is the set of
 * cg_correct calls since the last cg_build_tables; a call on an anchor that
 * the pass already corrected starts a new pass.  After a pass has covered
 * every read, cg_combine_results rewrites flags[j] of read first_read + j,
 * as cg_correct returned it, by the reference's rule: a low-quality anchor
 * correction (CG_RESULT_CORRECTED without CG_RESULT_HQ) with two or more
 * candidate corrections stays only if all of them equal it
 * (CG_RESULT_CANDIDATES, label care:q=2), else the read is written unchanged
 * (CG_RESULT_REJECTED, label care:q=0); CG_RESULT_CANDIDATE_RECORD marks
 * reads with a candidate correction record as a single-threaded reference run
 * saves them (a candidate record of read c made by anchor a is dropped when c
 * < a and c is a corrected HQ anchor; include/corrector.hpp:1678-1681).  The
 * corrected sequences need no change.  *num_candidate_records (may be NULL)
 * gets the number of those records among the reads of the call.
 */
int cg_combine_results(cg_ctx* ctx, uint64_t first_read, uint64_t num_reads, uint8_t* flags,
                       uint64_t* num_candidate_records);

/*
 * Load the anchor classifier for CG_CORR_FOREST from a file image in the
 * reference's forest format (reference: ForestClf, include/forest.hpp:38-55,
 * 141-162; descriptor "13 extract_anchor_v3").  At most max_trees trees are
 * used (0 = all; reference: maxForestTreesAnchor); the decision threshold is
 * options.threshold_anchor.  Needed before cg_correct in forest mode.
 */
int cg_load_forest(cg_ctx* ctx, const void* data, size_t size, uint32_t max_trees);

/* Counters of the context so far. */
int cg_get_stats(const cg_ctx* ctx, cg_stats* out);

/* Number of reads in the store, longest read length. */
int cg_get_read_info(const cg_ctx* ctx, uint64_t* num_reads, int32_t* max_length);

/*
 * Stage access for tests and tools (device results copied to host):
 *  cg_get_signatures:  num_maps keys of each read in [first, first+n), read-major
 *                      (reference: CPUSequenceHasher::hashInto, include/cpusequencehasher.hpp:86-125)
 *  cg_get_candidates:  candidate ids of one anchor after sort/unique/self removal
 *                      (reference: determineCandidateReadIds, include/corrector.hpp:571-650);
 *                      *count gets the number, at most `capacity` are written.
 */
int cg_get_signatures(cg_ctx* ctx, uint64_t first, uint64_t n, uint64_t* out);
/*
 * Whole file-to-file run (reference: care::performCorrection,
 * src/dispatch_care_correct_cpu.cpp:52-252): read 1 input file (single end, or
 * interleaved pairs) or 2 paired files, correct every read, write
 * output_directory/outputs[i] in the input's format (gzip if gz_output),
 * optionally with " care:q=N" header labels.  *num_records gets the number of
 * correction records (the changNum of the queue protocol).
 */
int cg_correct_files(const cg_options* options, const char* const* inputs, int num_inputs,
                     const char* output_directory, const char* const* outputs, int num_outputs,
                     int quality_labels, int gz_output, uint64_t* num_records);
int cg_get_candidates(cg_ctx* ctx, uint64_t anchor, uint32_t* out, uint32_t capacity, uint32_t* count);

/*
 * No counterpart in the reference: cg_get_candidates for callers that cannot
 * allocate device memory (an application that gives its whole device budget
 * to its own pool, or one that looks up single reads in a latency-sensitive
 * loop and must not pay the synchronisation cudaMalloc/cudaFree can imply).
 * Same arguments and result as cg_get_candidates; allocates nothing.  Its
 * scratch is a fixed 33 KiB device array inside the library, held by every
 * GPU that loads it until the process exits, shared by all calls and left
 * holding the last call's data; so calls must not overlap on the GPU.  The
 * first call on a device looks the array up (do it before any stream capture);
 * cg_release_cached_memory(device) makes the next call look it up again.
 * An anchor with more than 8192 raw bucket hits is rejected with
 * CG_ERR_INVALID_ARGUMENT (cg_get_candidates handles it).
 */
int cg_get_candidates_noalloc(cg_ctx* ctx, uint64_t anchor, uint32_t* out, uint32_t capacity, uint32_t* count);

/* ------------------------------------------------------------------------
 * Learned correction classifier (correction_type CG_CORR_LEARNED).  No
 * reference counterpart: it stands where the reference's forest/logistic-
 * regression classifier stands (include/classification.hpp:51-157 and
 * correctAnchorClf, include/corrector.hpp:1448-1472).  For every anchor whose
 * MSA is not high quality, each column whose consensus differs from the
 * anchor's base is scored by a 32-64-64-1 MLP (BF16 weights, FP32
 * accumulation, sigmoid output) over 32 features of the column; the column
 * takes the consensus base when the output reaches threshold_anchor (0.5),
 * otherwise the classic rule's decision (the fallback) stands.
 *
 * Features of a column c of an anchor of length L (in order; a ratio that
 * lies near 1 enters as 1 - ratio, where BF16 keeps its digits): the four
 * base counts / coverage (A, C, G, T); the four base weights / column weight;
 * coverage / estimated coverage; column weight / estimated coverage;
 * 1 - support (consensus weight / column weight); anchor-base weight / column
 * weight; anchor-base count / coverage; 1 - consensus count / coverage;
 * 1 - the mean weight of the anchor base's rows; 1 - the mean weight of the
 * consensus base's rows; 1 - the mean weight of the column's rows; the second
 * largest base weight / column weight; the consensus base one-hot (4); c / L;
 * min(c, L-1-c) / L; 1 - the anchor's average support; 1 - its minimum
 * support; its minimum coverage / estimated coverage; its maximum coverage /
 * estimated coverage; L / 256; the anchor's number of differing columns / L;
 * rows in the MSA / estimated coverage; the quality weight of the anchor base
 * (1 without quality scores).  They include every feature of the reference's
 * forest (extract_anchor_v3, include/classification.hpp:748-797).
 *
 * A serialized classifier is a 32-byte header {char magic[8] = "CGMLP001";
 * uint32 features = 32, hidden1 = 64, hidden2 = 64, payload bytes; uint32
 * reserved[2]} followed by the payload: w1 BF16[64][32], w2 BF16[64][64],
 * w3 BF16[64], b1 FP32[64], b2 FP32[64], b3 FP32, zero padding to 16 bytes.
 * ------------------------------------------------------------------------ */
#define CG_CLASSIFIER_FEATURES 32

/* Bytes of a serialized classifier. */
size_t cg_classifier_size(void);

/* Load the classifier a CG_CORR_LEARNED context uses. */
int cg_load_classifier(cg_ctx* ctx, const void* data, size_t size);

/*
 * The columns the learned decision scores for anchors [first, first+num),
 * without scoring them (needs correction_type CG_CORR_LEARNED, no classifier):
 * features[count][32], the anchor id, the position in the anchor and the
 * consensus base of each.  *count = number of columns; at most `capacity` are
 * written (CG_ERR_INVALID_ARGUMENT if there are more).  The order of the
 * columns is unspecified.
 */
int cg_get_columns(cg_ctx* ctx, uint64_t first, uint64_t num, float* features, uint64_t* anchors,
                   uint16_t* positions, char* consensus, uint64_t capacity, uint64_t* count);

typedef struct cg_train_options {
    int32_t device;
    int32_t epochs;                   /* passes over the training columns (4) */
    int32_t batch_rows;               /* columns per minibatch, a multiple of 16 (4096) */
    float learning_rate;              /* Adam step size (2e-3) */
    uint32_t seed;                    /* initial weights and minibatch order */
    int32_t reserved0;
    const void* init_model;           /* start from this serialized classifier (or NULL) */
    size_t init_model_size;
    int32_t reserved[8];
} cg_train_options;

void cg_default_train_options(cg_train_options* o);

/*
 * Train the classifier on the device (minibatch Adam on the mean binary
 * cross-entropy; forward and backward on the tensor cores).  features[n][32]
 * and labels[n] (1 = the consensus base is the true base).  Writes the
 * serialized classifier to model_out, the loss of every step to losses (up to
 * loss_capacity values) and the number of steps to *steps.
 */
int cg_train_classifier(const cg_train_options* o, const float* features, const uint8_t* labels, uint64_t n,
                        void* model_out, size_t model_capacity, float* losses, uint64_t loss_capacity,
                        uint64_t* steps);

/* Mean loss over the n columns and its gradient with respect to every
 * parameter (6337 values in the payload's order: w1, w2, w3, b1, b2, b3),
 * computed by the training kernels. */
int cg_classifier_gradients(int device, const void* model, size_t model_size, const float* features,
                            const uint8_t* labels, uint32_t n, float* grads, float* loss);

/* Output logits of the classifier for n feature rows (the inference kernel). */
int cg_classifier_logits(int device, const void* model, size_t model_size, const float* features, uint64_t n,
                         float* logits);

#ifdef __cplusplus
}
#endif

#endif /* CARE_GPU_H */
