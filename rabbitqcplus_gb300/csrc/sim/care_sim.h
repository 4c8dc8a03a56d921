// Seeded synthetic read generator for CARE correction workloads (C ABI).
#ifndef CARE_SIM_H
#define CARE_SIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cgsim_config {
    uint64_t seed;
    uint64_t genome_length;
    uint32_t repeat_families;   /* number of repeat source segments */
    uint32_t repeat_copies;     /* diverged copies written per family */
    uint32_t repeat_min_len;
    uint32_t repeat_max_len;
    double repeat_divergence;   /* per-base substitution rate of a copy */
    uint64_t num_reads;         /* total reads (2 x pairs when paired) */
    uint32_t read_len_min;
    uint32_t read_len_max;
    int32_t paired;
    int32_t insert_mean;
    int32_t insert_sd;
    int32_t qual_mean;
    double sub_rate_5p;         /* substitution rate at the 5' end */
    double sub_rate_3p;         /* ... rising linearly to this at the 3' end */
    double indel_rate;
    double n_read_fraction;     /* fraction of reads that get 1-3 'N' bases */
    int32_t qual_sd;
    int32_t qual_min;
    int32_t qual_max;
    int32_t err_qual_min;       /* Phred of an erroneous base ~ U[min,max] */
    int32_t err_qual_max;
    int32_t reserved;
} cgsim_config;

void cgsim_default_config(cgsim_config* c);
void* cgsim_create(const cgsim_config* cfg);
void cgsim_destroy(void* h);
uint64_t cgsim_num_reads(void* h);
uint64_t cgsim_total_bases(void* h);
const uint64_t* cgsim_offsets(void* h);
const char* cgsim_sequences(void* h);
const char* cgsim_qualities(void* h);
const char* cgsim_truth(void* h);
const uint8_t* cgsim_indel_flags(void* h);
int cgsim_write_fastq(void* h, const char* path1, const char* path2);
void cgsim_score(void* h, const char* corrected, uint64_t* tp, uint64_t* fp, uint64_t* fn, uint64_t* reads_scored);
void cgsim_score_results(void* h, uint64_t first, uint64_t count, const uint8_t* flags, const char* rows,
                         uint64_t pitch, uint64_t* tp, uint64_t* fp, uint64_t* fn, uint64_t* reads_scored);

#ifdef __cplusplus
}
#endif

#endif
