/* Clean-room subset of the htslib 1.23 API that breseq's sources call, written for this repository
 * from the SAM/BAM format specification and htslib's documented interface (names and signatures
 * only).  Test infrastructure: it lets the reference's own error_count / identify_mutations sources
 * compile into the reference oracle; nothing in the product links it. */
#ifndef BSQ_REF_HTS_H
#define BSQ_REF_HTS_H

#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "kstring.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t hts_pos_t;

/* htsExactFormat names a deprecated `json` value; breseq renames it around the include. */
enum htsExactFormat { unknown_format, binary_format, text_format, sam, bam, bai, cram, crai, vcf, bcf, csi, gzi, tbi,
                      bed, htsget, json, empty_format, fasta_format, fastq_format, fai_format, fqi_format, hts_crypt4gh_format,
                      d4_format, format_maximum = 32767 };

typedef struct hts_file_s htsFile;
typedef htsFile samFile;
typedef struct hts_idx_s hts_idx_t;
typedef struct hts_itr_s hts_itr_t;

enum hts_fmt_option { CRAM_OPT_DECODE_MD, HTS_OPT_COMPRESSION_LEVEL = 100, HTS_OPT_NTHREADS, HTS_OPT_BLOCK_SIZE = 106 };

htsFile* hts_open(const char* fn, const char* mode);
int hts_close(htsFile* fp);
int hts_set_opt(htsFile* fp, enum hts_fmt_option opt, ...);
void hts_idx_destroy(hts_idx_t* idx);
void hts_itr_destroy(hts_itr_t* iter);

#ifdef __cplusplus
}
#endif
#endif
