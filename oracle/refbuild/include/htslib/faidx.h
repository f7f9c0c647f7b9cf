/* Clean-room subset of htslib's FASTA index API (see hts.h).  Test infrastructure. */
#ifndef BSQ_REF_FAIDX_H
#define BSQ_REF_FAIDX_H

#include "hts.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct faidx_s faidx_t;

faidx_t* fai_load(const char* fn);
void fai_destroy(faidx_t* fai);
/* region "name" or "name:beg-end" (1-based, inclusive); caller frees; *len = bases returned */
char* fai_fetch(const faidx_t* fai, const char* reg, int* len);
int faidx_nseq(const faidx_t* fai);
const char* faidx_iseq(const faidx_t* fai, int i);
int faidx_seq_len(const faidx_t* fai, const char* seq);
int faidx_has_seq(const faidx_t* fai, const char* seq);
char* faidx_fetch_seq(const faidx_t* fai, const char* c_name, int p_beg_i, int p_end_i, int* len);

#ifdef __cplusplus
}
#endif
#endif
