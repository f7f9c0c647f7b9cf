/*
 * breseq_gb300.h -- C ABI of the GB300 read-evidence scoring library (libbsq_gb300.so).
 *
 * The library replaces these parts of breseq's read-evidence scoring path:
 *
 *   error_count pileup      breseq: src/breseq/error_count.cpp:50-68 (error_count)
 *                                   src/breseq/error_count.cpp:125-199 (error_count_pileup::pileup_callback)
 *                                   src/breseq/error_count.cpp:854-986 (cErrorTable::count_alignment_position)
 *   identify_mutations      breseq: src/breseq/identify_mutations.cpp:48-88 (identify_mutations)
 *                                   src/breseq/identify_mutations.cpp:1309-2022 (pileup_callback)
 *   coverage counts         breseq: src/breseq/error_count.cpp:239-253 (unique-only coverage histogram)
 *                                   src/breseq/identify_mutations.cpp:2173-2250 (coverage table rows)
 *   soft-clip tabulation    breseq: src/breseq/soft_clipping.cpp:285-666 (tabulate_soft_clipping_counts)
 *   coverage fit (host)     breseq: src/breseq/coverage_distribution.cpp:115-505 (CoverageDistribution::fit)
 *   BAM2COV table           breseq: src/breseq/coverage_output.cpp:190-470
 *   BAM input               breseq: src/breseq/pileup_base.cpp:61-88, 232-235 (htslib decode)
 *   DP / MP / PD scans      breseq: src/breseq/identify_mutations.cpp:1395-1555, 2358-2967
 *
 * The reference exposes these passes as two C++ free functions that read a BAM/FASTA pair.  Here the
 * host decodes the alignments once into the struct-of-arrays record set `bsq_read_soa`, the library
 * keeps it resident in device memory, and each pass is one call.  Every function returns BSQ_OK (0)
 * or a negative status; the message is available from bsq_last_error().  No function exits the
 * process or traps the device (the reference calls exit(1) from ASSERT, src/breseq/common.h:111-193;
 * a drop-in caller's wrappers with the reference signatures keep that convention on their side).
 *
 * A context is single-threaded.  Buffers passed in are borrowed for the duration of the call only.
 */
#ifndef BRESEQ_GB300_H
#define BRESEQ_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define BSQ_OK               0
#define BSQ_ERR_INVALID     -1   /* bad argument / unsorted records / malformed CIGAR            */
#define BSQ_ERR_CUDA        -2   /* a CUDA runtime call failed                                    */
#define BSQ_ERR_DATA        -3   /* data outside the table (covariate >= max, non-ACGTN base ...) */
#define BSQ_ERR_NOMEM       -4   /* device memory exhausted / admission budget exceeded           */
#define BSQ_ERR_SIZE        -5   /* caller buffer too small; required size returned               */
#define BSQ_ERR_NOSAMPLE    -6   /* unknown sample id                                             */

/* ---------------------------------------------------------------- BAM constants used by the path */
#define BSQ_FLAG_PAIRED      0x1
#define BSQ_FLAG_PROPER      0x2
#define BSQ_FLAG_UNMAP       0x4
#define BSQ_FLAG_MUNMAP      0x8
#define BSQ_FLAG_REVERSE     0x10
#define BSQ_FLAG_MREVERSE    0x20
#define BSQ_FLAG_READ2       0x80
#define BSQ_FLAG_SECONDARY   0x100
#define BSQ_FLAG_QCFAIL      0x200
#define BSQ_FLAG_DUP         0x400
#define BSQ_FLAG_SUPPLEMENTARY 0x800
/* htslib's default pileup filter (BAM_DEF_MASK); breseq never overrides it
 * (src/breseq/pileup_base.cpp:333-339). */
#define BSQ_PILEUP_SKIP_MASK (BSQ_FLAG_UNMAP | BSQ_FLAG_SECONDARY | BSQ_FLAG_QCFAIL | BSQ_FLAG_DUP)

/* ---------------------------------------------------------------- inputs */

/* Reference sequences.  Replaces the FASTA/faidx load of pileup_base::pileup_base
 * (src/breseq/pileup_base.cpp:61-88).  `seq` holds every target's bases, upper-case A/C/G/T/N,
 * concatenated in BAM header order; target t occupies seq[target_offset[t] .. target_offset[t+1]). */
typedef struct bsq_reference {
    uint32_t        n_targets;
    const uint64_t* target_offset;    /* n_targets + 1 */
    const char*     seq;
    /* coverage group of each target (Settings::seq_id_to_coverage_group, src/breseq/settings.cpp:224-258) */
    const uint32_t* coverage_group;
    uint32_t        n_coverage_groups;
    /* targets to pile up, in processing order: the reference walks
     * Settings::call_mutations_seq_id_set(), a std::set<string>, i.e. lexicographic seq_id order
     * (src/breseq/pileup_base.cpp:364-385).  Targets not listed are not scored. */
    const uint32_t* target_order;
    uint32_t        n_target_order;
} bsq_reference;

/* Decoded alignments, one entry per BAM record, coordinate-sorted (tid, pos) in BAM order.
 * Fields mirror the accessors of alignment_wrapper / pileup_wrapper (src/breseq/alignment.h:43-416).
 * Read i's bases are the 4-bit BAM codes at nibble index seq_off[i] + q of `seq` (high nibble first,
 * as in BAM), its qualities are qual[seq_off[i] + q]; seq_off[i] must be even.  CIGAR ops are the
 * BAM encoding (len << 4 | op) at cigar[cigar_off[i] ..]. */
typedef struct bsq_read_soa {
    uint64_t        n_reads;
    const int32_t*  tid;
    const int32_t*  pos;           /* 0-based leftmost reference position                        */
    const uint16_t* flag;
    const uint8_t*  mapq;
    const uint32_t* x1;            /* X1:i redundancy, 1 when the tag is absent (alignment.cpp:52-57) */
    const int32_t*  xl;            /* XL:i left trim,  -1 when absent (alignment.h:389-411)        */
    const int32_t*  xr;            /* XR:i right trim, -1 when absent                              */
    const uint8_t*  read_file;     /* flat read-file index: read group + mate (alignment.h:576-592)*/
    const uint16_t* read_group;    /* dense @RG index (alignment.h:533-573)                        */
    const uint32_t* l_qseq;
    const uint64_t* seq_off;
    const uint64_t* cigar_off;
    const uint16_t* n_cigar;
    const uint32_t* cigar;
    const uint8_t*  seq;
    const uint8_t*  qual;
    uint64_t        n_cigar_total;
    uint64_t        n_bases_total;   /* length of qual[] (and 2 x length of seq[])               */
    /* non-zero when the record carries an XJ:i tag (one side of a junction match); NULL when no
     * record does.  Only the soft-clipping tabulation reads it (src/breseq/soft_clipping.cpp:382-384). */
    const uint8_t*  xj;
    /* Pair annotations, read only by the discordant / missing-pair scans (bsq_pair_candidates);
     * NULL when absent.  isize: TLEN.  xp: the XP:Z pair orientation breseq writes
     * (src/breseq/resolve_alignments.cpp:1255-1273) as BSQ_XP_FR / _RF / _FF, BSQ_XP_NONE when the
     * tag is absent or holds anything else.  qname: read names concatenated without terminators,
     * read i at [qname_off[i], qname_off[i+1]), at most 254 bytes each (the BAM limit). */
    const int32_t*  isize;
    const uint8_t*  xp;
    const uint64_t* qname_off;
    const char*     qname;
    /* mate reference id and 0-based position (RNEXT / PNEXT), read only by the pair-distance scan;
     * NULL when absent */
    const int32_t*  mtid;
    const int32_t*  mpos;
} bsq_read_soa;

#define BSQ_XP_FR   0
#define BSQ_XP_RF   1
#define BSQ_XP_FF   2
#define BSQ_XP_NONE 3

/* ---------------------------------------------------------------- pass 1: error counts */

/* Parameters of error_count() (src/breseq/error_count.h:44-56).  The covariate string the pipeline
 * uses is "read_set=R,obs_base,ref_base,quality=Q" (src/breseq/breseq_cmdline.cpp:2304), giving the
 * table index  idx = rs + R*(ref + 5*(obs + 5*q))  (src/breseq/error_count.cpp:477-497). */
typedef struct bsq_ec_params {
    uint32_t n_read_files;           /* R */
    uint32_t n_quality;              /* Q = max_qual + 1 */
    int32_t  do_coverage;
    int32_t  do_errors;
    int32_t  preprocess_stage;
    /* Settings::required_junction_read_end_min_coordinate (src/breseq/settings.h:345-354) */
    uint32_t unmatched_end_minimum_read_length;
    double   unmatched_end_length_factor;
} bsq_ec_params;

/* Caller-owned outputs of pass 1. */
typedef struct bsq_ec_result {
    uint64_t* counts;          /* [R*5*5*Q] covariate counts                                 */
    uint64_t* coverage_hist;   /* [n_coverage_groups * hist_capacity]                        */
    uint32_t  hist_capacity;   /* bins per group supplied by the caller                      */
    uint32_t* hist_size;       /* [n_coverage_groups] out: reference vector size (max cov + 1) */
    double*   no_pos_hash_pr;  /* [n_targets] preprocess only (may be NULL)                  */
} bsq_ec_result;

/* ---------------------------------------------------------------- pass 2: identify mutations */

#define BSQ_PRECISION_FP64   0   /* plain form: FP64 sums and the EM at every column            */
#define BSQ_PRECISION_FP32C  1   /* FP32 Kahan-compensated sums, candidate screen, FP64 EM       */

typedef struct bsq_im_params {
    uint32_t n_read_files;                 /* R of the error table                               */
    uint32_t n_quality;                    /* Q of the error table                               */
    uint32_t base_quality_cutoff;          /* Settings::base_quality_cutoff (default 3)          */
    double   mutation_cutoff;              /* consensus score cutoff (mutation_log10_e_value_cutoff) */
    double   polymorphism_cutoff;          /* polymorphism_log10_e_value_cutoff                  */
    double   polymorphism_precision_decimal;
    uint32_t polymorphism_precision_places;
    int32_t  skip_missing_coverage_prediction;
    double   log10_ref_length;             /* log10 of the summed BAM target lengths (identify_mutations.cpp:848-852) */
    const double* deletion_propagation_cutoff;  /* [n_targets] */
    const double* deletion_seed_cutoff;         /* [n_targets] */
    int32_t  precision;                    /* BSQ_PRECISION_* */
    /* Discordant-pair groups of the identify_mutations pileup (identify_mutations.cpp:883-911):
     * dp_group[g] >= 0 for each dense read group g that is a paired read-file set with a paired
     * mapping-distance fit, -1 otherwise; n_read_groups entries, at most 256 of them DP groups.
     * 0 / NULL: no DP group.  At a read's first aligned column, insert position 0, breseq's
     * per-read loop leaves out (`continue`, :1399-1416) a primary, mapped, paired read of a DP
     * group that is not a proper pair, has a mapped mate, and has no XP tag or one other than
     * FR / RF / FF; the passes do the same (the record's XP comes from bsq_read_soa.xp, none
     * when that is NULL). */
    uint32_t n_read_groups;
    const int32_t* dp_group;
} bsq_im_params;

/* One RA evidence item with raw (unformatted) values; identify_mutations.cpp:1836-1910. */
typedef struct bsq_ra_record {
    uint32_t tid;
    uint32_t position;          /* 1-based */
    uint32_t insert_position;
    char     ref_base, new_base, major_base, minor_base;
    double   score;             /* variant presence score, NaN when there is no variant allele */
    double   consensus_score;   /* pure-genotype score minus log10(reference length)         */
    double   f[5];              /* fitted allele frequencies A,C,G,T,'.'                      */
    double   major_frequency;   /* reported (floored) frequency of the major allele          */
    double   frequency;         /* reported frequency of the variant allele                  */
    double   frequency_lower;
    double   frequency_upper;
    double   fisher_strand_p;
    double   ks_quality_p;
    int32_t  ref_cov[2], new_cov[2], major_cov[2], minor_cov[2], total_cov[2];   /* top, bottom */
    uint32_t n;                 /* read bases in the fit */
    uint8_t  passed_consensus;
    uint8_t  passed_polymorphism;
    uint8_t  pad[2];
} bsq_ra_record;

/* MC (missing coverage) item; identify_mutations.cpp:2262-2344, 2140-2159. */
typedef struct bsq_mc_record {
    uint32_t tid, start, end, start_range, end_range;
    uint32_t pad;
    double   left_outside_cov, left_inside_cov, right_inside_cov, right_outside_cov;  /* NaN = NA */
} bsq_mc_record;

/* UN (unknown base) interval; identify_mutations.cpp:2972-3007. */
typedef struct bsq_un_record {
    uint32_t tid, start, end;
} bsq_un_record;

/* Per-position outputs (insert position 0) for the coverage table and checks.  Arrays of length
 * total reference length, indexed by the global column target_offset[t] + position_0. */
typedef struct bsq_position_arrays {
    uint32_t* unique_top;       /* may be NULL */
    uint32_t* unique_bot;
    double*   redundant_top;
    double*   redundant_bot;
    uint32_t* raw_redundant_top;
    uint32_t* raw_redundant_bot;
    double*   consensus_score;  /* NaN where no read base scored */
    uint8_t*  best_base;        /* 0..4 = A,C,G,T,'.'; 5 = N */
    uint32_t* n_scored;
} bsq_position_arrays;

/* ---------------------------------------------------------------- RA classification */

/* The Settings fields test_RA_evidence reads (src/breseq/identify_mutations.cpp:143-749); defaults from
 * bsq_default_ra_settings (src/breseq/settings.cpp:857-950).  A cutoff of 0 switches its test off. */
typedef struct bsq_ra_settings {
    int32_t  polymorphism_prediction;
    uint32_t polymorphism_precision_places;
    double   mutation_log10_e_value_cutoff;
    double   consensus_frequency_cutoff;
    double   consensus_minimum_variant_coverage;
    double   consensus_minimum_total_coverage;
    double   consensus_minimum_variant_coverage_each_strand;
    double   consensus_minimum_total_coverage_each_strand;
    uint32_t consensus_reject_indel_homopolymer_length;
    uint32_t consensus_reject_surrounding_homopolymer_length;
    double   polymorphism_log10_e_value_cutoff;
    double   polymorphism_frequency_cutoff;
    double   polymorphism_minimum_variant_coverage;
    double   polymorphism_minimum_total_coverage;
    double   polymorphism_minimum_variant_coverage_each_strand;
    double   polymorphism_minimum_total_coverage_each_strand;
    uint32_t polymorphism_reject_indel_homopolymer_length;
    uint32_t polymorphism_reject_surrounding_homopolymer_length;
    double   polymorphism_fisher_strand_p_value_cutoff;
    double   polymorphism_ks_quality_p_value_cutoff;
    int32_t  polymorphism_no_indels;
} bsq_ra_settings;

/* Outcome of test_RA_evidence for one RA item. */
typedef struct bsq_ra_call {
    char    prediction[16];            /* "consensus" / "polymorphism" / "" */
    char    reject[96];                /* comma-separated reasons                  */
    char    consensus_reject[96];
    char    polymorphism_reject[96];
    uint8_t deleted;                   /* the reference drops the item             */
    uint8_t pad[7];
} bsq_ra_call;

int bsq_default_ra_settings(int polymorphism_prediction, bsq_ra_settings* s);

/* test_RA_evidence (src/breseq/identify_mutations.cpp:687-749) on RA items as they would be written to
 * and read back from the GenomeDiff (values formatted with the reference's precision first). */
int bsq_test_ra_evidence(const bsq_ra_record* ra, uint64_t n, const bsq_ra_settings* s, const bsq_reference* ref,
                         const char* const* target_names, bsq_ra_call* out);

/* ---------------------------------------------------------------- output files */

/* error_rates.tab: counts_to_log10_prob + write_log10_prob_table (src/breseq/error_count.cpp:660-690, 1005-1026) */
int bsq_write_error_rates(const char* path, const uint64_t* counts, uint32_t n_read_files, uint32_t n_quality);
/* base_qual_error_prob.#.tab, '#' replaced by each read file's name (error_count.cpp:697-785) */
int bsq_write_base_qual_error_prob(const char* path_pattern, const char* const* read_file_names, const uint64_t* counts,
                                   uint32_t n_read_files, uint32_t n_quality);
/* <group>.unique_only_coverage_distribution.tab (error_count.cpp:239-253); size = hist_size of the group */
int bsq_write_coverage_distribution(const char* path, const uint64_t* hist, uint32_t size);
/* <seq_id>.coverage.tsv aggregate columns from per-position arrays (identify_mutations.cpp:2028-2052, 2173-2204) */
int bsq_write_coverage_table(const char* path, const char* seq_id, const bsq_reference* ref, uint32_t tid,
                             const bsq_position_arrays* positions);
/* One RA item as its GenomeDiff fields (tab-separated, no type / id / evidence columns). */
int bsq_format_ra(const bsq_ra_record* ra, const char* seq_id, uint32_t precision_places, char* buf, uint64_t cap);
/* ra_mc_evidence.gd: RA / MC / UN lines with ids in the pileup's add order and cGenomeDiff's sort order
 * (src/breseq/genome_diff.cpp:685-760, genome_diff_entry.cpp:570-660).  `calls` (may be NULL) adds the
 * test_RA_evidence fields and leaves out deleted items. */
int bsq_write_gd(const char* path, const bsq_reference* ref, const char* const* target_names,
                 const double* deletion_propagation_cutoff, uint32_t precision_places,
                 const bsq_ra_record* ra, uint64_t n_ra, const bsq_ra_call* calls,
                 const bsq_mc_record* mc, uint64_t n_mc, const bsq_un_record* un, uint64_t n_un);

/* ---------------------------------------------------------------- coverage-distribution fit */

/* The negative-binomial fit of a coverage group's unique-only coverage histogram and the deletion-
 * propagation cutoff breseq derives from it (CoverageDistribution::fit and
 * analyze_unique_coverage_distribution, src/breseq/coverage_distribution.cpp:115-396, 437-505,
 * 566-588).  Host code: 48 Nelder-Mead restarts on host threads, the result independent of their
 * number.  Fields named after the Summary's unique_coverage entries; the nbinom_* parameters stay 0
 * when the fit fails (nbinom_mean == 0). */
typedef struct bsq_coverage_fit {
    double   nbinom_size;               /* nbinom_size_parameter */
    double   nbinom_mean;               /* nbinom_mean_parameter */
    double   nbinom_prob;               /* size / (mean + size) */
    double   nbinom_variance;           /* mean + mean^2 / size */
    double   nbinom_relative_variance;  /* variance / mean */
    double   average;                   /* histogram mean over coverage >= 1 */
    double   variance;                  /* sample variance */
    double   relative_variance;
    double   deletion_coverage_propagation_cutoff;   /* -1: the sequences themselves are deleted */
    double   nbinom_scale;              /* scales dnbinom to the histogram's counts (the plot's curve) */
    uint32_t censor_start;              /* fitting window [censor_start, censor_end]; equal: no fit */
    uint32_t censor_end;
    uint32_t restarts_converged;        /* of the 48 restarts */
    uint32_t reserved;
} bsq_coverage_fit;

/* hist / hist_size as bsq_ec_result gives them (the .tab file's rows 1 .. hist_size-1).
 * deletion_propagation_pr_cutoff: breseq uses 0.05 / sqrt(total length of the group's sequences)
 * (coverage_distribution.cpp:545).  n_threads <= 0: one per host core, at most 48.
 * BSQ_ERR_DATA where the reference would stop on an assertion (a probability mass function evaluated
 * at mean or size 0). */
int bsq_fit_coverage_distribution(const uint64_t* hist, uint32_t hist_size, double deletion_propagation_pr_cutoff,
                                  int n_threads, bsq_coverage_fit* out);
/* fit_negative_binomial_histogram (coverage_distribution.cpp:402-409): n[0..max_index], n[0] ignored.
 * Returns 1 when size and mu are both positive, 0 when the fit failed, < 0 on error. */
int bsq_fit_negative_binomial(const double* n, uint32_t max_index, int n_threads, double* size, double* mu);
/* The negative-binomial functions of src/breseq/stats.h:92-105 / stats.cpp:982-990, 2047-2072:
 * R's dnbinom(k, size, mu=mu), the CDF P(X <= k) with success probability p (Cephes nbdtr), and
 * qnbinom(target, size, mu=mu). */
double bsq_nbinom_pmf(double k, double size, double mu);
double bsq_nbinom_cdf(double k, double size, double p);
int    bsq_nbinom_quantile(double target_pr, double size, double mu, uint64_t* k);

/* ---------------------------------------------------------------- context API */

typedef struct bsq_ctx bsq_ctx;

/* Create a context on CUDA device `device`.  Fails with BSQ_ERR_CUDA when no device is present. */
int         bsq_create(bsq_ctx** out, int device);
void        bsq_destroy(bsq_ctx* ctx);
const char* bsq_last_error(const bsq_ctx* ctx);
const char* bsq_version(void);

/* Upload a sample (reference + records) to device memory and keep it resident.  Records are
 * validated (sorted, CIGAR consumes the reference, offsets inside the arrays).  Replaces the BAM/BAI/
 * FASTA open of pileup_base::pileup_base (src/breseq/pileup_base.cpp:61-88). */
int bsq_load_sample(bsq_ctx* ctx, const bsq_reference* ref, const bsq_read_soa* reads, int32_t* sample_id);
int bsq_free_sample(bsq_ctx* ctx, int32_t sample_id);
/* Device bytes a sample of this shape occupies (for admission by HBM footprint). */
uint64_t bsq_sample_footprint(const bsq_reference* ref, const bsq_read_soa* reads);

/* Pass 1.  Replaces error_count() (src/breseq/error_count.cpp:50-68) minus its file writers, which
 * are bsq_write_error_rates / bsq_write_coverage_distribution below. */
int bsq_error_count(bsq_ctx* ctx, int32_t sample_id, const bsq_ec_params* p, bsq_ec_result* out);

/* Convert pass-1 counts into the log10 probability table exactly as breseq round-trips it through
 * error_rates.tab: counts_to_log10_prob (error_count.cpp:1005-1026), printed with 6 significant
 * digits (write_log10_prob_table, :660-690) and parsed back (read_log10_prob_table, :629-654).
 * log10_prob must hold R*5*5*Q doubles. */
int bsq_counts_to_log10_prob(const uint64_t* counts, uint32_t n_read_files, uint32_t n_quality, double* log10_prob);
/* The same for n tables at once (host threads). */
int bsq_counts_to_log10_prob_batch(uint32_t n, const uint64_t* const* counts, const uint32_t* n_read_files,
                                   const uint32_t* n_quality, double* const* log10_prob);

/* Pass 2.  Replaces identify_mutations() (src/breseq/identify_mutations.cpp:48-88) for RA, MC, UN
 * and the coverage table.  Results are kept in the context until the next call and read with
 * bsq_im_result_counts / bsq_im_result_copy.  `pos_out` may be NULL. */
int bsq_identify_mutations(bsq_ctx* ctx, int32_t sample_id, const bsq_im_params* p,
                           const double* log10_prob_table, bsq_position_arrays* pos_out);
int bsq_im_result_counts(const bsq_ctx* ctx, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un);
int bsq_im_result_copy(const bsq_ctx* ctx, bsq_ra_record* ra, uint64_t ra_cap,
                       bsq_mc_record* mc, uint64_t mc_cap, bsq_un_record* un, uint64_t un_cap);

/* The MC and UN intervals of per-position arrays (identify_mutations.cpp:2107-2164 at the target ends,
 * check_deletion_completion :2262-2344, update_unknown_intervals :2972-3007): the state machines run
 * over every position of the targets in ref->target_order, with a position's consensus call predicted
 * when consensus_score >= p->mutation_cutoff (NaN: not).  Reads unique_top/bot, redundant_top/bot and
 * consensus_score of `positions` (indexed as bsq_identify_mutations fills them).  Host code: this is how
 * the results of position ranges scored apart (one per GPU) are joined into one sample's intervals.
 * BSQ_ERR_SIZE, with *n_mc / *n_un set, when a capacity is short. */
int bsq_intervals_from_positions(const bsq_reference* ref, const bsq_position_arrays* positions, const bsq_im_params* p,
                                 bsq_mc_record* mc, uint64_t mc_cap, uint64_t* n_mc, bsq_un_record* un, uint64_t un_cap,
                                 uint64_t* n_un);

/* Batch forms: n samples scored by one launch per kernel of the pass (every sample's reads or
 * column tiles are units of one persistent grid).  Element j of each array belongs to sample_ids[j];
 * the results of each sample equal those of the single-sample call.  breseq runs error_count and
 * identify_mutations once per sample (src/breseq/breseq_cmdline.cpp:1969, :2293); a caller scoring
 * many samples issues one batch call instead.  The single-sample functions above are batches of one.
 * All samples of one bsq_identify_mutations_batch call use the same `precision`.  Results of the
 * identify batch are read per job index j (0..n-1) until the next pass-2 call.  `pos_out` may be
 * NULL, and so may any pos_out[j]. */
int bsq_error_count_batch(bsq_ctx* ctx, uint32_t n, const int32_t* sample_ids, const bsq_ec_params* p,
                          bsq_ec_result* out);
int bsq_identify_mutations_batch(bsq_ctx* ctx, uint32_t n, const int32_t* sample_ids, const bsq_im_params* p,
                                 const double* const* log10_prob_tables, bsq_position_arrays* const* pos_out);
int bsq_im_batch_result_counts(const bsq_ctx* ctx, uint32_t job, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un);
int bsq_im_batch_result_copy(const bsq_ctx* ctx, uint32_t job, bsq_ra_record* ra, uint64_t ra_cap,
                             bsq_mc_record* mc, uint64_t mc_cap, bsq_un_record* un, uint64_t un_cap);

/* ---------------------------------------------------------------- soft-clipping tabulation */

/* Settings of tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666), which breseq runs
 * in the error-calibration step over the same BAM (src/breseq/breseq_cmdline.cpp:2307-2318) when
 * --predict-soft-clipping is given.  Defaults: src/breseq/settings.cpp:1369-1374 (bsq_default_sc_params). */
typedef struct bsq_sc_params {
    uint32_t minimum_clipped_bases;      /* soft_clipping_minimum_bases (12)               */
    double   consensus_base_fraction;    /* soft_clipping_consensus_base_fraction (0.95)   */
    double   dispersion_trim_frequency;  /* soft_clipping_dispersion_trim_frequency (0.25) */
    double   maximum_dispersion;         /* soft_clipping_maximum_dispersion (0.005)       */
    double   minimum_rate;               /* soft_clipping_minimum_rate (1e-5)              */
    /* every target once, in std::string order of the seq_ids: the order of the rows (the reference
     * keys its tallies by seq_id in std::map).  NULL = target index order. */
    const uint32_t* target_name_order;
} bsq_sc_params;

/* Summary::soft_clipping (src/breseq/summary.h:333-364), plus the unclamped values the reference
 * prints and the number of rows. */
typedef struct bsq_sc_summary {
    uint64_t total_spanning_read_bases;
    uint64_t total_clipped_read_ends;
    uint64_t total_agreeing_clipped_read_ends;
    double   soft_clipping_rate;
    double   null_rate;                  /* p0 used: agreeing rate after the minimum-rate floor */
    double   null_rate_raw;
    double   dispersion;                 /* rho used; 0 = plain binomial */
    double   dispersion_raw;
    double   pearson_phi;
    uint64_t tested_positions;           /* N': (position, direction) pairs entering the fit */
    uint64_t trimmed_positions;
    double   mean_tested_reads;
    uint64_t n_positions;                /* rows: (position, direction) pairs with clip events */
} bsq_sc_summary;

/* One row of soft_clipping_counts.tab (soft_clipping.cpp:520-545, 639-646). */
typedef struct bsq_sc_position {
    uint32_t target;
    uint32_t position;                   /* 1-based */
    int32_t  direction;                  /* -1: leading clip at reference_start_1; +1: trailing clip at reference_end_1 */
    uint32_t clipped_count;
    uint32_t total_count;                /* clipped reads + reads spanning the position */
    uint32_t agree_count;
    char     clipped_sequence[24];       /* consensus tail, reference-forward, NUL-terminated; "" = none */
} bsq_sc_position;

int bsq_default_sc_params(bsq_sc_params* p);
/* Tabulates the clip events of a resident sample.  Every mapped record counts except X1 > 1 and
 * XJ-tagged ones (the pileup's flag filter does not apply).  Rows are kept in the context until
 * the next call; read them with bsq_sc_result_copy (summary->n_positions rows, in the reference's
 * order: direction -1 then +1, targets in target_name_order, positions ascending). */
int bsq_soft_clipping(bsq_ctx* ctx, int32_t sample_id, const bsq_sc_params* p, bsq_sc_summary* summary);
int bsq_sc_result_copy(const bsq_ctx* ctx, bsq_sc_position* rows, uint64_t capacity);
/* soft_clipping_counts.tab (soft_clipping.cpp:625-646). */
int bsq_write_soft_clipping_counts(const char* path, const char* const* target_names, const bsq_sc_params* p,
                                   const bsq_sc_summary* s, const bsq_sc_position* rows, uint64_t n);

/* ---------------------------------------------------------------- BAM input on the device */

/* breseq reads reference.bam through htslib on the host (src/breseq/pileup_base.cpp:61-88,
 * 232-235): BGZF inflate, then record decode.  Here the file's bytes are uploaded once, every BGZF
 * block is inflated on the device by its own warp (its CRC-32 checked), and the records are
 * decoded there into the bsq_read_soa layout.  Records must not span BGZF blocks, which htslib's
 * writer guarantees for records under 64 KiB; a file that breaks this is refused (BSQ_ERR_INVALID).
 * Unplaced records (refID -1), which a coordinate-sorted file keeps last, are dropped. */
typedef struct bsq_bam bsq_bam;
int  bsq_bam_open(bsq_ctx* ctx, const uint8_t* data, uint64_t size, bsq_bam** out);
void bsq_bam_close(bsq_bam* bam);
/* The header text and the reference sequences it names (valid until bsq_bam_close). */
int bsq_bam_header(const bsq_bam* bam, const char** text, uint64_t* text_len, uint32_t* n_ref,
                   const char* const** ref_names, const uint32_t** ref_lengths);

/* Read groups as breseq resolves them: the @RG IDs in header order (read_group_index_map,
 * src/breseq/alignment.h:533-560: a record without RG, with an unknown ID, or in a header with at
 * most one group gets group 0) and each group's first flat read-file index and file count
 * (read_file_partition, :569-607).  file_base / file_count NULL: no read file sets, every record's
 * read file is 0. */
typedef struct bsq_bam_groups {
    uint32_t           n_groups;      /* at most 64 */
    const char* const* ids;
    const uint32_t*    file_base;
    const uint32_t*    file_count;
} bsq_bam_groups;

/* Decodes the records on the device; the counts size the arrays of bsq_bam_copy_records. */
int bsq_bam_decode(bsq_ctx* ctx, bsq_bam* bam, const bsq_bam_groups* groups, uint64_t* n_records,
                   uint64_t* n_cigar_total, uint64_t* n_bases_total);

/* Writable arrays in the bsq_read_soa layout (sizes: n_records, n_cigar_total, n_bases_total and
 * n_bases_total / 2 for seq). */
typedef struct bsq_read_arrays {
    int32_t*  tid;
    int32_t*  pos;
    uint16_t* flag;
    uint8_t*  mapq;
    uint32_t* x1;
    int32_t*  xl;
    int32_t*  xr;
    uint8_t*  read_file;
    uint16_t* read_group;
    uint32_t* l_qseq;
    uint64_t* seq_off;
    uint64_t* cigar_off;
    uint16_t* n_cigar;
    uint32_t* cigar;
    uint8_t*  seq;
    uint8_t*  qual;
    uint8_t*  xj;
    /* pair annotations, each optional (NULL: not copied): isize [n_records], xp [n_records],
     * qname_off [n_records + 1], qname [bsq_bam_name_bytes] */
    int32_t*  isize;
    uint8_t*  xp;
    uint64_t* qname_off;
    char*     qname;
    int32_t*  mtid;
    int32_t*  mpos;
} bsq_read_arrays;
int bsq_bam_copy_records(bsq_ctx* ctx, const bsq_bam* bam, const bsq_read_arrays* out);
/* Bytes of the decoded records' read names (no terminators). */
int bsq_bam_name_bytes(bsq_ctx* ctx, const bsq_bam* bam, uint64_t* bytes);

/* Makes the decoded records a resident sample with the given reference (whose targets must be the
 * header's, in order and length), as bsq_load_sample does with host arrays.  The decoded arrays move
 * into the sample; decode again to load another copy. */
int bsq_bam_load(bsq_ctx* ctx, bsq_bam* bam, const bsq_reference* ref, int32_t* sample_id);

/* ---------------------------------------------------------------- BAM2COV coverage table */

/* Per-position coverage of one region as `breseq BAM2COV --format TSV` tabulates it
 * (coverage_output::pileup_callback, src/breseq/coverage_output.cpp:307-470; command at
 * src/breseq/breseq_cmdline.cpp:294): over the records htslib's pileup keeps (flag filter only, on
 * every target), deletion entries skipped, N bases counted.  Each array holds end_1 - start_1 + 1
 * entries, position start_1 first; any may be NULL. */
typedef struct bsq_cov_columns {
    uint32_t* unique_top;                /* X1 = 1 records, forward strand              */
    uint32_t* unique_bot;
    double*   redundant_top;             /* sum of 1/X1 over X1 > 1 records, in BAM order */
    double*   redundant_bot;
    uint32_t* raw_redundant_top;
    uint32_t* raw_redundant_bot;
    uint32_t* unique_top_begin;          /* unique records whose first sequenced base is here */
    uint32_t* unique_bot_begin;
} bsq_cov_columns;
/* last_column_1 (may be NULL) gets the last reference position any kept record overlapping the
 * region reaches (the pileup's last column; 0 when there is none). */
int bsq_coverage_columns(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                         bsq_cov_columns* out, uint32_t* last_column_1);

#define BSQ_COV_TOTAL_ONLY  1   /* --total-only: unique_cov, redundant_cov, total_cov */
#define BSQ_COV_CSV         2   /* --format CSV (comma-separated) instead of TSV       */
#define BSQ_COV_PER_READ_GROUP 4   /* --per-read-group (bsq_write_coverage_region_rg)  */
/* coverage_output::table (coverage_output.cpp:190-284) for the region seq_id:start_1-end_1 with
 * --resolution (0 = every position), including the pileup driver's row selection
 * (pileup_base.cpp:130-133, 141-210, 308-355).  reference_average (may be NULL) adds the
 * reference_unique_average_cov line of --show-average. */
int bsq_write_coverage_region(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id, uint32_t tid,
                              uint32_t start_1, uint32_t end_1, uint32_t resolution, uint32_t flags,
                              const double* reference_average);
/* The same with BSQ_COV_PER_READ_GROUP honoured: after the aggregate columns, the columns of each read
 * group 0 .. max(n_read_groups, 1) - 1 prefixed "RG-<g>_" (the header's @RG count; a record's group is
 * its read_group), and per group the three region averages after number_of_positions
 * (coverage_output.cpp:236-247, 270-278, 364-500). */
int bsq_write_coverage_region_rg(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id, uint32_t tid,
                                 uint32_t start_1, uint32_t end_1, uint32_t resolution, uint32_t flags,
                                 const double* reference_average, uint32_t n_read_groups);
/* The columns of one read group's records (read_group < 0: all records, as bsq_coverage_columns). */
int bsq_coverage_columns_rg(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                            int32_t read_group, bsq_cov_columns* out, uint32_t* last_column_1);
/* identify_mutations' per-position coverage tally restricted to one read group's records (read_group < 0:
 * all), positions start_1..end_1 of target tid: at insert position 0 every pileup entry whose read base
 * is not N, deletions included (identify_mutations.cpp:1560-1610); where the target's coverage fit failed
 * (coverage_fit_failed != 0) tabulate_position_coverage's, which leaves deletions out too (:2218-2250).
 * dp_group (n_read_groups entries, as bsq_im_params.dp_group; NULL: none): in the main-loop tally a
 * record of a read group with a discordant-pair group that pass 2 leaves out of its first column
 * (the `continue` at :1399-1416) is left out of that column's tally too.
 * Fills unique_*, raw_redundant_* and redundant_* of `out`; the begin counters are zeroed. */
int bsq_im_coverage_columns_rg(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                               int32_t read_group, int coverage_fit_failed, uint32_t n_read_groups,
                               const int32_t* dp_group, bsq_cov_columns* out);
/* <seq_id>.coverage.tsv (identify_mutations.cpp:2028-2052, 2173-2250; written under --predict-copy-number):
 * the aggregate columns from pass 2's per-position arrays, as bsq_write_coverage_table, and with more than
 * one read group (:862) each group's unique_cov / redundant_cov / total_cov prefixed "RG-<g>_", tallied on
 * the device by bsq_im_coverage_columns_rg over the resident sample, 2^20 positions at a time.
 * dp_group: as for bsq_im_coverage_columns_rg (n_read_groups entries or NULL). */
int bsq_write_coverage_table_rg(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id,
                                const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* positions,
                                uint32_t n_read_groups, int coverage_fit_failed, const int32_t* dp_group);

/* Launch shape of the passes.  None of the knobs changes a result: every count is an integer sum
 * and every column and candidate is scored by one warp whatever the grid. */
typedef struct bsq_tuning {
    uint32_t ec_read_chunk;       /* reads per pass-1 work unit (default 1024)                  */
    uint32_t ec_blocks_per_sm;    /* pass-1 blocks per SM (default 8)                            */
    uint32_t col_blocks_per_sm;   /* column-pass blocks of 8 warps per SM (default 8)            */
    uint32_t cand_warps_per_sm;   /* candidate-kernel warps per SM (default 16)                  */
    uint32_t bound_warps_per_sm;  /* frequency-bound bisections in flight per SM, 1-8 (default 4) */
    int32_t  use_graphs;          /* capture each pass as one CUDA graph, updated in place (default 1) */
} bsq_tuning;
int bsq_get_tuning(const bsq_ctx* ctx, bsq_tuning* out);
int bsq_set_tuning(bsq_ctx* ctx, const bsq_tuning* t);
/* Times the passes over the given resident samples under candidate launch shapes (one knob at a
 * time, CUDA events around each pass), keeps the fastest in the context and returns it in *chosen.
 * Runs both passes several times; the samples' results are not kept. */
int bsq_autotune(bsq_ctx* ctx, uint32_t n, const int32_t* sample_ids, const bsq_ec_params* ec,
                 const bsq_im_params* im, const double* const* log10_prob_tables, bsq_tuning* chosen);

/* Timing of the last pass on the device (CUDA events around the kernels, milliseconds) and the
 * number of kernels launched by it. */
int bsq_last_pass_stats(const bsq_ctx* ctx, double* device_ms, uint32_t* kernel_launches,
                        double* main_kernel_ms);

/* Bytes the last pass call copied host-to-device and device-to-host (staged inputs, results). */
int bsq_last_pass_bytes(const bsq_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* ---------------------------------------------------------------- discordant / missing-pair / pair-distance scans */

/* The discordant-pair (DP) and missing-pair (MP) candidate-region scans that breseq runs inside the
 * identify_mutations pileup (identify_mutations.cpp:1395-1493 enter steps, 2358-2437 and 2439-2522
 * sliding windows, 2524-2586 writers; groups at :883-913).  Read groups map to DP groups: a paired
 * read-file set with a fitted paired-mapping distance, window width median + 2.42 * MAD.  Per bin
 * (focal strand x XP orientation for DP, strand for MP) a region is a maximal run of positions where
 * the reads that started within the window reach the seed; MP also needs the mate-unmapped reads to
 * be at least missing_pair_seed_fraction of all primary mapped reads of that strand in the window.
 * PD: per position, the rank-sum z of the distance quantiles of the concordant pairs whose
 * unsequenced gap covers it, and the count of those in the long or short tail. */
typedef struct bsq_pair_params {
    uint32_t        n_read_groups;       /* entries of dp_group (the sample's read-group indices) */
    const int32_t*  dp_group;            /* per read group: its DP group, -1 when none */
    uint32_t        n_dp_groups;         /* at most 255 */
    const double*   window_width;        /* per DP group: median + 2.42 * MAD */
    const uint32_t* r1_name_prefix;      /* per DP group: m_id + 1 of the set's R1 / R2 read file */
    const uint32_t* r2_name_prefix;
    int32_t         discordant_pair_seed;          /* --discordant-pair-seed, default 3 */
    int32_t         predict_missing_pairs;         /* --predict-missing-pairs */
    int32_t         missing_pair_seed;             /* --missing-pair-seed, default 3 */
    double          missing_pair_seed_fraction;    /* --missing-pair-seed-fraction, default 0.25 */
    /* per target: identify_mutations' deletion propagation cutoff; a target below 0 is not piled up
     * (pileup_callback returns at once, identify_mutations.cpp:1318-1329) */
    const double*   deletion_propagation_cutoff;
    /* Pair-distance (PD) scan (--predict-pair-distance; identify_mutations.cpp:920-1006 setup,
     * :1514-1555 enter step, :2588-2757 windows, :2758-2967 calibration and writer).  Needs the
     * records' mtid / mpos.  Per DP group: the null as pd_build_cdf builds it (:112-141: the mid-CDF
     * of the length-bias-corrected distance histogram in 2^20 fixed point, indexed by distance; length
     * 0 = no null for the group) and the majority orientation the null was built from. */
    int32_t                predict_pair_distance;
    const int64_t* const*  pd_cdf;
    const uint32_t*        pd_cdf_len;
    const uint8_t*         pd_orientation;      /* BSQ_XP_FR, BSQ_XP_RF, or BSQ_XP_NONE for "" (any) */
    int32_t                pd_max_span;         /* _pd_max_span as the constructor derives it */
    double                 pd_z_seed;           /* _pd_z_seed as the constructor derives it */
    int32_t                pair_distance_seed;  /* --pair-distance-seed */
    double                 pair_distance_tail_quantile;
    double                 pd_mean_covering_gap;     /* the largest group's covering gap (header line) */
    uint64_t               total_reference_length;   /* for n_effective_tests */
} bsq_pair_params;

/* One PD candidate region (identify_mutations.cpp:2713-2730) and the calibration lines of
 * pd_candidate_regions.csv (:2852-2862). */
typedef struct bsq_pd_region {
    uint32_t target;
    uint32_t start;
    uint32_t end;
    char     direction;         /* 'L' (pairs farther apart) or 'S' */
    char     reserved[3];
    uint32_t peak_position;
    int32_t  peak_covering;
    int32_t  peak_tail;
    uint32_t reserved2;
    double   peak_z;
} bsq_pd_region;

typedef struct bsq_pd_summary {
    double   mean_covering_gap;
    double   n_effective_tests;
    double   seed_z_used;
    double   z_iqr_inflation;
    int32_t  region_tail_fit_ok;
    int32_t  reserved;
    double   region_tail_log_intercept;
    double   region_tail_sigma;
    double   region_tail_fit_lo;
    double   region_tail_fit_hi;
    uint64_t ladder[21];        /* seeded regions at |z| >= 1 + 0.25 k, both directions */
    uint64_t regions_seeded;
} bsq_pd_summary;

/* One candidate region.  Text fields are in the result's text buffer at [text_off, text_off +
 * text_len): DP "<read1>__<read2>__<r1_insert_size>__<read_start>__<read_end>" per read, MP
 * "<read_start>__<read_end>", joined by ';'. */
typedef struct bsq_pair_region {
    uint32_t target;
    uint32_t start;
    uint32_t end;
    char     strand;            /* 'F' or 'R' */
    char     orientation[3];    /* DP: "FR", "RF" or "FF"; MP: "" */
    uint32_t max_count;         /* max_discordant_count / max_unpaired_count */
    uint32_t max_total;         /* MP: max_window_total_count; DP: 0 */
    uint32_t redundant;         /* a majority of the region's reads have X1 > 1 */
    uint32_t reserved;
    uint64_t text_off;
    uint64_t text_len;
} bsq_pair_region;

/* Runs the scans on a resident sample (needs the pair annotations of bsq_read_soa or a BAM load).
 * Regions come per target (pileup order): DP bins 0-5, then MP strands, each by position; the writers
 * sort them as breseq does. */
int bsq_pair_candidates(bsq_ctx* ctx, int32_t sample_id, const bsq_pair_params* params, uint64_t* n_dp,
                        uint64_t* n_mp, uint64_t* text_bytes);
int bsq_pair_result_copy(bsq_ctx* ctx, bsq_pair_region* dp, uint64_t n_dp, bsq_pair_region* mp, uint64_t n_mp,
                         char* text, uint64_t text_bytes);
/* The PD result of the last bsq_pair_candidates call: regions in the order the writer prints them
 * (after its rescan-budget cap, identify_mutations.cpp:2875-2904) and the calibration. */
int bsq_pd_result(bsq_ctx* ctx, uint64_t* n_regions, bsq_pd_region* regions, uint64_t capacity,
                  bsq_pd_summary* summary);
/* The PD setup of identify_mutations_pileup (identify_mutations.cpp:920-995), host code:
 *  - bsq_pd_build_null: one read-file set's null from the rows (distance, count) of its paired-mapping
 *    distance histogram file, as pd_load_weighted_histogram (pd_evidence.cpp:56-97) weights them and
 *    pd_build_cdf (identify_mutations.cpp:112-141) scales them; trunc = 2 x the rounded mean read
 *    length, max_distance = the span when above trunc, else 0.  cdf_len 0: no usable weight (the group
 *    has no null).  BSQ_ERR_SIZE with *cdf_len = the length needed when capacity is short.
 *  - bsq_pd_max_span: --pair-distance-maximum-span, or twice the largest distance cutoff;
 *  - bsq_pd_seed_z: --pair-distance-seed-z, or the analytic threshold over reference length /
 *    covering gap tests, clamped to [1, 2.5] (Cephes ndtri, stats.cpp:1747-1791). */
int     bsq_pd_build_null(const int32_t* distance, const double* count, uint64_t n_rows, int32_t trunc,
                          int32_t max_distance, int64_t* cdf, uint32_t capacity, uint32_t* cdf_len,
                          double* mean_covering_gap);
int32_t bsq_pd_max_span(int32_t pair_distance_maximum_span, const double* distance_cutoff, uint32_t n_groups);
double  bsq_pd_seed_z(double pair_distance_seed_z, double mean_covering_gap, uint64_t total_reference_length);
double  bsq_ndtri(double y);
/* pd_candidate_regions.csv (identify_mutations.cpp:2864-2967) */
int bsq_write_pd_candidate_regions(const char* path, const char* const* target_names, const bsq_pd_region* regions,
                                   uint64_t n, const bsq_pd_summary* summary);
/* dp_candidate_regions.csv / mp_candidate_regions.csv (identify_mutations.cpp:2524-2586) */
int bsq_write_dp_candidate_regions(const char* path, const char* const* target_names, const bsq_pair_region* regions,
                                   uint64_t n, const char* text);
int bsq_write_mp_candidate_regions(const char* path, const char* const* target_names, const bsq_pair_region* regions,
                                   uint64_t n, const char* text);

/* ---------------------------------------------------------------- scoring without allocation */

/* Raw values of one RA item as the scoring kernel writes them (device memory).  `column` is the
 * target's padded column: target_offset[tid] + tid + (position - 1).  Base indices are 0..4 =
 * A,C,G,T,'.', 5 = N; pos_info is [base][top, bottom] strand coverage of the scored read bases. */
typedef struct bsq_ra_raw {
    uint32_t column;
    uint32_t insert_position;
    double   score, consensus_score;
    double   f[5];
    double   frequency_lower, frequency_upper;
    uint32_t pos_info[5][2];
    uint32_t n;
    uint8_t  ref_idx, var_idx, major_idx, minor_idx, passed_consensus, passed_polymorphism, pad[2];
} bsq_ra_raw;

/* Score the given reference positions (all of their insert slots) of a resident sample and write the
 * RA items that pass into caller-owned device memory, allocating nothing.  It has no counterpart in
 * the reference, which scores every position of every target in one pileup.  It is for callers that
 * cannot call cudaMalloc while they run: a serving loop with jobs in flight on other streams, where
 * cudaMalloc/cudaFree may synchronize the device and stall them, or a program that has handed all
 * of HBM to its own arena.  The scoring is bsq_identify_mutations' candidate scoring (FP64 sums, EM,
 * bounds), with one difference: the likelihood-class table is computed on the device with CUDA's pow
 * and log10 (within 2 ulp) rather than on the host with the C library's, so scores and frequencies
 * agree with bsq_identify_mutations' to about 1e-12, not bit for bit.  The call reads the deletion
 * propagation cutoffs from `p` and changes nothing in the sample.
 *
 * d_tid / d_pos0 (0-based positions) are device arrays of n_positions entries.  d_ra (ra_capacity
 * records), d_n_ra (one counter, set by the call) and d_qhist (ra_capacity x 2 x n_quality counters:
 * the qualities of the major- and minor-allele read bases of each record) are device memory the
 * caller owns.  Records appear in completion order, not position order.  Targets whose deletion
 * propagation cutoff is negative are skipped, as bsq_identify_mutations skips them.
 *
 * Scratch: one fixed 20 MiB device array in the library, held by every GPU that loads it until the
 * process exits.  Limits: n_read_files x 25 x n_quality <= 32768, (distinct MAPQ values) x
 * n_read_files x 2 x n_quality x 5 <= 32768 likelihood classes, at most 32768 targets; larger inputs
 * are rejected with BSQ_ERR_SIZE.  The first call on a device fetches the array's device address (cudaGetSymbolAddress),
 * so make that first call before any stream capture.  All calls share the array and each clears its
 * counters on entry: calls that overlap on the GPU (other threads, other contexts on the same device)
 * race on it and must be serialized by the caller.  Returns BSQ_ERR_SIZE, with *d_n_ra holding the
 * number of passing items, when more than ra_capacity pass. */
int bsq_score_positions_noalloc(bsq_ctx* ctx, int32_t sample_id, const bsq_im_params* p,
                                const double* log10_prob_table, const uint32_t* d_tid, const uint32_t* d_pos0,
                                uint32_t n_positions, bsq_ra_raw* d_ra, uint32_t ra_capacity, uint32_t* d_n_ra,
                                uint32_t* d_qhist);

/* Device-timeline timer on the context's stream: CUDA events recorded where the passes launch
 * their kernels, so the interval covers exactly the work issued in between (and any idle gaps). */
int bsq_timer_start(bsq_ctx* ctx);
int bsq_timer_stop(bsq_ctx* ctx, double* elapsed_ms);

/* Page-lock caller memory (cudaHostRegister) so sample uploads run at full host-to-device speed. */
int bsq_host_register(void* ptr, uint64_t bytes);
int bsq_host_unregister(void* ptr);

/* ---------------------------------------------------------------- serving
 *
 * A scoring server over one context: jobs (one sample's reads + reference, both passes) are
 * submitted from any thread and admitted while the sum of the footprints of admitted jobs stays
 * within an HBM budget.  Admission threads upload admitted jobs (several at once, on the context's
 * load streams) while the GPU thread runs the jobs already resident; every round the GPU thread takes all
 * resident jobs (up to max_batch_jobs; with fewer than four ready while uploads are in progress it
 * first waits up to 2 ms for more) and runs pass 1, the log10 table of each job
 * (bsq_counts_to_log10_prob) and pass 2 as one batch call per pass.  Jobs that arrive while a round
 * runs join the next round (continuous batching).  A job's results are the same as those of the
 * single-sample calls on the same inputs.  breseq itself has no server: this replaces its
 * per-sample sequence error_count -> error_rates.tab -> identify_mutations
 * (src/breseq/breseq_cmdline.cpp:2293-2318, :2471) for a caller that scores many samples. */

#define BSQ_ERR_TIMEOUT     -7   /* bsq_server_wait: the job did not finish within the timeout  */

#define BSQ_JOB_QUEUED   0       /* waiting for HBM budget                                     */
#define BSQ_JOB_LOADING  1       /* admitted, upload in progress                               */
#define BSQ_JOB_READY    2       /* resident, waiting for the next GPU round                   */
#define BSQ_JOB_RUNNING  3       /* in the GPU round now                                       */
#define BSQ_JOB_DONE     4       /* results available; negative = error code                   */

typedef struct bsq_server bsq_server;

typedef struct bsq_job {
    const bsq_reference* ref;    /* borrowed until the job is done                               */
    const bsq_read_soa* reads;   /* borrowed until the job is done                               */
    bsq_ec_params ec;
    bsq_im_params im;            /* deletion cutoff arrays borrowed until done; precision is the server's */
    uint32_t hist_capacity;      /* coverage-histogram bins kept per coverage group               */
} bsq_job;

typedef struct bsq_job_info {
    int32_t  state;              /* BSQ_JOB_*, or a negative error code                         */
    uint32_t round_jobs;         /* jobs in the GPU round this job ran in                        */
    uint64_t footprint;          /* bytes charged against the HBM budget                        */
    uint64_t n_ra, n_mc, n_un;
    uint64_t read_bases;         /* aligned read bases of the sample (one pass)                  */
    double   submit_ms, admit_ms, ready_ms, start_ms, done_ms;   /* since server creation    */
} bsq_job_info;

typedef struct bsq_server_stats {
    uint64_t jobs_done, rounds, budget, in_use, peak_in_use;
    uint32_t max_round_jobs, max_resident_jobs;
    double   gpu_busy_ms;        /* summed wall time of the GPU rounds                           */
    double   phase_ms[5];        /* of which: pass 1, table conversion, pass 2, result copies, frees */
} bsq_server_stats;

/* Bytes one job holds on the device while admitted: the resident sample plus both passes'
 * per-column working set. */
uint64_t bsq_job_footprint(const bsq_reference* ref, const bsq_read_soa* reads);

int  bsq_server_create(bsq_server** out, int device, uint64_t hbm_budget_bytes, uint32_t max_batch_jobs,
                       int32_t precision);
/* Waits for every submitted job, then stops the threads. */
void bsq_server_destroy(bsq_server* srv);
const char* bsq_server_last_error(const bsq_server* srv);
/* BSQ_ERR_NOMEM when the job alone exceeds the budget. */
int  bsq_server_submit(bsq_server* srv, const bsq_job* job, uint64_t* job_id);
/* Blocks until the job is done or failed (BSQ_OK, info filled) or timeout_ms passes
 * (BSQ_ERR_TIMEOUT; timeout_ms < 0 waits without limit). */
int  bsq_server_wait(bsq_server* srv, uint64_t job_id, int64_t timeout_ms, bsq_job_info* info);
int  bsq_server_job_info(bsq_server* srv, uint64_t job_id, bsq_job_info* info);
const char* bsq_server_job_error(bsq_server* srv, uint64_t job_id);
/* Pass-1 results of a done job: counts [R*25*Q], coverage_hist [groups * hist_capacity], hist_size
 * [groups]; any may be NULL. */
int  bsq_server_error_counts(bsq_server* srv, uint64_t job_id, uint64_t* counts, uint64_t* coverage_hist,
                             uint32_t* hist_size);
/* Pass-2 records of a done job (sizes in bsq_job_info). */
int  bsq_server_results(bsq_server* srv, uint64_t job_id, bsq_ra_record* ra, uint64_t ra_cap, bsq_mc_record* mc,
                        uint64_t mc_cap, bsq_un_record* un, uint64_t un_cap);
/* Forget a done job and its results. */
int  bsq_server_release(bsq_server* srv, uint64_t job_id);
int  bsq_server_get_stats(bsq_server* srv, bsq_server_stats* out);
/* Launch shapes for the server's passes (e.g. from bsq_autotune on representative samples); the GPU
 * thread applies them before its next round, always with use_graphs = 0 (a stream capture waits
 * behind concurrent uploads).  Results do not depend on them. */
int  bsq_server_set_tuning(bsq_server* srv, const bsq_tuning* t);

#ifdef __cplusplus
}
#endif
#endif /* BRESEQ_GB300_H */
