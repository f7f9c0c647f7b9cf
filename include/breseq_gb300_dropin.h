/* C++ drop-in for breseq's two pileup entry points, with the reference's own signatures:
 *
 *   error_count()         src/breseq/error_count.h:44-56        (defined at error_count.cpp:50-68)
 *   identify_mutations()  src/breseq/identify_mutations.h:46-60 (defined at identify_mutations.cpp:48-88)
 *
 * They read reference.bam and reference.fasta from disk like the reference does, but decode the BAM
 * on the GPU (bsq_bam_*), keep the sample resident in HBM between the two calls, run both passes
 * through the C ABI of breseq_gb300.h, and write the reference's files:
 *
 *   error_count:         settings.error_rates_file_name, <outputdir>/base_qual_error_prob.<file>.tab,
 *                        <outputdir>/<group>.unique_only_coverage_distribution.tab (error_count.cpp:239-273)
 *   identify_mutations:  gd_file (the stage-08 ra_mc_evidence.gd: RA / MC / UN items before
 *                        test_RA_evidence), settings.dp_candidate_regions_file_name, and with
 *                        predict_copy_number the <seq_id>.coverage.tsv tables (identify_mutations.cpp:855)
 *
 * Errors follow the reference's convention (common.h:111-193): a message on stderr and exit(1).
 *
 * Types.  Built on its own (this repository's tests), the header declares minimal stand-ins for the
 * breseq types the two calls read -- Settings, Summary, cReadFileSet(s), cReferenceSequences -- with
 * breseq's member names and defaults.  Linked into breseq, define BSQ_DROPIN_WITH_BRESEQ before
 * including it: the stand-ins are then left out and breseq's own settings.h / summary.h /
 * reference_sequence.h provide the same members, so the implementation compiles unchanged against
 * them.  Not supported here: covariate strings other than the pipeline's
 * "read_set=R,obs_base,ref_base,quality=Q" (breseq_cmdline.cpp:2304), the per-position debug file
 * (print_per_position_file), user RA evidence, and the MP / PD / SC candidate files.
 */
#ifndef BRESEQ_GB300_DROPIN_H
#define BRESEQ_GB300_DROPIN_H

#include <stdint.h>

#include <map>
#include <set>
#include <string>
#include <vector>

#ifdef BSQ_DROPIN_WITH_BRESEQ
#include "libbreseq/reference_sequence.h"
#include "libbreseq/settings.h"
#include "libbreseq/summary.h"
#else
namespace breseq {

/* settings.h:92-129 */
struct cReadFile {
  std::string m_original_file_name;
  std::string m_base_name;
  uint32_t m_id = 0xFFFFFFFFu;
  std::string base_name() const { return m_base_name; }
};
struct cReadFileSet {
  std::vector<cReadFile> m_files;   // 1 file (unpaired) or 2 (paired, R1 first)
  std::string m_base_name;          // the @RG LB of its read group
  bool is_paired() const { return m_files.size() == 2; }
};
struct cReadFileSets : public std::vector<cReadFileSet> {};

/* The Settings members the two passes read (settings.h), with breseq's defaults (settings.cpp). */
struct Settings {
  cReadFileSets read_file_sets;
  // cReferenceSequenceSettings (settings.h:170-197)
  std::set<std::string> m_call_mutations_seq_id_set;
  std::vector<std::vector<std::string> > m_seq_ids_by_coverage_group;
  std::set<std::string> call_mutations_seq_id_set() const { return m_call_mutations_seq_id_set; }
  std::vector<std::vector<std::string> > seq_ids_by_coverage_group() const { return m_seq_ids_by_coverage_group; }
  // file names (settings.cpp:1555-1571)
  std::string error_rates_file_name = "07_error_calibration/error_rates.tab";
  std::string unique_only_coverage_distribution_file_name = "07_error_calibration/@.unique_only_coverage_distribution.tab";
  std::string error_rates_base_qual_error_prob_file_name = "07_error_calibration/base_qual_error_prob.#.tab";
  std::string complete_coverage_text_file_name = "08_mutation_identification/@.coverage.tsv";
  std::string dp_candidate_regions_file_name = "08_mutation_identification/DP_candidate_regions.csv";
  // scoring (settings.cpp:1335)
  uint32_t base_quality_cutoff = 3;
  bool skip_missing_coverage_prediction = false;
  bool predict_copy_number = false;
  // preprocess stage: required_junction_read_end_min_coordinate (settings.h:345-354, settings.cpp:1308-1309)
  uint32_t unmatched_end_minimum_read_length = 50;
  double unmatched_end_length_factor = 0.1;

  static std::string file_name(const std::string& key, const std::string& sub, const std::string& with);
  static std::string path_file_name(const std::string& path, const std::string& key, const std::string& sub = "",
                                    const std::string& with = "");
};

/* The Summary members the two passes read and write (summary.h). */
struct PairedMappingDistanceDistributionSummary {
  double median = 0.0, mad = 0.0;
  std::string majority_orientation;
};
struct ErrorCountSummary {
  double no_pos_hash_per_position_pr = 0.0;
};
struct Summary {
  struct { uint32_t max_qual = 0; } sequence_conversion;
  std::map<std::string, ErrorCountSummary> preprocess_error_count;
  std::map<std::string, PairedMappingDistanceDistributionSummary> preliminary_paired_mapping_distance_distribution;
};

/* identify_mutations() takes the loaded reference sequences for the soft-clip evidence, which this
 * drop-in does not write; the sequences come from the FASTA file. */
struct cReferenceSequences {};

}  // namespace breseq
#endif

namespace breseq {

void error_count(const Settings& settings, Summary& summary, const std::string& bam, const std::string& fasta,
                 const std::string& outputdir, const std::vector<std::string>& readfiles, bool do_coverage,
                 bool do_errors, bool preprocess_stage, uint8_t min_qual_score, const std::string& covariates);

void identify_mutations(const Settings& settings, const Summary& summary, const std::string& bam,
                        const std::string& fasta, const std::string& gd_file, const cReferenceSequences& ref_seq_info,
                        const std::vector<double>& deletion_propagation_cutoff,
                        const std::vector<double>& deletion_seed_cutoff, double mutation_cutoff,
                        double polymorphism_cutoff, double polymorphism_precision_decimal,
                        uint32_t polymorphism_precision_places, bool print_per_position_file);

}  // namespace breseq

/* GPU device the drop-in uses (default 0; also read from the BSQ_DEVICE environment variable), and
 * release of the resident samples and the device context (the process may also simply exit). */
extern "C" void bsq_dropin_set_device(int device);
extern "C" void bsq_dropin_release(void);

#endif
