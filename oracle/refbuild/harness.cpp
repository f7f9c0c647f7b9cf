// Driver of breseq's own error_count() and identify_mutations() (src/breseq/error_count.cpp:50-68,
// src/breseq/identify_mutations.cpp:48-88), compiled from the reference's unmodified sources against
// the clean-room htslib subset in this folder.  Test infrastructure: it produces the reference's own
// output files for a synthetic BAM so the oracle and the CUDA path can be compared with them.
//
//   ref_harness <config file>
//
// The config file holds one `key value...` per line:
//   bam, fasta, outdir        paths (outdir must exist)
//   groups g0 g1 ...          read-file count of each read group rg0, rg1, ... (1 = single-end, 2 = paired)
//   target name coverage_group called prop_cutoff seed_cutoff   one line per target
//   quality Q                 error-table quality bins (summary max_qual + 1)
//   polymorphism 0|1          polymorphism mode (settings.cpp:857-948 defaults)
//   copy_number 0|1           --predict-copy-number: write <seq_id>.coverage.tsv
//   classify 0|1              also run test_RA_evidence and write ra_mc_evidence.classified.gd
//   pmdd g median mad         paired-mapping-distance fit of read group g: makes it a discordant-pair
//                             group (identify_mutations.cpp:883-911; window median + 2.42 mad)
//   softclip 0|1              also tabulate_soft_clipping_counts (soft_clipping.cpp:288): writes
//                             soft_clipping_counts.tab and soft_clipping_summary.txt (the Summary fields)
//   bam2cov name region resolution format total_only per_read_group
//                             also `breseq BAM2COV` tables (coverage_output::table, breseq_cmdline.cpp:428-536)
//                             into bam2cov/<name>
//   covfit 0|1                also fit each coverage group's unique-only coverage distribution
//                             (fit_coverage_distribution, coverage_distribution.cpp:345-399, with the
//                             cutoff analyze_unique_coverage_distribution passes, :545): writes
//                             coverage_fit.<group>.txt (the fit result, %.17g)
// Outputs in outdir: error_rates.tab, base_qual_error_prob.<file>.tab, <group>.unique_only_coverage_distribution.tab,
// ra_mc_evidence.gd, 08_mutation_identification/ (DP candidate regions, coverage tables) and the
// classified GenomeDiff when asked.
#include <fstream>
#include <iostream>
#include <sstream>

#include "common.h"
#include "error_count.h"
#include "genome_diff.h"
#include "identify_mutations.h"
#include "coverage_distribution.h"
#include "coverage_output.h"
#include "reference_sequence.h"
#include "settings.h"
#include "soft_clipping.h"
#include "summary.h"

using namespace breseq;

namespace breseq {
// covfit.cpp: coverage_distribution.cpp:345's fit itself, without the plot CoverageDistribution::fit draws
CoverageDistributionFitResult harness_fit_coverage(const coverage_histogram_t& hist, double deletion_propagation_pr_cutoff,
                                                   uint32_t& censor_start, uint32_t& censor_end, double& nb_fit_scale);
}

int main(int argc, char** argv) {
  if (argc != 2) { cerr << "usage: ref_harness <config>" << endl; return 2; }
  ifstream cf(argv[1]);
  string bam, fasta, outdir;
  vector<uint32_t> group_files;
  struct Tgt { string name; uint32_t group; int called; double prop, seed; };
  vector<Tgt> targets;
  uint32_t Q = 42;
  bool poly = false, copy_number = false, classify = false;
  struct Pmdd { uint32_t g; double median, mad; };
  vector<Pmdd> pmdd;
  bool softclip = false, covfit = false;
  struct Cov { string name, region, format; uint32_t resolution; int total_only, per_rg; };
  vector<Cov> covs;
  string line;
  while (getline(cf, line)) {
    istringstream ls(line);
    string key;
    if (!(ls >> key)) continue;
    if (key == "bam") ls >> bam;
    else if (key == "fasta") ls >> fasta;
    else if (key == "outdir") ls >> outdir;
    else if (key == "groups") { uint32_t g; while (ls >> g) group_files.push_back(g); }
    else if (key == "quality") ls >> Q;
    else if (key == "polymorphism") { int v; ls >> v; poly = v != 0; }
    else if (key == "copy_number") { int v; ls >> v; copy_number = v != 0; }
    else if (key == "classify") { int v; ls >> v; classify = v != 0; }
    else if (key == "pmdd") { Pmdd d; ls >> d.g >> d.median >> d.mad; pmdd.push_back(d); }
    else if (key == "softclip") { int v; ls >> v; softclip = v != 0; }
    else if (key == "covfit") { int v; ls >> v; covfit = v != 0; }
    else if (key == "bam2cov") {
      Cov c;
      ls >> c.name >> c.region >> c.resolution >> c.format >> c.total_only >> c.per_rg;
      covs.push_back(c);
    }
    else if (key == "target") { Tgt t; ls >> t.name >> t.group >> t.called >> t.prop >> t.seed; targets.push_back(t); }
  }
  Settings::set_global_paths();      // data path from BRESEQ_DATA_PATH
  Settings settings(outdir);
  create_path(settings.mutation_identification_path);   // DP / MP / PD candidate files go there
  // read-file sets: one per read group, named by the @RG LB of the BAM (rg<g>); a paired set has
  // R1 and R2 files whose flat indices follow the sets' order (alignment.h:576-607)
  settings.read_file_sets.clear();
  vector<string> readfiles;
  uint32_t flat = 0;
  for (size_t g = 0; g < group_files.size(); g++) {
    cReadFileSet rfs;
    rfs.m_base_name = "rg" + to_string(g);
    for (uint32_t f = 0; f < group_files[g]; f++) {
      cReadFile rf;
      rf.m_original_file_name = rfs.m_base_name + "_" + to_string(f + 1);
      rf.m_base_name = rf.m_original_file_name;
      rf.m_id = flat;
      rf.m_paired_end_group = (uint32_t)g;
      rf.m_error_group = flat;
      rfs.m_files.push_back(rf);
      readfiles.push_back(rf.m_base_name);
      flat++;
    }
    settings.read_file_sets.push_back(rfs);
  }
  // targets: the pileup set and the coverage groups
  uint32_t n_groups = 0;
  for (const Tgt& t : targets) n_groups = max(n_groups, t.group + 1);
  settings.refseq_settings.m_seq_ids_by_coverage_group.assign(n_groups, vector<string>());
  for (const Tgt& t : targets) {
    if (t.called) settings.refseq_settings.m_call_mutations_seq_id_set.insert(t.name);
    settings.refseq_settings.m_seq_ids_by_coverage_group[t.group].push_back(t.name);
    settings.refseq_settings.m_seq_id_to_coverage_group_map[t.name] = t.group;
  }
  // the command line's mode-dependent defaults of the RA settings (settings.cpp:857-948)
  settings.polymorphism_prediction = poly;
  settings.minimum_mapping_quality = 0;
  settings.mutation_log10_e_value_cutoff = 10;
  settings.consensus_frequency_cutoff = poly ? 0.95 : 0.50;
  settings.consensus_minimum_variant_coverage = 0;
  settings.consensus_minimum_total_coverage = 0;
  settings.consensus_minimum_variant_coverage_each_strand = 0;
  settings.consensus_minimum_total_coverage_each_strand = 0;
  settings.consensus_reject_indel_homopolymer_length = 0;
  settings.consensus_reject_surrounding_homopolymer_length = 0;
  settings.polymorphism_log10_e_value_cutoff = poly ? 2 : 10;
  settings.polymorphism_frequency_cutoff = poly ? 0.05 : 0.10;
  settings.polymorphism_minimum_variant_coverage = 0;
  settings.polymorphism_minimum_total_coverage = 0;
  settings.polymorphism_minimum_variant_coverage_each_strand = 2;
  settings.polymorphism_minimum_total_coverage_each_strand = 0;
  settings.mixed_base_prediction = !poly;
  settings.polymorphism_reject_indel_homopolymer_length = 0;
  settings.polymorphism_reject_surrounding_homopolymer_length = 0;
  settings.polymorphism_fisher_strand_p_value_cutoff = 0.05;
  settings.polymorphism_ks_quality_p_value_cutoff = 0;
  settings.polymorphism_no_indels = false;
  settings.polymorphism_precision_decimal = 1e-6;
  settings.polymorphism_precision_places = poly ? 8 : 3;
  settings.predict_copy_number = copy_number;
  settings.error_rates_file_name = Settings::path_file_name(outdir, "error_rates.tab");
  // the pipeline's covariates (breseq_cmdline.cpp:2304)
  const string covariates = "read_set=" + to_string(flat) + ",obs_base,ref_base,quality=" + to_string(Q);
  Summary summary;
  summary.sequence_conversion.max_qual = Q - 1;
  for (const Pmdd& d : pmdd) {
    PairedMappingDistanceDistributionSummary& f = summary.preliminary_paired_mapping_distance_distribution["rg" + to_string(d.g)];
    f.median = d.median;
    f.mad = d.mad;
  }
  error_count(settings, summary, bam, fasta, outdir, readfiles, true, true, false, 0, covariates);

  vector<double> prop, seed;
  for (const Tgt& t : targets) { prop.push_back(t.prop); seed.push_back(t.seed); }
  cReferenceSequences ref_seq_info;
  ref_seq_info.LoadFiles(make_vector<string>(fasta));
  const string gd_file = Settings::path_file_name(outdir, "ra_mc_evidence.gd");
  identify_mutations(settings, summary, bam, fasta, gd_file, ref_seq_info, prop, seed, settings.mutation_log10_e_value_cutoff,
                     settings.polymorphism_log10_e_value_cutoff, settings.polymorphism_precision_decimal,
                     settings.polymorphism_precision_places, false);
  if (softclip) {
    settings.soft_clipping_counts_file_name = Settings::path_file_name(outdir, "soft_clipping_counts.tab");
    tabulate_soft_clipping_counts(settings, summary, make_vector<string>(bam), fasta, ref_seq_info);
    const SoftClippingSummary& c = summary.soft_clipping;
    FILE* f = fopen(Settings::path_file_name(outdir, "soft_clipping_summary.txt").c_str(), "w");
    fprintf(f, "total_spanning_read_bases %llu\ntotal_clipped_read_ends %llu\ntotal_agreeing_clipped_read_ends %llu\n",
            (unsigned long long)c.total_spanning_read_bases, (unsigned long long)c.total_clipped_read_ends,
            (unsigned long long)c.total_agreeing_clipped_read_ends);
    fprintf(f, "soft_clipping_rate %.17g\nsoft_clipping_null_rate %.17g\nsoft_clipping_dispersion %.17g\n",
            c.soft_clipping_rate, c.soft_clipping_null_rate, c.soft_clipping_dispersion);
    fprintf(f, "soft_clipping_pearson_phi %.17g\nsoft_clipping_tested_positions %llu\nsoft_clipping_trimmed_positions %llu\n",
            c.soft_clipping_pearson_phi, (unsigned long long)c.soft_clipping_tested_positions,
            (unsigned long long)c.soft_clipping_trimmed_positions);
    fprintf(f, "soft_clipping_mean_tested_reads %.17g\n", c.soft_clipping_mean_tested_reads);
    fclose(f);
  }
  if (covfit) {
    for (uint32_t g = 0; g < n_groups; g++) {
      uint32_t len = 0;
      for (const string& id : settings.refseq_settings.m_seq_ids_by_coverage_group[g])
        len += ref_seq_info.get_sequence_length(id);
      const coverage_histogram_t hist =
          read_coverage_histogram(Settings::path_file_name(outdir, to_string(g) + ".unique_only_coverage_distribution.tab"));
      uint32_t cs = 0, ce = 0;
      double scale = 0;
      const CoverageDistributionFitResult r = harness_fit_coverage(hist, 0.05 / sqrt(len), cs, ce, scale);
      FILE* f = fopen(Settings::path_file_name(outdir, "coverage_fit." + to_string(g) + ".txt").c_str(), "w");
      fprintf(f, "nbinom_size %.17g\nnbinom_mean %.17g\naverage %.17g\nvariance %.17g\nrelative_variance %.17g\n",
              r.nb_fit_size, r.nb_fit_mu, r.average, r.variance, r.relative_variance);
      fprintf(f, "deletion_coverage_propagation_cutoff %.17g\ncensor_start %u\ncensor_end %u\nnbinom_scale %.17g\n",
              r.deletion_coverage_propagation_cutoff, cs, ce, scale);
      fclose(f);
    }
  }
  if (!covs.empty()) create_path(outdir + "/bam2cov");
  for (const Cov& c : covs) {
    coverage_output co(bam, fasta);
    co.total_only(c.total_only != 0);
    co.per_read_group(c.per_rg != 0);
    co.output_format(c.format);
    co.table(c.region, outdir + "/bam2cov/" + c.name, c.resolution);
  }
  if (classify) {
    cGenomeDiff gd(gd_file);
    test_RA_evidence(gd, ref_seq_info, settings);
    gd.write(Settings::path_file_name(outdir, "ra_mc_evidence.classified.gd"));
  }
  return 0;
}
