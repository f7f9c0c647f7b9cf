// Drives the drop-in error_count() / identify_mutations() (include/breseq_gb300_dropin.h) from the same
// config file the reference oracle's harness reads (oracle/refbuild/harness.cpp), so the two write
// the same files into their output folders:
//   dropin_main <config>
// Outputs in outdir: error_rates.tab, base_qual_error_prob.<file>.tab,
// <group>.unique_only_coverage_distribution.tab, ra_mc_evidence.gd, 08_mutation_identification/...
#include <sys/stat.h>

#include <algorithm>
#include <fstream>
#include <iostream>
#include <sstream>

#include "../../include/breseq_gb300_dropin.h"

using namespace breseq;

int main(int argc, char** argv) {
  if (argc != 2) { std::cerr << "usage: dropin_main <config>" << std::endl; return 2; }
  std::ifstream cf(argv[1]);
  std::string bam, fasta, outdir, line;
  std::vector<uint32_t> group_files;
  struct Tgt { std::string name; uint32_t group; int called; double prop, seed; };
  std::vector<Tgt> targets;
  struct Pmdd { uint32_t g; double median, mad; };
  std::vector<Pmdd> pmdd;
  uint32_t Q = 42;
  bool poly = false, copy_number = false;
  while (std::getline(cf, line)) {
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key)) continue;
    if (key == "bam") ls >> bam;
    else if (key == "fasta") ls >> fasta;
    else if (key == "outdir") ls >> outdir;
    else if (key == "groups") { uint32_t g; while (ls >> g) group_files.push_back(g); }
    else if (key == "quality") ls >> Q;
    else if (key == "polymorphism") { int v; ls >> v; poly = v != 0; }
    else if (key == "copy_number") { int v; ls >> v; copy_number = v != 0; }
    else if (key == "pmdd") { Pmdd d; ls >> d.g >> d.median >> d.mad; pmdd.push_back(d); }
    else if (key == "target") { Tgt t; ls >> t.name >> t.group >> t.called >> t.prop >> t.seed; targets.push_back(t); }
  }
  Settings settings;
  settings.error_rates_file_name = Settings::path_file_name(outdir, "error_rates.tab");
  const std::string mi = outdir + "/08_mutation_identification";
  mkdir(mi.c_str(), 0755);
  settings.complete_coverage_text_file_name = mi + "/@.coverage.tsv";
  settings.dp_candidate_regions_file_name = mi + "/DP_candidate_regions.csv";
  settings.predict_copy_number = copy_number;
  std::vector<std::string> readfiles;
  uint32_t flat = 0;
  for (size_t g = 0; g < group_files.size(); g++) {
    cReadFileSet rfs;
    rfs.m_base_name = "rg" + std::to_string(g);
    for (uint32_t f = 0; f < group_files[g]; f++) {
      cReadFile rf;
      rf.m_base_name = rf.m_original_file_name = rfs.m_base_name + "_" + std::to_string(f + 1);
      rf.m_id = flat++;
      rfs.m_files.push_back(rf);
      readfiles.push_back(rf.m_base_name);
    }
    settings.read_file_sets.push_back(rfs);
  }
  uint32_t n_groups = 0;
  for (const Tgt& t : targets) n_groups = std::max(n_groups, t.group + 1);
  settings.m_seq_ids_by_coverage_group.assign(n_groups, std::vector<std::string>());
  std::vector<double> prop, seed;
  for (const Tgt& t : targets) {
    if (t.called) settings.m_call_mutations_seq_id_set.insert(t.name);
    settings.m_seq_ids_by_coverage_group[t.group].push_back(t.name);
    prop.push_back(t.prop);
    seed.push_back(t.seed);
  }
  Summary summary;
  summary.sequence_conversion.max_qual = Q - 1;
  for (const Pmdd& d : pmdd) {
    auto& f = summary.preliminary_paired_mapping_distance_distribution["rg" + std::to_string(d.g)];
    f.median = d.median;
    f.mad = d.mad;
  }
  const std::string covariates = "read_set=" + std::to_string(flat) + ",obs_base,ref_base,quality=" + std::to_string(Q);
  error_count(settings, summary, bam, fasta, outdir, readfiles, true, true, false, 0, covariates);
  cReferenceSequences ref_seq_info;
  identify_mutations(settings, summary, bam, fasta, Settings::path_file_name(outdir, "ra_mc_evidence.gd"), ref_seq_info,
                     prop, seed, 10.0, poly ? 2.0 : 10.0, 1e-6, poly ? 8 : 3, false);
  bsq_dropin_release();
  return 0;
}
