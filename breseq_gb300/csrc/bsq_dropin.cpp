// breseq's error_count() / identify_mutations() with their reference signatures
// (include/breseq_gb300_dropin.h), over the C ABI of include/breseq_gb300.h.
//
// The reference opens reference.bam through htslib in each call (pileup_base.cpp:61-88) and pipes the
// error table from one call to the next through error_rates.tab (error_count.cpp:660-690 writes it,
// identify_mutations.cpp:866-868 reads it back).  Here the BAM is read from disk once, inflated and
// decoded on the GPU, and kept resident as a sample keyed by its path, size and modification time;
// identify_mutations() reads error_rates.tab back from the path in Settings, as the reference does, so
// a table the caller edits in between is honoured.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "../../include/breseq_gb300_dropin.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
  // the reference's ERROR(): a message on stderr and exit(1) (common.h:111-193)
  fprintf(stderr, "!!!!> FATAL ERROR <!!!!\n%s\n", msg.c_str());
  exit(1);
}

int g_device = -1;
bsq_ctx* g_ctx = nullptr;
std::mutex g_mu;

bsq_ctx* ctx() {
  if (g_ctx) return g_ctx;
  if (g_device < 0) {
    const char* e = getenv("BSQ_DEVICE");
    g_device = e ? atoi(e) : 0;
  }
  if (bsq_create(&g_ctx, g_device) != BSQ_OK)
    die("no CUDA device for the GB300 scoring path: " + std::string(bsq_last_error(nullptr)));
  return g_ctx;
}

void check(int rc, const std::string& what) {
  if (rc != BSQ_OK) die(what + ": " + bsq_last_error(g_ctx));
}

std::string substitute(std::string s, const std::string& from, const std::string& to) {
  if (from.empty()) return s;
  for (size_t p = s.find(from); p != std::string::npos; p = s.find(from, p + to.size())) s.replace(p, from.size(), to);
  return s;
}

// A resident sample: the reference as the library takes it and the device sample id.
struct Resident {
  std::string key;
  std::vector<std::string> names;            // targets in BAM header order
  std::vector<const char*> name_ptrs;
  std::vector<uint64_t> offset;
  std::string seq;
  std::vector<uint32_t> group, order;
  std::vector<std::string> rg_ids;           // @RG IDs in header order
  bsq_reference ref;
  int32_t sid = -1;
  uint32_t n_coverage_groups = 1;
};
std::map<std::string, std::unique_ptr<Resident>> g_samples;

std::map<std::string, std::string> read_fasta(const std::string& path) {
  std::ifstream in(path);
  if (!in) die("Could not open reference FASTA file: " + path);
  std::map<std::string, std::string> out;
  std::string line, name;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (!line.empty() && line[0] == '>') {
      name = line.substr(1);
      const size_t sp = name.find_first_of(" \t");
      if (sp != std::string::npos) name.resize(sp);
      out[name];
    } else if (!name.empty()) {
      out[name] += line;
    }
  }
  return out;
}

// The BAM read once: header targets and @RG lines, records decoded on the device with the read
// groups resolved as breseq does (@RG LB matched to the read-file sets, alignment.h:569-607), the
// reference from the FASTA in header order, coverage groups and the pileup set from Settings.
Resident& resident(const breseq::Settings& settings, const std::string& bam, const std::string& fasta) {
  struct stat st;
  if (stat(bam.c_str(), &st) != 0) die("Could not load bam file: " + bam);
  const std::string key = bam + "\n" + std::to_string((long long)st.st_size) + "\n" +
                          std::to_string((long long)st.st_mtime) + "\n" + fasta;
  auto it = g_samples.find(bam);
  if (it != g_samples.end()) {
    if (it->second->key == key) return *it->second;
    check(bsq_free_sample(ctx(), it->second->sid), "free sample");
    g_samples.erase(it);
  }
  std::vector<uint8_t> data((size_t)st.st_size);
  FILE* f = fopen(bam.c_str(), "rb");
  if (!f || fread(data.data(), 1, data.size(), f) != data.size()) die("Could not read bam file: " + bam);
  fclose(f);
  std::unique_ptr<Resident> R(new Resident());
  R->key = key;
  bsq_bam* b = nullptr;
  check(bsq_bam_open(ctx(), data.data(), data.size(), &b), "BAM " + bam);
  const char* text = nullptr;
  uint64_t text_len = 0;
  uint32_t n_ref = 0;
  const char* const* ref_names = nullptr;
  const uint32_t* ref_len = nullptr;
  check(bsq_bam_header(b, &text, &text_len, &n_ref, &ref_names, &ref_len), "BAM header");
  // read groups: @RG ID and LB, header order
  std::vector<std::string> lb;
  {
    std::istringstream hs(std::string(text, (size_t)text_len));
    std::string l;
    while (std::getline(hs, l)) {
      if (l.compare(0, 4, "@RG\t") != 0) continue;
      std::string id, lib, field;
      std::istringstream fs(l);
      while (std::getline(fs, field, '\t')) {
        if (field.compare(0, 3, "ID:") == 0) id = field.substr(3);
        if (field.compare(0, 3, "LB:") == 0) lib = field.substr(3);
      }
      R->rg_ids.push_back(id);
      lb.push_back(lib);
    }
  }
  // read_file_partition: a group's files are those of the set whose base name is its LB; groups
  // without a match take the sets in header order
  std::vector<uint32_t> set_base, set_count;
  uint32_t flat = 0;
  for (const auto& rfs : settings.read_file_sets) {
    set_base.push_back(flat);
    set_count.push_back((uint32_t)rfs.m_files.size());
    flat += (uint32_t)rfs.m_files.size();
  }
  std::vector<uint32_t> base(R->rg_ids.size(), 0), count(R->rg_ids.size(), 1);
  for (size_t g = 0; g < R->rg_ids.size(); g++) {
    size_t s = g;
    for (size_t k = 0; k < settings.read_file_sets.size(); k++)
      if (settings.read_file_sets[k].m_base_name == lb[g]) { s = k; break; }
    if (s < set_base.size()) { base[g] = set_base[s]; count[g] = set_count[s]; }
  }
  std::vector<const char*> ids;
  for (const auto& x : R->rg_ids) ids.push_back(x.c_str());
  bsq_bam_groups groups;
  groups.n_groups = (uint32_t)ids.size();
  groups.ids = ids.data();
  groups.file_base = settings.read_file_sets.empty() ? nullptr : base.data();
  groups.file_count = settings.read_file_sets.empty() ? nullptr : count.data();
  uint64_t n_rec = 0, n_cig = 0, n_bases = 0;
  check(bsq_bam_decode(ctx(), b, &groups, &n_rec, &n_cig, &n_bases), "BAM decode");
  // reference, in the header's target order
  const std::map<std::string, std::string> fa = read_fasta(fasta);
  std::map<std::string, uint32_t> cov_group;
  const auto by_group = settings.seq_ids_by_coverage_group();
  for (size_t g = 0; g < by_group.size(); g++)
    for (const auto& n : by_group[g]) cov_group[n] = (uint32_t)g;
  R->n_coverage_groups = std::max<uint32_t>(1, (uint32_t)by_group.size());
  R->offset.push_back(0);
  for (uint32_t t = 0; t < n_ref; t++) {
    R->names.push_back(ref_names[t]);
    auto s = fa.find(ref_names[t]);
    if (s == fa.end()) die(std::string("Reference sequence not found in FASTA: ") + ref_names[t]);
    if (s->second.size() != ref_len[t]) die(std::string("Reference length differs from the BAM header: ") + ref_names[t]);
    R->seq += s->second;
    R->offset.push_back(R->seq.size());
    auto g = cov_group.find(ref_names[t]);
    R->group.push_back(g == cov_group.end() ? 0 : g->second);
  }
  for (const auto& n : settings.call_mutations_seq_id_set()) {   // std::set: lexicographic, as the pileup walks it
    auto p = std::find(R->names.begin(), R->names.end(), n);
    if (p == R->names.end()) die("Could not find seq_id: " + n);
    R->order.push_back((uint32_t)(p - R->names.begin()));
  }
  for (const auto& n : R->names) R->name_ptrs.push_back(n.c_str());
  R->ref.n_targets = n_ref;
  R->ref.target_offset = R->offset.data();
  R->ref.seq = R->seq.data();
  R->ref.coverage_group = R->group.data();
  R->ref.n_coverage_groups = R->n_coverage_groups;
  R->ref.target_order = R->order.data();
  R->ref.n_target_order = (uint32_t)R->order.size();
  check(bsq_bam_load(ctx(), b, &R->ref, &R->sid), "load " + bam);
  bsq_bam_close(b);
  Resident& out = *R;
  g_samples[bam] = std::move(R);
  return out;
}

// The pipeline's covariates, read_set=R, obs_base, ref_base and quality=Q in any order
// (breseq_cmdline.cpp:2304 passes "read_set=R,obs_base,ref_base,quality=Q"; the error_rates.tab
// header lists them in the covariate enum's order, error_count.h:69)
void parse_covariates(const std::string& cov, uint32_t& R, uint32_t& Q) {
  unsigned r = 0, q = 0;
  int seen = 0;
  std::istringstream in(cov);
  std::string tok;
  while (std::getline(in, tok, ',')) {
    char tail;
    if (sscanf(tok.c_str(), "read_set=%u%c", &r, &tail) == 1) seen |= 1;
    else if (sscanf(tok.c_str(), "quality=%u%c", &q, &tail) == 1) seen |= 2;
    else if (tok == "obs_base") seen |= 4;
    else if (tok == "ref_base") seen |= 8;
    else seen |= 16;
  }
  if (seen != 15 || r == 0 || q == 0)
    die("Unsupported covariates (the scoring path takes read_set=R,obs_base,ref_base,quality=Q): " + cov);
  R = r;
  Q = q;
}

// read_log10_prob_table (error_count.cpp:629-654): covariate line, header line, then one row per
// table index whose last field is the log10 probability
std::vector<double> read_error_rates(const std::string& path, uint32_t& R, uint32_t& Q) {
  std::ifstream in(path);
  if (!in) die("Could not open error rate table: " + path);
  std::string cov, header, line;
  std::getline(in, cov);
  std::getline(in, header);
  parse_covariates(cov, R, Q);
  std::vector<double> v;
  while (std::getline(in, line)) {
    if (line.empty()) continue;
    const size_t tab = line.find_last_of('\t');
    v.push_back(strtod(line.c_str() + (tab == std::string::npos ? 0 : tab + 1), nullptr));
  }
  if (v.size() != (size_t)R * 25 * Q) die("Error rate table has the wrong number of rows: " + path);
  return v;
}

}  // namespace

namespace breseq {

#ifndef BSQ_DROPIN_WITH_BRESEQ
std::string Settings::file_name(const std::string& key, const std::string& sub, const std::string& with) {
  return substitute(key, sub, with);
}
std::string Settings::path_file_name(const std::string& path, const std::string& key, const std::string& sub,
                                     const std::string& with) {
  const size_t slash = key.find_last_of('/');
  const std::string s = substitute(slash == std::string::npos ? key : key.substr(slash + 1), sub, with);
  return path.empty() ? s : path + "/" + s;
}
#endif

void error_count(const Settings& settings, Summary& summary, const std::string& bam, const std::string& fasta,
                 const std::string& outputdir, const std::vector<std::string>& readfiles, bool do_coverage,
                 bool do_errors, bool preprocess_stage, uint8_t min_qual_score, const std::string& covariates) {
  (void)min_qual_score;   // unused by the reference's pileup as well
  std::lock_guard<std::mutex> lk(g_mu);
  uint32_t R = 0, Q = 0;
  parse_covariates(covariates, R, Q);
  Resident& S = resident(settings, bam, fasta);
  const uint32_t G = S.n_coverage_groups, T = S.ref.n_targets;
  bsq_ec_params p;
  p.n_read_files = R;
  p.n_quality = Q;
  p.do_coverage = do_coverage;
  p.do_errors = do_errors;
  p.preprocess_stage = preprocess_stage;
  p.unmatched_end_minimum_read_length = settings.unmatched_end_minimum_read_length;
  p.unmatched_end_length_factor = settings.unmatched_end_length_factor;
  std::vector<uint64_t> counts((size_t)R * 25 * Q);
  uint32_t cap = 1 << 16;
  std::vector<uint64_t> hist;
  std::vector<uint32_t> hist_size(G);
  std::vector<double> pr(T);
  for (;;) {   // a coverage beyond the histogram capacity: grow it and rerun
    hist.assign((size_t)G * cap, 0);
    bsq_ec_result out;
    out.counts = counts.data();
    out.coverage_hist = hist.data();
    out.hist_capacity = cap;
    out.hist_size = hist_size.data();
    out.no_pos_hash_pr = pr.data();
    const int rc = bsq_error_count(ctx(), S.sid, &p, &out);
    if (rc == BSQ_ERR_SIZE && cap < (1u << 26)) { cap <<= 2; continue; }
    check(rc, "error_count");
    break;
  }
  if (do_coverage)
    for (uint32_t g = 0; g < G; g++) {
      const std::string path = Settings::path_file_name(outputdir, settings.unique_only_coverage_distribution_file_name,
                                                        "@", std::to_string(g));
      check(bsq_write_coverage_distribution(path.c_str(), hist.data() + (size_t)g * cap, hist_size[g]), "write " + path);
    }
  if (do_errors) {
    check(bsq_write_error_rates(settings.error_rates_file_name.c_str(), counts.data(), R, Q),
          "write " + settings.error_rates_file_name);
    if (readfiles.size() < R) die("fewer read files than the read_set covariate");
    std::vector<const char*> names;
    for (const auto& n : readfiles) names.push_back(n.c_str());
    const std::string pattern = Settings::path_file_name(outputdir, settings.error_rates_base_qual_error_prob_file_name);
    check(bsq_write_base_qual_error_prob(pattern.c_str(), names.data(), counts.data(), R, Q), "write " + pattern);
  }
  if (preprocess_stage)
    for (uint32_t t = 0; t < T; t++) summary.preprocess_error_count[S.names[t]].no_pos_hash_per_position_pr = pr[t];
}

void identify_mutations(const Settings& settings, const Summary& summary, const std::string& bam,
                        const std::string& fasta, const std::string& gd_file, const cReferenceSequences& ref_seq_info,
                        const std::vector<double>& deletion_propagation_cutoff,
                        const std::vector<double>& deletion_seed_cutoff, double mutation_cutoff,
                        double polymorphism_cutoff, double polymorphism_precision_decimal,
                        uint32_t polymorphism_precision_places, bool print_per_position_file) {
  (void)ref_seq_info;
  (void)print_per_position_file;   // the per-position debug file is not written
  std::lock_guard<std::mutex> lk(g_mu);
  Resident& S = resident(settings, bam, fasta);
  const uint32_t T = S.ref.n_targets;
  if (deletion_propagation_cutoff.size() != T || deletion_seed_cutoff.size() != T)
    die("Number of targets in BAM file [" + std::to_string(T) + "] does not match + number in cutoff table [" +
        std::to_string(deletion_propagation_cutoff.size()) + "].");
  uint32_t R = 0, Q = 0;
  const std::vector<double> table = read_error_rates(settings.error_rates_file_name, R, Q);
  // discordant-pair groups as the pileup's constructor builds them (identify_mutations.cpp:883-911),
  // indexed by read-file set, which the pileup looks up by the record's read-group index
  std::vector<int32_t> dp_group(S.rg_ids.size(), -1);
  std::vector<double> width;
  std::vector<uint32_t> r1, r2;
  for (size_t i = 0; i < settings.read_file_sets.size() && i < dp_group.size(); i++) {
    const auto& rfs = settings.read_file_sets[i];
    if (!rfs.is_paired()) continue;
    auto f = summary.preliminary_paired_mapping_distance_distribution.find(rfs.m_base_name);
    if (f == summary.preliminary_paired_mapping_distance_distribution.end() || f->second.median <= 0.0) continue;
    dp_group[i] = (int32_t)width.size();
    width.push_back(f->second.median + 2.42 * f->second.mad);
    r1.push_back(rfs.m_files[0].m_id + 1);
    r2.push_back(rfs.m_files[1].m_id + 1);
  }
  bsq_im_params p;
  memset(&p, 0, sizeof p);
  p.n_read_files = R;
  p.n_quality = Q;
  p.base_quality_cutoff = settings.base_quality_cutoff;
  p.mutation_cutoff = mutation_cutoff;
  p.polymorphism_cutoff = polymorphism_cutoff;
  p.polymorphism_precision_decimal = polymorphism_precision_decimal;
  p.polymorphism_precision_places = polymorphism_precision_places;
  p.skip_missing_coverage_prediction = settings.skip_missing_coverage_prediction;
  double total = 0;
  for (uint32_t t = 0; t < T; t++) total += (double)(S.offset[t + 1] - S.offset[t]);
  p.log10_ref_length = log10(total);   // BAM target lengths (identify_mutations.cpp:848-852)
  p.deletion_propagation_cutoff = deletion_propagation_cutoff.data();
  p.deletion_seed_cutoff = deletion_seed_cutoff.data();
  p.precision = BSQ_PRECISION_FP32C;
  p.n_read_groups = (uint32_t)dp_group.size();
  p.dp_group = dp_group.data();
  // per-position arrays only for the coverage tables
  const uint64_t cols = S.offset[T];
  std::vector<uint32_t> ut, ub, rt, rb, ns;
  std::vector<double> dt, db, cs;
  std::vector<uint8_t> bb;
  bsq_position_arrays pa;
  memset(&pa, 0, sizeof pa);
  if (settings.predict_copy_number) {
    ut.resize(cols); ub.resize(cols); rt.resize(cols); rb.resize(cols); ns.resize(cols);
    dt.resize(cols); db.resize(cols); cs.resize(cols); bb.resize(cols);
    pa.unique_top = ut.data(); pa.unique_bot = ub.data(); pa.redundant_top = dt.data(); pa.redundant_bot = db.data();
    pa.raw_redundant_top = rt.data(); pa.raw_redundant_bot = rb.data(); pa.consensus_score = cs.data();
    pa.best_base = bb.data(); pa.n_scored = ns.data();
  }
  check(bsq_identify_mutations(ctx(), S.sid, &p, table.data(), settings.predict_copy_number ? &pa : nullptr),
        "identify_mutations");
  uint64_t nra = 0, nmc = 0, nun = 0;
  check(bsq_im_result_counts(ctx(), &nra, &nmc, &nun), "identify_mutations results");
  std::vector<bsq_ra_record> ra(std::max<uint64_t>(1, nra));
  std::vector<bsq_mc_record> mc(std::max<uint64_t>(1, nmc));
  std::vector<bsq_un_record> un(std::max<uint64_t>(1, nun));
  check(bsq_im_result_copy(ctx(), ra.data(), nra, mc.data(), nmc, un.data(), nun), "identify_mutations results");
  // coverage tables of the targets the pileup visits (with per-read-group columns when the BAM has
  // more than one read group, identify_mutations.cpp:862)
  if (settings.predict_copy_number)
    for (uint32_t t : S.order) {
      const std::string path = Settings::file_name(settings.complete_coverage_text_file_name, "@", S.names[t]);
      check(bsq_write_coverage_table_rg(ctx(), S.sid, path.c_str(), S.names[t].c_str(), &S.ref, t, &pa,
                                        (uint32_t)S.rg_ids.size(), deletion_propagation_cutoff[t] < 0.0, dp_group.data()),
            "write " + path);
    }
  // discordant-pair candidate regions, always written (identify_mutations.cpp:73)
  {
    bsq_pair_params pp;
    memset(&pp, 0, sizeof pp);
    pp.n_read_groups = (uint32_t)dp_group.size();
    pp.dp_group = dp_group.data();
    pp.n_dp_groups = (uint32_t)width.size();
    pp.window_width = width.data();
    pp.r1_name_prefix = r1.data();
    pp.r2_name_prefix = r2.data();
    pp.discordant_pair_seed = 3;
    pp.missing_pair_seed = 3;
    pp.missing_pair_seed_fraction = 0.25;
    pp.deletion_propagation_cutoff = deletion_propagation_cutoff.data();
    uint64_t nd = 0, nm = 0, nt = 0;
    check(bsq_pair_candidates(ctx(), S.sid, &pp, &nd, &nm, &nt), "discordant-pair scan");
    std::vector<bsq_pair_region> dp(std::max<uint64_t>(1, nd)), mp(std::max<uint64_t>(1, nm));
    std::vector<char> text(std::max<uint64_t>(1, nt));
    check(bsq_pair_result_copy(ctx(), dp.data(), nd, mp.data(), nm, text.data(), nt), "discordant-pair regions");
    check(bsq_write_dp_candidate_regions(settings.dp_candidate_regions_file_name.c_str(), S.name_ptrs.data(), dp.data(),
                                         nd, text.data()),
          "write " + settings.dp_candidate_regions_file_name);
  }
  check(bsq_write_gd(gd_file.c_str(), &S.ref, S.name_ptrs.data(), deletion_propagation_cutoff.data(),
                     polymorphism_precision_places, ra.data(), nra, nullptr, mc.data(), nmc, un.data(), nun),
        "write " + gd_file);
}

}  // namespace breseq

extern "C" void bsq_dropin_set_device(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_device = device;
}

extern "C" void bsq_dropin_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_samples)
    if (g_ctx) bsq_free_sample(g_ctx, kv.second->sid);
  g_samples.clear();
  if (g_ctx) bsq_destroy(g_ctx);
  g_ctx = nullptr;
}
