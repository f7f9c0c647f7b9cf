// breseq's coverage_distribution.cpp compiled as part of this translation unit (the file is read in
// place from the reference tree, like the rest of the reference build), so that its file-local
// fit_coverage_distribution (coverage_distribution.cpp:345-399) can be called on its own: the
// public CoverageDistribution::fit runs it and then draws a plot through gnuplot, which is not part
// of the scored path.  Test infrastructure.
#include "coverage_distribution.cpp"

namespace breseq {

CoverageDistributionFitResult harness_fit_coverage(const coverage_histogram_t& hist, double deletion_propagation_pr_cutoff,
                                                   uint32_t& censor_start, uint32_t& censor_end, double& nb_fit_scale) {
  return fit_coverage_distribution(hist, deletion_propagation_pr_cutoff, censor_start, censor_end, nb_fit_scale);
}

}  // namespace breseq
