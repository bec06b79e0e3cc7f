// MASSolver's bad-DOF selections (use_bad_dof_precond): host selection on
// per-scalar-row scores in the partition order of the permuted operator.
#pragma once

#include <cstdint>
#include <vector>

namespace lss {

enum BadDofStrategy : int { BADDOF_GPUHYBRID = 0, BADDOF_ELBOW = 1, BADDOF_KMEAN = 2, BADDOF_GMM = 3 };

// Elbow of the ascending log|diag| curve against its chord: the positions from
// the largest deviation on (BadDOFPreconditioner.cu:61-100).
std::vector<int32_t> mas_select_elbow(const std::vector<double> &diag_abs);

// 2-means on the search_fraction largest max|off-diagonal| scores, centroid
// ratio test, positions above the midpoint widened by +-expand_neighbors
// (BadDofKMeanPreconditioner.cu:63-172).
std::vector<int32_t> mas_select_kmean(const std::vector<double> &offdiag_max, double search_fraction,
                                      double jump_threshold, int max_iterations, int expand_neighbors);

// Two-component GMM by EM on l1 row norms, mean ratio test, positions of the
// high component widened by +-expand_neighbors (BadDofGMMPreconditioner.cu:73-255).
std::vector<int32_t> mas_select_gmm(const std::vector<double> &l1, double jump_threshold, double tol,
                                    int max_iterations, int expand_neighbors);

}  // namespace lss
