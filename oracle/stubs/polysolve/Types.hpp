// Stand-in for polysolve/Types.hpp (not installed in this build environment):
// the two aliases the Solver interface uses, as the reference declares them
// (src/polysolve/Types.hpp:9-17).
#pragma once

#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <nlohmann/json.hpp>

namespace polysolve {
typedef Eigen::SparseMatrix<double, Eigen::ColMajor> StiffnessMatrix;
using json = nlohmann::json;
}  // namespace polysolve
