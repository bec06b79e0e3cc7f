// Stand-in for polysolve/linear/Solver.hpp, for compiling the adapter
// (include/lss_polysolve.hpp) where the reference's own header is absent.  It
// restates the virtual interface of polysolve::linear::Solver with the same
// signatures (src/polysolve/linear/Solver.hpp:32-149): the adapter's
// `override`s fail to compile if they drift from it.  Where a reference
// checkout exists, the adapter test compiles against the real header too.
#pragma once

#include <polysolve/Types.hpp>

#include <memory>
#include <set>
#include <string>

namespace spdlog {
class logger;
}

namespace polysolve::linear {

class Solver {
public:
    typedef Eigen::VectorXd VectorXd;
    template <typename T>
    using Ref = Eigen::Ref<T>;

    virtual ~Solver() = default;

protected:
    Solver() = default;

public:
    virtual void set_parameters(const json &params) {}
    virtual void get_info(json &params) const {}
    virtual void analyze_pattern(const StiffnessMatrix &A, const int precond_num) {}
    virtual void factorize(const StiffnessMatrix &A) {}
    virtual void analyze_pattern_dense(const Eigen::MatrixXd &A, const int precond_num) {}
    virtual void factorize_dense(const Eigen::MatrixXd &A) {}
    virtual bool is_dense() const { return false; }
    virtual void set_block_size(int block_size) {}
    virtual void set_is_nullspace(const VectorXd &x) {}
    virtual void set_tolerance(const double tol) {}
    virtual void set_problematic_dofs(const std::set<int> &bad_dofs) {}
    virtual void solve(const Ref<const VectorXd> b, Ref<VectorXd> x) = 0;
    virtual std::string name() const { return ""; }
};

}  // namespace polysolve::linear
