// Drives include/lss_polysolve.hpp the way polysolve's callers do
// (Solver::create -> set_parameters -> analyze_pattern -> factorize -> solve
// -> get_info; tests/linear_solve.cpp:433-475 of the reference): a 2D
// five-point Laplacian with a stiff square (x1e6), solved to 1e-8.
// Prints one line: "ok <name> <iterations> <relative residual> <FP64 floor
// eps || |A| |x| || / ||b||>", or "error <message>" (exit 2) when the library
// refuses, e.g. without a GPU.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <utility>
#include <memory>
#include <vector>

#include "lss_polysolve.hpp"

int main()
{
    using namespace polysolve;
    const int g = 64, n = g * g;
    std::vector<int> outer{0}, inner;
    std::vector<double> vals;
    auto kappa = [&](int i, int j) { return (i > 20 && i < 30 && j > 20 && j < 30) ? 1e6 : 1.0; };
    for (int j = 0; j < g; ++j)
        for (int i = 0; i < g; ++i) {
            const double k = kappa(i, j);
            double diag = 0.0;
            const int nb[4][2] = {{i, j - 1}, {i - 1, j}, {i + 1, j}, {i, j + 1}};
            std::vector<std::pair<int, double>> row;
            for (auto &q : nb) {
                const double w = (q[0] < 0 || q[0] >= g || q[1] < 0 || q[1] >= g) ? k : std::sqrt(k * kappa(q[0], q[1]));
                diag += w;
                if (q[0] >= 0 && q[0] < g && q[1] >= 0 && q[1] < g) row.push_back({q[1] * g + q[0], -w});
            }
            row.push_back({j * g + i, diag});
            std::sort(row.begin(), row.end());
            for (auto &e : row) {
                inner.push_back(e.first);
                vals.push_back(e.second);
            }
            outer.push_back((int)inner.size());
        }
    StiffnessMatrix A;
    A.assign_compressed(n, n, outer.data(), inner.data(), vals.data());
    Eigen::VectorXd b(n), x(n);
    for (int i = 0; i < n; ++i) {
        b[i] = std::sin(0.37 * i) + 0.5;
        x[i] = 0.0;
    }
    try {
        std::unique_ptr<linear::Solver> s = std::make_unique<linear::LssGPUHybrid>();
        s->set_parameters(json::parse(R"({"solver": "GPUHybrid", "GPUHybrid": {"block_size": 1,
            "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}})"));
        s->analyze_pattern(A, 1);
        s->factorize(A);
        const Eigen::VectorXd &cb = b;
        s->solve(linear::Solver::Ref<const Eigen::VectorXd>(cb), linear::Solver::Ref<Eigen::VectorXd>(x));
        json info;
        s->get_info(info);
        double rr = 0.0, bb = 0.0, ff = 0.0;
        for (int r = 0; r < n; ++r) {
            double ax = 0.0, aax = 0.0;
            for (int k = outer[r]; k < outer[r + 1]; ++k) {
                ax += vals[k] * x[inner[k]];
                aax += std::fabs(vals[k] * x[inner[k]]);
            }
            rr += (b[r] - ax) * (b[r] - ax);
            bb += b[r] * b[r];
            ff += aax * aax;
        }
        std::printf("ok %s %s %.3e %.3e\n", s->name().c_str(), info["num_iterations"].dump().c_str(),
                    std::sqrt(rr / bb), 2.220446049250313e-16 * std::sqrt(ff / bb));
        return 0;
    } catch (const std::exception &e) {
        std::printf("error %s\n", e.what());
        return 2;
    }
}
