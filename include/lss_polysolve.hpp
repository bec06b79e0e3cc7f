// Header-only polysolve adapter: a polysolve::linear::Solver named "GPUHybrid"
// whose factorize/solve run on the GB300 library behind include/lss.h.
//
// Drop-in for src/polysolve/linear/GPUHybrid.{hpp,cu} of the reference:
// same virtual interface (Solver.hpp:90-135), same JSON parameter object
// (GPUHybrid.cu:106-179), same name() values (GPUHybrid.hpp:57-67), same
// get_info keys (GPUHybrid.cu:181-185) plus extras.  Errors become
// std::runtime_error instead of exit() (GPUHybrid.cu:34-63).
//
// Requires Eigen 3.4, nlohmann::json and the polysolve headers; link liblss.so.
#pragma once

#include <polysolve/linear/Solver.hpp>

#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "lss.h"

namespace polysolve::linear
{
    class LssGPUHybrid : public Solver
    {
    public:
        LssGPUHybrid()
        {
            lss_solver *s = nullptr;
            const lss_status st = lss_create(nullptr, &s);
            if (st != LSS_OK)
                throw std::runtime_error(std::string("[GPUHybrid] ") + lss_last_error(nullptr));
            s_ = s;
        }
        ~LssGPUHybrid() override { lss_destroy(s_); }
        LssGPUHybrid(const LssGPUHybrid &) = delete;
        LssGPUHybrid &operator=(const LssGPUHybrid &) = delete;

        void set_parameters(const json &params) override { check(lss_set_parameters(s_, params.dump().c_str())); }

        void get_info(json &params) const override
        {
            size_t n = 0;
            lss_get_info(s_, nullptr, 0, &n);
            std::string buf(n + 1, '\0');
            check(lss_get_info(s_, buf.data(), buf.size(), &n));
            const json j = json::parse(buf.c_str());
            for (auto it = j.begin(); it != j.end(); ++it)
                params[it.key()] = it.value();
        }

        void analyze_pattern(const StiffnessMatrix &A, const int) override
        {
            const StiffnessMatrix &C = compressed(A);
            check(lss_analyze_pattern(s_, (int32_t)C.rows(), (int64_t)C.nonZeros(), C.outerIndexPtr(),
                                      C.innerIndexPtr()));
        }

        void factorize(const StiffnessMatrix &A) override
        {
            const StiffnessMatrix &C = compressed(A);
            check(lss_factorize(s_, (int32_t)C.rows(), (int64_t)C.nonZeros(), C.outerIndexPtr(), C.innerIndexPtr(),
                                C.valuePtr()));
        }

        void solve(const Ref<const VectorXd> b, Ref<VectorXd> x) override
        {
            check(lss_solve(s_, b.data(), x.data(), 1, (int64_t)b.size()));
        }

        std::string name() const override
        {
            char buf[64] = {0};
            lss_name(s_, buf, sizeof(buf));
            return buf;
        }

        void set_problematic_dofs(const std::set<int> &bad_dofs) override
        {
            std::vector<int32_t> v(bad_dofs.begin(), bad_dofs.end());
            check(lss_set_problematic_dofs(s_, v.data(), (int32_t)v.size()));
        }

    private:
        // The C ABI takes compressed storage (BSRMatrix.cu:444-452 compresses too).
        const StiffnessMatrix &compressed(const StiffnessMatrix &A)
        {
            if (A.isCompressed())
                return A;
            tmp_ = A;
            tmp_.makeCompressed();
            return tmp_;
        }
        void check(lss_status st) const
        {
            if (st != LSS_OK)
                throw std::runtime_error(std::string("[GPUHybrid] ") + lss_status_string(st) + ": " +
                                         lss_last_error(s_));
        }
        lss_solver *s_ = nullptr;
        StiffnessMatrix tmp_;
    };
} // namespace polysolve::linear
