// The GPUHybrid-compatible solver object behind the C ABI.
#pragma once

#include <chrono>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "kernels.hpp"
#include "lss_common.hpp"
#include "multifrontal.hpp"
#include "pattern.hpp"
#include "postproc.hpp"

namespace lss {

class HybridSolver {
public:
    explicit HybridSolver(const Params &p);
    ~HybridSolver();
    HybridSolver(const HybridSolver &) = delete;
    HybridSolver &operator=(const HybridSolver &) = delete;

    void set_parameters(const char *json);
    std::string info_json() const;
    std::string name() const;

    void analyze(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner);
    void factorize(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner, const double *values);
    // values in device memory (input storage order), pattern from a previous analyze/factorize
    void factorize_device(const double *d_values, cudaStream_t user_stream);
    void set_problematic_dofs(const int32_t *idx, int32_t count);
    void solve_host(const double *b, double *x);
    void solve_device(const double *d_b, double *d_x, cudaStream_t user_stream);
    void grad_pattern_host(const double *lambda, const double *x, double *dA);
    void grad_pattern_device(const double *d_lambda, const double *d_x, double *d_dA, cudaStream_t user_stream);
    void grad_params_device(const double *d_lambda, const double *d_x, int32_t nparams, const int64_t *d_rowptr,
                            const int32_t *d_cols, const double *d_vals, double *d_dtheta, cudaStream_t user_stream);

    // operator-level access (original ordering, host pointers)
    void op_spmv(const double *x, double *y);
    void op_spmv_outer(const double *x, double *y);
    void op_row_scores(double *diag, double *offmax, double *l1);
    void op_mas(const double *r, double *z);
    void op_precond(const double *r, double *z);
    void op_time(int kind, int reps, double *ms, double *bytes);

    const std::vector<int32_t> &gmm_selection() const { return gmm_sel_; }
    const std::vector<std::vector<int32_t>> &subdomains() const { return subs_; }
    std::vector<int32_t> selected() const;
    const Pattern &pattern() const { return pat_; }
    bool factorized() const { return factorized_; }
    int32_t n() const { return pat_.n; }
    int device() const { return p_.device; }
    int iterations() const { return num_iterations_; }

    std::string last_error;

private:
    friend class BatchSolver;  // merges factorized solvers into one batched image
    // Runs a device-pointer call on the caller's stream (a non-null stream);
    // the internal stream otherwise.  Graphs captured on either replay on both.
    struct StreamScope {
        HybridSolver *s;
        cudaStream_t saved;
        StreamScope(HybridSolver *h, cudaStream_t user) : s(h), saved(h->stream_)
        {
            if (user) {
                LSS_CUDA(cudaStreamSynchronize(saved));
                s->stream_ = user;
            }
        }
        ~StreamScope() { s->stream_ = saved; }
    };
    void factorize_common();
    void select_stiff(const CscView &A);
    void select_stiff_mas(const CscView &A);
    std::vector<double> row_scores(int kind);
    void setup_stiff();
    void setup_mas();
    void ensure_vectors();
    void run_pcg();
    // r32 (optional): r already rounded to FP32 (mixed precision); converted here otherwise
    void precond(const double *r, double *z, int dot_mode, const float *r32 = nullptr);
    void mas_apply(const double *xin, double *z, bool acc, const double *rdot, int dot_mode, double scale,
                   float *z32 = nullptr, const float *xin32 = nullptr, float *z_lo = nullptr);
    void estimate_omega();
    void autotune_spmv();
    void iteration();
    void launch_chunk(int iters);
    void invalidate_graph();
    void rz_dot(const double *r, const double *z, int dot_mode);
    int64_t n_vec() const { return (int64_t)pat_.nb * pat_.bd; }

    Params p_;
    cudaStream_t stream_ = nullptr;
    bool have_pattern_ = false;
    bool factorized_ = false;
    Pattern pat_;
    CoarseSpace cs_;
    std::vector<int32_t> user_dofs_;
    std::vector<int32_t> h_outer_, h_inner_;  // copy of the analysed pattern (adjoint)
    std::vector<int32_t> gmm_sel_;
    std::vector<std::vector<int32_t>> subs_;
    // the last decomposition (set, size limit, components), reused for the same set
    std::vector<int32_t> decomp_sel_;
    int64_t decomp_max_ = -1;
    std::vector<std::vector<int32_t>> decomp_subs_;
    std::map<std::string, double> stats_;
    std::map<std::string, std::string> sstats_;

    // operator
    BsrDev A_;
    DBuf<int32_t> d_rows_, d_cols_, d_perm_, d_outer_, d_inner_, d_row_of_;
    DBuf<double> d_vals_, d_csc_;
    DBuf<float> d_vals32_;
    DBuf<float2> d_vals_df_;  // df32 outer SpMV: operator values as (hi, lo) FP32 pairs
    DBuf<int64_t> d_src_;
    // MAS
    MasDev mas_;
    DBuf<int32_t> d_part_off_, d_cbase0_, d_part_of_, d_cmap_, d_memb_ptr_, d_memb_rows_, d_chunk_r0_;
    CoarseMembers memb_;
    DBuf<uint8_t> d_key0_, d_ccnt0_;
    std::vector<DBuf<uint8_t>> d_key_, d_ccnt_;
    std::vector<DBuf<int32_t>> d_cbase_;
    DBuf<char> d_inv0_, d_invc_, d_v_, d_u_;
    DBuf<double> d_stage0_, d_stagec_, d_cpartial_;  // MAS Galerkin staging, kept per pattern
    bool mas_fp32_ = false;
    // stiff blocks
    StiffDev stiff_;
    DBuf<int32_t> d_sdofs_, d_ssub_, d_soff_;
    DBuf<int64_t> d_sinvoff_;
    DBuf<double> d_sinv_, d_st_;
    DBuf<float> d_sinv32_;
    std::unique_ptr<MfFactor> mf_;  // subdomains above STIFF_DENSE_MAX DOFs
    // host copies of the stiff layout (batched solves merge them)
    std::vector<int32_t> h_sdofs_, h_soff_;
    std::vector<int64_t> h_sinvoff_;
    int32_t ndense_ = 0;
    int64_t inv_total_ = 0;
    std::vector<uint8_t> h_precise_;  // block rows of the double-float preconditioner residual
    void stiff_correct(double *z, const int *done, float *z32 = nullptr, float *z_lo = nullptr);
    // PCG
    DBuf<double> d_x_, d_b_, d_r_, d_p_, d_z_, d_ap_, d_w_, d_tmp_;
    DBuf<float> d_z32_;  // mixed precision: FP32 shadow of z, input of the FP32 residual SpMV
    DBuf<float2> d_p_df_, d_ap_df_;  // df32 outer SpMV: p and A p as (hi, lo) FP32 pairs
    DBuf<float> d_r32_, d_w32_;      // mixed precision: r and the preconditioner's residual in FP32
    DBuf<float> d_z_lo_;             // mixed precision: z - z32 rounded to FP32 (double-float residual rows)
    DBuf<uint8_t> d_precise_;        // mixed precision: block rows whose residual runs in double-float
    bool precise_rows_ = false;
    bool need_vals_df() const { return df32() || (p_.mixed && p_.precond_residual != 1); }
    void setup_precise_rows();
    // auto: double-float for block rows (a 3x3 block needs 9 DFMA per 76 bytes,
    // FP64-pipe-bound on this GPU); FP64 for scalar CSR rows, which it does not bind
    bool df32() const { return p_.outer_spmv == 2 || (p_.outer_spmv == 0 && p_.mixed && p_.block_size > 1); }
    bool refine_fp64_ = false;  // refinement restarts of the current solve use the FP64 product
    bool outer_df() const { return df32() && !refine_fp64_; }
    void outer_spmv_alpha();  // Ap, p.Ap, alpha with the configured outer SpMV
    void split_p();           // refresh the df32 split of p (after p = z)
    DBuf<PcgState> d_state_;
    PcgState *h_state_ = nullptr;
    DBuf<double> d_partials_, d_scalar_;
    DBuf<unsigned> d_counter_;
    DBuf<int> d_bad_;
    GridReduce gr_;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_iters_ = 0;
    size_t graph_nodes_ = 0;
    PinnedBuf pin_;
    cudaEvent_t copy_ev_[2] = {nullptr, nullptr};  // staged uploads: the two pinned halves

    // last solve
    int num_iterations_ = 0;
    double final_res_norm_ = 0.0, rhs_norm_ = 0.0;
    int stop_reason_ = 0;
    int refinements_ = 0;
    double omega_ = 1.0, lambda_max_ = 0.0;
    bool lanczos_mode_ = false;
    bool lanes_tuned_ = false;
};

}  // namespace lss
